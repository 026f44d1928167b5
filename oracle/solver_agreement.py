"""How much the labels depend on the metric solver (test infrastructure).

The reference solves each seed's metric with Eigen's float
BDCSVD(...).solve and decides positive semi-definiteness with Eigen's
eigenvalues() (GPU-AS/Image.cpp:874-1009; the nearest PSD matrix at
:786-835 and :1460-1534).  Eigen is not vendored, so the primary solver of
the oracle and the CUDA path (a one-sided Jacobi SVD with Eigen's rank rule
and an exact PSD test) is a restatement whose rounding differs from
Eigen's.  This script runs the oracle's whole pipeline twice on the same
inputs -- with the primary solver (whose labels equal the CUDA path's bit
for bit) and with the second FP32 restatement of Eigen's algorithms
(orc_set_solver(1): QR-preconditioned two-sided Jacobi SVD, Hessenberg +
Francis QR eigenvalues) -- and reports the fraction of voxels whose label is
the same and the relative difference of the final centroids.

    python oracle/solver_agreement.py [cfg1 cfg2 stream]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def centroid_rel_error(sa, sb):
    """max over seeds of |position difference| / |position| (positions in voxels)"""
    pa, pb = sa[:, :3].astype(np.float64), sb[:, :3].astype(np.float64)
    return float(np.max(np.linalg.norm(pa - pb, axis=1) / np.maximum(np.linalg.norm(pb, axis=1), 1.0)))


def compare_clip(rgb, fwd, bwd, K, iters, nthreads, truth=None, modes=(1, 8), **kw):
    """labels of the primary solver against those of each other mode
    (1: the Eigen-algorithm restatement; 8: the control, the primary solver
    with sequential sums), after the first iteration and after all"""
    from oracle import evaluate, oracle
    res = {}
    runs = {}
    for mode in (0,) + tuple(modes):
        oracle.set_solver(mode)
        runs[mode] = (oracle.run_clip(rgb, fwd, bwd, K, iters=iters, nthreads=nthreads, **kw),
                      oracle.run_clip(rgb, fwd, bwd, K, iters=1, nthreads=nthreads, **kw)[1])
    oracle.set_solver(0)
    (la, ra, sa, ia), r1a = runs[0]
    for mode in modes:
        (lb, rb, sb, ib), r1b = runs[mode]
        res[mode] = {"voxels": int(la.size), "iter1_raw_equal": float((r1a == r1b).mean()),
                     "raw_equal": float((ra == rb).mean()), "final_equal": float((la == lb).mean()),
                     "centroid_rel_error_max": centroid_rel_error(sa, sb) if sa.shape == sb.shape else None,
                     "seeds": int(ia["Kp"])}
        if truth is not None:
            qa, qb = evaluate.evaluate(la, truth), evaluate.evaluate(lb, truth)
            res[mode]["quality"] = {k: (round(qa[k], 4), round(qb[k], 4)) for k in
                                    ("undersegmentation", "segmentation_accuracy", "boundary_recall")}
    return res


def compare_stream(rgb, fwd, bwd, seeds100, iters, nthreads, modes=(1, 8)):
    from oracle import oracle
    out = {}
    for mode in (0,) + tuple(modes):
        oracle.set_solver(mode)
        out[mode] = oracle.run_stream(rgb, fwd, bwd, seeds_num_100=seeds100, iters=iters, nthreads=nthreads)[0]
    oracle.set_solver(0)
    return {mode: {"voxels": int(out[0].size), "final_equal": float((out[0] == out[mode]).mean())} for mode in modes}


def main(which):
    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    n = os.cpu_count() or 1
    res = {}
    def truth(w):
        return asv.synth_truth(w["W"], w["H"], w["D"], n_ellipses=w["n_ellipses"], noise_sigma=w["noise_sigma"],
                               vmax=w["vmax"], jitter=w.get("jitter", 0.0), seed=w["seed"])
    if "cfg1" in which:
        w = workloads.CLIP_240x160x30
        res["clip_240x160x30_K200_I10"] = compare_clip(*workloads.make_clip(w), w["K"], w["iters"], n,
                                                       truth=truth(w), full_ladder=w["full_ladder"])
    if "cfg2" in which:
        w = workloads.CLIP_320x240x85
        res["clip_320x240x85_K1000_I15"] = compare_clip(*workloads.make_clip(w), w["K"], w["iters"], n,
                                                        truth=truth(w))
    if "stream" in which:
        w = workloads.STREAM_720P
        rgb, fwd, bwd = workloads.stream_frames(w, 0, 50)
        res["stream_1280x720_two_windows_I20"] = compare_stream(rgb, fwd, bwd, w["seeds_num_100"], w["iters"], n)
    return res


if __name__ == "__main__":
    which = sys.argv[1:] or ["cfg1", "cfg2", "stream"]
    t = time.time()
    for k, v in main(which).items():
        print(k, v, flush=True)
    print(f"{time.time() - t:.0f} s")
