"""ctypes loader of the CPU restatement (asv_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "asv_oracle.c")
HDR = os.path.join(HERE, "asv_oracle.h")
LIB = os.path.join(HERE, "liboracle.so")

c_int, c_float, c_void_p, c_long = ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_long


class Params(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("W", "H", "D", "K", "iters", "variant", "full_ladder",
                                     "middlebury", "density_adjust", "nthreads")]


class StreamParams(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("W", "H", "D_all", "K_video", "seeds_num_100", "iters",
                                     "block_size", "nthreads")]


class GridInfo(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("s", "dNum", "hNum", "wNum", "Kp")]


# The seeded synthetic-clip generator (asv_synth_clip) compiled on its own,
# so that CPU-only runs (the timed CPU restatement) generate their inputs
# without loading libasv.so; same source and host flags as in libasv.so.
SYNTH_SRC = os.path.join(os.path.dirname(HERE), "anisotropic_supervoxel_gb300", "csrc", "asv_synth.cpp")
SYNTH_INC = [os.path.join(os.path.dirname(HERE), "include"),
             os.path.join(os.path.dirname(HERE), "anisotropic_supervoxel_gb300", "csrc")]
SYNTH_LIB = os.path.join(HERE, "libsynth.so")


def build_synth(force=False):
    if not force and os.path.exists(SYNTH_LIB) and os.path.getmtime(SYNTH_LIB) >= max(
            os.path.getmtime(SYNTH_SRC), os.path.getmtime(__file__)):
        return SYNTH_LIB
    tmp = SYNTH_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-DASV_SYNTH_ONLY",
           *[f"-I{d}" for d in SYNTH_INC], "-o", tmp, SYNTH_SRC]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("synthetic generator build failed:\n" + p.stdout + p.stderr)
    os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


class SynthParams(ctypes.Structure):
    _fields_ = [("W", c_int), ("H", c_int), ("frame0", c_int), ("nframes", c_int), ("n_ellipses", c_int),
                ("noise_sigma", c_float), ("vmax", c_float), ("jitter", c_float), ("drift_amp", c_float),
                ("drift_period", c_float), ("seed", ctypes.c_uint64)]


_SYNTH = None


def synth_clip(W, H, D, n_ellipses=12, noise_sigma=5.0, vmax=3.0, jitter=0.0, drift_amp=0.0,
               drift_period=60.0, seed=1, frame0=0):
    """The seeded synthetic clip (rgb uint8 [D,H,W,3], fwd/bwd float32
    [D,H,W,2]), identical to anisotropic_supervoxel_gb300.synth_clip."""
    global _SYNTH
    if _SYNTH is None:
        build_synth()
        _SYNTH = ctypes.CDLL(SYNTH_LIB)
        _SYNTH.asv_synth_clip.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
        _SYNTH.asv_synth_clip.restype = c_int
    rgb = np.empty((D, H, W, 3), np.uint8)
    fwd = np.empty((D, H, W, 2), np.float32)
    bwd = np.empty((D, H, W, 2), np.float32)
    p = SynthParams(W, H, frame0, D, n_ellipses, noise_sigma, vmax, jitter, drift_amp, drift_period, seed)
    if _SYNTH.asv_synth_clip(ctypes.byref(p), _p(rgb), _p(fwd), _p(bwd)) != 0:
        raise ValueError("bad synthetic clip parameters")
    return rgb, fwd, bwd


def build(force=False):
    """Compiles liboracle.so with -ffp-contract=off (no FMA contraction), and
    the generator library."""
    build_synth(force)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(HDR), os.path.getmtime(__file__)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-o", tmp, SRC, "-lm"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + p.stdout + p.stderr)
    os.replace(tmp, LIB)
    return LIB


_LIB = None


def load():
    global _LIB
    if _LIB is None:
        build()
        _LIB = ctypes.CDLL(LIB)
        _LIB.orc_ratio.restype = c_float
        _LIB.orc_ratio.argtypes = [c_int, c_float]
        _LIB.orc_float_to_half.restype = ctypes.c_uint16
        _LIB.orc_float_to_half.argtypes = [c_float]
        _LIB.orc_metric_solve.argtypes = [c_void_p, c_void_p, c_int, c_int, c_int, c_float,
                                          c_float, c_int, c_void_p]
        _LIB.orc_jfa_pass.argtypes = [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_int, c_float, c_int]
        _LIB.orc_rgb2lab.argtypes = [c_void_p, c_long, c_void_p]
    return _LIB


def _p(a):
    return a.ctypes.data_as(c_void_p) if a is not None else None


def set_solver(mode):
    """0: the primary metric solver (the CUDA path's twin); 1: the FP32
    restatement of the algorithms of the reference's Eigen calls."""
    load().orc_set_solver(int(mode))


def grid_seeds(W, H, D, K, middlebury=0):
    lib = load()
    g = GridInfo()
    kp = lib.orc_grid_seeds(W, H, D, K, middlebury, None, 0, ctypes.byref(g))
    if kp <= 0:
        raise ValueError("no seed grid for these sizes")
    s4 = np.zeros((kp, 4), np.float32)
    lib.orc_grid_seeds(W, H, D, K, middlebury, _p(s4), kp, ctypes.byref(g))
    return s4, g


def density_adjust(rgb, grid4, g):
    lib = load()
    D, H, W, _ = rgb.shape
    out = np.zeros((g.Kp, 4), np.float32)
    dens = np.zeros(g.Kp, np.float32)
    n = lib.orc_density_adjust(_p(np.ascontiguousarray(rgb)), W, H, D, _p(grid4), ctypes.byref(g),
                               _p(out), _p(dens))
    return out[:n], dens


def rgb2lab(rgb):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    n = rgb.size // 3
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    load().orc_rgb2lab(_p(rgb), n, _p(out))
    return out


def gradient_half(rgb):
    D, H, W, _ = rgb.shape
    out = np.zeros((D, H, W), np.uint16)
    load().orc_gradient_half(_p(np.ascontiguousarray(rgb)), W, H, D, _p(out))
    return out


def m6_negative(M):
    """exact test: the symmetric matrix (M00,M01,M02,M11,M12,M22) has an eigenvalue < 0"""
    M = np.ascontiguousarray(M, np.float32)
    return int(load().orc_m6_negative(_p(M)))


def enforce_connectivity(labels, supsz):
    """Image::EnforceLabelConnectivity3D restated; returns (labels, number of labels)."""
    labels = np.ascontiguousarray(labels, np.int32)
    D, H, W = labels.shape
    out = np.empty_like(labels)
    n = load().orc_enforce_connectivity(_p(labels), W, H, D, int(supsz), _p(out))
    if n < 0:
        raise MemoryError("oracle connectivity: allocation failed")
    return out, int(n)


def metric_solve(fwd, bwd, sx, sy, frame):
    D, H, W, _ = fwd.shape
    M = np.zeros(6, np.float32)
    neg = load().orc_metric_solve(_p(fwd), _p(bwd), W, H, D, sx, sy, frame, _p(M))
    return M, neg


def seed_metrics(fwd, bwd, pos3, reseed, angle_filter):
    D, H, W, _ = fwd.shape
    pos3 = np.ascontiguousarray(pos3, np.float32)
    kp = pos3.shape[0]
    M = np.zeros((kp, 6), np.float32)
    kind = np.zeros(kp, np.int32)
    load().orc_seed_metrics(_p(fwd), _p(bwd), W, H, D, kp, _p(pos3), reseed, angle_filter,
                            _p(M), _p(kind))
    return M, kind


def ladder(s, full=0, maxdim=0):
    steps = np.zeros(64, np.int32)
    rmul = np.zeros(64, np.float32)
    n = load().orc_ladder(s, full, maxdim, _p(steps), _p(rmul), 64)
    return list(steps[:n]), list(rmul[:n])


def ratio(s, compactness):
    return load().orc_ratio(s, compactness)


def draw_seeds(shape, pos3):
    D, H, W = shape
    out = np.zeros(shape, np.int32)
    pos3 = np.ascontiguousarray(pos3, np.float32)
    load().orc_draw_seeds(W, H, D, pos3.shape[0], _p(pos3), _p(out))
    return out


def jfa_pass(labels, lab4, seeds12, step, ratio_, nthreads=1):
    D, H, W = labels.shape
    out = np.zeros_like(labels)
    s = np.ascontiguousarray(seeds12, np.float32)
    pos3 = np.ascontiguousarray(s[:, 0:3])
    slab3 = np.ascontiguousarray(s[:, 3:6])
    M6 = np.ascontiguousarray(s[:, 6:12])
    load().orc_jfa_pass(W, H, D, _p(np.ascontiguousarray(labels, np.int32)), _p(out),
                        _p(np.ascontiguousarray(lab4)), _p(pos3), _p(slab3), _p(M6), step,
                        ratio_, nthreads)
    return out


def centroid_sums(labels, lab4, kp, nthreads=1):
    D, H, W = labels.shape
    out = np.zeros((kp + 1, 7), np.int64)
    load().orc_centroid_sums(W, H, D, kp, _p(np.ascontiguousarray(labels, np.int32)),
                             _p(np.ascontiguousarray(lab4)), _p(out), nthreads)
    return out


def finalize(shape, sums, lab4, pos3, slab3):
    D, H, W = shape
    pos3 = np.ascontiguousarray(pos3, np.float32).copy()
    slab3 = np.ascontiguousarray(slab3, np.float32).copy()
    load().orc_finalize(W, H, D, pos3.shape[0], _p(np.ascontiguousarray(sums)),
                        _p(np.ascontiguousarray(lab4)), _p(pos3), _p(slab3))
    return pos3, slab3


def postprocess(labels, sums, kp):
    D, H, W = labels.shape
    out = np.ascontiguousarray(labels, np.int32).copy()
    stats = np.zeros(3, np.int32)
    load().orc_postprocess(W, H, D, kp, _p(np.ascontiguousarray(sums)), _p(out), _p(stats))
    return out, stats


def run_clip(rgb, fwd, bwd, K, iters=20, variant=0, full_ladder=0, middlebury=0,
             density_adjust=1, nthreads=1):
    """Plain per-clip run; returns (labels, raw_labels, seeds[Kp,12], info)."""
    lib = load()
    D, H, W, _ = rgb.shape
    p = Params(W, H, D, K, iters, variant, full_ladder, middlebury, density_adjust, nthreads)
    labels = np.zeros((D, H, W), np.int32)
    raw = np.zeros((D, H, W), np.int32)
    seeds = np.zeros((32768, 12), np.float32)
    info = np.zeros(8, np.int32)
    kp = lib.orc_run_clip(ctypes.byref(p), _p(np.ascontiguousarray(rgb)),
                          _p(np.ascontiguousarray(fwd)), _p(np.ascontiguousarray(bwd)),
                          _p(labels), _p(raw), _p(seeds), _p(info))
    if kp <= 0:
        raise ValueError(f"oracle run failed ({kp})")
    return labels, raw, seeds[:kp].copy(), {"Kp": int(info[0]), "s": int(info[1]),
                                            "dead": int(info[2]), "neg": int(info[3]),
                                            "final_label_num": int(info[4])}


def run_stream(rgb, fwd, bwd, K_video=0, seeds_num_100=0, iters=20, block_size=30, nthreads=1):
    lib = load()
    D, H, W, _ = rgb.shape
    p = StreamParams(W, H, D, K_video, seeds_num_100, iters, block_size, nthreads)
    labels = np.zeros((D, H, W), np.int32)
    info = np.zeros(4, np.int32)
    nb = lib.orc_run_stream(ctypes.byref(p), _p(np.ascontiguousarray(rgb)),
                            _p(np.ascontiguousarray(fwd)), _p(np.ascontiguousarray(bwd)),
                            _p(labels), _p(info))
    if nb <= 0:
        raise ValueError(f"oracle stream run failed ({nb})")
    return labels, {"blocks": int(info[0]), "placed": int(info[1])}
