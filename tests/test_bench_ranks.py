"""The multi-GPU form is replicas only: each rank segments its own clips and
the job's throughput is all ranks' units over the slowest rank's time.  The
aggregation and the rank-0-only reference arm run here on CPU with two gloo
ranks."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    v, s = bench.replicas_value(100.0, [2.0, 5.0][rank])
    q.put((rank, v, s))
    dist.destroy_process_group()


def test_replicas_value_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 2000
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, v, s in got:
        assert s == 5.0                      # the slowest rank's time
        assert v == pytest.approx(200.0 / 5.0)


def test_reference_arm_prints_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert p.returncode == 0 and p.stdout.strip() == ""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "batch16", "--steps", "1", "--warmup", "0"], capture_output=True,
                       text=True, env=env, timeout=300)
    assert p.returncode == 0
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line


def test_reference_arm_loads_no_gpu_library():
    """The headline's CPU arm (stream_720p) times the oracle on one window of
    the crop sample, with inputs from the generator compiled on its own: the
    process maps the oracle's libraries and not libasv.so."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "m = open('/proc/self/maps').read();"
            "print('MAPPED', sorted({l.split()[-1].rsplit('/', 1)[-1] for l in m.splitlines() if '.so' in l}))")
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, env=env,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = p.stdout.strip().splitlines()
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["steps"] == 1 and line["windows_timed"] == 1
    assert line["config"]["workload"].startswith("stream_1280x720")
    mapped = lines[-1]
    assert "liboracle.so" in mapped and "libsynth.so" in mapped
    assert "libasv.so" not in mapped
