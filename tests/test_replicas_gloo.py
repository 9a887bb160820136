"""The multi-GPU bench is "replicas only": N ranks run N independent replicas, joined on the host by
a barrier and a max over ranks (gloo), with no collective on the data path.  These tests run that
host logic as two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, os.environ["PT_ROOT"])
import bench
rank, world, local = bench.dist_env()
d = bench.Dist(world)
d.barrier()
m = d.max(1.0 + 2.5 * rank)
d.barrier()
print("RESULT", rank, world, local, repr(m), flush=True)
d.close()
"""


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _env(rank: int, world: int, port: int) -> dict:
    return dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                MASTER_PORT=str(port), PT_ROOT=ROOT)


def test_barrier_and_max_over_two_gloo_ranks():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", CHILD], env=_env(r, 2, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    try:
        for p in procs:
            outs.append(p.communicate(timeout=180))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    results = {}
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
        line = [ln for ln in out.splitlines() if ln.startswith("RESULT")][0].split()
        results[int(line[1])] = (int(line[2]), int(line[3]), float(line[4]))
    # every rank sees the world size, its own local rank, and the max over both ranks
    assert results == {0: (2, 0, 3.5), 1: (2, 1, 3.5)}


def test_reference_arm_runs_on_rank_zero_only():
    # a rank other than 0 of the reference arm exits at once, without output or a process group
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=_env(1, 2, _free_port()), capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
