"""bench.py's multi-rank path on the CPU (gloo, two ranks, 127.0.0.1): the rank reductions the
timed region uses (max of the per-rank times, sum of the per-rank points), the barrier, and the
reference arm under torchrun, where rank 0 alone runs and prints one line and the other ranks exit
0 without work.  The path has no data-path collective (replicas), so these are all it needs."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


CHILD = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
rank, world, local = bench.dist_info()
d = bench.Dist(world, local, use_cuda=False)
d.barrier()
out = {{"rank": rank, "world": world, "max": d.max(10.0 * (rank + 1)), "sum": d.sum(rank + 1.5)}}
d.barrier()
d.close()
print(json.dumps(out), flush=True)
"""


def test_dist_reductions_over_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        so, se = p.communicate(timeout=300)
        assert p.returncode == 0, se
        outs.append(json.loads([ln for ln in so.splitlines() if ln.startswith("{")][-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["max"] == 20.0          # max over ranks of 10 (rank + 1)
        assert o["sum"] == 1.5 + 2.5     # sum over ranks of rank + 1.5
    assert sorted(o["rank"] for o in outs) == [0, 1]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "1", "--warmup", "0", "--cpu-nel", "8"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
