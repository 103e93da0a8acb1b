"""The multi-rank host path of bench.py on CPU (no GPU): one process per rank, as torchrun launches it.

With one GPU per rank the bench runs independent replicas of the step (the path has no exchange), so
the only cross-rank work is the barrier and the maximum of each timed figure over the ranks; that
reduction runs here over `gloo` at world size 2.  The reference arm under torchrun prints its line
from rank 0 alone, and the other rank exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK_SCRIPT = """
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
dist.init_process_group("gloo", init_method="env://")
import bench
r = dist.get_rank()
print("MAX", bench.rank_max(1.5 + r, "cpu"), "ONE", bench.rank_max(7.0, "cpu"), flush=True)
dist.barrier()
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_rank_max_over_two_gloo_ranks():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r), WORLD_SIZE="2",
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT.format(root=ROOT)], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=240) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
        line = [ln for ln in o.splitlines() if ln.startswith("MAX")][0].split()
        assert float(line[1]) == 2.5 and float(line[3]) == 7.0


def test_rank_max_without_a_process_group_is_the_value():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_max(3.25, "cpu") == 3.25


def test_reference_arm_under_torchrun_prints_from_rank_zero_only():
    # the launcher's own option parser takes "--n..." prefixes, so the default N = 1,048,576 is used (a
    # 32-target sample per step)
    port = _free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3", "--ref-targets", "32"],
                       capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
