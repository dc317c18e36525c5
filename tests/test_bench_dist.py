"""bench.py's multi-rank helpers over a 2-rank gloo group on CPU: replicas
agree on the barrier and report the maximum time over ranks."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
class A: pass
a = A(); a.world = int(os.environ["WORLD_SIZE"])
bench.barrier(a)
v = bench.max_over_ranks(a, 1.0 + int(os.environ["RANK"]))
print("RESULT", v, flush=True)
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_max(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(WORKER % ROOT)
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    assert all(p.returncode == 0 for p in procs)
    vals = [float(o.split("RESULT")[1]) for o in outs]
    assert vals == [2.0, 2.0]
