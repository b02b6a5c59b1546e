"""CPU tests of the multi-GPU form, which is replicas only: `bench.py --gpus N`
runs one independent replica per GPU, joined by a host-side gloo barrier and
max / sum reductions of the timings and path counts (no data-path
collective).  Two ranks on this machine, rendezvous on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, %r)
from bench import Dist
d = Dist()
d.barrier()
out = {"rank": d.rank, "world": d.world,
       "max": d.allreduce(10.0 * (d.rank + 1), "max"), "sum": d.allreduce(d.rank + 1, "sum")}
d.barrier()
d.close()
print(json.dumps(out))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_barrier_and_reductions_world_size_2():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT % ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e[-2000:]
        outs.append(json.loads(o.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["max"] == 20.0 and o["sum"] == 3.0


def test_reference_arm_prints_once_under_two_ranks():
    """`bench.py --impl reference` launched by torchrun with two ranks: rank 0
    alone times the CPU reference and prints one JSON line; rank 1 exits 0
    without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl",
           "reference", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
