"""The N > 1 path on CPU: bench.py's rank helpers over a world-size-2 gloo
group (barrier, max over ranks, sum over ranks), and the reference arm under
two ranks (rank 0 alone measures and prints; rank 1 exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank: int, world: int, port: int) -> dict:
    env = dict(os.environ)
    env.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1",
                "MASTER_PORT": str(port), "PYTHONPATH": ROOT})
    return env


RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
d = bench.Dist()
d.barrier()
r = d.rank
out = {"rank": r, "world": d.world, "max": d.max(10.0 + r), "sum": d.sum(100 * (r + 1))}
d.barrier()
print(json.dumps(out))
"""


def test_rank_helpers_world2():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=_env(r, 2, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda x: x["rank"])
    for x in res:
        assert x["world"] == 2
        assert x["max"] == 11.0  # the slower rank sets the step time
        assert x["sum"] == 300.0  # items of all ranks count toward the value


def test_reference_arm_two_ranks():
    pytest.importorskip("numpy")
    from oracle import c_oracle  # noqa: F401  (builds / loads the C oracle)

    port = _free_port()
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--n", "1024", "--cpu-seconds", "0.5"]
    procs = [subprocess.Popen(cmd, env=_env(r, 2, port), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, cwd=ROOT)
             for r in range(2)]
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    lines0 = [l for l in outs[0][0].splitlines() if l.strip()]
    assert len(lines0) == 1
    line = json.loads(lines0[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    assert not [l for l in outs[1][0].splitlines() if l.strip()]  # rank 1 prints nothing
