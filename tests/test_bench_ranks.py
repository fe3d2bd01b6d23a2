"""The bench's multi-rank logic on CPU: two gloo ranks run the same Ranks
object the GPU arms use (barriers around the timed region, the slowest
rank's time by all_reduce MAX, whole-job rate = all ranks' units over that
time). The projection shards into independent replicas, so this is the
only cross-rank traffic a multi-GPU bench run has."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys, time
sys.path.insert(0, sys.argv[1])
import bench
r = bench.Ranks("gloo")
r.barrier()
t0 = time.perf_counter()
time.sleep(0.05 * (r.rank + 1))      # rank 1 is the slower replica
r.barrier()
ms_local = 100.0 if r.rank == 0 else 250.0
out = {"rank": r.rank, "world": r.world, "max_ms": r.max_ms(ms_local),
       "rate": r.rate(10, ms_local), "wall_ms": 1000.0 * (time.perf_counter() - t0)}
r.close()
print(json.dumps(out), flush=True)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(world):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            so, se = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, se
        outs.append(json.loads(so.strip().splitlines()[-1]))
    return sorted(outs, key=lambda o: o["rank"])


def test_two_gloo_ranks_take_slowest_time_and_sum_units():
    outs = _run_ranks(2)
    assert [o["rank"] for o in outs] == [0, 1]
    for o in outs:
        assert o["world"] == 2
        assert o["max_ms"] == 250.0                     # slowest rank's time on every rank
        assert abs(o["rate"] - 2 * 10 / 0.25) < 1e-9    # 20 units over 0.25 s
    # the closing barrier holds the faster rank until the slower one is done
    assert outs[0]["wall_ms"] >= 95.0


def test_single_rank_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("RANK", "0")
    r = bench.Ranks("gloo")
    r.barrier()
    assert r.max_ms(40.0) == 40.0
    assert abs(r.rate(4, 40.0) - 100.0) < 1e-12
    r.close()
