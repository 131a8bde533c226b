"""The multi-process path on CPU: bench.py's Dist helper over gloo with two
ranks (barrier, max and sum as the bench uses them: the max of the ranks'
times, the sum of their work), and the window partition every rank computes
for the batched configuration (independent windows, no exchange)."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from zeroslam_gb300 import ba, scenes

    d = bench.Dist()
    d.barrier()
    mx = d.max(float(rank + 1))
    sm = d.sum(float(10 * (rank + 1)))
    wins = scenes.window_batch(24, seed=5)
    parts = ba.partition_windows(wins, world)
    mine = parts[rank]
    done = d.sum(float(len(mine)))
    d.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{mx} {sm} {done} {','.join(map(str, mine))}\n")
    d.pg.destroy_process_group()


def test_dist_two_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    for attempt in range(3):  # a port taken between the probe and the rendezvous: try another
        try:
            mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                               start_method="spawn")
            break
        except Exception:
            if attempt == 2:
                raise
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(2)]
    for mx, sm, done, _ in rows:
        assert float(mx) == 2.0 and float(sm) == 30.0 and float(done) == 24.0
    a = [int(x) for x in rows[0][3].split(",")]
    b = [int(x) for x in rows[1][3].split(",")]
    assert sorted(a + b) == list(range(24)) and not set(a) & set(b)


def test_partition_windows_balanced():
    sys.path.insert(0, ROOT)
    from zeroslam_gb300 import ba, scenes

    wins = scenes.window_batch(64, seed=7)
    cost = [w.M + (6 * w.K) ** 3 for w in wins]
    for parts in (1, 2, 3, 8):
        p = ba.partition_windows(wins, parts)
        assert sorted(i for q in p for i in q) == list(range(64))
        loads = [sum(cost[i] for i in q) for q in p]
        assert max(loads) - min(loads) <= max(cost)  # greedy largest-first bound
        assert p == ba.partition_windows(wins, parts)  # deterministic
