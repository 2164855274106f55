"""The N > 1 path of bench.py on the CPU: world-size-2 gloo ranks run the
host logic of the replica benchmark (barrier, max over ranks, whole-job
throughput) and the reference arm's rank-0-only rule."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        ms = 100.0 + 50.0 * rank            # rank 1 is the slow one
        value, ms_max = bench.replica_throughput(d, cells=1000, steps=4, ms=ms)
        with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
            f.write(f"{value} {ms_max}")
    finally:
        d.close()


def test_two_gloo_ranks_replica_throughput(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        value, ms_max = (float(x) for x in (tmp_path / f"r{r}.txt").read_text().split())
        assert ms_max == 150.0
        assert value == pytest.approx(2 * 1000 * 4 / 0.150 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench

    class FakeDist:
        rank, world, local = 1, 2, 1

    # rank 1 returns before any work (and prints nothing)
    assert bench.run_reference(object(), FakeDist()) is None
