"""Host-side logic of bench.py that needs no GPU: which recorded reference iteration counts
the CPU arm is scored on."""
import bench


def test_reference_window_takes_the_timed_steps():
    rec = {"iters": [0, 10, 20, 30, 40, 50]}  # steps 1..6; step 1 has no solve
    want, beyond = bench.reference_window_iters(rec, warmup=3, steps=2)
    assert want == [30, 40] and beyond == 0  # steps 4 and 5


def test_reference_window_beyond_the_record_uses_the_solve_mean():
    rec = {"iters": [0, 10, 20, 30]}
    want, beyond = bench.reference_window_iters(rec, warmup=2, steps=4)
    assert want[:2] == [20, 30] and want[2:] == [20.0, 20.0] and beyond == 2


def _replica(rank, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank), BENCH_GLOO="1")
    import bench as b
    d = b.Dist()
    d.barrier()
    t = d.max(10.0 + rank)  # each rank's timed region; the line reports the slowest
    d.barrier()
    d.close()
    q.put((rank, d.world, t))


def test_replicas_report_the_slowest_rank_gloo():
    """`bench.py --gpus 2` runs independent replicas: the barrier and the max over ranks
    of the timed region, on two gloo ranks (CPU)."""
    import multiprocessing as mp
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica, args=(r, port, q)) for r in (0, 1)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 11.0), (1, 2, 11.0)]


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.main(["--impl", "reference"]) == 0
    assert capsys.readouterr().out == ""
