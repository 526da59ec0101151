"""Host-side logic of bench.py that needs no GPU: which recorded reference iteration counts
the CPU arm is scored on."""
import json

import pytest

import bench


def test_reference_window_takes_the_timed_steps():
    rec = {"iters": [0, 10, 20, 30, 40, 50]}  # steps 1..6; step 1 has no solve
    assert bench.reference_window_iters(rec, warmup=3, steps=2) == [30, 40]  # steps 4 and 5
    assert bench.reference_window_iters(rec, warmup=3, steps=3) == [30, 40, 50]


def test_reference_window_beyond_the_record_is_refused():
    """Nothing is imputed: a timed window past the recorded run makes the arm unavailable."""
    rec = {"iters": [0, 10, 20, 30]}
    with pytest.raises(ValueError, match="lacks 2 recorded steps"):
        bench.reference_window_iters(rec, warmup=2, steps=4)


def test_committed_record_covers_the_default_and_the_twenty_step_windows():
    """The reference's own recorded run spans the windows the bench times by default (3
    warm-up steps, 10 timed) and with 5 warm-up steps and 20 timed, each solve to 1e-8."""
    rec = bench.reference_iteration_record("c2")
    assert rec["tol"] == 1e-8 and len(rec["iters"]) >= 25
    for warmup, steps in ((3, 10), (5, 20)):
        its = bench.reference_window_iters(rec, warmup=warmup, steps=steps)
        assert len(its) == steps and all(n > 0 for n in its)
    assert all(r < 1e-8 for r in rec["relres"][1:])


def test_reference_arm_unavailable_when_the_record_is_short(capsys, monkeypatch):
    monkeypatch.setattr(bench, "reference_iteration_record", lambda wl: {"iters": [0, 1, 2]})
    assert bench.main(["--impl", "reference", "--steps", "20", "--warmup", "5"]) == 0
    line = json.loads(capsys.readouterr().out)
    assert line["impl"] == "reference" and "lacks 22 recorded steps" in line["unavailable"]


def test_both_arms_print_the_same_config():
    a = bench.bench_config("c2", 5000, 1)
    assert a == bench.bench_config("c2", 5000, 1)
    assert {"workload", "nx", "solver", "tol", "maxit", "bc", "parallelism", "l2"} <= set(a)


def test_solve_record_counts_capped_and_unconverged_solves():
    from types import SimpleNamespace as S
    st = [S(step=1, iters=0, relres=0.0, status=0), S(step=2, iters=900, relres=5e-9, status=0),
          S(step=3, iters=5000, relres=3e-8, status=-3), S(step=4, iters=1200, relres=1e-8, status=0)]
    r = bench.solve_record(st, 1e-8)
    assert r["capped_solves"] == 1 and r["unconverged_solves"] == 2
    assert r["iters"] == [0, 900, 5000, 1200] and r["status"] == [0, 0, -3, 0]


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


def test_step_kernel_roofline_names_the_bound():
    """Each MIXED step kernel against both measured roofs: a kernel whose FP64 instruction
    rate is the larger fraction is FP64-bound, else HBM-bound; correct64's two launches
    count as one pass, mirror32 runs over the padded field."""
    cells, npad = 1_000_000, 1_200_000
    fp = {"fp64_tflops": 1.0}  # 5e11 FMA instructions per second
    prof = {"residual64": (2 * 0.1, 2),  # 100 us a launch
            "mirror32": (0.05, 1), "correct64": (0.1, 4)}
    r = bench.step_roofline(prof, cells, npad, 5000.0, fp)
    res = r["residual64"]
    nbytes, ninst = bench.STEP_KERNELS["residual64"]
    assert res["avg_launch_us"] == 100.0
    assert res["achieved_gbs"] == round(nbytes * cells / 1e-4 / 1e9, 1)
    assert res["fp64_frac"] == round(ninst * cells / 1e-4 / 5e11, 4) and res["bound"] == "fp64"
    assert r["mirror32"]["achieved_gbs"] == round(36 * npad / 5e-5 / 1e9, 1) and r["mirror32"]["bound"] == "hbm"
    assert r["correct64"]["launches"] == 2 and r["correct64"]["avg_launch_us"] == 50.0
    assert "update_uf" not in r
