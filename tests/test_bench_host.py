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
