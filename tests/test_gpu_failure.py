"""Failure paths that are exercised without faulting the GPU.

The FP32 bulk-copy pipeline bounds every mbarrier wait; a wait that gives up sets the
solver's fault word, the block stops (after its own copies have landed) and the host
returns CFDGB_ECUDA.  The test switch CFDGB_TEST_WAIT_FAULT (read at cfdgb_create) makes
one block of the next pipelined launch announce 16 bytes more than its first plane's
copies bring, with a short wait limit: that wait runs out while every copy issued still
completes.  The context must report the failure and keep working afterwards."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg

pytestmark = pytest.mark.gpu

KW = dict(nx=128, ny=64, nz=16, lx=32.0, ly=16.0, lz=4.0, cx=8.0, cy=8.0, precision="mixed", solver="cg")


def test_pipeline_wait_timeout_is_reported_and_the_context_recovers(monkeypatch):
    monkeypatch.setenv("CFDGB_TEST_WAIT_FAULT", "1")
    s = cg.Solver(**KW)
    monkeypatch.delenv("CFDGB_TEST_WAIT_FAULT")
    with s:
        s.init_fields()
        s.step(1)  # step 1 has no pressure solve
        with pytest.raises(cg.CfdgbError) as e:
            s.step(1)
        assert e.value.status == cg.ECUDA
        assert "bounded wait" in str(e.value)
        # the same context, restarted, steps as a fresh one does
        s.init_fields()
        st = s.step(3)
        f = s.get_fields()
    with cg.Solver(**KW) as ref:
        ref.init_fields()
        st_ref = ref.step(3)
        f_ref = ref.get_fields()
    assert [r.status for r in st] == [0, 0, 0]
    assert [r.cd for r in st] == [r.cd for r in st_ref]
    for k in "uvwp":
        np.testing.assert_array_equal(f[k], f_ref[k])
