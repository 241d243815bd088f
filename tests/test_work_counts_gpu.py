"""The YZ stage's device work counters (or_yz_work_counts) against the
oracle's counts in the reference's enumeration (orc_run_all_counted): the
combinations that reach the first y fit (reconstruction_kernels.cuh:1602)
and those that pass its 2-sigma cut (:1611).  The bench's combinations/s and
operation counts come from these counters."""
import numpy as np
import pytest

from helpers import mixed_events

pytestmark = pytest.mark.gpu


def test_yz_work_counts_equal_the_oracles(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle as O
    from orgpu import layout as L, pipeline
    plane, wp = geometry
    _, _, _, hits = mixed_events(plane, wp, 200, 300, seed=41)
    st = O.OracleState(hits.n)
    O.run_all(plane, hits.copy(), L.HostTracks(hits.n), st, counted=True)
    c = st.counts.reshape(hits.n, O.NCOUNTS)
    want_fitted, want_surv = int(c[:, 3].sum()), int(c[:, 4].sum())
    assert want_fitted > 10000 and want_surv > 100
    rc = pipeline.Reconstruction(plane, 0)
    rc.set_yz_work_counting(True)
    for shape in (1, 4, 16):  # every launch shape counts the same work
        from orgpu import _lib
        rc.lib.or_set_launch(rc.ctx, _lib.KERNELS["yz"], shape)
        b = pipeline.DeviceBatch(hits.n, 0)
        b.upload_hits(hits)
        rc.run_batch(b)
        rc.sync()
        fitted, hitsum, surv = rc.yz_work_counts()
        assert (fitted, surv) == (want_fitted, want_surv), shape
        assert 4 * fitted <= hitsum <= 8 * fitted
    # counting off: the counters stay at zero
    rc.set_yz_work_counting(False)
    b = pipeline.DeviceBatch(hits.n, 0)
    b.upload_hits(hits)
    rc.run_batch(b)
    rc.sync()
    assert rc.yz_work_counts() == (0, 0, 0)
    rc.close()
