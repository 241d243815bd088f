"""Launch shapes change timing only: the whole chain with every events-per-CTA
choice gives the oracle's result bit for bit, and the autotuner returns and
applies a shape for every stage."""
import numpy as np
import pytest

from helpers import Snapshots, hit_mismatches, mixed_events, track_mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import pipeline
    plane, wp = geometry
    geo, rec, off, hits0 = mixed_events(plane, wp, 120, 120, seed=41)
    return plane, hits0, Snapshots(plane, hits0), pipeline.Reconstruction(plane, 0)


@pytest.mark.parametrize("warps", [1, 2, 8, 16])
def test_every_launch_shape_gives_the_same_result(env, warps):
    from orgpu import autotune, pipeline
    plane, hits0, snap, rc = env
    for k in autotune.STAGES:
        autotune.set_launch(rc, k, min(warps, 8) if k == "xz" else warps)
    b = pipeline.DeviceBatch(hits0.n)
    b.upload_hits(hits0)
    rc.run_batch(b)
    rc.selection(b)
    rc.sync()
    np.testing.assert_array_equal(b.toomany.cpu().numpy(), snap.state.toomany)
    assert hit_mismatches(b.download_hits(), snap.hits_er) == []
    assert track_mismatches(b.download_tracks(), snap.tracks_sel, snap.state.toomany) == []
    for k in autotune.STAGES:
        autotune.set_launch(rc, k, 4)


def test_tuner_picks_a_shape_per_stage(env):
    from orgpu import _lib, autotune
    plane, hits0, snap, rc = env
    cfg = autotune.tune(rc, hits0, candidates=(2, 4, 8), repeats=1)
    assert set(cfg["best"]) == set(autotune.STAGES)
    for k, w in cfg["best"].items():
        assert autotune.get_launch(rc, k) == w
    assert rc.lib.or_set_launch(rc.ctx, _lib.KERNELS["xz"], 16) == _lib.OR_ERR_ARG
    for k in autotune.STAGES:
        autotune.set_launch(rc, k, 4)
