"""FP32 error of the fit parameters against the FP64 oracle (the same chain
with double fits, residuals and chi2 sums; tests/fp64_report.py prints the
full table).  The plain path is bit-exact with the float oracle, so these
are its errors.  The normal equations of the straight-line fits (sums of w,
w z, w z^2 with z ~ 1e3 cm) lose about seven digits in FP32, so the bounds
are those of the reference's own FP32 arithmetic, asserted to catch
regressions."""
import numpy as np


def test_fp32_fit_error_against_fp64_oracle():
    import fp64_report as F
    from orgpu import synth as S
    r = F.fp64_errors(S.config_small(400, 906021))
    assert r["compared"] >= 0.9 * r["global_tracks_fp32"] > 300
    assert r["x0"]["median"] < 1e-5 and r["tx"]["median"] < 1e-5
    assert r["ty"]["median"] < 1e-4 and r["y0"]["median"] < 1e-3
    assert r["invP"]["median"] < 1e-3 and r["chi2"]["median"] < 1e-2
    assert r["x0"]["abs_p99"] < 0.01 and r["y0"]["abs_p99"] < 0.1  # cm
