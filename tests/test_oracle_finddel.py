"""findDelAuto restatement (findDel/findDelAuto.m, interpTrajTime.m) and the product's
host-side pieces (modified Akima resampling, derivative kernel) on the CPU."""
import numpy as np
import pytest

from oracle.finddel_ref import deriv_same, find_del_auto, interp_traj_time


def test_makima_matches_scipy_modified_akima():
    from matmri_gb300.finddel import makima
    from scipy.interpolate import Akima1DInterpolator
    rng = np.random.default_rng(0)
    for n in (2, 3, 4, 7, 40):
        x = np.sort(rng.uniform(0, 10, n))
        y = rng.standard_normal((n, 3))
        if n >= 7:
            y[2:6] = 0.5                                   # a constant run: both weights vanish
        xq = np.linspace(x[0] - 1, x[-1] + 1, 301)
        got = makima(x, y, xq)
        if n == 2:
            ref = np.interp(xq, x, y[:, 0])[:, None] * np.ones((1, 3))
            ref = np.where(np.isnan(got), np.nan, (y[0] + (xq[:, None] - x[0]) * (y[1] - y[0]) / (x[1] - x[0])))
        else:
            ref = Akima1DInterpolator(x, y, method="makima", extrapolate=False)(xq)
        np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))        # NaN outside the nodes
        np.testing.assert_allclose(got[~np.isnan(got)], ref[~np.isnan(ref)], rtol=0, atol=1e-12)


def test_interp_traj_time_and_derivative_kernel():
    from matmri_gb300.finddel import _conv_same, DERIV_KERNEL, interpTrajTime
    tr = np.stack([np.arange(50.0), np.arange(50.0) ** 2], axis=1)
    dt = np.array([3.0, 10.5, 20.25])
    a, _ = interpTrajTime(tr, None, 0.5, 1.5, dt)          # trajectory time -1.5 + 0.5 n
    np.testing.assert_allclose(a[:, 0], (dt + 1.5) / 0.5, atol=1e-12)
    b, _ = interp_traj_time(tr, None, 0.5, 1.5, dt)
    np.testing.assert_allclose(a, b, atol=1e-10)
    a, _ = interpTrajTime(tr, None, 0.5, 0.0, np.array([-0.1, 30.0]))
    assert np.isnan(a[0]).all() and np.isnan(a[1]).all()    # outside the trajectory: NaN (interpTrajTime.m:23)
    d = _conv_same(tr, DERIV_KERNEL) / 0.5
    np.testing.assert_allclose(d[2:-2, 0], 2.0)             # d/dt of n at dwell 0.5
    np.testing.assert_allclose(d, deriv_same(tr, 0.5), atol=1e-12)
    with pytest.raises(ValueError):
        interpTrajTime(None, None, 0.5, 0.0, dt)


def test_find_del_auto_recovers_the_delay():
    from sho_cases import finddel_case
    c = finddel_case(N=16, C=3, M=768, true_delay=0.37, wobble=6.0)
    d, hist = find_del_auto(0.0, c["data"], c["tdwell"], c["traj"], c["conc"], c["datatime"], c["grid"],
                            c["b0"], c["maps"], 15)
    assert abs(d - c["true_delay"]) < 0.05
    assert hist[0] == 0.0 and abs(hist[-1] - hist[-2]) <= 0.005          # stops on |delChange| <= 0.005
