"""The damping schedule of the y-line smoothing sweeps (host logic, no GPU).

With the Chebyshev smoother a level's n pre-sweeps take w_k = 1 / theta_k,
theta_k = (hi + lo) / 2 + (hi - lo) / 2 cos((2k - 1) pi / (2n)) the roots of
the degree-n Chebyshev polynomial on [lo, hi] = [cheb_hi / cheb_ratio,
cheb_hi], and its post-sweeps the same in reverse order.  The n sweeps then
multiply the error by prod_k (1 - w_k lambda) on each eigenvalue lambda of
the line-preconditioned operator: the polynomial with the least maximum on
[lo, hi] among those with p(0) = 1, that maximum being 1 / T_n((hi + lo) /
(hi - lo))."""
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi


def _roots(n, hi, ratio):
    lo = hi / ratio
    return np.array([1.0 / ((hi + lo) / 2 + (hi - lo) / 2 * math.cos(math.pi * (2 * k - 1) / (2 * n)))
                     for k in range(1, n + 1)])


@pytest.mark.parametrize("n,hi,ratio", [(3, 2.0, 6.0), (1, 2.0, 6.0), (2, 1.8, 4.0), (5, 2.0, 10.0), (8, 2.2, 30.0)])
def test_chebyshev_schedule(n, hi, ratio):
    p = capi.default_params(nu1=n, nu2=n, cheb_hi=hi, cheb_ratio=ratio)
    assert p.smoother == capi.SMOOTH_CHEBYSHEV
    pre = capi.sweep_damping(p, True, False)
    post = capi.sweep_damping(p, True, True)
    want = _roots(n, hi, ratio)
    assert np.allclose(pre, want, rtol=1e-14, atol=0)
    assert np.array_equal(post, pre[::-1])
    # coarse levels take nu1 / nu2 unless nu1_coarse / nu2_coarse are set
    assert np.array_equal(capi.sweep_damping(p, False, False), pre)
    # minimax: max over [lo, hi] of |prod (1 - w lambda)| is 1 / T_n((hi+lo)/(hi-lo))
    lo = hi / ratio
    lam = np.linspace(lo, hi, 20001)
    poly = np.prod([1.0 - w * lam for w in pre], axis=0)
    tn = math.cosh(n * math.acosh((hi + lo) / (hi - lo)))
    assert abs(np.abs(poly).max() - 1.0 / tn) <= 1e-9 / tn
    assert abs(poly[0]) == pytest.approx(1.0 / tn, rel=1e-12)


def test_coarse_sweep_counts():
    p = capi.default_params(nu1=3, nu2=3, nu1_coarse=5, nu2_coarse=2)
    assert np.allclose(capi.sweep_damping(p, False, False), _roots(5, 2.0, 6.0), rtol=1e-14, atol=0)
    assert np.allclose(capi.sweep_damping(p, False, True), _roots(2, 2.0, 6.0)[::-1], rtol=1e-14, atol=0)


def test_jacobi_schedule():
    p = capi.default_params(smoother="jacobi", omega=0.85, nu1=4, nu2=2)
    assert np.array_equal(capi.sweep_damping(p, True, False), np.full(4, 0.85))
    assert np.array_equal(capi.sweep_damping(p, False, True), np.full(2, 0.85))


@pytest.mark.parametrize("kw", [dict(smoother=2), dict(cheb_ratio=1.0), dict(cheb_hi=0.0), dict(cheb_hi=4.5),
                                dict(nu1=65)])
def test_rejected(kw):
    with pytest.raises(capi.VfsError):
        capi.sweep_damping(capi.default_params(**kw), True, False)


def test_defaults():
    p = capi.default_params()
    assert (p.smoother, p.cheb_hi, p.cheb_ratio, p.nu1, p.nu2, p.nu1_coarse, p.nu2_coarse) == (
        capi.SMOOTH_CHEBYSHEV, 2.0, 6.0, 3, 3, -1, -1)
