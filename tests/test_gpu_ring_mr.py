"""Mixed-radix ring transforms (csrc/ring_mr.cu: one FFT of the ring length
for uniform rings whose length factors into radices <= 13) against the
Bluestein form of the same plan (cunusht_plan_set_ring_transform(plan, 1))
and the FP64 direct-sum oracle:

  * synthesis on the pointing geometry (GPU_nufft_transformer.py:356-367),
    spin 0, 1, 2, FP64 and mixed plans, ring lengths 64, 81, 105, 126, 128
    (radices 4, 9, 3 5 7, 2 7 9, 2 4 4 4);
  * dlm2pointing on the 4095-pixel GL rings of lmax 2047 (radices 5 7 9 13),
    the ring transform of the headline lensing configuration.

Tolerances: the two ring transforms differ only in rounding (1e-12
relative); against the oracle 1e-11 (FP64 plan) and 5e-8 (mixed plan, whose
Legendre stage carries the double-float / tensor-core error).
"""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def _pair(lmax, nphi, precision, eps):
    import cunusht_gb300 as cu
    from cunusht_gb300 import _lib
    mk = lambda: cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=2, epsilon=eps,
                                           precision=precision, max_spin=2)
    a, b = mk(), mk()
    _lib.check(b._lib.cunusht_plan_set_ring_transform(b._plan, 1))
    return a, b


@pytest.mark.parametrize("nphi", [64, 81, 105, 126, 128])
@pytest.mark.parametrize("precision,eps,tol_oracle", [("fp64", 1e-10, 1e-11), ("mixed", 1e-7, 5e-8)])
def test_ring_mr_synthesis_matches_bluestein_and_oracle(built_lib, nphi, precision, eps, tol_oracle):
    lmax = 31
    a, b = _pair(lmax, nphi, precision, eps)
    assert a._lib.cunusht_plan_ring_transform(a._plan) == 0
    assert b._lib.cunusht_plan_ring_transform(b._plan) == 1
    th, ph = a.geom.pixels()
    gclm, _ = orc.make_inputs(lmax, 2, seed=60 + nphi)
    for spin in (0, 1, 2):
        alm = gclm[:1] if spin == 0 else gclm
        A = torch.as_tensor(alm[0] if spin == 0 else alm, device="cuda")
        ma = a.synthesis(A, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
        mb = b.synthesis(A, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
        assert _rel(ma, mb) < 1e-12, (nphi, spin)
        ref = oracle.synth_points_c(lmax, spin, alm[0] if spin == 0 else alm, th, ph)
        assert _rel(ma, ref) < tol_oracle, (nphi, spin, _rel(ma, ref))


def test_ring_lengths_without_small_factors_keep_bluestein(built_lib):
    a, _ = _pair(31, 127, "fp64", 1e-10)  # 127 is prime
    assert a._lib.cunusht_plan_ring_transform(a._plan) == 1


@pytest.mark.parametrize("precision,eps", [("mixed", 1e-7), ("fp64", 1e-10)])
def test_ring_mr_pointing_lmax2047_nphi4095(built_lib, precision, eps):
    """dlm2pointing on GL 2048 x 4095 (the headline geometry): mixed radix
    against Bluestein (deflected angles to 1e-12 relative) and, at 2000
    sampled pixels, against the exact deflection of the oracle."""
    lmax, nphi = 2047, 4095
    a, b = _pair(lmax, nphi, precision, eps)
    assert a._lib.cunusht_plan_ring_transform(a._plan) == 0
    _, dls = orc.make_inputs(lmax, 0, seed=2048)
    d = torch.as_tensor(dls[0], device="cuda")
    pa = a.dlm2pointing(d, lmax).cpu().numpy()
    pb = b.dlm2pointing(d, lmax).cpu().numpy()
    dp = pa - pb
    dp[1] = (dp[1] + np.pi) % (2 * np.pi) - np.pi
    assert np.max(np.abs(dp)) < 1e-12 * np.pi
    th, ph = a.geom.pixels()
    idx = np.sort(np.random.default_rng(7).choice(th.size, 2000, replace=False))
    ll = np.arange(lmax + 1)
    dl = np.stack([orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)])
    dd = oracle.synth_points_c(lmax, 1, dl, th[idx], ph[idx])
    rt, rp = orc.pointing(th[idx], ph[idx], dd[0], dd[1])
    err_t = np.abs(pa[0, idx] - rt)
    err_p = np.abs((pa[1, idx] - rp + np.pi) % (2 * np.pi) - np.pi) * np.sin(rt)
    # against the deflection's size: 1e-7 of it (mixed), 1e-11 (FP64)
    dscale = float(np.sqrt(np.mean(dd[0] ** 2 + dd[1] ** 2)))
    tol = 1e-7 if precision == "mixed" else 1e-11
    assert np.max(err_t) < tol * dscale and np.max(err_p) < tol * dscale, \
        (np.max(err_t) / dscale, np.max(err_p) / dscale)
