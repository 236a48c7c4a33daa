"""Parity-split long transforms (lmax > 2047, rings > 4096 pixels): the split
form of every transform -- theta / phi passes forward and adjoint, Bluestein
ring synthesis and its adjoint -- forced at small sizes agrees with the
direct form, and an lmax 4095 / nphi 8191 lensing solve (spin 2, epsilon
1e-5, FP32 grid) agrees with the FP64 direct-sum oracle at sampled pixels."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pair(cu, lmax, eps, precision, nphi=None):
    gi = {"lmax": lmax} if nphi is None else {"lmax": lmax, "nphi": nphi}
    a = cu.get_transformer("GPU")(("gl", gi), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    b = cu.get_transformer("GPU")(("gl", gi), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    from cunusht_gb300 import _lib
    _lib.check(b._lib.cunusht_plan_force_split(b._plan, 1))
    return a, b


def _rel(x, y):
    x, y = x.cpu().numpy(), y.cpu().numpy()
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


@pytest.mark.parametrize("precision,eps,tol", [("fp64", 1e-10, 1e-12), ("mixed", 1e-7, 5e-8),
                                               ("mixed", 1e-5, 2e-6)])
@pytest.mark.parametrize("spin", [0, 2])
def test_split_transforms_match_direct(built_lib, precision, eps, tol, spin):
    import cunusht_gb300 as cu
    lmax = 127
    a, b = _pair(cu, lmax, eps, precision)
    gclm, dls = orc.make_inputs(lmax, spin, seed=21)
    g = torch.as_tensor(gclm if spin else gclm[0], device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    # lensing (dlm2pointing with the ring transform, theta / phi forward passes, interp)
    ra = a.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0)
    rb = b.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0)
    assert _rel(rb, ra) < tol
    # adjoint (spread, phi / theta adjoint passes)
    m = torch.as_tensor(np.random.default_rng(3).standard_normal(tuple(ra.shape)), device="cuda")
    aa = a.lenmap2gclm(m, d, None, lmax, lmax, spin=spin, verbose=0)
    ab = b.lenmap2gclm(m, d, None, lmax, lmax, spin=spin, verbose=0)
    assert _rel(ab, aa) < tol


def test_split_ring_transforms_match_direct(built_lib):
    """SHT-only synthesis / adjoint synthesis (Bluestein ring transforms, FP64)
    on a ring length with N < Mb/2 (nphi 255, Mb 512) and spin 0, 1, 2."""
    import cunusht_gb300 as cu
    lmax = 100
    for spin in (0, 1, 2):
        a, b = _pair(cu, lmax, 1e-10, "fp64", nphi=255)
        gclm, _ = orc.make_inputs(lmax, 2, seed=5)
        alm = torch.as_tensor(gclm[:1] if spin == 0 else gclm, device="cuda")
        ma = a.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax)
        mb = b.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax)
        assert _rel(mb, ma) < 1e-12
        y = torch.as_tensor(np.random.default_rng(9).standard_normal(tuple(ma.shape)), device="cuda")
        ya = a.adjoint_synthesis(y, spin=spin, lmax=lmax, mmax=lmax)
        yb = b.adjoint_synthesis(y, spin=spin, lmax=lmax, mmax=lmax)
        assert _rel(yb, ya) < 1e-12


def test_lmax4095_spin2_fp32_lensing_against_oracle(built_lib):
    """lmax 4095, GL 4096 x 8191 (prime ring length: Bluestein 16384 split),
    theta / phi fine transforms of 16384 points split; epsilon 1e-5."""
    import oracle
    import cunusht_gb300 as cu
    lmax, spin, nphi = 4095, 2, 8191
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=2, epsilon=1e-5,
                                  precision="auto", max_spin=2)
    assert T.info["ntheta_fine"] == 16384
    gclm, dls = orc.make_inputs(lmax, spin, seed=31, curl=True)
    g = torch.as_tensor(gclm, device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    c = torch.as_tensor(dls[1], device="cuda")
    out = T.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, dclm_scaled=c, spin=spin, verbose=0).cpu().numpy()
    th, ph = T.geom.pixels()
    idx = np.random.default_rng(2).choice(th.size, 24, replace=False)
    ll = np.arange(lmax + 1)
    fl = np.sqrt(ll * (ll + 1.0))
    dl = np.stack([orc.almxfl(dls[0], fl, lmax), orc.almxfl(dls[1], fl, lmax)])
    dd = oracle.synth_points_c(lmax, 1, dl, th[idx], ph[idx])
    rt, rp = orc.pointing(th[idx], ph[idx], dd[0], dd[1])
    v = oracle.synth_points_c(lmax, spin, gclm, rt, rp)
    z = (v[0] + 1j * v[1]) * np.exp(1j * spin * orc.rotation_gamma(th[idx], dd[0], dd[1]))
    ref = np.stack([z.real, z.imag])
    err = np.linalg.norm(out[:, idx] - ref) / np.linalg.norm(ref)
    assert err < 1e-4, err
