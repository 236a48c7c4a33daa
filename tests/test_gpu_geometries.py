"""Pointing geometries with different ring lengths (cunusht/geometry.py:195-298):
HEALPix (rings of 4 .. 4 nside pixels, shifted first longitudes), the
longitude-thinned Gauss-Legendre grid (rings shorter than 2 lmax + 1 near the
poles) and Fejer-1.  Pointing, synthesis, adjoint synthesis and the lensed
map on each, against the FP64 direct-sum oracle at sampled pixels."""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GEOMS = [("healpix", {"nside": 32, "lmax": 63}, 63), ("thingauss", {"lmax": 127, "smax": 2}, 127),
         ("f1", {"ntheta": 72, "nphi": 137, "lmax": 63}, 63)]


def _pixels(T, n, seed):
    th, ph = T.geom.pixels()
    idx = np.random.default_rng(seed).choice(th.size, min(n, th.size), replace=False)
    return idx, th[idx], ph[idx]


@pytest.mark.parametrize("name,kw,lmax", GEOMS)
def test_pointing_and_synthesis(built_lib, name, kw, lmax):
    import cunusht_gb300 as cu
    T = cu.get_transformer("GPU")((name, dict(kw)), nuFFTtype=2, epsilon=1e-10, precision="fp64", max_spin=2)
    assert len(np.unique(T.geom.nph)) > 1 or name == "f1"
    gclm, dls = orc.make_inputs(lmax, 2, seed=3)
    d = torch.as_tensor(dls[0], device="cuda")
    ptg = T.dlm2pointing(d, lmax).cpu().numpy()
    idx, th, ph = _pixels(T, 300, 1)
    ll = np.arange(lmax + 1)
    dd = oracle.synth_points_c(lmax, 1, orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)[None], th, ph)
    rt, rp = orc.pointing(th, ph, dd[0], dd[1])
    assert np.max(np.abs(ptg[0, idx] - rt)) < 1e-12
    assert np.max(np.abs(np.angle(np.exp(1j * (ptg[1, idx] - rp))))) < 1e-12
    # SHT-only mode: synthesis in the transformer's spatial layout, analysis =
    # adjoint synthesis of the quadrature-weighted map (SHTns analys)
    S = cu.get_transformer("GPU", mode="SHT")((name, dict(kw)))
    th_all, ph_all = S.geom.pixels()
    w = np.repeat(S.geom.weight, S.geom.nph.astype(np.int64))
    for spin in (0, 2):
        alm = torch.as_tensor(gclm[:1] if spin == 0 else gclm, device="cuda")
        m = _ring_major(S, S.synthesis(alm, lmax, lmax, spin=spin).cpu().numpy(), spin)
        ref = oracle.synth_points_c(lmax, spin, gclm[0] if spin == 0 else gclm, th, ph)
        got = m[idx] if spin == 0 else m[:, idx]
        assert np.max(np.abs(got - ref)) < 1e-11 * np.max(np.abs(ref)), (name, spin)
        y = np.random.default_rng(2).standard_normal(m.shape)
        ah = S.analysis(torch.as_tensor(_spatial(S, y, spin), device="cuda"), lmax, lmax, spin=spin).cpu().numpy()
        want = oracle.adjoint_synth_points_c(lmax, spin, y * w, th_all, ph_all, ncomp=1 if spin == 0 else 2)
        assert np.linalg.norm(ah - np.atleast_2d(want)) < 1e-11 * np.linalg.norm(want), (name, spin)


def _ring_major(S, m, spin):
    """Map(s) of the SHT transformer's spatial layout -> ring-major (.., npix)."""
    m = np.asarray(m).reshape((2, -1) if spin else (-1,))
    if not S.theta_contiguous:
        return m
    return np.swapaxes(m.reshape(m.shape[:-1] + (S.nphi, S.nlat)), -1, -2).reshape(m.shape)


def _spatial(S, m, spin):
    """Ring-major (.., npix) -> the SHT transformer's spatial layout, flattened."""
    m = np.asarray(m)
    if not S.theta_contiguous:
        return m
    return np.ascontiguousarray(np.swapaxes(m.reshape(m.shape[:-1] + (S.nlat, S.nphi)), -1, -2)).reshape(m.shape)


@pytest.mark.parametrize("name,kw,lmax", GEOMS)
@pytest.mark.parametrize("precision,eps,tol", [("fp64", 1e-10, 1e-9), ("mixed", 1e-7, 2e-7)])
def test_lensed_map(built_lib, name, kw, lmax, precision, eps, tol):
    import cunusht_gb300 as cu
    T = cu.get_transformer("GPU")((name, dict(kw)), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    gclm, dls = orc.make_inputs(lmax, 2, seed=7)
    out = T.gclm2lenmap(torch.as_tensor(gclm, device="cuda"), lmax, lmax,
                        dlm_scaled=torch.as_tensor(dls[0], device="cuda"), spin=2, verbose=0).cpu().numpy()
    idx, th, ph = _pixels(T, 200, 5)
    ll = np.arange(lmax + 1)
    dd = oracle.synth_points_c(lmax, 1, orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)[None], th, ph)
    rt, rp = orc.pointing(th, ph, dd[0], dd[1])
    v = oracle.synth_points_c(lmax, 2, gclm, rt, rp)
    z = (v[0] + 1j * v[1]) * np.exp(2j * orc.rotation_gamma(th, dd[0], dd[1]))
    ref = np.stack([z.real, z.imag])
    err = np.linalg.norm(out[:, idx] - ref) / np.linalg.norm(ref)
    assert err < tol, (name, precision, err)
