"""SHT-only mode with the reference's GPU_SHTns_transformer surface
(cunusht/sht/GPU_sht_transformer.py:11-127), every method called with the
reference's positional arguments, against the FP64 direct-sum oracle:

  synthesis(gclm, lmax, mmax)                       flattened theta-contiguous map
  synthesis_cupy(gclm, out, lmax, mmax)             (nphi, nlat) map
  adjoint_synthesis_cupy(synthmap, gclm, lmax, mmax, iw=1/w)   unweighted adjoint
  synthesis_der1(gclm, out)                         flattened theta-contiguous gradient
  synthesis_der1_cupy(gclm, out_theta, out_phi)     ring-major gradient
  analysis / adjoint_synthesis / map2alm / alm2map  SHTns analys / synth

Tolerances: 1e-11 relative (FP64 transforms, no nuFFT).  On the
Gauss-Legendre grid at the band limit analysis inverts synthesis exactly.
"""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

LMAX = 31


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def ralm(lmax, ncomp, rng, spin=0):
    n = orc.nalm(lmax)
    a = rng.standard_normal((ncomp, n)) + 1j * rng.standard_normal((ncomp, n))
    a[:, :lmax + 1] = a[:, :lmax + 1].real
    for m in range(lmax + 1):
        b = orc.almidx(lmax, m, m)
        for l in range(m, min(spin, lmax + 1)):
            a[:, b + l - m] = 0
    return a


@pytest.fixture(scope="module")
def S(built_lib):
    import cunusht_gb300 as cu
    return cu.get_transformer("GPU", "shtns", "SHT")(("gl", {"lmax": LMAX}))


def _theta_contig(S, ring_major):
    """Ring-major (.., nlat * nphi) -> flattened (nphi, nlat)."""
    m = np.asarray(ring_major)
    return np.swapaxes(m.reshape(m.shape[:-1] + (S.nlat, S.nphi)), -1, -2).reshape(m.shape)


def test_layout_attributes(S):
    assert S.theta_contiguous
    assert S.nlat == LMAX + 1 and S.nphi == int(S.geom.nph[0]) >= 2 * LMAX + 1
    assert S.spat_shape == (S.nphi, S.nlat)


def test_synthesis_positional(S):
    a = ralm(LMAX, 1, np.random.default_rng(1))[0]
    th, ph = S.geom.pixels()
    ref = _theta_contig(S, oracle.synth_points_c(LMAX, 0, a, th, ph))
    got = S.synthesis(torch.as_tensor(a, device="cuda"), LMAX, LMAX).cpu().numpy()
    assert got.shape == (S.npix(),)
    assert rel(got, ref) < 1e-11
    out = torch.empty(S.spat_shape, dtype=torch.float64, device="cuda")
    r2 = S.synthesis_cupy(torch.as_tensor(a, device="cuda"), out, LMAX, LMAX)
    assert r2 is out and tuple(out.shape) == S.spat_shape
    assert rel(out.cpu().numpy().reshape(-1), ref) < 1e-11
    assert rel(S.alm2map(torch.as_tensor(a, device="cuda"), lmax=LMAX, mmax=LMAX).cpu().numpy(), ref) < 1e-11


@pytest.mark.parametrize("spin", [0, 2])
def test_analysis_inverts_synthesis(S, spin):
    a = ralm(LMAX, 1 if spin == 0 else 2, np.random.default_rng(2 + spin), spin)
    A = torch.as_tensor(a[0] if spin == 0 else a, device="cuda")
    m = S.synthesis(A, LMAX, LMAX, spin=spin)
    back = S.analysis(m, LMAX, LMAX, spin=spin).cpu().numpy()
    assert back.shape == ((1 if spin == 0 else 2), orc.nalm(LMAX))
    assert rel(back, a) < 1e-11
    # the reference's aliases of analysis: adjoint_synthesis(map) takes a flat
    # map and reshapes it to the spatial grid; map2alm is analysis
    assert rel(S.adjoint_synthesis(m, spin=spin).cpu().numpy(), a) < 1e-11
    assert rel(S.map2alm(m.reshape(-1) if spin == 0 else m, spin=spin).cpu().numpy(), a) < 1e-11
    if spin == 0:  # the spatial (nphi, nlat) shape is accepted as well
        assert rel(S.analysis(m.reshape(S.spat_shape)).cpu().numpy(), a) < 1e-11


def test_adjoint_synthesis_cupy_with_inverse_weights(S):
    """analys(map * iw) with iw = 1 / w per ring is the unweighted adjoint
    synthesis, as the reference's nusht2d1 uses it (GPU_nufft_transformer.py:
    265-269, :483)."""
    rng = np.random.default_rng(4)
    y = rng.standard_normal(S.spat_shape)
    iw = torch.as_tensor(1.0 / S.geom.weight, device="cuda")      # (nlat,), broadcast over nphi
    got = S.adjoint_synthesis_cupy(torch.as_tensor(y, device="cuda"), None, LMAX, LMAX, iw=iw).cpu().numpy()
    th, ph = S.geom.pixels()
    ring_major = np.swapaxes(y, 0, 1).reshape(-1)
    want = oracle.adjoint_synth_points_c(LMAX, 0, ring_major, th, ph, ncomp=1)
    assert got.shape == (orc.nalm(LMAX),)
    assert rel(got, np.reshape(want, -1)) < 1e-11


def test_synthesis_der1_layouts(S):
    """synth_grad: (d/dtheta, 1/sin(theta) d/dphi), the spin-1 synthesis of
    sqrt(l(l+1)) a_lm; theta-contiguous from synthesis_der1, ring-major from
    synthesis_der1_cupy (the reference's .T.flatten())."""
    a = ralm(LMAX, 1, np.random.default_rng(5))[0]
    th, ph = S.geom.pixels()
    ll = np.arange(LMAX + 1)
    ref = oracle.synth_points_c(LMAX, 1, orc.almxfl(a, np.sqrt(ll * (ll + 1.0)), LMAX)[None], th, ph)
    A = torch.as_tensor(a, device="cuda")
    got_tc = S.synthesis_der1(A, None).cpu().numpy()
    assert got_tc.shape == (2, S.npix())
    assert rel(got_tc, _theta_contig(S, ref)) < 1e-11
    ot = torch.empty(S.npix(), dtype=torch.float64, device="cuda")
    op = torch.empty(S.npix(), dtype=torch.float64, device="cuda")
    got_rm = S.synthesis_der1_cupy(A, ot, op).cpu().numpy()
    assert rel(got_rm, ref) < 1e-11
    assert rel(np.stack([ot.cpu().numpy(), op.cpu().numpy()]), ref) < 1e-11
