"""Rows past the lensing solve itself: the magnification-matrix determinant
(dlm2A, helper_GPU.py:113-161) and the exact remapping at selected pixels
(gclm2lenpixs, CPU_nufft_transformer.py:531-558), against the FP64 oracle."""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dlm2A_oracle(lmax, dlm, dclm, th, ph):
    """helper_GPU.py:125-161 restated on direct sums at the pixels."""
    ll = np.arange(lmax + 1, dtype=float)
    d2k = 0.5 * np.sqrt(ll * (ll + 1.0))
    d2g = -0.5 * np.sqrt(np.maximum((ll - 1.0) * (ll + 2.0), 0.0))
    k = oracle.synth_points_c(lmax, 0, orc.almxfl(dlm, d2k, lmax), th, ph)
    gc = np.stack([orc.almxfl(dlm, d2g, lmax), orc.almxfl(dclm, d2g, lmax)])
    g1, g2 = oracle.synth_points_c(lmax, 2, gc, th, ph)
    d1, d2 = oracle.synth_points_c(lmax, 1, np.stack([dlm, dclm]), th, ph)
    w = oracle.synth_points_c(lmax, 0, orc.almxfl(dclm, d2k, lmax), th, ph) if np.any(dclm) else 0.0
    d = np.sqrt(d1 * d1 + d2 * d2)
    f0 = np.sin(d) / d
    f1 = np.cos(d) - f0
    A = f0 * ((1.0 - k) ** 2 - g1 * g1 - g2 * g2 + w * w)
    A += f1 * (1.0 - k - ((d1 * d1 - d2 * d2) * g1 + (2 * d1 * d2) * g2) / (d * d))
    return A


@pytest.mark.parametrize("curl", [False, True])
def test_dlm2A_matches_oracle(built_lib, curl):
    import cunusht_gb300 as cu
    from cunusht_gb300.helper import dlm2A
    lmax = 127
    _, dls = orc.make_inputs(lmax, 0, seed=13, curl=True, rms_arcmin=30.0)
    ll = np.arange(lmax + 1)
    fl = np.sqrt(ll * (ll + 1.0))
    dlm = orc.almxfl(dls[0], fl, lmax)
    dclm = orc.almxfl(dls[1], fl, lmax) if curl else np.zeros_like(dlm)
    A = dlm2A(torch.as_tensor(dlm, device="cuda"), lmax, lmax, ("gl", {"lmax": lmax}), 4,
              dclm=torch.as_tensor(dclm, device="cuda") if curl else None).cpu().numpy()
    th, ph = cu.get_geom(("gl", {"lmax": lmax})).pixels()
    idx = np.random.default_rng(3).choice(th.size, 300, replace=False)
    ref = _dlm2A_oracle(lmax, dlm, dclm, th[idx], ph[idx])
    assert np.max(np.abs(A[idx] - ref)) < 1e-12 * np.max(np.abs(ref))
    assert abs(np.mean(A) - 1.0) < 0.05  # a magnification matrix close to the identity


@pytest.mark.parametrize("spin", [0, 2])
def test_gclm2lenpixs_is_exact_and_matches_lensed_map(built_lib, spin):
    import cunusht_gb300 as cu
    lmax = 127
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-10, precision="fp64")
    gclm, dls = orc.make_inputs(lmax, spin, seed=17)
    g = torch.as_tensor(gclm if spin else gclm[0], device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    lenmap = T.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0).cpu().numpy()
    pixs = np.random.default_rng(4).choice(T.npix(), 64, replace=False)
    got = T.gclm2lenpixs(g, lmax, spin, pixs)
    got = np.stack([x.cpu().numpy() for x in got]) if spin else got.cpu().numpy()
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    dd = oracle.synth_points_c(lmax, 1, orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)[None], th[pixs], ph[pixs])
    rt, rp = orc.pointing(th[pixs], ph[pixs], dd[0], dd[1])
    ref = oracle.synth_points_c(lmax, spin, gclm if spin else gclm[0], rt, rp)
    if spin:
        z = (ref[0] + 1j * ref[1]) * np.exp(1j * spin * orc.rotation_gamma(th[pixs], dd[0], dd[1]))
        ref = np.stack([z.real, z.imag])
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) < 1e-12 * scale              # exact direct sum
    sel = lenmap[:, pixs] if spin else lenmap[pixs]
    assert np.max(np.abs(sel - got)) < 1e-9 * scale               # the nuFFT map at eps 1e-10


@pytest.mark.parametrize("precision,eps", [("fp64", 1e-10), ("mixed", 1e-7)])
@pytest.mark.parametrize("spin", [0, 2])
def test_mmax_below_lmax(built_lib, precision, eps, spin):
    """alm truncated at mmax < lmax (healpy layout) give the lensed map, its
    adjoint and the exact point synthesis of the full layout with the m > mmax
    coefficients zeroed."""
    import cunusht_gb300 as cu
    from cunusht_gb300.utils import Alm
    lmax, mmax = 127, 90
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    gclm, dls = orc.make_inputs(lmax, spin, seed=21)
    n = Alm.getsize(lmax, mmax)
    g = gclm.copy()
    g[:, n:] = 0.0
    d = dls[0].copy()
    d[n:] = 0.0
    gf = torch.as_tensor(g if spin else g[0], device="cuda")
    gt = torch.as_tensor(g[:, :n] if spin else g[0, :n], device="cuda")
    df, dt = torch.as_tensor(d, device="cuda"), torch.as_tensor(d[:n], device="cuda")
    ref = T.gclm2lenmap(gf, lmax, lmax, dlm_scaled=df, spin=spin, verbose=0).clone()
    got = T.gclm2lenmap(gt, lmax, mmax, dlm_scaled=dt, spin=spin, verbose=0)
    assert T.nalm == n
    scale = float(torch.max(torch.abs(ref)))
    assert float(torch.max(torch.abs(got - ref))) <= 1e-12 * scale
    # adjoint: the truncated output is the head of the full one
    y = torch.as_tensor(np.random.default_rng(4).standard_normal(tuple(ref.shape)), device="cuda")
    a_t = T.lenmap2gclm(y, dt, None, lmax, mmax, spin=spin, verbose=0).cpu().numpy()
    a_f = T.lenmap2gclm(y, df, None, lmax, lmax, spin=spin, verbose=0).cpu().numpy()
    tol = 1e-12 if precision == "fp64" else 1e-9
    assert np.max(np.abs(a_t - a_f[..., :n])) <= tol * np.max(np.abs(a_f))
    # exact point synthesis with mmax
    pix = np.random.default_rng(5).choice(T.npix(), 16, replace=False)
    T.gclm2lenmap(gt, lmax, mmax, dlm_scaled=dt, spin=spin, verbose=0)
    sp = T.gclm2lenpixs(gt, mmax, spin, pix)
    sp = np.stack([x.cpu().numpy() for x in sp]) if spin else sp.cpu().numpy()
    ptg = T.ptg.cpu().numpy()
    ex = oracle.synth_points_c(lmax, spin, g if spin else g[0], ptg[0, pix], ptg[1, pix])
    if spin:
        z = (ex[0] + 1j * ex[1]) * np.exp(1j * spin * T.gamma.cpu().numpy()[pix])
        ex = np.stack([z.real, z.imag])
    assert np.max(np.abs(sp - ex)) < 1e-12 * np.max(np.abs(ex))
