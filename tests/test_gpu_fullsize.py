"""Full-size parity of the headline configurations, through the public
transformer (gclm2lenmap = dlm2pointing + nusht2d2, lenmap2gclm =
dlm2pointing + nusht2d1; GPU_nufft_transformer.py:386-673):

  lmax 2047, GL 2048 x 4095, spin 0 and 2, eps 1e-10 (plain FP64) and 1e-7
  (mixed precision), seeded alm / deflection of the headline spectra:
    * lensing against the FP64 CPU restatement of the reference algorithm
      (oracle/fastcpu.c) on the full map, and against exact FP64 direct
      Y_lm sums at 2000 sampled pixels (oracle/direct.c);
    * delensing of a map that is nonzero at 2000 pixels (every one of the
      8.4 M points still goes through the spread) against the exact adjoint
      sums at their deflected positions, rotation included.
  lmax 4095, GL 4096 x 8191, spin 2 with a curl deflection at 10 % of the
  gradient power, complex64 alm in and float32 Q / U out, eps 1e-5: against
  exact direct sums at 2000 sampled pixels (the alm rounded to complex64 as
  the input; float32 output rounding is 6e-8, far below eps).

Tolerance: relative L2 error <= 2 eps for every case.
"""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NSAMPLE = 2000


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _deflected(lmax, dls, th, ph):
    """Exact deflected positions and rotation angles at the given pixels."""
    ll = np.arange(lmax + 1)
    fl = np.sqrt(ll * (ll + 1.0))
    dl = np.stack([orc.almxfl(d, fl, lmax) for d in dls])
    dd = oracle.synth_points_c(lmax, 1, dl, th, ph)
    rt, rp = orc.pointing(th, ph, dd[0], dd[1])
    return rt, rp, orc.rotation_gamma(th, dd[0], dd[1])


class _Case:
    """Inputs and CPU references of one (lmax, spin) configuration, shared by
    the precisions checked against it."""

    def __init__(self, lmax, nphi, spin, seed):
        self.lmax, self.nphi, self.spin = lmax, nphi, spin
        self.gclm, self.dls = orc.make_inputs(lmax, spin, seed=seed)
        from cunusht_gb300.geometry import get_geom
        G = get_geom(("gl", {"lmax": lmax, "nphi": nphi}))
        self.th_all, self.ph_all = G.pixels()
        self.geom = G
        rng = np.random.default_rng(seed + 100)
        self.idx = np.sort(rng.choice(self.th_all.size, NSAMPLE, replace=False))
        th, ph = self.th_all[self.idx], self.ph_all[self.idx]
        self.rt, self.rp, self.gam = _deflected(lmax, self.dls[:1], th, ph)
        g = self.gclm[0] if spin == 0 else self.gclm
        v = oracle.synth_points_c(lmax, spin, g, self.rt, self.rp)
        if spin:
            z = (v[0] + 1j * v[1]) * np.exp(1j * spin * self.gam)
            v = np.stack([z.real, z.imag])
        self.sample_ref = v
        self._full = None
        # delensing: a map nonzero at the sampled pixels only
        self.vals = rng.standard_normal(NSAMPLE if spin == 0 else (2, NSAMPLE))
        w = self.vals
        if spin:
            z = (w[0] + 1j * w[1]) * np.exp(-1j * spin * self.gam)
            w = np.stack([z.real, z.imag])
        self.adj_ref = np.atleast_2d(
            oracle.adjoint_synth_points_c(lmax, spin, w, self.rt, self.rp, ncomp=1 if spin == 0 else 2))

    def full_ref(self):
        if self._full is None:
            fc = oracle.FastCPU(self.lmax, self.geom.theta, self.geom.phi0, self.nphi, 1e-13)
            g = self.gclm if self.spin else self.gclm[:1]
            self._full = fc.lensing(g, self.dls[0], self.spin)
            fc.close()
        return self._full


_cases: dict = {}


def _case(lmax, nphi, spin, seed):
    key = (lmax, nphi, spin, seed)
    if key not in _cases:
        _cases.clear()   # one configuration's references at a time (memory)
        _cases[key] = _Case(lmax, nphi, spin, seed)
    return _cases[key]


@pytest.mark.parametrize("spin", [0, 2])
@pytest.mark.parametrize("precision,eps", [("fp64", 1e-10), ("mixed", 1e-7)])
def test_lmax2047_lensing_full_map_and_direct_sample(built_lib, spin, precision, eps):
    import cunusht_gb300 as cu
    lmax, nphi = 2047, 4095
    C = _case(lmax, nphi, spin, 2047 + spin)
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=2, epsilon=eps,
                                  precision=precision, max_spin=max(spin, 1))
    g = torch.as_tensor(C.gclm[0] if spin == 0 else C.gclm, device="cuda")
    out = T.gclm2lenmap(g, lmax, lmax, dlm_scaled=torch.as_tensor(C.dls[0], device="cuda"), spin=spin,
                        verbose=0).cpu().numpy()
    T._destroy()
    err_sample = rel(out[C.idx] if spin == 0 else out[:, C.idx], C.sample_ref)
    err_full = rel(out, C.full_ref())
    print(f"lmax 2047 spin {spin} {precision} eps {eps}: direct sample {err_sample:.3e}, "
          f"full map vs FP64 CPU port {err_full:.3e}")
    assert err_sample <= 2 * eps, err_sample
    assert err_full <= 2 * eps, err_full


@pytest.mark.parametrize("spin", [0, 2])
@pytest.mark.parametrize("precision,eps", [("fp64", 1e-10), ("mixed", 1e-7)])
def test_lmax2047_delensing_against_exact_adjoint_sums(built_lib, spin, precision, eps):
    import cunusht_gb300 as cu
    lmax, nphi = 2047, 4095
    C = _case(lmax, nphi, spin, 2047 + spin)
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=1, epsilon=eps,
                                  precision=precision, max_spin=max(spin, 1))
    npix = C.th_all.size
    m = np.zeros(npix if spin == 0 else (2, npix))
    if spin:
        m[:, C.idx] = C.vals
    else:
        m[C.idx] = C.vals
    alm = T.lenmap2gclm(torch.as_tensor(m, device="cuda"), torch.as_tensor(C.dls[0], device="cuda"), None,
                        lmax, lmax, spin=spin, verbose=0).cpu().numpy()
    T._destroy()
    err = rel(np.atleast_2d(alm), C.adj_ref)
    print(f"lmax 2047 delensing spin {spin} {precision} eps {eps}: {err:.3e}")
    assert err <= 2 * eps, err


def test_lmax4095_spin2_curl_complex64_float32(built_lib):
    """Config of the large single-precision solve: lmax 4095, complex64 alm,
    float32 Q / U maps, eps 1e-5, gradient + curl (10 % power) deflection."""
    import cunusht_gb300 as cu
    lmax, nphi, spin, eps = 4095, 8191, 2, 1e-5
    gclm, dls = orc.make_inputs(lmax, spin, seed=4095, curl=True)
    g64 = gclm.astype(np.complex64)
    d64 = dls.astype(np.complex64)
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=2, epsilon=eps,
                                  precision="auto", max_spin=2)
    out = T.gclm2lenmap(torch.as_tensor(g64, device="cuda"), lmax, lmax,
                        dlm_scaled=torch.as_tensor(d64[0], device="cuda"),
                        dclm_scaled=torch.as_tensor(d64[1], device="cuda"), spin=spin, verbose=0)
    assert out.dtype == torch.float32 and tuple(out.shape) == (2, T.npix())
    out = out.cpu().numpy().astype(np.float64)
    th_all, ph_all = T.geom.pixels()
    T._destroy()
    idx = np.sort(np.random.default_rng(4096).choice(th_all.size, NSAMPLE, replace=False))
    th, ph = th_all[idx], ph_all[idx]
    rt, rp, gam = _deflected(lmax, d64.astype(np.complex128), th, ph)
    v = oracle.synth_points_c(lmax, spin, g64.astype(np.complex128), rt, rp)
    z = (v[0] + 1j * v[1]) * np.exp(1j * spin * gam)
    err = rel(out[:, idx], np.stack([z.real, z.imag]))
    print(f"lmax 4095 spin 2 curl c64/f32 eps 1e-5: direct sample {err:.3e}")
    assert err <= 2 * eps, err
