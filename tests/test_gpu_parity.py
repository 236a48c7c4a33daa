"""GPU parity tests: every CUDA path through the C ABI against the FP64 oracle.

Tolerances are relative L2 errors, stated per test:
  * exact stages (doubling, pointing): bit-level / 1e-14;
  * FP64 transforms without nuFFT (ring synthesis): 1e-11;
  * nuFFT paths: the requested epsilon.
"""
import numpy as np
import pytest

from oracle import oracle as orc
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def ralm(lmax, ncomp, rng, spin=0):
    n = orc.nalm(lmax)
    a = rng.standard_normal((ncomp, n)) + 1j * rng.standard_normal((ncomp, n))
    a[:, :lmax + 1] = a[:, :lmax + 1].real
    if spin:
        for m in range(lmax + 1):
            b = orc.almidx(lmax, m, m)
            for l in range(m, min(spin, lmax + 1)):
                a[:, b + l - m] = 0
    return a


@pytest.fixture(scope="module")
def cu(built_lib):
    import cunusht_gb300
    return cunusht_gb300


def _T(cu, lmax, eps=1e-10, precision="fp64", nphi=None):
    gi = {"lmax": lmax}
    if nphi is not None:
        gi["nphi"] = nphi
    return cu.get_transformer("GPU")(("gl", gi), nuFFTtype=2, epsilon=eps, precision=precision)


# ------------------------------------------------------------------ doubling
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("spin", [0, 1, 2])
def test_doubling_matches_reference_slicing(built_lib, dtype, spin):
    import ctypes
    from cunusht_gb300 import _lib
    lib = built_lib
    rng = np.random.default_rng(3)
    nt, nphi = 36, 64  # ntheta = (good_size(lmax+2)+3)//4*4 at lmax 31, nphi = 2 good_size(lmax+1)
    ring = rng.standard_normal((nt, nphi)).astype(dtype)
    dt = _lib.F32 if dtype == np.float32 else _lib.F64
    # ring-major (CUdoubling_1D) and theta-contiguous (CUdoubling_contig_1D)
    ref = orc.doubling_ring_major(ring, nt, nphi, spin)
    for layout, inp, want in [(0, ring, ref), (1, ring.T.copy(), ref.T.copy())]:
        x = torch.as_tensor(inp, device="cuda")
        out = torch.empty(want.shape, dtype=x.dtype, device="cuda")
        _lib.check(lib.cunusht_doubling(x.data_ptr(), nt, nphi, layout, spin, dt, out.data_ptr(), None))
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)
    d = rng.standard_normal((2 * nt - 2, nphi)).astype(dtype)
    want = orc.adjoint_doubling_ring_major(d, nt, nphi, spin)
    x = torch.as_tensor(d, device="cuda")
    out = torch.empty((nt, nphi), dtype=x.dtype, device="cuda")
    _lib.check(lib.cunusht_adjoint_doubling(x.data_ptr(), nt, nphi, spin, dt, out.data_ptr(), None))
    torch.cuda.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-6 if dtype == np.float32 else 1e-15, atol=0)


# ------------------------------------------------------------------ pointing
def test_pointing_kernel_matches_formula(built_lib):
    from cunusht_gb300 import _lib
    lmax = 127
    th, ph0, nph, ofs, _ = orc.gl_geometry(lmax)
    tp, pp = orc.geometry_pixels(th, ph0, nph, ofs)
    rng = np.random.default_rng(5)
    dth = rng.standard_normal(tp.size) * 7e-4
    dph = rng.standard_normal(tp.size) * 7e-4
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    T_, P_, N_, O_ = dev(th), dev(ph0), dev(nph.astype(np.int64)), dev(ofs.astype(np.int64))
    A, B = dev(dth), dev(dph)
    ot = torch.empty_like(A)
    op = torch.empty_like(A)
    og = torch.empty_like(A)
    _lib.check(built_lib.cunusht_pointing(th.size, T_.data_ptr(), P_.data_ptr(), N_.data_ptr(), O_.data_ptr(),
                                          tp.size, A.data_ptr(), B.data_ptr(), ot.data_ptr(), op.data_ptr(),
                                          og.data_ptr(), None))
    torch.cuda.synchronize()
    rt, rp = orc.pointing(tp, pp, dth, dph)
    rg = orc.rotation_gamma(tp, dth, dph)
    assert np.max(np.abs(ot.cpu().numpy() - rt)) < 1e-14
    assert np.max(np.abs(op.cpu().numpy() - rp)) < 1e-13
    assert np.max(np.abs(np.angle(np.exp(1j * (og.cpu().numpy() - rg))))) < 1e-12


# ------------------------------------------------------------------ SHT on the ring geometry
@pytest.mark.parametrize("spin,ncomp", [(0, 1), (1, 1), (1, 2), (2, 2)])
@pytest.mark.parametrize("lmax,nphi", [(31, None), (40, 95), (63, 127)])
def test_synthesis_matches_direct_sum(cu, spin, ncomp, lmax, nphi):
    T = _T(cu, lmax, nphi=nphi)
    rng = np.random.default_rng(10 + spin)
    a = ralm(lmax, ncomp, rng, spin)
    th, ph = T.geom.pixels()
    A = a[0] if spin == 0 else a
    got = T.synthesis(torch.as_tensor(A, device="cuda"), spin=spin).cpu().numpy()
    ref = oracle.synth_points_c(lmax, spin, A, th, ph)
    assert rel(got, ref) < 1e-11


@pytest.mark.parametrize("spin,ncomp", [(0, 1), (1, 2), (2, 2)])
def test_adjoint_synthesis_matches_direct_sum(cu, spin, ncomp):
    lmax = 47
    T = _T(cu, lmax)
    rng = np.random.default_rng(20 + spin)
    th, ph = T.geom.pixels()
    v = rng.standard_normal(th.size if spin == 0 else (2, th.size))
    got = T.adjoint_synthesis(torch.as_tensor(v, device="cuda"), spin=spin, ncomp=ncomp).cpu().numpy()
    ref = oracle.adjoint_synth_points_c(lmax, spin, v, th, ph, ncomp=ncomp)
    assert rel(got, ref) < 1e-11


# ------------------------------------------------------------------ nusht2d2 / nusht2d1
def _random_loc(n, rng):
    loc = rng.uniform(0.0, 1.0, (n, 2))
    loc[:, 0] = np.arccos(1 - 2 * loc[:, 0])
    loc[:, 1] *= 2 * np.pi
    return loc


@pytest.mark.parametrize("spin", [0, 2])
@pytest.mark.parametrize("eps,tol", [(1e-10, 1e-10), (1e-7, 1e-7), (1e-5, 1e-5)])
def test_nusht2d2_matches_direct_sum(cu, spin, eps, tol):
    lmax = 63
    T = _T(cu, lmax, eps=eps, precision="auto")
    rng = np.random.default_rng(30 + spin)
    a = ralm(lmax, 1 if spin == 0 else 2, rng, spin)
    A = a[0] if spin == 0 else a
    loc = _random_loc(3000, rng)
    got = T.nusht2d2(lmax, lmax, torch.as_tensor(A, device="cuda"), torch.as_tensor(loc, device="cuda"),
                     spin=spin).cpu().numpy()
    ref = oracle.synth_points_c(lmax, spin, A, loc[:, 0], loc[:, 1])
    assert rel(got, ref) < tol


@pytest.mark.parametrize("spin", [0, 2])
@pytest.mark.parametrize("eps,tol", [(1e-10, 1e-10), (1e-7, 1e-7)])
def test_nusht2d1_matches_direct_sum(cu, spin, eps, tol):
    lmax = 63
    T = _T(cu, lmax, eps=eps, precision="auto")
    rng = np.random.default_rng(40 + spin)
    loc = _random_loc(3000, rng)
    v = rng.standard_normal(3000 if spin == 0 else (2, 3000))
    got = T.nusht2d1(lmax, lmax, torch.as_tensor(v, device="cuda"), torch.as_tensor(loc, device="cuda"),
                     spin=spin).cpu().numpy()
    ref = oracle.adjoint_synth_points_c(lmax, spin, v, loc[:, 0], loc[:, 1])
    assert rel(got, ref) < tol


@pytest.mark.parametrize("spin", [0, 2])
def test_nusht_adjointness(cu, spin):
    """<y, A x> = <A^H y, x> (test/test_adjointOperator.py:246-277 pattern)."""
    lmax = 127
    T = _T(cu, lmax, eps=1e-8)
    rng = np.random.default_rng(48)
    ncomp = 1 if spin == 0 else 2
    x = ralm(lmax, ncomp, rng, spin)
    X = x[0] if spin == 0 else x
    loc = torch.as_tensor(_random_loc(20000, rng), device="cuda")
    y = rng.uniform(-0.5, 0.5, 20000 if spin == 0 else (2, 20000))
    Ax = T.nusht2d2(lmax, lmax, torch.as_tensor(X, device="cuda"), loc, spin=spin).cpu().numpy()
    Ay = T.nusht2d1(lmax, lmax, torch.as_tensor(y, device="cuda"), loc, spin=spin).cpu().numpy()
    v1 = float(np.sum(y * Ax))
    Ay = Ay.reshape(ncomp, -1)
    v2 = sum(orc.alm_dot(Ay[c], x[c], lmax) for c in range(ncomp))
    np.testing.assert_allclose(v1, v2, rtol=1e-9)


# ------------------------------------------------------------------ pointing / lensing
def test_dlm2pointing_matches_oracle(cu):
    lmax = 127
    T = _T(cu, lmax)
    gclm, dls = orc.make_inputs(lmax, 0, seed=1)
    ptg = T.dlm2pointing(torch.as_tensor(dls[0], device="cuda"), lmax, 0).cpu().numpy()
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    dlm = orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)
    d = oracle.synth_points_c(lmax, 1, dlm[None], th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    assert np.max(np.abs(ptg[0] - rt)) < 1e-13
    dphi = np.angle(np.exp(1j * (ptg[1] - rp)))
    assert np.max(np.abs(dphi)) < 1e-12
    rg = orc.rotation_gamma(th, d[0], d[1])
    assert np.max(np.abs(np.angle(np.exp(1j * (T.gamma.cpu().numpy() - rg))))) < 1e-11


@pytest.mark.parametrize("spin", [0, 2])
def test_gclm2lenmap_lmax255_config0(cu, spin):
    """Config 0 (lmax 255, GL 256 x 511, eps 1e-7) against direct FP64 Y_lm
    summation at the deflected points."""
    lmax = 255
    T = _T(cu, lmax, eps=1e-7, precision="fp64", nphi=511)
    gclm, dls = orc.make_inputs(lmax, spin, seed=0)
    g = gclm[0] if spin == 0 else gclm
    out = T.gclm2lenmap(torch.as_tensor(g, device="cuda"), lmax, lmax,
                        dlm_scaled=torch.as_tensor(dls[0], device="cuda"), spin=spin, verbose=0).cpu().numpy()
    # exact deflection on the CPU
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    dlm = orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)
    d = oracle.synth_points_c(lmax, 1, dlm[None], th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    ref = oracle.synth_points_c(lmax, spin, g, rt, rp)
    if spin:
        z = (ref[0] + 1j * ref[1]) * np.exp(1j * spin * orc.rotation_gamma(th, d[0], d[1]))
        ref = np.stack([z.real, z.imag])
    assert rel(out, ref) < 1e-7


# ------------------------------------------------------------------ mixed precision (double-float Legendre)
@pytest.mark.parametrize("spin,ncomp", [(0, 1), (1, 1), (2, 2)])
def test_mixed_synthesis_matches_direct_sum(cu, spin, ncomp):
    """Double-float recursion + compensated FP32 accumulation: 5e-8 relative L2."""
    lmax = 127
    T = _T(cu, lmax, eps=1e-7, precision="mixed")
    rng = np.random.default_rng(60 + spin)
    a = ralm(lmax, ncomp, rng, spin)
    th, ph = T.geom.pixels()
    A = a[0] if spin == 0 else a
    got = T.synthesis(torch.as_tensor(A, device="cuda"), spin=spin).cpu().numpy()
    ref = oracle.synth_points_c(lmax, spin, A, th, ph)
    assert rel(got, ref) < 5e-8


@pytest.mark.parametrize("spin", [0, 2])
def test_mixed_nusht2d2_matches_direct_sum(cu, spin):
    lmax = 127
    T = _T(cu, lmax, eps=1e-7, precision="mixed")
    rng = np.random.default_rng(70 + spin)
    a = ralm(lmax, 1 if spin == 0 else 2, rng, spin)
    A = a[0] if spin == 0 else a
    loc = _random_loc(4000, rng)
    got = T.nusht2d2(lmax, lmax, torch.as_tensor(A, device="cuda"), torch.as_tensor(loc, device="cuda"),
                     spin=spin).cpu().numpy()
    ref = oracle.synth_points_c(lmax, spin, A, loc[:, 0], loc[:, 1])
    assert rel(got, ref) < 1e-7


def test_mixed_gclm2lenmap_spin2_lmax255(cu):
    lmax = 255
    T = _T(cu, lmax, eps=1e-7, precision="mixed", nphi=511)
    gclm, dls = orc.make_inputs(lmax, 2, seed=3)
    out = T.gclm2lenmap(torch.as_tensor(gclm, device="cuda"), lmax, lmax,
                        dlm_scaled=torch.as_tensor(dls[0], device="cuda"), spin=2, verbose=0).cpu().numpy()
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    dlm = orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)
    d = oracle.synth_points_c(lmax, 1, dlm[None], th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    assert np.max(np.abs(T.ptg.cpu().numpy()[0] - rt)) < 2e-9
    ref = oracle.synth_points_c(lmax, 2, gclm, rt, rp)
    z = (ref[0] + 1j * ref[1]) * np.exp(2j * orc.rotation_gamma(th, d[0], d[1]))
    assert rel(out, np.stack([z.real, z.imag])) < 1e-7


def test_mixed_dlm2pointing_matches_oracle(cu):
    """Small-angle FP32 increments added in FP64: pointing within 1e-10 rad."""
    lmax = 127
    T = _T(cu, lmax, eps=1e-7, precision="mixed")
    _, dls = orc.make_inputs(lmax, 0, seed=11)
    ptg = T.dlm2pointing(torch.as_tensor(dls[0], device="cuda"), lmax, 0).cpu().numpy()
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    dlm = orc.almxfl(dls[0], np.sqrt(ll * (ll + 1.0)), lmax)
    d = oracle.synth_points_c(lmax, 1, dlm[None], th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    dnorm = np.sqrt(np.mean(d[0] ** 2 + d[1] ** 2))
    dt = ptg[0] - rt
    dp = np.angle(np.exp(1j * (ptg[1] - rp))) * np.sin(th)
    # error relative to the deflection: the deflection itself carries the
    # double-float Legendre error (~3e-8), the increments add FP32 rounding
    assert np.sqrt(np.mean(dt ** 2 + dp ** 2)) / dnorm < 1e-7
    assert np.max(np.abs(dt)) < 2e-9 and np.max(np.abs(dp)) < 2e-9
    rg = orc.rotation_gamma(th, d[0], d[1])
    assert np.max(np.abs(np.angle(np.exp(1j * (T.gamma.cpu().numpy() - rg))))) < 1e-8


# ------------------------------------------------------------------ curl deflection, spin-2 adjoint lensing
def test_dlm2pointing_with_curl_matches_oracle(cu):
    """Gradient + curl deflection (config 2 pattern): spin-1 synthesis of
    (dlm, dclm) then the pointing rotation."""
    lmax = 127
    T = _T(cu, lmax)
    _, dls = orc.make_inputs(lmax, 0, seed=21, curl=True)
    ptg = T.dlm2pointing(torch.as_tensor(dls[0], device="cuda"), lmax, 0,
                         dclm_scaled=torch.as_tensor(dls[1], device="cuda")).cpu().numpy()
    th, ph = T.geom.pixels()
    ll = np.arange(lmax + 1)
    fl = np.sqrt(ll * (ll + 1.0))
    dd = np.stack([orc.almxfl(dls[0], fl, lmax), orc.almxfl(dls[1], fl, lmax)])
    d = oracle.synth_points_c(lmax, 1, dd, th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    assert np.max(np.abs(ptg[0] - rt)) < 1e-13
    assert np.max(np.abs(np.angle(np.exp(1j * (ptg[1] - rp))))) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lensing_adjointness_spin2_with_rotation(cu, precision):
    """<y, gclm2lenmap(x)> = <lenmap2gclm(y), x> for spin 2 with the exp(2 i gamma)
    rotation (E and B components)."""
    lmax = 127
    T = _T(cu, lmax, eps=1e-8 if precision == "fp64" else 1e-7, precision=precision)
    rng = np.random.default_rng(31)
    _, dls = orc.make_inputs(lmax, 0, seed=22)
    d = torch.as_tensor(dls[0], device="cuda")
    x = ralm(lmax, 2, rng, 2)
    Ax = T.gclm2lenmap(torch.as_tensor(x, device="cuda"), lmax, lmax, dlm_scaled=d, spin=2, verbose=0).cpu().numpy()
    y = rng.standard_normal(Ax.shape)
    AHy = T.lenmap2gclm(torch.as_tensor(y, device="cuda"), d, None, lmax, lmax, spin=2, verbose=0).cpu().numpy()
    lhs = float(np.sum(y * Ax))
    rhs = orc.alm_dot(AHy[0], x[0], lmax) + orc.alm_dot(AHy[1], x[1], lmax)
    # mixed: the forward carries ~1e-7 arithmetic error (eps 1e-7) while the
    # adjoint runs in FP64, so the two agree to a few eps, not to FP64 rounding
    np.testing.assert_allclose(lhs, rhs, rtol=5e-7 if precision == "mixed" else 1e-9)


def test_planar_pointing_reaches_the_library_without_a_copy(built_lib):
    """gclm2lenmap passes ptg.t() as loc (GPU_nufft_transformer.py:569): the
    planar (2, npix) device buffer reaches the C ABI as layout 1, not as a
    strided copy."""
    from cunusht_gb300.transformer import _loc_args, to_device
    ptg = torch.arange(20, dtype=torch.float64, device="cuda").reshape(2, 10)
    t, n, lay = _loc_args(to_device(ptg.t(), "loc", torch.float64, contiguous=False))
    assert (n, lay) == (10, 1) and t.data_ptr() == ptg.data_ptr()
