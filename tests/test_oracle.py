"""Pins the FP64 oracle (CPU, no GPU needed).

The reference cannot run here (cupy / shtns / cufinufft / ducc0 absent), so the
oracle is pinned by known answers: scipy's independent Y_lm, the Goldberg
closed form for spin-weighted harmonics, published closed forms, the gradient
identity behind SHTns synth_grad, the reference tests' own numpy slicing for
doubling, dot-product adjointness (test/test_adjointOperator.py:246-277) and the
committed golden fixtures.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


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


THETA = np.array([0.0, 1e-3, 0.3, 1.2, np.pi / 2, 2.0, np.pi - 1e-3, np.pi])


def test_spin0_lambda_matches_scipy():
    sp = pytest.importorskip("scipy.special")
    for m in range(0, 9):
        lam = orc.slambda(14, m, 0, THETA)
        for l in range(m, 15):
            ref = sp.sph_harm_y(l, m, THETA, 0.0).real
            np.testing.assert_allclose(lam[l], ref, atol=1e-14)


def test_closed_forms():
    t = THETA
    np.testing.assert_allclose(orc.slambda(3, 0, 0, t)[0], np.full_like(t, 0.5 / np.sqrt(np.pi)), atol=1e-16)
    np.testing.assert_allclose(orc.slambda(3, 0, 0, t)[1], np.sqrt(3 / (4 * np.pi)) * np.cos(t), atol=1e-15)
    np.testing.assert_allclose(orc.slambda(3, 1, 0, t)[1], -np.sqrt(3 / (8 * np.pi)) * np.sin(t), atol=1e-15)
    np.testing.assert_allclose(orc.slambda(3, 0, 2, t)[2], np.sqrt(15 / (32 * np.pi)) * np.sin(t) ** 2, atol=1e-15)


@pytest.mark.parametrize("s", [1, 2, 3])
def test_spin_recursion_matches_goldberg_closed_form(s):
    for m in range(0, 9):
        lam = orc.slambda(16, m, s, THETA)
        for l in range(max(m, s), 17):
            np.testing.assert_allclose(lam[l], orc.slambda_explicit(l, m, s, THETA), atol=2e-12)


def test_spin_symmetries_of_closed_form():
    """sLam_lm = (-1)^(s+m) (-s)Lam_{l,-m};  (-s)Lam_lm(t) = (-1)^(l+m) sLam_lm(pi - t)."""
    for s in (1, 2):
        for m in range(-4, 5):
            for l in range(max(abs(m), s), 8):
                a = orc.slambda_explicit(l, m, s, THETA)
                np.testing.assert_allclose(a, (-1) ** (s + m) * orc.slambda_explicit(l, -m, -s, THETA), atol=1e-15)
                c = orc.slambda_explicit(l, m, -s, THETA)
                np.testing.assert_allclose(c, (-1) ** (l + m) * orc.slambda_explicit(l, m, s, np.pi - THETA),
                                           atol=1e-14)


def test_large_m_no_underflow():
    lam = orc.slambda(2047, 1000, 2, np.array([0.3, 0.5, 1.0]))
    assert np.all(np.isfinite(lam))
    assert abs(lam[-1, 2]) > 1e-3  # oscillatory region is reached and finite


def test_spin2_pure_E20_known_answer():
    """HEALPix convention: Q + iU = -sum (E + iB) 2Y_lm, so E_20 = 1 gives
    Q = -sqrt(15/32pi) sin^2 theta, U = 0."""
    L = 6
    rng = np.random.default_rng(0)
    th = np.arccos(rng.uniform(-1, 1, 100))
    ph = rng.uniform(0, 2 * np.pi, 100)
    a = np.zeros((2, orc.nalm(L)), complex)
    a[0, 2] = 1.0
    q = orc.synth_points(L, 2, a, th, ph)
    np.testing.assert_allclose(q[0], -np.sqrt(15 / (32 * np.pi)) * np.sin(th) ** 2, atol=1e-15)
    np.testing.assert_allclose(q[1], 0.0, atol=1e-15)


def test_spin1_is_gradient():
    """spin-1 synthesis of dlm = sqrt(l(l+1)) phi_lm = (d_theta phi, d_phi phi / sin theta),
    the quantity SHTns synth_grad returns (GPU_sht_transformer.py:95)."""
    L = 10
    rng = np.random.default_rng(1)
    th = np.arccos(rng.uniform(-0.95, 0.95, 200))
    ph = rng.uniform(0, 2 * np.pi, 200)
    plm = ralm(L, 1, rng)[0]
    ll = np.arange(L + 1)
    dlm = orc.almxfl(plm, np.sqrt(ll * (ll + 1.0)), L)
    g = orc.synth_points(L, 1, dlm[None], th, ph)
    h = 1e-6
    dth = (orc.synth_points(L, 0, plm, th + h, ph) - orc.synth_points(L, 0, plm, th - h, ph)) / (2 * h)
    dph = (orc.synth_points(L, 0, plm, th, ph + h) - orc.synth_points(L, 0, plm, th, ph - h)) / (2 * h) / np.sin(th)
    assert np.max(np.abs(g[0] - dth)) < 1e-7 * np.max(np.abs(g))
    assert np.max(np.abs(g[1] - dph)) < 1e-7 * np.max(np.abs(g))


@pytest.mark.parametrize("spin", [0, 1, 2])
def test_oracle_adjointness(spin):
    L = 12
    rng = np.random.default_rng(2 + spin)
    th = np.arccos(rng.uniform(-1, 1, 300))
    ph = rng.uniform(0, 2 * np.pi, 300)
    a = ralm(L, 1 if spin == 0 else 2, rng, spin)
    A = a[0] if spin == 0 else a
    v = rng.standard_normal(300 if spin == 0 else (2, 300))
    f = orc.synth_points(L, spin, A, th, ph)
    ad = np.atleast_2d(orc.adjoint_synth_points(L, spin, v, th, ph))
    lhs = float(np.sum(v * f))
    rhs = sum(orc.alm_dot(ad[c], a[c], L) for c in range(a.shape[0]))
    np.testing.assert_allclose(lhs, rhs, rtol=1e-12)


@pytest.mark.parametrize("spin", [0, 1, 2])
def test_c_oracle_matches_numpy_oracle(spin):
    L = 20
    rng = np.random.default_rng(4 + spin)
    th = np.arccos(rng.uniform(-1, 1, 400))
    ph = rng.uniform(0, 2 * np.pi, 400)
    a = ralm(L, 1 if spin == 0 else 2, rng, spin)
    A = a[0] if spin == 0 else a
    f1 = orc.synth_points(L, spin, A, th, ph)
    f2 = oracle.synth_points_c(L, spin, A, th, ph)
    np.testing.assert_allclose(f2, f1, rtol=0, atol=1e-13 * np.max(np.abs(f1)))
    v = rng.standard_normal(f1.shape)
    g1 = orc.adjoint_synth_points(L, spin, v, th, ph)
    g2 = oracle.adjoint_synth_points_c(L, spin, v, th, ph)
    np.testing.assert_allclose(g2, g1, rtol=0, atol=1e-12 * np.max(np.abs(g1)))


def test_gl_nodes_and_good_size():
    x, w = orc.gl_nodes(64)
    xr, wr = np.polynomial.legendre.leggauss(64)
    np.testing.assert_allclose(np.sort(x), np.sort(xr), atol=1e-15)
    np.testing.assert_allclose(np.sort(w), np.sort(wr), atol=1e-14)
    # CC sizing of the reference at lmax 2047 (GPU_nufft_transformer.py:138-141)
    assert (orc.good_size(2047 + 2) + 3) // 4 * 4 == 2060
    assert 2 * orc.good_size(2047 + 1) == 4096
    assert orc.good_size(2 * 2047 + 1, True) == 4096


def test_doubling_matches_reference_test_slicing():
    """test/test_doublingGPU.py:50-53 and :74-83 restated; theta-contiguous
    index arithmetic of doubling.cu:180-201."""
    nt, nphi = 36, 64
    m = np.arange(nt * nphi, dtype=float).reshape(nt, nphi)
    d = orc.doubling_ring_major(m, nt, nphi)
    h = nphi // 2
    want = np.zeros((2 * nt - 2, nphi))
    want[:nt] = m
    want[nt:, :h] = want[nt - 2:0:-1, h:]
    want[nt:, h:] = want[nt - 2:0:-1, :h]
    assert np.array_equal(d, want)
    # theta-contiguous input (nphi, ntheta): explicit index formula of doubling.cu:194-196
    tc = m.T.copy().reshape(-1)
    dt = 2 * nt - 2
    out = np.empty(nphi * dt)
    for idx in range(nphi):
        for ringi in range(dt):
            if ringi < nt:
                out[idx * dt + ringi] = tc[idx * nt + ringi]
            elif idx < h:
                out[idx * dt + ringi] = tc[nt * h + nt + idx * nt - 2 + (nt - ringi)]
            else:
                out[idx * dt + ringi] = tc[(idx - h) * nt + nt - 2 + (nt - ringi)]
    assert np.array_equal(orc.doubling_theta_contig(tc, nt, nphi).reshape(-1), out)
    # adjoint = transpose of doubling (as a linear map)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((nt, nphi))
    y = rng.standard_normal((2 * nt - 2, nphi))
    for spin in (0, 1, 2):
        lhs = np.sum(y * orc.doubling_ring_major(x, nt, nphi, spin))
        rhs = np.sum(orc.adjoint_doubling_ring_major(y, nt, nphi, spin) * x)
        np.testing.assert_allclose(lhs, rhs, rtol=1e-13)


def test_pointing_formula_is_geodesic_displacement():
    """pointing.cu:210-213 equals moving the unit vector a = |d| along the
    great circle in direction d_theta e_theta + d_phi e_phi."""
    rng = np.random.default_rng(9)
    th = np.arccos(rng.uniform(-0.99, 0.99, 500))
    ph = rng.uniform(0, 2 * np.pi, 500)
    dt = rng.standard_normal(500) * 3e-3
    dp = rng.standard_normal(500) * 3e-3
    thp, php = orc.pointing(th, ph, dt, dp)
    n = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
    et = np.stack([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
    ep = np.stack([-np.sin(ph), np.cos(ph), np.zeros_like(ph)])
    a = np.hypot(dt, dp)
    e = (dt * et + dp * ep) / a
    n2 = np.cos(a) * n + np.sin(a) * e
    np.testing.assert_allclose(np.arccos(np.clip(n2[2], -1, 1)), thp, atol=1e-12)
    np.testing.assert_allclose(np.angle(np.exp(1j * (np.arctan2(n2[1], n2[0]) - php))), 0.0, atol=1e-12)


def test_make_inputs_rms_deflection():
    g, d = orc.make_inputs(255, 2, seed=0)
    ll = np.arange(256)
    dlm = orc.almxfl(d[0], np.sqrt(ll * (ll + 1.0)), 255)
    rms = orc.rms_deflection(dlm, 255)
    np.testing.assert_allclose(rms, 2.5 / 60 * np.pi / 180, rtol=1e-12)
    assert g.shape == (2, orc.nalm(255)) and np.all(g[1] == 0)


def test_golden_fixtures():
    """The oracle reproduces the committed fixtures (tests/golden/make_golden.py)."""
    path = os.path.join(GOLDEN, "golden_small.npz")
    z = np.load(path)
    L = int(z["lmax"])
    for spin in (0, 1, 2):
        a = z[f"alm_s{spin}"]
        A = a[0] if spin == 0 else a
        got = orc.synth_points(L, spin, A, z["theta"], z["phi"])
        np.testing.assert_allclose(got, z[f"map_s{spin}"], rtol=0, atol=1e-13)
        adj = orc.adjoint_synth_points(L, spin, z[f"val_s{spin}"], z["theta"], z["phi"])
        np.testing.assert_allclose(adj, z[f"adj_s{spin}"], rtol=0, atol=1e-12)
    thp, php = orc.pointing(z["ptheta"], z["pphi"], z["dth"], z["dph"])
    np.testing.assert_allclose(thp, z["thp"], atol=1e-15)
    np.testing.assert_allclose(php, z["php"], atol=1e-15)
