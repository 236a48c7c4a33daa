"""FP64 CPU oracle for the nuSHT / lensing path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this module, and only as the checker.  The product
(``cunusht_gb300``) never calls it.

It restates, in plain numpy, the algorithm of the reference (Sebastian-Belkner/
cunuSHT) and of the third-party libraries the reference calls for this path:

* geometry / alm layout    -- cunusht/geometry.py:229-245, :267-284;
                              cunusht/utils.py:16-58 (healpy m-major layout)
* seeded field generation  -- cunusht/utils.py:122-150 (synalm, but with an
                              explicit ``numpy.random.Generator``)
* spin-weighted harmonics  -- the orthonormal Condon-Shortley convention used by
                              SHTns / ducc0 (first_steps/quickstart.ipynb:211),
                              written through the Goldberg et al. (1967) closed
                              form and the Wigner-d three-term recursion in l;
                              spin>0 uses the HEALPix convention
                              s_a_lm = -(G_lm + i C_lm)  (E/B -> Q/U).
* pointing (deflected angles) -- cunusht/c/pointing.cu:210-222
* polarisation rotation angle -- cunusht/deflection/CPU_nufft_transformer.py:158-160
* map doubling and adjoint -- cunusht/c/doubling.cu:137-201, :53-72 and the
                              numpy slicing of test/test_doublingGPU.py:50-53, :74-83;
                              spin-aware form CPU_nufft_transformer.py:284-318
* FFT sizing (good_size)   -- ducc0.fft.good_size as called at
                              GPU_nufft_transformer.py:138-141

Pinning: the reference itself cannot run in this environment (it imports cupy,
shtns, cufinufft, ducc0, lenspyx at module top and ships no compiled code), so
this oracle is pinned by known-answer tests instead: scipy's independent
spherical-harmonic implementation (spin 0), the Goldberg closed form (spin s),
published closed forms (Y_00, Y_10, 2Y_20), the gradient identity behind
SHTns ``synth_grad`` (spin 1), the reference tests' own numpy slicing for
doubling, and dot-product adjointness (test/test_adjointOperator.py:246-277).
"""
from __future__ import annotations

import math
import numpy as np

FOURPI = 4.0 * math.pi


# --------------------------------------------------------------------------
# alm layout (cunusht/utils.py:16-58)
# --------------------------------------------------------------------------
def nalm(lmax: int, mmax: int | None = None) -> int:
    mmax = lmax if mmax is None else mmax
    return ((mmax + 1) * (mmax + 2)) // 2 + (mmax + 1) * (lmax - mmax)


def almidx(lmax: int, l, m):
    return m * (2 * lmax + 1 - m) // 2 + l


def almxfl(alm: np.ndarray, fl: np.ndarray, lmax: int) -> np.ndarray:
    """alm[l,m] * fl[l] (cunusht/utils.py:85-120, out-of-place form)."""
    out = np.empty_like(alm)
    for m in range(lmax + 1):
        b = almidx(lmax, m, m)
        out[b:b + lmax - m + 1] = alm[b:b + lmax - m + 1] * fl[m:lmax + 1]
    return out


def synalm(cl: np.ndarray, lmax: int, rng: np.random.Generator) -> np.ndarray:
    """Gaussian alm with spectrum cl (cunusht/utils.py:122-150, seeded)."""
    n = nalm(lmax)
    alm = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    alm = almxfl(alm, np.sqrt(cl[:lmax + 1] * 0.5), lmax)
    alm[:lmax + 1] = alm[:lmax + 1].real * np.sqrt(2.0)
    return alm


def alm2cl(alm: np.ndarray, lmax: int) -> np.ndarray:
    """Auto power spectrum (cunusht/utils.py:153-199)."""
    cl = 0.5 * alm[:lmax + 1].real ** 2
    for m in range(1, lmax + 1):
        b = almidx(lmax, m, m)
        a = alm[b:b + lmax - m + 1]
        cl[m:] += a.real ** 2 + a.imag ** 2
    return cl * 2.0 / (2 * np.arange(lmax + 1) + 1)


def alm_dot(a: np.ndarray, b: np.ndarray, lmax: int) -> float:
    """Real-field alm inner product, m>0 counted twice
    (test/test_adjointOperator.py:39-48, compress_alm/myalmdot)."""
    s = float(np.sum(a[:lmax + 1].real * b[:lmax + 1].real))
    s += 2.0 * float(np.sum((a[lmax + 1:] * np.conj(b[lmax + 1:])).real))
    return s


# --------------------------------------------------------------------------
# geometry (cunusht/geometry.py)
# --------------------------------------------------------------------------
def good_size(n: int, real: bool = False) -> int:
    """Smallest m >= n whose prime factors are {2,3,5} (real) or
    {2,3,5,7,11} (complex): the contract of ducc0.fft.good_size."""
    primes = (2, 3, 5) if real else (2, 3, 5, 7, 11)
    m = max(int(n), 1)
    while True:
        k = m
        for p in primes:
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def gl_nodes(n: int):
    """Gauss-Legendre nodes x=cos(theta) (descending) and weights, Newton on P_n."""
    k = np.arange(1, n + 1)
    x = np.cos(np.pi * (k - 0.25) / (n + 0.5))
    for _ in range(100):
        p0 = np.ones_like(x)
        p1 = x.copy()
        for j in range(2, n + 1):
            p0, p1 = p1, ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
        dp = n * (x * p1 - p0) / (x * x - 1.0)
        dx = p1 / dp
        x -= dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    p0 = np.ones_like(x)
    p1 = x.copy()
    for j in range(2, n + 1):
        p0, p1 = p1, ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
    dp = n * (x * p1 - p0) / (x * x - 1.0)
    w = 2.0 / ((1.0 - x * x) * dp * dp)
    return x, w


def gl_geometry(lmax: int, nphi: int | None = None):
    """(theta, phi0, nph, ofs, weight) of the GL grid (geometry.py:267-284)."""
    nlat = lmax + 1
    if nphi is None:
        nphi = good_size(2 * lmax + 1, True)
    x, w = gl_nodes(nlat)
    theta = np.arccos(x)
    nph = np.full(nlat, nphi, dtype=np.int64)
    ofs = np.concatenate([[0], np.cumsum(nph[:-1])]).astype(np.int64)
    return theta, np.zeros(nlat), nph, ofs, 2.0 * np.pi * w / nph


def geometry_pixels(theta, phi0, nph, ofs):
    """Flat (theta, phi) of every pixel of a ring geometry."""
    npix = int(np.sum(nph))
    th = np.empty(npix)
    ph = np.empty(npix)
    for t, p0, n, o in zip(theta, phi0, nph, ofs):
        th[o:o + n] = t
        ph[o:o + n] = p0 + 2.0 * np.pi * np.arange(n) / n
    return th, ph


# --------------------------------------------------------------------------
# spin-weighted harmonics
# --------------------------------------------------------------------------
def slambda_explicit(l: int, m: int, s: int, theta: np.ndarray) -> np.ndarray:
    """sY_lm(theta, 0) from the Goldberg et al. closed form
    sY_lm = (-1)^m sqrt((l+m)!(l-m)!(2l+1)/(4pi (l+s)!(l-s)!))
            sum_r C(l-s,r) C(l+s,r+s-m) (-1)^(l-r-s) sin^(2l-2r-s+m)(t/2) cos^(2r+s-m)(t/2).
    Exact integer combinatorics; for small l only (pinning)."""
    theta = np.asarray(theta, dtype=np.float64)
    if l < abs(m) or l < abs(s):
        return np.zeros_like(theta)
    pref = math.sqrt(math.factorial(l + m) * math.factorial(l - m) * (2 * l + 1)
                     / (FOURPI * math.factorial(l + s) * math.factorial(l - s)))
    pref *= (-1) ** (m % 2)
    sh, ch = np.sin(0.5 * theta), np.cos(0.5 * theta)
    acc = np.zeros_like(theta)
    for r in range(0, l - s + 1):
        k = r + s - m
        if k < 0 or k > l + s:
            continue
        c = math.comb(l - s, r) * math.comb(l + s, k) * (-1) ** ((l - r - s) % 2)
        acc += c * sh ** (2 * l - 2 * r - s + m) * ch ** (2 * r + s - m)
    return pref * acc


def recursion_coeffs(lmax: int, m: int, s: int):
    """alpha_l, gamma_l, beta_l of the normalised Wigner-d recursion
       lam_{l+1} = (alpha_l x + gamma_l) lam_l - beta_l lam_{l-1}
    for the spin-s, order-m functions, l = l0 .. lmax-1 (l0 = max(m, s))."""
    l0 = max(m, s)
    al = np.zeros(lmax + 2)
    ga = np.zeros(lmax + 2)
    be = np.zeros(lmax + 2)
    for l in range(l0, lmax + 1):
        lp = l + 1
        den = math.sqrt((lp * lp - m * m) * (lp * lp - s * s))
        al[l] = lp * math.sqrt((2 * l + 1) * (2 * l + 3)) / den
        ga[l] = al[l] * (m * s / (l * lp) if l > 0 else 0.0)
        if l > 0:
            be[l] = (lp / l) * math.sqrt((l * l - m * m) * (l * l - s * s)) / den \
                * math.sqrt((2 * l + 3) / (2 * l - 1))
    return al, ga, be


def log2_start(m: int, s: int) -> float:
    """log2 of |sY_{l0,m}| / (sin^(m+s)(t/2) cos^|m-s|(t/2)), l0 = max(m,s)."""
    l0 = max(m, s)
    v = math.log((2 * l0 + 1) / FOURPI) + math.lgamma(2 * l0 + 1) \
        - math.lgamma(m + s + 1) - math.lgamma(abs(m - s) + 1)
    return 0.5 * v / math.log(2.0)


def slambda(lmax: int, m: int, s: int, theta: np.ndarray) -> np.ndarray:
    """sLambda_lm(theta) for l = 0..lmax (rows), s >= 0, m >= 0, by the scaled
    three-term recursion (mantissa + integer exponent per point, so the
    sin^(m+s) start never underflows)."""
    theta = np.atleast_1d(np.asarray(theta, dtype=np.float64))
    out = np.zeros((lmax + 1, theta.size))
    l0 = max(m, s)
    if l0 > lmax:
        return out
    x = np.cos(theta)
    sh, ch = np.sin(0.5 * theta), np.cos(0.5 * theta)
    lg = np.full(theta.size, log2_start(m, s))
    with np.errstate(divide="ignore"):
        if m + s > 0:
            lg = lg + (m + s) * np.log2(sh)
        if m != s:
            lg = lg + abs(m - s) * np.log2(ch)
    zero = ~np.isfinite(lg)
    lg = np.where(zero, 0.0, lg)
    e = np.floor(lg)
    mant = np.exp2(lg - e) * (-1.0) ** (m % 2)
    mant = np.where(zero, 0.0, mant)
    al, ga, be = recursion_coeffs(lmax, m, s)
    prev = np.zeros_like(mant)
    cur = mant
    out[l0] = np.ldexp(cur, e.astype(np.int64))
    for l in range(l0, lmax):
        nxt = (al[l] * x + ga[l]) * cur - be[l] * prev
        prev, cur = cur, nxt
        big = np.abs(cur) > 2.0 ** 200
        if np.any(big):
            cur = np.where(big, cur * 2.0 ** -200, cur)
            prev = np.where(big, prev * 2.0 ** -200, prev)
            e = np.where(big, e + 200, e)
        out[l + 1] = np.ldexp(cur, np.maximum(e, -2000).astype(np.int64))
    return out


# --------------------------------------------------------------------------
# direct synthesis / adjoint at arbitrary points (exact, O(nalm * npts))
# --------------------------------------------------------------------------
def synth_points(lmax: int, spin: int, alm: np.ndarray, theta: np.ndarray,
                 phi: np.ndarray) -> np.ndarray:
    """spin 0: alm (nalm,) -> real values (npts,).
    spin s>0: alm (ncomp, nalm) with (G[, C]) -> (2, npts) real (Q, U) with
    Q + iU = sum_lm s_a_lm sY_lm, s_a_lm = -(G_lm + i C_lm)."""
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    if spin == 0:
        a = np.asarray(alm).reshape(-1)
        f = np.zeros(theta.size)
        for m in range(lmax + 1):
            lam = slambda(lmax, m, 0, theta)
            b = almidx(lmax, m, m)
            hm = a[b:b + lmax - m + 1] @ lam[m:]
            if m == 0:
                f += hm.real
            else:
                f += 2.0 * (hm * np.exp(1j * m * phi)).real
        return f
    alm = np.atleast_2d(alm)
    G = alm[0]
    C = alm[1] if alm.shape[0] > 1 else np.zeros_like(G)
    z = np.zeros(theta.size, dtype=np.complex128)
    sgn_s = (-1.0) ** (spin % 2)
    for m in range(lmax + 1):
        lp = slambda(lmax, m, spin, theta)           # sLam(theta)
        lpm = slambda(lmax, m, spin, np.pi - theta)  # sLam(pi-theta)
        b = almidx(lmax, m, m)
        ll = np.arange(lmax + 1)
        g = G[b:b + lmax - m + 1]
        c = C[b:b + lmax - m + 1]
        hm = -((g + 1j * c) @ lp[m:])
        z += hm * np.exp(1j * m * phi)
        if m > 0:
            par = (-1.0) ** ((ll[m:] + m) % 2)
            lminus = par[:, None] * lpm[m:]             # -sLam(theta)
            hmm = -sgn_s * ((np.conj(g) + 1j * np.conj(c)) @ lminus)
            z += hmm * np.exp(-1j * m * phi)
    return np.stack([z.real, z.imag])


def adjoint_synth_points(lmax: int, spin: int, values: np.ndarray,
                         theta: np.ndarray, phi: np.ndarray, ncomp: int = 2) -> np.ndarray:
    """Exact adjoint of synth_points w.r.t. the real map inner product and the
    real-field alm inner product (m>0 counted twice)."""
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    n = nalm(lmax)
    if spin == 0:
        v = np.asarray(values, dtype=np.float64).reshape(-1)
        out = np.zeros(n, dtype=np.complex128)
        for m in range(lmax + 1):
            lam = slambda(lmax, m, 0, theta)
            b = almidx(lmax, m, m)
            out[b:b + lmax - m + 1] = lam[m:] @ (v * np.exp(-1j * m * phi))
        return out
    v = np.asarray(values, dtype=np.float64)
    z = v[0] + 1j * v[1]
    G = np.zeros(n, dtype=np.complex128)
    C = np.zeros(n, dtype=np.complex128)
    sgn_s = (-1.0) ** (spin % 2)
    ll = np.arange(lmax + 1)
    for m in range(lmax + 1):
        lp = slambda(lmax, m, spin, theta)
        lpm = slambda(lmax, m, spin, np.pi - theta)
        b = almidx(lmax, m, m)
        hp = lp[m:] @ (z * np.exp(-1j * m * phi))
        if m == 0:
            G[b:b + lmax + 1] = -hp.real
            C[b:b + lmax + 1] = -hp.imag
            continue
        par = (-1.0) ** ((ll[m:] + m) % 2)
        lminus = par[:, None] * lpm[m:]
        hm = lminus @ np.conj(z * np.exp(1j * m * phi))   # sum lam- conj(h'_{-m})
        G[b:b + lmax - m + 1] = -0.5 * (hp + sgn_s * hm)
        C[b:b + lmax - m + 1] = 0.5j * (hp - sgn_s * hm)
    return np.stack([G, C])[:ncomp]


# --------------------------------------------------------------------------
# pointing (cunusht/c/pointing.cu:197-226) and rotation angle
# --------------------------------------------------------------------------
def pointing(theta_pix: np.ndarray, phi_pix: np.ndarray, dth: np.ndarray,
             dph: np.ndarray):
    """Deflected (theta', phi') per pixel, the formula of pointing.cu:210-213
    (phi' wrapped only when >= 2pi, pointing.cu:213)."""
    d2 = dth * dth + dph * dph
    a = np.sqrt(d2)
    with np.errstate(invalid="ignore", divide="ignore"):
        sinaoa = np.where(d2 > 1e-8, np.sin(a) / np.where(a > 0, a, 1.0),
                          1.0 - d2 / 6.0 * (1.0 - d2 / 20.0 * (1.0 - d2 / 42.0)))
    cosa = np.cos(a)
    st, ct = np.sin(theta_pix), np.cos(theta_pix)
    nx = st * cosa + ct * dth * sinaoa
    ny = -dph * sinaoa
    nz = ct * cosa - st * dth * sinaoa
    thp = np.arctan2(np.sqrt(nx * nx + ny * ny), nz)
    php = phi_pix - np.arctan2(ny, nx)
    php = np.where(php >= 2 * np.pi, php - 2 * np.pi, php)
    return thp, php


def rotation_gamma(theta_pix: np.ndarray, dth: np.ndarray, dph: np.ndarray):
    """Polarisation rotation angle, CPU_nufft_transformer.py:158-160."""
    cot = np.cos(theta_pix) / np.sin(theta_pix)
    d = np.sqrt(dth * dth + dph * dph)
    return np.arctan2(dph, dth) - np.arctan2(dph, d * np.sin(d) * cot + dth * np.cos(d))


# --------------------------------------------------------------------------
# doubling (cunusht/c/doubling.cu, test/test_doublingGPU.py)
# --------------------------------------------------------------------------
def doubling_ring_major(cc: np.ndarray, ntheta: int, nphi: int, spin: int = 0):
    """(ntheta, nphi) ring-major CC map -> (2 ntheta - 2, nphi) theta torus
    (test_doublingGPU.py:50-53; odd-spin sign CPU_nufft_transformer.py:294-295)."""
    m = np.asarray(cc).reshape(ntheta, nphi)
    h = nphi // 2
    out = np.zeros((2 * ntheta - 2, nphi), dtype=m.dtype)
    out[:ntheta] = m
    out[ntheta:, :h] = out[ntheta - 2:0:-1, h:]
    out[ntheta:, h:] = out[ntheta - 2:0:-1, :h]
    if spin % 2:
        out[ntheta:] *= -1
    return out


def doubling_theta_contig(cc: np.ndarray, ntheta: int, nphi: int):
    """theta-contiguous (nphi, ntheta) CC map -> (nphi, 2 ntheta - 2) torus
    (doubling.cu:180-201)."""
    ring = np.asarray(cc).reshape(nphi, ntheta).T
    return doubling_ring_major(ring, ntheta, nphi).T.copy()


def adjoint_doubling_ring_major(dmap: np.ndarray, ntheta: int, nphi: int, spin: int = 0):
    """(2 ntheta - 2, nphi) -> (ntheta, nphi) fold, test_doublingGPU.py:80-83 and
    CPU_nufft_transformer.py:301-309."""
    d = np.array(dmap, copy=True).reshape(2 * ntheta - 2, nphi)
    h = nphi // 2
    sg = -1.0 if spin % 2 else 1.0
    d[1:ntheta - 1, :h] += sg * d[-1:ntheta - 1:-1, h:]
    d[1:ntheta - 1, h:] += sg * d[-1:ntheta - 1:-1, :h]
    return d[:ntheta].copy()


# --------------------------------------------------------------------------
# seeded synthetic inputs of the benchmark configurations
# --------------------------------------------------------------------------
def cl_unlensed(lmax: int) -> np.ndarray:
    ll = np.arange(lmax + 1, dtype=np.float64)
    return 1e3 / (ll + 10.0) ** 2


def cl_phi(lmax: int) -> np.ndarray:
    ll = np.arange(lmax + 1, dtype=np.float64)
    return 4e-7 * (ll + 20.0) ** -4


def rms_deflection(dlm: np.ndarray, lmax: int) -> float:
    """sqrt(sum_l (2l+1)/(4pi) C_l^dd) (CPU_nufft_transformer.py:441-446)."""
    cl = alm2cl(dlm, lmax)
    return float(np.sqrt(np.sum(cl * (2 * np.arange(lmax + 1) + 1)) / FOURPI))


def make_inputs(lmax: int, spin: int, seed: int, curl: bool = False,
                rms_arcmin: float = 2.5):
    """Seeded (gclm, dlm_scaled) pair: gclm ~ CN(0, C_l) (spin 0) or
    E ~ CN(0, 0.1 C_l), B = 0 (spin 2); phi_lm ~ CN(0, C_l^pp) rescaled to the
    requested rms deflection; dlm = sqrt(l(l+1)) phi_lm, dlm_scaled = phi_lm.
    Returns gclm (ncomp, nalm), dlm_scaled (nd, nalm) complex128."""
    rng = np.random.default_rng(seed)
    cl = cl_unlensed(lmax)
    if spin == 0:
        gclm = synalm(cl, lmax, rng)[None, :]
    else:
        e = synalm(0.1 * cl, lmax, rng)
        gclm = np.stack([e, np.zeros_like(e)])
    ll = np.arange(lmax + 1, dtype=np.float64)
    fl = np.sqrt(ll * (ll + 1.0))
    plm = synalm(cl_phi(lmax), lmax, rng)
    dlm = almxfl(plm, fl, lmax)
    scale = (rms_arcmin / 60.0 * np.pi / 180.0) / rms_deflection(dlm, lmax)
    plm = plm * scale
    dls = [plm]
    if curl:
        olm = synalm(0.1 * cl_phi(lmax), lmax, rng) * scale
        dls.append(olm)
    return gclm, np.stack(dls)
