"""alm helpers (healpy m-major layout), restating cunusht/utils.py:9-199 with an
explicit random generator so that every synthetic field is reproducible."""
from __future__ import annotations

import numpy as np

# cunusht/utils.py:9 (lmax values with FFT-friendly grids)
good_lmax_array = np.array([4, 8, 16, 28, 36, 64, 76, 136, 148, 176, 244, 316, 344, 376, 568, 676, 736,
                            876, 1216, 1324, 1576, 1716, 1876, 2188, 2836, 3088, 3376, 3676, 4376, 5104]) - 1


class Alm:
    """alm array statics (cunusht/utils.py:10-83)."""

    @staticmethod
    def getsize(lmax: int, mmax: int) -> int:
        return ((mmax + 1) * (mmax + 2)) // 2 + (mmax + 1) * (lmax - mmax)

    @staticmethod
    def getidx(lmax: int, l, m):
        return m * (2 * lmax + 1 - m) // 2 + l

    @staticmethod
    def getlmax(s: int, mmax: int | None) -> int:
        if mmax is not None and mmax >= 0:
            x = (2 * s + mmax ** 2 - mmax - 2) / (2 * mmax + 2)
        else:
            x = (-3 + np.sqrt(1 + 8 * s)) / 2
        return int(x) if x == np.floor(x) else -1


def almxfl(alm: np.ndarray, fl: np.ndarray, mmax: int | None, inplace: bool):
    """alm_lm * fl_l (cunusht/utils.py:85-120)."""
    lmax = Alm.getlmax(alm.size, mmax)
    mmax = lmax if (mmax is None or mmax < 0) else mmax
    assert fl.size > lmax, (fl.size, lmax)
    out = alm if inplace else np.empty_like(alm)
    for m in range(mmax + 1):
        b = m * (2 * lmax + 1 - m) // 2 + m
        out[b:b + lmax - m + 1] = alm[b:b + lmax - m + 1] * fl[m:lmax + 1]
    return None if inplace else out


def synalm(cl: np.ndarray, lmax: int, mmax: int | None, rng: np.random.Generator | None = None,
           rlm_dtype=np.float64):
    """Gaussian alm of spectrum cl (cunusht/utils.py:122-150); ``rng`` makes it
    reproducible (the reference draws from an unseeded module generator)."""
    rng = np.random.default_rng() if rng is None else rng
    mmax = lmax if (mmax is None or mmax < 0) else mmax
    n = Alm.getsize(lmax, mmax)
    alm = rng.standard_normal(n, dtype=rlm_dtype) + 1j * rng.standard_normal(n, dtype=rlm_dtype)
    almxfl(alm, np.sqrt(cl[:lmax + 1] * 0.5), mmax, True)
    idx = Alm.getidx(lmax, np.arange(lmax + 1), 0)
    alm[idx] = alm[idx].real * np.sqrt(2.0)
    return alm


def alm2cl(alm: np.ndarray, blm: np.ndarray | None, lmax: int | None, mmax: int | None,
           lmaxout: int | None):
    """(Cross-)power spectrum (cunusht/utils.py:153-199)."""
    if lmax is None:
        lmax = Alm.getlmax(alm.size, mmax)
    if lmaxout is None:
        lmaxout = lmax
    if mmax is None:
        mmax = lmax
    blm = alm if blm is None else blm
    lo = min(lmaxout, lmax)
    cl = 0.5 * alm[:lo + 1].real * blm[:lo + 1].real
    for m in range(1, min(mmax, lo) + 1):
        i = Alm.getidx(lmax, m, m)
        a = alm[i:i + lo - m + 1]
        b = blm[i:i + lo - m + 1]
        cl[m:] += a.real * b.real + a.imag * b.imag
    cl *= 2.0 / (2 * np.arange(len(cl)) + 1)
    if lmaxout > lo:
        out = np.zeros(lmaxout + 1)
        out[:lo + 1] = cl
        return out
    return cl


def good_size(n: int, real: bool = False) -> int:
    """Smallest m >= n with prime factors {2,3,5} (real) or {2,3,5,7,11}
    (complex): the contract of ducc0.fft.good_size used by the reference."""
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
