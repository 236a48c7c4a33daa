"""Iso-latitude ring geometries (cunusht/geometry.py:29-298): Gauss-Legendre,
Clenshaw-Curtis, Fejer-1, longitude-thinned Gauss-Legendre and HEALPix."""
from __future__ import annotations

import inspect

import numpy as np

from .utils import good_size


def st2mmax(spin: int, tht, lmax: int):
    """Largest effective m on a ring at colatitude tht for a spin-s field of
    band limit lmax (libsharp polar optimisation, geometry.py:9-17); 2 mmax + 1
    longitudes then suffice on that ring."""
    T = max(0.01 * lmax, 100)
    b = -2 * spin * np.cos(tht)
    c = -(T + lmax * np.sin(tht)) ** 2 + spin ** 2
    return 0.5 * (-b + np.sqrt(b * b - 4 * c))


def _gl_nodes(n: int):
    """Gauss-Legendre nodes x = cos(theta) (descending) and weights; Newton
    iteration on P_n from the Tricomi initial guess, vectorised over nodes."""
    k = np.arange(1, n + 1)
    x = np.cos(np.pi * (k - 0.25) / (n + 0.5))

    def legendre(x):
        p0 = np.ones_like(x)
        p1 = x.copy()
        for j in range(2, n + 1):
            p0, p1 = p1, ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
        return p0, p1

    for _ in range(100):
        p0, p1 = legendre(x)
        dp = n * (x * p1 - p0) / (x * x - 1.0)
        dx = p1 / dp
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    p0, p1 = legendre(x)
    dp = n * (x * p1 - p0) / (x * x - 1.0)
    return x, 2.0 / ((1.0 - x * x) * dp * dp)


class Geom:
    """Ring geometry: colatitudes, first longitude, pixels per ring, first
    pixel index and quadrature weight per ring, sorted by first pixel
    (cunusht/geometry.py:29-57)."""

    def __init__(self, theta, phi0, nphi, ringstart, w):
        for a in (phi0, nphi, ringstart, w):
            assert np.asarray(a).size == np.asarray(theta).size
        order = np.argsort(ringstart)
        self.theta = np.asarray(theta, dtype=np.float64)[order]
        self.weight = np.asarray(w, dtype=np.float64)[order]
        self.phi0 = np.asarray(phi0, dtype=np.float64)[order]
        self.nph = np.asarray(nphi, dtype=np.uint64)[order]
        self.ofs = np.asarray(ringstart, dtype=np.uint64)[order]

    def npix(self) -> int:
        return int(np.sum(self.nph))

    def fsky(self) -> float:
        return float(np.sum(self.weight * self.nph) / (4 * np.pi))

    def nalm(self, lmax: int, mmax: int) -> int:
        return ((mmax + 1) * (mmax + 2)) // 2 + (mmax + 1) * (lmax - mmax)

    def pixels(self):
        """(theta, phi) of every pixel, ring by ring."""
        th = np.empty(self.npix())
        ph = np.empty(self.npix())
        for t, p0, n, o in zip(self.theta, self.phi0, self.nph.astype(np.int64), self.ofs.astype(np.int64)):
            th[o:o + n] = t
            ph[o:o + n] = p0 + 2.0 * np.pi * np.arange(n) / n
        return th, ph

    @staticmethod
    def get_gl_geometry(lmax: int, good_size_real: bool = True, nphi: int | None = None):
        """Gauss-Legendre grid, lmax + 1 rings (geometry.py:267-284)."""
        nlat = lmax + 1
        if nphi is None:
            nphi = good_size(2 * lmax + 1, good_size_real)
        x, wt = _gl_nodes(nlat)
        tht = np.arccos(x)
        nph = np.full(nlat, nphi, dtype=np.uint64)
        ofs = np.insert(np.cumsum(nph[:-1]), 0, 0)
        return Geom(tht, np.zeros(nlat), nph, ofs, 2 * np.pi * wt / nph)

    @staticmethod
    def get_cc_geometry(ntheta: int, nphi: int):
        """Clenshaw-Curtis grid with both poles (geometry.py:229-245);
        weights by the Waldvogel formula."""
        tht = np.linspace(0, np.pi, ntheta)
        nph = np.full(ntheta, nphi, dtype=np.uint64)
        ofs = np.insert(np.cumsum(nph[:-1]), 0, 0)
        n = ntheta - 1
        w = np.zeros(ntheta)
        for k in range(ntheta):
            s = 0.0
            for j in range(1, n // 2 + 1):
                b = 1.0 if 2 * j == n else 2.0
                s += b / (4 * j * j - 1) * np.cos(2 * j * k * np.pi / n)
            c = 1.0 if (k == 0 or k == n) else 2.0
            w[k] = c / n * (1.0 - s)
        return Geom(tht, np.zeros(ntheta), nph, ofs, w * 2 * np.pi / nphi)

    @staticmethod
    def get_f1_geometry(ntheta: int, nphi: int):
        """Fejer-1 grid: ntheta uniform colatitudes, the first and last pi / 2N
        from the poles (geometry.py:248-265); weights of Fejer's first rule."""
        tht = (np.arange(ntheta) + 0.5) * np.pi / ntheta
        j = np.arange(1, ntheta // 2 + 1)
        w = 2.0 / ntheta * (1.0 - 2.0 * np.sum(np.cos(2.0 * j[None, :] * tht[:, None]) / (4.0 * j * j - 1.0),
                                               axis=1))
        nph = np.full(ntheta, nphi, dtype=np.uint64)
        ofs = np.insert(np.cumsum(nph[:-1]), 0, 0)
        return Geom(tht, np.zeros(ntheta), nph, ofs, w * 2 * np.pi / nphi)

    @staticmethod
    def get_thingauss_geometry(lmax: int, smax: int, good_size_real: bool = True):
        """Longitude-thinned Gauss-Legendre grid (geometry.py:195-215): the GL
        rings of get_gl_geometry, each with good_size(2 mmax + 1) longitudes for
        its effective mmax (st2mmax), so rings near the poles are shorter."""
        nlat = lmax + 1
        x, wt = _gl_nodes(nlat)
        tht = np.arccos(x)
        mmax = np.minimum(np.maximum(st2mmax(smax, tht, lmax), st2mmax(-smax, tht, lmax)), np.ones(nlat) * lmax)
        nph = np.array([good_size(int(np.ceil(2 * m + 1)), good_size_real) for m in mmax], dtype=np.uint64)
        ofs = np.insert(np.cumsum(nph[:-1]), 0, 0)
        return Geom(tht, np.zeros(nlat), nph, ofs, 2 * np.pi * wt / nph)

    @staticmethod
    def get_tgl_geometry(lmax: int, smax: int, good_size_real: bool = True):
        """Alias of get_thingauss_geometry (geometry.py:287-297)."""
        return Geom.get_thingauss_geometry(lmax, smax, good_size_real=good_size_real)

    @staticmethod
    def get_healpix_geometry(nside: int):
        """HEALPix RING pixelisation (geometry.py:217-227), 4 nside - 1 rings,
        12 nside^2 equal-area pixels: polar-cap ring i has 4 i pixels starting
        at pi / (4 i), equatorial rings 4 nside pixels starting at pi / (4 nside)
        or pi / (2 nside) alternately (Gorski et al. 2005)."""
        nr = 4 * nside - 1
        tht = np.empty(nr)
        phi0 = np.empty(nr)
        nph = np.empty(nr, dtype=np.uint64)
        for r in range(nr):
            i = r + 1
            ip = min(i, 4 * nside - i)  # ring index from the nearer pole
            if ip < nside:  # polar caps
                t = 2.0 * np.arcsin(ip / (np.sqrt(6.0) * nside))
                tht[r] = t if i < nside else np.pi - t
                nph[r] = 4 * ip
                phi0[r] = np.pi / (4.0 * ip)
            else:  # equatorial belt
                tht[r] = np.arccos((4.0 / 3.0) - 2.0 * i / (3.0 * nside))
                nph[r] = 4 * nside
                sft = (i - nside + 1) % 2
                phi0[r] = np.pi / (2.0 * nside) * (1.0 - 0.5 * sft)
        ofs = np.insert(np.cumsum(nph[:-1]), 0, 0)
        area = 4 * np.pi / (12 * nside * nside)
        return Geom(tht, phi0, nph, ofs, np.full(nr, area))

    @staticmethod
    def get_supported_geometries():
        return "gl, cc, f1, thingauss, tgl, healpix"


def get_geom(geometry: tuple = ("gl", {"lmax": 255})) -> Geom:
    """Geometry from (name, kwargs) (cunusht/geometry.py:19-27)."""
    fn = getattr(Geom, "get_" + geometry[0] + "_geometry", None)
    if fn is None:
        raise ValueError(f"Geometry {geometry[0]} not found, available: {Geom.get_supported_geometries()}")
    # the transformers also read the band limit from the same dict
    # (GPU_nufft_transformer.py:138-141): pass each geometry only its own arguments
    params = inspect.signature(fn).parameters
    return fn(**{k: v for k, v in geometry[1].items() if k in params})
