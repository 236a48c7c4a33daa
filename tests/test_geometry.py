"""Ring geometries on the CPU: HEALPix (12 nside^2 pixels, 4 nside - 1 rings
of 4 .. 4 nside pixels, N/S symmetric, equal area), longitude-thinned GL
(shorter rings near the poles, the GL colatitudes), Fejer-1 weights."""
import numpy as np

from cunusht_gb300.geometry import get_geom


def test_healpix():
    for nside in (1, 4, 32):
        g = get_geom(("healpix", {"nside": nside, "lmax": 2 * nside}))
        assert g.npix() == 12 * nside * nside and g.theta.size == 4 * nside - 1
        assert np.allclose(np.sort(g.theta), np.sort(np.pi - g.theta), atol=1e-14)
        assert abs(g.fsky() - 1.0) < 1e-14
        assert g.nph[0] == 4 and int(g.nph.max()) == 4 * nside
        assert np.all(np.diff(g.ofs.astype(np.int64)) == g.nph[:-1].astype(np.int64))
        # z of the equatorial ring nside: 2/3
        assert abs(np.cos(g.theta[nside - 1]) - 2.0 / 3.0) < 1e-14


def test_thinned_gl_and_f1():
    g = get_geom(("thingauss", {"lmax": 511, "smax": 2}))
    gl = get_geom(("gl", {"lmax": 511}))
    assert np.allclose(g.theta, gl.theta) and g.nph.min() < g.nph.max() <= gl.nph[0]
    assert abs(g.fsky() - 1.0) < 1e-12
    assert g.nph[0] < g.nph[g.theta.size // 2]  # thinned at the poles
    f = get_geom(("f1", {"ntheta": 40, "nphi": 81}))
    assert abs(f.fsky() - 1.0) < 1e-13
    # Fejer-1 integrates cos^2 exactly: int cos^2 theta dOmega = 4 pi / 3
    assert abs(np.sum(f.weight * f.nph * np.cos(f.theta) ** 2) - 4 * np.pi / 3) < 1e-12
