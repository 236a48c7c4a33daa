"""Seeded inputs of the reference-pinned parity cases (pointing and doubling),
shared by make_ref_golden.py (which runs the reference's own kernels on them)
and tests/test_gpu_reference_pin.py.  TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import numpy as np


def _gl(lmax: int, nphi: int):
    from oracle import oracle as orc
    th, ph0, nph, ofs, _ = orc.gl_geometry(lmax, nphi)
    return th, ph0, nph.astype(np.int64), ofs.astype(np.int64)


def _healpix(nside: int):
    import cunusht_gb300.geometry as g
    G = g.get_geom(("healpix", {"nside": nside}))
    return G.theta.copy(), G.phi0.copy(), G.nph.astype(np.int64), G.ofs.astype(np.int64)


# name -> (geometry, deflection rms per component [rad], seed)
# 7e-4 rad (2.5 arcmin) keeps every ring on the series branch of the
# reference kernel (pointing.cu:213-222), 0.05 rad puts rings on its exact
# branch (:204-211)
POINTING = {
    "gl47_small": (lambda: _gl(47, 95), 7e-4, 11),
    "gl31_large": (lambda: _gl(31, 63), 5e-2, 12),
    "healpix8_small": (lambda: _healpix(8), 7e-4, 13),
}

# theta / phi sizes of the Clenshaw-Curtis grid at lmax 31 ((good_size(lmax + 2)
# + 3) // 4 * 4, 2 good_size(lmax + 1); test_doublingGPU.py:100-101) and a small
# grid whose phi half-length is odd
DOUBLING = {"cc_l31": (36, 64, 21), "cc_small": (12, 20, 22)}


def pointing_inputs(name: str):
    geom, rms, seed = POINTING[name]
    th, ph0, nph, ofs = geom()
    rng = np.random.default_rng(seed)
    npix = int(nph.sum())
    return th, ph0, nph, ofs, rng.standard_normal(npix) * rms, rng.standard_normal(npix) * rms


def doubling_inputs(name: str, dtype):
    nt, nphi, seed = DOUBLING[name]
    rng = np.random.default_rng(seed)
    cc = rng.standard_normal((nt, nphi)).astype(dtype)             # ring-major CC map
    dm = rng.standard_normal((2 * nt - 2, nphi)).astype(dtype)     # ring-major torus map
    return nt, nphi, cc, dm
