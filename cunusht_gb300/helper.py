"""Helpers of the reference's helper module (cunusht/helper_GPU.py) that sit
on the lensing path: spin raising / lowering response coefficients and the
magnification-matrix determinant for inverse lensing."""
from __future__ import annotations

import numpy as np

from .geometry import Geom, get_geom


def get_spin_raise(s: int, lmax: int) -> np.ndarray:
    """sqrt((l - s)(l + s + 1)) for |s| <= l <= lmax, else 0 (helper_GPU.py:92-100)."""
    ret = np.zeros(lmax + 1, dtype=float)
    l = np.arange(abs(s), lmax + 1, dtype=float)
    ret[abs(s):] = np.sqrt((l - s) * (l + s + 1))
    return ret


def get_spin_lower(s: int, lmax: int) -> np.ndarray:
    """-sqrt((l + s)(l - s + 1)) for |s| <= l <= lmax, else 0 (helper_GPU.py:102-110)."""
    ret = np.zeros(lmax + 1, dtype=float)
    l = np.arange(abs(s), lmax + 1, dtype=float)
    ret[abs(s):] = -np.sqrt((l + s) * (l - s + 1))
    return ret


_plans: dict = {}


def dlm2A(dlm, lmax_dlm: int, mmax_dlm: int, geom, nthreads=None, dclm=None):
    """Determinant of the magnification matrix of the deflection (gradient
    dlm = sqrt(l(l+1)) phi_lm, optional curl dclm) on the pixelisation
    ``geom`` (a Geom or a geominfo tuple such as ('gl', {'lmax': L})), on the
    GPU (helper_GPU.py:113-161; nthreads is accepted for the reference's
    signature and unused).  Returns a (npix,) torch CUDA tensor."""
    from .transformer import GPU_SHT_transformer
    assert mmax_dlm == lmax_dlm, "mmax must equal lmax"
    geominfo = geom if not isinstance(geom, Geom) else None
    if geominfo is None:
        raise TypeError("dlm2A takes the geometry as a geominfo tuple, e.g. ('gl', {'lmax': L})")
    key = (repr(geominfo), lmax_dlm)
    T = _plans.get(key)
    if T is None:
        gi = (geominfo[0], dict(geominfo[1], lmax=lmax_dlm))
        get_geom(gi)
        T = GPU_SHT_transformer(gi)
        _plans[key] = T
    return T.dlm2A(dlm, dclm)
