"""CPU oracle for the nuSHT / lensing path -- TEST INFRASTRUCTURE ONLY.

Importable by ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline``
leg of ``bench.py`` only, as the checker; the product never imports it.

* ``oracle.oracle``  numpy restatement (geometry, alm layout, spin-weighted
  harmonics, direct synthesis/adjoint, pointing, rotation angle, doubling).
* ``oracle.direct``  ctypes binding of ``direct.c``: the same exact direct
  summation in C + OpenMP, for sizes numpy cannot finish in seconds.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle_direct.so")


def build_oracle(force: bool = False) -> str:
    """Compile direct.c with gcc + OpenMP into oracle/liboracle_direct.so."""
    src = os.path.join(_HERE, "direct.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", src, "-o", _SO, "-lm"])
    return _SO


_lib = None


def _load():
    global _lib
    if _lib is None:
        build_oracle()
        lib = ctypes.CDLL(_SO)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_synth.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_long, dp, dp, dp, ctypes.c_int]
        lib.oracle_adjoint.argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_long, dp, dp, dp, dp, ctypes.c_int]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def synth_points_c(lmax, spin, alm, theta, phi, nthreads=0):
    """C version of oracle.synth_points (same conventions)."""
    lib = _load()
    alm = np.atleast_2d(np.ascontiguousarray(alm, dtype=np.complex128))
    G = np.ascontiguousarray(alm[0])
    C = np.ascontiguousarray(alm[1]) if (spin > 0 and alm.shape[0] > 1) else None
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    n = theta.size
    out = np.zeros(n if spin == 0 else 2 * n)
    lib.oracle_synth(lmax, spin, _p(G.view(np.float64)), _p(C.view(np.float64)) if C is not None else None,
                     n, _p(theta), _p(phi), _p(out), nthreads)
    return out if spin == 0 else out.reshape(2, n)


def adjoint_synth_points_c(lmax, spin, values, theta, phi, ncomp=2, nthreads=0):
    """C version of oracle.adjoint_synth_points (same conventions)."""
    from .oracle import nalm
    lib = _load()
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
    n = nalm(lmax)
    G = np.zeros(n, dtype=np.complex128)
    C = np.zeros(n, dtype=np.complex128) if spin > 0 else None
    lib.oracle_adjoint(lmax, spin, _p(v), theta.size, _p(theta), _p(phi), _p(G.view(np.float64)),
                       _p(C.view(np.float64)) if C is not None else None, nthreads)
    if spin == 0:
        return G
    return np.stack([G, C])[:ncomp]
