"""CPU oracle for the nuSHT / lensing path -- TEST INFRASTRUCTURE ONLY.

Importable by ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline``
leg of ``bench.py`` only, as the checker; the product never imports it.

* ``oracle.oracle``  numpy restatement (geometry, alm layout, spin-weighted
  harmonics, direct synthesis/adjoint, pointing, rotation angle, doubling).
* ``oracle.direct``  ctypes binding of ``direct.c``: the same exact direct
  summation in C + OpenMP, for sizes numpy cannot finish in seconds.
* ``FastCPU``        ctypes binding of ``fastcpu.c``: the reference's lensing
  algorithm (recursion SHT + FFTs + ES-kernel nuFFT) in FP64 C + OpenMP, the
  timed CPU baseline and a full-map cross-check.
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


_SO_FAST = os.path.join(_HERE, "liboracle_fastcpu.so")


def build_fastcpu(force: bool = False) -> str:
    """Compile fastcpu.c with gcc + OpenMP into oracle/liboracle_fastcpu.so."""
    src = os.path.join(_HERE, "fastcpu.c")
    if force or not os.path.exists(_SO_FAST) or os.path.getmtime(_SO_FAST) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-fcx-limited-range", "-shared", src, "-o",
                               _SO_FAST, "-lm"])
    return _SO_FAST


_lib = None
_fast = None


def _load_fast():
    global _fast
    if _fast is None:
        build_fastcpu()
        lib = ctypes.CDLL(_SO_FAST)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.fc_plan_create.restype = ctypes.c_void_p
        lib.fc_plan_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int,
                                       ctypes.c_double]
        lib.fc_plan_destroy.argtypes = [ctypes.c_void_p]
        lib.fc_plan_npix.restype = ctypes.c_long
        lib.fc_plan_npix.argtypes = [ctypes.c_void_p]
        lib.fc_lensing.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, ctypes.c_int]
        lib.fc_last_pointing.argtypes = [ctypes.c_void_p, dp]
        _fast = lib
    return _fast


class FastCPU:
    """FP64 CPU lensing solver on a GL-type geometry (rings of nphi pixels)."""

    def __init__(self, lmax, theta, phi0, nphi, eps, max_spin=2):
        self.lib = _load_fast()
        th = np.ascontiguousarray(theta, dtype=np.float64)
        p0 = np.ascontiguousarray(phi0, dtype=np.float64)
        self.lmax, self.nphi, self.nring = lmax, nphi, th.size
        self.plan = self.lib.fc_plan_create(lmax, max_spin, th.size, _p(th), _p(p0), nphi, eps)
        self.npix = self.lib.fc_plan_npix(self.plan)

    def lensing(self, gclm, dlm_scaled, spin, dclm_scaled=None, nthreads=0):
        g = np.ascontiguousarray(np.atleast_2d(gclm), dtype=np.complex128)
        d = np.ascontiguousarray(dlm_scaled, dtype=np.complex128).reshape(-1)
        c = np.ascontiguousarray(dclm_scaled, dtype=np.complex128).reshape(-1) if dclm_scaled is not None else None
        out = np.zeros((2, self.npix) if spin else (self.npix,))
        rc = self.lib.fc_lensing(self.plan, spin, g.shape[0], _p(g.view(np.float64)), _p(d.view(np.float64)),
                                 _p(c.view(np.float64)) if c is not None else None, _p(out), nthreads)
        if rc:
            raise ValueError("fc_lensing: spin outside the plan")
        return out

    def last_pointing(self):
        ptg = np.zeros((2, self.npix))
        self.lib.fc_last_pointing(self.plan, _p(ptg))
        return ptg

    def close(self):
        if self.plan:
            self.lib.fc_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


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
