"""GPU nuSHT / lensing transformer with the surface of the reference's
``GPU_cufinufft_transformer`` (cunusht/deflection/GPU_nufft_transformer.py:107-680).

Arrays in and out are torch CUDA tensors (cupy arrays and host arrays are
accepted and moved to the device, with the reference's warning for host
arrays).  All compute runs in the CUDA library through the C ABI on the current
torch stream; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .geometry import get_geom
from .utils import Alm

_PREC = {"auto": _lib.PREC_AUTO, "fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def to_device(x, name: str, dtype: torch.dtype | None = None, warn: bool = True,
              contiguous: bool = True) -> torch.Tensor:
    """Device tensor view of x (torch / cupy / numpy) of dtype, contiguous
    unless ``contiguous`` is False (the caller then handles strides)."""
    if isinstance(x, torch.Tensor) and x.is_cuda:
        t = x
    elif hasattr(x, "__cuda_array_interface__"):
        t = torch.as_tensor(x, device="cuda")
    else:
        if warn:
            print(f"WARNING: {name} not on the device and has automatically been transferred to device. "
                  "This may reduce performance. Consider passing a device array instead")
        t = torch.as_tensor(np.asarray(x), device="cuda")
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    return t.contiguous() if contiguous else t


def _loc_args(loc: torch.Tensor, npts_hint: int | None = None):
    """(pointer tensor, npts, layout) for a point array: (npts, 2) rows of
    (theta, phi) -> layout 0; (2, npts) or a transposed (npts, 2) view of a
    planar (2, npts) array -> layout 1."""
    if loc.dim() != 2:
        raise ValueError(f"loc must be 2-d, got shape {tuple(loc.shape)}")
    if loc.shape[1] == 2 and loc.is_contiguous():
        return loc, loc.shape[0], 0
    if loc.shape[1] == 2 and loc.t().is_contiguous():
        return loc.t(), loc.shape[0], 1
    if loc.shape[0] == 2:
        t = loc.contiguous()
        return t, t.shape[1], 1
    return loc.contiguous(), loc.shape[0], 0


class GPU_cufinufft_transformer:
    """Transformer with the reference's constructor and methods; see the
    C ABI (include/cunusht_gb300.h) for the math of each call."""

    def __init__(self, geominfo_deflection, shttransformer_desc="shtns", nuFFTtype=None, epsilon=None,
                 precision: str = "auto", max_spin: int = 2):
        if nuFFTtype:
            assert epsilon is not None, "epsilon must be provided if planned is True"
        if shttransformer_desc not in ("shtns", "ducc", "cunusht"):
            raise ValueError('shttransformer_desc must be either "ducc" or "shtns" or "cunusht"')
        self.backend = "GPU"
        self.shttransformer_desc = shttransformer_desc
        self.nuFFTtype = nuFFTtype
        self.geominfo = geominfo_deflection
        self.geom = get_geom(geominfo_deflection)
        self.lmax = int(geominfo_deflection[1]["lmax"])
        self.mmax = int(geominfo_deflection[1].get("mmax", self.lmax))
        self.execmode = "normal"
        self.dlm_scaled = None
        self.dclm_scaled = None
        self.ptg = None
        self.gamma = None
        self.ret = {}
        self.timings = {}
        self.precision = precision
        self.max_spin = max_spin
        self.epsilon = epsilon
        self.single_prec = bool(epsilon is not None and epsilon > 1e-6)
        self._plan = None
        self._lib = _lib.load()
        if epsilon is not None:
            self.plan(epsilon, nuFFTtype or 1)

    # -------------------------------------------------------------- plan
    def plan(self, epsilon, nuFFTtype=1):
        """Create the device plan (grid sizes, kernel tables, workspace) for
        this accuracy (GPU_nufft_transformer.py:227-246)."""
        self._destroy()
        g = self.geom
        th = np.ascontiguousarray(g.theta, dtype=np.float64)
        p0 = np.ascontiguousarray(g.phi0, dtype=np.float64)
        nph = np.ascontiguousarray(g.nph, dtype=np.int64)
        ofs = np.ascontiguousarray(g.ofs, dtype=np.int64)
        h = ctypes.c_void_p()
        torch.cuda.init()
        _lib.check(self._lib.cunusht_plan_create(
            ctypes.byref(h), self.lmax, float(epsilon), _PREC[self.precision], self.max_spin, th.size,
            th.ctypes.data, p0.ctypes.data, nph.ctypes.data, ofs.ctypes.data))
        self._plan = h
        if self.mmax != self.lmax:
            _lib.check(self._lib.cunusht_plan_set_mmax(h, self.mmax))
        self.epsilon = epsilon
        self.single_prec = epsilon > 1e-6
        info = (ctypes.c_int64 * 10)()
        self._lib.cunusht_plan_info(h, info, 10)
        self.info = dict(zip(["npix", "ntheta_torus", "nphi_torus", "ntheta_fine", "nphi_fine", "kernel_width",
                              "fine_rows", "workspace_bytes", "precision", "nalm"], list(info)))
        self.ptg = None
        self.dlm_scaled = None

    def _destroy(self):
        if getattr(self, "_plan", None) is not None:
            self._lib.cunusht_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass

    def _ensure_plan(self, epsilon):
        if self.nuFFTtype:
            assert epsilon is None or epsilon == self.epsilon, \
                "expected epsilon = {} as set during initialisation of nuFFT plan, but is {}".format(self.epsilon, epsilon)
            epsilon = self.epsilon
        else:
            assert epsilon is not None or self.epsilon is not None, "epsilon must be provided if not planned"
            epsilon = self.epsilon if epsilon is None else epsilon
        if self._plan is None or epsilon != self.epsilon:
            self.plan(epsilon)
        return epsilon

    def _check_lm(self, lmax, mmax):
        """lmax must be the plan's; mmax <= lmax selects the alm layout of the
        call (healpy m-major truncated at mmax) -- one mmax for every alm of
        the call, gclm and dlm alike.  The reference's GPU transformer only
        takes mmax == lmax (GPU_nufft_transformer.py:389-390)."""
        assert lmax == self.lmax, "Expected lmax={}. lmax must be same as during init, but is {}".format(self.lmax, lmax)
        mmax = self.lmax if mmax is None else int(mmax)
        assert 0 <= mmax <= self.lmax, "mmax must be in [0, lmax={}], got {}".format(self.lmax, mmax)
        if mmax != self.mmax:
            self.mmax = mmax
            if self._plan is not None:
                _lib.check(self._lib.cunusht_plan_set_mmax(self._plan, mmax))
                self.dlm_scaled = None  # the pointing cache was for another layout

    @property
    def nalm(self) -> int:
        return Alm.getsize(self.lmax, self.mmax)

    def npix(self) -> int:
        return self.geom.npix()

    def get_grid_uniform(self) -> torch.Tensor:
        """(2, npix) colatitude / longitude of every pixel of the geometry."""
        th, ph = self.geom.pixels()
        return torch.as_tensor(np.stack([th, ph]), device="cuda")

    # -------------------------------------------------------------- alm helpers
    def _alm_in(self, alm, name, spin):
        a = to_device(alm, name)
        if not a.is_complex():
            raise TypeError(f"{name} must be complex, got {a.dtype}")
        a = a.reshape(-1, self.nalm) if a.dim() > 1 or a.numel() != self.nalm else a.reshape(1, self.nalm)
        ncomp = a.shape[0]
        if spin == 0 and ncomp != 1:
            raise ValueError(f"spin 0 expects one alm array, got {ncomp}")
        if ncomp > 2:
            raise ValueError(f"at most 2 alm components, got {ncomp}")
        dt = _lib.F32 if a.dtype == torch.complex64 else _lib.F64
        if a.dtype not in (torch.complex64, torch.complex128):
            a = a.to(torch.complex128)
            dt = _lib.F64
        return a.contiguous(), ncomp, dt

    # -------------------------------------------------------------- transforms
    def nusht2d2(self, lmax, mmax, alm, loc, pointmap=None, epsilon=None, verbose=0, spin=0, gamma=None,
                 out_dtype=torch.float64):
        """alm -> values at loc (npts, 2) [theta, phi]: a new array, spin 0
        (npts,), spin s (2, npts) = (Q, U) (GPU_nufft_transformer.py:386-435)."""
        self._check_lm(lmax, mmax)
        self._ensure_plan(epsilon)
        a, ncomp, adt = self._alm_in(alm, "alm", spin)
        assert loc is not None, "loc must be provided"
        loc_t, npts, layout = _loc_args(to_device(loc, "loc", torch.float64, contiguous=False))
        out = torch.empty((npts,) if spin == 0 else (2, npts), dtype=out_dtype, device="cuda")
        odt = _lib.F32 if out_dtype == torch.float32 else _lib.F64
        g = None
        if gamma is not None and spin:
            g = to_device(gamma, "gamma", torch.float64)
        _lib.check(self._lib.cunusht_nusht2d2(
            self._plan, spin, ncomp, a.data_ptr(), adt, loc_t.data_ptr(), npts, layout,
            g.data_ptr() if g is not None else None, out.data_ptr(), odt, _stream()))
        return out

    def nusht2d1(self, lmax, mmax, pointmap, loc, epsilon=None, alm=None, verbose=0, spin=0, ncomp=None,
                 gamma=None, alm_dtype=torch.complex128):
        """values at loc -> alm, the exact adjoint of nusht2d2
        (GPU_nufft_transformer.py:439-484).  Returns a new alm array."""
        self._check_lm(lmax, mmax)
        self._ensure_plan(epsilon)
        m = to_device(pointmap, "pointmap")
        if m.is_complex():
            m = m.real.contiguous()
        if m.dtype not in (torch.float32, torch.float64):
            m = m.to(torch.float64)
        mdt = _lib.F32 if m.dtype == torch.float32 else _lib.F64
        loc_t, npts, layout = _loc_args(to_device(loc, "loc", torch.float64, contiguous=False))
        if spin == 0:
            m = m.reshape(-1)
            assert m.numel() == npts, (m.numel(), npts)
            ncomp = 1
        else:
            m = m.reshape(2, -1).contiguous()
            assert m.shape[1] == npts, (m.shape, npts)
            ncomp = 2 if ncomp is None else ncomp
        out = torch.empty((ncomp, self.nalm), dtype=alm_dtype, device="cuda")
        odt = _lib.F32 if alm_dtype == torch.complex64 else _lib.F64
        g = to_device(gamma, "gamma", torch.float64) if (gamma is not None and spin) else None
        _lib.check(self._lib.cunusht_nusht2d1(
            self._plan, spin, ncomp, m.data_ptr(), mdt, loc_t.data_ptr(), npts, layout,
            g.data_ptr() if g is not None else None, out.data_ptr(), odt, _stream()))
        return out[0] if spin == 0 else out

    def dlm2pointing(self, dlm_scaled, mmax_dlm, verbose=0, single_prec=False, dclm_scaled=None):
        """Deflected (theta', phi') of every pixel, (2, npix) float64
        (GPU_nufft_transformer.py:344-351); the rotation angle is kept in
        ``self.gamma``."""
        self._check_lm(self.lmax, mmax_dlm)
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        d, _, ddt = self._alm_in(dlm_scaled, "dlm_scaled", 0)
        c = None
        if dclm_scaled is not None:
            c = to_device(dclm_scaled, "dclm_scaled", d.dtype).reshape(-1)
        npix = self.npix()
        ptg = torch.empty((2, npix), dtype=torch.float64, device="cuda")
        gamma = torch.empty((npix,), dtype=torch.float64, device="cuda")
        _lib.check(self._lib.cunusht_dlm2pointing(
            self._plan, d.data_ptr(), c.data_ptr() if c is not None else None, ddt, ptg.data_ptr(),
            gamma.data_ptr(), _stream()))
        self.gamma = gamma
        return ptg

    def synthesis(self, alm, out=None, lmax=None, mmax=None, spin=0):
        """Spin-s synthesis on the pointing geometry (GPU_nufft_transformer.py:356-367)."""
        lmax = self.lmax if lmax is None else lmax
        self._check_lm(lmax, self.lmax if mmax is None else mmax)
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        a, ncomp, adt = self._alm_in(alm, "alm", spin)
        npix = self.npix()
        res = torch.empty((npix,) if spin == 0 else (2, npix), dtype=torch.float64, device="cuda")
        _lib.check(self._lib.cunusht_synthesis(self._plan, spin, ncomp, a.data_ptr(), adt, res.data_ptr(), _stream()))
        return res

    def adjoint_synthesis(self, synthmap, lmax=None, mmax=None, out=None, spin=0, ncomp=None):
        """Adjoint of ``synthesis`` (no quadrature weights) (GPU_nufft_transformer.py:372-383)."""
        lmax = self.lmax if lmax is None else lmax
        self._check_lm(lmax, self.lmax if mmax is None else mmax)
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        m = to_device(synthmap, "synthmap", torch.float64)
        ncomp = (1 if spin == 0 else 2) if ncomp is None else ncomp
        res = torch.empty((ncomp, self.nalm), dtype=torch.complex128, device="cuda")
        _lib.check(self._lib.cunusht_adjoint_synthesis(self._plan, spin, ncomp, m.data_ptr(), res.data_ptr(),
                                                       _lib.F64, _stream()))
        return res[0] if spin == 0 else res

    def synthesis_der1(self, alm, out=None):
        """(d/dtheta, 1/sin(theta) d/dphi) of a scalar field on the pointing
        geometry, as SHTns synth_grad (GPU_sht_transformer.py:88-97)."""
        a = to_device(alm, "alm", torch.complex128).reshape(-1)
        ll = torch.arange(self.lmax + 1, dtype=torch.float64, device="cuda")
        fl = torch.sqrt(ll * (ll + 1))
        mi = torch.repeat_interleave(torch.arange(self.lmax + 1, device="cuda"),
                                     torch.arange(self.lmax + 1, 0, -1, device="cuda"))
        li = torch.arange(self.nalm, device="cuda") - (mi * (2 * self.lmax + 1 - mi)) // 2
        return GPU_cufinufft_transformer.synthesis(self, (a * fl[li])[None], spin=1)

    def set_pts(self, ptg):
        self.ptg = to_device(ptg, "ptg", torch.float64)

    # -------------------------------------------------------------- profiling
    def profile(self, enable: bool = True):
        """Bracket every stage launch with CUDA events on the caller's stream."""
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        _lib.check(self._lib.cunusht_plan_set_profiling(self._plan, int(enable)))

    def stage_times(self) -> dict:
        """{stage: (total ms, launches)} since the last call (then reset)."""
        ms = (ctypes.c_double * _lib.NSTAGE)()
        cnt = (ctypes.c_int64 * _lib.NSTAGE)()
        _lib.check(self._lib.cunusht_plan_stage_times(self._plan, ms, cnt, _lib.NSTAGE))
        return {n: (ms[i], cnt[i]) for i, n in enumerate(_lib.STAGES) if cnt[i]}

    def set_spreading(self, method: str = "strips", deterministic: bool = False, max_points: int | None = None):
        """Spreading of the type-1 nuFFT (nusht2d1, lenmap2gclm), the choice of
        cuFINUFFT's gpu_method / gpu_sort in the reference's plan
        (GPU_nufft_transformer.py:242-246): "strips" (default; points in ring
        order, the lensing pointing) or "bins" (bin-sorted shared-memory
        spreading, points in any order, up to max_points per request,
        default the pixel count); deterministic=True accumulates in exact
        int64 fixed point, so results do not depend on the order of atomics."""
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        m = {"strips": 0, "bins": 1}[method]
        _lib.check(self._lib.cunusht_plan_set_spreading(self._plan, m, int(bool(deterministic)),
                                                        int(max_points or 0)))

    def reserve_batch(self, max_batch: int):
        """Allocate the per-request workspace for lensing_batch (once)."""
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        _lib.check(self._lib.cunusht_plan_reserve_batch(self._plan, int(max_batch)))
        self.batch_cap = max(getattr(self, "batch_cap", 0), int(max_batch))

    def lensing_batch(self, gclm: torch.Tensor, dlm_scaled: torch.Tensor, spin: int, out: torch.Tensor | None = None,
                      ptg: torch.Tensor | None = None, gamma: torch.Tensor | None = None,
                      dclm_scaled: torch.Tensor | None = None) -> torch.Tensor:
        """nreq lensing solves in one batched pass (served form).
        gclm (nreq, ncomp, nalm) complex128, dlm_scaled (nreq, nalm) complex128
        -> (nreq, 2, npix) Q/U (spin 2) or (nreq, npix) (spin 0)."""
        g = to_device(gclm, "gclm", torch.complex128)
        if g.dim() == 2:
            g = g[:, None, :]
        nreq, ncomp = g.shape[0], g.shape[1]
        d = to_device(dlm_scaled, "dlm_scaled", torch.complex128).reshape(nreq, self.nalm)
        c = to_device(dclm_scaled, "dclm_scaled", torch.complex128).reshape(nreq, self.nalm) if dclm_scaled is not None else None
        if getattr(self, "batch_cap", 0) < nreq:
            self.reserve_batch(nreq)
        npix = self.npix()
        if out is None:
            out = torch.empty((nreq, 2, npix) if spin else (nreq, npix), dtype=torch.float64, device="cuda")
        _lib.check(self._lib.cunusht_lensing_batch(
            self._plan, nreq, spin, ncomp, g.data_ptr(), d.data_ptr(), c.data_ptr() if c is not None else None,
            ptg.data_ptr() if ptg is not None else None, gamma.data_ptr() if gamma is not None else None,
            out.data_ptr(), _lib.F32 if out.dtype == torch.float32 else _lib.F64, _stream()))
        return out

    def delensing_batch(self, lenmap: torch.Tensor, dlm_scaled: torch.Tensor, spin: int, ncomp: int | None = None,
                        out: torch.Tensor | None = None, ptg: torch.Tensor | None = None,
                        gamma: torch.Tensor | None = None, dclm_scaled: torch.Tensor | None = None) -> torch.Tensor:
        """nreq delensing solves (lenmap2gclm) in one batched pass (served form).
        lenmap (nreq, 2, npix) (spin s) or (nreq, npix) (spin 0) float64,
        dlm_scaled (nreq, nalm) complex128 -> (nreq, ncomp, nalm) complex128."""
        m = to_device(lenmap, "lenmap")
        if m.dtype not in (torch.float32, torch.float64):
            m = m.to(torch.float64)
        nreq = m.shape[0]
        ncomp = (2 if spin else 1) if ncomp is None else ncomp
        d = to_device(dlm_scaled, "dlm_scaled", torch.complex128).reshape(nreq, self.nalm)
        c = to_device(dclm_scaled, "dclm_scaled", torch.complex128).reshape(nreq, self.nalm) if dclm_scaled is not None else None
        if getattr(self, "batch_cap", 0) < nreq:
            self.reserve_batch(nreq)
        if out is None:
            out = torch.empty((nreq, ncomp, self.nalm), dtype=torch.complex128, device="cuda")
        _lib.check(self._lib.cunusht_delensing_batch(
            self._plan, nreq, spin, ncomp, m.data_ptr(), _lib.F32 if m.dtype == torch.float32 else _lib.F64,
            d.data_ptr(), c.data_ptr() if c is not None else None, ptg.data_ptr() if ptg is not None else None,
            gamma.data_ptr() if gamma is not None else None, out.data_ptr(), _stream()))
        return out

    def lensing_solve(self, gclm: torch.Tensor, dlm_scaled: torch.Tensor, out: torch.Tensor, ptg: torch.Tensor,
                      gamma: torch.Tensor, spin: int, dclm_scaled: torch.Tensor | None = None):
        """One uncached lensing solve on device tensors (dlm2pointing + nusht2d2
        with rotation), no host synchronisation: the serving / benchmark step."""
        ncomp = 1 if gclm.dim() == 1 else gclm.shape[0]
        adt = _lib.F32 if gclm.dtype == torch.complex64 else _lib.F64
        s = _stream()
        _lib.check(self._lib.cunusht_dlm2pointing(self._plan, dlm_scaled.data_ptr(),
                                                  dclm_scaled.data_ptr() if dclm_scaled is not None else None,
                                                  _lib.F64 if dlm_scaled.dtype == torch.complex128 else _lib.F32,
                                                  ptg.data_ptr(), gamma.data_ptr(), s))
        odt = _lib.F32 if out.dtype == torch.float32 else _lib.F64
        _lib.check(self._lib.cunusht_nusht2d2(self._plan, spin, ncomp, gclm.data_ptr(), adt, ptg.data_ptr(),
                                              ptg.shape[1], 1, gamma.data_ptr() if spin else None,
                                              out.data_ptr(), odt, s))
        return out

    def delensing_solve(self, lenmap: torch.Tensor, dlm_scaled: torch.Tensor, alm_out: torch.Tensor,
                        ptg: torch.Tensor, gamma: torch.Tensor, spin: int,
                        dclm_scaled: torch.Tensor | None = None):
        """One uncached adjoint lensing solve on device tensors (dlm2pointing +
        nusht2d1 with the inverse rotation), no host synchronisation.
        lenmap (npix,) or (2, npix) float64 -> alm_out (ncomp, nalm)."""
        s = _stream()
        _lib.check(self._lib.cunusht_dlm2pointing(self._plan, dlm_scaled.data_ptr(),
                                                  dclm_scaled.data_ptr() if dclm_scaled is not None else None,
                                                  _lib.F64, ptg.data_ptr(), gamma.data_ptr(), s))
        ncomp = 1 if (spin == 0 or alm_out.dim() == 1) else alm_out.shape[0]
        mdt = _lib.F32 if lenmap.dtype == torch.float32 else _lib.F64
        adt = _lib.F32 if alm_out.dtype == torch.complex64 else _lib.F64
        _lib.check(self._lib.cunusht_nusht2d1(self._plan, spin, ncomp, lenmap.data_ptr(), mdt, ptg.data_ptr(),
                                              ptg.shape[1], 1, gamma.data_ptr() if spin else None,
                                              alm_out.data_ptr(), adt, s))
        return alm_out

    # -------------------------------------------------------------- lensing
    def _spin_of(self, gclm, spin):
        if spin is not None:
            return spin
        return 0 if (getattr(gclm, "ndim", 1) == 1 or gclm.shape[0] == 1) else 2

    def _pointing(self, ptg, dlm_scaled, dclm_scaled, lmax, verbose):
        if ptg is not None:
            ptg = to_device(ptg, "ptg", torch.float64)
            if ptg.shape[0] != 2 and ptg.shape[-1] == 2:
                ptg = ptg.t().contiguous()
            self.ptg = ptg
            return self.ptg, None
        assert dlm_scaled is not None or self.dlm_scaled is not None, "Need to provide dlm_scaled if ptg is None"
        d = to_device(dlm_scaled, "dlm_scaled") if dlm_scaled is not None else self.dlm_scaled
        c = to_device(dclm_scaled, "dclm_scaled") if dclm_scaled is not None else None
        same = (self.dlm_scaled is not None and self.ptg is not None and self.gamma is not None
                and self.dlm_scaled.shape == d.shape and torch.equal(self.dlm_scaled, d)
                and ((c is None and self.dclm_scaled is None) or
                     (c is not None and self.dclm_scaled is not None and torch.equal(self.dclm_scaled, c))))
        if not same:
            self.dlm_scaled = d.clone()
            self.dclm_scaled = c.clone() if c is not None else None
            self.ptg = self.dlm2pointing(d, self.mmax, verbose, dclm_scaled=c)
        return self.ptg, self.gamma

    def _timed(self, name, fn):
        if self.execmode != "timing":
            return fn()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        r = fn()
        e.record()
        e.synchronize()
        self.timings[name] = s.elapsed_time(e) * 1e-3
        return r

    def gclm2lenmap(self, gclm, lmax, mmax, ptg=None, dlm_scaled=None, epsilon=None, lenmap=None, verbose=1,
                    execmode="normal", runid=None, GPUdesc="", spin=None, polrot=True, dclm_scaled=None):
        """Lensed map from unlensed alm and the deflection
        (GPU_nufft_transformer.py:487-578; spin-s semantics of
        CPU_nufft_transformer.py:430-484 incl. the exp(i s gamma) rotation)."""
        assert execmode in ["normal", "debug", "timing"]
        self.execmode = execmode
        self.runid, self.GPUdesc = runid, GPUdesc
        self._check_lm(lmax, mmax)
        epsilon = self._ensure_plan(epsilon)
        spin = self._spin_of(gclm, spin)
        ptg, gamma = self._timed("dlm2pointing", lambda: self._pointing(ptg, dlm_scaled, dclm_scaled, lmax, verbose))
        g = gamma if (spin and polrot) else None
        # complex64 alm give float32 maps (the single-precision configuration),
        # complex128 alm float64 maps
        odt = torch.float32 if (isinstance(gclm, torch.Tensor) and gclm.dtype == torch.complex64) else torch.float64
        res = self._timed("nusht2d2", lambda: self.nusht2d2(lmax, mmax, gclm, ptg.t(), epsilon=epsilon, spin=spin,
                                                            gamma=g, out_dtype=odt))
        if execmode == "debug":
            self.ret = {"dlm2pointing": ptg, "gamma": gamma, "nusht2d2": res}
            return self.ret
        return res

    def lenmap2gclm(self, lenmap, dlm_scaled, gclm=None, lmax=None, mmax=None, epsilon=None, ptg=None, verbose=1,
                    execmode="normal", runid=None, GPUdesc="", spin=None, polrot=True, dclm_scaled=None, ncomp=None):
        """Adjoint lensing, values on the lensed grid -> alm
        (GPU_nufft_transformer.py:581-673); exact adjoint of gclm2lenmap."""
        assert execmode in ["normal", "debug", "timing"]
        self.execmode = execmode
        self.runid, self.GPUdesc = runid, GPUdesc
        lmax = self.lmax if lmax is None else lmax
        mmax = self.lmax if mmax is None else mmax
        self._check_lm(lmax, mmax)
        epsilon = self._ensure_plan(epsilon)
        lm = to_device(lenmap, "lenmap")
        if gclm is not None and hasattr(gclm, "dtype") and hasattr(lm, "dtype"):
            real_of = {torch.complex128: torch.float64, torch.complex64: torch.float32}
            gdt = gclm.dtype if isinstance(gclm, torch.Tensor) else None
            if gdt in real_of:
                ldt = lm.real.dtype if lm.is_complex() else lm.dtype
                assert ldt == real_of[gdt], \
                    "lenmap and gclm must have same precision, but are {} and {}".format(lm.dtype, gdt)
        if spin is None:
            spin = 0 if (lm.dim() == 1 or lm.shape[0] == 1) else 2
        if spin == 0:
            lm = lm.reshape(-1) if lm.dim() == 1 else lm[0]
        ptg_, gamma = self._timed("dlm2pointing", lambda: self._pointing(ptg, dlm_scaled, dclm_scaled, lmax, verbose))
        g = gamma if (spin and polrot) else None
        adt = torch.complex64 if (isinstance(gclm, torch.Tensor) and gclm.dtype == torch.complex64) else torch.complex128
        res = self._timed("nusht2d1", lambda: self.nusht2d1(lmax, mmax, lm, ptg_.t(), epsilon=epsilon, spin=spin,
                                                            gamma=g, ncomp=ncomp, alm_dtype=adt))
        if execmode == "debug":
            self.ret = {"dlm2pointing": ptg_, "gamma": gamma, "nusht2d1": res}
            return self.ret
        return res

    def dlm2A(self, dlm, dclm=None) -> torch.Tensor:
        """Determinant of the magnification matrix on the pointing geometry
        from the gradient deflection alm dlm = sqrt(l(l+1)) phi_lm (and the
        curl dclm), helper_GPU.py:113-161; (npix,) float64."""
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        d, _, ddt = self._alm_in(dlm, "dlm", 0)
        c = to_device(dclm, "dclm", d.dtype).reshape(-1) if dclm is not None else None
        A = torch.empty((self.npix(),), dtype=torch.float64, device="cuda")
        _lib.check(self._lib.cunusht_dlm2A(self._plan, d.data_ptr(), c.data_ptr() if c is not None else None, ddt,
                                           A.data_ptr(), _stream()))
        return A

    def gclm2lenpixs(self, gclm, mmax, spin, pixs, polrot=True, ptg=None):
        """The remapped field at the pixels ``pixs`` by exact direct summation
        at their deflected positions (CPU_nufft_transformer.py:531-558):
        spin 0 -> (npixs,), spin s -> (Q, U).  Uses ``ptg`` or the pointing of
        the last lensing call on this transformer."""
        assert spin >= 0, spin
        if mmax is not None:
            self._check_lm(self.lmax, mmax)
        if ptg is None:
            assert self.ptg is not None, "no pointing yet: call dlm2pointing / gclm2lenmap first or pass ptg"
            ptg = self.ptg
        ptg = to_device(ptg, "ptg", torch.float64)
        if ptg.shape[0] != 2:
            ptg = ptg.t().contiguous()
        pix = torch.as_tensor(np.asarray(pixs), device="cuda", dtype=torch.long).reshape(-1)
        loc = ptg[:, pix].contiguous()                          # (2, n) planar
        a, ncomp, adt = self._alm_in(gclm, "gclm", spin)
        n = pix.numel()
        out = torch.empty((2, n) if spin else (n,), dtype=torch.float64, device="cuda")
        g = None
        if spin and polrot:
            assert self.gamma is not None, "no rotation angle yet: call dlm2pointing / gclm2lenmap first"
            g = self.gamma[pix].contiguous()
        _lib.check(self._lib.cunusht_synth_points(self._plan, spin, ncomp, a.data_ptr(), adt, loc.data_ptr(), n, 1,
                                                  g.data_ptr() if g is not None else None, out.data_ptr(),
                                                  _stream()))
        if spin:
            return out[0], out[1]
        return out

    @staticmethod
    def hashdict():
        """Compatibility with delensalot (GPU_nufft_transformer.py:676-680)."""
        return "GPU_cufinufft_transformer"


class GPU_SHT_transformer(GPU_cufinufft_transformer):
    """SHT-only mode (cunusht.py:75-76) with the surface of the reference's
    ``GPU_SHTns_transformer`` (cunusht/sht/GPU_sht_transformer.py:11-127):
    synthesis / synthesis_cupy, adjoint_synthesis_cupy, synthesis_der1 /
    synthesis_der1_cupy, analysis, adjoint_synthesis, map2alm, alm2map, with
    the reference's argument order.

    Maps follow SHTns's theta-contiguous grid as the reference sets it up
    (SHT_THETA_CONTIGUOUS, GPU_sht_transformer.py:21-37): spatial shape
    (nphi, nlat), flattened by ``synthesis``; ``synthesis_der1_cupy``
    returns ring-major planes as the reference's ``.T.flatten()`` does
    (:106-107).  Geometries whose rings differ in length (HEALPix, thinned
    grids) have no such grid and use ring-major (npix,) maps throughout.
    ``analysis`` / ``adjoint_synthesis`` / ``map2alm`` are SHTns ``analys``:
    the quadrature-weighted adjoint (exact inverse of the synthesis on a
    Gauss-Legendre grid at the band limit).  ``spin`` (default 0, the
    reference's scalar SHTns transforms) extends every method to spin 1, 2.
    Compute runs in the library (cunusht_synthesis, cunusht_analysis); the
    layout change is a device transpose."""

    def __init__(self, geominfo, nthreads=None, max_spin: int = 2):
        super().__init__(geominfo, nuFFTtype=None, epsilon=1e-7, max_spin=max_spin)
        nph = np.asarray(self.geom.nph, dtype=np.int64)
        self.nlat = int(nph.size)
        self.nphi = int(nph[0])
        self.theta_contiguous = bool(np.all(nph == nph[0]))
        self.spat_shape = (self.nphi, self.nlat) if self.theta_contiguous else (self.npix(),)
        self._ring_w = torch.as_tensor(np.ascontiguousarray(self.geom.weight, dtype=np.float64), device="cuda")

    # ring-major (..., npix) <-> the transformer's spatial layout
    def _to_spat(self, ring: torch.Tensor) -> torch.Tensor:
        if not self.theta_contiguous:
            return ring
        lead = ring.shape[:-1]
        return ring.reshape(*lead, self.nlat, self.nphi).transpose(-1, -2).contiguous()

    def _from_spat(self, m: torch.Tensor, spin: int) -> torch.Tensor:
        npix = self.npix()
        ncomp = 2 if spin else 1
        m = m.reshape(ncomp, npix) if spin else m.reshape(1, npix)
        if self.theta_contiguous:
            m = m.reshape(ncomp, self.nphi, self.nlat).transpose(-1, -2).reshape(ncomp, npix)
        return (m if spin else m[0]).contiguous()

    def synthesis_cupy(self, gclm, out=None, lmax=None, mmax=None, mode=None, nthreads=None, spin=0):
        """gclm -> map(s) of spatial shape (GPU_sht_transformer.py:56-62).
        ``out`` (optional, spatial shape) receives the result and is returned."""
        ring = GPU_cufinufft_transformer.synthesis(self, gclm, None, lmax, mmax, spin=spin)
        res = self._to_spat(ring)
        if out is not None:
            o = out if isinstance(out, torch.Tensor) else torch.as_tensor(out, device="cuda")
            if o.numel() == res.numel():
                o.copy_(res.reshape(o.shape))
                return o
        return res

    def synthesis(self, gclm, lmax=None, mmax=None, mode=None, nthreads=None, spin=0):
        """gclm -> flattened map(s) (GPU_sht_transformer.py:47-54): (npix,)
        for spin 0, (2, npix) for spin s."""
        res = self.synthesis_cupy(gclm, None, lmax, mmax, spin=spin)
        return res.reshape(2, -1) if spin else res.reshape(-1)

    def alm2map(self, gclm, **kwargs):
        return self.synthesis(gclm, **kwargs)

    def analysis(self, map, lmax=None, mmax=None, nthreads=None, alm=None, mode=None, spin=0, ncomp=None):
        """Quadrature-weighted adjoint, SHTns analys (GPU_sht_transformer.py:
        99-105): map(s) in spatial shape or flattened -> (1, nalm) for spin 0
        (np.atleast_2d of the reference), (ncomp, nalm) for spin s."""
        lmax = self.lmax if lmax is None else lmax
        self._check_lm(lmax, self.lmax if mmax is None else mmax)
        if self._plan is None:
            self._ensure_plan(self.epsilon if self.epsilon is not None else 1e-7)
        m = self._from_spat(to_device(map, "map", torch.float64), spin)
        ncomp = (1 if spin == 0 else 2) if ncomp is None else ncomp
        res = torch.empty((ncomp, self.nalm), dtype=torch.complex128, device="cuda")
        _lib.check(self._lib.cunusht_analysis(self._plan, spin, ncomp, m.data_ptr(), self._ring_w.data_ptr(),
                                              res.data_ptr(), _lib.F64, _stream()))
        return res

    def adjoint_synthesis(self, map, **kwargs):
        """As the reference's SHT mode (GPU_sht_transformer.py:108-118): the
        map reshaped to the spatial shape, then ``analysis``."""
        return self.analysis(map, **kwargs)

    def map2alm(self, m, **kwargs):
        return self.analysis(m, **kwargs)

    def adjoint_synthesis_cupy(self, synthmap, gclm=None, lmax=None, mmax=None, mode=None, nthreads=None, iw=None,
                               spin=0):
        """SHTns analys of synthmap * iw (GPU_sht_transformer.py:65-73):
        (nalm,) for spin 0, (ncomp, nalm) for spin s.  With iw = 1 / w (the
        inverse quadrature weights) this is the unweighted adjoint synthesis
        the nuFFT adjoint uses (GPU_nufft_transformer.py:265-269)."""
        m = to_device(synthmap, "synthmap", torch.float64)
        if iw is not None:
            w = to_device(iw, "iw", torch.float64, warn=False)
            m = (m.reshape(*((2,) if spin else ()), *self.spat_shape) * w).contiguous()
        res = self.analysis(m, lmax, mmax, spin=spin)
        return res if spin else res[0]

    def synthesis_der1(self, gclm, out=None, nthreads=None):
        """(d/dtheta, 1/sin(theta) d/dphi) of a scalar field, SHTns
        synth_grad, as flattened spatial maps (GPU_sht_transformer.py:76-86):
        (2, npix)."""
        ring = GPU_cufinufft_transformer.synthesis_der1(self, gclm)
        return self._to_spat(ring).reshape(2, -1)

    def synthesis_der1_cupy(self, gclm, out_theta=None, out_phi=None, nthreads=None):
        """The gradient of synthesis_der1 as ring-major planes (2, npix), the
        reference's ``.T.flatten()`` of the theta-contiguous grid
        (GPU_sht_transformer.py:88-97); out_theta / out_phi (optional)
        receive the planes."""
        ring = GPU_cufinufft_transformer.synthesis_der1(self, gclm)
        for o, r in ((out_theta, ring[0]), (out_phi, ring[1])):
            if isinstance(o, torch.Tensor) and o.is_contiguous() and o.numel() == r.numel():
                o.view(-1).copy_(r)
        return ring
