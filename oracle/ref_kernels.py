"""The reference's own CUDA kernels, launched from oracle/_ref/*.cubin through
the CUDA driver API (ctypes on libcuda), for parity checks of the pointing and
doubling kernels against the reference itself.

TEST INFRASTRUCTURE ONLY: imported by tests/ and tests/golden/ scripts, never
by the product.  The cubins come from oracle/ref_build.py (the reference's
cunusht/c/pointing.cu and cunusht/c/doubling.cu compiled by nvcc).

Each launcher mirrors the reference's host wrapper: block size 256, the same
grid and the same kernel arguments:
  * pointing_lowmem   CUpointing_1Dto1D_lowmem (pointing.cu:228-255) ->
                      compute_pointing_1Dto1D_lowmem<double> (:197-226)
  * doubling_contig   CUdoubling_contig_1D (doubling.cu:203-220) ->
                      compute_doubling_spin0_contig_1D (:180-201)
  * doubling_ring     CUdoubling_1D (doubling.cu:160-178) ->
                      compute_doubling_spin0_1D (:137-158)
  * adjoint_doubling  CUadjoint_doubling_1D (doubling.cu:75-92) ->
                      compute_adjoint_doubling_spin0_1D (:53-72)
The pointing kernel tests ``idx <= nring`` (pointing.cu:202): thread nring
reads entry nring of every ring table.  pointing_lowmem therefore takes ring
tables padded with one entry (nphis[nring] = 0: that thread loops zero
times), checked here before the launch.

All arrays are torch CUDA tensors; launches go on torch's current stream in
the primary context torch uses.
"""
from __future__ import annotations

import ctypes
import os

from . import ref_build

_cuda = None
_modules: dict = {}


class RefKernelError(RuntimeError):
    pass


def available() -> bool:
    return all(os.path.exists(ref_build.cubin_path(n)) for n in ref_build.MODULES)


def _driver():
    global _cuda
    if _cuda is None:
        lib = ctypes.CDLL("libcuda.so.1")
        vp, u = ctypes.c_void_p, ctypes.c_uint
        lib.cuInit.argtypes = [u]
        lib.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        lib.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(u), vp]
        lib.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(vp), u, vp]
        lib.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), vp]
        lib.cuLaunchKernel.argtypes = [vp, u, u, u, u, u, u, u, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        _cuda = lib
    return _cuda


def _check(rc: int, what: str):
    if rc != 0:
        s = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(s))
        raise RefKernelError(f"{what}: CUDA driver error {rc} ({(s.value or b'').decode()})")


def _functions(name: str) -> dict:
    """{kernel name: CUfunction} of a cubin, loaded into the current context."""
    if name in _modules:
        return _modules[name]
    import torch
    torch.cuda.init()
    torch.empty(1, device="cuda")  # the primary context is current on this thread
    lib = _driver()
    _check(lib.cuInit(0), "cuInit")
    ctx = ctypes.c_void_p()
    _check(lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RefKernelError("no current CUDA context")
    path = ref_build.cubin_path(name)
    if not os.path.exists(path):
        raise RefKernelError(f"{path} missing: build it with oracle/ref_build.py where the reference is present")
    mod = ctypes.c_void_p()
    _check(lib.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad {path}")
    n = ctypes.c_uint()
    _check(lib.cuModuleGetFunctionCount(ctypes.byref(n), mod), "cuModuleGetFunctionCount")
    fns = (ctypes.c_void_p * n.value)()
    _check(lib.cuModuleEnumerateFunctions(fns, n.value, mod), "cuModuleEnumerateFunctions")
    out = {}
    for f in fns:
        s = ctypes.c_char_p()
        _check(lib.cuFuncGetName(ctypes.byref(s), f), "cuFuncGetName")
        out[s.value.decode()] = f
    _modules[name] = out
    return out


def _kernel(module: str, base: str, scalar: str):
    """The instantiation compute_<base><scalar> (scalar 'd' double, 'f' float)
    by its mangled name's template-argument part."""
    key = f"{base}I{scalar}E"
    hits = [f for nm, f in _functions(module).items() if key in nm and nm.startswith("_Z")]
    if len(hits) != 1:
        raise RefKernelError(f"{len(hits)} kernels match {key} in {module}.cubin")
    return hits[0]


def _launch(fn, grid: int, block: int, args: list):
    """cuLaunchKernel with each argument given as a ctypes object."""
    import torch
    ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
    stream = torch.cuda.current_stream().cuda_stream
    _check(_driver().cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, stream, ptrs, None), "cuLaunchKernel")


def _p(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _sz(v: int) -> ctypes.c_uint64:
    return ctypes.c_uint64(int(v))


class _KernelLocals(ctypes.Structure):
    """KernelLocals<double> (kernel_params.h:22-31): 16 device pointers."""
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("phi", "philocs", "sind_d", "a", "d", "cos_a", "twohav_aod", "e_a1", "e_a2", "e_a3",
                 "np1", "np2", "np3", "npt", "npp")]


assert ctypes.sizeof(_KernelLocals) == 15 * 8


def pointing_lowmem(thetas, phi0, nphis, ringstarts, spin1_theta, spin1_phi, out_pt, out_pp, nring: int):
    """compute_pointing_1Dto1D_lowmem<double> as CUpointing_1Dto1D_lowmem
    launches it: ceil(nring / 256) blocks of 256, one thread per ring, the
    scratch kl.cos_a of npix doubles.  Ring tables (float64 thetas / phi0,
    int64 nphis / ringstarts) hold nring + 1 entries, the last with
    nphis = 0 (see the module docstring)."""
    import torch
    npix = spin1_theta.numel()
    for t in (thetas, phi0, nphis, ringstarts):
        if t.numel() != nring + 1:
            raise RefKernelError("ring tables must hold nring + 1 entries (pointing.cu:202 reads entry nring)")
    if int(nphis[nring].item()) != 0 or int(nphis[:nring].sum().item()) != npix:
        raise RefKernelError("nphis[nring] must be 0 and the rings must cover npix pixels")
    for t in (spin1_phi, out_pt, out_pp):
        if t.numel() != npix:
            raise RefKernelError("pointing arrays must all hold npix entries")
    cos_a = torch.empty(npix, dtype=torch.float64, device="cuda")
    kl = _KernelLocals()
    kl.cos_a = cos_a.data_ptr()
    fn = _kernel("pointing", "compute_pointing_1Dto1D_lowmem", "d")
    _launch(fn, (nring + 255) // 256, 256,
            [_p(out_pt), _p(out_pp), _p(thetas), _p(phi0), _p(nphis), _p(ringstarts), _p(spin1_theta),
             _p(spin1_phi), _sz(nring), _sz(npix), kl, _sz(nring)])
    torch.cuda.synchronize()


def _scalar(t) -> str:
    import torch
    if t.dtype == torch.float64:
        return "d"
    if t.dtype == torch.float32:
        return "f"
    raise RefKernelError(f"unsupported dtype {t.dtype}")


def doubling_contig(synth, ntheta: int, nphi: int, out):
    """compute_doubling_spin0_contig_1D: theta-contiguous (nphi, ntheta) ->
    (nphi, 2 ntheta - 2); grid ceil(nphi / 256) x 256 (CUdoubling_contig_1D)."""
    import torch
    if synth.numel() != ntheta * nphi or out.numel() != (2 * ntheta - 2) * nphi:
        raise RefKernelError("doubling_contig sizes")
    fn = _kernel("doubling", "compute_doubling_spin0_contig_1D", _scalar(synth))
    _launch(fn, (nphi + 255) // 256, 256, [_p(synth), _sz(ntheta), _sz(nphi), _p(out)])
    torch.cuda.synchronize()


def doubling_ring(synth, ntheta: int, nphi: int, out):
    """compute_doubling_spin0_1D: ring-major (ntheta, nphi) -> (2 ntheta - 2,
    nphi).  The reference passes the DOUBLED ring count as its ``nring``
    (test_doublingGPU.py:115); grid ceil(nring / 256) x 256 (CUdoubling_1D)."""
    import torch
    nd = 2 * ntheta - 2
    if synth.numel() != ntheta * nphi or out.numel() != nd * nphi:
        raise RefKernelError("doubling_ring sizes")
    fn = _kernel("doubling", "compute_doubling_spin0_1D", _scalar(synth))
    _launch(fn, (nd + 255) // 256, 256, [_p(synth), _sz(nd), _sz(nphi), _p(out)])
    torch.cuda.synchronize()


def adjoint_doubling(dmap, ntheta: int, nphi: int, out):
    """compute_adjoint_doubling_spin0_1D: ring-major (2 ntheta - 2, nphi) ->
    (ntheta, nphi); grid ceil(ntheta / 256) x 256 (CUadjoint_doubling_1D)."""
    import torch
    if dmap.numel() != (2 * ntheta - 2) * nphi or out.numel() != ntheta * nphi:
        raise RefKernelError("adjoint_doubling sizes")
    fn = _kernel("doubling", "compute_adjoint_doubling_spin0_1D", _scalar(dmap))
    _launch(fn, (ntheta + 255) // 256, 256, [_p(dmap), _sz(ntheta), _sz(nphi), _p(out)])
    torch.cuda.synchronize()
