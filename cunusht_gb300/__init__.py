"""cunusht_gb300: GB300-native (sm_103a) non-uniform spherical harmonic
transforms and CMB lensing, with the Python surface of Sebastian-Belkner/cunuSHT
(``get_transformer(backend='GPU')`` -> nusht2d2, nusht2d1, gclm2lenmap,
lenmap2gclm, dlm2pointing).  Compute runs in hand-written CUDA kernels behind
the C ABI in include/cunusht_gb300.h; there is no CPU backend.
"""
from __future__ import annotations

from .geometry import Geom, get_geom
from .utils import Alm, almxfl, alm2cl, synalm, good_size, good_lmax_array

__all__ = ["get_transformer", "set_transformer", "get_geom", "Geom", "Alm", "almxfl", "alm2cl", "synalm",
           "good_size", "good_lmax_array"]


def get_transformer(backend, solver="default", mode="nuFFT"):
    """Transformer class for (backend, solver, mode) (cunusht/cunusht.py:63-82).
    Only the GPU backend exists here."""
    if backend != "GPU":
        raise ValueError(f"{backend} backend not available: cunusht_gb300 is the GPU engine only")
    if solver == "default":
        solver = "cufinufft"
    from .transformer import GPU_cufinufft_transformer, GPU_SHT_transformer
    if mode == "nuFFT":
        if solver not in ("cufinufft", "gb300"):
            raise ValueError(f"Solver not found: {solver}")
        return GPU_cufinufft_transformer
    if mode == "SHT":
        if solver not in ("shtns", "cufinufft", "gb300"):
            raise ValueError(f"Solver not found: {solver}")
        return GPU_SHT_transformer
    raise ValueError(f"{mode} mode not found")


def set_transformer(transf):
    """Not implemented in the reference either (cunusht/cunusht.py:59-60)."""
    raise NotImplementedError("implement if needed")
