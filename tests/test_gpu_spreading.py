"""Spreading options of the type-1 nuFFT (cunusht_plan_set_spreading; the
choices cuFINUFFT's gpu_method / gpu_sort make in the reference's plan,
GPU_nufft_transformer.py:242-246):

  * bin-sorted spreading of scattered points (any order) against exact FP64
    adjoint direct sums (nusht2d1 within the stated eps) and against the
    warp-strip path;
  * deterministic (int64 fixed-point) accumulation: repeated runs give
    bit-identical grids, and a delensing request gives the same alm alone and
    in a batch (to 1e-12; the Legendre stage sums exactly on the tensor cores).
"""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _random_loc(n, rng):
    loc = rng.uniform(0.0, 1.0, (n, 2))
    loc[:, 0] = np.arccos(1 - 2 * loc[:, 0])
    loc[:, 1] *= 2 * np.pi
    return loc


def _T(lmax, eps, precision, nuFFTtype=1):
    import cunusht_gb300 as cu
    return cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=nuFFTtype, epsilon=eps, precision=precision,
                                     max_spin=2)


@pytest.mark.parametrize("spin", [0, 2])
@pytest.mark.parametrize("eps,precision", [(1e-10, "fp64"), (1e-7, "mixed"), (1e-5, "auto")])
@pytest.mark.parametrize("det", [False, True])
def test_bins_nusht2d1_scattered_matches_direct_sum(built_lib, spin, eps, precision, det):
    lmax, n = 63, 20000
    T = _T(lmax, eps, precision)
    T.set_spreading("bins", deterministic=det, max_points=n)
    rng = np.random.default_rng(70 + spin)
    loc = _random_loc(n, rng)
    v = rng.standard_normal(n if spin == 0 else (2, n))
    got = T.nusht2d1(lmax, lmax, torch.as_tensor(v, device="cuda"), torch.as_tensor(loc, device="cuda"),
                     spin=spin).cpu().numpy()
    ref = oracle.adjoint_synth_points_c(lmax, spin, v, loc[:, 0], loc[:, 1])
    err = rel(got, ref)
    print(f"bins spin {spin} {precision} eps {eps} det {det}: {err:.2e}")
    assert err < max(eps, 1e-10) * 2


@pytest.mark.parametrize("spin", [0, 2])
def test_bins_equal_strips_on_scattered_points(built_lib, spin):
    """The two spreading paths agree within the FP32 grid's rounding on
    200000 scattered points (strips fall back to global atomics there)."""
    lmax, n = 255, 200000
    rng = np.random.default_rng(80 + spin)
    loc = torch.as_tensor(_random_loc(n, rng), device="cuda")
    v = torch.as_tensor(rng.standard_normal(n if spin == 0 else (2, n)), device="cuda")
    Ts, Tb = _T(lmax, 1e-7, "mixed"), _T(lmax, 1e-7, "mixed")
    Tb.set_spreading("bins", max_points=n)
    a_s = Ts.nusht2d1(lmax, lmax, v, loc, spin=spin).cpu().numpy()
    a_b = Tb.nusht2d1(lmax, lmax, v, loc, spin=spin).cpu().numpy()
    assert rel(a_b, a_s) < 1e-7


def test_bins_beyond_reserved_points_fall_back_to_strips(built_lib):
    """More points than the bin workspace holds run the warp-strip kernels
    (same result within the grid's rounding)."""
    lmax, n = 63, 5000
    rng = np.random.default_rng(90)
    loc = torch.as_tensor(_random_loc(n, rng), device="cuda")
    v = torch.as_tensor(rng.standard_normal(n), device="cuda")
    Ts, Tb = _T(lmax, 1e-10, "fp64"), _T(lmax, 1e-10, "fp64")
    Tb.set_spreading("bins", max_points=n // 2)
    assert rel(Tb.nusht2d1(lmax, lmax, v, loc).cpu().numpy(), Ts.nusht2d1(lmax, lmax, v, loc).cpu().numpy()) < 1e-12


@pytest.mark.parametrize("method", ["strips", "bins"])
@pytest.mark.parametrize("precision,eps", [("mixed", 1e-7), ("auto", 1e-5), ("fp64", 1e-10)])
def test_deterministic_spreading_is_bit_identical(built_lib, method, precision, eps):
    """Fixed-point accumulation: two runs of nusht2d1 on the same scattered
    points give identical alm (the adjoint Legendre stage sums exactly on the
    tensor cores in the mixed plan; the FP64 plan's CUDA-core adjoint adds
    in FP64 atomics, so only the grid is compared there)."""
    lmax, n = 127, 50000
    rng = np.random.default_rng(100)
    loc = torch.as_tensor(_random_loc(n, rng), device="cuda")
    v = torch.as_tensor(rng.standard_normal((2, n)), device="cuda")
    T = _T(lmax, eps, precision)
    T.set_spreading(method, deterministic=True, max_points=n)
    runs = [T.nusht2d1(lmax, lmax, v, loc, spin=2).cpu().numpy() for _ in range(3)]
    if precision in ("mixed", "auto"):  # "auto" at eps 1e-5: the mixed plan with an FP32 grid
        assert np.array_equal(runs[0], runs[1]) and np.array_equal(runs[0], runs[2])
    else:
        assert rel(runs[1], runs[0]) < 1e-14 and rel(runs[2], runs[0]) < 1e-14


@pytest.mark.parametrize("eps", [1e-7, 1e-5])
@pytest.mark.parametrize("spin", [0, 2])
def test_deterministic_delensing_alone_equals_batched(built_lib, spin, eps):
    """A delensing request gives the same alm alone and inside a batch of 4
    (deterministic spreading, exact tensor-core adjoint): to 1e-12.  At eps
    1e-5 the grid is FP32 and the pixels' strips flush FP32 strip sums."""
    lmax, nreq = 127, 4
    T = _T(lmax, eps, "mixed")
    T.reserve_batch(nreq)
    T.set_spreading("strips", deterministic=True)
    npix = T.npix()
    rng = np.random.default_rng(110 + spin)
    M = torch.as_tensor(rng.standard_normal((nreq, npix) if spin == 0 else (nreq, 2, npix)), device="cuda")
    D = torch.as_tensor(np.stack([orc.make_inputs(lmax, spin, seed=1400 + r)[1][0] for r in range(nreq)]),
                        device="cuda")
    batch = T.delensing_batch(M, D, spin).cpu().numpy()
    for r in range(nreq):
        single = np.atleast_2d(T.lenmap2gclm(M[r], D[r], None, lmax, lmax, spin=spin, verbose=0).cpu().numpy())
        assert rel(batch[r], single) < 1e-12, r
