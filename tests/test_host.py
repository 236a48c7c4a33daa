"""Host-side checks that need no GPU: the C-ABI library loads and exports every
symbol include/cunusht_gb300.h declares, and the Python host logic (geometry,
alm utilities, argument parsing, factory) matches the reference semantics."""
import json
import os
import re
import shutil

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cunusht_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cunusht_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from cunusht_gb300 import _lib, build
    have_nvcc = shutil.which("nvcc") is not None or os.path.exists("/usr/local/cuda/bin/nvcc")
    if have_nvcc:
        build.build()  # incremental: rebuilds only stale objects
    elif not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built and nvcc unavailable")
    return _lib.load()


def test_header_declares_expected_entry_points():
    syms = declared_symbols()
    for s in ["cunusht_plan_create", "cunusht_nusht2d2", "cunusht_nusht2d1", "cunusht_dlm2pointing",
              "cunusht_doubling", "cunusht_adjoint_doubling", "cunusht_pointing", "cunusht_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    from cunusht_gb300 import _lib
    for s in declared_symbols():
        assert hasattr(lib, s), f"{s} declared in the header but not exported"
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_library_rejects_bad_arguments_without_touching_the_gpu(lib):
    """Argument validation happens on the host before any CUDA call."""
    import ctypes
    from cunusht_gb300 import _lib
    h = ctypes.c_void_p()
    th = np.array([0.5, np.pi - 0.5])
    p0 = np.zeros(2)
    nph = np.array([8, 8], dtype=np.int64)
    ofs = np.array([0, 8], dtype=np.int64)
    rc = lib.cunusht_plan_create(ctypes.byref(h), 0, 1e-7, 0, 0, 2, th.ctypes.data, p0.ctypes.data,
                                 nph.ctypes.data, ofs.ctypes.data)
    assert rc == 1 and b"lmax" in lib.cunusht_last_error()
    rc = lib.cunusht_plan_create(ctypes.byref(h), 3, 1e-7, 0, 5, 2, th.ctypes.data, p0.ctypes.data,
                                 nph.ctypes.data, ofs.ctypes.data)
    assert rc == 1 and b"max_spin" in lib.cunusht_last_error()
    rc = lib.cunusht_doubling(None, 4, 8, 0, 0, 0, None, None)
    assert rc == 1
    rc = lib.cunusht_nusht2d2(None, 0, 1, None, 0, None, 0, 0, None, None, 0, None)
    assert rc == 1 and b"plan" in lib.cunusht_last_error()
    with pytest.raises(_lib.CunushtError):
        _lib.check(rc)


def test_gl_geometry_matches_oracle():
    from cunusht_gb300 import get_geom
    from oracle import oracle as orc
    for lmax, nphi in [(31, None), (255, 511), (2047, 4095)]:
        gi = {"lmax": lmax} if nphi is None else {"lmax": lmax, "nphi": nphi}
        g = get_geom(("gl", gi))
        th, p0, nph, ofs, w = orc.gl_geometry(lmax, nphi)
        np.testing.assert_allclose(g.theta, th, atol=1e-14)
        assert np.array_equal(g.nph.astype(np.int64), nph) and np.array_equal(g.ofs.astype(np.int64), ofs)
        np.testing.assert_allclose(g.weight, w, rtol=1e-12)
        assert abs(g.fsky() - 1.0) < 1e-12


def test_alm_utils_match_reference_semantics():
    from cunusht_gb300 import Alm, almxfl, alm2cl, synalm
    from oracle import oracle as orc
    L = 40
    assert Alm.getsize(L, L) == orc.nalm(L)
    assert Alm.getidx(L, 5, 3) == orc.almidx(L, 5, 3)
    assert Alm.getlmax(orc.nalm(L), L) == L
    cl = orc.cl_unlensed(L)
    a = synalm(cl, L, L, rng=np.random.default_rng(3))
    b = orc.synalm(cl, L, np.random.default_rng(3))
    np.testing.assert_allclose(a, b)
    np.testing.assert_allclose(alm2cl(a, None, L, L, L), orc.alm2cl(a, L))
    fl = np.arange(L + 1.0)
    np.testing.assert_allclose(almxfl(a, fl, L, False), orc.almxfl(a, fl, L))


def test_loc_layout_detection():
    torch = pytest.importorskip("torch")
    from cunusht_gb300.transformer import _loc_args
    loc = torch.arange(20, dtype=torch.float64).reshape(10, 2)
    t, n, lay = _loc_args(loc)
    assert (n, lay) == (10, 0)
    ptg = torch.arange(20, dtype=torch.float64).reshape(2, 10)
    t, n, lay = _loc_args(ptg.t())  # reference passes ptg.T as loc
    assert (n, lay) == (10, 1) and t.data_ptr() == ptg.data_ptr()
    t, n, lay = _loc_args(ptg)
    assert (n, lay) == (10, 1)


def test_factory_surface():
    import cunusht_gb300 as cu
    from cunusht_gb300.transformer import GPU_cufinufft_transformer, GPU_SHT_transformer
    assert cu.get_transformer("GPU") is GPU_cufinufft_transformer
    assert cu.get_transformer("GPU", "cufinufft", "nuFFT") is GPU_cufinufft_transformer
    assert cu.get_transformer("GPU", "shtns", "SHT") is GPU_SHT_transformer
    with pytest.raises(ValueError):
        cu.get_transformer("CPU")
    with pytest.raises(ValueError):
        cu.get_transformer("GPU", "nope")
    with pytest.raises(NotImplementedError):
        cu.set_transformer(None)


def test_bench_kernel_count_matches_launch_list():
    """bench.py's gpu_launches: kernels per stage execution.  The headline
    served launch of 8 requests (mixed, spin 2) launches 10 kernels: window
    records and tensor-core synthesis for the pointing and for the
    Clenshaw-Curtis grid, its pole pair, ring transform, pointing, theta pass,
    phi pass and interpolation (the ncu launch list of that workload)."""
    import bench
    stages = {s: (0.0, 10) for s in ("leg_synth", "ptg_leg", "theta_fwd", "phi_fwd", "interp", "ptg_ring",
                                      "ptg_rot")}
    n = sum(c * bench.kernels_per_stage(s, "mixed", 1e-7, 2, 8) for s, (_, c) in stages.items())
    assert n == 100
    # launches split greedily as the library does: 11 -> 8 + 2 + 1, 6 -> 4 + 2
    assert bench.kernels_per_stage("leg_synth", "mixed", 1e-7, 2, 11) == 2 * 3 + 1
    assert bench.kernels_per_stage("ptg_leg", "mixed", 1e-7, 2, 6) == 2 * 2
    assert bench.kernels_per_stage("leg_synth", "mixed", 1e-7, 0, 8) == 2
    assert bench.kernels_per_stage("leg_adj", "mixed", 1e-7, 2, 8) == 3
    # FP64 Legendre: one launch per request ("auto" at eps <= 1e-6 is FP64)
    assert bench.kernels_per_stage("leg_synth", "fp64", 1e-7, 2, 8) == 8
    assert bench.kernels_per_stage("ptg_leg", "auto", 1e-7, 2, 4) == 4
    assert bench.kernels_per_stage("interp", "mixed", 1e-7, 2, 8) == 1


def test_bench_tensor_roofline_counts_issued_mma_flops():
    """bench.py's Legendre roofline: achieved = ALGORITHMIC flops / stage
    time against the measured bf16 peak; the MMA flops the tensor-core
    launches issue (per block, order m and 16-l chunk: tiles x 4 MMAs of
    128 x N x 16, checked against a walk over the kernel's windows and
    chunks) only as the named issued-MMA view beside it."""
    import bench

    def walk(lmax, spin, nb, npairs):
        nt = 3 if nb >= 8 else 4
        nn = (20 * nb + 15) // 16 * 16
        blocks = -(-npairs // (64 * nt))
        total = 0
        for m in range(lmax + 1):
            wb = max(m, spin)
            while wb <= lmax:                         # windows of 128 l
                cnt = min(128, lmax - wb + 1)
                total += blocks * (-(-cnt // 16)) * nt * 4 * 2 * 128 * nn * 16
                wb += 128
        return total

    for lmax, spin, nb, npairs in ((300, 2, 8, 150), (300, 1, 4, 151), (1023, 2, 1, 512), (2047, 2, 8, 1024)):
        assert bench.tc_mma_flops(lmax, spin, nb, npairs) == walk(lmax, spin, nb, npairs)
    info = {"ntheta_torus": 4096}
    assert bench.tc_pairs("leg_synth", info, 2048, 8) == 1024      # 1025 pairs less the pole pair
    assert bench.tc_pairs("ptg_leg", info, 2048, 8) == 1024
    roof = bench.legendre_roofline("leg_synth", 41.2, 13.35e-3, info, 2047, 2, 2048, 8,
                                   {"bf16_tflops": 1901.2, "sm_max_mhz": 2070.0}, 2686e6)
    assert roof["bound"] == "tensor" and roof["unit"] == "TFLOP/s" and roof["peak"] == 1901.2
    assert roof["achieved"] == 41.2 and abs(roof["frac"] - 41.2 / 1901.2) < 1e-12
    iss = roof["issued_mma_view"]
    assert 380 < iss["achieved"] < 520 and abs(iss["frac"] - iss["achieved"] / 1901.2) < 1e-12
    assert abs(roof["fp32_view"]["frac"] - 41.2 / (152 * 128 * 2 * 2070e6 / 1e12)) < 1e-12
    assert roof["traffic"] == 2686e6
    json.dumps(roof)


def test_sht_mode_positional_signatures():
    """The SHT-only transformer takes the reference's positional arguments
    (GPU_SHTns_transformer, cunusht/sht/GPU_sht_transformer.py:47-127), so
    reference call sites bind the same parameters."""
    import inspect
    from cunusht_gb300.transformer import GPU_SHT_transformer
    ref = {
        "synthesis": ["gclm", "lmax", "mmax", "mode", "nthreads"],
        "synthesis_cupy": ["gclm", "out", "lmax", "mmax", "mode", "nthreads"],
        "adjoint_synthesis_cupy": ["synthmap", "gclm", "lmax", "mmax", "mode", "nthreads", "iw"],
        "synthesis_der1": ["gclm", "out", "nthreads"],
        "synthesis_der1_cupy": ["gclm", "out_theta", "out_phi", "nthreads"],
        "analysis": ["map", "lmax", "mmax", "nthreads", "alm", "mode"],
        "adjoint_synthesis": ["map"],
        "map2alm": ["m"],
        "alm2map": ["gclm"],
    }
    for name, params in ref.items():
        got = [p for p in inspect.signature(getattr(GPU_SHT_transformer, name)).parameters if p != "self"]
        assert got[:len(params)] == params, (name, got)

