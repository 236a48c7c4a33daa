"""Tensor-core Legendre synthesis (mixed precision, spin > 0).

The self test runs integer products through the same shared-memory
descriptors and tensor-memory path as the Legendre kernel and must be exact.
The synthesis on the tensor cores is compared with the FP64 path and with the
double-float CUDA-core kernels (plan switch cunusht_plan_set_tensor_cores),
for spin 1 and 2, several lmax (windows of 128 l, partial chunks of 16 l),
mmax < lmax, and batched (8 / 4 / 2 / 1 requests per launch) against single
requests.  The plan's device status word stays 0 (no bounded wait ran out)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def _status(t):
    from cunusht_gb300 import _lib
    st = ctypes.c_int(-1)
    _lib.check(t._lib.cunusht_plan_device_status(t._plan, ctypes.byref(st)))
    return st.value


@pytest.mark.parametrize("n", [16, 32, 64])
@pytest.mark.parametrize("reps,mode", [(1, 0), (16, 0), (16, 1), (16, 2)])
def test_tc_selftest_exact(built_lib, n, reps, mode):
    from cunusht_gb300 import _lib
    lib = _lib.load()
    err, to = ctypes.c_double(-1.0), ctypes.c_int(-1)
    _lib.check(lib.cunusht_tc_selftest(n, reps, mode, ctypes.byref(err), ctypes.byref(to)))
    print(f"selftest n {n} reps {reps} mode {mode}: max error {err.value}")
    assert to.value == 0
    assert err.value == 0.0


@pytest.mark.parametrize("n", [16, 32, 64])
@pytest.mark.parametrize("mode", [4, 5, 6])
def test_tc_selftest_mn_major_operands(built_lib, n, mode):
    """Operands stored MN-major (transposed, the tensor-core adjoint's layout:
    core matrices of 8 K-rows x 16 bytes, SBO along M / N, LBO along K) give
    the exact integer product."""
    from cunusht_gb300 import _lib
    lib = _lib.load()
    err, to = ctypes.c_double(-1.0), ctypes.c_int(-1)
    _lib.check(lib.cunusht_tc_selftest(n, 1, mode, ctypes.byref(err), ctypes.byref(to)))
    print(f"selftest MN-major mode {mode} n {n}: max error {err.value}")
    assert to.value == 0
    assert err.value == 0.0


def test_tc_wait_timeout_path_returns_and_leaves_the_context_usable(built_lib):
    """A bounded mbarrier wait that nothing arrives on (self test mode 3: no
    MMA issued, limit 64 polls) runs out: the kernel reports the timeout,
    releases its tensor memory and returns; an ordinary self test right after
    it in the same process is exact."""
    from cunusht_gb300 import _lib
    lib = _lib.load()
    err, to = ctypes.c_double(-1.0), ctypes.c_int(-1)
    _lib.check(lib.cunusht_tc_selftest(64, 1, 3, ctypes.byref(err), ctypes.byref(to)))
    assert to.value == 1
    for _ in range(2):
        err, to = ctypes.c_double(-1.0), ctypes.c_int(-1)
        _lib.check(lib.cunusht_tc_selftest(64, 16, 0, ctypes.byref(err), ctypes.byref(to)))
        assert to.value == 0 and err.value == 0.0


def _transformers(cu, lmax, mmax=None):
    geo = ("gl", {"lmax": lmax})
    mk = lambda prec: cu.get_transformer("GPU")(geo, nuFFTtype=2, epsilon=1e-7, precision=prec, max_spin=2)
    tc, cc, f64 = mk("mixed"), mk("mixed"), mk("fp64")
    from cunusht_gb300 import _lib
    _lib.check(cc._lib.cunusht_plan_set_tensor_cores(cc._plan, 0))
    return tc, cc, f64


@pytest.mark.parametrize("lmax", [40, 127, 300, 2047])
@pytest.mark.parametrize("spin", [0, 1, 2])
def test_tc_synthesis_matches_fp64(built_lib, lmax, spin):
    """lmax 2047 runs the recursion over 2048 steps and 16 windows: an error
    that grows with the number of steps (an unnormalised double-float step
    gave 4e-6 there and under 1e-8 at lmax 300) shows only at full size."""
    import cunusht_gb300 as cu
    tc, cc, f64 = _transformers(cu, lmax)
    gclm, _ = orc.make_inputs(lmax, 2, seed=40 + lmax + spin)
    alm = torch.as_tensor(gclm[0] if spin == 0 else gclm, device="cuda")
    m_tc = tc.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
    m_cc = cc.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
    m_64 = f64.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
    e_tc, e_cc = _rel(m_tc, m_64), _rel(m_cc, m_64)
    print(f"lmax {lmax} spin {spin}: tensor cores {e_tc:.2e}, CUDA cores {e_cc:.2e} vs FP64")
    # digit truncation (2^-32 of the lambda bound) leaves ~4e-9; the CUDA-core
    # kernels round each product to FP32 (~3e-8)
    assert e_tc < 1e-8
    assert e_tc < 0.5 * e_cc
    assert e_cc < 1e-7
    assert _status(tc) == 0


def test_tc_synthesis_mmax(built_lib):
    import cunusht_gb300 as cu
    lmax, mmax = 200, 150
    tc, _, f64 = _transformers(cu, lmax)
    gclm, _ = orc.make_inputs(lmax, 2, seed=77)
    full = np.asarray(gclm)
    n = orc.nalm(lmax, mmax)
    alm = torch.as_tensor(np.ascontiguousarray(full[:, :n]), device="cuda")
    m_tc = tc.synthesis(alm, spin=2, lmax=lmax, mmax=mmax).cpu().numpy()
    m_64 = f64.synthesis(alm, spin=2, lmax=lmax, mmax=mmax).cpu().numpy()
    assert _rel(m_tc, m_64) < 1e-8
    assert _status(tc) == 0


@pytest.mark.parametrize("nreq,spin", [(1, 2), (3, 2), (4, 2), (6, 2), (8, 2), (11, 2), (3, 0), (8, 0)])
def test_tc_lensing_batch_equals_single(built_lib, nreq, spin):
    """Batched launches (8, 4, 2, 1 requests sharing the recursion; 8 in blocks
    of two tiles) give each request exactly its single-request result: the
    digit products are summed exactly and each column's exponent depends on
    its own data only."""
    import cunusht_gb300 as cu
    lmax = 127
    t = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-7, precision="mixed",
                                  max_spin=2)
    G, D = [], []
    for r in range(nreq):
        gclm, dls = orc.make_inputs(lmax, spin, seed=500 + r)
        G.append(gclm if spin else gclm[0])
        D.append(dls[0])
    Gt = torch.as_tensor(np.stack(G), device="cuda")
    Dt = torch.as_tensor(np.stack(D), device="cuda")
    batch = t.lensing_batch(Gt, Dt, spin=spin).cpu().numpy()
    for r in range(nreq):
        single = t.gclm2lenmap(Gt[r], lmax, lmax, dlm_scaled=Dt[r], spin=spin, verbose=0).cpu().numpy()
        assert _rel(batch[r], single) < 1e-12
    assert _status(t) == 0


@pytest.mark.parametrize("spin", [0, 1, 2])
def test_tc_lensing_against_cuda_cores(built_lib, spin):
    """End to end (dlm2pointing + nusht2d2): tensor-core and CUDA-core Legendre
    stages agree well within epsilon, and both agree with the FP64 plan."""
    import cunusht_gb300 as cu
    lmax = 255
    tc, cc, f64 = _transformers(cu, lmax)
    gclm, dls = orc.make_inputs(lmax, spin, seed=90 + spin)
    g = torch.as_tensor(gclm if spin else gclm[0], device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    r_tc = tc.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0).cpu().numpy()
    r_cc = cc.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0).cpu().numpy()
    r_64 = f64.gclm2lenmap(g, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0).cpu().numpy()
    assert _rel(r_tc, r_64) < 1e-7
    assert _rel(r_cc, r_64) < 1e-7
    assert _rel(r_tc, r_cc) < 1e-7
    assert _status(tc) == 0


def test_tc_lensing_batch8_matches_fp64(built_lib):
    """Eight requests per launch (blocks of two tiles) over several l-windows
    (lmax 511: four windows of 128 l) against the FP64 plan, end to end."""
    import cunusht_gb300 as cu
    lmax, spin, nreq = 511, 2, 8
    geo = ("gl", {"lmax": lmax})
    t = cu.get_transformer("GPU")(geo, nuFFTtype=2, epsilon=1e-7, precision="mixed", max_spin=2)
    t64 = cu.get_transformer("GPU")(geo, nuFFTtype=2, epsilon=1e-7, precision="fp64", max_spin=2)
    G, D = [], []
    for r in range(nreq):
        gclm, dls = orc.make_inputs(lmax, spin, seed=700 + r)
        G.append(gclm)
        D.append(dls[0])
    Gt = torch.as_tensor(np.stack(G), device="cuda")
    Dt = torch.as_tensor(np.stack(D), device="cuda")
    batch = t.lensing_batch(Gt, Dt, spin=spin).cpu().numpy()
    for r in (0, nreq - 1):
        ref = t64.gclm2lenmap(Gt[r], lmax, lmax, dlm_scaled=Dt[r], spin=spin, verbose=0).cpu().numpy()
        err = _rel(batch[r], ref)
        print(f"request {r}: {err:.2e} vs FP64")
        assert err < 1e-7
    assert _status(t) == 0


@pytest.mark.parametrize("lmax", [40, 127, 300, 2047])
@pytest.mark.parametrize("spin", [0, 1, 2])
def test_tc_adjoint_synthesis_matches_fp64(built_lib, lmax, spin):
    """The adjoint Legendre stage on the tensor cores (integer-digit products
    summed exactly over 256 rings per block, exact int64 sums across blocks)
    against the FP64 plan and the double-float CUDA-core kernels, through
    the ring adjoint synthesis on the Gauss-Legendre grid."""
    import cunusht_gb300 as cu
    tc, cc, f64 = _transformers(cu, lmax)
    th, _ = tc.geom.pixels()
    rng = np.random.default_rng(900 + lmax + spin)
    y = torch.as_tensor(rng.standard_normal(th.size if spin == 0 else (2, th.size)), device="cuda")
    ncomp = 1 if spin == 0 else 2
    a_tc = tc.adjoint_synthesis(y, spin=spin, ncomp=ncomp).cpu().numpy()
    a_cc = cc.adjoint_synthesis(y, spin=spin, ncomp=ncomp).cpu().numpy()
    a_64 = f64.adjoint_synthesis(y, spin=spin, ncomp=ncomp).cpu().numpy()
    e_tc, e_cc = _rel(a_tc, a_64), _rel(a_cc, a_64)
    print(f"adjoint lmax {lmax} spin {spin}: tensor cores {e_tc:.2e}, CUDA cores {e_cc:.2e} vs FP64")
    # digit truncation at 2^-32 of lambda's bound sqrt((2l+1)/(4 pi)), while a
    # typical |lambda| is about bound / sqrt(l): 2.3e-9 at lmax 40, 1.2e-8 at
    # lmax 2047 (the double-float CUDA-core adjoint reaches 1e-11)
    assert e_tc < 2e-8
    assert e_cc < 1e-7
    assert _status(tc) == 0


@pytest.mark.parametrize("spin", [0, 2])
def test_tc_delensing_matches_fp64_and_is_deterministic(built_lib, spin):
    """lenmap2gclm (spread, adjoint FFTs, adjoint Legendre on the tensor cores
    over the Clenshaw-Curtis rings, pole pair in closed form) against the FP64
    plan; the adjoint Legendre stage sums exactly, so two runs agree to the
    spreading's atomics order only."""
    import cunusht_gb300 as cu
    lmax = 255
    tc, cc, f64 = _transformers(cu, lmax)
    gclm, dls = orc.make_inputs(lmax, spin, seed=95 + spin)
    th, _ = tc.geom.pixels()
    rng = np.random.default_rng(96 + spin)
    m = torch.as_tensor(rng.standard_normal(th.size if spin == 0 else (2, th.size)), device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    r_tc = tc.lenmap2gclm(m, d, None, lmax, lmax, spin=spin, verbose=0).cpu().numpy()
    r_cc = cc.lenmap2gclm(m, d, None, lmax, lmax, spin=spin, verbose=0).cpu().numpy()
    r_64 = f64.lenmap2gclm(m, d, None, lmax, lmax, spin=spin, verbose=0).cpu().numpy()
    print(f"delensing spin {spin}: tensor cores {_rel(r_tc, r_64):.2e}, CUDA cores {_rel(r_cc, r_64):.2e}")
    assert _rel(r_tc, r_64) < 1e-7
    assert _rel(r_cc, r_64) < 1e-7
    assert _rel(r_tc, r_cc) < 1e-7
    assert _status(tc) == 0


@pytest.mark.parametrize("nreq,spin", [(3, 2), (8, 2), (11, 2), (8, 0)])
def test_tc_delensing_batch_equals_single(built_lib, nreq, spin):
    """Batched delensing (8, 4, 2, 1 requests per tensor-core launch) gives each
    request its single-request result within the spreading's atomics order."""
    import cunusht_gb300 as cu
    lmax = 127
    t = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=1, epsilon=1e-7, precision="mixed",
                                  max_spin=2)
    npix = t.npix()
    rng = np.random.default_rng(1200 + nreq)
    M = torch.as_tensor(rng.standard_normal((nreq, npix) if spin == 0 else (nreq, 2, npix)), device="cuda")
    D = torch.as_tensor(np.stack([orc.make_inputs(lmax, spin, seed=1300 + r)[1][0] for r in range(nreq)]),
                        device="cuda")
    batch = t.delensing_batch(M, D, spin).cpu().numpy()
    for r in (0, nreq - 1):
        single = np.atleast_2d(t.lenmap2gclm(M[r], D[r], None, lmax, lmax, spin=spin, verbose=0).cpu().numpy())
        assert _rel(batch[r], single) < 1e-6
    assert _status(t) == 0


@pytest.mark.parametrize("lmax", [300, 2047])
def test_tc_start_states_give_the_full_recursion_result(built_lib, lmax):
    """The per-ring start states (each ring's first chunk outside the
    evanescent region and its recursion state there; blocks skip the chunks
    none of their rings accumulates) give what the recursion from
    l = max(m, s) gives: the synthesis on the Gauss-Legendre grid (spins 0, 1,
    2) and a lensing batch (Clenshaw-Curtis spin 2, pointing GL spin 1) agree
    to 1e-12 with their tables released (cunusht_plan_set_start_states) and
    again once the tables are rebuilt."""
    import cunusht_gb300 as cu
    from cunusht_gb300 import _lib
    t = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-7, precision="mixed", max_spin=2)
    gclm, dls = orc.make_inputs(lmax, 2, seed=90 + lmax)
    states = lambda grid, spin, on: _lib.check(t._lib.cunusht_plan_set_start_states(t._plan, grid, spin, on))
    for spin in (0, 1, 2):
        alm = torch.as_tensor(gclm[0] if spin == 0 else gclm, device="cuda")
        a = t.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
        states(0, spin, 0)
        b = t.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
        states(0, spin, 1)
        c = t.synthesis(alm, spin=spin, lmax=lmax, mmax=lmax).cpu().numpy()
        print(f"lmax {lmax} GL spin {spin}: tables vs none {_rel(a, b):.2e}")
        assert _rel(a, b) < 1e-12, spin
        assert np.array_equal(a, c), spin
    G = torch.as_tensor(np.stack([gclm, gclm]), device="cuda")
    D = torch.as_tensor(np.stack([dls[0], dls[0]]), device="cuda")
    a = t.lensing_batch(G, D, spin=2).cpu().numpy()
    states(1, 2, 0)
    states(0, 1, 0)
    b = t.lensing_batch(G, D, spin=2).cpu().numpy()
    states(1, 2, 1)
    states(0, 1, 1)
    c = t.lensing_batch(G, D, spin=2).cpu().numpy()
    print(f"lmax {lmax} lensing: tables vs none {_rel(a, b):.2e}")
    assert _rel(a, b) < 1e-12
    assert np.array_equal(a, c)
    assert _status(t) == 0
    from cunusht_gb300._lib import CunushtError
    with pytest.raises(CunushtError):
        states(1, 3, 0)  # spin above the plan's maximum
