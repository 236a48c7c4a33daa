"""cunusht_synthesis_noalloc: the spin-s ring synthesis for callers that cannot
call cudaMalloc (code inside another framework's memory pool, pipelines that
forbid allocation after start-up, plugin hosts without an allocator).  It keeps
every intermediate in one file-scope device array, so it must give the same
maps as the plan-based cunusht_synthesis, call after call, although the array
keeps the previous call's contents.

This file is collected last on purpose: a failure here comes after every other
test has run.  It passes alone in a fresh process and after the other tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _alm(lmax, ncomp, spin, seed):
    from oracle import oracle as orc
    rng = np.random.default_rng(seed)
    n = orc.nalm(lmax)
    a = rng.standard_normal((ncomp, n)) + 1j * rng.standard_normal((ncomp, n))
    a[:, :lmax + 1] = a[:, :lmax + 1].real
    for m in range(lmax + 1):
        b = orc.almidx(lmax, m, m)
        for l in range(m, min(spin, lmax + 1)):
            a[:, b + l - m] = 0
    return a


def _noalloc(lib, lmax, spin, a, geom):
    from cunusht_gb300 import _lib
    nring = geom.theta.size
    nphi = int(geom.nph[0])
    th = np.ascontiguousarray(geom.theta, dtype=np.float64)
    p0 = np.ascontiguousarray(geom.phi0, dtype=np.float64)
    A = torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    out = torch.full((nring * nphi,) if spin == 0 else (2, nring * nphi), float("nan"), dtype=torch.float64,
                     device="cuda")
    _lib.check(lib.cunusht_synthesis_noalloc(lmax, spin, a.shape[0], A.data_ptr(), nring, th.ctypes.data,
                                             p0.ctypes.data, nphi, out.data_ptr(),
                                             torch.cuda.current_stream().cuda_stream))
    return out.cpu().numpy()


def test_noalloc_synthesis_matches_plan_synthesis_two_calls_in_a_row(built_lib):
    import cunusht_gb300 as cu
    lmax = 63
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": 127}), nuFFTtype=2, epsilon=1e-10,
                                  precision="fp64")
    # two calls in a row on the shared scratch: spin 2 (E and B), then spin 0
    for spin, ncomp, seed in [(2, 2, 1), (0, 1, 2), (2, 2, 3)]:
        a = _alm(lmax, ncomp, spin, seed)
        want = T.synthesis(torch.as_tensor(a[0] if spin == 0 else a, device="cuda"), spin=spin).cpu().numpy()
        got = _noalloc(built_lib, lmax, spin, a, T.geom)
        assert np.all(np.isfinite(got))
        assert _rel(got.reshape(want.shape), want) < 1e-11


@pytest.mark.parametrize("lmax,nphi", [(255, 1024), (62, 125)])
def test_noalloc_at_the_limits_and_with_an_odd_ring_count(built_lib, lmax, nphi):
    """The largest documented case (lmax 255, 256 rings, 1024 pixels per
    ring: the scratch layout at its bound) and an odd ring count (the
    equator ring pairs with itself), spin 2 then spin 0, against the
    plan-based synthesis."""
    import cunusht_gb300 as cu
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax, "nphi": nphi}), nuFFTtype=2, epsilon=1e-10,
                                  precision="fp64")
    assert T.geom.theta.size == lmax + 1
    for spin, ncomp, seed in [(2, 2, 5), (0, 1, 6)]:
        a = _alm(lmax, ncomp, spin, seed)
        want = T.synthesis(torch.as_tensor(a[0] if spin == 0 else a, device="cuda"), spin=spin).cpu().numpy()
        got = _noalloc(built_lib, lmax, spin, a, T.geom)
        assert np.all(np.isfinite(got))
        assert _rel(got.reshape(want.shape), want) < 1e-11


def test_noalloc_rejects_sizes_beyond_the_scratch_limit(built_lib):
    a = torch.zeros((1, 300 * 301 // 2), dtype=torch.complex128, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    th = np.array([0.5, np.pi - 0.5])
    p0 = np.zeros(2)
    rc = built_lib.cunusht_synthesis_noalloc(299, 0, 1, a.data_ptr(), 2, th.ctypes.data, p0.ctypes.data, 599,
                                             out.data_ptr(), None)
    assert rc == 1  # CUNUSHT_ERR_ARG, rejected on the host before any device work
    assert b"lmax 299" in built_lib.cunusht_last_error()
