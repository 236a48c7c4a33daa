"""Served form: a batch of lensing requests through cunusht_lensing_batch
gives each request the same map as a single-request solve, and the
continuous-batching server returns for every request of a mixed stream
(lmax, spin, direction, accuracy) the result that request gets alone
(bitwise up to 1e-12 for lensing; for delensing, whose spreading uses
floating-point atomics, within a tenth of the request's epsilon)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _inputs(lmax, spin, nreq, seed):
    g, d = [], []
    for r in range(nreq):
        gc, dl = orc.make_inputs(lmax, spin, seed=seed + r)
        g.append(gc)
        d.append(dl[0])
    return (torch.as_tensor(np.stack(g), device="cuda"), torch.as_tensor(np.stack(d), device="cuda"))


def _lensed_ref(gclm, plm, lmax, spin, th, ph):
    """FP64 oracle: deflection, pointing, spin-s direct sum, rotation."""
    import oracle
    ll = np.arange(lmax + 1)
    dlm = orc.almxfl(plm, np.sqrt(ll * (ll + 1.0)), lmax)
    d = oracle.synth_points_c(lmax, 1, dlm[None], th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    v = oracle.synth_points_c(lmax, spin, gclm if spin else gclm[0], rt, rp)
    if spin:
        z = (v[0] + 1j * v[1]) * np.exp(1j * spin * orc.rotation_gamma(th, d[0], d[1]))
        v = np.stack([z.real, z.imag])
    return v


@pytest.mark.parametrize("precision,eps", [("fp64", 1e-10), ("mixed", 1e-7)])
@pytest.mark.parametrize("spin", [0, 2])
def test_batch_equals_single_requests(built_lib, precision, eps, spin):
    import cunusht_gb300 as cu
    lmax = 255
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    nreq = 6  # chunks of 4 + 2 requests sharing one recursion on the mixed path
    g, d = _inputs(lmax, spin, nreq, 40)
    T.reserve_batch(nreq)
    outb = T.lensing_batch(g, d, spin)
    npix = T.npix()
    for r in range(nreq):
        ptg = torch.empty((2, npix), dtype=torch.float64, device="cuda")
        gam = torch.empty(npix, dtype=torch.float64, device="cuda")
        out = torch.empty((2, npix) if spin else (npix,), dtype=torch.float64, device="cuda")
        gi = g[r] if spin else g[r, 0]
        T.lensing_solve(gi, d[r], out, ptg, gam, spin)
        rms = float(torch.sqrt(torch.mean(out ** 2)))
        diff = float(torch.max(torch.abs(outb[r] - out)))
        assert diff <= 1e-12 * rms, (r, diff, rms)


@pytest.mark.parametrize("precision,eps", [("fp64", 1e-10), ("mixed", 1e-7), ("mixed", 1e-5)])
@pytest.mark.parametrize("spin", [0, 2])
def test_delensing_batch_equals_single_requests(built_lib, precision, eps, spin):
    import cunusht_gb300 as cu
    lmax = 127
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=eps, precision=precision, max_spin=2)
    nreq = 5  # chunks of 4 + 1 requests sharing one recursion on the mixed path
    _, d = _inputs(lmax, spin, nreq, 60)
    npix = T.npix()
    rng = np.random.default_rng(8)
    maps = torch.as_tensor(rng.standard_normal((nreq, 2, npix) if spin else (nreq, npix)), device="cuda")
    ncomp = 2 if spin else 1
    T.reserve_batch(nreq)
    outb = T.delensing_batch(maps, d, spin, ncomp=ncomp)
    for r in range(nreq):
        ptg = torch.empty((2, npix), dtype=torch.float64, device="cuda")
        gam = torch.empty(npix, dtype=torch.float64, device="cuda")
        a = torch.empty((ncomp, T.nalm), dtype=torch.complex128, device="cuda")
        T.delensing_solve(maps[r], d[r], a, ptg, gam, spin)
        rel = float(torch.linalg.norm(outb[r] - a) / torch.linalg.norm(a))
        # the spread accumulates with floating-point atomics in an order that
        # varies between launches: FP64 grid ~1e-16, FP32 grid (eps > 1e-6) ~1e-7
        assert rel < (1e-10 if eps < 1e-6 else 1e-6), (r, rel)
    # and the batch is the adjoint of the lensing batch: <y, A x> = <A^H y, x>
    g, _ = _inputs(lmax, spin, nreq, 90)
    if not spin:
        g = g[:, :1]
    Ax = T.lensing_batch(g, d, spin)
    for r in range(nreq):
        lhs = float(torch.sum(maps[r] * Ax[r]))
        rhs = sum(orc.alm_dot(outb[r, c].cpu().numpy(), g[r, c].cpu().numpy(), lmax) for c in range(ncomp))
        tol = 1e-9 if precision == "fp64" else (5e-7 if eps < 1e-6 else 1e-5)
        assert abs(lhs - rhs) <= tol * abs(lhs), (r, lhs, rhs)


def test_batch_spread_over_launches_and_reference_accuracy(built_lib):
    """batches of 1..5 agree with the direct-sum oracle at sampled pixels."""
    import cunusht_gb300 as cu
    lmax, spin = 127, 2
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-7, precision="mixed", max_spin=2)
    g, d = _inputs(lmax, spin, 5, 70)
    T.reserve_batch(5)
    geom = T.geom
    th, ph = geom.pixels()
    rng = np.random.default_rng(1)
    idx = rng.choice(T.npix(), 60, replace=False)
    for nreq in (1, 3, 5):
        out = T.lensing_batch(g[:nreq], d[:nreq], spin).cpu().numpy()
        for r in range(nreq):
            ref = _lensed_ref(g[r].cpu().numpy(), d[r].cpu().numpy(), lmax, spin, th[idx], ph[idx])
            rms = np.sqrt(np.mean(out[r] ** 2))
            err = np.max(np.abs(out[r][:, idx] - ref)) / rms
            assert err < 2e-6, (nreq, r, err)


def test_batch_rejects_over_capacity(built_lib):
    import cunusht_gb300 as cu
    from cunusht_gb300._lib import CunushtError
    lmax = 63
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-7, precision="mixed", max_spin=2)
    T.reserve_batch(2)
    g, d = _inputs(lmax, 0, 3, 3)
    out = torch.empty((3, T.npix()), dtype=torch.float64, device="cuda")
    T.batch_cap = 3  # bypass the wrapper's automatic reservation: the library must refuse
    with pytest.raises(CunushtError):
        T.lensing_batch(g, d, 0, out=out)


@pytest.mark.parametrize("native", [False, True])
def test_server_mixed_stream_matches_isolated_results(built_lib, native):
    import cunusht_gb300 as cu
    from cunusht_gb300.serving import LensingServer, NativeLensingServer
    srv = NativeLensingServer(precision="mixed", policy={63: (4, 2), 127: (4, 2)}) if native else \
        LensingServer(max_batch=4, precision="mixed")
    rng = np.random.default_rng(11)
    kinds, reqs = [], []
    for i in range(14):
        lmax = [63, 127][i % 2]
        spin = [0, 2][(i // 2) % 2]
        eps = [1e-7, 1e-5][(i // 4) % 2]
        kind = "l2g" if i % 5 == 4 else "g2l"
        gc, dl = orc.make_inputs(lmax, spin, seed=100 + i)
        d = torch.as_tensor(dl[0], device="cuda")
        if kind == "g2l":
            data = torch.as_tensor(gc if spin else gc[0], device="cuda")
        else:
            npix = cu.get_geom(("gl", {"lmax": lmax})).npix()
            data = torch.as_tensor(rng.standard_normal((2, npix) if spin else npix), device="cuda")
        kinds.append((kind, lmax, spin, eps, data, d))
        reqs.append(srv.submit(kind, lmax, spin, eps, data, d))
    srv.run_until_idle()
    torch.cuda.synchronize()
    assert len(srv.completed) == len(kinds)
    if native:
        st = srv.stats()
        assert st["completed"] == len(kinds) and st["launches"] < len(kinds)  # batched
    lat = srv.latencies_ms()
    assert all(x >= 0 for x in lat)
    for i, (kind, lmax, spin, eps, data, d) in enumerate(kinds):
        got = reqs[i].result
        if native:
            # alone on the same (native) server vs in the mix; the native
            # server builds its GL rings in C++ (colatitudes within 1 ulp of
            # the Python geometry), so the Python plan is only compared at eps
            alone = NativeLensingServer(precision="mixed", policy={63: (4, 2), 127: (4, 2)})
            ra = alone.submit(kind, lmax, spin, eps, data, d)
            alone.run_until_idle()
            torch.cuda.synchronize()
            ref_alone = ra.result
            alone.close()
        T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=eps, precision="mixed",
                                       max_spin=max(spin, 1))
        if kind == "g2l":
            ref = T.gclm2lenmap(data, lmax, lmax, dlm_scaled=d, spin=spin, verbose=0)
        else:
            ref = T.lenmap2gclm(data, d, None, lmax, lmax, spin=spin, verbose=0)
        scale = float(torch.max(torch.abs(ref)))
        # lensing is deterministic (no atomics): the same bits up to 1e-12;
        # delensing spreads with floating-point atomics whose order varies
        # between runs, so alone and in the mix agree to a tenth of epsilon
        tol = 1e-12 if kind == "g2l" else 0.1 * eps
        if native:
            err = float(torch.max(torch.abs(got.reshape(ref_alone.shape) - ref_alone)))
            assert err <= tol * scale, (i, kind, lmax, spin, eps, err / scale)
            err = float(torch.max(torch.abs(got.reshape(ref.shape) - ref)))
            assert err <= eps * scale, (i, kind, lmax, spin, eps, err / scale)
        else:
            err = float(torch.max(torch.abs(got.reshape(ref.shape) - ref)))
            assert err <= tol * scale, (i, kind, lmax, spin, eps, err / scale)


@pytest.mark.parametrize("native", [False, True])
def test_server_admits_after_refusal_while_busy(built_lib, native):
    """Two buckets whose requests arrive together under a budget that holds
    only one: the second is refused while the first is busy, and must still
    be admitted once the first has gone idle (no further refusal or release
    event comes)."""
    import time
    from cunusht_gb300.serving import LensingServer, NativeLensingServer
    lmax = 63
    keys = [(lmax, 0, 1e-7), (lmax, 2, 1e-7)]

    def make(budget):
        if native:
            return NativeLensingServer(hbm_budget_bytes=budget, precision="mixed", policy={lmax: (2, 1)})
        return LensingServer(max_batch=2, slots_per_bucket=1, hbm_budget_bytes=budget, precision="mixed")

    def payload(spin, seed):
        gc, dl = orc.make_inputs(lmax, spin, seed=seed)
        return torch.as_tensor(gc if spin else gc[0], device="cuda"), torch.as_tensor(dl[0], device="cuda")

    def used(srv):
        return srv.stats()["bytes"] if native else srv.used_bytes()

    sizes = []
    for i, (L, s, e) in enumerate(keys):
        probe = make(1e13)
        probe.submit("g2l", L, s, e, *payload(s, 300 + i))
        probe.run_until_idle()
        torch.cuda.synchronize()
        sizes.append(used(probe))
        if native:
            probe.close()
        del probe
        torch.cuda.empty_cache()
    budget = max(sizes) + 0.5 * min(sizes)  # one bucket fits, both do not
    srv = make(budget)
    for i, (L, s, e) in enumerate(keys):
        srv.submit("g2l", L, s, e, *payload(s, 400 + i))
    t0 = time.perf_counter()
    while srv.step():
        assert time.perf_counter() - t0 < 120, "a refused bucket was never admitted"
        time.sleep(1e-3)
    torch.cuda.synchronize()
    assert len(srv.completed) == len(keys)
    refusals = srv.stats()["refusals"] if native else srv.rejected_admissions
    assert refusals >= 1  # the second bucket was refused while the first ran
    if native:
        srv.close()


@pytest.mark.parametrize("native", [False, True])
def test_server_prewarmed_graphs_match_lazy_capture(built_lib, native):
    """Buckets prewarmed with every (direction, batch size) graph captured
    ahead of traffic (zeroed inputs) give the results of a server that
    captures on first use: lensing to 1e-12, delensing (floating-point
    spreading atomics) to a tenth of epsilon."""
    import cunusht_gb300 as cu
    from cunusht_gb300.serving import LensingServer, NativeLensingServer
    lmax, eps = 63, 1e-7
    keys = [(lmax, 0, eps), (lmax, 2, eps)]

    def make():
        if native:
            return NativeLensingServer(precision="mixed", policy={lmax: (3, 2)})
        return LensingServer(max_batch=3, precision="mixed")

    rng = np.random.default_rng(21)
    npix = cu.get_geom(("gl", {"lmax": lmax})).npix()
    work = []
    for i in range(8):
        spin = keys[i % 2][1]
        kind = "l2g" if i % 3 == 2 else "g2l"
        gc, dl = orc.make_inputs(lmax, spin, seed=500 + i)
        d = torch.as_tensor(dl[0], device="cuda")
        data = torch.as_tensor(gc if spin else gc[0], device="cuda") if kind == "g2l" else \
            torch.as_tensor(rng.standard_normal((2, npix) if spin else npix), device="cuda")
        work.append((kind, spin, data, d))
    results = []
    for pre in (False, True):
        srv = make()
        if pre:
            assert srv.prewarm(keys, graphs=True) == keys
            if not native:
                for k in keys:
                    for sl in srv.buckets[k]:
                        assert len(sl.graphs) == 2 * sl.max_batch
        reqs = [srv.submit(kind, lmax, spin, eps, data, d) for kind, spin, data, d in work]
        srv.run_until_idle()
        torch.cuda.synchronize()
        results.append([r.result.clone() for r in reqs])
        if native:
            srv.close()
        del srv
    for (kind, spin, data, d), a, b in zip(work, *results):
        scale = float(torch.max(torch.abs(a)))
        tol = 1e-12 if kind == "g2l" else 0.1 * eps
        assert float(torch.max(torch.abs(a - b))) <= tol * scale, (kind, spin)
