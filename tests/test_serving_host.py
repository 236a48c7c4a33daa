"""Host logic of the continuous-batching server (serving.LensingServer) on the
CPU: slots and launches are replaced by fakes (a slot reports its device
bytes, a launch completes after a few polls), so queueing, batching,
admission within the HBM budget, release of idle buckets and the retry of a
refused bucket run without a GPU.  The GPU tests (test_gpu_serving.py) run
the same server on real plans."""
import pytest

torch = pytest.importorskip("torch")

from cunusht_gb300 import serving  # noqa: E402

SLOT_BYTES = {511: 10, 1023: 40, 2047: 100}


class _FakeEvent:
    def __init__(self, polls):
        self.left = polls

    def query(self):
        self.left -= 1
        return self.left <= 0


class _FakeSlot:
    def __init__(self, lmax, spin, eps, max_batch, nphi, precision, graphs):
        self.bytes = SLOT_BYTES[lmax]
        self.max_batch = max_batch
        self.spin = spin
        self.busy = []
        self.event = None


def _fake_launch(self, sl, q):
    kind = q[0].kind
    batch = []
    while q and q[0].kind == kind and len(batch) < sl.max_batch:
        batch.append(q.popleft())
    t = self.now()
    for r in batch:
        r.t_launch = t
        r.result = ("done", kind, r.rid)
    sl.busy = batch
    sl.event = _FakeEvent(3)
    self.launches += 1
    self.launch_log.append((r.lmax, len(batch)))


@pytest.fixture
def fake_server(monkeypatch):
    monkeypatch.setattr(serving, "_Slot", _FakeSlot)
    monkeypatch.setattr(serving.LensingServer, "_launch", _fake_launch)

    def make(budget, policy):
        s = serving.LensingServer(hbm_budget_bytes=budget, policy=policy, graphs=False)
        s.launch_log = []
        return s
    return make


def _drain(srv, max_steps=10000):
    live = []
    for _ in range(max_steps):
        live.append(len(srv.buckets))
        if not srv.step():
            return live
    raise AssertionError("server did not drain")


def test_batches_up_to_policy_and_completes_all(fake_server):
    srv = fake_server(1000, lambda lmax: (4, 2))
    for i in range(11):
        srv.submit("g2l", 511, 2, 1e-7, None, None)
    for i in range(3):
        srv.submit("l2g", 511, 2, 1e-7, None, None)
    _drain(srv)
    assert len(srv.completed) == 14
    # two slots of up to 4: lensing requests go 4 + 4 + 3, delensing 3 in one launch
    assert sorted(n for _, n in srv.launch_log) == [3, 3, 4, 4]
    assert all(r.result[1] == r.kind for r in srv.completed)
    assert srv.rejected_admissions == 0


def test_refused_bucket_admitted_after_idle_release(fake_server):
    """Budget for one lmax-2047 bucket (2 slots x 100) at a time: the second
    bucket is refused while the first runs, then admitted once the first has
    gone idle and been released; every request completes."""
    srv = fake_server(250, lambda lmax: (4, 2))
    for i in range(6):
        srv.submit("g2l", 2047, 2, 1e-7, None, None)
    for i in range(6):
        srv.submit("g2l", 2047, 0, 1e-5, None, None)
    live = _drain(srv)
    assert len(srv.completed) == 12
    assert srv.rejected_admissions >= 1
    assert max(live) == 1                      # never two 2047 buckets at once
    assert srv.used_bytes() <= 250


def test_small_buckets_coexist_within_budget(fake_server):
    srv = fake_server(1000, lambda lmax: (8, 2))
    keys = [(511, 0, 1e-5), (511, 2, 1e-7), (1023, 0, 1e-5), (1023, 2, 1e-7)]
    assert srv.prewarm(keys) == keys
    assert srv.used_bytes() == 2 * (10 + 10 + 40 + 40)
    for lmax, spin, eps in keys:
        srv.submit("g2l", lmax, spin, eps, None, None)
    _drain(srv)
    assert len(srv.completed) == 4
    assert len(srv.buckets) == 4               # nothing had to be released


def test_bucket_larger_than_budget_is_refused_not_admitted(fake_server):
    srv = fake_server(50, lambda lmax: (4, 1))
    srv.submit("g2l", 2047, 2, 1e-7, None, None)
    for _ in range(20):
        assert srv.step()                      # the request stays queued
    assert not srv.buckets
    assert srv.rejected_admissions >= 1
    assert srv.completed == []


def test_submit_rejects_unknown_direction(fake_server):
    srv = fake_server(100, lambda lmax: (1, 1))
    with pytest.raises(ValueError):
        srv.submit("both", 511, 0, 1e-5, None, None)


def test_lru_release_frees_only_what_the_new_bucket_needs(fake_server):
    """Four idle lmax-511 buckets (20 each) hold 80 of a 100 budget; an
    lmax-1023 bucket (2 slots of 40) does not fit even one slot, is refused
    once (its size becomes known), then releases the three least recently
    used 511 buckets (60 >= 60 needed) and no more."""
    srv = fake_server(100, lambda lmax: (4, 2))
    small = [(511, 0, 1e-5), (511, 2, 1e-7), (511, 0, 1e-7), (511, 2, 1e-5)]
    for k in small:                            # used in this order
        srv.submit("g2l", *k, None, None)
        _drain(srv)
    srv.submit("g2l", 1023, 2, 1e-7, None, None)
    _drain(srv)
    assert len(srv.completed) == 5
    assert srv.rejected_admissions == 1
    assert srv.evictions == 3
    assert set(srv.buckets) == {small[3], (1023, 2, 1e-7)}
    assert srv.used_bytes() <= 100


def test_prewarm_admits_in_order_and_releases_nothing(fake_server):
    srv = fake_server(100, lambda lmax: (4, 2))
    keys = [(1023, 0, 1e-5), (511, 0, 1e-5), (1023, 2, 1e-7)]
    assert srv.prewarm(keys) == keys[:2]       # 80 + 20; the second 1023 bucket waits
    assert srv.evictions == 0
    assert set(srv.buckets) == set(keys[:2])
