"""Continuous-batching lensing server.

Requests -- lensing (gclm -> lensed map, gclm2lenmap) or delensing (lensed
map -> gclm, lenmap2gclm) of any lmax, spin and accuracy -- are queued per
bucket (lmax, spin, epsilon).  A bucket owns ``slots_per_bucket`` device
slots; each slot is a plan with its batch workspace, static input/output
buffers and its own CUDA stream, and runs at most one launch at a time.  Every
call of :meth:`LensingServer.step` retires the launches whose completion
events have fired and fills every idle slot with the requests waiting in its
bucket's queue, so requests that arrive while others are on the GPU are
admitted as soon as a slot frees up, and launches of different slots and
buckets overlap on the device.  Slots of smaller lmax run on streams of
higher priority (slot_priority), so short launches are not queued behind the
blocks of long ones.

A launch is one CUDA-graph replay: lensing requests of a bucket go up to
``max_batch`` per launch through cunusht_lensing_batch, delensing requests
through cunusht_delensing_batch (on the mixed path one shared Legendre
recursion per launch of up to eight requests, on the tensor cores, in both
directions).  The graph of each (slot, direction, batch size) is captured on
first use, or for every batch size ahead of traffic by prewarm(graphs=True);
the request's inputs are copied into the slot's static buffers before the
replay and its result copied out after.

Admission: a bucket's slots are created when the bucket first has work (or
by prewarm) and only if the device memory they take (measured) stays within
the HBM budget; otherwise idle buckets are released, least recently used
first and only as many as it needs, or the bucket waits.

The reference has no serving layer: its transformers process one call at a
time with device-wide synchronisation (cunusht/helper_GPU.py:27-51).
"""
from __future__ import annotations

import collections
import dataclasses
import functools
import itertools
import time
from typing import Optional

import torch

from ._lib import CunushtError
from .transformer import GPU_cufinufft_transformer


@dataclasses.dataclass
class Request:
    kind: str                       # "g2l" (gclm2lenmap) or "l2g" (lenmap2gclm)
    lmax: int
    spin: int
    epsilon: float
    data: object                    # gclm (ncomp, nalm) / (nalm,) for g2l; lenmap (2, npix) / (npix,) for l2g;
                                    # or a callable returning (data, dlm_scaled), run on the slot's stream when
                                    # the request is admitted (payload materialised only once it has a slot)
    dlm_scaled: Optional[torch.Tensor]  # (nalm,) complex128 on the device (None with a callable payload)
    arrival: float = 0.0            # server clock, seconds
    rid: int = 0
    result: Optional[torch.Tensor] = None
    t_launch: Optional[float] = None
    t_done: Optional[float] = None


def slot_priority(lmax: int) -> int:
    """CUDA stream priority of a bucket's slots (lower is higher): the smaller
    the transform, the higher the priority, so that a short launch takes the
    SMs that free up while long launches of larger lmax are resident instead of
    waiting behind their thousands of blocks.  lmax <= 1023: two levels above
    the default, 2047: one, larger: the default.  torch maps values outside
    the device's range to its nearest end."""
    return -2 if lmax <= 1023 else (-1 if lmax <= 2047 else 0)


def release_unused_start_states(T, spin: int):
    """A served slot's batched solves read the tensor-core start states of the
    Clenshaw-Curtis grid at the bucket's spin and of the pointing grid at spin
    1 only; the plan's other tables are released (mixed plans)."""
    from . import _lib
    if T.info["precision"] != _lib.PREC_MIXED:
        return
    top = max(spin, 1)
    for s in range(top + 1):
        if s != 1:
            _lib.check(T._lib.cunusht_plan_set_start_states(T._plan, 0, s, 0))
        if s != spin:
            _lib.check(T._lib.cunusht_plan_set_start_states(T._plan, 1, s, 0))


class _Slot:
    """Plan + batch workspace + static buffers + stream; one launch in flight."""

    def __init__(self, lmax, spin, eps, max_batch, nphi, precision, graphs):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        self.stream = torch.cuda.Stream(priority=slot_priority(lmax))
        self.spin = spin
        self.max_batch = max_batch
        self.use_graphs = graphs
        with torch.cuda.stream(self.stream):
            gi = {"lmax": lmax} if nphi is None else {"lmax": lmax, "nphi": nphi}
            self.T = GPU_cufinufft_transformer(("gl", gi), nuFFTtype=2, epsilon=eps, precision=precision,
                                               max_spin=max(spin, 1))
            self.T.reserve_batch(max_batch)
            release_unused_start_states(self.T, spin)
            nalm, npix = self.T.nalm, self.T.npix()
            self.ncomp = 2 if spin else 1
            f64, c128 = torch.float64, torch.complex128
            self.gin = torch.zeros((max_batch, self.ncomp, nalm), dtype=c128, device="cuda")
            self.din = torch.zeros((max_batch, nalm), dtype=c128, device="cuda")
            self.out = torch.zeros((max_batch, 2, npix) if spin else (max_batch, npix), dtype=f64, device="cuda")
            # a launch runs one direction, so the delensing buffers share the
            # lensing ones: maps in = lensing maps out, alm out = lensing alm in
            self.lin = self.out
            self.aout = self.gin
        torch.cuda.synchronize()
        self.bytes = max(0, free0 - torch.cuda.mem_get_info()[0])
        self.graphs: dict[tuple, torch.cuda.CUDAGraph] = {}
        self.busy: list[Request] = []
        self.event: Optional[torch.cuda.Event] = None

    def _work(self, kind, n):
        if kind == "g2l":
            self.T.lensing_batch(self.gin[:n], self.din[:n], self.spin, out=self.out[:n])
        else:
            self.T.delensing_batch(self.lin[:n], self.din[:n], self.spin, ncomp=self.ncomp, out=self.aout[:n])

    def run(self, kind, n):
        """Launch the work of n staged requests on the slot's stream (the
        caller holds torch.cuda.stream(self.stream))."""
        if not self.use_graphs:
            self._work(kind, n)
            return
        g = self.graphs.get((kind, n))
        if g is None:
            g = self.capture(kind, n)
        g.replay()

    def capture(self, kind, n):
        """Capture the (kind, n) graph on the slot's stream (the caller holds
        torch.cuda.stream(self.stream)).  An eager run comes first (kernel
        attributes, lazy module loading).  capture_begin / capture_end rather
        than the torch.cuda.graph context: that one synchronises the whole
        device on entry, which would stall every other slot's launches."""
        self._work(kind, n)
        g = torch.cuda.CUDAGraph()
        g.capture_begin(capture_error_mode="thread_local")
        try:
            self._work(kind, n)
        finally:
            g.capture_end()
        self.graphs[(kind, n)] = g
        return g

    def prewarm_graphs(self):
        """Capture the graphs of both directions and every batch size."""
        if not self.use_graphs:
            return
        with torch.cuda.stream(self.stream):
            for kind in ("g2l", "l2g"):
                for n in range(1, self.max_batch + 1):
                    if (kind, n) not in self.graphs:
                        self.capture(kind, n)


class LensingServer:
    def __init__(self, max_batch: int = 4, hbm_budget_bytes: float = 150e9, precision: str = "mixed",
                 slots_per_bucket: int = 2, graphs: bool = True, nphi_of=lambda lmax: None, policy=None):
        """policy(lmax) -> (max_batch, slots) overrides max_batch / slots_per_bucket per size."""
        self.max_batch = max_batch
        self.budget = hbm_budget_bytes
        self.precision = precision
        self.slots_per_bucket = slots_per_bucket
        self.policy = policy or (lambda lmax: (max_batch, slots_per_bucket))
        self.graphs = graphs
        self.nphi_of = nphi_of
        self.buckets: dict[tuple, list[_Slot]] = {}
        self.queues: dict[tuple, collections.deque] = collections.defaultdict(collections.deque)
        self.t0 = time.perf_counter()
        self.ids = itertools.count()
        self.completed: list[Request] = []
        self.launches = 0
        self.rejected_admissions = 0
        self.evictions = 0
        self._sizes: dict[tuple, int] = {}       # measured device bytes of each bucket's slots
        self._last_use: dict[tuple, float] = {}  # server clock of each bucket's last launch
        self._refused: set = set()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    # ------------------------------------------------------------------ admission
    def used_bytes(self) -> int:
        return sum(sl.bytes for slots in self.buckets.values() for sl in slots)

    def _admit(self, key, evict: bool = True) -> bool:
        """Slots for bucket key within the HBM budget.  Once a bucket's size is
        known (measured when its slots were first made), a bucket that does
        not fit releases idle buckets (empty queue, nothing in flight), least
        recently used first and only as many as it needs, or none when all the
        idle ones together would not make room; it then waits and retries on
        later steps, where the size check comes before any allocation.  With
        evict=False (prewarm) nothing is released."""
        if key in self.buckets:
            return True
        used = self.used_bytes()
        need = self._sizes.get(key)
        if need is not None and used + need > self.budget:
            if not (evict and self._evict_lru(keep=key, free=used + need - self.budget)):
                self._refuse(key)
                return False
            torch.cuda.empty_cache()
            used = self.used_bytes()
        lmax, spin, eps = key
        nb, nslots = self.policy(lmax)
        slots = []
        for _ in range(nslots):
            try:
                sl = _Slot(lmax, spin, eps, nb, self.nphi_of(lmax), self.precision, self.graphs)
            except (CunushtError, torch.cuda.OutOfMemoryError):
                break
            slots.append(sl)
            if used + sum(s.bytes for s in slots) > self.budget:
                self._sizes[key] = nslots * sl.bytes  # known for the next attempt
                slots.pop()
                del sl
                break
        if not slots:
            self._refuse(key)
            torch.cuda.empty_cache()
            return False
        self._refused.discard(key)
        self._sizes[key] = sum(s.bytes for s in slots)
        self._last_use[key] = self.now()
        self.buckets[key] = slots
        return True

    def _refuse(self, key):
        if key not in self._refused:  # one count per refused episode, not per step
            self._refused.add(key)
            self.rejected_admissions += 1

    def _evict_lru(self, keep, free: int) -> bool:
        """Release idle buckets other than keep, least recently used first,
        until at least free bytes are released; release nothing and return
        False if all the idle buckets together hold less."""
        idle = [k for k in self.buckets
                if k != keep and not self.queues[k] and all(not sl.busy for sl in self.buckets[k])]
        idle.sort(key=lambda k: self._last_use.get(k, 0.0))
        chosen, got = [], 0
        for k in idle:
            if got >= free:
                break
            chosen.append(k)
            got += sum(sl.bytes for sl in self.buckets[k])
        if got < free:
            return False
        for k in chosen:
            del self.buckets[k]
            self.evictions += 1
        return True

    def prewarm(self, keys, graphs: bool = False) -> list:
        """Create the slots of these buckets ahead of traffic, in order, while
        they fit the budget (releasing none), and with graphs capture every
        (direction, batch size) graph of their slots; returns the keys
        admitted.  The others are admitted on first use."""
        admitted = []
        for k in keys:
            k = tuple(k)
            if not self._admit(k, evict=False):
                continue
            admitted.append(k)
            if graphs:
                for sl in self.buckets[k]:
                    sl.prewarm_graphs()
        if graphs:
            torch.cuda.synchronize()
        return admitted

    # ------------------------------------------------------------------ API
    def submit(self, kind, lmax, spin, epsilon, data, dlm_scaled, arrival=None) -> Request:
        if kind not in ("g2l", "l2g"):
            raise ValueError(f"kind must be 'g2l' or 'l2g', got {kind!r}")
        r = Request(kind, lmax, spin, epsilon, data, dlm_scaled, self.now() if arrival is None else arrival,
                    next(self.ids))
        self.queues[(lmax, spin, epsilon)].append(r)
        return r

    def _retire(self):
        for slots in self.buckets.values():
            for sl in slots:
                if sl.busy and sl.event.query():
                    t = self.now()
                    for r in sl.busy:
                        r.t_done = t
                        self.completed.append(r)
                    sl.busy = []
                    sl.event = None

    def busy(self) -> bool:
        return any(sl.busy for slots in self.buckets.values() for sl in slots)

    def step(self) -> bool:
        """Retire finished launches, launch queued work on idle slots; True
        while requests are queued or in flight."""
        self._retire()
        pending = False
        for key, q in list(self.queues.items()):
            if not q:
                continue
            pending = True
            if not self._admit(key):
                continue
            for sl in self.buckets[key]:
                if q and not sl.busy:
                    self._launch(sl, q)
                    self._last_use[key] = self.now()
        return pending or self.busy()

    def _launch(self, sl: _Slot, q: collections.deque):
        producer = torch.cuda.current_stream()
        with torch.cuda.stream(sl.stream):
            sl.stream.wait_stream(producer)     # request tensors were made on the caller's stream
            if q[0].kind == "l2g":
                batch = []
                while q and q[0].kind == "l2g" and len(batch) < sl.max_batch:
                    batch.append(q.popleft())
                for i, r in enumerate(batch):
                    data, dlm = r.data() if callable(r.data) else (r.data, r.dlm_scaled)
                    sl.lin[i].copy_(data.reshape(sl.lin.shape[1:]), non_blocking=True)
                    sl.din[i].copy_(dlm.reshape(-1), non_blocking=True)
                sl.run("l2g", len(batch))
                for i, r in enumerate(batch):
                    r.result = sl.aout[i, 0].clone() if sl.spin == 0 else sl.aout[i].clone()
            else:
                batch = []
                while q and q[0].kind == "g2l" and len(batch) < sl.max_batch:
                    batch.append(q.popleft())
                for i, r in enumerate(batch):
                    data, dlm = r.data() if callable(r.data) else (r.data, r.dlm_scaled)
                    sl.gin[i].copy_(data.reshape(sl.ncomp, -1), non_blocking=True)
                    sl.din[i].copy_(dlm.reshape(-1), non_blocking=True)
                sl.run("g2l", len(batch))
                for i, r in enumerate(batch):
                    r.result = sl.out[i].clone()
            ev = torch.cuda.Event()
            ev.record(sl.stream)
        t = self.now()
        for r in batch:
            r.t_launch = t
            r.data = None                       # inputs are staged; drop the caller's references
            r.dlm_scaled = None
        sl.busy = batch
        sl.event = ev
        self.launches += 1

    def run_until_idle(self, poll_s: float = 0.0):
        while self.step():
            if poll_s:
                time.sleep(poll_s)

    def latencies_ms(self):
        return [1e3 * (r.t_done - r.arrival) for r in self.completed]


@functools.lru_cache(maxsize=None)
def _default_nphi(lmax: int) -> int:
    """Pixels per ring of the package's default GL geometry for lmax (cached:
    building the geometry computes the Gauss-Legendre nodes)."""
    from .utils import good_size
    return good_size(2 * lmax + 1, True)


class NativeLensingServer:
    """The same continuous-batching server run by the library's C++ scheduler
    (cunusht_server_*): Python only submits device tensors and polls.

    submit() returns a request id; results land in ``out`` (allocated here if
    not given) once poll() has returned the id."""

    def __init__(self, hbm_budget_bytes: float = 150e9, precision: str = "mixed", policy=None):
        import ctypes
        from . import _lib
        from .transformer import _PREC
        self._lib = _lib.load()
        self._c = ctypes
        h = ctypes.c_void_p()
        _lib.check(self._lib.cunusht_server_create(ctypes.byref(h), float(hbm_budget_bytes), _PREC[precision]))
        self._srv = h
        self.policy = dict(policy or {})
        for lmax, (nb, ns) in self.policy.items():
            _lib.check(self._lib.cunusht_server_set_policy(self._srv, int(lmax), int(nb), int(ns)))
        self.t0 = time.perf_counter()
        self.live: dict[int, Request] = {}
        self.completed: list[Request] = []
        # requests with callable payloads wait here until their bucket has room
        self.waiting: dict[tuple, collections.deque] = collections.defaultdict(collections.deque)
        self.inflight: dict[tuple, int] = collections.defaultdict(int)
        self._streams: dict[int, "torch.cuda.Stream"] = {}  # input streams by slot priority

    def _input_stream(self, lmax: int):
        """Stream on which a request's inputs are materialised and converted:
        the priority of its bucket's slots, so that the inputs of a short
        request are not queued behind the blocks of long launches running at
        a lower priority (on the caller's stream they would be)."""
        pr = slot_priority(lmax)
        if pr not in self._streams:
            self._streams[pr] = torch.cuda.Stream(priority=pr)
        return self._streams[pr]

    def prewarm(self, keys, graphs: bool = True) -> list:
        """Admit these buckets (lmax, spin, epsilon) ahead of traffic on the
        package's default GL geometry and capture every (direction, batch
        size) graph of their slots (cunusht_server_prewarm); returns the keys
        admitted.  Without graphs the buckets are admitted on first use."""
        from . import _lib
        if not graphs:
            return list(keys)
        out = []
        for k in keys:
            lmax, spin, eps = int(k[0]), int(k[1]), float(k[2])
            ok = self._c.c_int()
            _lib.check(self._lib.cunusht_server_prewarm(self._srv, lmax, spin, eps, _default_nphi(lmax),
                                                        self._c.byref(ok)))
            if ok.value:
                out.append(tuple(k))
        return out

    def _cap(self, lmax: int) -> int:
        """Requests of one bucket handed to the library at a time: two full
        launches on every slot (the library's default policy otherwise)."""
        nb, ns = self.policy.get(lmax, (1, 1) if lmax >= 4095 else ((4, 2) if lmax >= 2047 else (8, 2)))
        return 2 * nb * ns

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, kind, lmax, spin, epsilon, data, dlm_scaled, arrival=None, out=None, nphi=0) -> Request:
        """Queue a request.  A callable payload (returning (data, dlm_scaled))
        is materialised only when its bucket has room in the library, so a
        backlog holds no device memory."""
        if kind not in ("g2l", "l2g"):
            raise ValueError(f"kind must be 'g2l' or 'l2g', got {kind!r}")
        r = Request(kind, lmax, spin, epsilon, data, dlm_scaled, self.now() if arrival is None else arrival, -1)
        r.out_arg, r.nphi = out, nphi
        key = (lmax, spin, float(epsilon), nphi)
        if callable(data) or self.waiting[key] or self.inflight[key] >= self._cap(lmax):
            self.waiting[key].append(r)
        else:
            self._hand_over(key, r)
        return r

    def _hand_over(self, key, r: Request):
        from . import _lib
        from .utils import Alm
        kind, lmax, spin, epsilon, nphi, out = r.kind, r.lmax, r.spin, r.epsilon, r.nphi, r.out_arg
        if not nphi:  # the package's default GL geometry (geometry.get_gl_geometry)
            nphi = _default_nphi(lmax)
        nalm = Alm.getsize(lmax, lmax)
        ncm = 2 if spin else 1
        npix = (lmax + 1) * nphi
        # the result on the caller's stream (its earlier work on the memory comes first)
        if out is not None:
            res = out
        elif kind == "g2l":
            res = torch.empty((ncm, npix) if spin else (npix,), dtype=torch.float64, device="cuda")
        else:
            res = torch.empty((ncm, nalm) if spin else (nalm,), dtype=torch.complex128, device="cuda")
        st = self._input_stream(lmax)
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            data, dlm_scaled = r.data() if callable(r.data) else (r.data, r.dlm_scaled)
            if kind == "g2l":
                inp = data.reshape(ncm, nalm).to(torch.complex128).contiguous()
            else:
                inp = data.reshape(ncm, npix).to(torch.float64).contiguous()
            d = dlm_scaled.reshape(-1).to(torch.complex128).contiguous()
        rid = self._c.c_int64()
        _lib.check(self._lib.cunusht_server_submit(self._srv, 0 if kind == "g2l" else 1, lmax, spin, float(epsilon),
                                                   int(nphi), inp.data_ptr(), d.data_ptr(), res.data_ptr(),
                                                   st.cuda_stream, self._c.byref(rid)))
        r.data, r.dlm_scaled, r.result, r.rid, r.key = inp, d, res, rid.value, key
        self.live[rid.value] = r
        self.inflight[key] += 1

    def step(self) -> bool:
        from . import _lib
        ids = (self._c.c_int64 * 256)()
        nd, pend = self._c.c_int(), self._c.c_int()
        while True:
            _lib.check(self._lib.cunusht_server_poll(self._srv, ids, 256, self._c.byref(nd), self._c.byref(pend)))
            t = self.now()
            for i in range(nd.value):
                r = self.live.pop(ids[i])
                r.t_done = t
                r.data = r.dlm_scaled = None  # inputs may be released now
                self.inflight[r.key] -= 1
                self.completed.append(r)
            if nd.value < 256:
                break
        handed = False
        for key, q in self.waiting.items():
            while q and self.inflight[key] < self._cap(key[0]):
                self._hand_over(key, q.popleft())
                handed = True
        if handed:  # launch what was just handed over
            _lib.check(self._lib.cunusht_server_poll(self._srv, None, 0, self._c.byref(nd), self._c.byref(pend)))
        return pend.value > 0 or bool(self.live) or any(self.waiting.values())

    def run_until_idle(self, poll_s: float = 0.0):
        while self.step():
            if poll_s:
                time.sleep(poll_s)

    def latencies_ms(self):
        return [1e3 * (r.t_done - r.arrival) for r in self.completed]

    def stats(self) -> dict:
        from . import _lib
        v = (self._c.c_double * 7)()
        _lib.check(self._lib.cunusht_server_stats(self._srv, v, 7))
        return dict(zip(["launches", "completed", "bytes", "buckets", "slots", "refusals", "evictions"], list(v)))

    def close(self):
        if getattr(self, "_srv", None):
            self._lib.cunusht_server_destroy(self._srv)
            self._srv = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
