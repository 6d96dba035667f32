"""Serving loop: continuous batching of KPM solves (moments + D on H's pattern).

Requests are queued as they arrive. A dispatcher admits them into slots while
device memory and slots allow (first fit in arrival order, with a guard so a
large request at the head is not starved); each slot is a worker thread with
its own GB300 engine and CUDA stream, so admitted solves of different sizes
run concurrently on the device, and a request that arrives while others are
running starts as soon as a slot and its memory are free. Probe and recursion
state stay on the device for the whole solve (moments -> autodiff_matrix).

Small autodiff solves share launches: a request whose footprint is at most
`pack_bytes` has a pack key (value kind, block size, order, precision, and the
packets per lane a batch gives its probe count -- probe counts 8 to 128 of FP32
complex blocks all take two); when one is admitted while queued requests have the same key, up to
`pack_max` of them are admitted together as one pack, solved by a Batch: every
Chebyshev step of every system in the pack is one launch, and the reverse
recursion and D of all of them too. A request admitted with no partner runs on
an engine of its own (creating a batch for one request costs more than it
saves). Every kernel's per-system reduction order depends only on that system
(its lanes per row follow its own probe count; the packets per lane are the key's),
so a request's result in a pack of any composition is bit-identical to its
result as a pack of one, and on its own engine the same as alone; the two paths
agree within the FP32 tolerance. Solves whose algorithmic traffic is below `urgent_bytes` run on
a high-priority CUDA stream, so that short requests are not queued behind the
CTAs of long ones.

    srv = Server(max_slots=8, memory_budget=100 << 30)
    t = srv.submit(Request(H, es, R, M, c))
    srv.wait(t)  ->  t.mu, t.D, t.latency
"""
import collections
import threading
import time

import numpy as np

from . import _lib as L
from .engine import Batch, Engine


# FK_OPT_CTA_WAVES of the slots' engines: grids of 8 resident-CTA waves (see Server)
DEFAULT_CTA_WAVES = 8


def batch_packets_per_lane(s, precision, complex_values):
    """The packets per lane a batch picks for a system of s probe columns when it is the widest
    (fk_batch.cu batch_configure): packets of 16 bytes per row, two per lane up to 32 packets, else
    enough for 32 lanes (1, 2 or 4)."""
    elem = {"fp32": 4, "ds": 8, "fp64": 8}[precision] * (2 if complex_values else 1)
    P = -(-s * elem // 16)
    if P <= 32:
        return 2 if P >= 2 else 1
    np_ = -(-P // 32)
    return 1 if np_ <= 1 else 2 if np_ <= 2 else 4


class Request:
    """One KPM solve: moments(M), then autodiff_matrix(c, D) ("autodiff") or
    stoch_matrix(c, D) ("stoch") on H's pattern. The probe block is R (dense, n x s) or, for
    colour probes, R_entries = (s, cols, vals): its nonzeros, k per row (Engine.set_R_sparse)."""

    _next = 0
    _lock = threading.Lock()

    def __init__(self, H, es, R, M, c, kind="autodiff", precision="fp32", arrival=None, R_entries=None):
        with Request._lock:
            self.id = Request._next
            Request._next += 1
        if (R is None) == (R_entries is None):
            raise ValueError("give the probe block as R or as R_entries, not both")
        self.H, self.es, self.M, self.c = H, es, int(M), np.asarray(c, float)
        if R is not None:
            self.R = np.asfortranarray(R)
            self.R_entries = None
            self.n_rows, self.s = self.R.shape
            cplx_r = np.iscomplexobj(R)
        else:
            s, cols, vals = R_entries
            self.R = None
            self.R_entries = (int(s), np.asarray(cols), np.asarray(vals))
            self.n_rows, self.s = len(self.R_entries[1]), int(s)
            cplx_r = np.iscomplexobj(vals)
        self.kind = kind
        self.precision = precision
        self.complex_values = bool(cplx_r or H.is_complex)
        self.arrival = time.perf_counter() if arrival is None else arrival
        self.admitted = None
        self.finished = None
        self.pack_size = 1   # requests in the batch that solved this one (1: its own engine)
        self.mu = None
        self.D = None
        self.error = None
        self.done = threading.Event()

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    def probe_steps(self):
        return float(self.n_rows) * self.M * self.s

    def pack_key(self, max_bytes):
        """Requests with equal keys can share one batched launch per Chebyshev step: autodiff solves
        of the same value kind, block size, order and precision whose probe counts give the batch
        the same packets per lane (batch_packets_per_lane), each of footprint at most max_bytes.
        None: the request runs on an engine of its own."""
        if self.kind != "autodiff" or self.footprint() > max_bytes:
            return None
        return (self.complex_values, self.H.b_len, batch_packets_per_lane(self.s, self.precision, self.complex_values),
                self.M, self.precision)

    def dense_R(self):
        """The probe block as a column-major n x s array (expanded from its nonzeros if needed)."""
        if self.R is not None:
            return self.R
        s, cols, vals = self.R_entries
        R = np.zeros((self.n_rows, s), np.complex128 if self.complex_values else np.float64, order="F")
        rows = np.arange(self.n_rows)
        for q in range(cols.shape[1]):
            R[rows, cols[:, q]] += vals[:, q]   # one entry per row in each slice q
        return R

    def algorithmic_bytes(self):
        """HBM bytes the solve must move at least: M/2 forward steps (read x, z, write y, H once)
        and, for autodiff, M/2 - 1 reverse steps (read alpha_m, alpha_{m+1}, beta_{m+1},
        beta_{m+2}, write alpha_{m-1}, beta_m, H once, D read and written as 8-byte reals).
        A stoch request counts its moments only (a lower bound)."""
        n, s = self.n_rows, self.s
        sv = {"fp64": 8, "ds": 8, "fp32": 4}[self.precision] * (2 if self.complex_values else 1)
        b = self.H.b_len
        nnzb = self.H.n_blocks()
        h = nnzb * (b * b * sv + 4) + 4 * (self.H.n_rows + 1)
        fwd = (self.M // 2) * (3.0 * n * s * sv + h)
        rev = 0.0
        if self.kind == "autodiff":
            d = 2.0 * nnzb * b * b * 8 * (2 if self.complex_values else 1)
            rev = (self.M // 2 - 1) * (6.0 * n * s * sv + h + d)
        return fwd + rev

    def footprint(self):
        """Device bytes an engine needs for this solve (vectors, H, D, scratch)."""
        n, s = self.n_rows, self.s
        es = {"fp64": 8, "ds": 8, "fp32": 4}[self.precision] * (2 if self.complex_values else 1)
        epp = 16 // es
        ld = (s + epp - 1) // epp * epp
        vec = 5 * n * ld * es
        nnzb = self.H.n_blocks() + self.H.n_rows
        b2 = self.H.b_len ** 2
        h = nnzb * (b2 * es + 4) + 4 * (self.H.n_rows + 1)
        d = nnzb * b2 * 16 * 2 + nnzb * 16
        stage = min(256 << 20, n * s * 16)
        scratch = self.M * 8 * 2 * 152 * 8 + (1 << 20)
        return vec + h + d + stage + scratch


def pack_group(req, queue, pack_bytes, pack_max):
    """req and, when it is packable, the requests of `queue` (in order) with its pack key, at most
    pack_max in all: the requests solved together by one batch."""
    group = [req]
    key = req.pack_key(pack_bytes)
    if key is None:
        return group
    for other in queue:
        if len(group) >= pack_max:
            break
        if other is not req and other.pack_key(pack_bytes) == key:
            group.append(other)
    return group


class _Slot:
    def __init__(self, server, idx):
        self.server = server
        self.idx = idx
        self.engines = {}
        self.req = None
        self.wake = threading.Event()
        self.thread = threading.Thread(target=self._run, name="fkpm-slot-%d" % idx, daemon=True)
        self.thread.start()

    def capacity(self):
        return sum(e.memory() for e in self.engines.values())

    def engine(self, req):
        key = (req.complex_values, req.precision)
        e = self.engines.get(key)
        if e is None:
            e = Engine(req.complex_values, req.precision, device=self.server.device)
            # grids of several CTA waves: a long solve's CTAs are short-lived, so the launches of a short
            # solve on the urgent stream find free SMs within a fraction of a long launch
            e.set_option(L.FK_OPT_CTA_WAVES, self.server.cta_waves)
            self.engines[key] = e
        return e

    def _run_pack(self, reqs):
        """Solve a pack of same-key requests with one Batch: moments and autodiff_matrix of all of
        them, one launch per Chebyshev step."""
        r0 = reqs[0]
        bt = Batch(r0.complex_values, r0.precision, device=self.server.device)
        try:
            for r in reqs:
                bt.add(r.H, r.es, r.dense_R())
            bt.commit()
            mu = bt.moments(r0.M)
            Ds = bt.autodiff_matrix(r0.M, np.stack([r.c for r in reqs]))
            for k, r in enumerate(reqs):
                r.mu = mu[k].copy()
                r.D = Ds[k].val.copy()
        finally:
            bt.close()

    def _run(self):
        while True:
            self.wake.wait()
            self.wake.clear()
            reqs = self.req
            if reqs is None:
                if self.server._stopping:
                    return
                continue
            if len(reqs) > 1:
                try:
                    self._run_pack(reqs)
                except Exception as ex:   # the pack fails, the server keeps serving
                    for r in reqs:
                        r.error = ex
                t = time.perf_counter()
                for r in reqs:
                    r.finished = t
                self.req = None
                self.server._slot_done(self, reqs)
                continue
            req = reqs[0]
            try:
                eng = self.engine(req)
                # short solves run on an urgent stream so their launches are not queued behind
                # the CTAs of long solves sharing the GPU (lower p50 latency)
                urgent = req.algorithmic_bytes() < self.server.urgent_bytes
                eng.set_option(L.FK_OPT_PRIORITY, -100 if urgent else 0)
                eng.set_H(req.H, req.es)
                if req.R is not None:
                    eng.set_R(req.R)
                else:
                    s, cols, vals = req.R_entries
                    eng.set_R_sparse(req.n_rows, s, cols, vals)
                req.mu = eng.moments(req.M)
                D = req.H.pattern_like(req.complex_values)
                if req.kind == "autodiff":
                    eng.autodiff_matrix(req.c, D)
                elif req.kind == "stoch":
                    eng.stoch_matrix(req.c, D)
                req.D = D.val
            except Exception as ex:   # the request fails, the server keeps serving
                req.error = ex
            req.finished = time.perf_counter()
            self.req = None
            self.server._slot_done(self, [req])


class Server:
    def __init__(self, device=0, max_slots=8, memory_budget=None, lookahead=64, max_bypass=16,
                 urgent_bytes=100e9, pack_bytes=256 << 20, pack_max=16, cta_waves=DEFAULT_CTA_WAVES):
        self.device = device
        self.cta_waves = int(cta_waves)   # FK_OPT_CTA_WAVES of the slots' engines
        self.pack_bytes = int(pack_bytes) if pack_max > 1 else -1   # footprint bound of packable requests
        self.pack_max = max(1, int(pack_max))
        self.urgent_bytes = float(urgent_bytes)   # solves moving less than this get the urgent stream
        if memory_budget is None:
            memory_budget = int(0.8 * self.device_free(device))
        self.budget = int(memory_budget)
        self.lookahead = lookahead
        self.max_bypass = max_bypass
        self._lock = threading.Condition()
        self._queue = collections.deque()
        self._stopping = False
        self._slots = [_Slot(self, k) for k in range(max_slots)]
        self._reserved = {}           # slot idx -> bytes reserved by its request
        self.completed = []
        self.rejected = []
        self.packs = []               # sizes of the packs solved by a Batch
        self.max_concurrent = 0
        self._head_bypassed = 0
        self._dispatcher = threading.Thread(target=self._dispatch, name="fkpm-dispatch", daemon=True)
        self._dispatcher.start()

    @staticmethod
    def device_free(device=0):
        import ctypes as C
        free = C.c_size_t(0)
        total = C.c_size_t(0)
        st = L.load().fk_device_memory(device, C.byref(free), C.byref(total))
        if st != L.FK_OK:
            raise L.FkError(st, "device_memory")
        return free.value

    # -- client side --
    def submit(self, req):
        if req.footprint() > self.budget:
            req.error = L.FkError(L.FK_ERR_OOM, "admission", "request needs %d bytes, budget %d" % (req.footprint(), self.budget))
            req.finished = time.perf_counter()
            req.done.set()
            with self._lock:
                self.rejected.append(req)
            return req
        with self._lock:
            self._queue.append(req)
            self._lock.notify_all()
        return req

    def wait(self, req, timeout=None):
        if not req.done.wait(timeout):
            raise TimeoutError("request %d not finished" % req.id)
        if req.error is not None:
            raise req.error
        return req

    def drain(self, timeout=None):
        t_end = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while self._queue or any(s.req is not None for s in self._slots):
                left = None if t_end is None else t_end - time.perf_counter()
                if left is not None and left <= 0:
                    raise TimeoutError("server did not drain")
                self._lock.wait(left if left is not None else 1.0)

    def stop(self):
        self.drain()
        with self._lock:
            self._stopping = True
            self._lock.notify_all()
        for s in self._slots:
            s.wake.set()
        for s in self._slots:
            s.thread.join(timeout=30)
            for e in s.engines.values():
                e.close()

    # -- server side --
    def _used(self):
        return sum(self._reserved.values())

    def _need(self, slot, group):
        """Bytes this slot would hold with the requests admitted (engine buffers only grow; a pack's
        batch holds about the sum of its requests' footprints while it runs)."""
        if len(group) > 1:
            return slot.capacity() + sum(r.footprint() for r in group)
        return max(slot.capacity(), group[0].footprint())

    def _dispatch(self):
        with self._lock:
            while not self._stopping:
                admitted = False
                free_slots = [s for s in self._slots if s.req is None]
                if self._queue and free_slots:
                    # first fit in arrival order; the head may be bypassed at most max_bypass times
                    for qi, req in enumerate(list(self._queue)[:self.lookahead]):
                        if qi > 0 and self._head_bypassed >= self.max_bypass:
                            break
                        slot = min(free_slots, key=lambda s: abs(s.capacity() - req.footprint()))
                        group = pack_group(req, list(self._queue)[:self.lookahead], self.pack_bytes, self.pack_max)
                        need = self._need(slot, group)
                        while len(group) > 1 and self._used() - self._reserved.get(slot.idx, 0) + need > self.budget:
                            group.pop()
                            need = self._need(slot, group)
                        if self._used() - self._reserved.get(slot.idx, 0) + need <= self.budget:
                            for r in group:
                                self._queue.remove(r)
                            self._head_bypassed = self._head_bypassed + 1 if qi > 0 else 0
                            self._reserved[slot.idx] = need
                            t_adm = time.perf_counter()
                            for r in group:
                                r.admitted = t_adm
                            if len(group) > 1:
                                self.packs.append(len(group))
                            for r in group:
                                r.pack_size = len(group)
                            slot.req = group
                            slot.wake.set()
                            admitted = True
                            busy = sum(1 for s in self._slots if s.req is not None)
                            self.max_concurrent = max(self.max_concurrent, busy)
                            break
                if not admitted:
                    self._lock.wait(0.05)

    def _slot_done(self, slot, reqs):
        with self._lock:
            self._reserved[slot.idx] = slot.capacity()
            for req in reqs:
                if req.error is None:
                    self.completed.append(req)
                else:
                    self.rejected.append(req)
                req.done.set()
            self._lock.notify_all()

    def stats(self):
        lat = np.array([r.latency for r in self.completed]) if self.completed else np.zeros(1)
        t0 = min((r.arrival for r in self.completed), default=0.0)
        t1 = max((r.finished for r in self.completed), default=0.0)
        work = sum(r.probe_steps() for r in self.completed)
        # time with at least one solve in service (union of the admitted..finished intervals)
        busy, end = 0.0, None
        for a, f in sorted((r.admitted, r.finished) for r in self.completed if r.admitted is not None):
            if end is None or a > end:
                busy += f - a
                end = f
            elif f > end:
                busy += f - end
                end = f
        return {"busy_s": busy, "algorithmic_bytes": sum(r.algorithmic_bytes() for r in self.completed),"completed": len(self.completed), "rejected": len(self.rejected),
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "queue_p50_s": float(np.median([r.admitted - r.arrival for r in self.completed])) if self.completed else 0.0,
                "service_p50_s": float(np.median([r.finished - r.admitted for r in self.completed])) if self.completed else 0.0,
                "probe_steps_per_s": work / max(t1 - t0, 1e-9), "wall_s": t1 - t0,
                "max_concurrent": self.max_concurrent, "budget_bytes": self.budget,
                "packs": len(self.packs), "packed_requests": int(sum(self.packs))}
