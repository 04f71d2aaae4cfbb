"""A request loop for basis solves with continuous batching.

Requests (a deck: {electrode index: mask}, solved into unit bases at
v_basis) arrive at any time.  Each admitted request runs on a worker thread
that drives its own resident MixedSession (own CUDA stream), so requests
that arrive while others are on the GPU start as soon as a worker slot and
device memory free up, and their kernels overlap on the device.

Admission is by HBM footprint: a request needs ig_mixed_bytes(grid, bases)
of device memory; it waits until the sum of the footprints of the sessions
in use fits the budget.  Finished geometries stay resident (keyed by the
bytes of their metal mask and basis count, or by the caller's key) and are
reused by a later request for the same geometry; an edited deck whose metal
changed takes over an idle session of the same grid shape and basis count
by rebinding it (its masks recomputed, its buffers and captured graphs
kept), else gets a new session; least-recently-used idle sessions are
closed when the budget is needed.

Each result is computed by the same kernels in the same order whether the
request runs alone or among others (sessions share no memory), so it is the
same alone and in the mix (tests/test_gpu_serve.py).
"""
import hashlib
import threading
import time
from collections import OrderedDict
from concurrent.futures import Future

import numpy as np

from ion_gym_gb300.physics.mixed import MixedSession, session_bytes


class Request:
    __slots__ = ("rid", "masks", "v_basis", "accuracy", "arrival", "start",
                 "end", "future", "key", "bytes", "n_bases", "shape")

    def __init__(self, rid, masks, v_basis, accuracy, bytes_fn, key=None):
        self.rid = rid
        self.masks = masks
        self.v_basis = v_basis
        self.accuracy = accuracy
        self.arrival = time.perf_counter()
        self.start = self.end = None
        self.future = Future()
        first = np.asarray(next(iter(masks.values())), bool)
        self.shape = first.shape
        self.n_bases = len(masks)
        if key is None:
            h = hashlib.sha256(np.packbits(metal_of(masks, self.shape)).tobytes())
            h.update(repr((self.shape, self.n_bases)).encode())
            key = h.hexdigest()
        else:
            key = f"{key}|{self.shape}|{self.n_bases}"
        self.key = key
        self.bytes = bytes_fn(self.shape, self.n_bases)


def metal_of(masks, shape):
    """The union of a deck's electrode masks."""
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= np.asarray(m, bool)
    return metal


class FieldServer:
    """Continuous-batching basis-solve server on one GPU.

    workers: requests in flight at once (CUDA streams in use).
    hbm_budget: device bytes the resident sessions may hold (default: 80 %
    of the free memory at start-up).
    session_factory / bytes_fn: the session class and its footprint
    function (MixedSession and session_bytes; replaceable for tests of the
    admission logic without a GPU).
    auto_cycle (off by default): a session's second solve tries the other
    smoothing (three pairs each side of the coarse correction instead of
    two, or two instead of three), and the session keeps whichever moved
    fewer algorithmic bytes over its refinement steps (`_tune_cycle`); a
    rebind to another geometry tries again.  On the board and ring-stack
    request mix it measured no gain (knee p50 147 against 119 ms,
    saturation 26.2 against 27.2 requests/s): the trials' graph captures,
    repeated after every rebind, cost what the boards' cheaper cycle saves.
    results: "host" -- each basis a float64 numpy array (the reference's
    solve_bases_mg return); "device" -- each basis a float64 CUDA tensor
    that stays in HBM for consumers on the GPU (the field build reads bases
    in place), with no device-to-host copy in the request's latency.
    Device results are the caller's: they count against free HBM, not
    against the server's session budget."""

    def __init__(self, workers=4, hbm_budget=None, device=0,
                 session_factory=MixedSession, bytes_fn=session_bytes,
                 results="host", auto_cycle=False):
        if results not in ("host", "device"):
            raise ValueError('results must be "host" or "device"')
        self.results = results
        self.auto_cycle = auto_cycle
        self.device = device
        self._factory = session_factory
        self._bytes_fn = bytes_fn
        if device is not None:
            import torch
            torch.cuda.set_device(device)
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.8 * free)
        self.budget = int(hbm_budget)
        self._cv = threading.Condition()
        self._queue = []
        self._in_use = 0                  # bytes of sessions running
        self._idle = OrderedDict()        # key -> session (resident, idle)
        self._idle_bytes = 0
        self._closed = False
        self._next = 0
        self.completed = []
        self._threads = [threading.Thread(target=self._worker, daemon=True)
                         for _ in range(int(workers))]
        for t in self._threads:
            t.start()

    # -------------------------------------------------------------- API
    def submit(self, masks, v_basis=1e4, accuracy=1e-9, key=None):
        """Queue a deck; returns a Future of {index: basis float64}.
        key: the caller's identity of the deck's geometry (the same key for
        the same metal, e.g. its cache key); without it the server hashes
        the union of the masks, which costs a pass over every mask on the
        submitting thread."""
        r = Request(None, dict(sorted(masks.items())), v_basis, accuracy,
                    self._bytes_fn, key=key)
        with self._cv:
            if self._closed:
                raise RuntimeError("server is closed")
            r.rid = self._next
            self._next += 1
            if r.bytes > self.budget:
                r.future.set_exception(MemoryError(
                    f"request needs {r.bytes} device bytes, budget "
                    f"{self.budget}"))
                return r.future
            self._queue.append(r)
            self._cv.notify_all()
        return r.future

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        for s in self._idle.values():
            s.close()
        self._idle.clear()

    def latencies(self):
        """(queue wait, service, total) seconds of every finished request
        (finished requests keep their timing only; results live in the
        callers' futures)."""
        return [(r.start - r.arrival, r.end - r.start, r.end - r.arrival)
                for r in self.completed]

    # -------------------------------------------------------------- internals
    def _admit(self):
        """Pick the oldest queued request that fits; returns (request,
        session or None, whether the session must be rebound to the
        request's metal).  Caller holds the lock."""
        for i, r in enumerate(self._queue):
            sess = self._idle.pop(r.key, None)
            if sess is not None:
                self._idle_bytes -= sess.nbytes
                self._in_use += sess.nbytes
                del self._queue[i]
                return r, sess, False
            # an idle session of the same shape and basis count takes the
            # new geometry by rebinding (no session build)
            for k, other in self._idle.items():
                if (getattr(other, "shape", None) == r.shape
                        and getattr(other, "max_problems", None) == r.n_bases
                        and hasattr(other, "rebind")):
                    del self._idle[k]
                    self._idle_bytes -= other.nbytes
                    self._in_use += other.nbytes
                    del self._queue[i]
                    return r, other, True
            # evict idle sessions (least recently used first) until it fits
            while (self._in_use + self._idle_bytes + r.bytes > self.budget
                   and self._idle):
                _, old = self._idle.popitem(last=False)
                self._idle_bytes -= old.nbytes
                old.close()
            if self._in_use + self._idle_bytes + r.bytes <= self.budget:
                self._in_use += r.bytes
                del self._queue[i]
                return r, None, False
            return None, None, False  # the oldest waits: no overtaking by size
        return None, None, False

    def _worker(self):
        if self.device is not None:
            import torch
            torch.cuda.set_device(self.device)
        while True:
            with self._cv:
                while True:
                    if self._closed and not self._queue:
                        return
                    r, sess, rebind = self._admit()
                    if r is not None:
                        break
                    self._cv.wait(0.05)
            r.start = time.perf_counter()
            held = sess.nbytes if sess is not None else r.bytes
            try:
                if sess is None:
                    sess = self._factory(metal_of(r.masks, r.shape), r.n_bases)
                elif rebind:
                    sess.rebind(metal_of(r.masks, r.shape))
                    sess._cycle_trial = None
                result, err = self._solve(sess, r), None
                self._tune_cycle(sess)
            except Exception as e:     # delivered through the future
                result, err = None, e
            r.end = time.perf_counter()
            fut = r.future
            # the finished request keeps only its timing: the result belongs
            # to the caller's future (device results would otherwise stay in
            # HBM as long as the server lives), the masks to the caller
            r.future = r.masks = None
            with self._cv:
                self._in_use -= held
                if sess is not None:
                    if r.key in self._idle:      # an identical deck ran too
                        sess.close()
                    else:
                        self._idle[r.key] = sess
                        self._idle_bytes += sess.nbytes
                self.completed.append(r)
                self._cv.notify_all()
            if err is None:
                fut.set_result(result)
            else:
                fut.set_exception(err)
            del result, fut


    def _tune_cycle(self, sess):
        """After a solve on a session: the first solve's cycle and the
        algorithmic bytes of its refinement steps are noted and the other
        smoothing set; after the second solve the session keeps the cycle
        whose solve moved fewer bytes (3 % margin, so ties keep the
        batch-size default).  Bytes rather than time: counted by the
        session itself, they do not depend on what else the GPU runs.
        (Planar boards converge in fewer steps with three pairs; the ring
        stack takes the same steps with two, so it keeps two.)"""
        if not self.auto_cycle or not hasattr(sess, "set_cycle"):
            return
        trial = getattr(sess, "_cycle_trial", None)
        if trial == "done":
            return
        cyc = dict(sess.cycle)
        cost = sess.solve_bytes()
        if trial is None:
            pairs = 3 if (cyc["nu1"], cyc["nu2"]) == (2, 2) else 2
            sess._cycle_trial = (cyc, cost)
            sess.set_cycle(pairs, pairs, cyc["cg_iters"])
        else:
            first, first_cost = trial
            if not cost < 0.97 * first_cost:
                sess.set_cycle(first["nu1"], first["nu2"], first["cg_iters"])
            sess._cycle_trial = "done"

    def _solve(self, sess, r):
        """{index: basis} of a request on its session (host or device
        arrays as the server's results kind says)."""
        if self.results == "device":
            import torch
            out = torch.empty((r.n_bases,) + r.shape, dtype=torch.float64,
                              device=f"cuda:{self.device or 0}")
            phi = sess.solve_bases(list(r.masks.values()), r.v_basis,
                                   r.accuracy, out=out)
        else:
            phi = sess.solve_bases(list(r.masks.values()), r.v_basis,
                                   r.accuracy)
        return {i: phi[b] for b, i in enumerate(r.masks)}


def poisson_schedule(rate, duration, seed=0):
    """Arrival times of a Poisson process of `rate` per second."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append(t)


def percentile(values, q):
    v = np.sort(np.asarray(values))
    if len(v) == 0:
        return None
    return float(np.percentile(v, q))
