"""Continuous-batching request loop for transforms of mixed shapes.

Requests arrive over time (``arrivals``, seconds from the start).  The loop
keeps up to ``max_inflight`` batches on the device at once, each on a CUDA
stream of its own.  Whenever a stream slot is free it packs the oldest waiting
requests into a new batch, as many as fit the device-memory budget left by the
batches in flight (each request's workspace bytes, ``footprint``), at most
``max_jobs`` per batch.  A request that arrives while earlier batches run is
admitted as soon as a slot and memory free up, and its work overlaps theirs on
the device.  Admission is first come, first served: the head of the queue is
never overtaken, so no request starves.  A request whose own footprint exceeds
the whole budget can never run and is failed at once.

The loop is host logic only; the device work sits behind an executor:

    footprint(request) -> bytes      launch(requests) -> handle
    poll() -> [(handle, results or the exception that ended the batch)]
    wait(until)                      now()

``GpuExecutor`` runs each batch as one :class:`~qsft_gb300.engine.Batch`
(evaluation, GWHT with device noise, peeling, collection; one launch per
phase) and reads its results back asynchronously.  Tests drive the same loop
with a simulated executor and clock.

Failures are handled on the host.  ``launch`` raising fails that batch's
requests and frees its memory, and so does a batch whose results could not be
read (a device status or table overflow reported by ``poll``).  A batch that has not finished after
``batch_timeout`` seconds has its requests failed; its memory stays reserved
until the executor reports it finished, because its kernels may still be
writing there.
"""
import time
from collections import deque

import numpy as np

__all__ = ["Server", "ServeReport", "GpuExecutor", "random_mix_request", "poisson_arrivals"]


class ServeReport:
    """Per request: ``latency`` (s, completion - arrival; NaN if failed),
    ``results`` (the executor's result or None) and ``errors`` (None or a
    message).  ``batches`` logs (launch time, request indices, bytes) per batch,
    ``peak_bytes`` is the largest total footprint that was in flight."""

    def __init__(self, n):
        self.latency = np.full(n, np.nan)
        self.results = [None] * n
        self.errors = [None] * n
        self.batches = []
        self.peak_bytes = 0
        self.max_inflight_seen = 0
        self.wall = 0.0

    def completed(self):
        return int(np.isfinite(self.latency).sum())

    def percentiles(self, ps=(50, 99)):
        ok = self.latency[np.isfinite(self.latency)]
        return {f"p{p}": float(np.percentile(ok, p)) if ok.size else float("nan") for p in ps}


class Server:
    def __init__(self, executor, budget_bytes, max_jobs=64, max_inflight=4, batch_timeout=None):
        if max_jobs < 1 or max_inflight < 1 or budget_bytes <= 0:
            raise ValueError("max_jobs, max_inflight and budget_bytes must be positive")
        self.ex = executor
        self.budget = int(budget_bytes)
        self.max_jobs = int(max_jobs)
        self.max_inflight = int(max_inflight)
        self.batch_timeout = batch_timeout

    def run(self, requests, arrivals):
        """Serve `requests` arriving at `arrivals` (non-decreasing seconds from
        the start of the call); returns a :class:`ServeReport`."""
        n = len(requests)
        arrivals = np.asarray(arrivals, dtype=np.float64)
        if arrivals.shape != (n,) or (n and np.any(np.diff(arrivals) < 0)):
            raise ValueError("arrivals must be one non-decreasing time per request")
        ex = self.ex
        rep = ServeReport(n)
        foot = [int(ex.footprint(r)) for r in requests]
        t0 = ex.now()
        nxt = 0                    # next request to arrive
        queue = deque()            # arrived, not yet launched
        inflight = {}              # handle -> [request indices, bytes, launch time, timed out]
        used = 0
        finished = 0

        def fail(idx, msg):
            nonlocal finished
            for i in idx:
                if rep.errors[i] is None and not np.isfinite(rep.latency[i]):
                    rep.errors[i] = msg
                    finished += 1

        while finished < n:
            now = ex.now() - t0
            while nxt < n and arrivals[nxt] <= now:
                queue.append(nxt)
                nxt += 1
            # completions
            for h, results in ex.poll():
                idx, nbytes, _, timed_out = inflight.pop(h)
                used -= nbytes
                if timed_out:
                    continue
                if isinstance(results, Exception):
                    fail(idx, f"batch failed: {type(results).__name__}: {results}")
                    continue
                t_done = ex.now() - t0
                for i, res in zip(idx, results):
                    rep.results[i] = res
                    rep.latency[i] = t_done - arrivals[i]
                finished += len(idx)
            if self.batch_timeout is not None:
                for h, rec in inflight.items():
                    if not rec[3] and now - rec[2] >= self.batch_timeout:
                        rec[3] = True
                        fail(rec[0], f"batch did not finish within {self.batch_timeout} s")
            # admission: new batches while a stream slot is free
            while queue and len(inflight) < self.max_inflight:
                head = queue[0]
                if foot[head] > self.budget:
                    queue.popleft()
                    fail([head], f"footprint {foot[head]} B exceeds the device budget {self.budget} B")
                    continue
                take, nbytes = [], 0
                while queue and len(take) < self.max_jobs and used + nbytes + foot[queue[0]] <= self.budget:
                    i = queue.popleft()
                    take.append(i)
                    nbytes += foot[i]
                if not take:
                    break          # the head waits for memory held by batches in flight
                t_launch = ex.now() - t0
                try:
                    h = ex.launch([requests[i] for i in take])
                except Exception as e:  # noqa: BLE001 -- any launch failure fails exactly this batch
                    fail(take, f"launch failed: {type(e).__name__}: {e}")
                    continue
                inflight[h] = [take, nbytes, t_launch, False]
                used += nbytes
                rep.batches.append((t_launch, list(take), nbytes))
                rep.peak_bytes = max(rep.peak_bytes, used)
                rep.max_inflight_seen = max(rep.max_inflight_seen, len(inflight))
            if finished >= n:
                break
            # sleep until the next arrival, a completion or a batch's deadline
            wake = [arrivals[nxt]] if nxt < n else []
            if self.batch_timeout is not None:
                wake += [rec[2] + self.batch_timeout for rec in inflight.values() if not rec[3]]
            until = t0 + min(wake) if wake else None
            if not inflight and until is None:
                if queue:      # nothing in flight and the head still does not fit: cannot happen
                    raise RuntimeError("admission stalled with an empty device")
                break
            ex.wait(until)
        rep.wall = ex.now() - t0
        return rep


# ---------------------------------------------------------------- the mix
MIX_Q = (2, 3, 4, 5, 20)
MIX_SNR = (10.0, 20.0, np.inf)


def random_mix_request(n_range=(8, 60), b_range=(3, 8), s_range=(10, 2000), max_bins=1 << 20, rng=None):
    """One request of the serving mix: q in {2,3,4,5,20}, n and b uniform in
    their ranges, with b redrawn until 40 <= q^b <= `max_bins` (S <= q^b/4
    needs q^b >= 40; the cap keeps one request's bins in a few hundred MB), S
    uniform in [10, min(2000, q^b/4)], SNR in {10, 20, inf} dB.  Noiseless
    requests use identity delays (R=1); noisy ones NSO delays with R=2.  The
    source is the identity (q=20 is not prime, so no Reed-Solomon delays).
    Draws from the host numpy RNG (seed it for a reproducible mix)."""
    from .serve import random_request
    rnd = np.random if rng is None else rng
    q = int(MIX_Q[rnd.randint(len(MIX_Q))])
    n = int(rnd.randint(n_range[0], n_range[1] + 1))
    while True:
        b = int(rnd.randint(b_range[0], b_range[1] + 1))
        if 40 <= q ** b <= max_bins and b <= n:
            break
    S = int(rnd.randint(s_range[0], min(s_range[1], q ** b // 4) + 1))
    snr = float(MIX_SNR[rnd.randint(len(MIX_SNR))])
    if np.isfinite(snr):
        r = random_request(q, n, b, S, C=3, R=2, snr_db=snr, chan="nso", src="identity")
    else:
        r = random_request(q, n, b, S, C=3, R=1, snr_db=None, chan="identity", src="identity")
    r.locq = r.locq.astype(np.int8)        # digits < 128: 8x less host memory for a long mix
    return r


def poisson_arrivals(n, rate, rng=None):
    """Arrival times (s) of a Poisson process of `rate` requests/s."""
    rnd = np.random if rng is None else rng
    return np.cumsum(rnd.exponential(1.0 / rate, size=n))


# ---------------------------------------------------------------- the GPU
class GpuExecutor:
    """Batches on CUDA streams of their own: each ``launch`` packs its requests
    into a fresh :class:`~qsft_gb300.engine.Batch` (allocated and uploaded on
    the current stream), issues the whole step and an asynchronous result
    read-back on a stream of its own, and returns at once.  ``poll`` hands back a
    batch's results, or the exception raised while reading them."""

    def __init__(self, precision="fp32", max_inflight=4, device=None):
        import torch
        self.torch = torch
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max_inflight)]
        self.free_streams = list(range(max_inflight))
        self.inflight = {}
        self._next = 0

    def footprint(self, request):
        from .engine import workspace_bytes
        return workspace_bytes([request.spec()], self.precision)

    def now(self):
        return time.perf_counter()

    def launch(self, requests):
        from .engine import Batch
        from .serve import _rows_hint
        torch = self.torch
        if not self.free_streams:
            raise RuntimeError("no free stream: more batches in flight than streams")
        si = self.free_streams.pop()
        st = self.streams[si]
        try:
            # allocated (and its inputs uploaded) on the current stream, so every
            # batch draws on one pool of the caching allocator; the batch is
            # freed only after its stream's last operation has completed
            b = Batch([r.spec() for r in requests], precision=self.precision, device=self.device)
            st.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(st):
                b.step(stream=st)
                b.fetch_async(st, _rows_hint(requests))
        except Exception:
            self.free_streams.append(si)
            raise
        h = self._next
        self._next += 1
        self.inflight[h] = (b, si)
        return h

    def poll(self):
        from .serve import TransformResult
        out = []
        for h in [h for h, (b, _) in self.inflight.items() if b.fetched_event.query()]:
            b, si = self.inflight.pop(h)
            self.free_streams.append(si)
            try:
                res = [TransformResult(k, v, c, int(ctrl.iter)) for k, v, c, ctrl in b.results_fetched()]
            except Exception as e:  # noqa: BLE001 -- a device error fails this batch's requests only
                res = e
            out.append((h, res))
        return out

    def wait(self, until):
        """Until a batch in flight has finished, or the clock reaches `until`."""
        if until is None:
            if self.inflight:
                first = min(self.inflight)
                self.inflight[first][0].fetched_event.synchronize()
            return
        while time.perf_counter() < until:
            if any(b.fetched_event.query() for b, _ in self.inflight.values()):
                return
            time.sleep(min(5e-5, max(until - time.perf_counter(), 0.0)))
