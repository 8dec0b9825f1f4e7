"""Host logic of the continuous-batching loop (qsft_gb300/server.py), driven by
a simulated device and clock: admission by memory, overlap of batches, FIFO
order, failures injected on the host."""
import numpy as np
import pytest

from qsft_gb300.server import Server, poisson_arrivals, random_mix_request


class Req:
    def __init__(self, i, nbytes, work):
        self.i, self.nbytes, self.work = i, nbytes, work


class SimExecutor:
    """A device that runs the batches in flight one after another (in launch
    order), a batch taking the sum of its requests' work; `fail_launch` makes
    ``launch`` raise for batches containing those requests, `hang` makes those
    batches finish only after `hang_s` seconds, `fail_result` makes ``poll``
    report an exception instead of those batches' results."""

    def __init__(self, launch_cost=1e-4, fail_launch=(), hang=(), hang_s=100.0, fail_result=()):
        self.t = 0.0
        self.launch_cost = launch_cost
        self.fail_launch, self.hang, self.hang_s = set(fail_launch), set(hang), hang_s
        self.fail_result = set(fail_result)
        self.device_free = 0.0
        self.inflight = {}
        self.launched = []
        self.max_bytes = 0
        self.bytes = 0
        self._h = 0

    def footprint(self, r):
        return r.nbytes

    def now(self):
        return self.t

    def launch(self, reqs):
        self.t += self.launch_cost
        if any(r.i in self.fail_launch for r in reqs):
            raise RuntimeError("injected launch failure")
        work = sum(r.work for r in reqs)
        if any(r.i in self.hang for r in reqs):
            work += self.hang_s
        start = max(self.t, self.device_free)
        self.device_free = start + work
        h = self._h
        self._h += 1
        self.inflight[h] = (reqs, self.device_free)
        self.launched.append((self.t, [r.i for r in reqs]))
        self.bytes += sum(r.nbytes for r in reqs)
        self.max_bytes = max(self.max_bytes, self.bytes)
        return h

    def poll(self):
        out = []
        for h in [h for h, (_, tf) in self.inflight.items() if tf <= self.t]:
            reqs, _ = self.inflight.pop(h)
            self.bytes -= sum(r.nbytes for r in reqs)
            if any(r.i in self.fail_result for r in reqs):
                out.append((h, RuntimeError("injected device status")))
            else:
                out.append((h, [("done", r.i) for r in reqs]))
        return out

    def wait(self, until):
        nxt = min((tf for _, tf in self.inflight.values()), default=None)
        cands = [x for x in (nxt, until) if x is not None]
        if cands:
            self.t = max(self.t, min(cands))


def test_every_request_served_once_in_its_own_slot():
    rng = np.random.RandomState(1)
    reqs = [Req(i, int(rng.randint(1, 50)), float(rng.uniform(1e-4, 2e-3))) for i in range(300)]
    arr = poisson_arrivals(len(reqs), 2000.0, rng)
    ex = SimExecutor()
    rep = Server(ex, budget_bytes=400, max_jobs=16, max_inflight=3).run(reqs, arr)
    assert rep.completed() == len(reqs)
    assert all(e is None for e in rep.errors)
    assert [r for r in rep.results] == [("done", i) for i in range(len(reqs))]
    assert np.all(rep.latency > 0)
    launched = sorted(i for _, idx in ex.launched for i in idx)
    assert launched == list(range(len(reqs)))


def test_memory_budget_and_stream_slots_are_respected():
    rng = np.random.RandomState(2)
    reqs = [Req(i, int(rng.randint(10, 120)), 1e-3) for i in range(200)]
    ex = SimExecutor()
    rep = Server(ex, budget_bytes=300, max_jobs=8, max_inflight=2).run(reqs, np.zeros(len(reqs)))
    assert rep.completed() == len(reqs)
    assert ex.max_bytes <= 300 and rep.peak_bytes <= 300
    assert rep.max_inflight_seen <= 2
    assert all(len(idx) <= 8 for _, idx, _ in rep.batches)


def test_admission_is_first_come_first_served():
    rng = np.random.RandomState(3)
    reqs = [Req(i, int(rng.randint(1, 100)), 5e-4) for i in range(150)]
    arr = poisson_arrivals(len(reqs), 5000.0, rng)
    ex = SimExecutor()
    Server(ex, budget_bytes=250, max_jobs=5, max_inflight=4).run(reqs, arr)
    order = [i for _, idx in ex.launched for i in idx]
    assert order == sorted(order)


def test_arrivals_join_while_earlier_batches_run():
    # a long batch is in flight; requests arriving later start before it ends
    reqs = [Req(0, 10, 1.0)] + [Req(i, 10, 1e-3) for i in range(1, 6)]
    arr = np.array([0.0, 0.1, 0.2, 0.3, 0.4, 0.5])
    ex = SimExecutor()
    rep = Server(ex, budget_bytes=100, max_jobs=1, max_inflight=4).run(reqs, arr)
    assert rep.completed() == 6
    t_launch = {idx[0]: t for t, idx, _ in rep.batches}
    assert all(t_launch[i] < 1.0 for i in range(1, 4))   # admitted while request 0 is on the device
    assert rep.max_inflight_seen >= 2


def test_head_waits_for_memory_then_runs():
    reqs = [Req(0, 80, 0.5), Req(1, 80, 0.5), Req(2, 10, 0.1)]
    ex = SimExecutor()
    rep = Server(ex, budget_bytes=100, max_jobs=4, max_inflight=4).run(reqs, np.zeros(3))
    assert rep.completed() == 3
    t_launch = {i: t for t, idx, _ in rep.batches for i in idx}
    assert t_launch[1] >= 0.5                      # waited for request 0's memory
    assert t_launch[2] >= t_launch[1]              # and request 2 did not overtake it


def test_oversized_request_fails_alone():
    reqs = [Req(0, 10, 1e-3), Req(1, 1000, 1e-3), Req(2, 10, 1e-3)]
    rep = Server(SimExecutor(), budget_bytes=100).run(reqs, np.zeros(3))
    assert rep.errors[1] is not None and "exceeds" in rep.errors[1]
    assert rep.errors[0] is None and rep.errors[2] is None
    assert np.isnan(rep.latency[1]) and rep.completed() == 2


def test_launch_failure_fails_only_that_batch():
    reqs = [Req(i, 10, 1e-3) for i in range(12)]
    arr = np.arange(12) * 0.01
    ex = SimExecutor(fail_launch={5})
    rep = Server(ex, budget_bytes=1000, max_jobs=1).run(reqs, arr)
    assert rep.errors[5] is not None and "injected" in rep.errors[5]
    assert rep.completed() == 11
    assert ex.bytes == 0


def test_batch_whose_results_fail_fails_only_its_requests():
    reqs = [Req(i, 10, 1e-3) for i in range(10)]
    arr = np.arange(10) * 0.01
    ex = SimExecutor(fail_result={3})
    rep = Server(ex, budget_bytes=1000, max_jobs=1).run(reqs, arr)
    assert rep.errors[3] is not None and "injected device status" in rep.errors[3]
    assert np.isnan(rep.latency[3]) and rep.results[3] is None
    assert rep.completed() == 9 and ex.bytes == 0


def test_stuck_batch_times_out_but_keeps_its_memory():
    reqs = [Req(0, 60, 1e-3)] + [Req(i, 60, 1e-3) for i in range(1, 4)]
    arr = np.array([0.0, 0.01, 0.02, 0.03])
    ex = SimExecutor(hang={0}, hang_s=5.0)
    rep = Server(ex, budget_bytes=100, max_jobs=1, max_inflight=2, batch_timeout=1.0).run(reqs, arr)
    assert rep.errors[0] is not None and "did not finish" in rep.errors[0]
    assert rep.completed() == 3
    t_launch = {idx[0]: t for t, idx, _ in rep.batches}
    # 60 + 60 > 100: request 1 could not start until the stuck batch released its memory
    assert t_launch[1] >= 5.0
    assert ex.max_bytes <= 100


def test_rejects_bad_arguments():
    with pytest.raises(ValueError):
        Server(SimExecutor(), budget_bytes=0)
    with pytest.raises(ValueError):
        Server(SimExecutor(), budget_bytes=10).run([Req(0, 1, 1e-3), Req(1, 1, 1e-3)], [1.0, 0.0])


def test_mix_generator_stays_in_its_ranges():
    np.random.seed(7)
    for _ in range(300):
        r = random_mix_request()
        assert r.q in (2, 3, 4, 5, 20)
        assert 8 <= r.n <= 60 and 3 <= r.b <= 8
        assert 40 <= r.q ** r.b <= (1 << 20)
        assert 10 <= r.S <= min(2000, r.q ** r.b // 4)
        if r.noise_sd == 0:
            assert r.chan == "identity" and len(r.Ds[0]) == 1
        else:
            assert r.chan == "nso" and len(r.Ds[0]) == 2
        assert r.locq.dtype == np.int8 and r.locq.max() < r.q


def test_mix_is_reproducible():
    np.random.seed(11)
    a = [random_mix_request() for _ in range(20)]
    np.random.seed(11)
    b = [random_mix_request() for _ in range(20)]
    for x, y in zip(a, b):
        assert (x.q, x.n, x.b, x.S, x.noise_sd, x.noise_seed) == (y.q, y.n, y.b, y.S, y.noise_sd, y.noise_seed)
        assert np.array_equal(x.locq, y.locq) and np.array_equal(x.strengths, y.strengths)


def test_footprint_matches_layout_on_host():
    from qsft_gb300.engine import workspace_bytes
    np.random.seed(5)
    reqs = [random_mix_request() for _ in range(12)]
    one = [workspace_bytes([r.spec()]) for r in reqs]
    both = workspace_bytes([r.spec() for r in reqs])
    assert all(x > 0 for x in one)
    # a packed batch needs about the sum of its members (wider key rows when n differs)
    assert 0.5 * sum(one) <= both <= 2.0 * sum(one)


def test_index_block_segments_decode_back():
    """The small index arrays of a mixed batch, packed for one copy to the device:
    every segment is 16-byte aligned and holds exactly its host array."""
    import torch
    from qsft_gb300 import _lib
    from qsft_gb300.engine import Batch, precision_code
    np.random.seed(5)
    specs = [random_mix_request().spec() for _ in range(12)]
    for prec in ("fp32", "fp64"):
        b = Batch.__new__(Batch)
        b.lib, b.prec = _lib.load(), precision_code(prec)
        b._build_layout(specs)
        block, place, gm = b._index_block()
        assert (gm is not None) == (prec == "fp32")
        raw = block.view(np.uint8)
        want = {"eval_prefix": np.asarray(b.eval_prefix_host, np.int64),
                "tc_prefix": np.asarray(b.tc_prefix_host, np.int64),
                "gf": np.asarray(b.gf_host, np.int32)}
        want.update({("rows", k): v.astype(np.int64) for k, v in b.gwht_rows_host.items()})
        want.update({("meta", k): v.astype(np.int32) for k, v in b.gwht_meta_host.items()})
        if gm is not None:
            want["gm_index"] = gm
        for name, arr in want.items():
            w, n, dt = place[name]
            assert (w * 8) % 16 == 0 and n == arr.size
            got = raw[w * 8:w * 8 + arr.nbytes].view(np.int64 if dt == torch.int64 else np.int32)
            assert np.array_equal(got, arr), name
        spans = sorted((w, w + max(2, (n * (8 if dt == torch.int64 else 4) + 15) // 16 * 2))
                       for w, n, dt in place.values())
        assert all(a[1] <= b_[0] for a, b_ in zip(spans, spans[1:]))   # no overlap
