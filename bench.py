"""Throughput of the q-SFT hot path on GB300: batched FP32 transforms vs plain FP64.

Workload (the noisy robust configuration): q=4, n=20, b=7 (16384 bins), C=3
random M_c, NSO delays with num_repeat=2 (P=21, 126 GWHT rows), S=1000 support
vectors uniform in Z_4^20, |a|~U[1,10] with uniform phase, complex bin-domain
AWGN at 10 dB SNR.  Synthetic, seeded inputs drawn with the reference's own
generators on the host.

A step = one batch of `--batch` transforms end to end: coset evaluation,
GWHT, noise, peeling (all 15 loop iterations issued; finished jobs no-op) and
result collection.  Every batch holds > 129 MB of bins, so successive steps
stream from HBM rather than L2.

  value  transforms/s with inputs resident on the device (CUDA events); the
         steps go round four captured workspaces on four streams, so four
         batches are in flight as in e2e (the serial replay of one workspace
         on one stream is reported beside it)
  e2e    transforms/s through qsft_gb300.serve.transform_batch with host
         inputs, host->device copies of those inputs and the device->host read
         of every result inside the timed region (wall clock + sync)

--impl reference times the reference's CPU algorithm (the numpy restatement in
oracle/) on the host cores: every step is one whole transform of the same
workload, timed (oracle/cpu_baseline.py).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(q=4, n=20, b=7, S=1000, C=3, R=2, snr_db=10.0, chan="nso", src="identity")
METRIC = "sparse transforms/s (q=4,n=20,b=7,C=3,NSO R=2,S=1000,10 dB), FP32-batched vs FP64-plain"
UNIT = "transforms/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=16)
    p.add_argument("--precision", default="fp32")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--peel-mode", default="graph", choices=["graph", "persistent"],
                   help="peeling loop: a launch per phase (WHILE node in the captured step) or one persistent launch")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--serve-requests", type=int, default=10000, help="serving-mix requests (0: skip)")
    p.add_argument("--serve-rate", type=float, default=0.0,
                   help="Poisson arrival rate, requests/s (0: 80%% of the closed-loop capacity)")
    p.add_argument("--serve-budget-gb", type=float, default=32.0)
    return p.parse_args()


def make_requests(J, seed):
    from qsft_gb300.serve import random_request
    np.random.seed(seed)
    w = WORKLOAD
    return [random_request(w["q"], w["n"], w["b"], w["S"], C=w["C"], R=w["R"], snr_db=w["snr_db"], chan=w["chan"],
                           src=w["src"]) for _ in range(J)]


# ------------------------------------------------------------------ clocks
class Clocks:
    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={q}", "--format=csv,noheader",
                                       "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1].split()[0]))
                mx = float(r[2].split()[0])
                for nm, v in zip(names, r[5:9]):
                    if "Active" in v and "Not" not in v:
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline
# The reference itself (Python, numpy/scipy, multiprocess pool), measured by
# running it on 8 x86 cores at this workload and seed 0: 107.4 s per transform.
REFERENCE_MEASURED_S = 107.4


def cpu_transforms(steps, warmup, seed=0):
    """Time `steps` whole transforms of the workload with the oracle (the numpy
    restatement of the reference) on all host cores, in a child process whose
    BLAS runs one thread per worker (oracle/cpu_baseline.py).  Nothing is
    sampled or scaled.  Returns the child's JSON record (per-step seconds,
    threads used)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-m", "oracle.cpu_baseline", "--steps", str(steps), "--warmup", str(warmup),
                        "--seed", str(seed)], cwd=ROOT, env=env, capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_record(rec):
    steps = len(rec["step_s"])
    value = steps / sum(rec["step_s"])
    sample = (f"{steps} whole transforms (signal, all {WORKLOAD['C'] * WORKLOAD['R'] * (WORKLOAD['n'] + 1)} coset "
              f"rows evaluated with the reference's exp(2 pi i XK/q)@a, GWHT, noise, peeling; nothing scaled), "
              f"{rec['threads']} threads x 1 BLAS thread on {rec['machine']}: "
              f"{np.mean(rec['step_s']):.2f} s per transform; the reference itself measured "
              f"{REFERENCE_MEASURED_S} s per transform on 8 x86 cores")
    return {"value": value, "unit": UNIT, "cores": rec["threads"], "kind": "port", "sample": sample,
            "step_s": rec["step_s"], "reference_measured_s_per_transform": REFERENCE_MEASURED_S}


def coef_nmse(keys, vals, req):
    """||beta_hat - beta||^2 / ||beta||^2 over the union of the recovered and the
    true support (by Parseval, the time-domain test NMSE of
    qsft/test_helper.py:235-260 on the full domain)."""
    true = {tuple(k): complex(a) for k, a in zip(req.locq.T.tolist(), req.strengths)}
    est = {tuple(k): complex(a) for k, a in zip(keys.tolist(), vals)}
    err = sum(abs(est.get(k, 0) - true.get(k, 0)) ** 2 for k in set(true) | set(est))
    return float(err / sum(abs(a) ** 2 for a in true.values()))


def _key_dict(keys, vals):
    return {tuple(int(x) for x in k): complex(v) for k, v in zip(keys, vals)}


def pin_vs_oracle(reqs, dev, precision="fp32", seed=123, max_entries=1 << 22):
    """Each request through the GPU path and through the oracle on the same bin
    noise, drawn on the host (numpy, one RandomState per request): the GPU
    evaluates the cosets and transforms them (its bins are compared with the
    oracle's closed-form bins, sum_{s: M^T k_s = j} a_s omega^<d, k_s>, the
    identity that sampling + GWHT reproduces), adds the noise and peels; the
    oracle peels (qsft/qsft.py:151-255 restated in numpy, FP64) the closed-form
    bins plus the same noise.  Requests with more than `max_entries` bin
    entries (C*R*P*q^b) are skipped.  Returns one record per request compared."""
    import torch
    import oracle as O
    from qsft_gb300.engine import Batch
    out = []
    for i, r in enumerate(reqs):
        C, R, P, B = len(r.Ms), len(r.Ds[0]), r.Ds[0][0].shape[0], r.q ** r.b
        if C * R * P * B > max_entries:
            continue
        locq = np.asarray(r.locq, dtype=np.int64)
        Ds = [np.vstack(d) for d in r.Ds]
        clean = O.closed_form_bins(r.Ms, Ds, locq, r.strengths, r.q)
        nu = r.noise_sd / np.sqrt(2 * B)
        noise = np.random.RandomState(seed + i).normal(0, nu, clean.shape + (2,)).view(np.complex128)[..., 0] \
            if nu > 0 else np.zeros_like(clean)
        sp = r.spec()
        sp.noise_nu = 0.0                                  # no device noise: the host's is added below
        bt = Batch([sp], precision=precision, device=dev)
        bt.eval()
        bt.gwht()
        got_bins = bt.job_U(0).cpu().numpy()
        bins_err = float(np.max(np.abs(got_bins - clean)) / max(np.max(np.abs(clean)), 1e-300))
        if nu > 0:
            bt.add_bins(0, torch.from_numpy(noise))
        bt.peel()
        keys, vals, _, ctrl = bt.results()[0]
        got = _key_dict(keys, vals)
        gw, _, iters = O.peel([clean[c] + noise[c] for c in range(C)], r.Ms, Ds, r.q, r.n, r.b, r.cutoff, r.chan,
                              r.src, P)
        want = {tuple(int(x) for x in k): complex(v) for k, v in gw.items()}
        true = _key_dict(locq.T, r.strengths)
        same = set(got) == set(want)
        num = sum(abs(got[k] - want[k]) ** 2 for k in want) if same else float("nan")
        den = sum(abs(v) ** 2 for v in want.values())
        out.append({"index": i, "q": r.q, "n": r.n, "b": r.b, "S": r.S, "noisy": bool(nu > 0),
                    "same_support": bool(same), "same_iterations": int(ctrl.iter) == int(iters),
                    "coef_rel_l2": float(np.sqrt(num / den)) if den > 0 else 0.0,
                    "nmse_gpu": O.nmse(true, got), "nmse_oracle": O.nmse(true, want), "bins_rel_err": bins_err})
    return out


def pin_own_inputs(batch, req):
    """The timed workload's own inputs through the oracle, for job 0 of the
    batch: (1) the step's evaluation + GWHT without noise against the oracle's
    closed-form bins; (2) the step as timed (evaluation, GWHT with the device
    Philox noise fused), its noisy bins read back before the peeling, then the
    oracle's peeling (FP64 numpy restatement of qsft/qsft.py:151-255) on
    exactly those bins against the GPU's peeling of them."""
    import oracle as O
    sp = batch.specs[0]
    C, RP = sp.C, sp.R * sp.P
    Ds = [np.vstack(d) for d in req.Ds]
    clean = O.closed_form_bins(req.Ms, Ds, np.asarray(req.locq, dtype=np.int64), req.strengths, req.q)
    batch.eval()
    batch.gwht()
    got = batch.job_U(0).cpu().numpy()
    bins_err = float(np.max(np.abs(got - clean)) / np.max(np.abs(clean)))
    batch.eval()
    batch.gwht_noise()
    noisy = batch.job_U(0).cpu().numpy().astype(np.complex128)
    batch.peel()
    keys, vals, _, ctrl = batch.results()[0]
    gpu = _key_dict(keys, vals)
    gw, _, iters = O.peel([noisy[c].copy() for c in range(C)], req.Ms, Ds, req.q, req.n, req.b, req.cutoff, req.chan,
                          req.src, sp.P)
    want = {tuple(int(x) for x in k): complex(v) for k, v in gw.items()}
    same = set(gpu) == set(want)
    l2 = float(np.sqrt(sum(abs(gpu[k] - want[k]) ** 2 for k in want) / sum(abs(v) ** 2 for v in want.values()))) \
        if same and want else float("nan")
    resid = noisy - clean
    nu = req.noise_sd / np.sqrt(2 * req.q ** req.b)
    return {"job": 0, "clean_bins_rel_err_vs_closed_form": bins_err, "same_support": bool(same),
            "same_iterations": int(ctrl.iter) == int(iters), "coef_rel_l2_vs_oracle": l2,
            "noise_std_over_nu": float(np.std(np.concatenate([resid.real.ravel(), resid.imag.ravel()])) / nu),
            "note": "the bench's own device-noise bins of transform 0, peeled by the oracle (FP64) and by the GPU"}


def pin_summary(recs):
    noisy = [x for x in recs if x["noisy"]]
    rel = [abs(x["nmse_gpu"] - x["nmse_oracle"]) / x["nmse_oracle"] for x in noisy if x["nmse_oracle"] > 0]
    return {"requests": len(recs), "same_support": f"{sum(x['same_support'] for x in recs)}/{len(recs)}",
            "same_iterations": f"{sum(x['same_iterations'] for x in recs)}/{len(recs)}",
            "max_coef_rel_l2": float(max([x["coef_rel_l2"] for x in recs], default=0.0)),
            "max_bins_rel_err": float(max([x["bins_rel_err"] for x in recs], default=0.0)),
            "max_nmse_rel_diff_noisy": float(max(rel, default=0.0)),
            "worst_nmse_oracle": float(max([x["nmse_oracle"] for x in recs], default=0.0))}


# DRAM bytes per launch from one ncu capture of this workload (dram__bytes_read.sum +
# dram__bytes_write.sum; profiles/eval_gemm_q4n20b7_batch16.md for the GEMM kernel, an
# earlier capture for its operand kernel, profiles/gwht_rowc_q4n20b7_batch16.md)
NCU_TRAFFIC = {"eval": (35.07e6 + 203.15e6) + (12.94e6 + 12.53e6), "gwht": 264.32e6 + 203.06e6, "batch": 16}


def run_reference(args):
    """The reference arm: the reference's CPU algorithm (restated in oracle/) on
    the host cores, `--steps` whole transforms, each timed (warm-up: `--warmup`
    transforms of the small noiseless q=4, n=10, b=4 case, untimed)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    rec = cpu_transforms(max(args.steps, 1), args.warmup, args.seed)
    cb = cpu_baseline_record(rec)
    value = cb["value"]
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(rec["step_s"]), "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(rec["step_s"])),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": "q4_n20_b7_C3_nso_R2_S1000_10dB", **WORKLOAD, "batch": 1,
                   "parallelism": "cpu host threads"},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ------------------------------------------------------------------ serving mix
def run_serving(args, dev):
    """The serving mix: `--serve-requests` requests drawn with q in {2,3,4,5,20},
    n in [8,60], b in [3,8] (40 <= q^b <= 2^20), S in [10, min(2000, q^b/4)],
    SNR in {10, 20, inf} dB, arriving as a Poisson process; admitted into
    batches by device-memory footprint, up to 4 batches in flight.  Requests are
    drawn before the clock starts.  FP64 plain = the same requests one at a
    time in FP64 (a bounded sample)."""
    import torch
    from qsft_gb300.engine import Batch
    from qsft_gb300.server import GpuExecutor, Server, poisson_arrivals, random_mix_request
    N = args.serve_requests
    np.random.seed(args.seed + 7)
    t = time.perf_counter()
    reqs = [random_mix_request() for _ in range(N)]
    t_gen = time.perf_counter() - t
    budget = int(args.serve_budget_gb * (1 << 30))
    # every shape's GWHT schedule tuned before the clock starts (first use would
    # otherwise time the candidates inside the serving loop)
    from qsft_gb300 import autotune
    t = time.perf_counter()
    for q, b in sorted({(r.q, r.b) for r in reqs}):
        autotune.ensure(q, b, "fp32", dev)
    t_tune = time.perf_counter() - t
    ex = GpuExecutor(max_inflight=4, device=dev)
    srv = Server(ex, budget_bytes=budget, max_jobs=32, max_inflight=4)
    srv.run(reqs[:128], np.zeros(128))                  # warm-up: allocator pool, kernel attributes
    torch.cuda.synchronize()
    ncal = min(N, 2000)
    cal = srv.run(reqs[:ncal], np.zeros(ncal))          # closed loop: capacity
    capacity = cal.completed() / cal.wall
    rate = args.serve_rate if args.serve_rate > 0 else 0.8 * capacity
    arr = poisson_arrivals(N, rate, np.random.RandomState(args.seed + 8))
    rep = srv.run(reqs, arr)
    torch.cuda.synchronize()
    lat = rep.percentiles((50, 99))
    sizes = [len(idx) for _, idx, _ in rep.batches]
    # accuracy on the mix, by SNR class: NMSE against the true coefficients
    by_snr, nm = {}, {}
    for i, (r, res) in enumerate(zip(reqs, rep.results)):
        if res is None:
            continue
        key = "inf" if r.noise_sd == 0 else "noisy"
        nm[i] = coef_nmse(res.keys, res.values, r)
        by_snr.setdefault(key, []).append(nm[i])
    acc = {k: {"median": float(np.median(v)), "p99": float(np.percentile(v, 99)),
               "frac_le_1e-4": float(np.mean(np.array(v) <= 1e-4))} for k, v in by_snr.items()}
    # pin to the oracle: the first 50 requests whose bins fit the oracle's size
    # cap, plus the 5 noisy and 5 noiseless ones of worst NMSE among those that
    # fit, each with host-drawn noise on both sides (pin_vs_oracle)
    cap = 1 << 22

    def fits(r):
        return len(r.Ms) * len(r.Ds[0]) * r.Ds[0][0].shape[0] * r.q ** r.b <= cap
    fit = [i for i in range(N) if i in nm and fits(reqs[i])]
    pick = fit[:50]
    for noisy in (True, False):
        cls = sorted((i for i in fit if (reqs[i].noise_sd > 0) == noisy), key=lambda i: -nm[i])
        pick += [i for i in cls[:5] if i not in pick]
    t = time.perf_counter()
    recs = pin_vs_oracle([reqs[i] for i in pick], dev, max_entries=cap)
    for x in recs:
        x["index"] = pick[x["index"]]
    pin = pin_summary(recs)
    pin["seconds"] = time.perf_counter() - t
    pin["worst"] = sorted(recs, key=lambda x: -x["nmse_oracle"])[:5]
    pin["selection"] = ("first 50 mix requests with C*R*P*q^b <= 2^22, plus the 5 noisy and 5 noiseless of worst "
                        "NMSE (in the timed mix) among those; host-drawn noise on both sides")
    # FP64 plain: one request at a time, eager, results read back
    n64 = min(N, 200)
    agree, t64 = 0, 0.0
    for r, res in zip(reqs[:n64], rep.results[:n64]):
        torch.cuda.synchronize()
        t = time.perf_counter()
        b = Batch([r.spec()], precision="fp64", device=dev)
        b.step()
        k, v, _, _ = b.results(collected=True)[0]
        t64 += time.perf_counter() - t
        if res is not None and set(map(tuple, k.tolist())) == set(map(tuple, res.keys.tolist())):
            agree += 1
    fp64_tps = n64 / t64
    tps = rep.completed() / rep.wall
    return {"requests": N, "completed": rep.completed(), "failed": int(sum(e is not None for e in rep.errors)),
            "arrival_rate": rate, "closed_loop_capacity": capacity, "throughput": tps, "unit": UNIT,
            "wall_s": rep.wall, "latency_ms": {k: v * 1e3 for k, v in lat.items()},
            "batches": len(rep.batches), "mean_batch": float(np.mean(sizes)) if sizes else 0.0,
            "max_inflight": rep.max_inflight_seen, "peak_bytes": rep.peak_bytes, "budget_bytes": budget,
            "fp64_plain": {"value": fp64_tps, "unit": UNIT, "sample": n64,
                           "same_support_as_fp32_mix": f"{agree}/{n64}"},
            "batched_fp32_over_fp64_plain": tps / fp64_tps,
            "nmse_vs_truth": acc, "oracle_pin": pin, "request_generation_s": t_gen, "gwht_tuning_s": t_tune,
            "mix": "q{2,3,4,5,20} n[8,60] b[3,8] 40<=q^b<=2^20 S[10,min(2000,q^b/4)] SNR{10,20,inf}dB; "
                   "noisy: NSO R=2, noiseless: identity R=1; C=3"}


# ------------------------------------------------------------------ GPU
def run_ours(args):
    import torch
    from qsft_gb300 import _lib
    from qsft_gb300 import replicas as RP
    from qsft_gb300.engine import Batch
    from qsft_gb300.serve import TransformStream, transform_batch

    # N GPUs = N independent replicas (no data-path collective): each rank runs
    # its own batches; barriers and the max of the per-rank times for timing
    rank, world, local = RP.init_from_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    J = args.batch
    reqs = make_requests(J, args.seed + 1000 * rank)

    def barrier():
        RP.barrier()
        torch.cuda.synchronize()

    max_over_ranks = RP.max_over_ranks

    # ---- device-resident throughput (value) + per-kernel timing
    batch = Batch([r.spec() for r in reqs], precision=args.precision, device=dev, peel_mode=args.peel_mode)
    stream = torch.cuda.current_stream()
    ev = {k: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for k in ("eval", "gwht+noise", "peel", "collect")}
    acc = {k: 0.0 for k in ev}

    phases = (("eval", batch.eval), ("gwht+noise", batch.gwht_noise), ("peel", batch.peel),
              ("collect", batch.collect_async))
    phase_graphs = {}

    def step(timed):
        # each phase replayed from a graph of its own, as in the captured step
        # (the peeling loop is a conditional node there, not 15 eager iterations)
        for k, fn in phases:
            if k not in phase_graphs:
                torch.cuda.synchronize()
                pg = torch.cuda.CUDAGraph()
                with torch.cuda.graph(pg):
                    fn()
                phase_graphs[k] = pg
            if timed:
                ev[k][0].record(stream)
            phase_graphs[k].replay()
            if timed:
                ev[k][1].record(stream)
        if timed:
            torch.cuda.synchronize()
            for k in ev:
                acc[k] += ev[k][0].elapsed_time(ev[k][1])

    batch.capture()                         # one CUDA graph per step
    # three more workspaces with the same inputs: the timed steps go round the
    # four on four streams, four batches in flight as in the end-to-end run
    # (ms per step, same box: one in flight 1.163, two 1.005, three 0.996, four 0.983)
    NW = 4
    ring = [batch]
    for _ in range(NW - 1):
        bx = Batch([r.spec() for r in reqs], precision=args.precision, device=dev, peel_mode=args.peel_mode)
        bx.capture()
        ring.append(bx)
    streams = [torch.cuda.Stream(dev) for _ in range(NW)]
    for _ in range(max(args.warmup, 3)):
        for bx in ring:
            bx.run()
    barrier()
    # clocks: sampled every 50 ms from an untimed ~0.4 s run of the same step
    # just before the timed steps until their end (the K timed steps alone are
    # shorter than one sample)
    clk = Clocks(local)
    t_soak = time.perf_counter()
    while time.perf_counter() - t_soak < 0.4:
        for _ in range(20):
            batch.run()
        torch.cuda.synchronize()
    barrier()
    # serial replays on one stream (kept for comparison)
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0e.record(stream)
    for _ in range(args.steps):
        batch.run()
    t1e.record(stream)
    barrier()
    serial_ms = max_over_ranks(t0e.elapsed_time(t1e))
    # the headline: steps go round the workspaces on their streams (step i
    # waits for step i-NW on its own stream only), CUDA events from a start
    # event every stream waits on to the latest of their end events
    t0e, ends = torch.cuda.Event(enable_timing=True), [torch.cuda.Event(enable_timing=True) for _ in range(NW)]
    t0e.record(stream)
    for s in streams:
        s.wait_event(t0e)
    for i in range(args.steps):
        ring[i % NW].run(streams[i % NW])
    for e, s in zip(ends, streams):
        e.record(s)
    barrier()
    launches = sum(ring[i % NW].launches_per_run() for i in range(args.steps))   # library kernels the replays ran
    dev_ms = max(t0e.elapsed_time(e) for e in ends)
    clocks = clk.stop()
    dev_ms = max_over_ranks(dev_ms)
    value = J * args.steps * world / (dev_ms / 1e3)
    # per-phase timing pass (separate, so the headline loop has no extra syncs)
    for _ in range(args.steps):
        step(True)
    phase_ms = {k: v / args.steps for k, v in acc.items()}
    res = batch.results(collected=True)
    truth = [set(map(tuple, r.locq.T.tolist())) for r in reqs]
    found = [len(set(map(tuple, k.tolist())) & t) for (k, _, _, _), t in zip(res, truth)]
    iters = [int(c.iter) for (_, _, _, c) in res]
    nmse32 = [coef_nmse(k, v, r) for (k, v, _, _), r in zip(res, reqs)]

    # ---- end to end through the public API, host buffers: a TransformStream
    # pipelines the steps (host packing / parsing of one batch overlaps the
    # GPU's work on the next); every step still packs and uploads its inputs
    # and reads back its results inside the timed region
    # a ring of five workspaces, four batches in flight: the host's packing and
    # parsing of one batch hides behind the GPU's work on the next four (ms
    # per batch, same box: two in flight 1.18, three 1.10, four 1.08)
    from collections import deque
    AHEAD = 4
    ts = TransformStream(precision=args.precision, depth=AHEAD + 1)
    for _ in range(max(args.warmup, 3)):
        tks = [ts.submit(reqs) for _ in range(AHEAD + 1)]
        for tk in tks:
            ts.result(tk)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    inflight = deque()
    for i in range(args.steps):
        inflight.append(ts.submit(reqs))
        if len(inflight) > AHEAD:
            ts.result(inflight.popleft())
    while inflight:
        ts.result(inflight.popleft())
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = J * args.steps * world / e2e_s
    b2 = ts.last_batch()
    h2d = int(b2.h2d_bytes)
    d2h = int(b2.d2h_bytes)
    # batch completion latency: one synchronous call at a time
    lat = []
    for i in range(max(args.warmup, 3) + args.steps):
        barrier()
        t = time.perf_counter()
        transform_batch(reqs, precision=args.precision)
        torch.cuda.synchronize()
        if i >= max(args.warmup, 3):
            lat.append(time.perf_counter() - t)

    # ---- FP64 plain: one transform per launch sequence, FP64 everywhere
    b64 = Batch([reqs[0].spec()], precision="fp64", device=dev)

    def step64():
        b64.eval(); b64.gwht_noise(); b64.peel(); b64.collect_async()
    for _ in range(2):
        step64()
    barrier()
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n64 = max(2, args.steps // 2)
    a.record(stream)
    for _ in range(n64):
        step64()
    z.record(stream)
    torch.cuda.synchronize()
    fp64_tps = n64 / (a.elapsed_time(z) / 1e3)
    k64, v64, _, _ = b64.results(collected=True)[0]
    nmse64 = coef_nmse(k64, v64, reqs[0])
    same_support = set(map(tuple, k64.tolist())) == set(map(tuple, res[0][0].tolist()))

    own = pin_own_inputs(batch, reqs[0])
    # the optional FP64 re-projection against the raw bins (off on the parity
    # path): its NMSE against the truth beside the default's, and its cost
    brp = Batch([r.spec() for r in reqs], precision=args.precision, device=dev, reproject=True)
    brp.step()
    torch.cuda.synchronize()
    a_, z_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record(stream)
    brp.collect_async()
    z_.record(stream)
    res_rp = brp.results(collected=True)
    nmse_rp = [coef_nmse(k, v, r) for (k, v, _, _), r in zip(res_rp, reqs)]
    reproj = {"nmse_vs_truth_mean": float(np.mean(nmse_rp)), "nmse_vs_truth_max": float(np.max(nmse_rp)),
              "same_support_as_default": sum(set(map(tuple, k.tolist())) == set(map(tuple, k0.tolist()))
                                             for (k, _, _, _), (k0, _, _, _) in zip(res_rp, res)),
              "collect_plus_reprojection_ms": a_.elapsed_time(z_),
              "note": "FP64 re-projection of every recovered coefficient against the raw bins, all other "
                      "recovered coefficients removed (qsft_reproject); not the reference's estimate"}
    del brp
    serving = run_serving(args, dev) if args.serve_requests > 0 else None

    if rank != 0:
        RP.shutdown()
        return
    # ---- roofline of the dominant kernel (coset evaluation) and of the GWHT
    w = WORKLOAD
    samples = w["C"] * w["R"] * (w["n"] + 1) * w["q"] ** w["b"]
    # algorithmic work of the evaluation: one complex multiply-add (8 flops)
    # per (sample, support vector); the GEMM issues more tensor-core flops
    # (hi/lo halves, the real embedding of the complex product, N padding)
    eval_flops = 8.0 * samples * w["S"] * J
    p = batch.plan
    if batch.eval_method() == "gemm":
        spc = 64 // p.gm_kps
        s_pad = -(-w["S"] // spc) * spc
        issued = 2.0 * J * w["C"] * w["q"] ** w["b"] * (p.gm_kps * s_pad) * p.gm_npmax
    else:
        issued = None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    bf16 = peaks.get("bf16_tflops", 1900.0)
    hbm = peaks.get("hbm_gbs", 6800.0)
    e_ms = phase_ms["eval"]
    g_ms = phase_ms["gwht+noise"]
    gwht_bytes = 2.0 * samples * 8 * J
    roofline = {"kernel": "eval_cosets_gemm (operand + GEMM kernels)", "bound": "tensor",
                "achieved": eval_flops / (e_ms / 1e3) / 1e12,
                "peak": bf16, "unit": "TFLOP/s",
                "traffic": NCU_TRAFFIC["eval"] * J / NCU_TRAFFIC["batch"],
                "peak_source": "measured" if "bf16_tflops" in peaks else "fallback",
                "issued_tflops": None if issued is None else issued / (e_ms / 1e3) / 1e12}
    roofline["frac"] = roofline["achieved"] / roofline["peak"]
    roofline["traffic_unit"] = "bytes per launch (ncu, prep + GEMM kernels)"
    from qsft_gb300 import autotune
    sched = _lib.GWHT_SCHEDULES.get(autotune.selected(w["q"], w["b"], args.precision), "?")
    roof_gwht = {"kernel": f"gwht, schedule {sched} (transform + bin noise, one read and one write)", "bound": "hbm",
                 "achieved": gwht_bytes / (g_ms / 1e3) / 1e9, "peak": hbm,
                 "unit": "GB/s", "traffic": NCU_TRAFFIC["gwht"] * J / NCU_TRAFFIC["batch"],
                 "algorithmic_bytes": gwht_bytes,
                 "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    roof_gwht["frac"] = roof_gwht["achieved"] / roof_gwht["peak"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
        "data": "synthetic (seeded, reference generators)",
        "config": {"workload": "q4_n20_b7_C3_nso_R2_S1000_10dB", **WORKLOAD, "batch": J,
                   "parallelism": f"replicas x{world}", "peel_mode": args.peel_mode, "l2": "inputs > L2 (bins %.0f MB/step)" %
                   (samples * 8 * J / 1e6)},
        "value_note": "inputs resident on the device; steps go round four captured workspaces on four "
                      "streams (four batches in flight, as in e2e)",
        "value_serial_replay": J * args.steps * world / (serial_ms / 1e3),
        "latency_ms": {"p50": float(np.percentile(lat, 50) * 1e3), "p99": float(np.percentile(lat, 99) * 1e3),
                       "note": "batch completion latency through transform_batch"},
        "phase_ms": phase_ms,
        "fp64_plain": {"value": fp64_tps, "unit": UNIT, "batched_fp32_over_fp64_plain": value / fp64_tps},
        "accuracy": {"true_support_found": f"{sum(found)}/{J * w['S']}", "iterations": iters[:8],
                     "nmse_vs_truth_fp32": {"mean": float(np.mean(nmse32)), "max": float(np.max(nmse32))},
                     "nmse_limit": 1e-4,
                     "transform0": {"nmse_fp32_batched": nmse32[0], "nmse_fp64_plain": nmse64,
                                    "nmse_rel_diff": abs(nmse32[0] - nmse64) / max(nmse64, 1e-300),
                                    "same_support": bool(same_support)},
                     "oracle_on_own_inputs": own, "reprojection_fp64": reproj},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": roofline, "roofline_gwht": roof_gwht, "clocks": clocks,
        "gwht_schedules": __import__("qsft_gb300.autotune", fromlist=["table"]).table(),
    }
    if serving is not None:
        line["serving_mix"] = serving
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_record(cpu_transforms(2, 1, args.seed))
    print(json.dumps(line), flush=True)
    RP.shutdown()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
