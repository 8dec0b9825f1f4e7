"""Timed CPU baseline: the oracle's restatement of the reference q-SFT on this
host's cores -- BENCHMARK INFRASTRUCTURE, never part of the product path.

A step is one whole transform of the noisy robust workload (q=4, n=20, b=7,
C=3, NSO delays with num_repeat=2, S=1000, 10 dB), end to end as the
reference runs it (get_random_subsampled_signal + QSFT.transform,
synt_exp/synt_src/synthetic_signal.py:70-130, qsft/qsft.py:56-281): draw the
signal and the query design, evaluate f on all C*R*P cosets with the
reference's formula exp(2 pi i X K / q) @ a (synthetic_signal.py:100-102),
take the GWHT of every row, add the bin noise and run the peeling loop.
Nothing is sampled or scaled: every step's time is one full transform.

Cores: the reference spreads the evaluation over a process pool
(synthetic_signal.py:108-118); here a thread pool over all host cores takes
batches of 1024 query points, each with one BLAS thread (the parent sets
OPENBLAS_NUM_THREADS=1 / OMP_NUM_THREADS=1 before this process imports numpy;
a multi-threaded BLAS under a thread pool oversubscribes the cores).

Run:  OPENBLAS_NUM_THREADS=1 OMP_NUM_THREADS=1 python -m oracle.cpu_baseline --steps K --warmup W
Prints one JSON line: {"step_s": [...], "threads": T, ...}.
"""
import argparse
import json
import os
import platform
import time

import numpy as np

from .qsft_oracle import OracleQSFT, OracleSignal, eval_points, noise_sd_for_snr, subsample_qsft

WORKLOAD = dict(q=4, n=20, b=7, S=1000, C=3, R=2, snr_db=10.0)
SMALL = dict(q=4, n=10, b=4, S=50, C=3, R=1, snr_db=None)   # warm-up: same code paths, 0.1 s
EVAL_BATCH = 1024


def one_transform(w, seed, threads):
    """Seconds of one end-to-end transform of workload `w`, and its result size."""
    q, n, b, S, C, R = w["q"], w["n"], w["b"], w["S"], w["C"], w["R"]
    noisy = w["snr_db"] is not None
    qa = dict(query_method="complex", num_subsample=C, b=b, delays_method_source="identity",
              delays_method_channel="nso" if noisy else "identity", num_repeat=R)
    t0 = time.perf_counter()
    np.random.seed(seed)
    sig = OracleSignal(n, q, S, 1, 10, noise_sd_for_snr(S, w["snr_db"]) if noisy else 0.0, qa, skip_sampling=True)
    sig.Us = subsample_qsft(sig.Ms, sig.Ds, q, lambda X: eval_points(X, sig.locq, sig.strengths, q, threads=threads,
                                                                     batch=EVAL_BATCH))
    res = OracleQSFT(num_subsample=C, num_repeat=R, b=b, reconstruct_method_source="identity",
                     reconstruct_method_channel=qa["delays_method_channel"]).transform(sig)
    return time.perf_counter() - t0, len(res)


def run(steps, warmup, seed=0, threads=None):
    threads = threads or os.cpu_count() or 1
    for i in range(warmup):
        one_transform(SMALL, seed + 10_000 + i, threads)
    times, found = [], []
    for i in range(steps):
        dt, m = one_transform(WORKLOAD, seed + i, threads)
        times.append(dt)
        found.append(m)
    return {"step_s": times, "found": found, "threads": threads, "nproc": os.cpu_count(),
            "machine": platform.machine(), "blas_threads": os.environ.get("OPENBLAS_NUM_THREADS"),
            "workload": WORKLOAD, "warmup_workload": SMALL}


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(run(a.steps, a.warmup, a.seed, a.threads or None)), flush=True)
