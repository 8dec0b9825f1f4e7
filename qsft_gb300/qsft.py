"""QSFT: the sparse q-ary Fourier transform driver (qsft/qsft.py), peeling on the GPU."""
import time

import numpy as np
import torch

from .engine import MAX_ITER, Batch, JobSpec
from .input_signal_subsampled import SubsampledSignal
from .reed_solomon import ReedSolomon
from .utils import calc_hamming_weight, sort_qary_vecs


class QSFT:
    """Same constructor keywords as the reference (qsft/qsft.py:47-53):
    reconstruct_method_source ("identity" | "coded"), reconstruct_method_channel
    ("identity" | "nso"), num_subsample, num_repeat, b, source_decoder.
    ``noise_sd`` is accepted and ignored like the reference does.  Extra:
    ``max_iter`` (default 15, qsft/qsft.py:142); ``reproject`` (default False):
    re-estimate every recovered coefficient in FP64 against the raw bins with
    all other recovered coefficients removed (qsft_reproject) instead of the
    reference's running mean of the peeling's estimates (qsft/qsft.py:247-255)."""

    def __init__(self, **kwargs):
        self.reconstruct_method_source = kwargs.get("reconstruct_method_source")
        self.reconstruct_method_channel = kwargs.get("reconstruct_method_channel")
        self.num_subsample = kwargs.get("num_subsample")
        self.num_repeat = kwargs.get("num_repeat")
        self.b = kwargs.get("b")
        self.source_decoder = kwargs.get("source_decoder", None)
        self.max_iter = kwargs.get("max_iter", MAX_ITER)
        self.reproject = bool(kwargs.get("reproject", False))

    def _rs(self, signal):
        dec = self.source_decoder
        if isinstance(dec, ReedSolomon):
            return dec
        if hasattr(dec, "__self__") and isinstance(dec.__self__, ReedSolomon):
            return dec.__self__
        t = signal.query_args.get("t")
        if t is None:
            raise ValueError("coded source needs source_decoder=get_reed_solomon_dec(n, t, q) or query_args['t']")
        return ReedSolomon(signal.n, t, signal.q)

    def transform(self, signal, verbosity=0, report=False, timing_verbose=False, **kwargs):
        """qsft/qsft.py:56-281.  Returns the dict k -> coefficient, or the report dict."""
        if not isinstance(signal, SubsampledSignal):
            raise NotImplementedError("QSFT currently only supports signals that inherit from SubsampledSignal")
        if self.reconstruct_method_channel not in ("identity", "nso"):
            raise NotImplementedError(f"reconstruct_method_channel={self.reconstruct_method_channel!r}")
        q, n, b = signal.q, signal.n, self.b
        Ms, Ds, Us, Ts = signal.get_MDU(self.num_subsample, self.num_repeat, self.b, trans_times=True)
        transform_time = float(np.sum(Ts))
        if timing_verbose:
            print(f"Transform Time:{transform_time}", flush=True)
        C, R = len(Ms), len(Ds[0])
        P = signal.get_source_parity()
        D = np.stack([np.vstack(d) for d in Ds])
        U = torch.stack([torch.cat(list(u), dim=0) for u in Us])   # (C, R*P, q^b) on the device
        cutoff = 1e-9 + 1.5 * (signal.noise_sd ** 2) / (q ** b)     # qsft/qsft.py:124-126
        cutoff = kwargs.get("cutoff", cutoff)
        if verbosity >= 2:
            print("cutoff = ", cutoff, flush=True)
        src = self.reconstruct_method_source or "identity"
        rs = self._rs(signal) if src == "coded" else None
        nz = getattr(signal, "_device_noise", None)
        spec = JobSpec(q, n, b, np.stack(Ms), D, R, P, chan=self.reconstruct_method_channel, src=src, cutoff=cutoff,
                       U=U, rs=rs, max_iter=self.max_iter,
                       noise_nu=nz[0] if nz else 0.0, noise_seed=nz[1] if nz else 0)
        peeling_start = time.time()
        batch = Batch([spec], precision=U.dtype, reproject=self.reproject)
        if nz:
            batch.add_noise()
        batch.peel(self.max_iter)
        keys, vals, counts, ctrl = batch.results()[0]
        peeling_time = time.time() - peeling_start
        if timing_verbose:
            print(f"Peeling Time:{peeling_time}", flush=True)
        if verbosity >= 2:
            print(f"iterations {ctrl.iter}, balls peeled {ctrl.num_peeling}", flush=True)
        gwht = {tuple(int(x) for x in k): complex(v) for k, v in zip(keys, vals)}
        self.last_iterations = int(ctrl.iter)
        if not report:
            return gwht
        n_samples = C * R * P * q ** b
        if len(gwht) > 0:
            loc = list(gwht.keys())
            if kwargs.get("sort", False):
                loc = sort_qary_vecs(loc)
            hw = calc_hamming_weight(loc)
            avg_hw, max_hw = float(np.mean(hw)), int(np.max(hw))
        else:
            loc, avg_hw, max_hw = [], 0, 0
        return {"gwht": gwht, "runtime": transform_time + peeling_time, "n_samples": n_samples, "locations": loc,
                "avg_hamming_weight": avg_hw, "max_hamming_weight": max_hw}
