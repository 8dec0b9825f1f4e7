"""Synthetic sparse signals (synt_exp/synt_src/synthetic_signal.py), evaluated on the GPU.

``SyntheticSubsampledSignal`` evaluates f(x) = sum_s a_s exp(2 pi i <x, k_s> / q)
on every query coset with ``qsft_eval_cosets`` (no decimal indices), and
adds the bin-domain noise of its ``get_MDU`` override either from the host's
numpy stream in the reference's draw order (``noise="host"``, the default:
same seed -> same noise as the reference) or from the device Philox stream
(``noise="device"``).
"""
import numpy as np
import torch

from .engine import Batch, JobSpec, add_bins_, eval_points_device, precision_code, complex_dtype
from .input_signal_subsampled import SubsampledSignal
from .reed_solomon import ReedSolomon
from .utils import dec_to_qary_vec, qary_vec_to_dec, random_signal_strength_model, sort_qary_vecs


def generate_signal_w(n, q, sparsity, a_min, a_max, noise_sd=0, full=True, max_weight=None):
    """Random sparse transform, in the reference's RNG order
    (synt_exp/synt_src/synthetic_signal.py:10-38).  full=True is not supported
    (it materialises all q^n coefficients)."""
    locq, strengths = draw_support(n, q, sparsity, a_min, a_max, max_weight)
    if full:
        raise NotImplementedError("full=True materialises q^n coefficients; use full=False")
    signal_w = dict(zip(list(map(tuple, locq.T)), strengths))
    return signal_w, locq, strengths


def draw_support(n, q, sparsity, a_min, a_max, max_weight=None):
    """The support (n x S, sorted) and coefficients of ``generate_signal_w``, drawn
    in the same RNG order, without building the {k: a} dict."""
    max_weight = n if max_weight is None else max_weight
    if max_weight == n:
        locq = sort_qary_vecs(np.random.randint(q, size=(n, sparsity)).T).T
    else:
        vals = np.random.randint(q - 1, size=(max_weight, sparsity)) + 1
        pos = np.random.choice(a=n, size=(sparsity, max_weight))
        locq = np.zeros((n, sparsity), dtype=int)
        for i in range(sparsity):
            locq[pos[i, :], i] = vals[:, i]
        locq = sort_qary_vecs(locq.T).T
    strengths = random_signal_strength_model(sparsity, a_min, a_max)
    return locq, strengths


def get_random_subsampled_signal(n, q, noise_sd, sparsity, a_min, a_max, query_args, max_weight=None, **kw):
    """synt_exp/synt_src/synthetic_signal.py:70-85 (extra keywords: precision, noise)."""
    signal_w, locq, strengths = generate_signal_w(n, q, sparsity, a_min, a_max, noise_sd, full=False,
                                                  max_weight=max_weight)
    return SyntheticSubsampledSignal(signal_w=signal_w, locq=locq, strengths=strengths, noise_sd=noise_sd, n=n, q=q,
                                     query_args=query_args, **kw)


class SyntheticSubsampledSignal(SubsampledSignal):
    """synt_exp/synt_src/synthetic_signal.py:88-130 on the GPU."""

    def __init__(self, **kwargs):
        self.q = kwargs["q"]
        self.n = kwargs["n"]
        self.locq = kwargs["locq"]
        self.noise_sd = kwargs["noise_sd"]
        self.strengths = kwargs["strengths"]
        self.noise = kwargs.get("noise", "host")
        self.precision = kwargs.get("precision", "fp32")
        super().__init__(**kwargs)

    def _sample_device(self):
        """All C x R x P cosets in one qsft_eval_cosets launch."""
        C, R, P = len(self.Ms), len(self.Ds[0]), self._rows_P()
        D = np.stack([np.vstack(self.Ds[i]) for i in range(C)])
        coded = self.delays_method_source == "coded"
        rs = ReedSolomon(self.n, self.query_args.get("t"), self.q) if coded else None
        spec = JobSpec(self.q, self.n, self.b, np.stack(self.Ms), D, R, P, K=np.asarray(self.locq).T,
                       A=self.strengths, src="coded" if coded else "identity", rs=rs,
                       chan=self.delays_method_channel or "identity")
        batch = Batch([spec], precision=self.precision)
        batch.eval()
        return batch.job_U(0).view(C, R, P, -1)

    def subsample(self, query_indices):
        """f at decimal query indices (synthetic_signal.py:108-118), evaluated on the GPU."""
        X = dec_to_qary_vec(np.asarray(query_indices), self.q, self.n).T
        out = eval_points_device(X, np.asarray(self.locq).T, self.strengths, self.q, precision="fp64")
        return out.cpu().numpy()

    def get_MDU(self, ret_num_subsample, ret_num_repeat, b, trans_times=False):
        """Adds bin-domain AWGN N(0, nu^2)(1+i), nu = sigma / sqrt(2 q^b), to a copy of
        each selected (P, q^b) block (synthetic_signal.py:120-130)."""
        mdu = super().get_MDU(ret_num_subsample, ret_num_repeat, b, trans_times)
        nu = self.noise_sd / np.sqrt(2 * self.q ** b)
        for i in range(len(mdu[2])):
            for j in range(len(mdu[2][i])):
                U = mdu[2][i][j]
                size = tuple(U.shape)
                Un = U.clone()
                if self.noise == "host":
                    w = np.random.normal(0, nu, size=size + (2,)).view(np.complex128).reshape(size)
                    add_bins_(Un, torch.from_numpy(w).to(U.device))
                mdu[2][i][j] = Un
        if self.noise != "host":
            self._device_noise = (nu, int(np.random.randint(0, 2 ** 62)))
        else:
            self._device_noise = None
        return mdu


__all__ = ["generate_signal_w", "get_random_subsampled_signal", "SyntheticSubsampledSignal",
           "qary_vec_to_dec", "precision_code", "complex_dtype"]
