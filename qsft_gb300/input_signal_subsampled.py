"""SubsampledSignal: the plugin point of the q-SFT API (qsft/input_signal_subsampled.py).

Subclass it and implement ``subsample(query_indices)`` exactly as with the
reference; the framework forms the query cosets, calls ``subsample`` once per
(group, delay block) with decimal indices, and computes every sub-transform on
the GPU.  Subclasses that can evaluate their function on the device (like
``SyntheticSubsampledSignal``) override ``_sample_device`` and never see a
decimal index.

The bins of every (group c, repeat r, delay p) live on the device as a
``(C, R, P, q^b)`` complex tensor per b in ``all_bs``; ``Us[i][j][b]`` exposes
the reference's nested layout as ``(P, q^b)`` CUDA tensor views.
"""
from pathlib import Path

import numpy as np
import torch

from .engine import complex_dtype, gwht_device, precision_code
from .query import get_Ms_and_Ds
from .utils import load_data, qary_ints, qary_vec_to_dec, save_data


class Signal:
    """Base signal (qsft/input_signal.py:17-96), reduced to the parameters the
    subsampled path reads."""

    def __init__(self, **kwargs):
        self._set_params(**kwargs)
        self._init_signal()

    def _set_params(self, **kwargs):  # qsft/input_signal.py:42-51
        self.n = kwargs.get("n")
        self.q = kwargs.get("q")
        self.noise_sd = kwargs.get("noise_sd", 0)
        self.N = self.q ** self.n
        self.signal_t = kwargs.get("signal_t")
        self.signal_w = kwargs.get("signal_w")
        self.foldername = kwargs.get("folder")

    def _init_signal(self):
        raise NotImplementedError

    def shape(self):  # qsft/input_signal.py:73-80
        return tuple([self.q for _ in range(self.n)])


class _UsView:
    """Us[i][j][b] -> (P, q^b) device view of the bins (reference layout)."""

    def __init__(self, sig):
        self._sig = sig

    def __len__(self):
        return len(self._sig.Ms)

    def __getitem__(self, i):
        sig = self._sig
        return [{b: sig._bins[b][i, j] for b in sig.all_bs} for j in range(len(sig.Ds[i]))]


class SubsampledSignal(Signal):
    """See module docstring.  Extra keyword arguments over the reference:
    ``precision`` ("fp32" | "fp64", default "fp32") of the device bins."""

    def _set_params(self, **kwargs):  # qsft/input_signal_subsampled.py:47-63
        self.n = kwargs.get("n")
        self.q = kwargs.get("q")
        self.N = self.q ** self.n
        self.signal_w = kwargs.get("signal_w")
        self.query_args = kwargs.get("query_args")
        self.b = self.query_args.get("b")
        self.all_bs = self.query_args.get("all_bs", [self.b])
        self.num_subsample = self.query_args.get("num_subsample")
        if "num_repeat" not in self.query_args:
            self.query_args["num_repeat"] = 1
        self.num_repeat = self.query_args.get("num_repeat")
        self.subsampling_method = self.query_args.get("subsampling_method")
        self.delays_method_source = self.query_args.get("delays_method_source")
        self.delays_method_channel = self.query_args.get("delays_method_channel")
        self.L = None
        self.foldername = kwargs.get("folder")
        self.precision = kwargs.get("precision", getattr(self, "precision", "fp32"))
        self._bins = {}

    def _init_signal(self):  # qsft/input_signal_subsampled.py:65-73
        if self.subsampling_method == "uniform":
            self._subsample_uniform()
        else:
            self._set_Ms_and_Ds_qsft()
            self._subsample_qsft()

    def _set_Ms_and_Ds_qsft(self):  # qsft/input_signal_subsampled.py:92-105
        if self.foldername:
            Path(f"{self.foldername}").mkdir(exist_ok=True)
            path = Path(f"{self.foldername}/Ms_and_Ds.pickle")
            if path.is_file():
                self.Ms, self.Ds = load_data(path)
            else:
                self.Ms, self.Ds = get_Ms_and_Ds(self.n, self.q, **self.query_args)
                save_data((self.Ms, self.Ds), path)
        else:
            self.Ms, self.Ds = get_Ms_and_Ds(self.n, self.q, **self.query_args)

    # ------------------------------------------------------------ sampling
    def _rows_P(self):
        return self.Ds[0][0].shape[0]

    def _sample_device(self):
        """Device samples (C, R, P, q^b) of every coset, or None when the
        subclass evaluates on the host through ``subsample``."""
        return None

    def _sample_host(self):
        """The reference's sampling loop (qsft/input_signal_subsampled.py:119-149):
        decimal query indices per (group, repeat), ``subsample`` per block."""
        C, R, P, B = len(self.Ms), len(self.Ds[0]), self._rows_P(), self.q ** self.b
        out = np.zeros((C, R, P, B), dtype=np.complex128)
        for i in range(C):
            for j in range(R):
                path = Path(f"{self.foldername}/samples/M{i}_D{j}.pickle") if self.foldername else None
                if path is not None and path.is_file():
                    samples = np.asarray(load_data(path))
                else:
                    query_indices = self._get_qsft_query_indices(self.Ms[i], self.Ds[i][j])
                    block_length = len(query_indices[0])
                    samples = np.zeros((len(query_indices), block_length), dtype=np.complex128)
                    if block_length > 10000:
                        for k in range(len(query_indices)):
                            samples[k] = self.subsample(query_indices[k])
                    else:
                        all_samples = self.subsample(np.concatenate(query_indices))
                        for k in range(len(query_indices)):
                            samples[k] = all_samples[k * block_length:(k + 1) * block_length]
                    if path is not None:
                        Path(f"{self.foldername}/samples").mkdir(exist_ok=True, parents=True)
                        save_data(samples, path)
                out[i, j] = samples
        dev = torch.device("cuda", torch.cuda.current_device())
        return torch.from_numpy(out).to(dev).to(complex_dtype(precision_code(self.precision)))

    def _subsample_qsft(self):
        """Sample every coset and take the sub-transforms for each b in all_bs
        (qsft/input_signal_subsampled.py:107-155, 264-266), on the GPU.

        With a folder, the reference's cache files are read and written:
        ``transforms/U{i}_{j}.pickle`` holds (Us[i][j], transformTimes[i][j]) --
        {b: (P, q^b) complex array}, {b: seconds} -- and
        ``samples/M{i}_D{j}.pickle`` the (P, q^b) samples of group i, repeat j
        (zlib pickles, qsft/utils.py:189-197).  A folder the reference filled
        is thus reused, and the reference can reuse one filled here."""
        C, R = len(self.Ms), len(self.Ds[0])
        cached = self._load_transforms()
        if cached is not None:
            self._bins, self.transformTimes = cached
            return
        samples = self._load_samples()
        if samples is None:
            samples = self._sample_device()
            if samples is None:
                samples = self._sample_host()
            self._save_samples(samples)
        P = samples.shape[2]
        bins = {}
        times = {}
        for b in sorted(self.all_bs):
            stride = self.q ** (self.b - b)
            x = samples.reshape(C, R, P, -1)[..., ::stride].contiguous() if b != self.b else None
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            if b != self.b:
                gwht_device(x, self.q, b)
                bins[b] = x
            else:
                bins[b] = gwht_device(samples.contiguous(), self.q, b)
            ev1.record()
            ev1.synchronize()
            times[b] = ev0.elapsed_time(ev1) / 1e3 / (C * R)
        self._bins = bins
        # per-(group, repeat) GWHT time: the batched launch's time split evenly
        self.transformTimes = [[dict(times) for _ in range(R)] for _ in range(C)]
        self._save_transforms()

    def _cache_path(self, kind, i, j):
        if kind == "transforms":
            return Path(f"{self.foldername}/transforms/U{i}_{j}.pickle")   # qsft/input_signal_subsampled.py:122
        return Path(f"{self.foldername}/samples/M{i}_D{j}.pickle")         # qsft/input_signal_subsampled.py:128

    def _load_transforms(self):
        """Every (group, repeat) from transforms/U{i}_{j}.pickle when all files
        exist and hold every b of all_bs; else None."""
        if not self.foldername:
            return None
        C, R = len(self.Ms), len(self.Ds[0])
        paths = [[self._cache_path("transforms", i, j) for j in range(R)] for i in range(C)]
        if not all(p.is_file() for row in paths for p in row):
            return None
        data = [[load_data(p) for p in row] for row in paths]
        if not all(b in d[0] for row in data for d in row for b in self.all_bs):
            return None
        dev = torch.device("cuda", torch.cuda.current_device())
        cdt = complex_dtype(precision_code(self.precision))
        bins = {b: torch.from_numpy(np.stack([np.stack([np.asarray(d[0][b], dtype=np.complex128) for d in row])
                                              for row in data])).to(dev).to(cdt) for b in self.all_bs}
        times = [[dict(d[1]) for d in row] for row in data]
        return bins, times

    def _save_transforms(self):
        if not self.foldername:
            return
        Path(f"{self.foldername}/transforms").mkdir(exist_ok=True, parents=True)
        host = {b: t.cpu().numpy().astype(np.complex128) for b, t in self._bins.items()}
        for i in range(len(self.Ms)):
            for j in range(len(self.Ds[i])):
                save_data(({b: host[b][i, j] for b in host}, dict(self.transformTimes[i][j])),
                          self._cache_path("transforms", i, j))

    def _load_samples(self):
        """(C, R, P, q^b) device samples from samples/M{i}_D{j}.pickle when every
        file exists; else None."""
        if not self.foldername:
            return None
        C, R = len(self.Ms), len(self.Ds[0])
        paths = [[self._cache_path("samples", i, j) for j in range(R)] for i in range(C)]
        if not all(p.is_file() for row in paths for p in row):
            return None
        arr = np.stack([np.stack([np.asarray(load_data(p), dtype=np.complex128) for p in row]) for row in paths])
        dev = torch.device("cuda", torch.cuda.current_device())
        return torch.from_numpy(arr).to(dev).to(complex_dtype(precision_code(self.precision)))

    def _save_samples(self, samples):
        if not self.foldername:
            return
        Path(f"{self.foldername}/samples").mkdir(exist_ok=True, parents=True)
        host = samples.cpu().numpy().astype(np.complex128)
        for i in range(host.shape[0]):
            for j in range(host.shape[1]):
                p = self._cache_path("samples", i, j)
                if not p.is_file():
                    save_data(host[i, j], p)

    def _subsample_uniform(self):  # qsft/input_signal_subsampled.py:157-173
        import random
        from math import floor
        n_samples = self.query_args["n_samples"]
        query_indices = [floor(random.uniform(0, 1) * self.N) for _ in range(n_samples)]
        samples = self.subsample(query_indices)
        self.signal_t = dict(zip(query_indices, samples))

    @property
    def Us(self):
        return _UsView(self)

    def get_all_qary_vectors(self):  # qsft/input_signal_subsampled.py:175-178
        if self.L is None:
            self.L = np.array(qary_ints(self.b, self.q))
        return self.L

    def subsample(self, query_indices):  # qsft/input_signal_subsampled.py:180-181
        raise NotImplementedError

    def _get_qsft_query_indices(self, M, D_sub):  # qsft/input_signal_subsampled.py:183-206
        b = M.shape[1]
        L = self.get_all_qary_vectors()
        ML = (M @ L) % self.q
        base = np.array([(ML + np.outer(d, np.ones(self.q ** b, dtype=int))) % self.q for d in D_sub])
        return [qary_vec_to_dec(base[i], self.q) for i in range(len(base))]

    # ------------------------------------------------------------ access
    def get_MDU(self, ret_num_subsample, ret_num_repeat, b, trans_times=False):
        """qsft/input_signal_subsampled.py:225-262: a random selection (two
        ``np.random.choice`` draws) of groups and repeats; bins stay on the device."""
        if ret_num_subsample <= self.num_subsample and ret_num_repeat <= self.num_repeat and b <= self.b:
            subsample_idx = np.random.choice(self.num_subsample, ret_num_subsample, replace=False)
            delay_idx = np.random.choice(self.num_repeat, ret_num_repeat, replace=False)
            Ms, Ds, Us, Ts = [], [], [], []
            for i in subsample_idx:
                Ms.append(self.Ms[i][:, :b])
                Ds.append([self.Ds[i][j] for j in delay_idx])
                Us.append([self._bins[b][i, j] for j in delay_idx])
                Ts.append([self.transformTimes[i][j][b] for j in delay_idx])
            self._last_selection = (subsample_idx, delay_idx)
            return (Ms, Ds, Us, Ts) if trans_times else (Ms, Ds, Us)
        raise ValueError("There are not enough Ms or Ds.")

    def get_source_parity(self):  # qsft/input_signal_subsampled.py:268-269
        return self.Ds[0][0].shape[0]

