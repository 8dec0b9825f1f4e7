"""The reference's experiment harness (qsft/test_helper.py) with the QSFT
methods and the time-domain test NMSE on the GPU.

``TestHelper`` keeps the reference's constructor, data-loading conventions
(train data per method in ``exp_dir/train*``, uniform test samples without
noise in ``exp_dir/test``), ``compute_model`` and ``test_model``.  Subclasses
provide ``generate_signal(signal_args)`` as in the reference.

``test_nmse`` is ``_test_qary`` (qsft/test_helper.py:235-260):
||y_hat - y||^2 / ||y||^2 with y_hat(x) = sum_k beta_k omega^(<x, k>) at the
test points -- the same sparse exponential sum as the coset evaluation,
computed by ``qsft_eval_points`` in FP64 over the recovered support.
"""
import json

import numpy as np
import torch

from .engine import eval_points_device, gwht_device
from .qsft import QSFT
from .query import get_reed_solomon_dec
from .utils import dec_to_qary_vec

__all__ = ["TestHelper", "test_nmse"]


def test_nmse(beta, query_indices, samples, q, n, batch_size=1 << 20):
    """NMSE of the sparse transform `beta` ({k tuple: coefficient}) against
    `samples` taken at decimal `query_indices` (qsft/test_helper.py:235-260).
    An empty `beta` scores 1, as in the reference."""
    if len(beta) == 0:
        return 1
    keys = np.array([list(k) for k in beta.keys()], dtype=np.int64).reshape(-1, n)
    vals = np.array(list(beta.values()), dtype=np.complex128)
    samples = np.asarray(samples, dtype=np.complex128)
    idx = list(query_indices)
    y_hat = []
    for i in range(0, len(idx), batch_size):
        X = dec_to_qary_vec(np.array(idx[i:i + batch_size]), q, n).T
        y_hat.append(eval_points_device(X, keys, vals, q, precision="fp64").cpu().numpy())
    y_hat = np.concatenate(y_hat)
    return float(np.linalg.norm(y_hat - samples) ** 2 / np.linalg.norm(samples) ** 2)


test_nmse.__test__ = False  # a library function, not a pytest test


class NpEncoder(json.JSONEncoder):  # qsft/utils.py NpEncoder: numpy scalars/arrays in config.json
    def default(self, obj):
        if isinstance(obj, np.integer):
            return int(obj)
        if isinstance(obj, np.floating):
            return float(obj)
        if isinstance(obj, np.ndarray):
            return obj.tolist()
        return super().default(obj)


class TestHelper:
    """qsft/test_helper.py:9-52 (constructor) and :120-140, 235-260."""
    __test__ = False  # not a pytest class

    def __init__(self, signal_args, methods, subsampling_args, test_args, exp_dir, subsampling=True):
        self.n = signal_args["n"]
        self.q = signal_args["q"]
        self.exp_dir = exp_dir
        self.subsampling = subsampling
        config_path = self.exp_dir / "config.json"
        if not config_path.is_file():
            with open(config_path, "w") as f:
                json.dump({"query_args": subsampling_args}, f, cls=NpEncoder)
        self.signal_args = signal_args
        self.subsampling_args = subsampling_args
        self.test_args = test_args
        if self.subsampling:
            if "qsft" in methods:
                self.train_signal = self.load_train_data()
            if "qsft_coded" in methods:
                self.train_signal_coded = self.load_train_data_coded()
            if "qsft_binary" in methods or "lasso" in methods:
                raise NotImplementedError("binary QSFT and LASSO are outside the GPU path")
            self.test_signal = self.load_test_data()
        else:
            raise NotImplementedError("full (non-subsampled) data loading is not implemented in the reference either")

    def generate_signal(self, signal_args):
        raise NotImplementedError

    def load_train_data(self):  # qsft/test_helper.py:54-66
        signal_args = self.signal_args.copy()
        query_args = self.subsampling_args.copy()
        query_args.update({"subsampling_method": "qsft", "query_method": "complex",
                           "delays_method_source": "identity", "delays_method_channel": "nso"})
        signal_args["folder"] = self.exp_dir / "train"
        signal_args["query_args"] = query_args
        return self.generate_signal(signal_args)

    def load_train_data_coded(self):  # qsft/test_helper.py:68-81
        signal_args = self.signal_args.copy()
        query_args = self.subsampling_args.copy()
        query_args.update({"subsampling_method": "qsft", "query_method": "complex",
                           "delays_method_source": "coded", "delays_method_channel": "nso",
                           "t": signal_args["t"]})
        signal_args["folder"] = self.exp_dir / "train_coded"
        signal_args["query_args"] = query_args
        return self.generate_signal(signal_args)

    def load_test_data(self):  # qsft/test_helper.py:109-115
        signal_args = self.signal_args.copy()
        (self.exp_dir / "test").mkdir(exist_ok=True)
        signal_args["query_args"] = {"subsampling_method": "uniform", "n_samples": self.test_args.get("n_samples")}
        signal_args["folder"] = self.exp_dir / "test"
        signal_args["noise_sd"] = 0
        return self.generate_signal(signal_args)

    def compute_model(self, method, model_kwargs, report=False, verbosity=0):  # qsft/test_helper.py:121-133
        if method == "gwht":
            return self._calculate_gwht(model_kwargs, report, verbosity)
        if method == "qsft":
            return self._calculate_qsft(model_kwargs, report, verbosity)
        if method == "qsft_coded":
            return self._calculate_qsft_coded(model_kwargs, report, verbosity)
        raise NotImplementedError()

    def test_model(self, method, **kwargs):  # qsft/test_helper.py:135-141
        if method in ("qsft", "qsft_coded", "lasso"):
            return self._test_qary(**kwargs)
        raise NotImplementedError()

    def _calculate_gwht(self, model_kwargs, report=False, verbosity=0):  # qsft/test_helper.py:143-154
        """Full q^n-point GWHT of `train_signal` (an array of q^n samples), on the GPU.  The
        reference passes q=4 (its RNA application's alphabet); the signal's own q is used here."""
        x = torch.as_tensor(np.ascontiguousarray(self.train_signal, dtype=np.complex128)).cuda().contiguous()
        return gwht_device(x, q=self.q, b=self.n).cpu().numpy()

    def _calculate_qsft(self, model_kwargs, report=False, verbosity=0):  # qsft/test_helper.py:156-171
        qsft = QSFT(reconstruct_method_source="identity", reconstruct_method_channel="nso",
                    num_subsample=model_kwargs["num_subsample"], num_repeat=model_kwargs["num_repeat"],
                    b=model_kwargs["b"])
        self.train_signal.noise_sd = model_kwargs["noise_sd"]
        return qsft.transform(self.train_signal, verbosity=verbosity, timing_verbose=(verbosity >= 1), report=report)

    def _calculate_qsft_coded(self, model_kwargs, report=False, verbosity=0):  # qsft/test_helper.py:173-191
        decoder = get_reed_solomon_dec(self.signal_args["n"], self.signal_args["t"], self.signal_args["q"])
        qsft = QSFT(reconstruct_method_source="coded", reconstruct_method_channel="nso",
                    num_subsample=model_kwargs["num_subsample"], num_repeat=model_kwargs["num_repeat"],
                    b=model_kwargs["b"], source_decoder=decoder)
        self.train_signal_coded.noise_sd = model_kwargs["noise_sd"]
        return qsft.transform(self.train_signal_coded, verbosity=verbosity, timing_verbose=(verbosity >= 1),
                              report=report)

    def _test_qary(self, beta):  # qsft/test_helper.py:235-260
        test_signal = self.test_signal.signal_t
        return test_nmse(beta, list(test_signal.keys()), list(test_signal.values()), self.q, self.n)
