import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def golden_cases(full_only=False):
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        name = os.path.basename(f)[:-4]
        if name.endswith("_pins"):  # single-function fixtures, not transform runs
            continue
        if full_only:
            with np.load(f) as z:
                if "Us_clean" not in z:
                    continue
        out.append(name)
    return out


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def case_query_args(z):
    qa = dict(query_method=str(z["query_method"]), num_subsample=int(z["C"]),
              delays_method_source=str(z["src"]), subsampling_method="qsft",
              delays_method_channel=str(z["ch"]), num_repeat=int(z["R"]), b=int(z["b"]))
    if "all_bs" in z and len(z["all_bs"]) > 1:
        qa["all_bs"] = [int(x) for x in z["all_bs"]]
    return qa


def transform_b(z):
    """b of the QSFT call (smaller than the signal's b for all_bs cases)."""
    return int(z["transform_b"]) if "transform_b" in z else int(z["b"])


def golden_dict(z):
    return {tuple(int(x) for x in k): complex(v) for k, v in zip(z["gwht_keys"], z["gwht_vals"])}


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)
