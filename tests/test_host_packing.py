"""Host side of a batch, without a GPU: packing the requests' digits and
coefficients into the staging arrays (one concatenation per array) gives
exactly the per-job layout the workspace offsets describe, zero padding
included; and the result parsing (one conversion for all rows, a view per
job) gives every job's keys -- high parts of coded entries included --,
values and counts, in arrays that do not share memory with the staging
buffers the next read-back overwrites; a device error in the read-back (a
job's table overflow in its control record, a nonzero status word) raises
instead of returning truncated results."""
import ctypes

import numpy as np
import pytest
import torch

from qsft_gb300 import _lib
from qsft_gb300.engine import Batch
from qsft_gb300.serve import random_request


def _specs():
    np.random.seed(3)
    reqs = [random_request(4, 20, 7, 300, C=3, R=2, snr_db=10.0),
            random_request(2, 24, 9, 100, C=3, R=1, snr_db=None, chan="identity"),
            random_request(5, 16, 3, 25, C=3, R=2, snr_db=20.0, src="coded", t=4, max_weight=4),
            random_request(3, 12, 5, 40, C=2, R=2, snr_db=10.0)]
    return [r.spec() for r in reqs]


def _host_batch(specs):
    b = Batch.__new__(Batch)
    b.lib = _lib.load()
    b.reproject = False
    b.prec = _lib.QSFT_F32
    b._build_layout(list(specs))
    return b


def test_pack_host_matches_layout():
    specs = _specs()
    b = _host_batch(specs)
    i8 = np.full(b.n_i8, 0x55, np.int8)            # garbage: the padding must come out zero
    a = np.full(max(b.n_a, 1), 7 + 7j, np.complex64)
    b._pack_host(specs, i8, a)
    want = np.zeros(b.n_i8, np.int8)
    wa = np.zeros(max(b.n_a, 1), np.complex64)
    for j, sp in enumerate(specs):
        jb = b.jobs_host[j]
        want[jb.off_M:jb.off_M + sp.M.size] = sp.M.ravel()
        want[jb.off_D:jb.off_D + sp.D.size] = sp.D.ravel()
        if sp.K is not None:
            want[jb.off_K:jb.off_K + sp.K.size] = sp.K.ravel()
        if sp.A is not None:
            wa[jb.off_A:jb.off_A + sp.A.size] = sp.A
        assert jb.max_iter == sp.max_iter and jb.noise_seed == sp.noise_seed
        assert jb.cutoff == sp.cutoff and jb.noise_nu == sp.noise_nu
    assert np.array_equal(i8, want)
    assert np.array_equal(a[:b.n_a], wa[:b.n_a])


def _read_back(b, counts, seed=11):
    """Synthetic read-back buffers of a batch: metadata (row count, per-job
    output index with the jobs' rows in reverse order, control records, status
    word) and random output rows."""
    J, ks = b.njobs, b.kstride
    cs = ctypes.sizeof(_lib.QsftCtrl) // 8
    rng = np.random.RandomState(seed)
    total = sum(counts)
    meta = np.zeros(1 + 2 * J + cs * J + 1, np.int64)
    meta[0] = total
    starts = np.cumsum([0] + counts[:-1])
    for j in range(J):   # job rows in reverse order in the output, as any order may come back
        meta[1 + 2 * j] = total - starts[j] - counts[j]
        meta[2 + 2 * j] = counts[j]
    out_k = rng.randint(0, 256, size=(total + 4) * ks).astype(np.uint8)
    out_val = rng.randn((total + 4) * 2)
    out_cnt = rng.randint(1, 5, size=total + 4).astype(np.int32)
    b.meta = torch.zeros(meta.size, dtype=torch.int64)
    return meta, out_k, out_val, out_cnt


def test_parse_views_and_coded_keys():
    specs = _specs()
    b = _host_batch(specs)
    ks = b.kstride
    meta, out_k, out_val, out_cnt = _read_back(b, [5, 0, 7, 3])
    res = b._parse(meta, out_k, out_val, out_cnt)
    rows_k = out_k.reshape(-1, ks)
    for j, (keys, vals, cnts, ctrl) in enumerate(res):
        s, c = int(meta[1 + 2 * j]), int(meta[2 + 2 * j])
        q, n = b.shapes[j][0], b.shapes[j][1]
        want_k = rows_k[s:s + c, :n].astype(np.int64)
        if b.coded[j]:
            want_k = want_k + q * rows_k[s:s + c, n:2 * n].astype(np.int64)
        assert keys.shape == (c, n) and np.array_equal(keys, want_k)
        assert np.array_equal(vals, out_val[2 * s:2 * (s + c):2] + 1j * out_val[2 * s + 1:2 * (s + c):2])
        assert np.array_equal(cnts, out_cnt[s:s + c])
        assert int(ctrl.err) == 0
    saved = [(k.copy(), v.copy(), c.copy()) for k, v, c, _ in res]
    out_k[:] = 0                                    # the next read-back into the same buffers
    out_val[:] = 0
    out_cnt[:] = 0
    for (k, v, c, _), (k0, v0, c0) in zip(res, saved):
        assert np.array_equal(k, k0) and np.array_equal(v, v0) and np.array_equal(c, c0)


def test_parse_raises_on_device_errors():
    b = _host_batch(_specs())
    J = b.njobs
    meta, out_k, out_val, out_cnt = _read_back(b, [5, 0, 7, 3])
    # job 2's ball table overflowed: its control record's err field
    raw = meta.view(np.uint8)
    at = (1 + 2 * J) * 8 + 2 * ctypes.sizeof(_lib.QsftCtrl) + _lib.QsftCtrl.err.offset
    raw[at:at + 4] = np.frombuffer(np.int32(-4).tobytes(), np.uint8)      # QSFT_ERR_OVERFLOW
    with pytest.raises(_lib.QsftError, match="job 2"):
        b._parse(meta, out_k, out_val, out_cnt)
    # a bounded device wait gave up: the status word (low 32 bits of the last word)
    meta, out_k, out_val, out_cnt = _read_back(b, [5, 0, 7, 3])
    meta[-1] = np.int64(np.uint32(np.int32(-5)))                             # QSFT_ERR_TIMEOUT
    with pytest.raises(_lib.QsftError, match="device status -5"):
        b._parse(meta, out_k, out_val, out_cnt)
