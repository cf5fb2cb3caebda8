"""The allocation-free sort entry point against the regular one.

rt_radix_sort_pairs_noalloc serves callers that may not allocate device
memory while they run (an engine handing out all device memory from its own
pool, or a per-frame loop where cudaMalloc would synchronise the device); it
sorts out of a fixed scratch array instead.  Its result must be the same as
rt_radix_sort_pairs' on the same input -- bit for bit, this being integer
work -- on two calls in a row that reuse the shared scratch.  This file is
collected last so that a stop-at-first-failure run has run everything else.
"""
import numpy as np
import pytest

from _helpers import dptr

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 18


def _sort_both(R, torch, keys, bits):
    dt = np.int32 if keys.dtype == np.uint32 else np.int64
    vals = np.arange(len(keys), dtype=np.uint32)
    k1 = torch.from_numpy(keys.view(dt).copy()).cuda()
    v1 = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    k2 = k1.clone()
    v2 = v1.clone()
    R.check(R.lib().rt_radix_sort_pairs(dptr(k1), dptr(v1), len(keys), bits, None))
    R.check(R.lib().rt_radix_sort_pairs_noalloc(dptr(k2), dptr(v2), len(keys), bits, None))
    torch.cuda.synchronize()
    return (k1.cpu().numpy(), v1.cpu().numpy()), (k2.cpu().numpy(), v2.cpu().numpy())


def test_noalloc_sort_matches_regular_sort_twice(product, cuda):
    R, torch = product, cuda
    rng = np.random.default_rng(2024)
    # first call: 60-bit Morton-like keys at the size limit, many duplicates
    keys64 = (rng.integers(0, 1 << 12, MAX_PAIRS, dtype=np.uint64) << np.uint64(48)) | \
        rng.integers(0, 8, MAX_PAIRS, dtype=np.uint64)
    a, b = _sort_both(R, torch, keys64, 60)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    order = np.argsort(keys64, kind="stable")
    assert np.array_equal(b[0].view(np.uint64), keys64[order])
    # second call right after, reusing the scratch: 30-bit keys, odd size
    keys32 = rng.integers(0, 1 << 30, 100003, dtype=np.uint64).astype(np.uint32)
    a, b = _sort_both(R, torch, keys32, 30)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_noalloc_sort_rejects_sizes_beyond_its_scratch(product, cuda):
    R, torch = product, cuda
    k = torch.zeros(MAX_PAIRS + 1, dtype=torch.int64, device="cuda")
    v = torch.zeros(MAX_PAIRS + 1, dtype=torch.int32, device="cuda")
    st = R.lib().rt_radix_sort_pairs_noalloc(dptr(k), dptr(v), MAX_PAIRS + 1, 60, None)
    assert st == R.RT_ERR_INVALID_ARG
    assert b"262144" in R.lib().rt_last_error_string()
