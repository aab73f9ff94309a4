"""The sort entry point that allocates nothing (Q_cuda_radix_sort_pairs_noalloc).

It exists for callers that cannot let the library allocate device memory, such as a real-time
frame loop where cudaMalloc/cudaFree could synchronise the device mid-frame, or a host that
owns all device memory through its own pool. It uses the same kernels as
Q_cuda_radix_sort_pairs but takes its scratch from a fixed array in device memory, so its
output must equal that entry point's exactly (integer keys: no tolerance). Two calls in a
row check that the shared scratch carries nothing wrong from one call into the next. This
file is collected last so a failure here cannot hide the other tests' results.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import _abi as A

pytestmark = pytest.mark.gpu

MAX_KEYS = 1048576


def _sort(lib, fn_name: str, keys: np.ndarray, vals: np.ndarray, bits: int):
    import torch

    kt = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    vt = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    stream = torch.cuda.current_stream()
    rc = getattr(lib, fn_name)(C.c_void_p(kt.data_ptr()), C.c_void_p(vt.data_ptr()), keys.size, bits,
                               C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    assert rc == A.QUASI_OK, (fn_name, rc)
    return kt.cpu().numpy().view(np.uint32), vt.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_on_two_calls_in_a_row(cuda_ok):
    lib = q.load_library()
    rng = np.random.default_rng(2024)
    # Call 1 fills the whole scratch (32 bits: 4 passes of 8 bits, so the result ends in the
    # caller's buffer). Calls 2 and 3 are smaller and take an odd number of passes (24 bits:
    # 3, 8 bits: 1), so their result ends in the static scratch and is copied back to the
    # caller's buffer; anything read back from an earlier call's leftovers would show up as
    # a mismatch.
    cases = [(MAX_KEYS, 32), (300_001, 24), (5_003, 8)]
    for n, bits in cases:
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 4] = keys[7]  # duplicates: the sort must stay stable
        vals = rng.permutation(n).astype(np.uint32)
        ref_k, ref_v = _sort(lib, "Q_cuda_radix_sort_pairs", keys, vals, bits)
        got_k, got_v = _sort(lib, "Q_cuda_radix_sort_pairs_noalloc", keys, vals, bits)
        assert np.array_equal(got_k, ref_k)
        assert np.array_equal(got_v, ref_v)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(got_v, vals[order])


def test_noalloc_sort_rejects_inputs_above_its_capacity(cuda_ok):
    import torch

    lib = q.load_library()
    k = torch.zeros(MAX_KEYS + 1, dtype=torch.int32, device="cuda")
    v = torch.arange(MAX_KEYS + 1, dtype=torch.int32, device="cuda")
    rc = lib.Q_cuda_radix_sort_pairs_noalloc(C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()), MAX_KEYS + 1, 32,
                                             None)
    assert rc == -7  # QUASI_ERR_TOO_LARGE
    torch.cuda.synchronize()
    assert torch.equal(v.cpu(), torch.arange(MAX_KEYS + 1, dtype=torch.int32))  # untouched
