"""stc_sort_pairs_u32_noalloc (fixed library-owned scratch, no device
allocation) against stc_sort_pairs_u32 (allocating) and numpy's stable sort
on the same inputs: two calls in a row with different inputs, so the second
runs on scratch the first left behind. Kept in a file collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20  # STC_SORT_NOALLOC_MAX_PAIRS in include/stc.h
STC_ERR_CAPACITY = 3


def _fn(lib, name):
    lib.stc_last_error.restype = ctypes.c_char_p
    lib.stc_last_error.argtypes = [ctypes.c_void_p]
    f = getattr(lib, name)
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
    f.restype = ctypes.c_int
    return f


def _sort(f, keys, vals, bits):
    import torch
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    ok = torch.empty_like(dk)
    ov = torch.empty_like(dv)
    st = f(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), len(keys), bits, 0)
    return st, ok.cpu().numpy().view(np.uint32), ov.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_twice(built_cuda):
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    ref = _fn(lib, "stc_sort_pairs_u32")
    na = _fn(lib, "stc_sort_pairs_u32_noalloc")
    # a full-size call followed by a smaller one with fewer key bits
    for seed, n, bits in [(5, MAX_PAIRS, 32), (6, 123_457, 21)]:
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        vals = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        st_r, k_r, v_r = _sort(ref, keys, vals, bits)
        st_n, k_n, v_n = _sort(na, keys, vals, bits)
        assert st_r == 0 and st_n == 0, lib.stc_last_error(None)
        # integer sort: bit-exact, against the allocating sort and against
        # numpy's stable sort on the masked keys
        assert np.array_equal(k_n, k_r)
        assert np.array_equal(v_n, v_r)
        mask = np.uint32((1 << bits) - 1) if bits < 32 else np.uint32(0xFFFFFFFF)
        order = np.argsort(keys & mask, kind="stable")
        assert np.array_equal(k_n, keys[order])
        assert np.array_equal(v_n, vals[order])


def test_noalloc_sort_rejects_more_than_its_scratch_holds(built_cuda):
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    na = _fn(lib, "stc_sort_pairs_u32_noalloc")
    # rejected on the host before any device access, so the pointers are never used
    assert na(1, 2, 3, 4, MAX_PAIRS + 1, 32, 0) == STC_ERR_CAPACITY
    assert b"exceeds" in lib.stc_last_error(None)
