"""stc_sort_pairs_u32 (the pipeline's stable radix sort through the C ABI)
against numpy's stable sort."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort_fn(lib):
    f = lib.stc_sort_pairs_u32
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
    f.restype = ctypes.c_int
    return f


# (n, bits, keys): tile-edge sizes (4096 items a tile), partial last digits,
# and key sets whose digits all fall in one or two buckets, so that every
# tile's look-back runs through the same digit.
@pytest.mark.parametrize("n,bits,dist", [(1, 8, "uniform"), (1000, 20, "uniform"), (300_001, 19, "uniform"),
                                         (2_000_000, 32, "uniform"), (4096, 12, "uniform"),
                                         (4097, 1, "uniform"), (1_000_003, 32, "equal"),
                                         (1_000_003, 17, "two"), (3_000_000, 32, "small"),
                                         (12_000_000, 25, "uniform")])
def test_sort_pairs_matches_stable_numpy(built_cuda, n, bits, dist):
    import torch
    from stcdb_gb300._lib import load_library
    f = _sort_fn(load_library("libstc"))
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    if dist == "equal":
        keys[:] = np.uint32(0x5A5A5A5A)
    elif dist == "two":
        keys = np.where(keys & 1, np.uint32(0x1FFFF), np.uint32(0x10000)).astype(np.uint32)
    elif dist == "small":
        keys &= np.uint32(15)
    vals = np.arange(n, dtype=np.uint32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    ok = torch.empty_like(dk)
    ov = torch.empty_like(dv)
    assert f(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n, bits, 0) == 0
    mask = np.uint32((1 << bits) - 1) if bits < 32 else np.uint32(0xFFFFFFFF)
    order = np.argsort(keys & mask, kind="stable")
    assert np.array_equal(ok.cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(ov.cpu().numpy().view(np.uint32), vals[order])


def test_sort_pairs_rejects_bad_arguments(built_cuda):
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    f = _sort_fn(lib)
    assert f(None, None, None, None, 10, 8, 0) == 1
    assert f(1, 2, 3, 4, 10, 0, 0) == 1  # key_bits out of range, rejected before any device call


def test_random_access_probe_runs(built_cuda):
    """stc_measure_random_access (the table update's random-access ceiling
    used by bench.py) runs and reports a positive device time that grows
    with the number of accesses."""
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    f = lib.stc_measure_random_access
    f.argtypes = [ctypes.c_uint32, ctypes.c_ulonglong, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int
    small, large = ctypes.c_float(0.0), ctypes.c_float(0.0)
    assert f(24, 1 << 20, 0, ctypes.byref(small)) == 0
    assert f(24, 1 << 24, 0, ctypes.byref(large)) == 0
    assert 0.0 < small.value < large.value
