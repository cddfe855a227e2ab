"""The allocation-free cell-key sort (sph_sort_pairs_noalloc).

This entry point exists for callers that cannot call cudaMalloc: a host
whose device memory is held by another allocator, or a loop where an
allocation (which may synchronise the device) is not allowed.  Its scratch
is a fixed array inside the library, so the test checks, through the C ABI,
that two calls in a row give exactly the sorted output of the allocating
sph_sort_pairs (integer keys and indices: bit-exact), that the second call
is not affected by what the first left in the shared scratch, and that an
input above the fixed maximum is refused before any work is queued.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from mysph_gb300 import params as P

pytestmark = pytest.mark.gpu


def _dev(a, torch):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _sort_with_alloc(lib, torch, keys, vals, bits):
    n = len(keys)
    kd, vd = _dev(keys, torch), _dev(vals, torch)
    ko, vo = torch.empty_like(kd), torch.empty_like(vd)
    nbytes = lib.sph_sort_scratch_bytes(n, bits)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    st = lib.sph_sort_pairs(_ptr(kd), _ptr(vd), _ptr(ko), _ptr(vo), n, bits, _ptr(scratch), nbytes, None)
    torch.cuda.synchronize()
    assert st == P.SPH_OK
    return ko.cpu().numpy().view(np.uint32), vo.cpu().numpy().view(np.uint32)


def _sort_no_alloc(lib, torch, keys, vals, bits, stream=None):
    kd, vd = _dev(keys, torch), _dev(vals, torch)
    ko, vo = torch.empty_like(kd), torch.empty_like(vd)
    torch.cuda.synchronize()
    st = lib.sph_sort_pairs_noalloc(_ptr(kd), _ptr(vd), _ptr(ko), _ptr(vo), len(keys), bits, stream)
    torch.cuda.synchronize()
    assert st == P.SPH_OK
    return ko.cpu().numpy().view(np.uint32), vo.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort(gpu):
    import torch
    lib = gpu
    rng = np.random.default_rng(1234)
    # two calls in a row: a large input first, then a smaller one with other
    # key widths, so stale scratch from the first call would show up
    for n, bits in [(P.NOALLOC_MAX_PAIRS, 21), (70001, 13)]:
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.int64).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        want_k, want_v = _sort_with_alloc(lib, torch, keys, vals, bits)
        got_k, got_v = _sort_no_alloc(lib, torch, keys, vals, bits)
        assert np.array_equal(got_k, want_k)
        assert np.array_equal(got_v, want_v)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(got_v, vals[order])


def test_noalloc_sort_on_a_stream(gpu):
    import torch
    lib = gpu
    rng = np.random.default_rng(77)
    n, bits = 4097, 9
    keys = rng.integers(0, 1 << bits, size=n, dtype=np.int64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    s = torch.cuda.Stream()
    got_k, got_v = _sort_no_alloc(lib, torch, keys, vals, bits, C.c_void_p(s.cuda_stream))
    want_k, want_v = _sort_with_alloc(lib, torch, keys, vals, bits)
    assert np.array_equal(got_k, want_k) and np.array_equal(got_v, want_v)


def test_noalloc_sort_rejects_oversize(gpu):
    lib = gpu
    n = P.NOALLOC_MAX_PAIRS + 1
    # pointers are never dereferenced: the size check comes first
    dummy = C.c_void_p(16)
    st = lib.sph_sort_pairs_noalloc(dummy, dummy, dummy, dummy, n, 21, None)
    assert st == P.SPH_E_TOO_LARGE
    assert lib.sph_sort_pairs_noalloc(None, None, None, None, 10, 8, None) == P.SPH_E_INVALID
