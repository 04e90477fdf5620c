"""rtp_radix_sort_noalloc: the radix sort for callers that cannot allocate device memory
where they sort (a plugin whose host application owns the GPU heap, a frame loop that must
not stall on cudaMalloc, code that must not fail with out-of-memory after start-up).

It must give exactly the allocating entry point's result (integer work: bit-exact), on
two calls in a row through the C ABI, and refuse sizes beyond its fixed scratch.  This
file is collected last so that a run stopping at the first failure has run every other
test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from realtimeparticles_gb300 import _lib, abi

pytestmark = pytest.mark.gpu

MAX_KEYS = 262144  # RTP_NOALLOC_SORT_MAX_KEYS


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "CUDA device required"
    return t


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _sort_allocating(torch, kin, n, bits):
    kout = torch.empty_like(kin)
    perm = torch.empty_like(kin)
    sz = C.c_size_t()
    _lib.call("rtp_radix_sort_scratch_bytes", n, bits, C.byref(sz))
    scratch = torch.empty(max(1, sz.value), dtype=torch.uint8, device="cuda")
    _lib.call("rtp_radix_sort", _ptr(kin), n, bits, _ptr(kout), _ptr(perm), _ptr(scratch), sz.value, None)
    return kout, perm


def _sort_noalloc(torch, kin, n, bits, with_perm=True):
    kout = torch.full_like(kin, -1)
    perm = torch.full_like(kin, -1) if with_perm else None
    _lib.call("rtp_radix_sort_noalloc", _ptr(kin), n, bits, _ptr(kout), _ptr(perm) if with_perm else None, None)
    return kout, perm


def test_noalloc_sort_matches_allocating_sort_on_two_calls(torch):
    rng = np.random.default_rng(2024)
    # First call fills the whole scratch (maximum size, 32-bit keys); the second, smaller
    # one must not be affected by what the first left behind.
    for n, bits in [(MAX_KEYS, 32), (131072 - 5, 17)]:
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys[rng.integers(0, n, n // 4)] = keys[7]  # duplicates: stability matters
        kin = torch.from_numpy(keys.view(np.int32)).cuda()
        ka, pa = _sort_allocating(torch, kin, n, bits)
        kb, pb = _sort_noalloc(torch, kin, n, bits)
        torch.cuda.synchronize()
        assert torch.equal(ka, kb), "sorted keys differ from rtp_radix_sort"
        assert torch.equal(pa, pb), "permutation differs from rtp_radix_sort"
        ref = np.argsort(keys, kind="stable")
        assert np.array_equal(pb.cpu().numpy().view(np.uint32), ref)


def test_noalloc_sort_rejects_sizes_beyond_its_limit(torch):
    n = MAX_KEYS + 1
    kin = torch.zeros(n, dtype=torch.int32, device="cuda")
    kout = torch.full_like(kin, -1)
    rc = _lib.lib().rtp_radix_sort_noalloc(_ptr(kin), n, 17, _ptr(kout), None, None)
    torch.cuda.synchronize()
    assert rc == abi.ERR_CAPACITY
    assert "262144" in _lib.last_error()
    assert bool((kout == -1).all()), "nothing may run when the size is refused"


@pytest.mark.parametrize("n,bits,with_perm", [(1000, 9, True), (1000, 9, False), (3, 0, False), (5000, 17, False)])
def test_noalloc_sort_other_plans(torch, n, bits, with_perm):
    """The single-pass plan (keyBits <= 9: nothing to clear), keyBits = 0 and calls without a
    permutation output give the allocating sort's keys and a stable order."""
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    ka, pa = _sort_allocating(torch, kin, n, bits)
    kb, pb = _sort_noalloc(torch, kin, n, bits, with_perm)
    torch.cuda.synchronize()
    assert torch.equal(ka, kb)
    assert np.array_equal(kb.cpu().numpy().view(np.uint32), np.sort(keys, kind="stable"))
    if with_perm:
        assert torch.equal(pa, pb)
        assert np.array_equal(pb.cpu().numpy().view(np.uint32), np.argsort(keys, kind="stable"))
