"""Bit-exact parity of the grid/sort operators (fillCellIDs, RadixSort::sort, the
start/end cell table) with the oracle, through the C ABI on caller-owned device memory."""
import ctypes as C

import numpy as np
import pytest

from realtimeparticles_gb300 import _lib, abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "CUDA device required"
    return t


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _sort_gpu(torch, keys, bits):
    n = keys.shape[0]
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    kout = torch.empty_like(kin)
    perm = torch.empty_like(kin)
    sz = C.c_size_t()
    _lib.call("rtp_radix_sort_scratch_bytes", n, bits, C.byref(sz))
    scratch = torch.empty(max(1, sz.value), dtype=torch.uint8, device="cuda")
    _lib.call("rtp_radix_sort", _ptr(kin), n, bits, _ptr(kout), _ptr(perm), _ptr(scratch), sz.value, None)
    torch.cuda.synchronize()
    return kout.cpu().numpy().view(np.uint32), perm.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [1, 2, 33, 2047, 2048, 2049, 65537, 131072, 1000003])
@pytest.mark.parametrize("bits", [1, 9, 17, 32])
def test_radix_sort_is_a_stable_sort(torch, n, bits):
    rng = np.random.default_rng(n * 131 + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    if n > 100:
        keys[rng.integers(0, n, n // 3)] = keys[0]  # many duplicates: stability matters
    sk, perm = _sort_gpu(torch, keys, bits)
    ref = np.argsort(keys, kind="stable")
    assert np.array_equal(perm, ref)
    assert np.array_equal(sk, keys[ref])


@pytest.mark.parametrize("n,bits", [(262145, 25), (4194403, 24), (20000003, 25)])
def test_radix_sort_large_tile_counts(torch, n, bits):
    """Tile counts that take the grouped digit scan (above 128 tiles), up to more tiles than
    the 64 groups x 128 tiles the groups start from (20M keys = 9766 tiles)."""
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
    keys[rng.integers(0, n, n // 4)] = keys[1]
    sk, perm = _sort_gpu(torch, keys, bits)
    ref = np.argsort(keys, kind="stable")
    assert np.array_equal(perm, ref)
    assert np.array_equal(sk, keys[ref])


def test_radix_sort_nearly_sorted_cell_keys(torch, oracle_mod):
    # The step's real input: keys of the previous order, slightly perturbed.
    rng = np.random.default_rng(7)
    keys = np.sort(rng.integers(0, 65641, 131072)).astype(np.uint32)
    keys[rng.integers(0, 131072, 2000)] += 1
    sk, perm = _sort_gpu(torch, keys, 17)
    osk, operm = oracle_mod.stable_sort(keys)
    assert np.array_equal(perm, operm) and np.array_equal(sk, osk)


def test_radix_sort_empty(torch):
    _lib.call("rtp_radix_sort", None, 0, 17, None, None, None, 0, None)


def _consts(box=1.0, res=40, mtype=abi.FLUIDS):
    from realtimeparticles_gb300 import model
    return model.get_constants(mtype, abi.model_params(16, 16, (box,) * 3, (res,) * 3))


def test_fill_cell_ids_bit_exact(torch, oracle_mod):
    c = _consts()
    rng = np.random.default_rng(11)
    n = 200000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-0.6, 0.6, (n, 3))
    # Exact cell boundaries and their float neighbours, walls, infinities.
    edges = (np.arange(41, dtype=np.float32) * np.float32(c.cellSize) - np.float32(0.5)).astype(np.float32)
    cand = np.concatenate([edges, np.nextafter(edges, np.float32(-1)), np.nextafter(edges, np.float32(1)),
                           np.array([0.5, -0.5, np.inf, -np.inf, 0.0, -0.0], np.float32)])
    m = len(cand)
    pos[:m ** 1, 0] = cand
    pos[:m, 1] = cand[::-1]
    pos[m:2 * m, 2] = cand
    pos[2 * m:3 * m, :3] = cand[:, None]
    d = torch.from_numpy(pos).cuda()
    keys = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.call("rtp_fill_cell_ids", C.byref(c), _ptr(d), n, _ptr(keys), None)
    torch.cuda.synchronize()
    got = keys.cpu().numpy().view(np.uint32)
    ref = oracle_mod.fill_cell_ids(c, pos)
    assert np.array_equal(got, ref)
    assert got.max() == c.keyBound - 1


@pytest.mark.parametrize("case", ["random", "quirk_first_cell", "capped", "aliased", "single", "runs"])
def test_cell_table_bit_exact(torch, oracle_mod, case):
    c = _consts(res=8)  # 512 cells, cap 100
    rng = np.random.default_rng(5)
    if case == "random":
        sk = np.sort(rng.integers(0, c.keyBound, 5000)).astype(np.uint32)
    elif case == "quirk_first_cell":
        sk = np.array([3, 3, 3, 4, 9, 9], np.uint32)
    elif case == "capped":
        sk = np.sort(np.concatenate([np.full(350, 17), np.full(101, 40), np.full(102, 41), [0]])).astype(np.uint32)
    elif case == "aliased":
        sk = np.sort(rng.integers(500, c.keyBound, 300)).astype(np.uint32)
    elif case == "runs":  # runs around the table kernel's 32-particle look-ahead, first and last
        sk = np.concatenate([np.full(33, 5), np.full(32, 6), np.full(34, 7), [8], np.full(40, 9)]).astype(np.uint32)
    else:
        sk = np.array([77], np.uint32)
    d = torch.from_numpy(sk.view(np.int32)).cuda()
    t = torch.empty((c.numCells, 2), dtype=torch.int32, device="cuda")
    _lib.call("rtp_build_cell_table", C.byref(c), _ptr(d), len(sk), _ptr(t), None)
    torch.cuda.synchronize()
    got = t.cpu().numpy().view(np.uint32)
    ref = oracle_mod.cell_table(c, sk)
    assert np.array_equal(got, ref)


def _pass_offsets(keys, shift, bits, tile=2048, bins=512):
    """Per-tile exclusive prefix of each digit over the tiles before it, and digit totals."""
    n = keys.shape[0]
    tiles = (n + tile - 1) // tile
    d = (keys >> np.uint32(shift)) & np.uint32((1 << bits) - 1)
    counts = np.zeros((tiles, bins), np.uint32)
    for t in range(tiles):
        counts[t, :] = np.bincount(d[t * tile:(t + 1) * tile], minlength=bins)[:bins]
    prefix = np.zeros_like(counts)
    prefix[1:] = np.cumsum(counts, axis=0)[:-1]
    return prefix, counts.sum(axis=0).astype(np.uint32)


def _run_pass(torch, keys, shift, bits, prefix, totals):
    n = keys.shape[0]
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    kout = torch.full_like(kin, -1)
    perm = torch.full_like(kin, -1)
    hp = torch.from_numpy(prefix.view(np.int32).ravel().copy()).cuda()
    ht = torch.from_numpy(totals.view(np.int32).copy()).cuda()
    fault = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("rtp_radix_sort_pass", _ptr(kin), n, shift, bits, _ptr(hp), _ptr(ht), _ptr(kout), _ptr(perm),
              _ptr(fault), None)
    torch.cuda.synchronize()
    return kout.cpu().numpy().view(np.uint32), perm.cpu().numpy().view(np.uint32), int(fault.item())


def test_sort_pass_with_consistent_offsets(torch):
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1 << 20, 5000, dtype=np.uint64).astype(np.uint32)
    prefix, totals = _pass_offsets(keys, 4, 9)
    kout, perm, fault = _run_pass(torch, keys, 4, 9, prefix, totals)
    ref = np.argsort((keys >> 4) & 511, kind="stable")
    assert fault == 0
    assert np.array_equal(perm, ref)
    assert np.array_equal(kout, keys[ref])


def test_sort_pass_flags_inconsistent_offsets(torch):
    """Digit offsets that do not match the keys (a histogram built wrongly) would place elements
    past the end: the pass writes none of them and raises the fault word instead of writing out
    of bounds or dropping them silently (a model step reports the same word as RTP_ERR_CUDA)."""
    rng = np.random.default_rng(6)
    n = 5000
    keys = rng.integers(0, 512, n, dtype=np.uint64).astype(np.uint32)
    keys[-1] = 511  # the largest digit occurs in the last tile: its run ends the output
    prefix, totals = _pass_offsets(keys, 0, 9)
    bad = prefix.copy()
    bad[-1, 511] += 1000  # the last tile's run of digit 511 now starts beyond n
    kout, perm, fault = _run_pass(torch, keys, 0, 9, bad, totals)
    assert fault == 1
    in_last = int(np.count_nonzero(keys[2 * 2048:] == 511))
    # exactly those elements were not written (their output slots keep the fill value); every
    # other element is where the consistent pass puts it
    unwritten = perm == 0xFFFFFFFF
    assert int(np.count_nonzero(unwritten)) == in_last
    ref = np.argsort(keys, kind="stable")
    assert np.array_equal(perm[~unwritten], ref[~unwritten])
