"""GPU test of pe_broadphase_find_pairs_noalloc, the broadphase query for
callers that may not allocate device memory (an engine that hands the library a
fixed slice of its own arena, a frame loop where cudaMalloc's implicit
synchronisation breaks the time budget, a process holding nearly all of the
GPU's memory).

The test owns every device buffer (inputs, pairs, result words) and checks the
allocation-free query against pe_broadphase_find_pairs with sweep-and-prune, on
two different scenes called one after the other: the second call runs on the
scratch the first call left behind, so it also shows that nothing stale leaks
from one call into the next.  Pairs are integers: they must match exactly.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one; it passes alone or after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BOXES = 8192
MAX_PAIRS = 32768


def random_boxes(seed, n, extent, half_lo, half_hi):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-extent, extent, (n, 3)).astype(np.float32)
    h = rng.uniform(half_lo, half_hi, (n, 3)).astype(np.float32)
    return c - h, c + h


def noalloc_pairs(engine, mins, maxs, capacity, out=None):
    """Runs the allocation-free query on caller-owned torch buffers; returns
    (pairs[count, 2], count, status)."""
    import torch

    dev = torch.device("cuda:0")
    d_mins = torch.from_numpy(np.ascontiguousarray(mins, np.float32)).to(dev)
    d_maxs = torch.from_numpy(np.ascontiguousarray(maxs, np.float32)).to(dev)
    if out is None:
        out = torch.full((max(capacity, 1), 2), 0xFFFFFFF, dtype=torch.int32, device=dev)
    result = torch.full((2,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = engine.lib().pe_broadphase_find_pairs_noalloc(
        0, ctypes.c_void_p(d_mins.data_ptr()), ctypes.c_void_p(d_maxs.data_ptr()), len(mins),
        ctypes.c_void_p(out.data_ptr()), capacity, ctypes.c_void_p(result.data_ptr()),
        ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, engine.lib().pe_last_error()
    stream.synchronize()
    count, status = (int(v) for v in result.cpu().numpy().view(np.uint32))
    pairs = out.cpu().numpy().view(np.uint32)[: min(count, capacity)]
    return pairs, count, status, out


def test_noalloc_matches_find_pairs_on_two_calls_in_a_row(gpu):
    # Call 1: a dense cloud (many pairs); call 2: a smaller, sparser one run on
    # the scratch call 1 left behind, into the same output buffer.
    from oracle import cpu

    a_min, a_max = random_boxes(11, 6000, 20.0, 0.2, 1.2)
    b_min, b_max = random_boxes(12, 1500, 30.0, 0.1, 0.8)
    want_a, _ = gpu.broadphase(a_min, a_max, gpu.SAP)
    want_b, _ = gpu.broadphase(b_min, b_max, gpu.SAP)
    assert 1000 < len(want_a) <= MAX_PAIRS and 0 < len(want_b) < len(want_a)
    # The oracle's sweep (the reference's algorithm on the CPU) pins both
    # expectations independently of the device-wide GPU path.
    oracle_a, _ = cpu.broadphase("oracle", a_min, a_max, 0)
    oracle_b, _ = cpu.broadphase("oracle", b_min, b_max, 0)
    np.testing.assert_array_equal(want_a, oracle_a)
    np.testing.assert_array_equal(want_b, oracle_b)

    got_a, count_a, status_a, out = noalloc_pairs(gpu, a_min, a_max, MAX_PAIRS)
    assert (count_a, status_a) == (len(want_a), 0)
    np.testing.assert_array_equal(got_a, want_a)

    got_b, count_b, status_b, _ = noalloc_pairs(gpu, b_min, b_max, MAX_PAIRS, out=out)
    assert (count_b, status_b) == (len(want_b), 0)
    np.testing.assert_array_equal(got_b, want_b)


def test_noalloc_ties_signed_zero_and_small_capacity(gpu):
    # Shared min.x values (including -0 and +0) exercise the (min.x, index)
    # ordering; a capacity below the pair count writes the first pairs only.
    rng = np.random.default_rng(5)
    n = 700
    mins = rng.integers(-4, 4, (n, 3)).astype(np.float32)
    mins[::7, 0] = -0.0
    mins[3::7, 0] = 0.0
    maxs = mins + rng.integers(0, 3, (n, 3)).astype(np.float32)
    want, _ = gpu.broadphase(mins, maxs, gpu.SAP)
    assert len(want) > 100
    got, count, status, _ = noalloc_pairs(gpu, mins, maxs, MAX_PAIRS)
    assert (count, status) == (len(want), 0)
    np.testing.assert_array_equal(got, want)
    cap = len(want) // 3
    got, count, status, _ = noalloc_pairs(gpu, mins, maxs, cap)
    assert (count, status) == (len(want), 1)
    np.testing.assert_array_equal(got, want[:cap])


def test_noalloc_limits(gpu):
    lib = gpu.lib()
    # Empty input: zero pairs, complete.
    got, count, status, _ = noalloc_pairs(gpu, np.zeros((0, 3)), np.zeros((0, 3)), 16)
    assert (count, status, len(got)) == (0, 0, 0)
    # More boxes than the fixed scratch holds: rejected before any GPU work
    # (the buffers are real and large enough all the same).
    import torch

    big = torch.zeros((MAX_BOXES + 1, 3), dtype=torch.float32, device="cuda:0")
    words = torch.zeros(2 * 16 + 2, dtype=torch.int32, device="cuda:0")
    ptr = ctypes.c_void_p
    rc = lib.pe_broadphase_find_pairs_noalloc(0, ptr(big.data_ptr()), ptr(big.data_ptr()), MAX_BOXES + 1,
                                              ptr(words.data_ptr()), 16, ptr(words[32:].data_ptr()), None)
    assert rc == 1 and b"PE_NOALLOC_MAX_BOXES" in lib.pe_last_error()
    # More pairs than the scratch holds: status 2, count still reported.
    mins = np.zeros((300, 3), np.float32)
    maxs = np.ones((300, 3), np.float32)  # every box overlaps every other: 44,850 pairs
    got, count, status, _ = noalloc_pairs(gpu, mins, maxs, 16)
    assert (count, status) == (300 * 299 // 2, 2)


def test_noalloc_keeps_the_callers_current_device(gpu):
    # The call selects its device to enqueue the kernel and puts the caller's
    # current device back, on success and on a rejected call alike.
    import torch

    lib = gpu.lib()
    torch.cuda.set_device(0)
    before = torch.cuda.current_device()
    mins, maxs = random_boxes(21, 200, 5.0, 0.2, 0.6)
    noalloc_pairs(gpu, mins, maxs, MAX_PAIRS)
    assert torch.cuda.current_device() == before
    words = torch.zeros(4, dtype=torch.int32, device="cuda:0")
    ptr = ctypes.c_void_p
    rc = lib.pe_broadphase_find_pairs_noalloc(0, ptr(words.data_ptr()), ptr(words.data_ptr()), MAX_BOXES + 1,
                                              ptr(words.data_ptr()), 1, ptr(words.data_ptr()), None)
    assert rc != 0
    assert torch.cuda.current_device() == before
