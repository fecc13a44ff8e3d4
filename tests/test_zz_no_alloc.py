"""The allocation-free sort entry point (pbd_sort_keys_noalloc) against the step's own sort.

Hosts that own all device memory, or frame loops that must not stall on cudaMalloc, sort with
pbd_sort_keys_noalloc, whose working memory is a fixed array inside the library.  Its output
must be the same as the sort the step runs with the memory it allocated at pbd_create
(pbd_debug_front + pbd_debug_dump): integer keys and indices, so bit for bit.  Two calls in a
row with different inputs check that the shared fixed array is cleared between calls.
This file is collected last on purpose: it keeps a fixed array on the GPU for the rest of the
process."""
import ctypes as C

import numpy as np
import pytest

from helpers import workload

pytestmark = pytest.mark.gpu


def _step_sort(pbd, scenes, shape, seed):
    """Keys before the sort, sorted keys and permutation from the step's own sort."""
    params, pos, vel = workload(pbd, scenes, shape=shape, box=max(shape) + 8, seed=seed)
    rng = np.random.default_rng(seed)
    vel[:, :3] = rng.normal(0, 20, size=(len(vel), 3)).astype(np.float32)
    with pbd.Sim(params, len(pos)) as sim:
        sim.add_particles(pos, vel)
        sim.front()
        d = sim.debug()
    keys_sorted, perm = d["keys"], d["perm"]
    keys_in = np.empty_like(keys_sorted)
    keys_in[perm] = keys_sorted
    return keys_in, keys_sorted, perm


def _sort_noalloc(pbd, keys_in, key_bits=24):
    import torch
    d_in = torch.tensor(keys_in.view(np.int32), device="cuda")
    d_keys = torch.full_like(d_in, -1)
    d_perm = torch.full_like(d_in, -1)
    stream = torch.cuda.current_stream()
    rc = pbd.lib().pbd_sort_keys_noalloc(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_keys.data_ptr()),
                                         C.c_void_p(d_perm.data_ptr()), len(keys_in), key_bits,
                                         C.c_void_p(stream.cuda_stream))
    pbd.check(rc)
    stream.synchronize()
    return d_keys.cpu().numpy().view(np.uint32), d_perm.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_the_step_sort_twice(need_gpu, pbd, scenes):
    for shape, seed in (((40, 40, 40), 31), ((70, 33, 50), 32)):
        keys_in, keys_sorted, perm = _step_sort(pbd, scenes, shape, seed)
        k, p = _sort_noalloc(pbd, keys_in)
        assert np.array_equal(k, keys_sorted)
        assert np.array_equal(p, perm)


@pytest.mark.parametrize("key_bits", [1, 8, 16, 20, 24, 32])
@pytest.mark.parametrize("n", [1, 100, 4097, 65537, 1 << 20])
def test_noalloc_sort_orders_by_the_low_key_bits(need_gpu, pbd, key_bits, n):
    # every pass count (1 to 4, so both ends of the ping-pong through the fixed array), partial
    # last tiles, one key, the 1,048,576-key limit; keys carry bits above key_bits, which must
    # not take part in the order (a stable sort by the low bits)
    rng = np.random.default_rng(key_bits * 1000003 + n)
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    keys[::2] &= np.uint32(0xFFFF003F)   # plenty of equal low bits, so stability is exercised
    mask = np.uint32(0xFFFFFFFF if key_bits == 32 else (1 << key_bits) - 1)
    order = np.argsort(keys & mask, kind="stable")
    k, p = _sort_noalloc(pbd, keys, key_bits=key_bits)
    assert np.array_equal(p, order.astype(np.uint32))
    assert np.array_equal(k, keys[order])
    assert pbd.lib().pbd_sort_noalloc_status(None) == pbd.OK


def test_noalloc_sort_reports_a_wait_that_ran_out(need_gpu, pbd):
    # a short wait limit and a first tile that never publishes its counts: every look-back wait
    # on it gives up (no hang, no trap), the status says so, and the next call is clean again
    L = pbd.lib()
    keys = np.random.default_rng(7).integers(0, 1 << 24, size=50000, dtype=np.uint64).astype(np.uint32)
    try:
        pbd.check(L.pbd_debug_set_wait_limit(None, 2000, 1))
        _sort_noalloc(pbd, keys)
        assert L.pbd_sort_noalloc_status(None) == pbd.ERR_TIMEOUT
        assert b"gave up" in L.pbd_last_error()
    finally:
        pbd.check(L.pbd_debug_set_wait_limit(None, 0, 0))
    k, p = _sort_noalloc(pbd, keys)
    assert L.pbd_sort_noalloc_status(None) == pbd.OK
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(p, order.astype(np.uint32)) and np.array_equal(k, keys[order])


def test_noalloc_sort_rejects_more_keys_than_its_fixed_memory(need_gpu, pbd):
    import torch
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    ptr = C.c_void_p(buf.data_ptr())
    rc = pbd.lib().pbd_sort_keys_noalloc(ptr, ptr, ptr, (1 << 20) + 1, 24, None)
    assert rc == pbd.ERR_CAPACITY
    assert b"at most 1048576" in pbd.lib().pbd_last_error()
