"""Failure paths, injected on the host (no GPU fault, trap or hang):
 - a radix-sort look-back wait that runs out (a first tile that never publishes, a short wait
   limit) sets the device error word; pbd_sync reports PBD_ERR_TIMEOUT and the next frames are
   clean again;
 - device and pinned-host allocations that fail as on a GPU out of memory: pbd_create, the
   collisionType 1 workspace and pbd_step_readback's buffers return PBD_ERR_ALLOC and leave no
   memory behind."""
import numpy as np
import pytest

from helpers import workload

pytestmark = pytest.mark.gpu


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_sort_wait_that_runs_out_is_reported_by_sync(need_gpu, pbd, scenes):
    params, pos, vel = workload(pbd, scenes, shape=(30, 30, 30), box=40, seed=4)
    L = pbd.lib()
    with pbd.Sim(params, len(pos)) as sim:
        sim.add_particles(pos, vel)
        pbd.check(L.pbd_debug_set_wait_limit(sim.h, 2000, 1))
        sim.front()                                  # predict, sort (7 tiles a pass), re-order
        assert L.pbd_sync(sim.h) == pbd.ERR_TIMEOUT
        assert b"gave up" in L.pbd_last_error()
        pbd.check(L.pbd_debug_set_wait_limit(sim.h, 0, 0))
        sim.clear()
        sim.add_particles(pos, vel)
        sim.step(2)
        assert L.pbd_sync(sim.h) == pbd.OK
        got = sim.state()
    with pbd.Sim(params, len(pos)) as ref:
        ref.add_particles(pos, vel)
        ref.step(2)
        want = ref.state()
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["v"], want["v"])


def test_failed_create_returns_alloc_and_leaks_nothing(need_gpu, pbd, scenes):
    import ctypes as C
    L = pbd.lib()
    params, pos, vel = workload(pbd, scenes, shape=(8, 8, 8), box=128)
    cap = 2_000_000                                   # a ~3 GB arena: a leak would show
    before = _free_bytes()
    h = C.c_void_p()
    try:
        pbd.check(L.pbd_debug_fail_allocations(0, 1))
        assert L.pbd_create(C.byref(params), cap, C.byref(h)) == pbd.ERR_ALLOC and not h.value
        p1 = params.copy()
        p1.collision_type = 1                         # the arena succeeds, the contact workspace fails
        pbd.check(L.pbd_debug_fail_allocations(1, 1))
        assert L.pbd_create(C.byref(p1), cap, C.byref(h)) == pbd.ERR_ALLOC and not h.value
    finally:
        pbd.check(L.pbd_debug_fail_allocations(0, 0))
    assert abs(_free_bytes() - before) < 64 * 2 ** 20
    with pbd.Sim(params, cap) as sim:                 # allocations work again
        sim.add_particles(pos, vel)
        sim.step(1)
        sim.sync()


def test_failed_readback_buffers_return_alloc(need_gpu, pbd, scenes):
    params, pos, vel = workload(pbd, scenes, shape=(8, 8, 8), box=16)
    L = pbd.lib()
    with pbd.Sim(params, len(pos)) as sim:
        sim.add_particles(pos, vel)
        try:
            pbd.check(L.pbd_debug_fail_allocations(0, 1))
            with pytest.raises(pbd.PBDError) as e:
                sim.step_readback(1)
            assert e.value.code == pbd.ERR_ALLOC
        finally:
            pbd.check(L.pbd_debug_fail_allocations(0, 0))
        x, v = sim.step_readback(1)
        assert x.shape == (len(pos), 4) and np.all(np.isfinite(x))
