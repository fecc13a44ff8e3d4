"""Near lists against the full cell walk (PBD_FLAG_FULL_WALK).

A walking pass (lambda, omega) records the entries within the cut for the pass after it at the
same positions (delta, viscosity); the entries left out add exact zeros there, so a step with
near lists must be bit-identical to a step that walks the cells in every pass, over many frames,
for every pass mix (density solve, contacts, vorticity, viscosity, solids, batches, the
cell-end quirk's long ranges, fast motion)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(pbd, params, pos, vel, frames, inv_mass=None, full_walk=False):
    p = params.copy()
    if full_walk:
        p.flags |= pbd.FLAG_FULL_WALK
    sim = pbd.Sim(p, len(pos))
    if inv_mass is None:
        sim.add_particles(pos, vel)
    else:
        sim.add_particles_mass(pos, vel, inv_mass)
    sim.step(frames)
    sim.sync()
    st = sim.state()
    sim.close()
    return st


def _same(a, b):
    for k in ("x", "v", "p", "ids"):
        assert np.array_equal(a[k], b[k]), k


CASES = [
    # shape, box, vorticity, viscosity, quirk, velocity sigma
    ((20, 20, 20), 32, 0.0, 0.0, True, 0.0),
    ((20, 20, 20), 32, 0.0005, 0.01, True, 0.0),
    ((16, 24, 16), 32, 0.0, 0.01, False, 0.0),
    ((13, 7, 11), 24, 0.0, 0.0, True, 3.0),
]


@pytest.mark.parametrize("shape,box,vort,visc,quirk,sigma", CASES)
def test_lists_bit_identical_to_full_walk(need_gpu, pbd, scenes, shape, box, vort, visc, quirk, sigma):
    params = scenes.workload_params(pbd, box, 1000.0, vorticity=vort, viscosity=visc)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    if not quirk:
        params.flags &= ~pbd.FLAG_CELL_END_QUIRK
    pos, vel = scenes.lattice(*shape, seed=3)
    if sigma:
        vel[:, :3] = np.random.default_rng(3).normal(0, sigma, size=(len(vel), 3)).astype(np.float32)
    a = _run(pbd, params, pos, vel, 40)
    b = _run(pbd, params, pos, vel, 40, full_walk=True)
    _same(a, b)


def test_lists_fast_motion(need_gpu, pbd, scenes):
    # fast random motion: particles move up to a few cells per frame
    params = scenes.workload_params(pbd, 24, 1000.0)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(12, 12, 12, spacing=0.8, seed=4)
    vel[:, :3] = np.random.default_rng(4).normal(0, 40, size=(len(vel), 3)).astype(np.float32)
    a = _run(pbd, params, pos, vel, 12)
    b = _run(pbd, params, pos, vel, 12, full_walk=True)
    _same(a, b)


def test_lists_with_solids(need_gpu, pbd, scenes):
    pos, vel, w = scenes.solids_scene(fluid_shape=(16, 16, 16), n_boxes=2, box_shape=(6, 6, 8), box=48, seed=5)
    params = scenes.workload_params(pbd, 48, 1000.0)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    a = _run(pbd, params, pos, vel, 30, inv_mass=w)
    b = _run(pbd, params, pos, vel, 30, inv_mass=w, full_walk=True)
    _same(a, b)


def test_lists_in_batches(need_gpu, pbd, scenes):
    sl = scenes.batched_scenes(nscenes=4, n_range=(500, 3000), box_range=(20, 32), seed=9)
    shared = scenes.workload_params(pbd, 32, 1000.0)
    shared.lambda_epsilon = 0.1
    out = []
    for fw in (False, True):
        p = shared.copy()
        if fw:
            p.flags |= pbd.FLAG_FULL_WALK
        descs = [pbd.scene_desc(sc["n"], sc["rest_density"], sc["gravity"], sc["box"]) for sc in sl]
        b = pbd.Batch(p, descs)
        for k, sc in enumerate(sl):
            b.add_particles(k, sc["pos"], sc["vel"])
        b.step(25)
        b.sync()
        out.append([b.state(k) for k in range(len(sl))])
        b.close()
    for s1, s2 in zip(*out):
        assert np.array_equal(s1["x"], s2["x"]) and np.array_equal(s1["v"], s2["v"])


@pytest.mark.parametrize("vort,visc", [(0.0, 0.0), (0.0005, 0.01), (0.0, 0.01)])
def test_lists_dense_blob_without_lists(need_gpu, pbd, scenes, vort, visc):
    """a blob at spacing 0.35 inside a lattice at spacing 1: the blob's particles have more than
    128 entries (no full list) and up to ~100 within the cut (no near list), so every pass hands
    them to its cooperative blocks through the noted sets; the rest walk stored lists"""
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=vort, viscosity=visc)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    params.flags &= ~pbd.FLAG_CELL_END_QUIRK
    pos, vel = scenes.lattice(16, 12, 16, spacing=1.0, seed=6)
    lo, sp = np.array([8.0, 6.0, 8.0]), 0.35
    blob, bv = scenes.lattice(9, 9, 9, origin=tuple(lo), spacing=sp, jitter=0.02, seed=7)
    inside = np.all((pos[:, :3] > lo - 0.5) & (pos[:, :3] < lo + 8 * sp + 0.5), axis=1)
    pos = np.concatenate([pos[~inside], blob]); vel = np.concatenate([vel[~inside], bv])
    a = _run(pbd, params, pos, vel, 8)
    b = _run(pbd, params, pos, vel, 8, full_walk=True)
    _same(a, b)


@pytest.mark.parametrize("cap", [20, 40])
def test_lists_with_a_small_cap(need_gpu, pbd, scenes, cap):
    """maxNeighboursPerParticle below the ~32 candidates of the 27 cells: every stored list is
    cut at the cap in the cells' order, as the walk cuts it"""
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=0.0005, viscosity=0.01, max_neighbours=cap)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(20, 16, 20, spacing=0.9, seed=8)
    a = _run(pbd, params, pos, vel, 12)
    b = _run(pbd, params, pos, vel, 12, full_walk=True)
    _same(a, b)


def test_block_size_leaves_results_unchanged(need_gpu, pbd, scenes, tmp_path):
    """pbd_autotune picks the neighbour passes' block size; every size gives the same bits (the
    particles without a list are walked by whichever blocks, each on its own)"""
    import json
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=0.0005, viscosity=0.01)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(20, 16, 20, spacing=0.9, seed=12)
    probe = tmp_path / "probe.jsonl"
    sim = pbd.Sim(params, len(pos))
    sim.add_particles(pos, vel)
    assert sim.autotune(str(probe)) in (64, 128, 256)
    sim.close()
    sig = json.loads(probe.read_text().splitlines()[0])["signature"]
    states = []
    for block in (64, 128, 256):
        cache = tmp_path / f"b{block}.jsonl"
        cache.write_text(json.dumps({"signature": sig, "block": block}) + "\n")
        sim = pbd.Sim(params, len(pos))
        sim.add_particles(pos, vel)
        assert sim.autotune(str(cache)) == block          # served from the cache: no frames run
        sim.step(10)
        sim.sync()
        states.append(sim.state())
        sim.close()
    for st in states[1:]:
        _same(states[0], st)


@pytest.mark.parametrize("vort,visc", [(0.0, 0.0), (0.0005, 0.01), (0.0005, 0.0), (0.0, 0.01)])
def test_step_readback_matches_step_and_get_state(need_gpu, pbd, scenes, vort, visc):
    """pbd_step_readback (positions, and velocities that viscosity leaves alone, copied beside the
    last passes; velocities that viscosity changes stored into host memory by that pass) returns
    the state pbd_step + pbd_get_state return, and the simulation continues from it identically"""
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=vort, viscosity=visc)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(20, 16, 20, spacing=0.9, seed=13)
    a = pbd.Sim(params, len(pos)); a.add_particles(pos, vel)
    b = pbd.Sim(params, len(pos)); b.add_particles(pos, vel)
    for n in (1, 3, 1):
        xa, va = a.step_readback(n)
        b.step(n)
        sb = b.state()
        assert np.array_equal(xa, sb["x"]) and np.array_equal(va, sb["v"])
    _same(a.state(), b.state())
    a.close(); b.close()


def test_readback_arrays_fed_back_in(need_gpu, pbd, scenes):
    """A host loop that feeds pbd_step_readback's own arrays back through pbd_clear +
    pbd_add_particles (the copy is queued, not waited for) gives, frame by frame, the bits of a
    loop that restarts from host copies of the same state with the synchronous path"""
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=0.0005, viscosity=0.01)
    params.lambda_epsilon = 0.1
    pos, vel = scenes.lattice(20, 16, 20, spacing=0.9, seed=13)
    n = len(pos)
    a = pbd.Sim(params, n); a.add_particles(pos, vel)
    b = pbd.Sim(params, n); b.add_particles(pos, vel)
    L = pbd.lib()
    rx, rv = pbd.C.POINTER(pbd.C.c_float)(), pbd.C.POINTER(pbd.C.c_float)()
    pbd.check(L.pbd_step_readback(a.h, 1, None, pbd.C.byref(rx), pbd.C.byref(rv)))
    b.step(1)
    for _ in range(4):
        pbd.check(L.pbd_clear(a.h))
        pbd.check(L.pbd_add_particles(a.h, n, rx, rv, None))
        pbd.check(L.pbd_step_readback(a.h, 1, None, pbd.C.byref(rx), pbd.C.byref(rv)))
        sb = b.state()
        b.clear()
        b.add_particles(sb["x"], sb["v"])
        b.step(1)
        sb = b.state()
        xa = np.ctypeslib.as_array(rx, shape=(n, 4))
        va = np.ctypeslib.as_array(rv, shape=(n, 4))
        assert np.array_equal(xa, sb["x"]) and np.array_equal(va, sb["v"])
    a.close(); b.close()
