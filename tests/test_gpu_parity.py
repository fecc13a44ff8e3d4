"""GPU parity: the CUDA step through the C ABI against the CPU oracle on the same seeded inputs.

Bit-exact: predicted positions, Morton keys, sort permutation, re-ordered state, cell ranges
and the neighbour lists of the front of a frame (applyForces .. findNeighbours).
Tolerance (FP32 arithmetic, different summation/rounding of sqrt, rsqrt, division): positions
and velocities after 1 and 10 frames, against the FP32 transliteration and the FP64 oracle."""
import numpy as np
import pytest

from helpers import by_id, maxdiff, morton_np, setup_pair, workload

pytestmark = pytest.mark.gpu

# tolerances (absolute, world units = cell widths; velocities in cells/s)
TOL_X1 = 2e-5      # positions after one frame
TOL_V1 = 2e-3      # velocities after one frame (= position difference / dt)
TOL_X10 = 2e-3     # positions after ten frames
TOL_V10 = 2e-1


def _front_compare(pbd, oracle_mod, params, pos, vel, ncells=1 << 15):
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
    sim.front()
    orc.step_phase(oracle_mod.PHASE_FRONT)
    g, o = sim.debug(ncells), orc.debug(ncells)
    gs, os_ = sim.state(), orc.state()
    return sim, orc, g, o, gs, os_


SCENES = [((8, 8, 8), 16, 1), ((13, 7, 11), 24, 2), ((20, 20, 20), 32, 3)]


@pytest.mark.parametrize("shape,box,seed", SCENES)
def test_front_bit_exact(need_gpu, pbd, scenes, oracle_mod, shape, box, seed):
    params, pos, vel = workload(pbd, scenes, shape=shape, box=box, seed=seed, flags_extra=pbd.FLAG_TRACK_IDS)
    # non-zero initial velocities exercise the FMA chain of applyForces and the walls
    rng = np.random.default_rng(seed)
    vel[:, :3] = rng.normal(0, 20, size=(len(vel), 3)).astype(np.float32)
    sim, orc, g, o, gs, os_ = _front_compare(pbd, oracle_mod, params, pos, vel, ncells=box ** 3 * 2)
    assert np.array_equal(g["keys"], o["keys"])
    assert np.array_equal(g["perm"], o["perm"])
    assert np.array_equal(gs["ids"], os_["ids"])
    # state after the gather: bit-exact
    assert np.array_equal(gs["p"], os_["p"].astype(np.float32))
    assert np.array_equal(gs["v"], os_["v"].astype(np.float32))
    assert np.array_equal(gs["x"], os_["x"].astype(np.float32))
    occ = np.unique(g["keys"])
    assert np.array_equal(g["cell_start"][occ], o["cell_start"][occ])
    n = len(g["keys"])
    ends_ok = occ[occ != n - 1]
    assert np.array_equal(g["cell_end"][ends_ok], o["cell_end"][ends_ok])
    empty = np.setdiff1d(np.arange(len(g["cell_start"])), occ)
    assert np.all(g["cell_start"][empty] == 0xFFFFFFFF)
    assert np.array_equal(morton_np(gs["p"]), g["keys"])


@pytest.mark.parametrize("shape,box,seed", SCENES[:2])
def test_neighbour_lists_bit_exact(need_gpu, pbd, scenes, oracle_mod, shape, box, seed):
    params, pos, vel = workload(pbd, scenes, shape=shape, box=box, seed=seed)
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
    sim.front()
    orc.step_phase(oracle_mod.PHASE_LISTS)
    gl, gc, gk = sim.neighbours(64)
    ol, oc, ok = orc.neighbours(64)
    assert np.array_equal(gc, oc) and np.array_equal(gk, ok)
    for i in range(len(gc)):
        assert np.array_equal(gl[i, :gc[i]], ol[i, :oc[i]])


def test_neighbour_lists_shells_and_cap(need_gpu, pbd, scenes, oracle_mod):
    """kernelWidthNeighbours = 2 (findNeighbours shells, Collision.h:126-155) and a cap M
    small enough to truncate (Collision.h:61-63,144-146)."""
    params, pos, vel = workload(pbd, scenes, shape=(10, 10, 10), box=16, seed=9)
    params.kernel_width_neighbours = 2
    for cap in (512, 40, 20):
        params.max_neighbours_per_particle = cap
        sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
        sim.front()
        orc.step_phase(oracle_mod.PHASE_LISTS)
        ol, oc, ok = orc.neighbours(cap)
        for walker in (0, 1):
            gl, gc, gk = sim.neighbours(cap, walker=walker)
            assert np.array_equal(gc, oc) and np.array_equal(gk, ok)
            assert np.array_equal(gl, ol)


@pytest.mark.parametrize("cap", [512, 100, 30])
def test_cell_end_quirk_long_range(need_gpu, pbd, scenes, oracle_mod, cap):
    """8^3 lattice at cells 2..9: cell N-1 = 511 = (7,7,7) is occupied and not the last cell, so
    SortReorder.h:183-184 stretches its range to N (~300 entries).  Those particles take the
    warp-per-particle walker; lists, lambda and positions must match the oracle, with the cap
    M falling inside the stretched range for the smaller caps."""
    params, pos, vel = workload(pbd, scenes, shape=(8, 8, 8), box=16, seed=21, vorticity=0.0005, viscosity=0.01)
    params.max_neighbours_per_particle = cap
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
    sim.front()
    orc.step_phase(oracle_mod.PHASE_LISTS)
    ol, oc, ok = orc.neighbours(cap)
    assert oc.max() == min(cap, 512) or oc.max() > 64     # the stretched range is present
    for walker in (0, 1):
        gl, gc, gk = sim.neighbours(cap, walker=walker)
        assert np.array_equal(gc, oc) and np.array_equal(gk, ok)
        assert np.array_equal(gl, ol)
    g, o, sim2, orc2 = _run_both(pbd, oracle_mod, params, pos, vel, 2)
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 10 * TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < 10 * TOL_V1


def _run_both(pbd, oracle_mod, params, pos, vel, steps, precision="f32"):
    params.flags |= pbd.FLAG_TRACK_IDS
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel, precision=precision)
    sim.step(steps)
    sim.sync()
    orc.step(steps)
    return by_id(sim.state()), by_id(orc.state()), sim, orc


@pytest.mark.parametrize("shape,box,seed", SCENES)
def test_one_frame(need_gpu, pbd, scenes, oracle_mod, shape, box, seed):
    params, pos, vel = workload(pbd, scenes, shape=shape, box=box, seed=seed)
    g, o, sim, orc = _run_both(pbd, oracle_mod, params, pos, vel, 1)
    assert np.array_equal(g["ids"], o["ids"])
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < TOL_V1
    gd, od = sim.debug(), orc.debug()
    assert np.allclose(gd["lambda"], od["lambda"], rtol=1e-3, atol=1e-3)


def test_one_frame_vs_fp64(need_gpu, pbd, scenes, oracle_mod):
    params, pos, vel = workload(pbd, scenes, shape=(12, 12, 12), box=24, seed=11)
    g, o, _, _ = _run_both(pbd, oracle_mod, params, pos, vel, 1, precision="f64")
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 5 * TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < 5 * TOL_V1


@pytest.mark.parametrize("shape,box,seed", SCENES[:2])
def test_ten_frames(need_gpu, pbd, scenes, oracle_mod, shape, box, seed):
    params, pos, vel = workload(pbd, scenes, shape=shape, box=box, seed=seed)
    g, o, _, _ = _run_both(pbd, oracle_mod, params, pos, vel, 10)
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < TOL_X10
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < TOL_V10


def test_vorticity_viscosity_frames(need_gpu, pbd, scenes, oracle_mod):
    params, pos, vel = workload(pbd, scenes, shape=(12, 12, 12), box=24, seed=12, vorticity=0.0005, viscosity=0.01)
    g, o, sim, orc = _run_both(pbd, oracle_mod, params, pos, vel, 3)
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 10 * TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < 10 * TOL_V1
    gd, od = sim.debug(), orc.debug()
    # omega and f_ext are in the frame's sorted order on both sides (same permutation)
    assert np.allclose(gd["omega"][:, :3], od["omega"][:, :3], rtol=1e-2, atol=1e-3)
    assert maxdiff(gd["fext"][:, :3], od["fext"][:, :3]) < 1e-4


@pytest.mark.parametrize("variant", ["stab2", "stab0", "iter0", "no_apply", "no_delta", "no_lambda",
                                     "no_update", "no_forces", "no_contacts", "shells2"])
def test_flag_variants(need_gpu, pbd, scenes, oracle_mod, variant):
    params, pos, vel = workload(pbd, scenes, shape=(10, 10, 10), box=16, seed=13, vorticity=0.001, viscosity=0.02)
    A = pbd.ACTIVE
    if variant == "stab2":
        params.stabilization_iterations = 2
    elif variant == "stab0":
        params.stabilization_iterations = 0
    elif variant == "iter0":
        params.solver_iterations = 0
    elif variant == "no_apply":
        params.active &= ~A["applyDeltaPositions"]
    elif variant == "no_delta":
        params.active &= ~A["computeDeltaPositions"]
    elif variant == "no_lambda":
        params.active &= ~A["computeLambda"]
    elif variant == "no_update":
        params.active &= ~A["updatePositions"]
    elif variant == "no_forces":
        params.active &= ~A["applyForces"]
    elif variant == "no_contacts":
        params.active &= ~A["findContacts"]
        params.kernel_width_neighbours = 2
    elif variant == "shells2":
        params.kernel_width_neighbours = 2
    g, o, _, _ = _run_both(pbd, oracle_mod, params, pos, vel, 2)
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 10 * TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < 10 * TOL_V1


def test_add_clear_and_capacity(need_gpu, pbd, scenes, oracle_mod):
    params, pos, vel = workload(pbd, scenes, shape=(8, 8, 8), box=16, seed=14)
    params.flags |= pbd.FLAG_TRACK_IDS
    n = len(pos)
    sim = pbd.Sim(params, n + 10)
    orc = oracle_mod.Oracle(params, n + 10, "f32")
    for s in (sim, orc):
        s.add_particles(pos[: n // 2], vel[: n // 2])
    sim.step(2); orc.step(2)
    for s in (sim, orc):
        s.add_particles(pos[n // 2:], vel[n // 2:])
        s.add_particle([8.0, 12.0, 8.0], [0.0, -0.1, 0.2])
    sim.step(2); orc.step(2)
    g, o = by_id(sim.state()), by_id(orc.state())
    assert sim.n == orc.n == n + 1
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 10 * TOL_X1
    with pytest.raises(pbd.PBDError) as e:
        sim.add_particles(pos[:10], vel[:10])
    assert e.value.code == pbd.ERR_CAPACITY
    sim.clear(); orc.clear()
    assert sim.n == 0
    sim.step(3)   # N == 0: no work (Fluid.cu:19)
    for s in (sim, orc):
        s.add_particles(pos[:100], vel[:100])
    sim.step(1); orc.step(1)
    g, o = by_id(sim.state()), by_id(orc.state())
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < TOL_X1


def test_collision_type_1_rejects_oversized_constraint_indices(need_gpu, pbd, scenes):
    """collisionType 1 numbers its constraints i * M + k in 32 bits"""
    params, pos, vel = workload(pbd, scenes)
    params.collision_type = 1
    params.max_neighbours_per_particle = 512
    with pytest.raises(pbd.PBDError) as e:
        pbd.Sim(params, (1 << 23) + 1)
    assert e.value.code == pbd.ERR_UNSUPPORTED


def test_sort_full_size_properties(need_gpu, pbd, scenes):
    """1,000,000 particles (the large-fluid workload): keys sorted, keys == morton(p*), the
    permutation a bijection and stable within equal keys, cell ranges consistent."""
    w = scenes.WORKLOADS["fluid_1m"]
    params = scenes.workload_params(pbd, w["box"], 1000.0)
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(*w["shape"], seed=w["seed"])
    rng = np.random.default_rng(0)
    vel[:, :3] = rng.normal(0, 30, size=(len(vel), 3)).astype(np.float32)
    sim = pbd.Sim(params, len(pos))
    sim.add_particles(pos, vel)
    for _ in range(2):
        sim.front()
        d = sim.debug(ncells=1 << 21)
        st = sim.state()
        keys, perm = d["keys"], d["perm"]
        assert np.all(np.diff(keys.astype(np.int64)) >= 0)
        assert np.array_equal(np.sort(perm), np.arange(len(perm), dtype=np.uint32))
        assert np.array_equal(morton_np(st["p"]), keys)
        same = np.diff(keys.astype(np.int64)) == 0
        assert np.all(np.diff(perm.astype(np.int64))[same] > 0)
        occ, first = np.unique(keys, return_index=True)
        assert np.array_equal(d["cell_start"][occ], first.astype(np.uint32))
    sim.sync()


def test_full_size_workload_vs_oracle(need_gpu, pbd, scenes, oracle_mod):
    """The bench's own workload (fluid_1m: 1,000,000 particles, 128^3 cells, vorticity and XSPH,
    the cell-end quirk's long range inside the fluid) against the FP32 oracle on the same inputs:
    the front of the frame bit for bit, then 1 and 3 whole frames within the step's tolerances"""
    import bench
    params, pos, vel, _ = bench.build_workload(pbd, scenes, "fluid_1m")
    params.flags |= pbd.FLAG_TRACK_IDS
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
    sim.front()
    orc.step_phase(oracle_mod.PHASE_FRONT)
    g, o = sim.debug(0), orc.debug(0)
    assert np.array_equal(g["keys"], o["keys"]) and np.array_equal(g["perm"], o["perm"])
    gs, os_ = sim.state(), orc.state()
    assert np.array_equal(gs["p"], os_["p"].astype(np.float32))
    sim.close()
    for frames, tx, tv in ((1, 10 * TOL_X1, 10 * TOL_V1), (3, TOL_X10, TOL_V10)):
        g, o, sim, _ = _run_both(pbd, oracle_mod, params.copy(), pos, vel, frames)
        assert np.array_equal(g["ids"], o["ids"])
        dx = np.abs(g["x"][:, :3] - o["x"][:, :3]).max(axis=1)
        dv = np.abs(g["v"][:, :3] - o["v"][:, :3]).max(axis=1)
        assert dx.max() < tx and dv.max() < tv, (frames, dx.max(), dv.max())
        sim.close()


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 4095, 4097, 8193])
def test_ragged_particle_counts(need_gpu, pbd, scenes, oracle_mod, n):
    """Particle counts around a warp and a sort tile (4096 keys): one particle alone, pairs,
    partial warps and partial last tiles; uniform random positions in a 24^3-cell box (several
    particles share cells, some start outside the walls and are clamped) and random velocities.
    The front is bit-exact, then three frames within the one-frame tolerance x 10."""
    params = scenes.workload_params(pbd, 24, 1000.0)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    rng = np.random.default_rng(1000 + n)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.5, 23.5, size=(n, 3))
    vel[:, :3] = rng.normal(0.0, 2.0, size=(n, 3))
    sim, orc, g, o, gs, os_ = _front_compare(pbd, oracle_mod, params, pos, vel)
    assert np.array_equal(g["keys"], o["keys"]) and np.array_equal(g["perm"], o["perm"])
    assert np.array_equal(gs["p"], os_["p"].astype(np.float32))
    sim.close(); orc.close()
    g, o, sim, orc = _run_both(pbd, oracle_mod, params, pos, vel, 3)
    assert sim.n == n
    assert np.array_equal(g["ids"], o["ids"])
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < 10 * TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < 10 * TOL_V1
