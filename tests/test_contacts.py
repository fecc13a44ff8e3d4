"""collisionType 1: contact constraints solved in batches of disjoint pairs (Collision.h:288-436).

The batches are defined as in the oracle (solve_collisions_batched): constraints are the frame's
list entries c = i * M + k; per batch each particle takes its highest-priority pending overlapping
constraint (priority lowbias32(c + 1)) and a constraint both of whose particles took it is solved,
in place on p* and x.
CPU: the oracle's batches on isolated overlapping pairs give the exact separations, and FP32 and
FP64 oracles agree.
GPU: the CUDA path against the FP32 oracle after 1 and 5 frames (tolerances of the step's parity
tests: 2e-5 after one frame, 2e-3 after five, in cell widths), exact separations on isolated
pairs, solids, and the stored lists against the cell walk."""
import numpy as np
import pytest

from helpers import maxdiff, setup_pair, by_id

TOL_X1, TOL_X5 = 2e-5, 2e-3


def contact_scene(pbd, scenes, shape=(10, 8, 10), spacing=0.8, box=20, batches=6, iterations=2, seed=8,
                  density=True):
    p = scenes.workload_params(pbd, box, 1000.0, iterations=iterations)
    p.lambda_epsilon = 0.1
    p.collision_type = 1
    p.max_collision_batches = batches
    p.flags |= pbd.FLAG_TRACK_IDS
    if not density:
        for k in ("computeLambda", "computeDeltaPositions", "applyDeltaPositions"):
            p.active &= ~pbd.ACTIVE[k]
    pos, vel = scenes.lattice(*shape, spacing=spacing, seed=seed)
    vel[:, :3] = np.random.default_rng(seed).normal(0, 1.0, size=(len(vel), 3)).astype(np.float32)
    return p, pos, vel


def pair_scene(pbd, scenes, r0=0.6, n_side=5, spacing=3.0, batches=4, seed=9):
    """isolated overlapping pairs: (n_side^3) pairs 3 cells apart, partners r0 apart along a
    seeded direction; no gravity, no density solve, one iteration"""
    p = scenes.workload_params(pbd, 24, 1000.0, iterations=1)
    p.collision_type = 1
    p.max_collision_batches = batches
    p.gravity = 0.0
    p.flags |= pbd.FLAG_TRACK_IDS
    p.flags &= ~pbd.FLAG_CELL_END_QUIRK
    for k in ("computeLambda", "computeDeltaPositions", "applyDeltaPositions"):
        p.active &= ~pbd.ACTIVE[k]
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3) * spacing + 4.0
    d = np.random.default_rng(seed).normal(size=g.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = np.zeros((2 * len(g), 4), np.float32)
    pos[0::2, :3] = g - 0.5 * r0 * d
    pos[1::2, :3] = g + 0.5 * r0 * d
    return p, pos, np.zeros_like(pos)


@pytest.mark.parametrize("batches,expect", [(0, 0.6), (1, 0.88), (4, 0.964)])
def test_oracle_batches_on_isolated_pairs(pbd, scenes, oracle_mod, batches, expect):
    """one pass: the pair's two constraints (i, j) and (j, i) are solved in successive batches,
    each moving the particles apart by (1 - stiffness) of the overlap"""
    p, pos, vel = pair_scene(pbd, scenes, batches=batches)
    o = oracle_mod.Oracle(p, len(pos), "f64")
    o.add_particles(pos, vel)
    o.step(1)
    x = by_id(o.state())["x"]
    r = np.linalg.norm(x[0::2, :3] - x[1::2, :3], axis=1)
    assert np.allclose(r, expect, atol=1e-5)
    mid0 = 0.5 * (pos[0::2, :3] + pos[1::2, :3])
    assert np.allclose(0.5 * (x[0::2, :3] + x[1::2, :3]), mid0, atol=1e-5)   # equal and opposite moves


@pytest.mark.parametrize("shape,spacing", [((10, 8, 10), 0.8), ((9, 8, 9), 0.45)])
def test_oracle_precisions_agree(pbd, scenes, oracle_mod, shape, spacing):
    """FP32 and FP64 oracles agree, also on a packed block whose lists mostly exceed 64 entries"""
    p, pos, vel = contact_scene(pbd, scenes, shape=shape, spacing=spacing)
    a = oracle_mod.Oracle(p, len(pos), "f32"); a.add_particles(pos, vel); a.step(1)
    b = oracle_mod.Oracle(p, len(pos), "f64"); b.add_particles(pos, vel); b.step(1)
    sa, sb = by_id(a.state()), by_id(b.state())
    assert maxdiff(sa["x"][:, :3], sb["x"][:, :3]) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("frames,tol", [(1, TOL_X1), (5, TOL_X5)])
@pytest.mark.parametrize("density", [True, False])
def test_gpu_contact_batches_match_oracle(need_gpu, pbd, scenes, oracle_mod, frames, tol, density):
    p, pos, vel = contact_scene(pbd, scenes, density=density)
    sim, orc = setup_pair(pbd, oracle_mod, p, pos, vel)
    sim.step(frames)
    orc.step(frames)
    g, o = by_id(sim.state()), by_id(orc.state())
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) <= tol
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) <= tol * 100


@pytest.mark.gpu
@pytest.mark.parametrize("density", [True, False])
def test_gpu_contact_batches_long_lists(need_gpu, pbd, scenes, oracle_mod, density):
    """a packed block (~8 particles per cell): most lists hold more than 64 entries, which the
    claim pass hands to whole warps"""
    p, pos, vel = contact_scene(pbd, scenes, shape=(9, 8, 9), spacing=0.45, density=density)
    sim, orc = setup_pair(pbd, oracle_mod, p, pos, vel)
    sim.step(1)
    orc.step(1)
    _, cnt, _ = sim.neighbours(512)
    assert (cnt > 64).mean() > 0.5 and (cnt <= 64).sum() > 0
    g, o = by_id(sim.state()), by_id(orc.state())
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) <= TOL_X1
    assert maxdiff(g["v"][:, :3], o["v"][:, :3]) <= TOL_X1 * 100


@pytest.mark.gpu
def test_gpu_contact_batches_on_isolated_pairs(need_gpu, pbd, scenes):
    p, pos, vel = pair_scene(pbd, scenes)
    sim = pbd.Sim(p, len(pos)); sim.add_particles(pos, vel); sim.step(1)
    x = by_id(sim.state())["x"]
    r = np.linalg.norm(x[0::2, :3].astype(np.float64) - x[1::2, :3], axis=1)
    assert np.allclose(r, 0.964, atol=1e-5)


@pytest.mark.gpu
def test_gpu_contact_batches_with_solids(need_gpu, pbd, scenes, oracle_mod):
    pos, vel, w = scenes.solids_scene(fluid_shape=(10, 10, 10), n_boxes=2, box_shape=(6, 6, 8), box=40, seed=5)
    p = scenes.workload_params(pbd, 40, 1000.0)
    p.lambda_epsilon = 0.1
    p.collision_type = 1
    p.max_collision_batches = 8
    p.flags |= pbd.FLAG_TRACK_IDS
    sim = pbd.Sim(p, len(pos)); sim.add_particles_mass(pos, vel, w)
    orc = oracle_mod.Oracle(p, len(pos), "f32"); orc.add_particles_mass(pos, vel, w)
    sim.step(3); orc.step(3)
    g, o = by_id(sim.state()), by_id(orc.state())
    assert maxdiff(g["x"][:, :3], o["x"][:, :3]) <= TOL_X5
    solid = w == 0
    assert np.array_equal(g["x"][solid, :3], pos[solid, :3])    # solids never move


@pytest.mark.gpu
def test_gpu_contact_batches_lists_match_cell_walk(need_gpu, pbd, scenes):
    p, pos, vel = contact_scene(pbd, scenes)
    out = []
    for fw in (False, True):
        q = p.copy()
        if fw:
            q.flags |= pbd.FLAG_FULL_WALK
        sim = pbd.Sim(q, len(pos)); sim.add_particles(pos, vel); sim.step(8)
        out.append(sim.state())
    assert np.array_equal(out[0]["ids"], out[1]["ids"])
    for k in ("x", "v"):
        assert np.array_equal(out[0][k], out[1][k]), k
