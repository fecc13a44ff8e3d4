"""Shared-memory-staged neighbour passes (PBD_FLAG_STAGED_PASSES) against the stored lists and
the full cell walk.

With the flag, the later lambda passes and the delta passes stage each block's neighbourhood in
shared memory and walk it in the reference's list order; the results must be the same bits as
the default walk over the stored lists and as the cell walk of every pass (PBD_FLAG_FULL_WALK),
over many frames: the dense regime (kernel widths of a few cells, as in the reference's
config.txt) with its cell-end quirk, vorticity and viscosity, fast motion, three shells, and the
h = 1 regime; solids keep the lists."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(pbd, params, pos, vel, frames, flags=0, inv_mass=None):
    p = params.copy()
    p.flags |= flags
    with pbd.Sim(p, len(pos)) as sim:
        if inv_mass is None:
            sim.add_particles(pos, vel)
        else:
            sim.add_particles_mass(pos, vel, inv_mass)
        sim.step(frames)
        sim.sync()
        st = sim.state()
        prof = sim.profile(1)
        sim.sync()
    return st, prof


def _same(a, b):
    for k in ("x", "v", "p", "ids"):
        assert np.array_equal(a[k], b[k]), k


def dense_params(pbd, scenes, box, K=2, vort=0.0, visc=0.0, quirk=True):
    p = scenes.workload_params(pbd, box, 1995.0, vorticity=vort, viscosity=visc)
    p.kernel_width_poly, p.kernel_width_spiky, p.kernel_width_neighbours = 4.1, 3.5, K
    p.lambda_epsilon = 1e-4
    p.flags |= pbd.FLAG_TRACK_IDS
    if not quirk:
        p.flags &= ~pbd.FLAG_CELL_END_QUIRK
    return p


CASES = [
    # shape, box, shells, vorticity, viscosity, quirk, velocity sigma
    ((24, 24, 24), 40, 2, 0.0, 0.0, True, 0.0),
    ((24, 30, 24), 40, 2, 0.0005, 0.00015, True, 0.0),
    ((17, 9, 23), 32, 2, 0.0, 0.00015, False, 4.0),
    ((14, 14, 14), 32, 3, 0.0, 0.0, True, 0.0),
]


@pytest.mark.parametrize("shape,box,K,vort,visc,quirk,sigma", CASES)
def test_staged_passes_bit_identical_to_lists_and_walk(need_gpu, pbd, scenes, shape, box, K, vort, visc, quirk, sigma):
    params = dense_params(pbd, scenes, box, K, vort, visc, quirk)
    pos, vel = scenes.lattice(*shape, seed=5)
    if sigma:
        vel[:, :3] = np.random.default_rng(5).normal(0, sigma, size=(len(vel), 3)).astype(np.float32)
    a, prof = _run(pbd, params, pos, vel, 30, pbd.FLAG_STAGED_PASSES)
    assert "delta_staged" in prof and "lambda_staged" in prof      # the staged kernels ran
    b, prof_b = _run(pbd, params, pos, vel, 30)
    assert "delta_staged" not in prof_b
    _same(a, b)
    c, _ = _run(pbd, params, pos, vel, 30, pbd.FLAG_FULL_WALK)
    _same(a, c)


def test_solids_keep_the_lists(need_gpu, pbd, scenes):
    # inverse masses are not staged: a simulation with solids runs the list passes, same bits
    params = dense_params(pbd, scenes, 40)
    fpos, fvel = scenes.lattice(16, 20, 16, seed=6)
    spos = scenes.solid_boxes(2, (4, 4, 6), (22.0, 1.5, 2.0), (38.0, 38.0, 38.0), 9)
    pos = np.concatenate([fpos, spos])
    vel = np.zeros_like(pos)
    w = np.concatenate([np.ones(len(fpos), np.float32), np.zeros(len(spos), np.float32)])
    a, prof = _run(pbd, params, pos, vel, 20, pbd.FLAG_STAGED_PASSES, inv_mass=w)
    assert "delta_staged" not in prof
    b, _ = _run(pbd, params, pos, vel, 20, pbd.FLAG_FULL_WALK, inv_mass=w)
    _same(a, b)


def test_staging_forced_in_the_h1_regime(need_gpu, pbd, scenes):
    # kernel radius 1 (near lists by default): staging the passes instead gives the same bits
    params = scenes.workload_params(pbd, 32, 1000.0, vorticity=0.0005, viscosity=0.01)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(20, 20, 20, seed=7)
    a, prof = _run(pbd, params, pos, vel, 30, pbd.FLAG_STAGED_PASSES)
    assert "delta_staged" in prof
    b, _ = _run(pbd, params, pos, vel, 30)
    _same(a, b)


def test_staged_dense_against_the_oracle(need_gpu, pbd, scenes, oracle_mod):
    # the dense regime against the FP32 oracle after 1 and 5 frames (tolerances of the parity tests)
    from helpers import by_id, maxdiff
    params = dense_params(pbd, scenes, 32)
    pos, vel = scenes.lattice(16, 16, 16, seed=8)
    for frames, tol_x, tol_v in ((1, 2e-5, 2e-3), (5, 2e-3, 0.2)):
        g, prof = _run(pbd, params, pos, vel, frames, pbd.FLAG_STAGED_PASSES)
        assert "delta_staged" in prof
        o = oracle_mod.Oracle(params, len(pos), "f32")
        o.add_particles(pos, vel)
        o.step(frames)
        r = o.state()
        o.close()
        g, r = by_id(g), by_id(r)
        assert maxdiff(g["x"][:, :3], r["x"][:, :3]) < tol_x
        assert maxdiff(g["v"][:, :3], r["v"][:, :3]) < tol_v
