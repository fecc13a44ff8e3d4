"""Unified solids: particles with inverse mass 0 (static boxes) in the fluid.

The reference has no solids (mass forced to 1, Forces.h:75,94, Collision.h:223-224); these
tests check the extension against the oracle, which implements the same rules, and that with
every inverse mass 1 the step is exactly the reference's."""
import numpy as np
import pytest

from helpers import by_id, maxdiff

TOL_X1, TOL_V1 = 2e-5, 2e-3


def _scene(pbd, scenes):
    pos, vel, w = scenes.solids_scene((8, 8, 8), 2, (4, 4, 6), 32, 5)
    params = scenes.workload_params(pbd, 32, 1000.0)
    params.lambda_epsilon = 0.1
    params.flags |= pbd.FLAG_TRACK_IDS
    return params, pos, vel, w


def test_oracle_solids_stay_and_unit_masses_change_nothing(pbd, scenes, oracle_mod):
    params, pos, vel, w = _scene(pbd, scenes)
    o = oracle_mod.Oracle(params, len(pos), "f32")
    o.add_particles_mass(pos, vel, w)
    o.step(5)
    s = by_id(o.state())
    solid = w == 0
    assert np.array_equal(s["x"][solid, :3].astype(np.float32), pos[solid, :3])
    assert np.all(s["v"][solid, :3] == 0)
    assert np.abs(s["x"][~solid, :3] - pos[~solid, :3]).max() > 0.01    # the fluid moved
    a = oracle_mod.Oracle(params, len(pos), "f32")
    b = oracle_mod.Oracle(params, len(pos), "f32")
    a.add_particles(pos, vel)
    b.add_particles_mass(pos, vel, np.ones(len(pos), np.float32))
    a.step(3)
    b.step(3)
    assert np.array_equal(a.state()["x"], b.state()["x"])


@pytest.mark.gpu
def test_gpu_solids_match_oracle(need_gpu, pbd, scenes, oracle_mod):
    params, pos, vel, w = _scene(pbd, scenes)
    sim = pbd.Sim(params, len(pos))
    sim.add_particles_mass(pos, vel, w)
    orc = oracle_mod.Oracle(params, len(pos), "f32")
    orc.add_particles_mass(pos, vel, w)
    for frames, tx, tv in ((1, TOL_X1, TOL_V1), (4, 20 * TOL_X1, 20 * TOL_V1)):
        sim.step(frames if frames == 1 else frames - 1)
        sim.sync()
        orc.step(frames if frames == 1 else frames - 1)
        g, o = by_id(sim.state()), by_id(orc.state())
        assert np.array_equal(g["ids"], o["ids"])
        assert maxdiff(g["x"][:, :3], o["x"][:, :3]) < tx
        assert maxdiff(g["v"][:, :3], o["v"][:, :3]) < tv
    solid = w == 0
    assert np.array_equal(g["x"][solid, :3], pos[solid, :3])
    assert np.all(g["v"][solid, :3] == 0)


@pytest.mark.gpu
def test_gpu_unit_masses_are_the_reference_step(need_gpu, pbd, scenes):
    params, pos, vel, w = _scene(pbd, scenes)
    a = pbd.Sim(params, len(pos))
    b = pbd.Sim(params, len(pos))
    a.add_particles(pos, vel)
    b.add_particles_mass(pos, vel, np.ones(len(pos), np.float32))
    a.step(3)
    b.step(3)
    assert np.array_equal(a.state()["x"], b.state()["x"])


@pytest.mark.gpu
def test_gpu_rejects_negative_inverse_mass(need_gpu, pbd, scenes):
    params, pos, vel, w = _scene(pbd, scenes)
    sim = pbd.Sim(params, len(pos))
    w2 = w.copy()
    w2[0] = -1.0
    with pytest.raises(pbd.PBDError) as e:
        sim.add_particles_mass(pos, vel, w2)
    assert e.value.code == pbd.ERR_RANGE
