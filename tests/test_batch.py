"""Batched scenes: many independent scenes in one simulation must evolve exactly as each scene
stepped alone (same sort order, same arithmetic), bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene_list(scenes):
    out = []
    for k, (shape, box, rho, g, seed) in enumerate([((6, 5, 7), 16, 950.0, -9.0, 41), ((8, 8, 8), 16, 1050.0, -10.5, 42),
                                                      ((4, 9, 3), 20, 1000.0, -8.2, 43), ((10, 6, 10), 24, 900.0, -11.0, 44)]):
        pos, vel = scenes.lattice(*shape, seed=seed)
        rng = np.random.default_rng(seed)
        vel[:, :3] = rng.normal(0, 3, size=(len(vel), 3)).astype(np.float32)
        out.append(dict(pos=pos, vel=vel, box=box, rho=rho, g=g))
    return out


def _shared(pbd, scenes):
    p = scenes.workload_params(pbd, 16, 1000.0, vorticity=0.0005, viscosity=0.01)
    p.lambda_epsilon = 0.1
    return p


def _single(pbd, shared, sc):
    p = shared.copy()
    p.rest_density = sc["rho"]
    p.gravity = sc["g"]
    for a in range(3):
        p.bounds_min[a] = 1.5
        p.bounds_max[a] = sc["box"] - 1.5
    return p


def test_batch_equals_scenes_stepped_alone(need_gpu, pbd, scenes):
    shared = _shared(pbd, scenes)
    sl = _scene_list(scenes)
    descs = [pbd.scene_desc(len(sc["pos"]) + 5, sc["rho"], sc["g"], sc["box"]) for sc in sl]
    with pbd.Batch(shared, descs) as b:
        for k, sc in enumerate(sl):
            b.add_particles(k, sc["pos"], sc["vel"])
        b.step(6)
        b.sync()
        got = [b.state(k) for k in range(len(sl))]
    for k, sc in enumerate(sl):
        with pbd.Sim(_single(pbd, shared, sc), len(sc["pos"])) as s:
            s.add_particles(sc["pos"], sc["vel"])
            s.step(6)
            s.sync()
            ref = s.state()
        assert np.array_equal(got[k]["x"], ref["x"]), k
        assert np.array_equal(got[k]["v"], ref["v"]), k


def test_batch_add_between_frames_and_autotune(need_gpu, pbd, scenes, tmp_path):
    shared = _shared(pbd, scenes)
    sl = _scene_list(scenes)
    descs = [pbd.scene_desc(len(sc["pos"]) + 5, sc["rho"], sc["g"], sc["box"]) for sc in sl]
    cache = tmp_path / "tune.jsonl"
    with pbd.Batch(shared, descs) as b:
        for k, sc in enumerate(sl):
            b.add_particles(k, sc["pos"][:-5], sc["vel"][:-5])
        b.step(2)
        for k, sc in enumerate(sl):
            b.add_particles(k, sc["pos"][-5:], sc["vel"][-5:])
        assert b.count(0) == len(sl[0]["pos"])
        with pytest.raises(pbd.PBDError) as e:
            b.add_particles(0, sl[0]["pos"][:6], sl[0]["vel"][:6])
        assert e.value.code == pbd.ERR_CAPACITY
        blk = b.autotune(str(cache))
        assert blk in (64, 128, 256)
        assert cache.read_text().count("signature") == 1
        assert b.autotune(str(cache)) == blk            # served from the cache
        b.step(3)
        b.sync()
        assert all(np.all(np.isfinite(b.state(k)["x"])) for k in range(len(sl)))
