"""The CUDA step (through the C ABI) against the reference's own outputs (tests/golden).

Bit-exact: keys, permutation and state after the front of a frame; neighbour lists with both
walkers.  Tolerance: state after 1 and 3 frames (FP32 with hardware sqrt/rsqrt/division in the
neighbour passes), lambda, omega, f_ext; the state after 10 frames particle by particle."""
import numpy as np
import pytest

from helpers import GOLDEN_SCENES, check_fext, check_ten_frames, golden_frame_tolerances, golden_lists, load_golden, scale

pytestmark = pytest.mark.gpu
CAP = 1024


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_gpu_front_matches_reference(need_gpu, pbd, name):
    g = load_golden(pbd, name)
    with pbd.Sim(g["params_struct"], CAP) as sim:
        sim.add_particles(g["pos"], g["vel"])
        sim.front()
        d, s = sim.debug(), sim.state()
    assert np.array_equal(d["keys"], g["front_keys"])
    assert np.array_equal(d["perm"], g["front_perm"])
    for k in ("x", "v", "p"):
        assert np.array_equal(s[k], g[f"front_{k}"]), k


@pytest.mark.parametrize("name", GOLDEN_SCENES)
@pytest.mark.parametrize("walker", [0, 1])
def test_gpu_lists_match_reference(need_gpu, pbd, name, walker):
    g = load_golden(pbd, name)
    p = g["params_struct"]
    with pbd.Sim(p, CAP) as sim:
        sim.add_particles(g["pos"], g["vel"])
        sim.front()
        lst, cnt, con = sim.neighbours(p.max_neighbours_per_particle, walker=walker)
    assert np.array_equal(cnt, g["list_count"])
    assert np.array_equal(con, g["list_contacts"])
    for i, ref in enumerate(golden_lists(g)):
        assert np.array_equal(lst[i, :cnt[i]], ref)


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_gpu_frames_match_reference(need_gpu, pbd, name):
    g = load_golden(pbd, name)
    for frames, tx, tv in golden_frame_tolerances(name):
        with pbd.Sim(g["params_struct"], CAP) as sim:
            sim.add_particles(g["pos"], g["vel"])
            sim.step(frames)
            sim.sync()
            s, d = sim.state(), sim.debug()
        assert np.array_equal(d["perm"], g[f"f{frames}_perm"])
        assert np.max(np.abs(s["x"][:, :3] - g[f"f{frames}_x"][:, :3])) < tx
        assert np.max(np.abs(s["v"][:, :3] - g[f"f{frames}_v"][:, :3])) < tv
        lam = g[f"f{frames}_lambda"]
        assert np.max(np.abs(d["lambda"] - lam)) < 1e-3 * scale(lam)
        om = g[f"f{frames}_omega"]
        assert np.max(np.abs(d["omega"][:, :3] - om[:, :3])) < 1e-2 * scale(om)
        check_fext(d["fext"], g[f"f{frames}_fext"])


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_gpu_ten_frames_match_reference(need_gpu, pbd, name):
    g = load_golden(pbd, name)
    p = g["params_struct"].copy()
    p.flags |= pbd.FLAG_TRACK_IDS
    with pbd.Sim(p, CAP) as sim:
        sim.add_particles(g["pos"], g["vel"])
        sim.step(10)
        sim.sync()
        check_ten_frames(name, sim.state(), g)
