"""The oracle against the reference's own outputs (tests/golden, made by running the
reference's kernel code on the CPU, see tests/golden/make_golden.py).  No GPU.

Bit-exact: predicted positions, keys, permutation and state after the front of a frame, and
the neighbour lists.  Tolerance (FP32, different sqrt/pow/rsqrt rounding): state after 1 and 3
frames, lambda, omega, f_ext; the state after 10 frames particle by particle."""
import numpy as np
import pytest

from helpers import GOLDEN_SCENES, check_fext, check_ten_frames, golden_frame_tolerances, golden_lists, load_golden, scale

WIDTH_CAP = 1024


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_oracle_front_matches_reference(pbd, oracle_mod, name):
    g = load_golden(pbd, name)
    o = oracle_mod.Oracle(g["params_struct"], WIDTH_CAP, "f32")
    o.add_particles(g["pos"], g["vel"])
    o.step_phase(oracle_mod.PHASE_FRONT)
    d, s = o.debug(), o.state()
    assert np.array_equal(d["keys"], g["front_keys"])
    assert np.array_equal(d["perm"], g["front_perm"])
    for k in ("x", "v", "p"):
        assert np.array_equal(s[k].astype(np.float32), g[f"front_{k}"]), k


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_oracle_lists_match_reference(pbd, oracle_mod, name):
    g = load_golden(pbd, name)
    p = g["params_struct"]
    o = oracle_mod.Oracle(p, WIDTH_CAP, "f32")
    o.add_particles(g["pos"], g["vel"])
    o.step_phase(oracle_mod.PHASE_LISTS)
    lst, cnt, con = o.neighbours(p.max_neighbours_per_particle)
    assert np.array_equal(cnt, g["list_count"])
    assert np.array_equal(con, g["list_contacts"])
    for i, ref in enumerate(golden_lists(g)):
        assert np.array_equal(lst[i, :cnt[i]], ref)


@pytest.mark.parametrize("name", GOLDEN_SCENES)
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_oracle_frames_match_reference(pbd, oracle_mod, name, precision):
    g = load_golden(pbd, name)
    for frames, tx, tv in golden_frame_tolerances(name):
        o = oracle_mod.Oracle(g["params_struct"], WIDTH_CAP, precision)
        o.add_particles(g["pos"], g["vel"])
        o.step(frames)
        s, d = o.state(), o.debug()
        assert np.array_equal(d["perm"], g[f"f{frames}_perm"])
        assert np.max(np.abs(s["x"][:, :3] - g[f"f{frames}_x"][:, :3])) < tx
        assert np.max(np.abs(s["v"][:, :3] - g[f"f{frames}_v"][:, :3])) < tv
        lam = g[f"f{frames}_lambda"]
        assert np.max(np.abs(d["lambda"] - lam)) < 1e-3 * scale(lam)
        om = g[f"f{frames}_omega"]
        assert np.max(np.abs(d["omega"][:, :3] - om[:, :3])) < 1e-2 * scale(om)
        if precision == "f32":   # FP64 rounds the near-vanishing |omega| gradients differently
            check_fext(d["fext"], g[f"f{frames}_fext"])


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_oracle_ten_frames_match_reference(pbd, oracle_mod, name):
    g = load_golden(pbd, name)
    p = g["params_struct"].copy()
    p.flags |= pbd.FLAG_TRACK_IDS
    o = oracle_mod.Oracle(p, WIDTH_CAP, "f32")
    o.add_particles(g["pos"], g["vel"])
    o.step(10)
    check_ten_frames(name, o.state(), g)


def test_fixtures_reproduce_from_reference_sources(pbd):
    """Where the reference is mounted, rebuilding the fixtures gives the committed bytes."""
    from oracle.refexec import build_refexec
    if not build_refexec.available():
        pytest.skip("reference sources not mounted")
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    for name in GOLDEN_SCENES:
        committed = load_golden(pbd, name)
        p, pos, vel = mg.SCENES[name]()
        assert np.array_equal(pos, committed["pos"]) and np.array_equal(vel, committed["vel"])
        from oracle.refexec.refexec import RefExec
        r = RefExec(p, mg.WIDTH)
        r.add_particles(pos, vel)
        r.step(1)
        s = r.state()
        r.close()
        assert np.array_equal(s["x"], committed["f1_x"])
