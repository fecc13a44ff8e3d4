"""Shared helpers for the parity tests (scene set-up on both backends, comparisons)."""
import numpy as np


def workload(pbd, scenes, shape=(8, 8, 8), box=16, seed=1, rho0=1000.0, eps=0.1, vorticity=0.0, viscosity=0.0,
             iterations=4, flags_extra=0):
    p = scenes.workload_params(pbd, box, rho0, vorticity=vorticity, viscosity=viscosity, iterations=iterations)
    p.lambda_epsilon = eps
    p.flags |= flags_extra
    pos, vel = scenes.lattice(*shape, seed=seed)
    return p, pos, vel


def by_id(state):
    order = np.argsort(state["ids"], kind="stable")
    return {k: (v[order] if hasattr(v, "__len__") and len(v) == len(order) else v) for k, v in state.items()}


def maxdiff(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b))) if a.size else 0.0


def expand_bits_np(v):
    v = v.astype(np.uint64)
    v = (v * np.uint64(0x00010001)) & np.uint64(0xFF0000FF)
    v = (v * np.uint64(0x00000101)) & np.uint64(0x0F00F00F)
    v = (v * np.uint64(0x00000011)) & np.uint64(0xC30C30C3)
    v = (v * np.uint64(0x00000005)) & np.uint64(0x49249249)
    return v.astype(np.uint32)


def morton_np(p):
    """Hash.h:21-29 on float32 (n, >=3) positions."""
    c = np.clip(np.asarray(p, np.float32)[:, :3], np.float32(0), np.float32(1023)).astype(np.uint32)
    with np.errstate(over="ignore"):
        return (expand_bits_np(c[:, 0]) << np.uint32(2)) + (expand_bits_np(c[:, 1]) << np.uint32(1)) + expand_bits_np(c[:, 2])


def setup_pair(pbd, oracle_mod, params, pos, vel, precision="f32", capacity=None):
    cap = capacity or pos.shape[0]
    sim = pbd.Sim(params, cap)
    sim.add_particles(pos, vel)
    orc = oracle_mod.Oracle(params, cap, precision)
    orc.add_particles(pos, vel)
    return sim, orc


GOLDEN_DIR = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")
GOLDEN_SCENES = ("config_txt", "h1_quirk", "dense", "contact_pairs")

# Ten frames against the reference, particle by particle (ids carried by the frames' sort
# permutations): the largest, 99th-percentile and median position / velocity difference per scene.
# config_txt (1 iteration, dt 0.01) stays close; dense (4 iterations of a stiff density solve) and
# h1_quirk (random velocities of sigma 5 colliding in a 16^3-cell box) amplify FP32 rounding
# differences, so their checks are on the distribution.
GOLDEN_TEN = {
    "config_txt": dict(x=(1e-3, 1e-3, 1e-4), v=(2e-2, 2e-2, 2e-3)),
    "dense": dict(x=(0.2, 2e-2, 2e-3), v=(5.0, 1.0, 5e-2)),
    "h1_quirk": dict(x=(2.0, 0.5, 2e-2), v=(100.0, 30.0, 2.0)),
    "contact_pairs": dict(x=(1e-4, 1e-4, 1e-4), v=(1e-2, 1e-2, 1e-2)),
}


def golden_frame_tolerances(name):
    """(frames, |dx| max, |dv| max) of the 1- and 3-frame checks; the dense scene's stiff density
    solve (4 iterations, eps 1e-4) moves rounding differences further in 3 frames."""
    return ((1, 2e-5, 3e-3), (3, 5e-4 if name == "dense" else 1e-4, 2e-2))


def check_ten_frames(name, state, golden):
    """The state after 10 frames (with ids) against the fixture's, within GOLDEN_TEN[name]."""
    a = np.argsort(state["ids"], kind="stable")
    b = np.argsort(golden["f10_ids"], kind="stable")
    dx = np.abs(np.asarray(state["x"])[a, :3] - golden["f10_x"][b, :3]).max(axis=1)
    dv = np.abs(np.asarray(state["v"])[a, :3] - golden["f10_v"][b, :3]).max(axis=1)
    for d, (mx, p99, p50), what in ((dx, GOLDEN_TEN[name]["x"], "x"), (dv, GOLDEN_TEN[name]["v"], "v")):
        got = (float(d.max()), float(np.percentile(d, 99)), float(np.percentile(d, 50)))
        assert got[0] < mx and got[1] < p99 and got[2] < p50, (name, what, got)


def check_fext(fext, ref):
    """f_ext (sorted order of the frame) against the reference's: the 99th percentile of the
    difference within 2% of the largest |f_ext|, and at most 1% of the particles beyond that.  No
    bound on the largest difference: the vorticity direction is the normalised gradient of |omega|
    (Density.h:209-216), which rounding turns freely where that gradient nearly vanishes."""
    sc = max(float(np.abs(ref[:, :3]).max()), 1e-30)
    d = np.abs(np.asarray(fext)[:, :3] - ref[:, :3]).max(axis=1)
    assert np.percentile(d, 99) < 0.02 * sc and np.mean(d > 0.02 * sc) <= 0.01, (float(np.percentile(d, 99)), float(d.max()), sc)


def load_golden(pbd, name):
    """Inputs and the reference's own outputs (tests/golden/make_golden.py)."""
    import os
    d = dict(np.load(os.path.join(GOLDEN_DIR, f"{name}.npz")))
    d["params_struct"] = pbd.Params.from_buffer_copy(d["params"].tobytes())
    return d


def golden_lists(g):
    """Per-particle lists from the flattened fixture."""
    cnt = g["list_count"].astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    return [g["list_entries"][int(offs[i]):int(offs[i + 1])] for i in range(len(cnt))]


def scale(a):
    return max(1.0, float(np.max(np.abs(a))))
