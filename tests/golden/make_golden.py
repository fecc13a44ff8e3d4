"""Generate tests/golden/*.npz from the reference's own kernel code run on the CPU.

    python tests/golden/make_golden.py

Needs the reference sources (oracle/refexec/build_refexec.py reads them where they lie and
builds oracle/_ref/librefexec.so).  The fixtures hold the inputs and the reference's outputs,
so the tests that read them need neither the reference nor this script.

Scenes:
  config_txt  the reference's own config.txt parameters (kernel widths 6.1 x diameter and 4.1,
              rest density 1200, kernelWidthNeighbours 2, 1 iteration, vorticity 1, viscosity
              1e-4), 10^3 particles spaced 1.2 as Particles.cc:189-203 spawns them, seed 7
  h1_quirk    the h = 1 workload parameters with rest density 1e5, vorticity 5e-4 and XSPH 0.01,
              8^3 particles with random velocities (seed 8): cell N-1 = 511 is occupied, so
              SortReorder.h:183-184 stretches its range to N
  dense       the density-active workload's parameters (fluid_1m_dense: poly6 width 4.1, spiky
              3.5 diameters, two shells, rest density 1995, eps 1e-4, 4 iterations, dt 1/60,
              vorticity 5e-4, XSPH 1.5e-4) on a 10^3 unit lattice in a 24^3-cell box, seed 9
  contact_pairs  collisionType 1 (16 batches) on 216 isolated overlapping pairs, the h = 1 workload
              parameters with the density solve off: the reference's own claim and solve kernels
              (Collision.h:344-459)
For each: the front of a frame (keys, permutation, state), the neighbour lists, and the state,
lambda, omega and f_ext after 1, 3 and 10 frames.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import pbd  # noqa: E402
import scenes  # noqa: E402
from oracle.refexec.refexec import RefExec  # noqa: E402

WIDTH = 32   # texture width: capacity 1024


def scene_config_txt():
    p = pbd.default_params()
    pos, vel = scenes.lattice(10, 10, 10, origin=(30.0, 32.0, 30.0), spacing=1.2, jitter=0.05, seed=7)
    return p, pos, vel


def scene_h1_quirk():
    p = scenes.workload_params(pbd, 16, 1e5, vorticity=0.0005, viscosity=0.01)
    pos, vel = scenes.lattice(8, 8, 8, seed=8)
    rng = np.random.default_rng(8)
    vel[:, :3] = rng.normal(0, 5, size=(len(vel), 3)).astype(np.float32)
    return p, pos, vel


def scene_dense():
    p, pos, vel, _ = scenes.workload("fluid_1m_dense", pbd, shape=(10, 10, 10))
    for a in range(3):
        p.bounds_max[a] = 22.5
    pos, vel = scenes.lattice(10, 10, 10, seed=9)
    return p, pos, vel


def scene_contact_pairs():
    """collisionType 1 on 216 isolated overlapping pairs (separations 0.55-0.95 of a diameter,
    seeded directions), 4 cells apart: every particle's list holds its partner alone, so each batch
    of the reference's claim kernel pairs the same particles whatever its schedule."""
    p = scenes.workload_params(pbd, 32, 1000.0)
    p.collision_type = 1
    p.max_collision_batches = 16
    # the contact projection alone (no density solve): forces, the lists, the batches, the update
    A = pbd.ACTIVE
    p.active = A["applyForces"] | A["findContacts"] | A["findNeighbours"] | A["updatePositions"]
    u = scenes.uniform01(11, 4 * 216).reshape(216, 4)
    pos = np.zeros((432, 4), np.float32)
    k = 0
    for a in range(6):
        for b in range(6):
            for c in range(6):
                centre = np.array([4.0 + 4 * a, 4.0 + 4 * b, 4.0 + 4 * c]) + 0.5
                z = 2.0 * u[k, 0] - 1.0
                phi = 2.0 * np.pi * u[k, 1]
                d = np.array([np.sqrt(1.0 - z * z) * np.cos(phi), np.sqrt(1.0 - z * z) * np.sin(phi), z])
                sep = 0.55 + 0.4 * u[k, 2]
                pos[2 * k, :3] = centre - 0.5 * sep * d
                pos[2 * k + 1, :3] = centre + 0.5 * sep * d
                k += 1
    return p, pos, np.zeros_like(pos)


SCENES = {"config_txt": scene_config_txt, "h1_quirk": scene_h1_quirk, "dense": scene_dense,
          "contact_pairs": scene_contact_pairs}
FRAMES = (1, 3, 10)


def params_array(p):
    return np.frombuffer(bytes(p), dtype=np.uint8).copy()


def generate(name):
    p, pos, vel = SCENES[name]()
    out = {"params": params_array(p), "pos": pos, "vel": vel}
    r = RefExec(p, WIDTH)
    r.add_particles(pos, vel)
    r.step_phase(1)
    d, s = r.debug(), r.state()
    out.update({"front_keys": d["keys"], "front_perm": d["perm"], "front_x": s["x"], "front_v": s["v"], "front_p": s["p"]})
    r.close()
    r = RefExec(p, WIDTH)
    r.add_particles(pos, vel)
    r.step_phase(2)
    lst, cnt, con = r.neighbours(p.max_neighbours_per_particle)
    out["list_count"], out["list_contacts"] = cnt, con
    out["list_entries"] = np.concatenate([lst[i, :cnt[i]] for i in range(len(cnt))]).astype(np.uint32)
    r.close()
    # one frame at a time: each frame's sort permutation carries the particles' input indices
    # along (ids), so later frames can be compared particle by particle
    r = RefExec(p, WIDTH)
    r.add_particles(pos, vel)
    ids = np.arange(len(pos), dtype=np.uint32)
    for frame in range(1, max(FRAMES) + 1):
        r.step(1)
        d = r.debug()
        ids = ids[d["perm"]]
        if frame in FRAMES:
            s = r.state()
            for k in ("x", "v", "p"):
                out[f"f{frame}_{k}"] = s[k]
            for k in ("perm", "lambda", "omega", "fext"):
                out[f"f{frame}_{k}"] = d[k]
            out[f"f{frame}_ids"] = ids.copy()
    r.close()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


if __name__ == "__main__":
    for name in SCENES:
        o = generate(name)
        print(name, len(o["pos"]), "particles, max list", int(o["list_count"].max()))
