"""Seeded synthetic scenes and parameter sets for the step's standard workloads.

The reference spawns a lattice box from config.txt's Particles.Box keys
(src/app/rendering/Particles.cc:189-222); the workloads here are lattices at cell centres,
jittered by SplitMix64 (Vigna's published 64-bit mixer, restated below), so every backend
(GPU library, CPU oracle) is fed the same bytes.

Workloads (kernel radius h = 1 = particle diameter, dt = 1/60, 4 solver iterations):
  dam_break_32k   32^3 fluid particles in a 64^3-cell box, seed 1
  fluid_1m        100^3 fluid particles in a 128^3-cell domain, vorticity 5e-4, XSPH 0.01, seed 2
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, n):
    """n consecutive SplitMix64 outputs for `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        state = np.uint64(seed) + _GOLDEN * np.arange(1, n + 1, dtype=np.uint64)
        z = state
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed, n):
    """n floats in [0, 1) with 24 random bits each."""
    return (splitmix64(seed, n) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))


def lattice(nx, ny, nz, origin=(2.5, 2.5, 2.5), spacing=1.0, jitter=0.05, seed=1):
    """float32 (n, 4) positions (w = 0, as Particles.cc:200 spawns them) on a jittered lattice
    and zero velocities.  Lattice order is x outer, y, z inner (Particles.cc:196-203)."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64) * spacing + np.asarray(origin)
    n = base.shape[0]
    u = uniform01(seed, 3 * n).reshape(n, 3)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (base + (2.0 * u - 1.0) * jitter).astype(np.float32)
    vel = np.zeros((n, 4), np.float32)
    return pos, vel


def workload_params(pbd, box, rest_density, vorticity=0.0, viscosity=0.0, iterations=4, max_neighbours=512):
    """pbd_params for the standard workloads: radius 0.5 (diameter 1 = cell width), kernel widths
    1.0 (spiky factor 1 x diameter, poly 1.0 absolute), q = 0.2 h, gravity -9.82, dt = 1/60,
    walls at 1.5 and box - 1.5, 27-cell neighbourhood (kernelWidthNeighbours = 1)."""
    p = pbd.default_params()
    p.particle_radius = 0.5
    p.kernel_width_spiky = 1.0
    p.kernel_width_poly = 1.0
    p.q_scorr = 0.2
    p.gravity = -9.82
    p.delta_t = 1.0 / 60.0
    p.solver_iterations = iterations
    p.stabilization_iterations = 1
    p.kernel_width_neighbours = 1
    p.max_neighbours_per_particle = max_neighbours
    p.rest_density = rest_density
    for a in range(3):
        p.bounds_min[a] = 1.5
        p.bounds_max[a] = float(box) - 1.5
    p.e_vorticity = vorticity
    p.c_viscosity = viscosity
    act = pbd.ACTIVE_ALL
    if vorticity == 0.0:
        act &= ~(pbd.ACTIVE["computeOmegas"] | pbd.ACTIVE["computeVorticity"])
    if viscosity == 0.0:
        act &= ~pbd.ACTIVE["computeViscosity"]
    p.active = act
    return p


WORKLOADS = {
    "dam_break_32k": dict(shape=(32, 32, 32), box=64, seed=1, vorticity=0.0, viscosity=0.0),
    "fluid_1m": dict(shape=(100, 100, 100), box=128, seed=2, vorticity=0.0005, viscosity=0.01),
}
