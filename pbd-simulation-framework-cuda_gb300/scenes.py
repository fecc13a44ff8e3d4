"""Seeded synthetic scenes and parameter sets for the step's standard workloads.

The reference spawns a lattice box from config.txt's Particles.Box keys
(src/app/rendering/Particles.cc:189-222); the workloads here are lattices at cell centres,
jittered by SplitMix64 (Vigna's published 64-bit mixer, restated below), so every backend
(GPU library, CPU oracle) is fed the same bytes.

Workloads (dt = 1/60, gravity -9.82, 4 solver iterations):
  dam_break_32k   32^3 unit lattice in a 64^3-cell box, kernel radius h = 1, seed 1
  fluid_1m        100^3 unit lattice in a 128^3-cell domain, h = 1, vorticity 5e-4, XSPH 0.01, seed 2
  fluid_1m_dense  the same 1,000,000 particles with the density regime of the reference's own
                  config.txt: poly6 width 4.1, spiky width 3.5 particle diameters, two cell shells
                  (kernelWidthNeighbours 2, ~125 list entries per particle), rest density 1995 (the
                  lattice's own poly6 density), lambda eps 1e-4 as Density.h:90 hard-codes it,
                  vorticity 5e-4, XSPH 1.5e-4 (c * rest density = 0.3)
  solids_328k     64^3 fluid particles + 8 static solid boxes of 8,192 particles (inverse mass 0)
                  in a 128^3-cell domain, seed 3
  adjoint_64k     32 x 64 x 32 fluid column in a 72^3-cell box with a seeded target, seed 5

With h = 1 on a unit lattice the reference's density (no self term, unit mass, Density.h:67-84)
is ~0, so the h = 1 workloads run with lambda eps 0.1 and their density constraint is inactive
(C ~ -1): they measure gravity, contacts, vorticity and viscosity.  fluid_1m_dense is the
workload whose density solve acts.
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


def config_txt_params(params_type):
    """A `params_type` (pbd.Params) holding the reference's config.txt values (config.txt:9-131,
    Particles.cc:8 for maxGrid, Density.h:90 for eps) -- the same values pbd_params_default
    writes, filled here without loading the library (the CPU reference arm uses it)."""
    p = params_type()
    p.struct_size = 128
    p.threads_per_block = 512
    p.particle_radius = 0.5
    p.max_neighbours_per_particle = 512
    p.delta_t = 0.01
    p.gravity = -29.82
    p.rest_density = 1200.0
    p.kernel_width_spiky = 6.1
    p.k_scorr = 0.2
    p.n_scorr = 4
    p.q_scorr = 0.2
    p.c_viscosity = 0.0001
    p.kernel_width_poly = 4.1
    p.e_vorticity = 1.0
    p.collision_type = 0
    p.kernel_width_neighbours = 2
    p.max_collision_batches = 16
    p.stiffness = 0.3
    p.enclosure_position_damping = 0.0
    p.enclosure_velocity_damping = 1.0
    for a in range(3):
        p.bounds_min[a] = 1.5
        p.bounds_max[a] = 62.5
    p.solver_iterations = 1
    p.stabilization_iterations = 1
    p.active = 0x3FF
    p.max_grid = 128 ** 3
    p.lambda_epsilon = 0.0001
    p.flags = 1            # PBD_FLAG_CELL_END_QUIRK
    return p


_ACTIVE_OMEGAS, _ACTIVE_VORTICITY, _ACTIVE_VISCOSITY = 1 << 7, 1 << 8, 1 << 9


def workload_params(pbd, box, rest_density, vorticity=0.0, viscosity=0.0, iterations=4, max_neighbours=512,
                    base=None):
    """pbd_params for the standard workloads: radius 0.5 (diameter 1 = cell width), kernel widths
    1.0 (spiky factor 1 x diameter, poly 1.0 absolute), q = 0.2 h, gravity -9.82, dt = 1/60,
    walls at 1.5 and box - 1.5, 27-cell neighbourhood (kernelWidthNeighbours = 1).  `base` (a
    filled pbd.Params) replaces the library's defaults as the starting point."""
    p = base.copy() if base is not None else pbd.default_params()
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
    act = 0x3FF
    if vorticity == 0.0:
        act &= ~(_ACTIVE_OMEGAS | _ACTIVE_VORTICITY)
    if viscosity == 0.0:
        act &= ~_ACTIVE_VISCOSITY
    p.active = act
    return p


def solid_boxes(n_boxes, box_shape, region_min, region_max, seed):
    """Static solid boxes on the floor: unit-spacing lattices of `box_shape` cells, placed at
    seeded cell-aligned offsets inside [region_min, region_max) on a grid that keeps them apart."""
    bx, by, bz = box_shape
    nx = max(1, int((region_max[0] - region_min[0]) // (bx + 2)))
    nz = max(1, int((region_max[2] - region_min[2]) // (bz + 2)))
    slots = [(a, c) for a in range(nx) for c in range(nz)]
    u = uniform01(seed, 4 * len(slots))
    order = np.argsort(u[: len(slots)], kind="stable")
    if n_boxes > len(slots):
        raise ValueError("solid boxes do not fit the region")
    pos = []
    for k in range(n_boxes):
        a, c = slots[order[k]]
        sx = int(u[len(slots) + k] * ((region_max[0] - region_min[0]) / nx - bx - 1))
        sz = int(u[2 * len(slots) + k] * ((region_max[2] - region_min[2]) / nz - bz - 1))
        ox = region_min[0] + a * (region_max[0] - region_min[0]) / nx + sx
        oz = region_min[2] + c * (region_max[2] - region_min[2]) / nz + sz
        i, j, l = np.meshgrid(np.arange(bx), np.arange(by), np.arange(bz), indexing="ij")
        b = np.stack([i.ravel() + np.floor(ox) + 0.5, j.ravel() + region_min[1] + 0.5, l.ravel() + np.floor(oz) + 0.5], axis=1)
        pos.append(b)
    p = np.concatenate(pos).astype(np.float32)
    out = np.zeros((len(p), 4), np.float32)
    out[:, :3] = p
    return out


def solids_scene(fluid_shape=(64, 64, 64), n_boxes=8, box_shape=(16, 16, 32), box=128, seed=3):
    """Fluid lattice in the low-x corner and static solid boxes in the high-x half.
    Returns pos, vel, inverse mass (1 fluid, 0 solid)."""
    fpos, fvel = lattice(*fluid_shape, seed=seed)
    x0 = 2.5 + fluid_shape[0] + 2.0
    spos = solid_boxes(n_boxes, box_shape, (x0, 1.5, 2.0), (box - 2.0, box - 2.0, box - 2.0), seed + 1000)
    pos = np.concatenate([fpos, spos])
    vel = np.zeros_like(pos)
    w = np.concatenate([np.ones(len(fpos), np.float32), np.zeros(len(spos), np.float32)])
    return pos, vel, w


def batched_scenes(nscenes=256, seed=4, n_range=(4096, 65536), rho_range=(900.0, 1100.0),
                   g_range=(8.0, 11.0), box_range=(32, 96)):
    """Seeded batch of dam breaks: per scene a particle count, rest density, gravity magnitude and
    cubic domain (cells per side), each drawn uniformly; a domain too small to hold its count as a
    unit lattice cube with room to fall is raised to cbrt(n) + 8 cells.  The fluid block is a
    lattice cube of that count in the domain's lower corner."""
    u = uniform01(seed, 4 * nscenes).reshape(nscenes, 4)
    out = []
    for k in range(nscenes):
        n = int(n_range[0] + u[k, 0] * (n_range[1] - n_range[0] + 1))
        box = int(box_range[0] + u[k, 3] * (box_range[1] - box_range[0] + 1))
        box = min(box_range[1], max(box, int(np.ceil(n ** (1.0 / 3.0))) + 8))
        rho = float(rho_range[0] + u[k, 1] * (rho_range[1] - rho_range[0]))
        g = -float(g_range[0] + u[k, 2] * (g_range[1] - g_range[0]))
        side = box - 4                       # lattice columns that fit between the walls
        nx = min(side, max(1, int(round(n ** (1.0 / 3.0)))))
        nz = nx
        ny = -(-n // (nx * nz))
        if ny > side:                         # too tall: widen the base
            nx = nz = side
            ny = -(-n // (nx * nz))
        pos, vel = lattice(nx, ny, nz, seed=seed * 1000 + k)
        out.append(dict(n=n, rest_density=rho, gravity=g, box=box, pos=pos[:n], vel=vel[:n]))
    return out


def adjoint_dam_break(shape=(32, 64, 32), box=72, seed=5):
    """Differentiable dam break: a unit lattice column of 65,536 particles (32 x 64 x 32) at rest
    in a 72^3-cell box and a seeded target configuration (uniform in the lower half of the box
    between the walls).  Returns pos, vel, target (n, 3) float64."""
    pos, vel = lattice(*shape, seed=seed)
    n = len(pos)
    u = uniform01(seed + 7000, 3 * n).reshape(n, 3)
    lo, hi = 2.0, box - 2.0
    target = lo + u * (hi - lo)
    target[:, 1] = lo + u[:, 1] * (box / 2.0 - lo)
    return pos, vel, target


WORKLOADS = {
    "dam_break_32k": dict(shape=(32, 32, 32), box=64, seed=1, vorticity=0.0, viscosity=0.0,
                          rest_density=1000.0, lambda_epsilon=0.1),
    "fluid_1m": dict(shape=(100, 100, 100), box=128, seed=2, vorticity=0.0005, viscosity=0.01,
                     rest_density=1000.0, lambda_epsilon=0.1),
    "fluid_1m_dense": dict(shape=(100, 100, 100), box=128, seed=2, vorticity=0.0005, viscosity=0.00015,
                           rest_density=1995.0, lambda_epsilon=0.0001, kernel_width_poly=4.1,
                           kernel_width_spiky=3.5, kernel_width_neighbours=2),
    "solids_328k": dict(shape=(64, 64, 64), box=128, seed=3, vorticity=0.0, viscosity=0.0, solids=(8, (16, 16, 32)),
                        rest_density=1000.0, lambda_epsilon=0.1),
}


def workload(name, pbd, base=None, shape=None):
    """(params, pos, vel, spec) of a standard workload; `base` as in workload_params; `shape`
    overrides the lattice (a smaller case of the same parameters, for the oracle)."""
    w = WORKLOADS[name]
    p = workload_params(pbd, w["box"], w["rest_density"], vorticity=w["vorticity"], viscosity=w["viscosity"], base=base)
    p.lambda_epsilon = w["lambda_epsilon"]
    for key in ("kernel_width_poly", "kernel_width_spiky", "kernel_width_neighbours"):
        if key in w:
            setattr(p, key, w[key])
    pos, vel = lattice(*(shape or w["shape"]), spacing=w.get("spacing", 1.0), seed=w["seed"])
    return p, pos, vel, w
