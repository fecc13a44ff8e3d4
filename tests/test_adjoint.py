"""Adjoint of the frame: dL/dv0, dL/dx0, dL/drest_density and dL/deps of L = sum(c . x_final).

CPU: the FP64 restatement (oracle/adjoint.py) is pinned to the C oracle's FP64 trajectory and
its reverse pass to central differences of its own forward, with and without XSPH viscosity,
unified solids (inverse mass 0) and vorticity confinement (whose force enters the next frame).
GPU: pbd_adjoint_forward/backward through the C ABI against that FP64 reverse pass on the same
seeded scene, with several checkpoint spacings, and the state the forward left restored.
Tolerance of the GPU gradients against the FP64 reverse pass (FP32 forward and reverse): 2% of
the largest component for the arrays, 2% for the scalars.  Between GPU runs the gradients are
bit-identical (the scattered terms are summed in fixed point)."""
import copy

import numpy as np
import pytest

from helpers import maxdiff

FRAMES = 8


def adjoint_scene(pbd, scenes, shape=(7, 7, 7), box=14, spacing=0.75, iterations=3, seed=5, vel_sigma=1.0,
                  viscosity=0.0, vorticity=0.0):
    prm = scenes.workload_params(pbd, box, 1000.0, iterations=iterations, viscosity=viscosity, vorticity=vorticity)
    prm.lambda_epsilon = 0.1
    prm.flags &= ~pbd.FLAG_CELL_END_QUIRK
    prm.flags |= pbd.FLAG_TRACK_IDS
    pos, vel = scenes.lattice(*shape, spacing=spacing, seed=seed)
    rng = np.random.default_rng(seed)
    vel[:, :3] = rng.normal(0, vel_sigma, size=(len(vel), 3)).astype(np.float32)
    weights = rng.normal(size=(len(pos), 3))
    return prm, pos, vel, weights


def with_solids(pos, vel, seed=5):
    """Unified solids in an adjoint scene: the lowest layer and a seeded tenth of the other
    particles get inverse mass 0 and no velocity.  Returns (vel, inverse masses)."""
    rng = np.random.default_rng(seed + 100)
    m = np.ones(len(pos), np.float32)
    m[pos[:, 1] < pos[:, 1].min() + 0.5] = 0.0
    m[rng.random(len(pos)) < 0.1] = 0.0
    vel = vel.copy()
    vel[m == 0.0, :3] = 0.0
    return vel, m


@pytest.fixture(scope="module")
def adj():
    from oracle import adjoint as m
    return m


@pytest.mark.parametrize("viscosity,solids,vorticity", [(0.0, False, 0.0), (0.01, False, 0.0), (0.0, True, 0.0),
                                                        (0.01, True, 0.0), (0.0, False, 0.01), (0.01, True, 0.01)])
def test_restatement_follows_oracle(pbd, scenes, oracle_mod, adj, viscosity, solids, vorticity):
    prm, pos, vel, _ = adjoint_scene(pbd, scenes, viscosity=viscosity, vorticity=vorticity)
    m = None
    if solids:
        vel, m = with_solids(pos, vel)
    C = adj.Consts(prm, m)
    o = oracle_mod.Oracle(prm, len(pos), "f64")
    if solids:
        o.add_particles_mass(pos, vel, m)
    else:
        o.add_particles(pos, vel)
    x, v = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    f = None
    for _ in range(FRAMES):
        o.step(1)
        x, v, f = adj.frame(C, x, v, f)
    s = o.state()
    order = np.argsort(s["ids"])
    assert maxdiff(s["x"][order, :3], x) < 1e-8
    assert maxdiff(s["v"][order, :3], v) < 1e-6
    if solids:   # the solids never moved
        assert np.array_equal(x[m == 0], pos[m == 0, :3].astype(np.float64))


def _loss(adj, C, x0, v0, w):
    x, _ = adj.rollout(C, x0, v0, FRAMES)
    return float(np.sum(w * x))


@pytest.mark.parametrize("viscosity,solids,vorticity", [(0.0, False, 0.0), (0.01, False, 0.0), (0.01, True, 0.0),
                                                        (0.0, False, 0.01), (0.01, True, 0.01)])
def test_reverse_pass_matches_central_differences(pbd, scenes, adj, viscosity, solids, vorticity):
    prm, pos, vel, w = adjoint_scene(pbd, scenes, viscosity=viscosity, vorticity=vorticity)
    m = None
    if solids:
        vel, m = with_solids(pos, vel)
    C = adj.Consts(prm, m)
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    gv, gx, gr, ge = adj.backward(C, x0, v0, FRAMES, w)
    rng = np.random.default_rng(11)
    dirn = rng.normal(size=x0.shape)
    # with solids or vorticity a step of 1e-6 straddles a contact threshold within the 8 frames
    # (the differences at 1e-7 agree with the reverse pass to 1e-8)
    h = 1e-7 if (solids or vorticity) else 1e-6
    fd_v = (_loss(adj, C, x0, v0 + h * dirn, w) - _loss(adj, C, x0, v0 - h * dirn, w)) / (2 * h)
    assert abs(fd_v - np.sum(gv * dirn)) <= 1e-4 * abs(fd_v), (fd_v, np.sum(gv * dirn))
    fd_x = (_loss(adj, C, x0 + h * dirn, v0, w) - _loss(adj, C, x0 - h * dirn, v0, w)) / (2 * h)
    assert abs(fd_x - np.sum(gx * dirn)) <= 1e-3 * abs(fd_x)
    for attr, g in (("rho0", gr), ("eps", ge)):
        base = getattr(C, attr)
        hh = (1e-5 if (solids or vorticity) else 1e-4) * base   # 1e-4 straddles the same threshold there
        cp, cm = copy.copy(C), copy.copy(C)
        setattr(cp, attr, base + hh)
        setattr(cm, attr, base - hh)
        fd = (_loss(adj, cp, x0, v0, w) - _loss(adj, cm, x0, v0, w)) / (2 * hh)
        assert abs(fd - g) <= 1e-3 * abs(fd), (attr, fd, g)


def test_adjoint_symbols_and_argument_checks_declared(pbd):
    L = pbd.lib()
    assert hasattr(L, "pbd_adjoint_forward") and hasattr(L, "pbd_adjoint_backward")


# ---------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------

def _gpu_grads(pbd, prm, pos, vel, weights, frames, every, inv_mass=None):
    sim = pbd.Sim(prm, len(pos))
    if inv_mass is not None:
        sim.add_particles_mass(pos, vel, inv_mass)
    else:
        sim.add_particles(pos, vel)
    sim.adjoint_forward(frames, every)
    fin = sim.state()
    dl = np.zeros((len(pos), 4), np.float32)
    dl[:, :3] = weights[fin["ids"]]
    gv, gx, gr, ge = sim.adjoint_backward(dl)
    after = sim.state()
    return sim, fin, after, gv[:, :3], gx[:, :3], gr, ge


def _close(a, b, rel=0.02):
    return maxdiff(a, b) <= rel * max(1e-30, float(np.max(np.abs(b))))


def _close_l2(a, b, rel=0.02):
    """relative L2 error: robust to the few particles whose FP32 and FP64 trajectories meet a
    wall clamp on different frames (the clamp zeroes that particle's gradient on that axis)"""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b)) <= rel * float(np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("every,viscosity,solids,vorticity", [(FRAMES, 0.0, False, 0.0), (3, 0.0, False, 0.0),
                                                              (1, 0.0, False, 0.0), (3, 0.01, False, 0.0),
                                                              (3, 0.01, True, 0.0), (3, 0.0, False, 0.01),
                                                              (3, 0.01, True, 0.01)])
def test_gpu_adjoint_matches_fp64(need_gpu, pbd, scenes, adj, every, viscosity, solids, vorticity):
    prm, pos, vel, w = adjoint_scene(pbd, scenes, viscosity=viscosity, vorticity=vorticity)
    m = None
    if solids:
        vel, m = with_solids(pos, vel)
    C = adj.Consts(prm, m)
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), FRAMES, w)
    sim, fin, after, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, FRAMES, every, m)
    assert _close(gv, rv) and _close(gx, rx)
    assert abs(gr - rr) <= 0.02 * abs(rr) and abs(ge - re) <= 0.02 * abs(re)
    # the backward leaves the simulation as the forward left it
    for k in ("x", "v", "p", "ids"):
        assert np.array_equal(fin[k], after[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("iterations,viscosity,solids", [(1, 0.0, False), (4, 0.0, False), (4, 0.01, False),
                                                         (4, 0.01, True)])
def test_gpu_adjoint_one_frame_exact(need_gpu, pbd, scenes, adj, iterations, viscosity, solids):
    """one frame: the FP32 reverse pass equals the FP64 one up to FP32 rounding"""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(12, 10, 12), box=20, iterations=iterations, seed=7,
                                     viscosity=viscosity)
    m = None
    if solids:
        vel, m = with_solids(pos, vel, seed=7)
    C = adj.Consts(prm, m)
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), 1, w)
    _, _, _, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, 1, 1, m)
    assert _close_l2(gv, rv, 2e-5) and _close_l2(gx, rx, 2e-5)
    assert abs(gr - rr) <= 1e-4 * abs(rr) and abs(ge - re) <= 1e-4 * abs(re)


@pytest.mark.gpu
def test_gpu_adjoint_larger_scene(need_gpu, pbd, scenes, adj):
    """1,440 particles with random velocities: FP32 and FP64 trajectories drift apart quickly
    here (5e-4 by frame 12), so the comparison stays at 5 frames (3 checkpoint segments)"""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(12, 10, 12), box=20, iterations=4, seed=7)
    C = adj.Consts(prm)
    frames = 5
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), frames, w)
    sim, _, _, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, frames, 2)
    assert _close_l2(gv, rv) and _close_l2(gx, rx)
    assert abs(gr - rr) <= 0.02 * abs(rr) and abs(ge - re) <= 0.02 * abs(re)
    # a second reverse pass on the same forward recomputes every segment: the same gradients, bit
    # for bit (the partners' terms are summed in fixed point, whatever order the atomics land in)
    fin = sim.state()
    dl = np.zeros((len(pos), 4), np.float32)
    dl[:, :3] = w[fin["ids"]]
    gv2, gx2, gr2, ge2 = sim.adjoint_backward(dl)
    assert np.array_equal(gv2[:, :3], gv) and np.array_equal(gx2[:, :3], gx)
    assert gr2 == gr and ge2 == ge


@pytest.mark.gpu
@pytest.mark.parametrize("solids,vorticity", [(False, 0.0), (True, 0.0), (False, 0.01)])
def test_gpu_step_after_backward_is_unchanged(need_gpu, pbd, scenes, solids, vorticity):
    """the reverse pass recomputes earlier segments (re-ordering the state and, with solids, the
    inverse masses; with vorticity, from each segment's force) and puts everything back: later
    frames are bit-identical to a plain run"""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(10, 10, 10), box=18, vorticity=vorticity)
    if solids:
        vel, m = with_solids(pos, vel)
        a = pbd.Sim(prm, len(pos)); a.add_particles_mass(pos, vel, m)
        b = pbd.Sim(prm, len(pos)); b.add_particles_mass(pos, vel, m)
    else:
        a = pbd.Sim(prm, len(pos)); a.add_particles(pos, vel)
        b = pbd.Sim(prm, len(pos)); b.add_particles(pos, vel)
    a.adjoint_forward(6, 4)
    b.step(6)
    dl = np.ones((len(pos), 4), np.float32)
    a.adjoint_backward(dl)
    a.step(3)
    b.step(3)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "ids"):
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.gpu
def test_gpu_adjoint_rejects_unsupported(need_gpu, pbd, scenes):
    prm, pos, vel, _ = adjoint_scene(pbd, scenes)
    sim = pbd.Sim(prm, len(pos))
    sim.add_particles(pos, vel)
    with pytest.raises(pbd.PBDError) as e:
        sim.adjoint_backward(np.zeros((len(pos), 4), np.float32))
    assert e.value.code == pbd.ERR_INVALID_ARG
    # a frame between the forward and the reverse pass invalidates the tape
    sim.adjoint_forward(2, 1)
    sim.step(1)
    with pytest.raises(pbd.PBDError) as e:
        sim.adjoint_backward(np.zeros((len(pos), 4), np.float32))
    assert e.value.code == pbd.ERR_INVALID_ARG
    p2 = pbd.Params.from_buffer_copy(prm)
    p2.e_vorticity = 0.01
    p2.active |= pbd.ACTIVE["computeVorticity"]          # without computeOmegas: a stale omega
    p2.active &= ~pbd.ACTIVE["computeOmegas"]
    sim.set_params(p2)
    with pytest.raises(pbd.PBDError) as e:
        sim.adjoint_forward(2, 1)
    assert e.value.code == pbd.ERR_UNSUPPORTED


@pytest.mark.gpu
def test_gpu_adjoint_through_torch_autograd(need_gpu, pbd, scenes, adj):
    """mean squared distance to a seeded target, differentiated by torch through the shim"""
    import torch
    from adjoint_autograd import rollout
    prm, pos, vel, _ = adjoint_scene(pbd, scenes, shape=(8, 8, 8), box=16, seed=9)
    rng = np.random.default_rng(9)
    target = rng.uniform(2.0, 14.0, size=(len(pos), 3))
    sim = pbd.Sim(prm, len(pos))
    v0 = torch.tensor(vel[:, :3], requires_grad=True)
    rho0 = torch.tensor(float(prm.rest_density), dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(float(prm.lambda_epsilon), dtype=torch.float64, requires_grad=True)
    x = rollout(sim, pos, v0, rho0, eps, FRAMES, 4)
    loss = ((x.double() - torch.from_numpy(target)) ** 2).sum(dim=1).mean()
    loss.backward()
    C = adj.Consts(prm)
    x0, vv0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    xf, _ = adj.rollout(C, x0, vv0, FRAMES)
    w = 2.0 * (xf - target) / len(pos)
    rv, _, rr, re = adj.backward(C, x0, vv0, FRAMES, w)
    assert _close(v0.grad.numpy(), rv)
    assert abs(float(rho0.grad) - rr) <= 0.02 * abs(rr)
    assert abs(float(eps.grad) - re) <= 0.02 * abs(re)


@pytest.mark.gpu
def test_gpu_adjoint_is_reproducible(need_gpu, pbd, scenes):
    """two simulations built from the same inputs give bit-identical gradients over a horizon
    long enough for float atomics in varying order to have made them differ"""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(12, 10, 12), box=20, iterations=4, seed=7)
    runs = [_gpu_grads(pbd, prm, pos, vel, w, 30, 10)[3:] for _ in range(2)]
    (gv1, gx1, gr1, ge1), (gv2, gx2, gr2, ge2) = runs
    assert np.array_equal(gv1, gv2) and np.array_equal(gx1, gx2)
    assert gr1 == gr2 and ge1 == ge2


def _workload_grads(pbd, scenes, adj, frames, every):
    """The differentiable dam break at its stated size (65,536 particles, 4 iterations, the loss
    mean |x_F - target|^2): the GPU gradients for the FP64 trajectory's dL/dx_F, and the FP64
    reverse pass's, with dL/dv0 along a seeded direction."""
    pos, vel, target = scenes.adjoint_dam_break()
    prm = scenes.workload_params(pbd, 72, 1000.0)
    prm.lambda_epsilon = 0.1
    prm.flags &= ~pbd.FLAG_CELL_END_QUIRK
    prm.flags |= pbd.FLAG_TRACK_IDS
    n = len(pos)
    C = adj.Consts(prm)
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    xF, _ = adj.rollout(C, x0, v0, frames)
    w = 2.0 * (xF - target) / n
    rv, rx, rr, re = adj.backward(C, x0, v0, frames, w)
    _, _, _, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, frames, every)
    dirn = np.random.default_rng(5).normal(size=(n, 3))
    return (gv, gx, gr, ge, float(np.sum(gv * dirn))), (rv, rx, rr, re, float(np.sum(rv * dirn)))


@pytest.mark.gpu
def test_gpu_adjoint_at_the_workload_size_one_frame(need_gpu, pbd, scenes, adj):
    """One frame of the workload: dL/drest_density and dL/deps within 1e-4 of the FP64 reverse
    pass (measured 1.4e-5).  The loss is averaged over 65,536 particles, so the partners' terms
    are ~1e-7..1e-5: with a fixed 2^-32 fixed-point resolution for the scattered terms dL/deps
    was 3.2e-3 off here.  dL/dv0 within 1% (measured 1.6e-3): on this unit lattice many pairs sit
    at the contact distance, and the FP64 reverse pass's own dL/dv0 moves by 3.6e-3 when its
    positions are rounded to FP32 after every iteration."""
    (gv, gx, gr, ge, gd), (rv, rx, rr, re, rd) = _workload_grads(pbd, scenes, adj, 1, 1)
    assert abs(gr - rr) <= 1e-4 * abs(rr) and abs(ge - re) <= 1e-4 * abs(re), (gr, rr, ge, re)
    assert abs(gd - rd) <= 1e-2 * abs(rd), (gd, rd)
    assert _close_l2(gv, rv, 2e-3) and _close_l2(gx, rx, 2e-3)


@pytest.mark.gpu
def test_gpu_adjoint_at_the_workload_size(need_gpu, pbd, scenes, adj):
    """The workload over 10 frames (checkpoints every 5), against the FP64 reverse pass on the
    FP64 trajectory: the rest-density and eps gradients within 1e-3 (measured 3.7e-4), dL/dv0
    along a seeded direction and as a whole within 2% (the GPU differentiates its own FP32
    trajectory, which has left the FP64 one by up to ~4e-4 cells by frame 10)."""
    (gv, gx, gr, ge, gd), (rv, rx, rr, re, rd) = _workload_grads(pbd, scenes, adj, 10, 5)
    assert abs(gd - rd) <= 0.02 * abs(rd), (gd, rd)
    assert _close_l2(gv, rv, 0.02)
    assert abs(gr - rr) <= 1e-3 * abs(rr) and abs(ge - re) <= 1e-3 * abs(re), (gr, rr, ge, re)


@pytest.mark.gpu
def test_gpu_adjoint_scales_with_the_loss(need_gpu, pbd, scenes):
    """The scattered terms' fixed point is scaled per frame by the entering gradient's binary
    exponent, so a loss gradient scaled by 2^-40 or 2^+20 gives gradients scaled by exactly that
    power of two (the same integers in the fixed point), and nothing underflows or saturates."""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(12, 10, 12), box=20, iterations=4, seed=7)
    sim = pbd.Sim(prm, len(pos))
    sim.add_particles(pos, vel)
    sim.adjoint_forward(6, 3)
    fin = sim.state()
    dl = np.zeros((len(pos), 4), np.float32)
    dl[:, :3] = w[fin["ids"]]
    gv, gx, gr, ge = sim.adjoint_backward(dl)
    assert np.any(gv[:, :3] != 0) and gr != 0 and ge != 0
    for k in (-40, 20):
        f = np.float32(2.0 ** k)
        gv2, gx2, gr2, ge2 = sim.adjoint_backward(dl * f)
        assert np.array_equal(gv2, gv * f) and np.array_equal(gx2, gx * f), k
        assert gr2 == gr * 2.0 ** k and ge2 == ge * 2.0 ** k, k
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("viscosity,solids", [(0.0, False), (0.01, True)])
def test_gpu_adjoint_vorticity_two_frames(need_gpu, pbd, scenes, adj, viscosity, solids):
    """Vorticity confinement's force acts in the next frame, so two frames are the shortest
    rollout it changes.  With e = 0.01 (20x the fluid workload's) it moves dL/dv0 by 4.3e-4
    (8e-4 with solids and viscosity); the FP32 reverse pass is within 2e-5 (9e-5) of the FP64
    one.  Stronger vorticity makes the gradient stiff (its force's direction sums
    1/(p_j - p_i + 1e-8)): at e = 0.3 the FP32 and FP64 trajectories' forces differ by 9e-4 after
    one frame and the GPU gradient departs from the FP64 one by ~1%."""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(12, 10, 12), box=20, iterations=4, seed=7,
                                     viscosity=viscosity, vorticity=0.01)
    m = None
    if solids:
        vel, m = with_solids(pos, vel, seed=7)
    C = adj.Consts(prm, m)
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    rv, rx, rr, re = adj.backward(C, x0, v0, 2, w)
    # the vorticity force matters: the gradients differ from those of the same rollout without it
    C0 = adj.Consts(prm, m)
    C0.evort = 0.0
    rv0 = adj.backward(C0, x0, v0, 2, w)[0]
    assert not _close_l2(rv0, rv, 3e-4)
    _, _, _, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, 2, 1, m)
    assert _close_l2(gv, rv, 2.5e-4) and _close_l2(gx, rx, 2.5e-4)
    assert abs(gr - rr) <= 5e-4 * abs(rr) and abs(ge - re) <= 5e-4 * abs(re)


@pytest.mark.gpu
@pytest.mark.parametrize("solids", [False, True])
def test_gpu_adjoint_segments_agree(need_gpu, pbd, scenes, solids):
    """Recomputing a segment from its checkpoint (x, v, the inverse masses and the force the next
    frame applies) gives the forward's own tape, bit for bit: gradients through 6 frames of
    vorticity and viscosity are the same with one segment and with segments of 1 and 2 frames."""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, shape=(10, 10, 10), box=18, viscosity=0.01, vorticity=0.01)
    m = None
    if solids:
        vel, m = with_solids(pos, vel)
    runs = [_gpu_grads(pbd, prm, pos, vel, w, 6, every, m)[3:] for every in (6, 2, 1)]
    gv0, gx0, gr0, ge0 = runs[0]
    for gv, gx, gr, ge in runs[1:]:
        assert np.array_equal(gv, gv0) and np.array_equal(gx, gx0)
        assert gr == gr0 and ge == ge0


@pytest.mark.parametrize("stab,frames", [(0, 4), (2, FRAMES), (3, FRAMES)])
def test_restatement_stabilization_passes(pbd, scenes, oracle_mod, adj, stab, frames):
    """stabilizationIterations S: solveCollisions S times per iteration, each on the positions the
    pass before left, the density correction applied after the last (S = 0: no contacts).  The
    FP64 restatement follows the C oracle's FP64 trajectory and its reverse pass matches central
    differences (without contacts the dam break's particles pass through one another and the
    gradients grow fast, hence 4 frames there)."""
    prm, pos, vel, w = adjoint_scene(pbd, scenes, viscosity=0.01)
    prm.stabilization_iterations = stab
    C = adj.Consts(prm)
    o = oracle_mod.Oracle(prm, len(pos), "f64")
    o.add_particles(pos, vel)
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    x, v, f = x0, v0, None
    for _ in range(frames):
        o.step(1)
        x, v, f = adj.frame(C, x, v, f)
    s = o.state()
    order = np.argsort(s["ids"])
    assert maxdiff(s["x"][order, :3], x) < 1e-8 and maxdiff(s["v"][order, :3], v) < 1e-6
    gv, gx, gr, ge = adj.backward(C, x0, v0, frames, w)
    loss = lambda c, xx, vv: float(np.sum(w * adj.rollout(c, xx, vv, frames)[0]))
    dirn = np.random.default_rng(11).normal(size=x0.shape)
    h = 1e-7
    fd_v = (loss(C, x0, v0 + h * dirn) - loss(C, x0, v0 - h * dirn)) / (2 * h)
    fd_x = (loss(C, x0 + h * dirn, v0) - loss(C, x0 - h * dirn, v0)) / (2 * h)
    assert abs(fd_v - np.sum(gv * dirn)) <= 1e-4 * abs(fd_v), (fd_v, np.sum(gv * dirn))
    assert abs(fd_x - np.sum(gx * dirn)) <= 1e-4 * abs(fd_x), (fd_x, np.sum(gx * dirn))
    for attr, g in (("rho0", gr), ("eps", ge)):
        base = getattr(C, attr)
        hh = 1e-7 * base
        cp, cm = copy.copy(C), copy.copy(C)
        setattr(cp, attr, base + hh)
        setattr(cm, attr, base - hh)
        fd = (loss(cp, x0, v0) - loss(cm, x0, v0)) / (2 * hh)
        assert abs(fd - g) <= 1e-4 * abs(fd), (attr, fd, g)


def calm_scene(pbd, scenes, stab):
    """A tight lattice (spacing 0.9, jitter 0.01) with slow random velocities (sigma 0.1): every
    touching pair overlaps by ~0.1 and no pair comes near the contact distance within a few
    frames, so no contact switches on or off between the FP32 and FP64 trajectories.  With the
    wider jitter and faster particles of adjoint_scene, the FP64 gradients themselves move by
    1e-3 to 2e-1 when the initial positions move by 1e-5 once there are several contact passes;
    here by at most 7e-4 over 2 frames."""
    prm = scenes.workload_params(pbd, 20, 1000.0, iterations=4, viscosity=0.01)
    prm.lambda_epsilon = 0.1
    prm.flags &= ~pbd.FLAG_CELL_END_QUIRK
    prm.flags |= pbd.FLAG_TRACK_IDS
    prm.stabilization_iterations = stab
    pos, vel = scenes.lattice(12, 10, 12, spacing=0.9, jitter=0.01, seed=7)
    rng = np.random.default_rng(7)
    vel[:, :3] = rng.normal(0, 0.1, size=(len(vel), 3)).astype(np.float32)
    return prm, pos, vel, rng.normal(size=(len(pos), 3))


@pytest.mark.gpu
@pytest.mark.parametrize("stab,frames", [(2, 1), (2, 2), (3, 2), (0, 2)])
def test_gpu_adjoint_stabilization_passes(need_gpu, pbd, scenes, adj, stab, frames):
    """stabilizationIterations 0, 2 and 3 (the positions each later contact pass starts from are
    taped; the density correction's terms take the iteration's final gradient) against the FP64
    reverse pass on a well-conditioned scene, within 2e-3"""
    prm, pos, vel, w = calm_scene(pbd, scenes, stab)
    C = adj.Consts(prm)
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), frames, w)
    _, fin, after, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, frames, 1)
    assert _close_l2(gv, rv, 2e-3) and _close_l2(gx, rx, 2e-3)
    assert abs(gr - rr) <= 2e-3 * abs(rr) and abs(ge - re) <= 2e-3 * abs(re), (gr, rr, ge, re)
    for k in ("x", "v", "p", "ids"):
        assert np.array_equal(fin[k], after[k]), k


def walled_scene(pbd, scenes, damping=0.5):
    """The adjoint scene started against the low walls (origin 1.6, walls at 1.5) with
    enclosurePositionDamping: particles are clamped on some axis in most frames, and a clamped
    particle's x is pulled toward its clamped position (Forces.h:56-58)."""
    prm = scenes.workload_params(pbd, 14, 1000.0, iterations=3, viscosity=0.01)
    prm.lambda_epsilon = 0.1
    prm.flags &= ~pbd.FLAG_CELL_END_QUIRK
    prm.flags |= pbd.FLAG_TRACK_IDS
    prm.enclosure_position_damping = damping
    pos, vel = scenes.lattice(7, 7, 7, spacing=0.75, origin=(1.6, 1.6, 1.6), seed=5)
    rng = np.random.default_rng(5)
    vel[:, :3] = rng.normal(0, 1.0, size=(len(vel), 3)).astype(np.float32)
    return prm, pos, vel, rng.normal(size=(len(pos), 3))


def test_restatement_position_damping(pbd, scenes, oracle_mod, adj):
    """enclosurePositionDamping 0.5 with particles at the walls: the FP64 restatement follows the
    C oracle's FP64 trajectory and its reverse pass matches central differences"""
    prm, pos, vel, w = walled_scene(pbd, scenes)
    C = adj.Consts(prm)
    o = oracle_mod.Oracle(prm, len(pos), "f64")
    o.add_particles(pos, vel)
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    x, v, f = x0, v0, None
    clamped = 0
    for _ in range(FRAMES):
        clamped += int((~np.all(adj._predict(C, x, v, f)[1], axis=1)).sum())
        o.step(1)
        x, v, f = adj.frame(C, x, v, f)
    assert clamped > 100
    s = o.state()
    order = np.argsort(s["ids"])
    assert maxdiff(s["x"][order, :3], x) < 1e-8 and maxdiff(s["v"][order, :3], v) < 1e-6
    gv, gx, gr, ge = adj.backward(C, x0, v0, FRAMES, w)
    dirn = np.random.default_rng(11).normal(size=x0.shape)
    h = 1e-7
    fd_v = (_loss(adj, C, x0, v0 + h * dirn, w) - _loss(adj, C, x0, v0 - h * dirn, w)) / (2 * h)
    fd_x = (_loss(adj, C, x0 + h * dirn, v0, w) - _loss(adj, C, x0 - h * dirn, v0, w)) / (2 * h)
    assert abs(fd_v - np.sum(gv * dirn)) <= 1e-5 * abs(fd_v)
    assert abs(fd_x - np.sum(gx * dirn)) <= 1e-5 * abs(fd_x)


@pytest.mark.gpu
@pytest.mark.parametrize("frames,tol,tol_scalar", [(1, 1e-4, 3e-4), (4, 0.02, 0.02)])
def test_gpu_adjoint_position_damping(need_gpu, pbd, scenes, adj, frames, tol, tol_scalar):
    """against the FP64 reverse pass (one frame: the scalars' sums over the wall particles, whose
    clamped coordinate bmin + 0.001 rounds differently in FP32, agree to 1.3e-4)"""
    prm, pos, vel, w = walled_scene(pbd, scenes)
    C = adj.Consts(prm)
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), frames, w)
    _, _, _, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, frames, 2)
    assert _close_l2(gv, rv, tol) and _close_l2(gx, rx, tol)
    assert abs(gr - rr) <= tol_scalar * abs(rr) and abs(ge - re) <= tol_scalar * abs(re), (gr, rr, ge, re)


def test_restatement_everything_at_once(pbd, scenes, oracle_mod, adj):
    """Solids, vorticity, XSPH viscosity, two stabilization passes and wall damping together
    (particles started against the walls): the FP64 restatement follows the C oracle and its
    reverse pass matches central differences for v0, x0, the rest density and eps"""
    prm, pos, vel, w = walled_scene(pbd, scenes)
    prm.e_vorticity = 0.01
    prm.active |= pbd.ACTIVE["computeOmegas"] | pbd.ACTIVE["computeVorticity"]
    prm.stabilization_iterations = 2
    vel, m = with_solids(pos, vel)
    C = adj.Consts(prm, m)
    o = oracle_mod.Oracle(prm, len(pos), "f64")
    o.add_particles_mass(pos, vel, m)
    frames = 4
    x0, v0 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    x, v, f = x0, v0, None
    for _ in range(frames):
        o.step(1)
        x, v, f = adj.frame(C, x, v, f)
    s = o.state()
    order = np.argsort(s["ids"])
    assert maxdiff(s["x"][order, :3], x) < 1e-8 and maxdiff(s["v"][order, :3], v) < 1e-6
    gv, gx, gr, ge = adj.backward(C, x0, v0, frames, w)
    loss = lambda c, xx, vv: float(np.sum(w * adj.rollout(c, xx, vv, frames)[0]))
    dirn = np.random.default_rng(11).normal(size=x0.shape)
    h = 1e-7
    fd_v = (loss(C, x0, v0 + h * dirn) - loss(C, x0, v0 - h * dirn)) / (2 * h)
    fd_x = (loss(C, x0 + h * dirn, v0) - loss(C, x0 - h * dirn, v0)) / (2 * h)
    assert abs(fd_v - np.sum(gv * dirn)) <= 1e-4 * abs(fd_v), (fd_v, np.sum(gv * dirn))
    assert abs(fd_x - np.sum(gx * dirn)) <= 1e-4 * abs(fd_x), (fd_x, np.sum(gx * dirn))
    for attr, g in (("rho0", gr), ("eps", ge)):
        base = getattr(C, attr)
        hh = 1e-7 * base
        cp, cm = copy.copy(C), copy.copy(C)
        setattr(cp, attr, base + hh)
        setattr(cm, attr, base - hh)
        fd = (loss(cp, x0, v0) - loss(cm, x0, v0)) / (2 * hh)
        assert abs(fd - g) <= 1e-4 * abs(fd), (attr, fd, g)


@pytest.mark.gpu
def test_gpu_adjoint_everything_at_once(need_gpu, pbd, scenes, adj):
    """Solids, vorticity, XSPH viscosity and two stabilization passes together over two frames
    (the vorticity force acts in the second) against the FP64 reverse pass, on the calm scene
    (there the FP64 gradients move by at most 4e-3 when the initial positions move by 1e-5)"""
    prm, pos, vel, w = calm_scene(pbd, scenes, 2)
    prm.enclosure_position_damping = 0.5
    prm.e_vorticity = 0.01
    prm.active |= pbd.ACTIVE["computeOmegas"] | pbd.ACTIVE["computeVorticity"]
    vel, m = with_solids(pos, vel)
    C = adj.Consts(prm, m)
    rv, rx, rr, re = adj.backward(C, pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), 2, w)
    _, fin, after, gv, gx, gr, ge = _gpu_grads(pbd, prm, pos, vel, w, 2, 1, m)
    assert _close_l2(gv, rv, 1e-2) and _close_l2(gx, rx, 1e-2)
    assert abs(gr - rr) <= 1e-2 * abs(rr) and abs(ge - re) <= 1e-2 * abs(re), (gr, rr, ge, re)
    for k in ("x", "v", "p", "ids"):
        assert np.array_equal(fin[k], after[k]), k
