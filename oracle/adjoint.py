"""FP64 NumPy restatement of the frame and of its reverse pass (test infrastructure only).

Only tests/ and bench.py's checks import this module; the shipped library never does.  It
restates, for the adjoint's supported configuration (applyForces, the density solve with
stabilizationIterations S, solveCollisions, updatePositions, XSPH viscosity, vorticity,
enclosurePositionDamping = 0, unit cell width, the cell-end quirk off), the frame that
Fluid::compute runs (src/app/simulation/Fluid.cu:14-97):

  applyForces     v* = v + g dt (y), p = x + v* dt, clamped to the walls  (kernel/Forces.h:65-101)
  lists           j is a candidate of i when their anchor cells are adjacent (27 cells,
                  kernel/Collision.h:11-66); the anchor is p right after the re-order
  computeLambda   (kernel/Density.h:48-93)
  computeDelta    (kernel/Density.h:104-145), solveCollisions (kernel/Collision.h:171-242),
  applyDelta      p <- p + c - Delta, x <- x + c (Jacobi: all reads from the iteration's snapshot)
  updatePositions v = (p - x)/dt, x = p (kernel/Update.h:11-32)
  computeOmega    omega_i = sum_j (v_j - v_i) x grad W_spiky(p_i - p_j)          (kernel/Density.h:232-269)
  vorticity       eta_i = sum_j |omega_j - omega_i| / (p_j - p_i + 1e-8), componentwise, over
                  every list entry; n = (eta + 1e-8) / (|eta| + 1e-8); f_i = e (n x omega_i),
                  the external force of the next frame's applyForces       (kernel/Density.h:179-221)
  viscosity       v <- v + c sum_j (v_j - v_i) W(|p_i - p_j|), Jacobi (kernel/Density.h:280-310)

Unified solids (per-particle inverse mass w, the library's extension of the reference's
inverseMass terms, kernel/Collision.h:223-225): a particle with w = 0 takes no gravity, its
density correction is scaled by w_i, the contact overlap is split w_i / (w_i + w_j) (1/2 each
with unit masses) and the viscosity coefficient is c w_i.

Omega, vorticity and viscosity read the positions and velocities right after updatePositions.
Particles stay in id order here (the re-order is a permutation: it changes summation order
only).  `rollout` runs frames and can keep a tape; `backward` returns dL/dv0, dL/dx0,
dL/drest_density and dL/deps for L = sum(c . x_final) and is checked against central
differences of `rollout` itself and against the C oracle's FP64 trajectory.
"""
import numpy as np

PI = 3.14159265359    # Globals.h:122


class Consts:
    def __init__(self, prm, inv_mass=None):
        d = 2.0 * prm.particle_radius
        if abs(d - 1.0) > 1e-12:
            raise ValueError("the restatement assumes a unit cell width (particle radius 0.5)")
        self.d = d
        self.dt = float(prm.delta_t)
        self.g = float(prm.gravity)
        self.rho0 = float(prm.rest_density)
        self.eps = float(prm.lambda_epsilon)
        self.hs = d * float(prm.kernel_width_spiky)
        self.hp = float(prm.kernel_width_poly)
        self.k = float(prm.k_scorr)
        self.n = int(prm.n_scorr)
        self.ac = 0.5 * (1.0 - float(prm.stiffness))
        self.bmin = np.array([prm.bounds_min[a] for a in range(3)], np.float64)
        self.bmax = np.array([prm.bounds_max[a] for a in range(3)], np.float64)
        self.pd = float(prm.enclosure_position_damping)
        self.iters = int(prm.solver_iterations)
        self.M = int(prm.max_neighbours_per_particle)
        # solveCollisions runs S times per iteration (Fluid.cu:60-65), each on the positions the
        # pass before left; the density correction is applied after the last
        self.stab = int(prm.stabilization_iterations)
        self.collide = prm.collision_type == 0 and self.stab > 0
        self.poly_inv_den = 1.0 / (0.001 + 64.0 * PI * self.hp ** 9)
        self.spiky_k = 15.0 / (PI * self.hs ** 6)
        q = self.hs * float(prm.q_scorr)
        self.wq = self.poly6(np.array([q]))[0][0]
        c = max(self.hp, self.hs, d)
        self.cut2 = c * c * 1.0001
        # XSPH viscosity (Density.h:280-310, Jacobi) after updatePositions, when active
        self.cvisc = float(prm.c_viscosity) if (prm.active & (1 << 9)) else 0.0
        # vorticity confinement (needs computeOmegas): its force enters the next frame's predict
        self.evort = 0.0
        if prm.active & (1 << 8):
            if not prm.active & (1 << 7):
                raise ValueError("vorticity without computeOmegas reads a stale omega")
            self.evort = float(prm.e_vorticity)
        # inverse masses in id order (None: every particle 1, the reference's)
        self.w = None if inv_mass is None else np.asarray(inv_mass, np.float64)

    def share(self, I, J):
        """Contact share of particle I in pair (I, J) times (1 - stiffness) (Collision.h:223-225)."""
        if self.w is None:
            return np.full(len(I), self.ac)
        wi, wj = self.w[I], self.w[J]
        tot = wi + wj
        return np.where(tot > 0.0, wi / np.where(tot > 0.0, tot, 1.0), 0.0) * (2.0 * self.ac)

    def poly6(self, L):
        inside = (L > 0.001) & (L < self.hp - 0.001)
        t = np.where(inside, self.hp * self.hp - L * L, 0.0)
        W = 315.0 * t ** 6 * self.poly_inv_den
        dW = -12.0 * L * 315.0 * t ** 5 * self.poly_inv_den
        return np.where(inside, W, 0.0), np.where(inside, dW, 0.0)

    def spiky(self, L):
        inside = (L > 0.0001) & (self.hs - L > 0.0001)
        a = np.where(inside, self.hs - L, 0.0)
        return self.spiky_k * a * a, -2.0 * self.spiky_k * a


def candidate_pairs(anchor, M):
    """Directed pairs (i, j), i != j, whose anchor cells are adjacent (trunc of the clamped
    position, Hash.h:21-29).  Raises if a list would reach the cap M (the cap cuts lists in
    the reference's cell order, which this restatement does not follow)."""
    cell = np.clip(anchor, 0.0, 1023.0).astype(np.int64)
    n = len(cell)
    key = (cell[:, 0] << 20) | (cell[:, 1] << 10) | cell[:, 2]
    order = np.argsort(key, kind="stable")
    skey = key[order]
    I, J = [], []
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            for c in (-1, 0, 1):
                nk = ((cell[:, 0] + a) << 20) | ((cell[:, 1] + b) << 10) | (cell[:, 2] + c)
                ok = np.all((cell + np.array([a, b, c])) >= 0, axis=1) & np.all((cell + np.array([a, b, c])) <= 1023, axis=1)
                lo = np.searchsorted(skey, nk, "left")
                hi = np.searchsorted(skey, nk, "right")
                cnt = np.where(ok, hi - lo, 0)
                ii = np.repeat(np.arange(n), cnt)
                start = np.repeat(lo - np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt)
                jj = order[start + np.arange(len(ii))]
                I.append(ii); J.append(jj)
    I = np.concatenate(I); J = np.concatenate(J)
    keep = I != J
    I, J = I[keep], J[keep]
    if n and np.bincount(I, minlength=n).max() >= M:
        raise ValueError("a neighbour list reaches the cap")
    return I, J


def _pair_geometry(C, P, I, J):
    r = P[I] - P[J]
    r2 = np.einsum("ij,ij->i", r, r)
    m = (r2 < C.cut2) & (r2 > 0.0)
    I, J, r, r2 = I[m], J[m], r[m], r2[m]
    L = np.sqrt(r2)
    rh = r / L[:, None]
    return I, J, r, L, rh


def _sum(I, vals, n):
    if vals.ndim == 1:
        return np.bincount(I, weights=vals, minlength=n)
    return np.stack([np.bincount(I, weights=vals[:, a], minlength=n) for a in range(vals.shape[1])], axis=1)


def _lambda(C, n, I, L, rh):
    W, dW = C.poly6(L)
    g, dg = C.spiky(L)
    rho = _sum(I, W, n)
    B = _sum(I, g * g, n)
    S = _sum(I, g[:, None] * rh, n)
    s2 = np.einsum("ij,ij->i", S, S)
    Cc = rho / C.rho0 - 1.0
    D = (B + s2) / C.rho0 + C.eps
    return -Cc / D, dict(W=W, dW=dW, g=g, dg=dg, rho=rho, B=B, S=S, s2=s2, C=Cc, D=D)


def _predict(C, x, v, f=None):
    vv = v.copy()
    moves = np.ones(len(v)) if C.w is None else (C.w != 0.0).astype(np.float64)   # solids: no gravity, no force
    vv[:, 1] += C.g * C.dt * moves
    if f is not None:
        vv += C.dt * f * moves[:, None]
    p = x + vv * C.dt
    lo, hi = p < C.bmin, p > C.bmax
    p = np.where(lo, C.bmin + 0.001, np.where(hi, C.bmax - 0.001, p))
    return p, ~(lo | hi)


def _damp(C, x, p, mask):
    """enclosurePositionDamping (Forces.h:56-58): a particle clamped on some axis has x moved
    toward its clamped p by that fraction, on every axis; returns (x', any clamp)."""
    anyc = ~np.all(mask, axis=1)
    if not C.pd:
        return x, anyc
    return np.where(anyc[:, None], x + C.pd * (p - x), x), anyc


def _omega(C, pf, vu, I0, J0):
    """omega_i = sum_j (v_j - v_i) x G_ij over the pairs within the cut (spiky is 0 beyond)."""
    n = len(pf)
    I, J, r, L, rh = _pair_geometry(C, pf, I0, J0)
    g, dg = C.spiky(L)
    G = g[:, None] * rh
    return _sum(I, np.cross(vu[J] - vu[I], G), n), (I, J, L, rh, g, dg, G)


def _eta(C, pf, om, I0, J0):
    """eta_i = sum_j |omega_j - omega_i| / (p_j - p_i + 1e-8) over every list entry."""
    n = len(pf)
    D = pf[J0] - pf[I0] + 1e-8
    u = om[J0] - om[I0]
    ol = np.sqrt(np.einsum("ij,ij->i", u, u))
    return _sum(I0, ol[:, None] / D, n), (D, u, ol)


def _vort_force(C, eta, om):
    gl = np.sqrt(np.einsum("ij,ij->i", eta, eta))
    nv = (eta + 1e-8) / (gl + 1e-8)[:, None]
    return C.evort * np.cross(nv, om), nv, gl


def frame(C, x, v, f=None, tape=None):
    """One frame on (n, 3) float64 positions and velocities with the external force f of the
    frame before (None: none); returns (x', v', f') with f' the vorticity force for the next
    frame (zeros without vorticity)."""
    n = len(x)
    p, mask = _predict(C, x, v, f)
    I0, J0 = candidate_pairs(p, C.M)
    if tape is not None:
        tape.append(dict(x=x.copy(), v=v.copy(), f=None if f is None else f.copy(), I=I0, J=J0, p=[]))
    x, _ = _damp(C, x.copy(), p, mask)
    for _ in range(C.iters):
        if tape is not None:
            tape[-1]["p"].append(p.copy())
        I, J, r, L, rh = _pair_geometry(C, p, I0, J0)
        lam, q = _lambda(C, n, I, L, rh)
        sc = -C.k * (q["W"] / C.wq) ** C.n
        coef = lam[I] + lam[J] + sc
        delta = _sum(I, (coef * q["g"])[:, None] * rh, n) / C.rho0
        if C.w is not None:
            delta = C.w[:, None] * delta
        if tape is not None:
            tape[-1].setdefault("ps", []).append([])
        for k in range(C.stab if C.collide else 0):
            if k > 0:   # a later pass: the contacts at the positions the pass before left
                if tape is not None:
                    tape[-1]["ps"][-1].append(p.copy())
                I, J, r, L, rh = _pair_geometry(C, p, I0, J0)
            ov = C.d - L
            cm = (ov > 0.0) & (L > 0.00001)
            c = _sum(I[cm], (C.share(I[cm], J[cm]) * ov[cm])[:, None] * rh[cm], n)
            p = p + c
            x = x + c
        p = p - delta
    v = (p - x) / C.dt
    if tape is not None and (C.cvisc or C.evort):
        tape[-1]["pf"], tape[-1]["vu"] = p.copy(), v.copy()
    fn = np.zeros_like(p)
    if C.evort:   # omega and the vorticity force at the final positions, from v before viscosity
        om, _ = _omega(C, p, v, I0, J0)
        eta, _ = _eta(C, p, om, I0, J0)
        fn, _, _ = _vort_force(C, eta, om)
        if tape is not None:
            tape[-1]["om"], tape[-1]["eta"] = om, eta
    if C.cvisc:   # v += c sum_j (v_j - v_i) W(|p_i - p_j|) over the frame's list, at the final positions
        I, J, r, L, rh = _pair_geometry(C, p, I0, J0)
        W, _ = C.poly6(L)
        ci = C.cvisc if C.w is None else (C.cvisc * C.w)[:, None]
        v = v + ci * _sum(I, W[:, None] * (v[J] - v[I]), n)
    return p.copy(), v, fn


def rollout(C, x, v, frames, tape=None):
    f = None
    for _ in range(frames):
        x, v, f = frame(C, x, v, f, tape)
    return x, v


def _hess_mul(g, dg, L, rh, a):
    ra = np.einsum("ij,ij->i", rh, a)
    return dg[:, None] * ra[:, None] * rh + (g / L)[:, None] * (a - ra[:, None] * rh)


def _vort_backward(C, rec, gf):
    """Reverse of omega + the vorticity force for dL/df' = gf: (dL/dp, dL/dv) at the final
    positions and the velocities before viscosity."""
    pf, vu, om, eta = rec["pf"], rec["vu"], rec["om"], rec["eta"]
    I0, J0 = rec["I"], rec["J"]
    n = len(pf)
    _, nv, gl = _vort_force(C, eta, om)
    nbar = C.evort * np.cross(om, gf)                 # f = e (n x omega)
    obar = C.evort * np.cross(gf, nv)
    ge = gl + 1e-8
    safe = np.where(gl > 0.0, gl, 1.0)
    etabar = nbar / ge[:, None] - eta * (np.einsum("ij,ij->i", eta + 1e-8, nbar) / (ge * ge * safe) * (gl > 0.0))[:, None]
    _, (D, u, ol) = _eta(C, pf, om, I0, J0)
    sq = np.einsum("ij,ij->i", etabar[I0], 1.0 / D)
    du = np.where(ol[:, None] > 0.0, (sq / np.where(ol > 0.0, ol, 1.0))[:, None] * u, 0.0)
    obar = obar + _sum(J0, du, n) - _sum(I0, du, n)
    tp = -etabar[I0] * ol[:, None] / (D * D)          # d eta_i / d p_j (componentwise)
    pbar = _sum(J0, tp, n) - _sum(I0, tp, n)
    _, (I, J, L, rh, g, dg, G) = _omega(C, pf, vu, I0, J0)
    gG = np.cross(G, obar[I])                         # (u x G) . obar = u . (G x obar)
    vbar = _sum(J, gG, n) - _sum(I, gG, n)
    rb = _hess_mul(g, dg, L, rh, np.cross(obar[I], vu[J] - vu[I]))   # dG = H dr, r = p_i - p_j
    pbar = pbar + _sum(I, rb, n) - _sum(J, rb, n)
    return pbar, vbar


def frame_backward(C, rec, gxo, gvo, acc, gf=None):
    """Reverse of `frame` for the taped record `rec`: (dL/dx', dL/dv', dL/df') ->
    (dL/dx, dL/dv, dL/df) with f the external force the frame's applyForces took."""
    n = len(gxo)
    I0, J0 = rec["I"], rec["J"]
    vbar = None
    if C.evort and gf is not None and np.any(gf):
        pbar, vbar = _vort_backward(C, rec, gf)
        gxo = gxo + pbar
    if C.cvisc:   # reverse of the viscosity: dL/dv' -> dL/dv (before it) and dL/dp (final positions)
        pf, vu = rec["pf"], rec["vu"]
        I, J, r, L, rh = _pair_geometry(C, pf, I0, J0)
        W, dW = C.poly6(L)
        c = np.full(n, C.cvisc) if C.w is None else C.cvisc * C.w
        gv_u = gvo * (1.0 - c * _sum(I, W, n))[:, None] + _sum(J, (c[I] * W)[:, None] * gvo[I], n)
        term = c[I] * np.einsum("ij,ij->i", gvo[I], vu[J] - vu[I]) * dW
        gxo = gxo + _sum(I, term[:, None] * rh, n) - _sum(J, term[:, None] * rh, n)
        gvo = gv_u
    if vbar is not None:   # omega read the velocities before the viscosity
        gvo = gvo + vbar
    gp = gxo + gvo / C.dt
    gx = -gvo / C.dt
    for it in range(C.iters - 1, -1, -1):
        # the contact passes after the first, last first: gc = dL/dp entering each (the density
        # correction, applied after the last pass, keeps the iteration's final gradient gp)
        gc = gp
        for pk in reversed(rec["ps"][it] if C.collide else []):
            I, J, r, L, rh = _pair_geometry(C, pk, I0, J0)
            cbar = (gc + gx)[I]
            ov = C.d - L
            cm = ((ov > 0.0) & (L > 0.00001)).astype(np.float64)
            rc = np.einsum("ij,ij->i", rh, cbar)
            ol = ov / L
            rb = (C.share(I, J) * cm)[:, None] * (-rc[:, None] * rh + ol[:, None] * (cbar - rc[:, None] * rh))
            gc = gc + _sum(I, rb, n) - _sum(J, rb, n)
        p = rec["p"][it]
        I, J, r, L, rh = _pair_geometry(C, p, I0, J0)
        lam, q = _lambda(C, n, I, L, rh)
        W, dW, g, dg = q["W"], q["dW"], q["g"], q["dg"]
        qq = W / C.wq
        sc = -C.k * qq ** C.n
        dsc = -C.k * C.n * qq ** (C.n - 1) * dW / C.wq if C.n != 0 else np.zeros_like(W)
        coef = lam[I] + lam[J] + sc
        G = g[:, None] * rh
        # Delta (scaled by the inverse mass) and contacts
        a = -gp / C.rho0 if C.w is None else -(C.w[:, None] * gp) / C.rho0
        gd = np.einsum("ij,ij->i", G, a[I])
        glam = _sum(I, gd, n) + _sum(J, gd, n)
        rbar = coef[:, None] * _hess_mul(g, dg, L, rh, a[I]) + (gd * dsc)[:, None] * rh
        if C.collide:
            cbar = (gc + gx)[I]
            ov = C.d - L
            cm = ((ov > 0.0) & (L > 0.00001)).astype(np.float64)
            rc = np.einsum("ij,ij->i", rh, cbar)
            ol = ov / L
            rbar += (C.share(I, J) * cm)[:, None] * (-rc[:, None] * rh + ol[:, None] * (cbar - rc[:, None] * rh))
        sdelta = _sum(I, coef[:, None] * G, n)
        wgp = gp if C.w is None else C.w[:, None] * gp
        acc[0] += float(np.sum(wgp * sdelta)) / (C.rho0 * C.rho0)
        gnew = gc + _sum(I, rbar, n) - _sum(J, rbar, n)
        # lambda
        Cbar = -glam / q["D"]
        Dbar = glam * q["C"] / q["D"] ** 2
        acc[0] += float(np.sum(Cbar * (-q["rho"] / C.rho0 ** 2) + Dbar * (-(q["B"] + q["s2"]) / C.rho0 ** 2)))
        acc[1] += float(np.sum(Dbar))
        S = q["S"]
        rbar2 = (Cbar[I] / C.rho0 * dW)[:, None] * rh + (2.0 * Dbar[I] / C.rho0)[:, None] * _hess_mul(g, dg, L, rh, G + S[I])
        gnew += _sum(I, rbar2, n) - _sum(J, rbar2, n)
        gp = gnew
    p0, mask = _predict(C, rec["x"], rec["v"], rec["f"])
    _, anyc = _damp(C, rec["x"], p0, mask)
    # p = clamp(x + v* dt); x' = x + pd any (p - x): dx'/dx = 1 - pd any + pd any mask,
    # dx'/dv* = pd any mask dt (per axis; gx is dL/dx')
    k = C.pd * anyc.astype(np.float64)[:, None]
    gx_in = mask * gp + gx * (1.0 - k + k * mask)
    gv_in = mask * (gp + k * gx) * C.dt
    moves = np.ones(n) if C.w is None else (C.w != 0.0).astype(np.float64)
    return gx_in, gv_in, gv_in * (C.dt * moves)[:, None]     # v* = v + dt (g + f): dL/df = dt dL/dv*


def backward(C, x0, v0, frames, weights):
    """Gradients of L = sum(weights . x_final) (all (n, 3)); returns (dL/dv0, dL/dx0, dL/drho0, dL/deps)."""
    tape = []
    rollout(C, np.asarray(x0, np.float64), np.asarray(v0, np.float64), frames, tape)
    gx = np.asarray(weights, np.float64).copy()
    gv = np.zeros_like(gx)
    gf = np.zeros_like(gx)      # the last frame's vorticity force acts on no frame
    acc = [0.0, 0.0]
    for rec in reversed(tape):
        gx, gv, gf = frame_backward(C, rec, gx, gv, acc, gf)
    return gv, gx, acc[0], acc[1]
