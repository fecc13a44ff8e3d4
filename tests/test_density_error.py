"""pbd_density_error against the oracle's density constraint (orc_density_error): C_i = rho_i /
rest_density - 1 over the last frame's list at the current positions (FP32 sums in list order on
both sides, positions within the step's parity tolerance).  Tolerances: 1e-6 absolute on C in the
workloads' regime (C ~ -1), 1e-3 of the largest density on rho_i where C is of order one."""
import numpy as np
import pytest

from helpers import setup_pair, workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("frames,solve", [(1, True), (6, True), (4, False)])
def test_density_error_matches_oracle(need_gpu, pbd, scenes, oracle_mod, frames, solve):
    # spacing 0.8: every particle has neighbours inside the kernel radius.  With the density
    # solve on, rest density 1000 keeps the workloads' regime (C close to -1, compared through
    # rho); with it off, a rest density of the lattice's own order makes C of order one.
    rho0 = 1000.0 if solve else 0.02
    params, _, _ = workload(pbd, scenes, box=24, rho0=rho0, eps=0.1, flags_extra=pbd.FLAG_TRACK_IDS)
    if not solve:
        for k in ("computeLambda", "computeDeltaPositions", "applyDeltaPositions"):
            params.active &= ~pbd.ACTIVE[k]
    pos, vel = scenes.lattice(14, 12, 14, spacing=0.8, seed=6)
    sim, orc = setup_pair(pbd, oracle_mod, params, pos, vel)
    sim.step(frames)
    orc.step(frames)
    err, mean, mx = sim.density_error()
    st = sim.state()
    ref = orc.density_error()
    ost = orc.state()
    g = np.empty(len(err)); g[st["ids"]] = err
    o = np.empty(len(ref)); o[ost["ids"]] = ref
    if solve:   # C + 1 = rho / 1000 is ~1e-5: compare the FP32 C itself
        assert np.max(np.abs(g - o)) <= 1e-6
    else:
        rho_g, rho_o = (g + 1.0) * rho0, (o + 1.0) * rho0
        assert np.max(np.abs(rho_g - rho_o)) <= 1e-3 * np.max(np.abs(rho_o))
        assert np.max(np.abs(o)) > 0.1          # the check sees a non-trivial constraint
    assert abs(mean - np.mean(np.abs(err))) <= 1e-6 * max(1.0, mean)
    assert mx == pytest.approx(float(np.max(np.abs(err))), rel=1e-6)


def test_density_error_needs_a_frame(need_gpu, pbd, scenes):
    params, pos, vel = workload(pbd, scenes)
    sim = pbd.Sim(params, len(pos))
    sim.add_particles(pos, vel)
    with pytest.raises(pbd.PBDError) as e:
        sim.density_error()
    assert e.value.code == pbd.ERR_INVALID_ARG
    sim.step(1)
    _, mean, mx = sim.density_error()
    assert 0.0 <= mean <= mx
