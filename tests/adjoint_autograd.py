"""torch.autograd.Function over the C ABI's adjoint (a test-harness shim, not part of the library).

`rollout(sim, pos, v0, rest_density, eps, frames, every)` runs pbd_adjoint_forward from the state
(pos, v0) and returns the final positions in particle-id order as an (n, 3) float32 tensor;
its backward hands dL/dx_final to pbd_adjoint_backward and returns dL/dv0, dL/drest_density and
dL/deps.  The simulation handle must track ids (PBD_FLAG_TRACK_IDS)."""
import numpy as np
import torch


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0, rest_density, eps, sim, pos, frames, every):
        prm = sim.params()
        prm.rest_density = float(rest_density)
        prm.lambda_epsilon = float(eps)
        sim.set_params(prm)
        sim.clear()
        vel = np.zeros((len(pos), 4), np.float32)
        vel[:, :3] = v0.detach().cpu().numpy()
        sim.add_particles(pos, vel)
        sim.adjoint_forward(frames, every)
        st = sim.state()
        ctx.sim, ctx.ids = sim, st["ids"].astype(np.int64)
        x = np.zeros((len(pos), 3), np.float32)
        x[ctx.ids] = st["x"][:, :3]
        return torch.from_numpy(x)

    @staticmethod
    def backward(ctx, gx):
        g = np.zeros((len(ctx.ids), 4), np.float32)
        g[:, :3] = gx.detach().cpu().numpy()[ctx.ids]
        gv, _, gr, ge = ctx.sim.adjoint_backward(g)
        return (torch.from_numpy(gv[:, :3].copy()), torch.tensor(gr, dtype=torch.float64),
                torch.tensor(ge, dtype=torch.float64), None, None, None, None)


def rollout(sim, pos, v0, rest_density, eps, frames, every):
    return _Rollout.apply(v0, rest_density, eps, sim, pos, frames, every)
