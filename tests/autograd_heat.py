"""torch.autograd.Function around the hand-written heat adjoint (test harness only).

HeatLoss.apply(T0, lam, Ttarget, steps, dt) returns J = 1/2 sum_interior (T_N - T_target)^2 for
T_N = steps FP64 heat steps (nebo_heat_run) and back-propagates dJ/dT0, dJ/dlambda from
nebo_heat_gradient (sqrt(N) checkpointing).  Tensors are ghosted SVol windows (gz, gy, gx) with
one ghost layer; the ghost entries are periodic images of the interior, so the gradients returned
for them are zero (perturbing a ghost entry alone is not a periodic perturbation)."""
import torch

import spatialops_gb300 as N


def _field(t):
    gz, gy, gx = t.shape
    return N.Field("SVol", (gx - 2, gy - 2, gz - 2), 1, tensor=t.detach().contiguous().clone())


class HeatLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, T0, lam, Ttarget, steps, dt):
        L = _field(lam)
        N.fill_periodic(L)  # lambda's ghosts are read at boundary faces: periodic images
        J, gT, gl = N.heat_gradient(_field(T0), L, _field(Ttarget), int(steps), float(dt))
        gT, gl = gT.tensor.clone(), gl.tensor.clone()
        for g in (gT, gl):
            g[0], g[-1], g[:, 0], g[:, -1], g[:, :, 0], g[:, :, -1] = 0, 0, 0, 0, 0, 0
        ctx.save_for_backward(gT, gl)
        return torch.tensor(J, dtype=torch.float64, device=T0.device)

    @staticmethod
    def backward(ctx, gout):
        gT, gl = ctx.saved_tensors
        return gout * gT, gout * gl, None, None, None
