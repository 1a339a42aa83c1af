"""torch.autograd wrapper of the GPU PBF rollout and its hand-written adjoint.

``rollout(sim, x0, v0, rho0, steps, dt)`` runs ``steps`` GPU steps (pbf_step on the
simulator's handle) and returns the final positions and velocities. Its backward
walks the steps in reverse: the state (x_t, v_t) entering every step is kept as a
checkpoint during the forward ((steps, n, 3) float32 each, on the device), and the
backward of step t calls ``pbf_adjoint_step_device``, which recomputes that step from
its checkpoint -- prediction, neighbour search, the Jacobi iterations -- and applies
its reverse mode with the step's neighbour sets fixed. Gradients flow to the initial
positions, the initial velocities and the rest density.

The reference (src/particles.cpp) has no gradients; the step differentiated here is
Particles::timeStep (particles.cpp:250-297) in the form of the GPU kernels.

The rest density is a parameter of the simulator's handle: ``rho0`` must hold the
value the simulator was created with (it is the handle to the gradient, not a
setting). The simulator's state after the backward is the output of step 0.
"""
from __future__ import annotations

import torch

from .pbf import Simulator


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class PbfRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sim: Simulator, x0: torch.Tensor, v0: torch.Tensor, rho0: torch.Tensor, steps: int,
                dt: float):
        n = sim.n
        if x0.shape != (n, 3) or v0.shape != (n, 3):
            raise ValueError(f"x0 / v0 must be ({n}, 3)")
        if x0.dtype != torch.float32 or v0.dtype != torch.float32 or not x0.is_cuda or not v0.is_cuda:
            raise ValueError("x0 / v0 must be float32 CUDA tensors")
        r = float(rho0.detach().cpu())
        if abs(r - sim.params.rest_density) > 1e-6 * abs(sim.params.rest_density):
            raise ValueError(f"rho0 = {r} is not the simulator's rest density {sim.params.rest_density}")
        x0 = x0.contiguous()
        v0 = v0.contiguous()
        s = _stream()
        ckx = torch.empty((steps, n, 3), dtype=torch.float32, device=x0.device)
        ckv = torch.empty_like(ckx)
        sim.set_state_device(x0.data_ptr(), v0.data_ptr(), s)
        for t in range(steps):
            sim.get_state_device(ckx[t].data_ptr(), ckv[t].data_ptr(), None, s)
            sim.step_async(dt, 1)
        xT = torch.empty_like(x0)
        vT = torch.empty_like(v0)
        sim.get_state_device(xT.data_ptr(), vT.data_ptr(), None, s)
        sim.sync()
        ctx.sim = sim
        ctx.dt = dt
        ctx.steps = steps
        ctx.rho0_dtype = rho0.dtype
        ctx.save_for_backward(ckx, ckv)
        return xT, vT

    @staticmethod
    def backward(ctx, gxT, gvT):
        ckx, ckv = ctx.saved_tensors
        sim: Simulator = ctx.sim
        s = _stream()
        gx = torch.zeros_like(ckx[0]) if gxT is None else gxT.contiguous().to(torch.float32)
        gv = torch.zeros_like(ckx[0]) if gvT is None else gvT.contiguous().to(torch.float32)
        parts = torch.zeros(max(ctx.steps, 1), dtype=torch.float64, device=ckx.device)
        for t in range(ctx.steps - 1, -1, -1):
            gx_in = torch.empty_like(gx)
            gv_in = torch.empty_like(gv)
            sim.adjoint_step_device(ctx.dt, ckx[t].data_ptr(), ckv[t].data_ptr(), gx.data_ptr(), gv.data_ptr(),
                                    gx_in.data_ptr(), gv_in.data_ptr(), parts[t].data_ptr(), stream=s)
            gx, gv = gx_in, gv_in
        sim.sync()
        g_rho0 = parts.sum().to(ctx.rho0_dtype)
        return None, gx, gv, g_rho0, None, None


def rollout(sim: Simulator, x0: torch.Tensor, v0: torch.Tensor, rho0: torch.Tensor, steps: int,
            dt: float | None = None):
    """``steps`` GPU steps from (x0, v0); differentiable in x0, v0 and rho0."""
    return PbfRollout.apply(sim, x0, v0, rho0, steps, sim.params.dt if dt is None else dt)
