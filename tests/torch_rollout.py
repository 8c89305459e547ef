"""torch.autograd.Function around the library's checkpointed rollout (tests only).

forward(x0, v0) loads the particle state into a FluidSimulation handle and runs k
differentiable substeps on the GPU; backward maps (dL/dx_k, dL/dv_k) to (dL/dx0, dL/dv0)
through FluidSimulation_gb300_rollout_adjoint.  Tensors are CPU float32 (N, 3); the C ABI
takes host buffers."""
import numpy as np
import torch


class FlipRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, sim, k, dt):
        x = np.ascontiguousarray(x0.detach().cpu().numpy(), np.float32)
        v = np.ascontiguousarray(v0.detach().cpu().numpy(), np.float32)
        sim.set_marker_particle_data(x.shape[0], x.tobytes(), v.tobytes())
        sim.rollout_forward(k, dt)
        xk = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3).copy()
        vk = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3).copy()
        ctx.sim = sim
        return torch.from_numpy(xk), torch.from_numpy(vk)

    @staticmethod
    def backward(ctx, gxk, gvk):
        gx = None if gxk is None else gxk.detach().cpu().numpy()
        gv = gvk.detach().cpu().numpy() if gvk is not None else np.zeros((gx.shape[0], 3), np.float32)
        gx0, gv0, _ = ctx.sim.rollout_adjoint(gx, gv)
        return torch.from_numpy(gx0), torch.from_numpy(gv0), None, None, None
