"""torch.autograd.Function wrapper: displacement u(E) of an elasticity formulation as a
differentiable function of the per-element Young's moduli.

forward  -- assemble + solve on the GPU through the C ABI (the formulation's own solver);
backward -- the hand-written adjoint: K lambda = dL/du solved with the same solver, then
            dL/dE_e = -lambda_e^T (K_e / E_e) u_e from the recomputed element operator.
The penalty scale of the constraints is held at its value of the first solve, so the gradient
is that of u(E) with fixed constraint stiffness.
"""
import numpy as np
import torch


class ElasticDisplacement(torch.autograd.Function):
    @staticmethod
    def forward(ctx, E, formulation, mode="mixed", tol=1e-10):
        f = formulation
        f.elastic_modulus = E.detach().to("cpu", torch.float64).numpy()
        f.set_result(np.zeros(f.n))
        f.solve(tol, mode=mode)
        if f.get_penalty_scale() > 0:
            f.set_penalty_scale(f.get_penalty_scale())
        ctx.f, ctx.mode, ctx.tol = f, mode, tol
        u = torch.from_numpy(f.get_result()).to(device=E.device)
        return u.to(E.dtype)

    @staticmethod
    def backward(ctx, grad_u):
        c = grad_u.detach().to("cpu", torch.float64).contiguous().numpy()
        _, g, _ = ctx.f.adjoint_grad("linear", target=c, mode=ctx.mode, tol=ctx.tol)
        return torch.from_numpy(g).to(device=grad_u.device, dtype=grad_u.dtype), None, None, None


def elastic_displacement(E, formulation, mode="mixed", tol=1e-10):
    """u = K(E)^-1 F, differentiable in E (a tensor with one modulus per element)."""
    return ElasticDisplacement.apply(E, formulation, mode, tol)
