"""Differentiable misfit of the variable-coefficient Helmholtz solve (torch.autograd.Function).

J(kappa) = sum_q Jw_q (u(x_q) - u_t(x_q))^2,  A(kappa) u = b,  A(kappa) = lambda M + L_kappa.
Forward: one FP64 CG solve on the GPU. Backward: the adjoint solve A(kappa) psi = dJ/du
(A is symmetric, so it is the same solver) and the GPU gradient kernel
dJ/dkappa_q = -Jw_q grad psi . grad u. The reference has no adjoint; the operator
is its LaplacianMatrixOp_MatFree with eVarCoeffD00 = eVarCoeffD11 = kappa
(StdRegions/StdExpansion.cpp:664-717).
"""
import torch


class HelmholtzKappaMisfit(torch.autograd.Function):
    """misfit = HelmholtzKappaMisfit.apply(kappa, system, lam, rhs, u_target, tol)

    kappa: CUDA float64 tensor (E*Q^d) at the quadrature points; system: a
    GlobalLinSysIterativeFullGPU over a deformed FP64 collection; rhs: CUDA float64
    global right-hand side; u_target: CUDA float64 values at the quadrature points.
    """

    @staticmethod
    def forward(ctx, kappa, system, lam, rhs, u_target, tol=1e-12):
        kappa = kappa.detach().contiguous()
        system.set_varcoeff(kappa)
        x = torch.zeros_like(rhs)
        system.solve(lam, rhs, x, tol=tol)
        J = torch.zeros(1, dtype=torch.float64, device=kappa.device)
        g = torch.zeros_like(rhs)
        system.misfit(x, u_target, J, g)
        ctx.system, ctx.lam, ctx.tol = system, lam, tol
        ctx.save_for_backward(kappa, x, g)
        return J[0].clone()

    @staticmethod
    def backward(ctx, grad_out):
        kappa, x, g = ctx.saved_tensors
        system = ctx.system
        system.set_varcoeff(kappa)
        psi = torch.zeros_like(g)
        system.solve(ctx.lam, g, psi, tol=ctx.tol)
        grad = torch.empty_like(kappa)
        system.kappa_gradient(x, psi, grad)
        return grad_out * grad, None, None, None, None, None


def misfit(kappa, system, lam, rhs, u_target, tol=1e-12):
    return HelmholtzKappaMisfit.apply(kappa, system, lam, rhs, u_target, tol)
