"""torch.autograd binding of the converged response and its adjoint gradients.

A thin autograd.Function over the C ABI (include/kgb.h): the forward pass
installs per-material cross sections, solves the source iteration to a
tolerance and returns the detector response R; the backward pass runs one
adjoint solve and returns dR/dsigma_t [3][G], dR/dsigma_s [3][G] (the
isotropic in-group entries sigs(m, 0, g, g)) and dR/dq.  All work runs on the
context's GPU; the tensors here are small host parameters.
"""
import numpy as np
import torch

from . import abi


class ConvergedResponse(torch.autograd.Function):
    """R(sigma_t, sigma_s, q) at the fixed point of the source iteration."""

    @staticmethod
    def forward(ctx_, sigt, sigs_diag, q, problem):
        problem.install(sigt.detach().cpu().numpy(), sigs_diag.detach().cpu().numpy())
        problem.ctx.solve_converged(float(q), problem.tol, problem.max_iter)
        r = problem.ctx.response()
        ctx_.problem = problem
        ctx_.token = problem.token
        ctx_.q = float(q)
        ctx_.params = (sigt.detach().cpu().numpy().copy(), sigs_diag.detach().cpu().numpy().copy())
        ctx_.dtype, ctx_.device = sigt.dtype, sigt.device
        return torch.tensor(r, dtype=sigt.dtype, device=sigt.device)

    @staticmethod
    def backward(ctx_, grad_r):
        pr = ctx_.problem
        if pr.token != ctx_.token:  # another forward ran on this problem since: restore this one's state
            pr.install(*ctx_.params)
            pr.ctx.solve_converged(ctx_.q, pr.tol, pr.max_iter)
        pr.ctx.adjoint_solve(pr.tol, pr.max_iter)
        _, dt, ds, dq = pr.ctx.gradient()
        g = grad_r.detach().to("cpu", torch.float64).item()
        as_t = lambda a: torch.as_tensor(np.asarray(a) * g, dtype=ctx_.dtype, device=ctx_.device)
        return as_t(dt), as_t(ds), as_t(dq), None


class Problem:
    """A generated Kripke problem with a detector response, differentiable in
    its per-material cross sections and source strength."""

    def __init__(self, inp=None, detector=None, tol=1e-12, max_iter=1000, device=0, **kw):
        self.ctx = abi.Context(device)
        self.inp = self.ctx.generate(inp, **kw)
        self.sigt0, self.sigs0 = abi.material_tables(self.inp)
        self.ctx.set_response(detector)
        self.tol, self.max_iter = tol, max_iter
        self.token = 0

    def parameters(self, dtype=torch.float64):
        """Generator values: (sigma_t [3][G], in-group sigma_s [3][G], q) as leaf tensors."""
        diag = np.stack([np.diagonal(self.sigs0[m, 0]) for m in range(3)])
        return (torch.tensor(self.sigt0, dtype=dtype, requires_grad=True),
                torch.tensor(diag, dtype=dtype, requires_grad=True),
                torch.tensor(1.0, dtype=dtype, requires_grad=True))

    def install(self, sigt, sigs_diag):
        sg = self.sigs0.copy()
        for m in range(3):
            np.fill_diagonal(sg[m, 0], sigs_diag[m])
        self.ctx.set_materials(np.asarray(sigt, dtype=np.float64), sg)
        self.token += 1

    def response(self, sigt, sigs_diag, q):
        return ConvergedResponse.apply(sigt, sigs_diag, q, self)
