"""torch.autograd wrapper of the GPU energy gradient (test harness only).

``EnergyFunction.apply(one, eri, solver)`` returns the lowest eigenvalues of the Hamiltonian
built on the GPU from the packed one-electron table ``one`` and the canonical two-electron
table ``eri`` (both float64 CPU tensors); its backward pass contracts the incoming gradient
with dE_r/d(table) from psoci_energy_gradient, evaluated at the converged eigenvectors
(Hellmann-Feynman), so torch.autograd.gradcheck can compare it with central differences of
the GPU eigenvalues themselves.
"""
import numpy as np
import torch


class Solver:
    """A GPU context holding one configuration space; every call re-builds H from new tables
    and solves for nroots in FP64."""

    def __init__(self, problem, nroots, rtol=1e-10):
        from psoci_gb300 import api

        self.p = problem
        self.nroots = nroots
        self.rtol = rtol
        self.ctx = api.Context(0)
        self.ctx.set_integrals(problem.nbf, problem.one_packed(), problem.eri, problem.ecore)
        self.ctx.set_configs(problem.nbf, problem.nelec, problem.ksym, problem.mx_open, problem.jsym, problem.occ)
        self.ctx.build_determinants()

    def solve(self, one, eri):
        c = self.ctx
        c.set_integrals(self.p.nbf, one, eri, self.p.ecore)
        c.build_hamiltonian(mixed=False)
        r = c.davidson(self.nroots, rtol=self.rtol, mixed=False, want_vectors=True)
        return r.evals, r.evecs

    def gradient(self, vecs):
        return self.ctx.energy_gradient(vecs)


class EnergyFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, one, eri, solver):
        ev, vecs = solver.solve(one.detach().cpu().numpy(), eri.detach().cpu().numpy())
        ctx.solver = solver
        ctx.vecs = vecs
        return torch.from_numpy(np.array(ev))

    @staticmethod
    def backward(ctx, grad_out):
        g1, g2 = ctx.solver.gradient(ctx.vecs)
        go = grad_out.detach().cpu().numpy()
        return torch.from_numpy(go @ g1), torch.from_numpy(go @ g2), None
