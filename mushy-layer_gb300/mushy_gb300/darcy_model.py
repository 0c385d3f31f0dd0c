"""A differentiable diffusive-convective solidification model built from the
path's operators: the workload on which the discrete adjoint is measured.

State phi = (H, C) on a 2D box, periodic in x, walls in z (the second
index).  One step of length dt:

1. (T, C_l, porosity) = closure(H, C)                       [Closure]
2. thermal Darcy buoyancy on the interior z faces (z up),
   u*_z = Ra Da Pi_f (T - T_top)_f, with the
   face permeability Pi_f = exp of the mean log-permeability of the two
   cells (the cell value at a wall); u*_x = 0
3. u = u* - Pi G p with D Pi G p = D u*                      [MacProject]
4. explicit advection sources, centred fluxes:
   src_H = -div(u T), src_C = -div(u C_l)
5. backward-Euler (H, C) step with those sources, heat diffusion 1, solute
   diffusion D_C, T Dirichlet at the bottom (T_b, differentiable) and top,
   no solute flux at the walls                                [BackwardEulerStep]

Defaults: liquid H = 6.3 + 0.2 cos(2 pi x) (T = 1.1 .. 1.5), C = -1, with
1e-3 noise; T = 1.3 at the top and T_b = 0.5 (below the liquidus T = 1 of
C = -1, above the eutectic) at the bottom, so a mushy layer grows from the
bottom while the horizontal temperature contrast drives a cellular flow
(buoyancy that depends on z alone would be hydrostatic: the projection
removes it).

Objective: final mean solid fraction (1 - porosity) plus the mean heat flux
through the top wall, 2 (T_top - T)/dx on its row.  Gradients with respect
to the per-cell log-permeability, Ra and T_b come from the adjoint Functions
through torch.autograd, with two-level checkpointing across steps.
Advection, buoyancy and the objective are composition glue (torch ops), not
part of the operator path.
"""
import math

import torch

from . import abi, ops
from .adjoint import (BEStepper, BackwardEulerStep, Closure, MacProject, Projector, checkpointed,
                      revolve)


class DarcySolidification:
    def __init__(self, n, dt=5e-4, Da=2e-5, Dc=1e-2, T_top=1.3, tol=1e-12, params=None,
                 precision=abi.PREC_F64, newton=True):
        self.n, self.dt, self.Da, self.T_top = n, dt, Da, T_top
        self.grid = abi.make_grid([n, n], 1.0 / n, [1, 0, 0])
        self.params = params or abi.make_params(stefan=5.0, compositionRatio=5.0,
                                                waterDistributionCoeff=1e-3,
                                                specificHeatRatio=1.0)
        g = self.grid
        dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda").contiguous()
        b = []
        for d in range(2):
            fs = abi.face_shape(g, d)
            b.append(dev(torch.stack([-torch.ones(fs, dtype=torch.float64),
                                      -Dc * torch.ones(fs, dtype=torch.float64)])))
        self.bcoef = b
        der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, 0.5),
                           (1, 1, 0): (abi.BC_DIRICHLET, T_top)})
        self.hop = ops.NLMultiCompOp(g, self.params, abi.make_bc(), der, 1.0, -dt, None, b)
        # the step: Newton on the Jacobian hierarchy (newton=True) or the FAS
        # solver; iterate through a transient residual growth (stop only on a
        # doubling); the adjoint solves to the same tolerance
        o = ops.default_options(True)
        o.tolerance, o.hang, o.max_iter = tol, -1.0, 200
        o.precision = precision
        oa = ops.default_options(True)
        oa.tolerance, oa.hang, oa.max_iter = tol, -1.0, 200
        self.stepper = BEStepper(self.hop, o, oa, wall=(1, 0, 0), newton=newton)
        self.popts = ops.default_options(False)
        self.popts.tolerance, self.popts.hang, self.popts.max_iter = tol, 0.0, 400
        self.projector = None
        self._pi_key = None

    # ---- glue (torch)
    def pi_faces(self, logperm):
        L = logperm
        lo = torch.roll(L, 1, dims=-1)
        px = torch.exp(0.5 * (lo + L))
        pi_x = torch.cat([px, px[..., :1]], dim=-1)
        mid = torch.exp(0.5 * (L[..., :-1, :] + L[..., 1:, :]))
        pi_z = torch.cat([torch.exp(L[..., :1, :]), mid, torch.exp(L[..., -1:, :])], dim=-2)
        return pi_x.contiguous(), pi_z.contiguous()

    def _z_faces_interior(self, f):
        z = torch.zeros_like(f[..., :1, :])
        return torch.cat([z, 0.5 * (f[..., :-1, :] + f[..., 1:, :]), z], dim=-2)

    def _x_faces(self, f):
        fx = 0.5 * (torch.roll(f, 1, dims=-1) + f)
        return torch.cat([fx, fx[..., :1]], dim=-1)

    def _div(self, Fx, Fz):
        return ((Fx[..., 1:] - Fx[..., :-1]) + (Fz[..., 1:, :] - Fz[..., :-1, :])) / self.grid.dx

    def projector_for(self, pi_x, pi_z):
        key = (pi_x.data_ptr(), pi_z.data_ptr(), pi_x._version, pi_z._version)
        if self.projector is None or key != self._pi_key:
            self.projector = Projector(self.grid, [pi_x, pi_z], self.popts)
            self._pi_key = key
        return self.projector

    def step(self, phi, pi_x, pi_z, Ra, Tb):
        T, Cl, _ = Closure.apply(phi, self.grid, self.params)
        uz_star = Ra * self.Da * pi_z * self._z_faces_interior(T - self.T_top)
        ux_star = torch.zeros_like(pi_x)
        ux, uz = MacProject.apply(ux_star, uz_star.contiguous(), pi_x, pi_z,
                                  self.projector_for(pi_x, pi_z))
        srcH = -self._div(ux * self._x_faces(T), uz * self._z_faces_interior(T))
        srcC = -self._div(ux * self._x_faces(Cl), uz * self._z_faces_interior(Cl))
        src = torch.stack([srcH, srcC]).contiguous()
        return BackwardEulerStep.apply(phi, src, Tb, self.stepper, self.dt)

    def objective(self, phi):
        T, Cl, por = Closure.apply(phi, self.grid, self.params)
        solid = (1.0 - por).mean()
        flux = (2.0 * (self.T_top - T[..., -1, :]) / self.grid.dx).mean()
        return solid + flux

    def run(self, phi0, logperm, Ra, Tb, nsteps, every=10, snapshots=None):
        """Objective after nsteps; checkpoints every `every` steps, or, with
        `snapshots` given, the binomial (revolve) schedule holding at most
        that many intermediate states."""
        pi_x, pi_z = self.pi_faces(logperm)
        self.projector_for(pi_x.detach(), pi_z.detach())

        def step(s, px, pz, ra, tb):
            return self.step(s, px, pz, ra, tb)

        if snapshots is not None and torch.is_grad_enabled():
            phi = revolve(step, phi0, nsteps, snapshots, pi_x, pi_z, Ra, Tb)
        else:
            phi = checkpointed(step, phi0, nsteps, every, pi_x, pi_z, Ra, Tb)
        return self.objective(phi)


def initial_state(n, seed=0, H0=6.3, amp=0.2):
    """Liquid H = H0 + amp cos(2 pi x) (1 + St = 6 is the liquidus at
    C = -1), C = -1, with 1e-3 seeded noise."""
    g = torch.Generator().manual_seed(seed)
    phi = torch.empty((2, 1, n, n), dtype=torch.float64)
    x = (torch.arange(n, dtype=torch.float64) + 0.5) / n
    phi[0] = (H0 + amp * torch.cos(2 * math.pi * x)).reshape(1, 1, n) + \
        1e-3 * torch.randn((1, n, n), generator=g, dtype=torch.float64)
    phi[1] = -1.0 + 1e-3 * torch.randn((1, n, n), generator=g, dtype=torch.float64)
    return phi.cuda()


def log_permeability(n, seed=0, std=0.5, corr=8.0):
    """Seeded smooth Gaussian field (periodic spectral filter) with the given
    standard deviation."""
    g = torch.Generator().manual_seed(seed + 1000)
    w = torch.randn((n, n), generator=g, dtype=torch.float64)
    k = torch.fft.fftfreq(n, dtype=torch.float64) * n
    kk = k[:, None] ** 2 + k[None, :] ** 2
    f = torch.fft.ifft2(torch.fft.fft2(w) * torch.exp(-0.5 * kk * (corr / n * 2 * math.pi) ** 2)).real
    f = f / f.std() * std
    return f.reshape(1, n, n).cuda()
