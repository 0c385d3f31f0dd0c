"""torch.autograd bindings of the discrete adjoint in libmlgpu.

Each Function runs the path's forward on the GPU and, in backward, its
hand-written adjoint kernels:

* ``Closure``            (H, C) -> (T, C_l, porosity); backward through the
                         closure Jacobian and the porosity derivative.
* ``BackwardEulerStep``  phi_new = BE step of phi_old with source and one
                         wall temperature (Newton on the Jacobian hierarchy, or
                         the FAS solver); backward = one transposed-Jacobian
                         multigrid solve (mlgpu_hc_backward_euler_adjoint).
* ``MacProject``         u = u* - Pi G p; backward = the projection's adjoint
                         solve (mlgpu_mac_project_adjoint), giving u*-bar and
                         Pi-bar.

``checkpointed(steps, ...)`` runs a time loop keeping only every k-th state
and recomputes a segment during the backward sweep (two-level checkpointing;
the recomputation is bitwise deterministic); ``revolve(...)`` reverses the
loop with a bounded number of snapshots on the optimal binomial schedule.
"""
import torch
import torch.utils.checkpoint as tcp

from . import abi, ops


class Closure(torch.autograd.Function):
    @staticmethod
    def forward(ctx, HC, grid, params):
        full = ops.closureFull(grid, params, HC.contiguous())
        ctx.save_for_backward(HC)
        ctx.grid, ctx.params = grid, params
        return full["T"], full["Cl"], full["porosity"]

    @staticmethod
    def backward(ctx, gT, gCl, gpor):
        (HC,) = ctx.saved_tensors
        J = ops.closureJacobian(ctx.grid, ctx.params, HC.contiguous())
        dp = ops.porosityJacobian(ctx.grid, ctx.params, HC.contiguous())
        z = torch.zeros_like(HC[0])
        gT = z if gT is None else gT
        gCl = z if gCl is None else gCl
        gpor = z if gpor is None else gpor
        gH = J[0] * gT + J[2] * gCl + dp[0] * gpor
        gC = J[1] * gT + J[3] * gCl + dp[1] * gpor
        return torch.stack([gH, gC]), None, None


class BEStepper:
    """The solvers of one backward-Euler (H, C) step whose derived-variable
    wall value at `wall` = (dir, side, comp) is a differentiable input."""

    def __init__(self, op, opts, adj_opts, wall=(1, 0, 0), accept=1e-10, newton=True):
        self.op, self.wall, self.accept, self.newton = op, wall, accept, newton
        self.S = None if newton else ops.AMRFASMultiGrid(op, opts)
        self.A = ops.AdjointMultiGrid(op, adj_opts)
        self._value = None
        self.iterations = {"forward": [], "adjoint": []}  # per solve, for reporting

    def set_wall(self, v):
        v = float(v)
        if v == self._value:
            return
        d, s, c = self.wall
        bc = abi.BC()
        bc.type, bc.value = self.op.derived_bc.type, self.op.derived_bc.value
        bc.value[d][s][c] = v
        self.op.derived_bc = bc
        if self.S is not None:
            self.S.setBCs(derived_bc=bc)
        self.A.setBCs(derived_bc=bc)
        self._value = v

    def slot(self):
        d, s, c = self.wall
        return (d * 2 + s) * 2 + c


def _accept(st, rc, accept, what):
    """A solve is used if it converged, or stopped (stagnation / iteration
    cap) with its residual already `accept` times below the initial one."""
    if rc == abi.OK:
        return
    if rc in (abi.ERR_HANG, abi.ERR_NOT_CONVERGED) and st.final_norm <= accept * st.initial_norm:
        return
    raise RuntimeError("%s: solve stopped at %.3g of its initial residual (status %d)"
                       % (what, st.final_norm / max(st.initial_norm, 1e-300), rc))


class BackwardEulerStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi_old, src, wall_value, stepper, dt):
        stepper.set_wall(wall_value.item())
        phi_new = phi_old.detach().clone()
        solve = stepper.A.backwardEulerNewton if stepper.newton else stepper.S.backwardEuler
        st, rc = solve(phi_new, phi_old.detach().contiguous(), dt, src=src.detach().contiguous())
        _accept(st, rc, stepper.accept, "BackwardEulerStep")
        stepper.iterations["forward"].append(st.iterations)
        ctx.save_for_backward(phi_new, wall_value)
        ctx.stepper, ctx.dt = stepper, dt
        return phi_new

    @staticmethod
    def backward(ctx, g):
        phi_new, wall_value = ctx.saved_tensors
        stp = ctx.stepper
        stp.set_wall(wall_value.item())
        mu = torch.zeros_like(phi_new)
        old_bar, src_bar, bcg, st, rc = stp.A.backwardEulerAdjoint(
            phi_new, g.contiguous(), ctx.dt, mu)
        _accept(st, rc, stp.accept, "BackwardEulerStep.backward")
        stp.iterations["adjoint"].append(st.iterations)
        wbar = torch.tensor(bcg[stp.slot()], dtype=torch.float64, device=phi_new.device)
        return old_bar, src_bar, wbar, None, None


class Projector:
    """A projection solver bound to one set of face permeabilities."""

    def __init__(self, grid, pi_faces, opts, bc=None, accept=1e-10):
        self.grid, self.accept = grid, accept
        self.pi = [p.detach().contiguous() for p in pi_faces]
        self.bc = bc if bc is not None else abi.make_bc()
        self.op = ops.ProjectionOp(grid, self.bc, 0.0, 1.0, None, [-p for p in self.pi])
        self.S = ops.AMRMultiGrid(self.op, opts)


class MacProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ux, uz, pi_x, pi_z, projector):
        u = [ux.detach().clone().contiguous(), uz.detach().clone().contiguous()]
        p = torch.zeros(abi.cell_shape(projector.grid), dtype=torch.float64, device=ux.device)
        st, rc = projector.S.levelMacProject(u, projector.pi, p)
        _accept(st, rc, projector.accept, "MacProject")
        ctx.save_for_backward(p)
        ctx.projector = projector
        return u[0], u[1]

    @staticmethod
    def backward(ctx, gx, gz):
        (p,) = ctx.saved_tensors
        P = ctx.projector
        ub = [gx.contiguous() if gx is not None else torch.zeros_like(P.pi[0]),
              gz.contiguous() if gz is not None else torch.zeros_like(P.pi[1])]
        usb, pib, q, st, rc = ops.macProjectAdjoint(P.S, ub, P.pi, p, phi_bc=P.bc)
        _accept(st, rc, P.accept, "MacProject.backward")
        return usb[0], usb[1], pib[0], pib[1], None


def checkpointed(step, state, nsteps, every, *params):
    """state <- step(state, *params) nsteps times, storing the state only at
    every `every`-th step: each segment is recomputed in the backward sweep."""

    def segment(k):
        def run(s, *pp):
            for _ in range(k):
                s = step(s, *pp)
            return s
        return run

    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        if torch.is_grad_enabled():
            state = tcp.checkpoint(segment(k), state, *params, use_reentrant=False)
        else:
            state = segment(k)(state, *params)
        done += k
    return state


# ------------------------------------------------ binomial (revolve) schedule
def revolve_schedule(n, s):
    """Optimal reversal of an n-step chain holding at most `s` snapshots
    besides the chain's first state (the recursive scheme of binomial
    checkpointing): reversing steps [a, b) costs
        cost(1, s) = 1,   cost(n, 0) = n (n + 1) / 2,
        cost(n, s) = min_m  m + cost(n - m, s - 1) + cost(m, s),
    i.e. advance m steps to a new snapshot, reverse the tail with one
    snapshot fewer, then reverse the head.  Returns (cost table, split
    table) indexed [n][s]; split[n][s] is the best m (0 for the base
    cases).  Costs count step evaluations during the reversal; cost - n is
    Griewank and Walther's binomial optimum t n - C(c + t, t - 1) for
    c = s + 1 checkpoints (tested)."""
    INF = float("inf")
    cost = [[0] * (s + 1) for _ in range(n + 1)]
    split = [[0] * (s + 1) for _ in range(n + 1)]
    for k in range(1, n + 1):
        for j in range(s + 1):
            if k == 1:
                cost[k][j] = 1
            elif j == 0:
                cost[k][j] = k * (k + 1) // 2
            else:
                best, arg = INF, 1
                for m in range(1, k):
                    c = m + cost[k - m][j - 1] + cost[m][j]
                    if c < best:
                        best, arg = c, m
                cost[k][j] = best
                split[k][j] = arg
    return cost, split


class _Revolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, step, nsteps, snapshots, state, *params):
        with torch.no_grad():
            s = state
            for _ in range(nsteps):
                s = step(s, *params)
        ctx.step, ctx.n, ctx.snaps = step, nsteps, snapshots
        ctx.save_for_backward(state, *params)
        return s

    @staticmethod
    def backward(ctx, g):
        state0, *params = ctx.saved_tensors
        step = ctx.step
        _, split = revolve_schedule(ctx.n, ctx.snaps)
        pgrads = [torch.zeros_like(p) if p.requires_grad else None for p in params]

        def advance(s, k):
            with torch.no_grad():
                for _ in range(k):
                    s = step(s, *params)
            return s

        def one_step_adjoint(s, gout):
            # the step recomputed with its tape, then backpropagated
            with torch.enable_grad():
                x = s.detach().requires_grad_(True)
                ps = [p.detach().requires_grad_(p.requires_grad) for p in params]
                y = step(x, *ps)
                wrt = [x] + [p for p in ps if p.requires_grad]
                gr = torch.autograd.grad(y, wrt, gout, allow_unused=True)
            it = iter(gr[1:])
            for i, p in enumerate(params):
                if p.requires_grad:
                    gi = next(it)
                    if gi is not None:
                        pgrads[i] = pgrads[i] + gi
            return gr[0] if gr[0] is not None else torch.zeros_like(s)

        def reverse(s_a, n, free, gout):
            # adjoint of n steps starting from state s_a, `free` snapshots left
            if n == 1:
                return one_step_adjoint(s_a, gout)
            if free == 0:
                for k in range(n - 1, -1, -1):
                    gout = one_step_adjoint(advance(s_a, k), gout)
                return gout
            m = split[n][free]
            s_m = advance(s_a, m)  # the new snapshot
            gout = reverse(s_m, n - m, free - 1, gout)
            del s_m
            return reverse(s_a, m, free, gout)

        g0 = reverse(state0, ctx.n, ctx.snaps, g)
        return (None, None, None, g0) + tuple(pgrads)


def revolve(step, state, nsteps, snapshots, *params):
    """state <- step(state, *params) nsteps times, differentiable with at
    most `snapshots` intermediate states alive in the backward sweep (plus
    the first one): the binomial schedule of revolve_schedule, so the
    recomputation is the least possible for that memory."""
    if nsteps < 1:
        return state
    return _Revolve.apply(step, int(nsteps), int(snapshots), state, *params)
