#!/usr/bin/env python3
"""Benchmark: multigrid cell-updates/s to a 1e-10 relative residual on one
GB300, mixed precision against FP64, on the 3D 256^3 mushy-layer step.

Workload (synthetic, seeded; no dataset is involved): a 256^3 box (16.8M
cells, dx = 1/256), periodic in x and y, walls in z.  Porosity chi = 1 - s
with the solid fraction s falling linearly from 0.6 at the bottom to 0 at the
top plus 1e-2 seeded noise; Kozeny-Carman permeability Pi = chi^3/(1-chi)^2
capped at 1e4, geometric-mean faces (the library's face kernel).  One step of
the workload is one time step of Darcy convection in the mushy layer:

* the projection Poisson solve div(Pi grad p) = div u*, u* the Darcy
  buoyancy flux Ra Pi theta on z faces (Ra = 400, theta a conductive profile
  from -1 at the bottom to 0.5 at the top plus 0.05 seeded noise), from
  p = 0 to 1e-10 of the initial residual (max norm);
* the backward-Euler (H, C) step (dt = 1e-4, St = 5, CR = 5, heat / salt
  diffusivities 1 / 1e-2) from a state with H falling linearly from 6 at the
  top to 2 at the bottom (1e-2 noise), C = -1, the bottom wall held at
  T = C_l = -1: Newton's method on the Jacobian multigrid to 1e-10 of the
  initial residual (the reference's FAS smoother ignores dT/dH and stalls
  above 1e-10 on this problem; Newton's linear cycles use each cell's exact
  2x2 diagonal block).

Mixed = FP32 multigrid cycles inside FP64 defect correction / FP64 Newton
residuals (closure in FP64); FP64 = the same solvers in FP64 (the projection
bit for bit the reference's algorithm).  `value` is device-timed with inputs
resident in HBM, the 129 MB L2 flushed (512 MiB write) between steps; `e2e`
times the same step through the public API with the step's inputs copied from
pinned host memory and its results copied back (the (H, C) state's copy in
overlaps the projection, the pressure's copy back the (H, C) solve, on a copy
stream).  `roofline` is for the
dominant kernel of the mixed step, timed with CUDA events on its stream after
the timed region.  --config N measures another configuration (2: the 2D
512^2 projection solve).  --impl reference times the CPU restatement of the
reference's algorithms (oracle) on the host cores.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mushy-layer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

TOL = 1e-10
METRIC = "FAS V-cycle cell-updates/s on 1 GB300: mixed vs FP64 at 1e-10 rel residual"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
PROFILES = os.path.join(ROOT, "profiles")

C4_N = 256
C4_SEED = 4
C4_RA = 400.0
C4_DT = 1e-4
C4_WORKLOAD = ("3D 256^3 mushy-layer step: projection Poisson div(Pi grad p) = div u* "
               "(Kozeny-Carman Pi of a linear-in-depth solid fraction 0-0.6 + 1e-2 noise, "
               "Darcy buoyancy Ra=400) and the backward-Euler (H, C) solve (dt=1e-4, "
               "St=5, CR=5, cold bottom), both to 1e-10 max-norm rel residual; "
               "periodic x/y, walls in z")


# ------------------------------------------------------------ the workload
def c4_host_fields(n=C4_N, seed=C4_SEED):
    """Seeded host fields of the 256^3 step: porosity, permeability,
    temperature perturbation profile and the (H, C) state."""
    rng = np.random.default_rng(seed)
    z = (np.arange(n) + 0.5) / n
    shape = (n, n, n)  # [k][j][i]
    solid = 0.6 * (1.0 - z)[:, None, None] + 1e-2 * rng.standard_normal(shape)
    chi = np.clip(1.0 - solid, 0.05, 1.0)
    with np.errstate(divide="ignore"):
        perm = np.where(chi < 1.0, chi ** 3 / np.maximum((1.0 - chi) ** 2, 1e-300), 1e4)
    perm = np.minimum(perm, 1e4)
    theta = (-1.0 + 1.5 * z)[:, None, None] + 0.05 * rng.standard_normal(shape)
    phi0 = np.empty((2,) + shape)
    phi0[0] = 6.0 - 4.0 * (1.0 - z)[:, None, None] * (1.0 + 1e-2 * rng.standard_normal(shape))
    phi0[1] = -1.0
    return perm.reshape((1,) + shape), theta, phi0


def c4_problem(torch, abi, ops, n=C4_N, seed=C4_SEED):
    """Device operators and inputs of the step (built through the library's
    own face and divergence kernels)."""
    perm, theta, phi0 = c4_host_fields(n, seed)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    g = abi.make_grid([n, n, n], 1.0 / n, (1, 1, 0))
    lib = abi.load()
    pif = [ops.face_tensor(g, d, 1)[0] for d in range(3)]
    arr = (C.c_void_p * 3)(*[t.data_ptr() for t in pif])
    abi.check(lib.mlgpu_face_geomean(C.byref(g), ops._ptr(dev(perm)), arr, ops._stream()),
              "face_geomean")
    # u*: Darcy buoyancy on z faces, zero through the z walls
    th = dev(theta)
    u = [torch.zeros_like(pif[0]), torch.zeros_like(pif[1]), torch.zeros_like(pif[2])]
    u[2][1:-1] = C4_RA * pif[2][1:-1] * 0.5 * (th[1:] + th[:-1])
    f = ops.cell_tensor(g, 1)
    uarr = (C.c_void_p * 3)(*[t.data_ptr() for t in u])
    abi.check(lib.mlgpu_mac_divergence(C.byref(g), ops._ptr(f), uarr, ops._stream()),
              "mac_divergence")
    f -= f.mean()
    pop = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, [-x for x in pif])
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    der = abi.make_bc({(2, 0, 0): (abi.BC_DIRICHLET, -1.0), (2, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    bh = [torch.stack([-torch.ones_like(pif[d]), torch.full_like(pif[d], -1e-2)])
          for d in range(3)]
    hop = ops.NLMultiCompOp(g, prm, abi.make_bc(), der, 1.0, -C4_DT, None, bh)
    torch.cuda.synchronize()
    return {"g": g, "n": n, "f": f, "pop": pop, "hop": hop, "phi0": dev(phi0), "pif": pif,
            "prm": prm, "der": der, "bh": bh}


class C4Runner:
    """The two solves of one step, FP64 or mixed; solvers built once."""

    def __init__(self, torch, abi, ops, prob, use_graph=None,
                 precs=("mixed", "fp64", "fp64_fast")):
        self.torch, self.abi, self.ops, self.P = torch, abi, ops, prob
        self.S = {}
        for prec in precs:
            code = abi.PREC_MIXED if prec == "mixed" else abi.PREC_F64
            po = ops.default_options(False)
            po.tolerance, po.hang, po.max_iter, po.precision = TOL, 1e-15, 300, code
            ho = ops.default_options(True)
            ho.tolerance, ho.hang, ho.max_iter, ho.precision = TOL, -1.0, 60, code
            if prec == "fp64_fast":
                # the mixed path's kernels in FP64: Newton's lean cycles and
                # outer loops, the projection's lean split cycles and outer
                # step -- the same design, FP64 data
                ho.fuse_levels = 2
                po.fuse_levels = 2
            if use_graph is not None:
                po.use_graph = ho.use_graph = use_graph
            self.S[prec] = (ops.AMRMultiGrid(prob["pop"], po), ops.AdjointMultiGrid(prob["hop"], ho))
        self.p = {k: torch.zeros_like(prob["f"]) for k in self.S}
        self.u = {k: torch.empty_like(prob["phi0"]) for k in self.S}

    def step(self, prec, f=None, phi0=None):
        """One step from the resident inputs (or the given device inputs)."""
        PS, HS = self.S[prec]
        f = self.P["f"] if f is None else f
        phi0 = self.P["phi0"] if phi0 is None else phi0
        p, u = self.p[prec], self.u[prec]
        p.zero_()
        stp, rcp = PS.solve(p, f)
        u.copy_(phi0)
        sth, rch = HS.backwardEulerNewton(u, phi0, C4_DT)
        return (stp, rcp), (sth, rch)

    def step_e2e(self, prec, h_f, h_phi, h_p, h_u, d_f, d_phi, cs):
        """One step from pinned host inputs to pinned host results through the
        public API, the copies a solve does not wait for on the copy stream
        `cs`: the (H, C) state goes in while the projection runs, the pressure
        comes back while the (H, C) solve runs."""
        torch = self.torch
        main = torch.cuda.current_stream()
        PS, HS = self.S[prec]
        p, u = self.p[prec], self.u[prec]
        d_f.copy_(h_f, non_blocking=True)
        cs.wait_stream(main)
        with torch.cuda.stream(cs):
            d_phi.copy_(h_phi, non_blocking=True)
        phi_in = cs.record_event()
        p.zero_()
        stp, rcp = PS.solve(p, d_f)
        p_done = main.record_event()
        main.wait_event(phi_in)
        u.copy_(d_phi)
        sth, rch = HS.backwardEulerNewton(u, d_phi, C4_DT)
        cs.wait_event(p_done)
        with torch.cuda.stream(cs):
            h_p.copy_(p, non_blocking=True)
        h_u.copy_(u, non_blocking=True)
        main.wait_stream(cs)
        return (stp, rcp), (sth, rch)

    def cells(self):
        return self.P["n"] ** 3

    @staticmethod
    def summary(out):
        (stp, rcp), (sth, rch) = out
        return {"projection": {"rc": rcp, "iterations": stp.iterations, "cycles": stp.cycles,
                               "final_rel_residual": stp.final_norm / stp.initial_norm,
                               "cell_updates": stp.cell_updates},
                "hc": {"rc": rch, "newton_iterations": sth.iterations,
                       "linear_cycles": sth.cycles,
                       "final_rel_residual": sth.final_norm / sth.initial_norm,
                       "rel_residual_history": [
                           sth.norm_history[q] / sth.initial_norm
                           for q in range(min(sth.iterations + 1, 64))],
                       "cell_updates": sth.cell_updates}}


def run_gpu(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from mushy_gb300 import abi, ops

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    prob = c4_problem(torch, abi, ops)
    R = C4Runner(torch, abi, ops, prob)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    ncell = C4_N ** 3

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            out = R.step(prec)
            assert out[0][1] == 0 and out[1][1] == 0, ("warm-up step failed", prec,
                                                       C4Runner.summary(out))
        tot_ms, upd, last = 0.0, 0.0, None
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = R.step(prec)
            e1.record(stream)
            torch.cuda.synchronize()
            assert out[0][1] == 0 and out[1][1] == 0, ("step failed", prec, C4Runner.summary(out))
            tot_ms += e0.elapsed_time(e1)
            upd += out[0][0].cell_updates + out[1][0].cell_updates
            last = out
        if world > 1:
            torch.distributed.barrier()
        tot_ms = aggregate_max(tot_ms, world, "cuda")
        return tot_ms, upd, last

    def e2e_run():
        # end to end through the public API: the step's inputs (rhs of the
        # projection, old (H, C) state) from pinned host memory, results back
        h_f = torch.from_numpy(prob["f"].cpu().numpy()).pin_memory()
        h_phi = torch.from_numpy(prob["phi0"].cpu().numpy()).pin_memory()
        h_p = torch.empty_like(h_f).pin_memory()
        h_u = torch.empty_like(h_phi).pin_memory()
        d_f, d_phi = torch.empty_like(prob["f"]), torch.empty_like(prob["phi0"])
        cs = torch.cuda.Stream()
        for _ in range(args.warmup):  # the whole timed sequence, copies back included
            R.step_e2e("mixed", h_f, h_phi, h_p, h_u, d_f, d_phi, cs)
        torch.cuda.synchronize()
        e2e_ms, e2e_upd = 0.0, 0.0
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = R.step_e2e("mixed", h_f, h_phi, h_p, h_u, d_f, d_phi, cs)
            e1.record(stream)
            torch.cuda.synchronize()
            e2e_ms += e0.elapsed_time(e1)
            e2e_upd += out[0][0].cell_updates + out[1][0].cell_updates
        e2e_ms = aggregate_max(e2e_ms, world, "cuda")
        h2d = h_f.numel() * 8 + h_phi.numel() * 8
        d2h = h_p.numel() * 8 + h_u.numel() * 8
        return e2e_ms, e2e_upd, h2d, d2h

    with Clocks() as clk:
        ms_m, upd_m, out_m = timed("mixed", args.steps, args.warmup)
        # end to end right after the device-timed mixed arm (the same GPU state)
        e2e_ms, e2e_upd, h2d, d2h = e2e_run()
        ms_d, upd_d, out_d = timed("fp64", args.steps, args.warmup)
        ms_f, upd_f, out_f = timed("fp64_fast", args.steps, args.warmup)
    clocks = clk.summary()

    # mixed against FP64: pressure up to its constant, (H, C) state
    a, m = R.p["fp64"], R.p["mixed"]
    p_err = float(((a - a.mean()) - (m - m.mean())).abs().max() / (a - a.mean()).abs().max())
    u64, um = R.u["fp64"], R.u["mixed"]
    hc_err = float((um - u64).abs().max() / u64.abs().max())
    hc_err_fast = float((R.u["fp64_fast"] - u64).abs().max() / u64.abs().max())
    launches = {k: int(v[0][0].kernel_launches) for k, v in (("mixed", out_m), ("fp64", out_d))}


    roof = dominant_kernel_roofline(torch, abi, ops, R)
    value = upd_m * world / (ms_m * 1e-3)
    sm = C4Runner.summary(out_m)
    sd = C4Runner.summary(out_d)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "cell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_m / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-inner/f64-outer",
        "data": "synthetic (seeded porosity, buoyancy and (H, C) fields of the 256^3 step)",
        "config": {"workload": C4_WORKLOAD, "cells": ncell,
                   "hc_solver": "Newton on the Jacobian multigrid (FP32 cycles in mixed), "
                                "60-iteration cap, no stall test",
                   "projection_solver": "multigrid V(2,4), 300-iteration cap",
                   "l2": "flushed (512 MiB write) between steps; every field > 129 MB",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "mixed": {**sm, "ms_per_step": ms_m / args.steps, "gpu_launches_per_step": None},
        "fp64": {**sd, "value": upd_d * world / (ms_d * 1e-3), "ms_per_step": ms_d / args.steps,
                 "note": "reference expression order (bitwise the oracle's kernels)"},
        "fp64_fast": {**C4Runner.summary(out_f), "value": upd_f * world / (ms_f * 1e-3),
                      "ms_per_step": ms_f / args.steps,
                      "note": "FP64 with the mixed path's kernel design (lean colour-split "
                              "cycles and lean FP64 outer loops, for Newton's step "
                              "and the projection)",
                      "hc_rel_vs_fp64": hc_err_fast},
        "time_to_solution_ratio_fp64_over_mixed": ms_d / ms_m,
        "time_to_solution_ratio_fp64_fast_over_mixed": ms_f / ms_m,
        "mixed_vs_fp64": {"pressure_rel": p_err, "hc_rel": hc_err},
        "e2e": {"value": e2e_upd * world / (e2e_ms * 1e-3), "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_ms / args.steps,
                "copies": "pinned host buffers; the (H, C) state's copy in overlaps the "
                          "projection and the pressure's copy back the (H, C) solve (a copy "
                          "stream); the rhs in and the (H, C) result back are serial"},
        "roofline": roof,
        "clocks": clocks,
        "gpu_launches": None,
    }
    line["gpu_launches"] = int(args.steps * (out_m[0][0].kernel_launches +
                                             out_m[1][0].kernel_launches))
    line["mixed"]["gpu_launches_per_step"] = int(out_m[0][0].kernel_launches +
                                                 out_m[1][0].kernel_launches)
    if rank == 0:
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(args)
            line["oracle_check"] = oracle_check(prob, R)
        print(json.dumps(line))


# ------------------------------------------------------- CPU (oracle) legs
def _cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for key in ("Model name", "Vendor ID"):
            for ln in out.splitlines():
                if ln.startswith(key):
                    return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _oracle_step(O, abi, host, it_proj=1, it_hc=1):
    """One bounded sample of the step on the host: `it_proj` iterations of the
    oracle's projection multigrid and `it_hc` FAS iterations of the (H, C)
    backward-Euler step (the reference's own algorithms), 256^3.  Returns
    cell updates."""
    ref_p, f, ref_h, phi0 = host
    op = O.default_options(0)
    op.tolerance, op.hang, op.max_iter = TOL, 1e-15, it_proj
    _, st, _ = O.vc_solve(ref_p, op, np.zeros_like(f), f)
    oh = O.default_options(1)
    oh.tolerance, oh.hang, oh.max_iter = TOL, -1.0, it_hc
    _, st2, _ = O.hc_backward_euler(ref_h, oh, phi0, phi0, C4_DT)
    return st.cell_updates + st2.cell_updates


def _host_problem(O, abi):
    n = C4_N
    perm, theta, phi0 = c4_host_fields(n)
    g = abi.make_grid([n, n, n], 1.0 / n, (1, 1, 0))
    pif = O.face_geomean(g, perm[0])
    u = [np.zeros(abi.face_shape(g, d)) for d in range(3)]
    u[2][1:-1] = C4_RA * pif[2][1:-1] * 0.5 * (theta[1:] + theta[:-1])
    f = O.mac_divergence(g, u)
    f -= f.mean()
    ref_p = O.VCOpHost(g, abi.make_bc(), 0.0, 1.0, None, [-x for x in pif])
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    der = abi.make_bc({(2, 0, 0): (abi.BC_DIRICHLET, -1.0), (2, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    bh = [np.stack([-np.ones(abi.face_shape(g, d)), np.full(abi.face_shape(g, d), -1e-2)])
          for d in range(3)]
    ref_h = O.NLOpHost(g, prm, abi.make_bc(), der, 1.0, -C4_DT, None, bh)
    return ref_p, f, ref_h, phi0


def cpu_baseline(args):
    """The oracle (FP64 restatement of the reference's algorithms) on the host
    cores, at 1 thread and at all threads, each on one bounded sample of the
    256^3 step: one projection multigrid iteration and one FAS iteration of
    the (H, C) step."""
    from oracle import oracle as O
    from mushy_gb300 import abi
    host = _host_problem(O, abi)
    allc = os.cpu_count() or 1
    res = {}
    for nt in (1, allc):
        O.set_threads(nt)
        t0 = time.time()
        upd = _oracle_step(O, abi, host)
        res[nt] = (upd / (time.time() - t0), time.time() - t0)
    O.set_threads(allc)
    return {"value": res[allc][0], "unit": "cell-updates/s", "cores": allc, "kind": "port",
            "cpu_model": _cpu_model(),
            "one_thread": {"value": res[1][0], "seconds": res[1][1]},
            "sample": "one projection multigrid iteration + one FAS iteration of the (H, C) "
                      "backward-Euler step on the full 256^3 problem (%.1f s at %d threads, "
                      "%.1f s at 1 thread)" % (res[allc][1], allc, res[1][1])}


def oracle_check(prob, R):
    """Error of the mixed step against the FP64 oracle: the oracle's own
    residuals (max norm) of the mixed pressure and (H, C) state, relative to
    the initial ones."""
    from oracle import oracle as O
    from mushy_gb300 import abi
    ref_p, f, ref_h, phi0 = _host_problem(O, abi)
    p = R.p["mixed"].cpu().numpy()
    u = R.u["mixed"].cpu().numpy()
    rp = O.norm(O.vc_residual(ref_p, p, f)) / O.norm(f)
    rh = O.norm(O.nl_residual(ref_h, u, phi0)) / O.norm(O.nl_residual(ref_h, phi0, phi0))
    return {"projection_rel_residual": rp, "hc_rel_residual": rh}


def run_reference(args):
    """CPU restatement of the reference's algorithms (oracle, FP64, all host
    threads) on the same 256^3 step: each step one bounded sample (one
    projection multigrid iteration + one FAS iteration of the (H, C) step)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    from mushy_gb300 import abi
    host = _host_problem(O, abi)
    allc = os.cpu_count() or 1
    O.set_threads(allc)
    for _ in range(args.warmup):
        _oracle_step(O, abi, host)
    t0 = time.time()
    upd = 0.0
    for _ in range(args.steps):
        upd += _oracle_step(O, abi, host)
    el = time.time() - t0
    v = upd / el
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (same seeded fields)",
        "config": {"workload": C4_WORKLOAD, "cells": C4_N ** 3},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": allc, "kind": "port",
                         "cpu_model": _cpu_model(),
                         "sample": "per step: one projection multigrid iteration + one FAS "
                                   "iteration of the (H, C) step, 256^3, %d steps" % args.steps},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


# Compulsory bytes per cell of the box of one FP32 red/black half sweep of
# the Newton step's cycles (lean_gsrb_kernel, colour-split arrays): the
# updated half of the cells read g (2 floats), K (4) and J (4) and write x (2)
# and w (2); every face coefficient is read once (3 directions x 2
# components); the other half's w is read once (2 floats each):
# (7 + 6 + 1) floats = 56 B per cell of the box.
LEAN_HALF_SWEEP_BYTES_PER_CELL = 56
LEAN_SWEEP_PROFILE = os.path.join(PROFILES, "lean_gsrb_kernel_256cubed.md")


def profiled_traffic(path, key):
    """DRAM bytes per launch recorded in a committed ncu summary (a line
    `key: <bytes>`), or None."""
    try:
        for ln in open(path):
            if ln.strip().startswith(key + ":"):
                return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def _sweep_time(abi, HS, kind, reps=40):
    ms = C.c_double()
    abi.check(abi.load().mlgpu_hc_newton_sweep_time(HS.h, kind, reps, C.byref(ms)), "sweep time")
    return ms.value


def dominant_kernel_roofline(torch, abi, ops, R):
    """The mixed step's dominant HBM-bound kernel, the FP32 red/black half
    sweep of the Newton cycles on the 256^3 level (lean_gsrb_kernel<3>),
    timed with CUDA events on the solver's stream at the state of the last
    timed step; achieved = its compulsory bytes / its time."""
    HS = R.S["mixed"][1]
    ncell = R.cells()
    hbm, kind = peaks()
    ms = _sweep_time(abi, HS, 0)
    # the one-cell-per-thread variant of the same sweep (the same bits), for
    # comparison; then the library default again
    HS.setNewtonParams(vector_sweeps=0)
    ms_scalar = _sweep_time(abi, HS, 0)
    HS.setNewtonParams()
    alg = LEAN_HALF_SWEEP_BYTES_PER_CELL * ncell
    achieved = alg / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": "lean_gsrb_vec_kernel<float, 3> (FP32 red/black half "
                                       "sweep, 4-cell vector loads, Newton linear cycles, "
                                       "256^3 level)",
            "achieved": achieved, "peak": hbm, "peak_kind": kind, "unit": "GB/s",
            "frac": achieved / hbm,
            "traffic": profiled_traffic(LEAN_SWEEP_PROFILE, "dram_bytes_per_launch_256cubed"),
            "alg_bytes_per_launch": alg, "launch_us": ms * 1e3,
            "scalar_variant_launch_us": ms_scalar * 1e3,
            "timing": "CUDA events on the solver stream, 40 launches after the timed region"}



class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self):
        self.samples, self.stop = [], threading.Event()
        self.t = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                      "--query-gpu=" + q, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 2 + i and s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def aggregate_max(value, world, device):
    """Replica timing: the slowest rank bounds the whole job (max over ranks).
    Replicas share no data, so this is the only collective of the run."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, ms):
    """Units processed by all ranks divided by the (max-over-ranks) time."""
    return units_per_rank * world / (ms * 1e-3)


def peaks():
    try:
        d = json.load(open(PEAKS))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _events_ms(fn):
    """Device time of fn() on the current stream (CUDA events, synchronised)."""
    import torch
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def _compatible_u(u):
    """MAC velocity with zero net flux: periodic x seam faces equal, zero
    normal velocity on the non-periodic walls (y, and z in 3D)."""
    u[0][..., -1] = u[0][..., 0]
    u[1][..., 0, :] = 0.0
    u[1][..., -1, :] = 0.0
    if len(u) == 3:
        u[2][0] = 0.0
        u[2][-1] = 0.0
    return u


def _c1_setup(torch, abi, ops, P, n):
    """(H, C) problem of the 64x64 diffusive-solidification configuration:
    liquid H = 1 + St, C = -1; T = -1 at the bottom, 0.5 at the top, C_l = -1
    on both; side walls Neumann; k_T = 1, D_C = 0 (Le infinite)."""
    g = P.grid((n, n))
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 1, 0): (abi.BC_DIRICHLET, 0.5),
                       (1, 0, 1): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0], phi0[1] = 6.0, -1.0
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
         for d in range(2)]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, 1.0, None, [dev(x) for x in b])
    return g, prm, phi_bc, der, phi0, b, dev, op


def config1(args, torch, abi, ops, O, P):
    """64x64 diffusive solidification, no flow: ten backward-Euler steps of the
    nonlinear (H, C) system, each solved by FAS multigrid to 1e-10 (FP64).
    Checked against the CPU restatement step by step."""
    n, dt, steps = 64, 1e-3, 10
    g, prm, phi_bc, der, phi0, b, dev, op = _c1_setup(torch, abi, ops, P, n)
    om = ops.default_options(True)
    om.precision = abi.PREC_MIXED
    SM = ops.AMRFASMultiGrid(op, om)
    S = ops.AMRFASMultiGrid(op, ops.default_options(True))

    def march():
        cur, upd, its, rcs = dev(phi0), 0.0, 0, []
        for _ in range(steps):
            new = cur.clone()
            st, rc = S.backwardEuler(new, cur, dt)
            upd, its, cur = upd + st.cell_updates, its + st.iterations, new
            rcs.append((rc, float("%.2e" % (st.final_norm / st.initial_norm))))
        return cur, upd, its, rcs

    march()
    ms, (cur, upd, its, rcs) = _events_ms(march)
    S, S64 = SM, S
    march()
    ms_m, (cur_m, upd_m, its_m, rcs_m) = _events_ms(march)
    S = S64
    ref = O.NLOpHost(g, prm, phi_bc, der, 1.0, 1.0, None, b)
    oo = O.default_options(1)
    t0 = time.time()
    h = phi0.copy()
    for _ in range(steps):
        h, st_ref, rc_ref = O.hc_backward_euler(ref, oo, h, h, dt)
    cpu_s = time.time() - t0
    diff = float(np.abs(cur.cpu().numpy() - h).max())
    # the same ten steps solved to 1e-10 by Newton on the Jacobian hierarchy
    # (the reference's FAS with its 10-iteration cap stops above it), FP64 and
    # mixed, and the mixed states against the FP64 ones
    newton = {}
    states = {}
    for key, code in (("fp64", abi.PREC_F64), ("mixed", abi.PREC_MIXED)):
        no = ops.default_options(True)
        no.tolerance, no.hang, no.max_iter, no.precision = TOL, -1.0, 60, code
        NS = ops.AdjointMultiGrid(op, no)

        def nmarch():
            cur, out = dev(phi0), []
            for _ in range(steps):
                new = cur.clone()
                st, rc = NS.backwardEulerNewton(new, cur, dt)
                out.append((rc, st.iterations, float("%.2e" % (st.final_norm / st.initial_norm))))
                cur = new
            return cur, out
        nmarch()
        ms_n, (cur_n, out_n) = _events_ms(nmarch)
        states[key] = cur_n.cpu().numpy()
        newton[key] = {"ms_per_step": ms_n / steps, "steps": out_n,
                       "converged": all(r == 0 and f <= TOL for r, _, f in out_n)}
    newton["mixed_vs_fp64_max_abs"] = float(np.abs(states["mixed"] - states["fp64"]).max())
    return {"metric": "backward-Euler steps/s (FAS to 1e-10, FP64)", "value": steps / (ms * 1e-3),
            "unit": "steps/s", "higher_is_better": True, "ms_per_step": ms / steps,
            "cell_updates_per_s": upd / (ms * 1e-3), "fas_iterations": its, "status": rcs,
            "config": {"workload": "64x64 diffusive solidification, St=5, CR=5, k=1e-3, "
                                   "T=-1 bottom / 0.5 top, C_l=-1, 10 steps dt=1e-3"},
            "parity": {"max_abs_diff_vs_oracle": diff, "oracle_s": cpu_s},
            "mixed": {"ms_per_step": ms_m / steps, "fas_iterations": its_m, "status": rcs_m,
                      "max_abs_diff_vs_fp64": float(np.abs(cur_m.cpu().numpy() -
                                                           cur.cpu().numpy()).max())},
            "newton_to_1e-10": newton,
            "note": "latency bound (4096 cells): report only; status (rc, final/initial) per "
                    "step; Newton steps (rc, iterations, final/initial)"}


def config3(args, torch, abi, ops, O, P):
    """1024x1024 mushy-layer step: (H, C) backward-Euler nonlinear solve, the
    two Darcy-Brinkman velocity solves and the MAC projection, all FP64 against
    all mixed precision."""
    n = 1024
    g, chi, perm, u = P.projection_problem((n, n), 3, sigma=32.0)
    u = _compatible_u(u)
    rng = np.random.default_rng(3)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    # (H, C): liquid plus 1e-3 noise, cold bottom
    prm = abi.make_params(stefan=5.0, compositionRatio=25.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0] = 6.0 + 1e-3 * rng.standard_normal(abi.cell_shape(g))
    phi0[1] = -1.0 + 1e-3 * rng.standard_normal(abi.cell_shape(g))
    bh = [np.stack([-np.ones(abi.face_shape(g, d)), -np.full(abi.face_shape(g, d), 1.0 / 200)])
          for d in range(2)]
    hop = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, 1.0, None, [dev(x) for x in bh])
    hom = ops.default_options(True)
    hom.precision = abi.PREC_MIXED
    HSS = {"fp64": ops.AMRFASMultiGrid(hop, ops.default_options(True)),
           "mixed": ops.AMRFASMultiGrid(hop, hom)}
    d_phi0 = dev(phi0)
    # Darcy-Brinkman: (Da^-1 chi/Pi) u - visc lap u = rho per component
    cC = dev(chi / (1e-3 * perm))
    bdb = [dev(-np.ones(abi.face_shape(g, d))) for d in range(2)]
    noslip = abi.make_bc({(d, s, 0): (abi.BC_DIRICHLET, 0.0) for d in range(2) for s in range(2)})
    dbop = ops.DarcyBrinkmanOp(g, noslip, 0.0, -1.0, None, bdb, cC)
    rho = [dev(1e-3 * rng.standard_normal(abi.cell_shape(g))) for _ in range(2)]
    pif = O.face_geomean(g, perm)
    pop = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, [dev(-x) for x in pif])
    d_pif = [dev(x) for x in pif]
    out = {}
    for prec in ("fp64", "mixed"):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter = TOL, 1e-15, 300
        o.precision = abi.PREC_MIXED if prec == "mixed" else abi.PREC_F64
        DS, PS = ops.AMRMultiGrid(dbop, o), ops.AMRMultiGrid(pop, o)
        HS = HSS[prec]

        def step():
            new = d_phi0.clone()
            st_h, rc_h = HS.backwardEuler(new, d_phi0, 1e-5)
            vel = []
            its = [(st_h.iterations, rc_h, st_h.final_norm / st_h.initial_norm)]
            for c in range(2):
                v = torch.zeros_like(rho[c])
                st_v, rc_v = DS.solve(v, rho[c])
                vel.append(v)
                its.append(st_v.iterations)
            du = [dev(x) for x in u]
            p = torch.zeros(abi.cell_shape(g), dtype=torch.float64, device="cuda")
            st_p, rc_p = PS.levelMacProject(du, d_pif, p)
            its.append(st_p.iterations)
            return new, vel, du, its

        step()
        ms, res = _events_ms(step)
        out[prec] = (ms, res)
    # the (H, C) step solved to 1e-10 by Newton on the Jacobian hierarchy
    # (the FAS solve above stops at the reference's 10-iteration cap)
    on = ops.default_options(True)
    on.tolerance, on.hang, on.max_iter = TOL, -1.0, 60
    AN = ops.AdjointMultiGrid(hop, on)

    def newton_step():
        new = d_phi0.clone()
        return AN.backwardEulerNewton(new, d_phi0, 1e-5), new

    newton_step()
    ms_newton, ((st_n, rc_n), h_newton) = _events_ms(newton_step)
    ms64, (h64, v64, u64, it64) = out["fp64"]
    msm, (hm, vm, um, itm) = out["mixed"]
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
    return {"metric": "mushy-layer step time, 1024^2 (HC FAS + 2 Darcy-Brinkman + MAC projection)",
            "value": msm, "unit": "ms/step (mixed)", "higher_is_better": False,
            "fp64_ms": ms64, "ratio_fp64_over_mixed": ms64 / msm,
            "iterations": {"fp64": it64, "mixed": itm},
            "hc_newton_to_1e-10": {"ms": ms_newton, "iterations": st_n.iterations, "rc": rc_n,
                                   "final_rel_residual": st_n.final_norm / st_n.initial_norm,
                                   "linear_cycles": st_n.cycles},
            "mixed_vs_fp64": {"hc_rel": rel(hm, h64),
                              "velocity_rel": max(rel(vm[c], v64[c]) for c in range(2)),
                              "mac_u_rel": max(rel(um[d], u64[d]) for d in range(2))},
            "config": {"workload": "2D 1024x1024, Kozeny-Carman Pi of a smooth porosity, "
                                   "Da=1e-3, CR=25, Le=200, liquid + 1e-3 noise, dt=1e-5; "
                                   "linear solves to 1e-10, (H, C) solve capped at the "
                                   "reference's 10 FAS iterations"},
            "note": "iterations: [(H, C) (iterations, status, final/initial residual), DB x, "
                    "DB y, MAC projection]"}


# ------------------------------------------------ 2D 512^2 projection (config 2)
def c2_problem(n=512, seed=1):
    from problems import projection_problem
    from oracle import oracle as O
    g, chi, perm, u = projection_problem((n, n), seed, sigma=32.0)
    faces = O.face_geomean(g, perm)
    b = [-f for f in faces]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    return g, b, f


def c2_options(abi, ops, mixed):
    # library defaults: whole outer loop as one device-resident graph, fused
    # levels; only the stopping rule and the precision are set here
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter = TOL, 1e-15, 300
    o.precision = abi.PREC_MIXED if mixed else abi.PREC_F64
    return o


# Algorithmic bytes of one mixed-precision outer iteration (2D): the FP64
# outer step reads phi, rhs, diag (8 B each), two face weights (16 B), the
# FP32 correction (4 B) and writes phi (8 B) and the FP32 residual (4 B):
# 56 B per finest cell.  Every level above the single-CTA coarse cycle runs
# two lean tile launches: pre-smoothing (r, 1/diag, diag, two FP32 face
# weights in, correction and a quarter-cell restricted residual out: 25 B per
# cell) and post-smoothing (correction, r, 1/diag, face weights and a
# quarter-cell coarse correction in, correction out: 25 B per cell).  The
# coarse cycle (at most 1024-cell top) moves under 1% of that and is left out.
OUTER_BYTES_PER_CELL = 56
TILE_BYTES_PER_CELL = 50
COARSE_CYCLE_CELLS = 1024


def iteration_bytes(n0, n1, levels, cycles=1):
    """Algorithmic bytes of one outer iteration: the FP64 outer step plus
    `cycles` FP32 V-cycles."""
    cells = [(n0 >> l) * (n1 >> l) for l in range(levels)]
    tiled = sum(c for l, c in enumerate(cells) if c > COARSE_CYCLE_CELLS and l < levels - 1)
    return OUTER_BYTES_PER_CELL * cells[0] + cycles * TILE_BYTES_PER_CELL * tiled


def config2(args, torch, abi, ops, O, P):
    """2D 512x512 projection Poisson (the configuration of the earlier
    default line): one complete solve per step, mixed vs FP64."""
    world = 1
    g, b, f = c2_problem()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    db = [dev(x) for x in b]
    df = dev(f)
    op = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, db)
    solvers = {"mixed": ops.AMRMultiGrid(op, c2_options(abi, ops, True)),
               "fp64": ops.AMRMultiGrid(op, c2_options(abi, ops, False))}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ncell = g.n[0] * g.n[1]
    stream = torch.cuda.current_stream()

    def timed(name, steps, warmup):
        S = solvers[name]
        phi = torch.zeros_like(df)
        for _ in range(warmup):
            phi.zero_()
            st, rc = S.solve(phi, df)
            assert rc == 0, "solve failed rc=%d" % rc
        tot_ms, upd, last, launches, iters = 0.0, 0.0, None, 0.0, 0
        for _ in range(steps):
            phi.zero_()
            flush.fill_(1.0)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st, rc = S.solve(phi, df)
            e1.record(stream)
            torch.cuda.synchronize()
            assert rc == 0, "solve failed rc=%d" % rc
            tot_ms += e0.elapsed_time(e1)
            upd += st.cell_updates
            launches += st.kernel_launches
            iters += st.iterations
            last = st
        tot_ms = aggregate_max(tot_ms, world, "cuda")
        return tot_ms, upd, last, phi, launches, iters

    with Clocks() as clk:
        ms_mixed, upd_mixed, st_mixed, phi_mixed, nl_mixed, it_mixed = timed("mixed", args.steps,
                                                                             args.warmup)
        ms_f64, upd_f64, st_f64, phi_f64, nl_f64, it_f64 = timed("fp64", args.steps, args.warmup)

    # error of the mixed solution against the FP64 solution (null space removed)
    a = phi_f64.cpu().numpy()
    m = phi_mixed.cpu().numpy()
    err = float(np.abs((a - a.mean()) - (m - m.mean())).max() / np.abs(a - a.mean()).max())

    # end to end through the C ABI: pinned host rhs -> device -> solve -> host
    h_rhs = torch.from_numpy(f.copy()).pin_memory()
    h_out = torch.empty_like(h_rhs).pin_memory()
    d_rhs = torch.empty_like(df)
    phi = torch.zeros_like(df)
    S = solvers["mixed"]
    for _ in range(args.warmup):
        d_rhs.copy_(h_rhs, non_blocking=True)
        phi.zero_()
        S.solve(phi, d_rhs)
        h_out.copy_(phi, non_blocking=True)
    torch.cuda.synchronize()
    e2e_ms, e2e_upd = 0.0, 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        d_rhs.copy_(h_rhs, non_blocking=True)
        phi.zero_()
        st, rc = S.solve(phi, d_rhs)
        h_out.copy_(phi, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms += e0.elapsed_time(e1)
        e2e_upd += st.cell_updates

    # roofline of the timed unit the events see: one outer iteration of the
    # mixed solve (its ~10 kernels run back to back inside the device-resident
    # graph loop; their individual shares come from the ncu launch list)
    hbm, kind = peaks()
    it_us = ms_mixed * 1e3 / max(it_mixed, 1)
    cyc_per_it = st_mixed.cycles / max(st_mixed.iterations, 1)
    alg_bytes = iteration_bytes(g.n[0], g.n[1], st_mixed.levels, round(cyc_per_it))
    achieved = alg_bytes / (it_us * 1e-6) / 1e9
    clocks = clk.summary()
    value = upd_mixed / (ms_mixed * 1e-3) * world
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "cell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-inner/f64-outer",
        "data": "synthetic (seeded Kozeny-Carman permeability of a Gaussian-filtered porosity)",
        "config": {"workload": "projection Poisson div(Pi grad p)=div u*, 2D 512x512, "
                               "periodic x / Neumann y, to 1e-10 max-norm rel residual",
                   "cells": ncell, "levels": st_mixed.levels, "l2": "flushed (512 MiB write) between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"value": upd_f64 / (ms_f64 * 1e-3) * world, "ms_per_step": ms_f64 / args.steps,
                 "iterations": st_f64.iterations, "cycles": st_f64.cycles,
                 "gpu_launches": int(nl_f64)},
        "mixed": {"iterations": st_mixed.iterations, "cycles": st_mixed.cycles,
                  "final_rel_residual": st_mixed.final_norm / st_mixed.initial_norm,
                  "rel_err_vs_fp64_solution": err},
        "time_to_solution_ratio_fp64_over_mixed": ms_f64 / ms_mixed,
        "e2e": {"value": e2e_upd / (e2e_ms * 1e-3) * world, "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(ncell * 8), "d2h_bytes_per_step": int(ncell * 8)},
        "roofline": {"bound": "hbm", "kernel": "one mixed outer iteration (graph body: FP64 outer "
                                               "step, lean FP32 tiles, single-CTA coarse cycle)",
                     "achieved": achieved, "peak": hbm, "peak_kind": kind, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None,
                     "iteration_us": it_us, "alg_bytes_per_iteration": alg_bytes},
        "clocks": clocks,
        "gpu_launches": int(nl_mixed),
    }
    return line


def config5(args, torch, abi, ops, O, P):
    """Discrete adjoint of a 50-step 256x256 diffusive-convective
    solidification rollout (Ra 2e5, dt 5e-4, checkpoints every 10 steps):
    forward and gradient times, and the gradient against central differences
    along 8 seeded directions in (log-permeability field, Ra, T_bottom)."""
    from mushy_gb300 import darcy_model as M
    n, nsteps, every, Ra, Tb = 256, 50, 10, 2e5, 0.5
    model = M.DarcySolidification(n, dt=5e-4)
    phi0 = M.initial_state(n, seed=5)
    logk = M.log_permeability(n, seed=5, std=0.5)
    scalar = lambda v: torch.tensor(v, dtype=torch.float64, device="cuda")

    def forward_only(lk, ra, tb):
        with torch.no_grad():
            return float(model.run(phi0, lk, scalar(ra), scalar(tb), nsteps, every))

    forward_only(logk, Ra, Tb)  # warm-up: solver graphs, projector workspace
    ms_fwd, J0 = _events_ms(lambda: forward_only(logk, Ra, Tb))

    def gradient():
        lk = logk.clone().requires_grad_(True)
        ra = scalar(Ra).requires_grad_(True)
        tb = scalar(Tb).requires_grad_(True)
        J = model.run(phi0, lk, ra, tb, nsteps, every)
        J.backward()
        return float(J.detach()), lk.grad, float(ra.grad), float(tb.grad)

    its = model.stepper.iterations
    its["forward"].clear()
    ms_grad, (J1, gk, gra, gtb) = _events_ms(gradient)
    fwd_its, adj_its = list(its["forward"]), list(its["adjoint"])
    rng = np.random.default_rng(5)
    # central differences along each direction at three steps: truncation
    # error falls as h^2 while the forward solves' round-off (relative 1e-12
    # residual) grows as 1/h, and which one dominates at a given h depends on
    # the direction, so each direction reports its smallest error over the
    # steps (the finite-difference accuracy limit), and the table of all
    h_steps = (1e-4, 1e-5, 1e-6)
    rels, table, dirs = [], [], []
    t0 = time.time()

    def central(dk, dra, dtb, hh):
        return (forward_only(logk + hh * dk, Ra + hh * dra, Tb + hh * dtb) -
                forward_only(logk - hh * dk, Ra - hh * dra, Tb - hh * dtb)) / (2 * hh)

    for _ in range(8):
        dk = torch.from_numpy(rng.standard_normal(tuple(logk.shape))).cuda()
        dra = float(rng.standard_normal()) * Ra
        dtb = float(rng.standard_normal())
        ad = float((gk * dk).sum()) + gra * dra + gtb * dtb
        row = [abs(ad - fd) / abs(fd) for fd in (central(dk, dra, dtb, hh) for hh in h_steps)]
        table.append(row)
        rels.append(min(row))
        dirs.append((dk, dra, dtb, ad))
    # the direction furthest from the adjoint, over a wider range of steps
    worst = int(np.argmax(rels))
    dk, dra, dtb, ad = dirs[worst]
    sweep = []
    for hh in (3e-4, 1e-4, 3e-5, 1e-5, 3e-6, 1e-6, 3e-7, 1e-7, 1e-8):
        fd = central(dk, dra, dtb, hh)
        sweep.append({"step": hh, "fd": fd, "rel_err": abs(ad - fd) / abs(fd)})
    fd_s = time.time() - t0
    return {"metric": "adjoint gradient of a 50-step 256^2 rollout: time and FD agreement",
            "value": ms_grad, "unit": "ms per gradient (forward + checkpointed backward)",
            "higher_is_better": False, "forward_ms": ms_fwd, "gradient_over_forward": ms_grad / ms_fwd,
            "objective": J0, "objective_in_gradient_run": J1,
            "fd_rel_err": {"max": max(rels), "per_direction": rels,
                           "steps": list(h_steps), "per_direction_per_step": table},
            "fd_step_sweep": {"direction": worst, "adjoint": dirs[worst][3], "steps": sweep},
            "dJ_dRa": gra, "dJ_dTb": gtb, "dJ_dlogk_abs_sum": float(gk.abs().sum()),
            "fd_wall_s": fd_s,
            "solves_in_gradient": {"forward_steps": len(fwd_its),
                                   "forward_newton_iterations_mean": float(np.mean(fwd_its)),
                                   "adjoint": len(adj_its),
                                   "adjoint_iterations_mean": float(np.mean(adj_its))},
            "config": {"workload": "2D 256x256 Darcy solidification, periodic x, T_b=0.5 / "
                                   "T_top=1.3, liquid H=6.3+0.2cos(2 pi x), C=-1, thermal "
                                   "buoyancy Ra=2e5, Da=2e-5, log-permeability std 0.5 "
                                   "(seeded smooth field), dt=5e-4, 50 steps, checkpoints "
                                   "every 10; FP64 Newton steps, projection and adjoint solves to 1e-12",
                       "objective": "final mean solid fraction + mean top heat flux"}}


def run_config(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from mushy_gb300 import abi, ops
    from oracle import oracle as O
    import problems as P
    fn = {1: config1, 2: config2, 3: config3, 5: config5}[args.config]
    line = fn(args, torch, abi, ops, O, P)
    line.update({"n_gpus": 1, "data": "synthetic (seeded)", "config_index": args.config})
    print(json.dumps(line))


def run_profile(args):
    """Short runs for ncu launch lists and captures: c4 / c4-fp64 1 + --warmup
    steps of the 256^3 workload, c2-mixed / c2-fp64
    two 3-iteration solves of the 512^2 projection problem, hc two FAS steps
    at 64^2, adjoint one Newton step and its adjoint solve at 256^2."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from mushy_gb300 import abi, ops
    if args.profile == "hc":
        # two backward-Euler FAS steps of the 64x64 solidification problem
        import problems as P
        g, prm, phi_bc, der, phi0, b, dev, op = _c1_setup(torch, abi, ops, P, 64)
        o = ops.default_options(True)
        o.use_graph = 0
        S = ops.AMRFASMultiGrid(op, o)
        cur = dev(phi0)
        for _ in range(2):
            new = cur.clone()
            st, rc = S.backwardEuler(new, cur, 1e-3)
            cur = new
        torch.cuda.synchronize()
        print(json.dumps({"profile": "hc", "iterations": st.iterations,
                          "kernel_launches": st.kernel_launches}))
        return
    if args.profile == "adjoint":
        # one Newton backward-Euler step and its adjoint solve on the 256^2
        # solidification state (the adjoint workload's first step), plain
        # launches
        from mushy_gb300 import darcy_model as M
        model = M.DarcySolidification(256)
        phi0 = M.initial_state(256, seed=5)
        o = ops.default_options(True)
        o.tolerance, o.hang, o.max_iter, o.use_graph = 1e-12, -1.0, 60, 0
        A = ops.AdjointMultiGrid(model.hop, o)
        new = phi0.clone()
        st_n, rc_n = A.backwardEulerNewton(new, phi0, model.dt)
        g_bar = torch.ones_like(new)
        mu = torch.zeros_like(new)
        _, _, _, st_a, rc_a = A.backwardEulerAdjoint(new, g_bar, model.dt, mu)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "adjoint", "newton_iterations": st_n.iterations,
                          "newton_linear_cycles": st_n.cycles,
                          "adjoint_cycles": st_a.iterations}))
        return
    if args.profile in ("c4", "c4-fp64", "c4-fp64-fast"):
        # one step of the 256^3 workload (or --n^3) with plain launches
        # (profilers do not see kernel nodes inside graphs with conditional
        # nodes)
        prob = c4_problem(torch, abi, ops, n=args.n)
        prec = {"c4": "mixed", "c4-fp64": "fp64", "c4-fp64-fast": "fp64_fast"}[args.profile]
        R = C4Runner(torch, abi, ops, prob, use_graph=0, precs=(prec,))
        for _ in range(1 + args.warmup):
            out = R.step(prec)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, **C4Runner.summary(out)}))
        return
    g, b, f = c2_problem()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    op = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, [dev(x) for x in b])
    o = c2_options(abi, ops, args.profile == "c2-mixed")
    o.max_iter = 3
    # same kernels as the timed solve, launched one by one: profilers do not
    # see kernel nodes inside a graph with a conditional (WHILE) node
    o.use_graph = 0
    S = ops.AMRMultiGrid(op, o)
    for _ in range(2):
        phi = torch.zeros_like(dev(f))
        st, rc = S.solve(phi, dev(f))
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "iterations": st.iterations,
                      "kernel_launches": st.kernel_launches}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=C4_N,
                    help="box edge of the --profile c4 runs (ncu captures of a smaller case)")
    ap.add_argument("--profile", choices=["c4", "c4-fp64", "c4-fp64-fast", "c2-mixed", "c2-fp64",
                                          "hc", "adjoint"],
                    help="run one short solve for a profiler and exit")
    ap.add_argument("--config", type=int, choices=[1, 2, 3, 5],
                    help="measure another configuration (one JSON line) and exit")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
    elif args.config:
        run_config(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
