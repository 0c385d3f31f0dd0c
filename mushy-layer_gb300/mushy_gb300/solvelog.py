"""JSON-lines log of the solves, one line per solve: what ran (solver kind,
box, precision, stopping rule), how it ended (status code and the
reference's exit status: 0 converged, 2 hang, 4 iteration limit, 8
non-finite), the FP64 residual history, the work (cell updates, kernel
launches), the host wall time of the call and the algorithmic bytes and
bandwidth that work implies.

The reference reports the same facts per solve in its log lines (exit
status, residual and iterations of the (H, C) solve,
srcSubcycle/AMRLevelMushyLayer.cpp:1806-1809; "MAC Projection ... exit
status" in srcSubcycle/Projector.cpp).

Algorithmic bytes per cell update follow the stencil-sweep model: read the
state, the right-hand side and one face coefficient per direction per
component, write the state: s n_c (3 + D + [a]) for the (H, C) operator,
s (3 + D + [a] + [c]) for the projection / Darcy-Brinkman operator, s = 8
in FP64.  In mixed precision every outer iteration's FP64 residual over the
finest box counts at s = 8 and the remaining updates (FP32 cycles) at s = 4.
"""
import json
import time

from . import abi

_STATUS = {abi.OK: "ok", abi.ERR_ARG: "bad argument", abi.ERR_CUDA: "cuda error",
           abi.ERR_NAN: "non-finite", abi.ERR_NOT_CONVERGED: "not converged",
           abi.ERR_WORKSPACE: "workspace", abi.ERR_HANG: "hang", abi.ERR_SCRATCH: "scratch"}


def bytes_per_cell_update(kind, dim, elem, has_a=False, has_c=False):
    """Stencil-sweep bytes of one cell update (kind "hc" / "adj": two
    components; "vc": one)."""
    if kind in ("hc", "adj"):
        return elem * 2 * (3 + dim + int(has_a))
    return elem * (3 + dim + int(has_a) + int(has_c))


class SolveLog:
    """Appends one JSON object per solve to `sink` (a path, opened for
    append, or a writable text stream) and keeps the records in memory."""

    def __init__(self, sink=None):
        self.records = []
        self._own = isinstance(sink, str)
        self._f = open(sink, "a") if self._own else sink

    def close(self):
        if self._own and self._f:
            self._f.close()
        self._f = None

    def record(self, what, kind, grid, opts, st, rc, seconds, has_a=False, has_c=False):
        dim = int(grid.dim)
        n = [int(grid.n[d]) for d in range(3)]
        cells0 = n[0] * n[1] * n[2]
        mixed = int(opts.precision) == abi.PREC_MIXED
        upd = float(st.cell_updates)
        b64 = bytes_per_cell_update(kind, dim, 8, has_a, has_c)
        if mixed:
            fp64 = min(upd, (st.iterations + 1) * float(cells0))
            alg = fp64 * b64 + (upd - fp64) * bytes_per_cell_update(kind, dim, 4, has_a, has_c)
        else:
            alg = upd * b64
        hist = [float(st.norm_history[i]) for i in range(min(int(st.iterations) + 1, 64))]
        line = {
            "what": what, "solver": kind, "cells": n[:dim], "dx": float(grid.dx),
            "precision": "mixed" if mixed else "f64",
            "tolerance": float(opts.tolerance), "max_iter": int(opts.max_iter),
            "rc": int(rc), "status": _STATUS.get(int(rc), "code %d" % int(rc)),
            "exit_status": int(st.exit_status), "iterations": int(st.iterations),
            "cycles": int(st.cycles), "levels": int(st.levels),
            "initial_norm": float(st.initial_norm), "final_norm": float(st.final_norm),
            "residual_history": hist,
            "cell_updates": upd, "kernel_launches": float(st.kernel_launches),
            "seconds": float(seconds),
            "cell_updates_per_s": upd / seconds if seconds > 0 else None,
            "alg_bytes": alg,
            "alg_gbs": alg / seconds / 1e9 if seconds > 0 else None,
            "time": time.time(),
        }
        self.records.append(line)
        if self._f is not None:
            # NaN / Inf norms are written as JSON null
            self._f.write(json.dumps(_finite(line)) + "\n")
            self._f.flush()
        return line


def _finite(v):
    if isinstance(v, float) and (v != v or v in (float("inf"), float("-inf"))):
        return None
    if isinstance(v, list):
        return [_finite(x) for x in v]
    if isinstance(v, dict):
        return {k: _finite(x) for k, x in v.items()}
    return v
