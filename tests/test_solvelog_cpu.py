"""The JSON-lines solve log (mushy_gb300/solvelog.py) and the hook every
solver wrapper of mushy_gb300/ops.py calls, driven on the host with filled
stats records (the solves themselves run in the GPU tests)."""
import ctypes as C
import io
import json
import types

import pytest

from mushy_gb300 import abi
from mushy_gb300 import solvelog


def _opts(hc, mixed=False):
    o = abi.MGOptions()
    abi.load().mlgpu_mg_default_options(C.byref(o), int(hc))
    if mixed:
        o.precision = abi.PREC_MIXED
    return o


def _stats(iters, updates, status=0, hist=None):
    st = abi.SolveStats()
    st.iterations, st.cycles, st.levels = iters, 3 * iters, 7
    st.exit_status = status
    st.cell_updates = updates
    st.kernel_launches = 42
    hist = hist or [10.0 ** -k for k in range(iters + 1)]
    st.initial_norm, st.final_norm = hist[0], hist[-1]
    for i, v in enumerate(hist):
        st.norm_history[i] = v
    return st


def test_bytes_model():
    # (H, C) 2D FP64 with a: 2 * 8 * (3 + 2 + 1) = 96 B, the sweep model's figure
    assert solvelog.bytes_per_cell_update("hc", 2, 8, has_a=True) == 96
    assert solvelog.bytes_per_cell_update("hc", 3, 8, has_a=True) == 112
    # projection (no a, no c): 8 (3 + D)
    assert solvelog.bytes_per_cell_update("vc", 2, 8) == 40
    assert solvelog.bytes_per_cell_update("vc", 3, 8) == 48
    # Darcy-Brinkman adds c
    assert solvelog.bytes_per_cell_update("vc", 2, 8, has_a=True, has_c=True) == 56


def test_record_fp64_and_mixed():
    buf = io.StringIO()
    log = solvelog.SolveLog(buf)
    g = abi.make_grid([64, 32], 1.0 / 64)
    st = _stats(4, 64 * 32 * 10.0)
    rec = log.record("solve", "vc", g, _opts(False), st, abi.OK, 0.002)
    assert rec["cells"] == [64, 32] and rec["precision"] == "f64" and rec["status"] == "ok"
    assert rec["residual_history"] == [1.0, 0.1, 0.01, 0.001, 0.0001]
    assert rec["alg_bytes"] == 64 * 32 * 10.0 * 40
    assert rec["alg_gbs"] == pytest.approx(rec["alg_bytes"] / 0.002 / 1e9)
    assert rec["cell_updates_per_s"] == pytest.approx(64 * 32 * 10.0 / 0.002)
    # mixed: (iterations + 1) FP64 residuals over the finest box, the rest FP32
    st = _stats(2, 64 * 32 * 20.0)
    rec = log.record("solve", "vc", g, _opts(False, mixed=True), st, abi.OK, 0.001)
    assert rec["precision"] == "mixed"
    assert rec["alg_bytes"] == 3 * 64 * 32 * 40 + 17 * 64 * 32 * 20
    lines = buf.getvalue().splitlines()
    assert len(lines) == 2 and json.loads(lines[0])["iterations"] == 4
    assert len(log.records) == 2


def test_record_failure_writes_valid_json(tmp_path):
    path = str(tmp_path / "solves.jsonl")
    log = solvelog.SolveLog(path)
    g = abi.make_grid([16, 16, 16], 1.0 / 16)
    st = _stats(0, 16.0 ** 3, status=8, hist=[float("nan")])
    rec = log.record("solve", "hc", g, _opts(True), st, abi.ERR_NAN, 0.0)
    log.close()
    assert rec["status"] == "non-finite" and rec["exit_status"] == 8
    assert rec["alg_gbs"] is None and rec["cells"] == [16, 16, 16]
    d = json.loads(open(path).read())
    assert d["initial_norm"] is None and d["residual_history"] == [None]


def test_ops_hook_records_through_the_installed_log():
    import time
    from mushy_gb300 import ops
    buf = io.StringIO()
    ops.setSolveLog(solvelog.SolveLog(buf))
    try:
        desc = abi.VCOp()
        desc.grid = abi.make_grid([32, 32], 1.0 / 32)
        solver = types.SimpleNamespace(kind="vc", desc=desc, opts=_opts(False))
        ops._log("levelMacProject", solver, _stats(3, 32 * 32 * 8.0), abi.ERR_HANG,
                 time.perf_counter())
    finally:
        ops.setSolveLog(None)
    rec = json.loads(buf.getvalue())
    assert rec["what"] == "levelMacProject" and rec["status"] == "hang"
    assert rec["cells"] == [32, 32] and rec["alg_bytes"] == 32 * 32 * 8.0 * 40
    # without a log the hook does nothing
    ops._log("solve", None, None, 0, 0.0)
