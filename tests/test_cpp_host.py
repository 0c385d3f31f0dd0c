"""C++ host classes (include/mlgpu.hpp): the header compiles against the C
ABI and links against libmlgpu.so alone (CPU), and a program written with
the reference's method names reproduces the oracle bit for bit (GPU)."""
import json
import os
import subprocess

import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "host_classes.cpp")
LIBDIR = os.path.join(ROOT, "mushy-layer_gb300", "_build")


def _build_program(out, src=SRC):
    import __graft_entry__
    __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           src, "-o", out, "-L", LIBDIR, "-lmlgpu", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_host_classes_compile_and_link(tmp_path):
    _build_program(str(tmp_path / "host_classes"))


def test_cpp_host_logic_without_gpu(tmp_path):
    """Box arithmetic, the factories' coarsening limit and the status-code
    exceptions of the C++ layer, run on the host."""
    exe = str(tmp_path / "host_logic")
    _build_program(exe, os.path.join(ROOT, "tests", "cpp", "host_logic.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.stdout, r.stderr)


@pytest.mark.gpu
def test_cpp_host_classes_match_oracle(tmp_path):
    nx, ny = 32, 16
    exe = str(tmp_path / "host_classes")
    _build_program(exe)
    rng = np.random.default_rng(70)
    g = abi.make_grid([nx, ny], 1.0 / nx)
    p = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                        specificHeatRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 0, 1): (abi.BC_DIRICHLET, -1.0),
                       (1, 1, 0): (abi.BC_DIRICHLET, 0.5), (1, 1, 1): (abi.BC_DIRICHLET, -1.0)})
    phi = P.hc_state(g, rng)
    rhs = phi + 0.01 * rng.standard_normal(phi.shape)
    b = P.faces(g, rng, 2)
    vb = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(2)]
    f = rng.standard_normal(abi.cell_shape(g))
    f -= f.mean()
    for name, arr in (("phi", phi), ("rhs", rhs), ("bx", b[0]), ("by", b[1]),
                      ("pb0", vb[0]), ("pb1", vb[1]), ("f", f)):
        np.ascontiguousarray(arr, dtype=np.float64).tofile(str(tmp_path / (name + ".bin")))
    r = subprocess.run([exe, str(tmp_path), str(nx), str(ny)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    stats = json.loads(r.stdout.strip().splitlines()[-1])
    out = lambda name, shape: np.fromfile(str(tmp_path / ("out_" + name + ".bin"))).reshape(shape)

    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -1e-3, None, b)
    assert np.array_equal(out("residual", phi.shape), O.nl_residual(ref, phi, rhs))
    assert np.array_equal(out("gsrb", phi.shape), O.nl_relax(ref, phi, rhs, 1))
    # MGnewOp: coefficients averaged, applied to the restricted state
    cg = abi.make_grid([nx // 2, ny // 2], 2.0 / nx)
    cb = [O.coarsen_faces(g, 2, d, b[d]) for d in range(2)]
    cref = O.NLOpHost(cg, p, phi_bc, der, 1.0, -1e-3, None, cb)
    pc = O.restrict_average(g, 2, phi)
    assert np.array_equal(out("coarse_apply", pc.shape), O.nl_apply(cref, pc))
    sol, st, rc = O.hc_solve(ref, O.default_options(1), phi, rhs)
    assert stats["fas_iterations"] == st.iterations and stats["fas_status"] == st.exit_status
    assert np.array_equal(out("fas", phi.shape), sol)
    tga, st_t, rc_t = O.hc_tga_step(ref, O.default_options(1), phi, phi, 1e-3)
    assert np.array_equal(out("tga", phi.shape), tga)
    vref = O.VCOpHost(g, abi.make_bc(), 0.0, 1.0, None, vb)
    cvb = [O.coarsen_faces(g, 1, d, vb[d]) for d in range(2)]
    cvref = O.VCOpHost(cg, abi.make_bc(), 0.0, 1.0, None, cvb)
    fc = O.restrict_average(g, 1, f)
    assert np.array_equal(out("projection_coarse_apply", fc.shape), O.vc_apply(cvref, fc))
    psol, pst, prc = O.vc_solve(vref, O.default_options(0), np.zeros(abi.cell_shape(g)), f)
    assert stats["projection_iterations"] == pst.iterations
    assert np.array_equal(out("projection", abi.cell_shape(g)), psol)
