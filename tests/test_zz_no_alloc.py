"""mlgpu_vc_jacobi_noalloc (temporary in a fixed device array) against
mlgpu_vc_jacobi (temporary provided by the caller).

Both run the same sm_103a Jacobi kernel, so the tolerance is zero: two calls
in a row must give the same bits in FP64 and in FP32.  Sizes above the fixed
scratch are refused with MLGPU_ERR_SCRATCH before anything is launched.
"""
import ctypes as C

import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    yield


def _op(n, per, dtype, seed):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    b = [x[0] for x in P.faces(g, rng, 1)]
    a = rng.uniform(0.5, 1.5, abi.cell_shape(g))
    c = rng.uniform(0.1, 3.0, abi.cell_shape(g))
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda().to(dtype)
    op = ops.DarcyBrinkmanOp(g, P.vc_bc("mixed"), 0.7, -0.9, dev(a), [dev(x) for x in b], dev(c))
    phi = dev(rng.standard_normal(abi.cell_shape(g)))
    rhs = dev(rng.standard_normal(abi.cell_shape(g)))
    return op, phi, rhs


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("n,per,dtype", [
    ((64, 48), (1, 0, 0), torch.float64),
    ((40, 24), (0, 1, 0), torch.float32),
    ((16, 12, 8), (1, 0, 1), torch.float64),
    ((1024, 1024), (1, 0, 0), torch.float64),   # exactly the FP64 limit
])
def test_noalloc_jacobi_matches_tmp_version(n, per, dtype):
    op, phi, rhs = _op(n, per, dtype, 91)
    lib = abi.load()
    desc = op.desc()
    a, b = phi.clone(), phi.clone()
    tmp = torch.empty_like(phi)
    for _ in range(2):
        abi.check(lib.mlgpu_vc_jacobi(C.byref(desc), C.c_void_p(a.data_ptr()),
                                      C.c_void_p(rhs.data_ptr()), C.c_void_p(tmp.data_ptr()),
                                      _stream()), "vc_jacobi")
        abi.check(lib.mlgpu_vc_jacobi_noalloc(C.byref(desc), C.c_void_p(b.data_ptr()),
                                              C.c_void_p(rhs.data_ptr()), _stream()),
                  "vc_jacobi_noalloc")
    torch.cuda.synchronize()
    assert not torch.equal(a, phi)
    assert torch.equal(a, b)


def test_noalloc_jacobi_refuses_oversize():
    op, phi, rhs = _op((1024, 1025), (1, 0, 0), torch.float64, 92)
    before = phi.clone()
    rc = abi.load().mlgpu_vc_jacobi_noalloc(C.byref(op.desc()), C.c_void_p(phi.data_ptr()),
                                            C.c_void_p(rhs.data_ptr()), _stream())
    assert rc == abi.ERR_SCRATCH
    torch.cuda.synchronize()
    assert torch.equal(phi, before)
    # the same cell count fits in FP32 (4-byte cells)
    op32, phi32, rhs32 = _op((1024, 1025), (1, 0, 0), torch.float32, 92)
    rc = abi.load().mlgpu_vc_jacobi_noalloc(C.byref(op32.desc()), C.c_void_p(phi32.data_ptr()),
                                            C.c_void_p(rhs32.data_ptr()), _stream())
    assert rc == abi.OK
