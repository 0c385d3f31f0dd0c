"""torch.autograd over the discrete adjoint: gradients of the
diffusive-convective solidification objective with respect to the per-cell
log-permeability, Ra and the bottom temperature, through checkpointed time
stepping, against central finite differences of the forward model."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    yield


def _problem(n=32):
    from mushy_gb300 import darcy_model as M
    model = M.DarcySolidification(n, dt=5e-4)
    phi0 = M.initial_state(n, seed=5)
    logk = M.log_permeability(n, seed=5)
    return model, phi0, logk


def _grads(model, phi0, logk, Ra, Tb, nsteps, every):
    lk = logk.clone().requires_grad_(True)
    ra = torch.tensor(Ra, dtype=torch.float64, device="cuda", requires_grad=True)
    tb = torch.tensor(Tb, dtype=torch.float64, device="cuda", requires_grad=True)
    J = model.run(phi0, lk, ra, tb, nsteps, every)
    J.backward()
    return float(J.detach()), lk.grad.clone(), float(ra.grad), float(tb.grad)


def test_checkpointing_gives_the_same_gradient():
    model, phi0, logk = _problem()
    a = _grads(model, phi0, logk, 2e5, 0.5, 6, 6)
    b = _grads(model, phi0, logk, 2e5, 0.5, 6, 2)
    assert a[0] == b[0]
    assert torch.equal(a[1], b[1]) and a[2] == b[2] and a[3] == b[3]


def test_gradient_matches_finite_differences():
    model, phi0, logk = _problem()
    Ra, Tb, nsteps = 2e5, 0.5, 6
    J0, gk, gra, gtb = _grads(model, phi0, logk, Ra, Tb, nsteps, 3)
    # the flow matters: the permeability and Ra gradients are not round-off
    assert abs(gra) * Ra > 1e-6 * abs(J0) and float(gk.abs().max()) > 1e-8 * abs(J0)
    rng = np.random.default_rng(7)
    h = 1e-6
    for _ in range(3):
        dk = torch.from_numpy(rng.standard_normal(tuple(logk.shape))).cuda()
        dra = float(rng.standard_normal()) * Ra
        dtb = float(rng.standard_normal())

        def J(s):
            with torch.no_grad():
                return float(model.run(phi0, logk + s * dk,
                                       torch.tensor(Ra + s * dra, dtype=torch.float64,
                                                    device="cuda"),
                                       torch.tensor(Tb + s * dtb, dtype=torch.float64,
                                                    device="cuda"), nsteps, 3))
        fd = (J(h) - J(-h)) / (2 * h)
        ad = float((gk * dk).sum()) + gra * dra + gtb * dtb
        assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)


def test_revolve_schedule_gives_the_same_gradient():
    """Binomial checkpointing with 2 snapshots over 6 steps reverses the
    same rollout as the segment checkpoints (recomputation is bitwise
    deterministic; parameter gradients summed in another order)."""
    model, phi0, logk = _problem()
    a = _grads(model, phi0, logk, 2e5, 0.5, 6, 3)
    lk = logk.clone().requires_grad_(True)
    ra = torch.tensor(2e5, dtype=torch.float64, device="cuda", requires_grad=True)
    tb = torch.tensor(0.5, dtype=torch.float64, device="cuda", requires_grad=True)
    J = model.run(phi0, lk, ra, tb, 6, snapshots=2)
    J.backward()
    assert float(J.detach()) == a[0]
    assert torch.allclose(lk.grad, a[1], rtol=1e-10, atol=1e-16)
    assert abs(float(ra.grad) - a[2]) <= 1e-10 * abs(a[2])
    assert abs(float(tb.grad) - a[3]) <= 1e-10 * abs(a[3])
