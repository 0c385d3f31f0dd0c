"""Binomial (revolve) checkpointing of mushy_gb300.adjoint on the CPU with a
toy differentiable step: gradients equal plain autograd through the unrolled
loop and the step count of the reversal is the schedule's optimum."""
import pytest

torch = pytest.importorskip("torch")

from mushy_gb300.adjoint import revolve, revolve_schedule  # noqa: E402


def _toy(counter):
    def step(s, w, c):
        counter[0] += 1
        return torch.tanh(w * s + c * torch.roll(s, 1)) + 0.1 * s
    return step


def test_schedule_known_values():
    cost, split = revolve_schedule(10, 3)
    # no snapshot: restart from the first state for every step
    assert cost[10][0] == 55
    # more snapshots never cost more, and enough snapshots give one pass
    for n in range(1, 11):
        for s in range(1, 4):
            assert cost[n][s] <= cost[n][s - 1]
    cost2, _ = revolve_schedule(8, 7)
    assert cost2[8][7] == 8 + 7  # advance 1 step per snapshot, then one taped step each


@pytest.mark.parametrize("n,s", [(1, 0), (5, 0), (7, 2), (12, 3), (20, 4)])
def test_revolve_gradient_matches_plain_autograd(n, s):
    torch.manual_seed(n * 10 + s)
    x0 = torch.randn(16, dtype=torch.float64, requires_grad=True)
    w = torch.randn(16, dtype=torch.float64, requires_grad=True)
    c = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    counter = [0]
    step = _toy(counter)
    y = x0
    for _ in range(n):
        y = step(y, w, c)
    (y ** 2).sum().backward()
    ref = (x0.grad.clone(), w.grad.clone(), c.grad.clone())
    for t in (x0, w, c):
        t.grad = None
    counter[0] = 0
    yr = revolve(step, x0, n, s, w, c)
    assert torch.equal(yr.detach(), y.detach())
    fwd = counter[0]
    (yr ** 2).sum().backward()
    back = counter[0] - fwd
    cost, _ = revolve_schedule(n, s)
    assert fwd == n and back == cost[n][s]
    for a, b in zip((x0.grad, w.grad, c.grad), ref):
        assert torch.allclose(a, b, rtol=1e-12, atol=1e-14)


def test_schedule_is_the_binomial_optimum():
    """The dynamic program reproduces Griewank and Walther's minimal number
    of forward steps for reversing n steps with c checkpoints (the first
    state counted): t n - C(c + t, t - 1), t the least with C(c + t, t) >= n."""
    from math import comb

    def optimum(n, c):
        t = 0
        while comb(c + t, t) < n:
            t += 1
        return t * n - comb(c + t, t - 1) if t > 0 else 0

    cost, _ = revolve_schedule(80, 9)
    for n in range(1, 81):
        for s in range(0, 9):
            assert cost[n][s] - n == optimum(n, s + 1), (n, s)
