"""Differentiating a loss through evaluate! with respect to the control points (the
reference's Enzyme test, test/test_EnzymeExt.jl:14-60: loss = sum(eval) on a (10, 10)
degree-2 grid with 50 x 50 samples and Nout 2 gives a nonzero gradient) through torch
autograd, whose backward is the library's adjoint."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gradient_of_sum_is_the_adjoint_of_ones(sg):
    import torch
    dims = tuple(sg.SplineDimension(10, 2, 50) for _ in range(2))
    g = sg.SplineGrid(dims, 2)
    rng = np.random.default_rng(1)
    cp = sg.arrays.from_any(torch.as_tensor(rng.random((10, 10, 2), dtype=np.float32)),
                            torch.float32)
    cp.requires_grad_(True)
    loss = sg.autograd.evaluate(g, cp).sum()
    loss.backward()
    assert cp.grad is not None and bool((cp.grad != 0).any())
    ones = sg.arrays.ones(tuple(g.eval.shape), torch.float32)
    ref = sg.arrays.empty((10, 10, 2), torch.float32)
    sg.evaluate_adjoint_(g, eval=ones, control_points=ref)
    assert torch.equal(cp.grad, ref)
    # the forward value is evaluate!'s
    ev = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
    sg.evaluate_(g, control_points=cp.detach(), eval=ev)
    assert torch.equal(sg.autograd.evaluate(g, cp.detach()), ev)


def test_gradient_matches_finite_differences_fp64(sg):
    """A nonlinear loss in FP64: autograd gradient vs central differences (h = 1e-6)."""
    import torch
    dims = (sg.SplineDimension(9, 3, 40, max_derivative_order=1, float_type=torch.float64),
            sg.SplineDimension(7, 2, 33, max_derivative_order=1, float_type=torch.float64))
    g = sg.SplineGrid(dims, 3)
    rng = np.random.default_rng(2)
    cp0 = torch.as_tensor(rng.standard_normal((9, 7, 3)))
    target = torch.as_tensor(rng.standard_normal(tuple(g.eval.shape))).cuda()

    def loss_of(cp):
        ev = sg.autograd.evaluate(g, cp, derivative_order=(1, 0))
        return ((ev - target) ** 2).sum() + (ev ** 3).mean()

    cp = sg.arrays.from_any(cp0, torch.float64).requires_grad_(True)
    loss_of(cp).backward()
    grad = cp.grad.cpu().numpy()
    h = 1e-6
    for flat in rng.choice(cp0.numel(), 12, replace=False):
        idx = np.unravel_index(flat, cp0.shape)
        vals = []
        for sgn in (1, -1):
            c = cp0.clone()
            c[idx] += sgn * h
            with torch.no_grad():
                vals.append(float(loss_of(sg.arrays.from_any(c, torch.float64))))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(grad[idx] - fd) <= 1e-5 * max(1.0, abs(fd)), (idx, grad[idx], fd)
