"""Least-squares fitting through LinearMap + the device LSQR, against the reference's
fitting tests (test/test_LinearMapsExt.jl:14-61) and the oracle's LSQR.

The reference fits random control points back from their evaluation with
IterativeSolvers' lsqr and asks for ``fit ≈ control_points`` with rtol 1e-5 (Julia's
isapprox on arrays: ||fit - ref|| <= rtol * max(||fit||, ||ref||)), on a plain 2D grid
and on a locally refined one.  Here the same cases run through the library's device LSQR
(one graph launch per solve), and the device iterates are checked against the oracle's
restatement of LSQR driven by the oracle's evaluate / evaluate_adjoint.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _isapprox(a, b, rtol):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def _grid(sg, torch, dtype=None):
    dtype = dtype or torch.float64
    dims = tuple(sg.SplineDimension(n, d, s, float_type=dtype)
                 for n, d, s in zip((12, 10), (3, 4), (26, 73)))
    return sg.SplineGrid(dims, 3)


def _spec(oracle, g):
    sidx, bs = [], []
    for d in g.spline_dimensions:
        knots = d.knot_vector.knots_all.cpu().numpy().astype(np.float64)
        samples = d.sample_points.cpu().numpy().astype(np.float64)
        si = oracle.sample_indices(samples, knots, d.degree)
        sidx.append(si)
        bs.append(oracle.basis(knots, samples, si, d.degree, d.max_derivative_order))
    return oracle.GridSpec(sidx, bs, [d.degree for d in g.spline_dimensions],
                           [d.n_basis_functions for d in g.spline_dimensions])


def test_least_squares_fitting(sg):
    """test_LinearMapsExt.jl:14-32: plain grid (12, 10) x degree (3, 4) x samples (26, 73),
    Nout 3, Float64."""
    import torch
    rng = np.random.default_rng(1)
    g = _grid(sg, torch)
    cp_rand = rng.random(tuple(sg.obtain(g.control_points).shape))
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp_rand))
    sg.evaluate_(g)
    A = sg.LinearMap(g)
    assert A.shape == (26 * 73 * 3, 12 * 10 * 3)
    fit, info = sg.lsqr(A, sg.arrays.vec(g.eval).clone(), log=True)
    assert info["istop"] in (1, 2), info
    ref = np.asfortranarray(cp_rand).ravel(order="F")
    assert _isapprox(fit.cpu().numpy(), ref, 1e-5), info


def test_locally_refined_least_squares_fitting(sg):
    """test_LinearMapsExt.jl:34-61: default local refinement, three activated ranges,
    overwritten control points deactivated."""
    import torch
    rng = np.random.default_rng(1)
    g = _grid(sg, torch)
    g = sg.add_default_local_refinement(g)
    sg.activate_local_control_point_range_(g, range(0, 4), range(0, 6))
    sg.activate_local_control_point_range_(g, range(0, 6), range(0, 2))
    sg.activate_local_control_point_range_(g, range(8, 10), range(6, 10))
    sg.deactivate_overwritten_control_points_(g.control_points)
    ncp = sg.get_n_control_points(g)
    cp_rand = rng.random((ncp, 3))
    g.control_points.copy_(torch.as_tensor(cp_rand))
    sg.evaluate_control_points_(g.control_points)
    sg.evaluate_(g)
    target = sg.arrays.vec(g.eval).clone()
    A = sg.LinearMap(g)
    assert A.shape == (26 * 73 * 3, ncp * 3)
    fit, info = sg.lsqr(A, target, log=True)
    assert info["istop"] in (1, 2), info
    assert _isapprox(fit.cpu().numpy(), np.asfortranarray(cp_rand).ravel(order="F"), 1e-5), info


@pytest.mark.parametrize("damp,maxiter", [(0.0, 12), (0.0, None), (0.5, None)])
def test_device_lsqr_matches_oracle(sg, oracle, damp, maxiter):
    """Device LSQR vs the oracle's LSQR on the same operator and a random right-hand side
    (an inconsistent system): the same stop code; after a fixed number of iterations x
    agrees to 1e-9, run to convergence to 1e-6 within two iterations of the oracle."""
    import torch
    rng = np.random.default_rng(2)
    g = _grid(sg, torch)
    spec = _spec(oracle, g)
    cps = tuple(sg.obtain(g.control_points).shape)
    evs = tuple(g.eval.shape)
    b = rng.standard_normal(int(np.prod(evs)))
    mv = lambda x: oracle.evaluate(spec, np.asfortranarray(x.reshape(cps, order="F"))).ravel(order="F")
    rmv = lambda y: oracle.evaluate_adjoint(spec, np.asfortranarray(y.reshape(evs, order="F"))).ravel(order="F")
    x_ref, istop, itn, _ = oracle.lsqr(mv, rmv, b, int(np.prod(cps)), damp=damp, maxiter=maxiter)
    A = sg.LinearMap(g)
    solver = sg.LSQRSolver(A, damp=damp, maxiter=maxiter)
    x = solver.solve(torch.as_tensor(b, device="cuda"))
    info = solver.info()
    assert info["istop"] == istop, (info, istop, itn)
    if maxiter is not None:
        # a fixed number of iterations: the iterates agree to rounding
        assert info["iterations"] == itn == maxiter
        assert np.abs(x.cpu().numpy() - x_ref).max() <= 1e-9 * np.abs(x_ref).max()
    else:
        # run to convergence: rounding differences may move the stop by an iteration
        assert abs(info["iterations"] - itn) <= 2, (info, itn)
        assert np.abs(x.cpu().numpy() - x_ref).max() <= 1e-6 * np.abs(x_ref).max()


def test_graph_and_eager_agree_bitwise_and_relaunch(sg):
    """The captured while-loop solve equals the host-driven loop bit for bit, and a
    relaunch with a new right-hand side starts afresh."""
    import torch
    rng = np.random.default_rng(3)
    g = _grid(sg, torch)
    A = sg.LinearMap(g)
    b1 = torch.as_tensor(rng.standard_normal(A.shape[0]), device="cuda")
    b2 = torch.as_tensor(rng.standard_normal(A.shape[0]), device="cuda")
    gs = sg.LSQRSolver(A, maxiter=40)
    es = sg.LSQRSolver(A, maxiter=40, graph=False)
    for b in (b1, b2, b1):
        xg = gs.solve(b)
        ig = gs.info()
        xe = es.solve(b)
        ie = es.info()
        assert torch.equal(xg, xe)
        assert ig["iterations"] == ie["iterations"] and ig["istop"] == ie["istop"]
    x_first = gs.solve(b1)
    assert torch.equal(x_first, xg)


def test_float32_fit_and_derivative_map(sg, oracle):
    """Float32 grid: the fit stops at the Float32 default tolerances and, with tighter
    ones, reaches Float32's attainable accuracy; a derivative-order map applies the
    derivative basis (forward against the oracle) and its adjoint is the transpose."""
    import torch
    rng = np.random.default_rng(4)
    g = _grid(sg, torch, torch.float32)
    cp = rng.random(tuple(sg.obtain(g.control_points).shape)).astype(np.float32)
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp))
    sg.evaluate_(g)
    # the Float32 defaults (atol = btol = sqrt(eps) = 3.5e-4) stop at a relative residual
    # of that size; with cond(A) ~ 500 the control points are then off by ~1e-2
    b = sg.arrays.vec(g.eval).clone()
    fit, info = sg.lsqr(sg.LinearMap(g), b, log=True)
    assert info["istop"] in (1, 2), info
    tol = float(np.sqrt(np.finfo(np.float32).eps))
    if info["istop"] == 1:  # the paper's rule 1, from the solver's own estimates
        assert info["rnorm"] / info["bnorm"] <= 1.0001 * (
            tol + tol * info["anorm"] * info["xnorm"] / info["bnorm"])
    assert _isapprox(fit.cpu().numpy(), cp.ravel(order="F"), 5e-2), info
    # tighter tolerances reach Float32's attainable accuracy (~cond * eps)
    fit, info = sg.lsqr(sg.LinearMap(g), b, atol=1e-7, btol=1e-7, maxiter=400, log=True)
    assert _isapprox(fit.cpu().numpy(), cp.ravel(order="F"), 1e-3), info

    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=1, float_type=torch.float64)
                 for n, d, s in zip((12, 10), (3, 4), (26, 73)))
    gd = sg.SplineGrid(dims, 2)
    A = sg.LinearMap(gd, derivative_order=(1, 0))
    x = torch.as_tensor(rng.standard_normal(A.shape[1]), device="cuda")
    y = A @ x
    spec = _spec(oracle, gd)
    cps = tuple(sg.obtain(gd.control_points).shape)
    ref = oracle.evaluate(spec, np.asfortranarray(x.cpu().numpy().reshape(cps, order="F")),
                          order=(1, 0)).ravel(order="F")
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    # and its adjoint is the transpose: <A x, y'> == <x, A' y'>
    yp = torch.as_tensor(rng.standard_normal(A.shape[0]), device="cuda")
    lhs = float(torch.dot(A @ x, yp))
    rhs = float(torch.dot(x, A.T @ yp))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1.0)
