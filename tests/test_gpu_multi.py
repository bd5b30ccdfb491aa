"""evaluate_multi_: several derivative orders of one grid in one call (shared prefix
passes), against separate evaluate_ calls (bitwise) and the oracle."""
import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu


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


def _grid(sg, torch, ncp, deg, ns, nout, dtype, maxd, seed):
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=min(maxd, d), float_type=dtype)
                 for n, d, s in zip(ncp, deg, ns))
    g = sg.SplineGrid(dims, nout)
    rng = np.random.default_rng(seed)
    cp = rng.standard_normal(tuple(sg.obtain(g.control_points).shape))
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp))
    return g, cp


CASES = [
    # (n_control, degree, samples, nout, dtype, orders)
    ((37, 29), (3, 2), (301, 257), 3, "float32",
     [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2), (1, 0)]),
    ((12, 9, 7), (3, 2, 3), (65, 48, 33), 2, "float64",
     [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (2, 0, 1)]),
    ((40,), (3,), (513,), 1, "float32", [(0,), (1,), (2,)]),
    ((6, 5, 5, 4), (2, 1, 2, 1), (17, 9, 11, 8), 1, "float64",
     [(0, 0, 0, 0), (1, 0, 0, 0), (0, 1, 0, 1)]),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"nin{len(c[0])}_{c[4]}")
def test_multi_order_matches_separate_calls_and_oracle(sg, oracle, case):
    import torch
    ncp, deg, ns, nout, dt, orders = case
    dtype = getattr(torch, dt)
    g, cp = _grid(sg, torch, ncp, deg, ns, nout, dtype, 2, 11)
    evals = sg.evaluate_multi_(g, orders)
    spec = _spec(oracle, g)
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    for o, ev in zip(orders, evals):
        sep = sg.arrays.empty(tuple(g.eval.shape), dtype)
        sg.evaluate_(g, derivative_order=o, eval=sep)
        assert torch.equal(ev, sep), o
        ref = oracle.evaluate(spec, np.asfortranarray(cp), order=list(o))
        assert normwise_rel(ev.cpu().numpy(), ref) <= tol, o


def test_multi_order_bf16_control_points_and_nurbs(sg):
    import torch
    g, cp = _grid(sg, torch, (33, 21), (3, 3), (200, 150), 2, torch.float32, 1, 12)
    cpb = sg.arrays.empty(tuple(sg.obtain(g.control_points).shape), torch.bfloat16)
    cpb.copy_(sg.obtain(g.control_points))
    orders = [(0, 0), (1, 0), (0, 1), (1, 1)]
    evals = sg.evaluate_multi_(g, orders, control_points=cpb)
    for o, ev in zip(orders, evals):
        sep = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
        sg.evaluate_(g, derivative_order=o, eval=sep, control_points=cpb)
        assert torch.equal(ev, sep), o
    # NURBS: order zero only, like evaluate!; derivatives are rejected with the
    # reference's message
    ng = sg.NURBSGrid(g.spline_dimensions, 2)
    ng.weights.copy_(torch.rand_like(ng.weights) + 0.5)
    (e0,) = sg.evaluate_multi_(ng, [(0, 0)])
    sep = sg.arrays.empty(tuple(ng.eval.shape), torch.float32)
    sg.evaluate_(ng, eval=sep)
    assert torch.equal(e0, sep)
    with pytest.raises(ValueError, match="Computing derivatives of NURBS"):
        sg.evaluate_multi_(ng, [(0, 0), (1, 0)])
