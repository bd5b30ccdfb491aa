"""NURBS + 3-level local refinement in 3D at full size, against the FP64 oracle.

Base n_control (16, 16, 8), degree 2, three default local refinements (every knot
span bisected: (30, 30, 14) -> (58, 58, 26) -> (114, 114, 50)), each activating a
seeded random box of ~25 % of the level's control points; samples (512, 512, 256),
Nout 1, FP32 on the GPU.  The finest control points come from the refinement chain
(evaluate!(::LocallyRefinedControlPoints): mult! then the overwrite, per level), which
the oracle recomputes from the same level data.  NURBS variant: weights U[0.5, 2] on
the finest grid, forward.  Plain variant: forward and adjoint.  The reference cannot
refine NURBS grids (src/refinement.jl:220), so the NURBS variant is pinned to the
oracle only.
"""
import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


def _np(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def _build(sg, torch):
    rng = np.random.default_rng(6)
    dims = tuple(sg.SplineDimension(n, 2, s) for n, s in zip((16, 16, 8), (512, 512, 256)))
    g = sg.SplineGrid(dims, 1)
    sg.obtain(g.control_points).copy_(torch.as_tensor(rng.standard_normal((16, 16, 8, 1))))
    for _ in range(3):
        g = sg.add_default_local_refinement(g)
        shape = sg.obtain(g.control_points).shape[:-1]
        ranges = []
        for n in shape:
            ln = max(1, int(round(n * 0.25 ** (1 / 3))))
            s0 = int(rng.integers(0, n - ln + 1))
            ranges.append(range(s0, s0 + ln))
        sg.activate_local_control_point_range_(g, *ranges)
    cps = g.control_points
    # every level's overwritten values become seeded random numbers
    for lr in cps.local_refinements:
        v = rng.standard_normal(tuple(lr.refinement_values.shape))
        lr.refinement_values.copy_(torch.as_tensor(v))
    sg.evaluate_control_points_(cps)
    return g, rng


def _oracle_chain(oracle, cps):
    """The finest control points from the level data, in FP64 on the CPU."""
    lrs = cps.local_refinements
    shapes = [tuple(c.shape) for c in cps.control_points_refined]
    prev = None
    for i, lr in enumerate(lrs):
        if i == 0:
            cur = np.zeros(shapes[0], dtype=np.float64, order="F")
        else:
            cur = oracle.mult(shapes[i], lr.refinement_matrices, prev, lr.dims_refinement,
                              dtype=np.float64)
        oracle.local_refinement(cur, lr.refinement_indices.cpu().numpy(),
                                lr.refinement_values.cpu().numpy().astype(np.float64))
        prev = cur
    return prev


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


def test_config5_refinement_chain_nurbs_and_plain(sg, oracle):
    import torch
    g, rng = _build(sg, torch)
    cps = g.control_points
    assert [tuple(c.shape[:-1]) for c in cps.control_points_refined] == \
        [(16, 16, 8), (30, 30, 14), (58, 58, 26), (114, 114, 50)]
    finest = sg.obtain(cps)
    ref_cp = _oracle_chain(oracle, cps)
    assert normwise_rel(_np(finest), ref_cp) <= TOL32

    spec = _spec(oracle, g)
    # plain variant: forward
    sg.evaluate_(g)
    ref = oracle.evaluate(spec, ref_cp)
    assert normwise_rel(_np(g.eval), ref) <= TOL32

    # plain variant: adjoint of the grid (cotangent N(0,1)) against the oracle
    e = rng.standard_normal(tuple(g.eval.shape)).astype(np.float32)
    et = sg.arrays.from_any(torch.as_tensor(e), torch.float32)
    grad = sg.arrays.zeros(tuple(finest.shape), torch.float32)
    sg.evaluate_adjoint_(g, eval=et, control_points=grad)
    g.plan(torch.float32).check()
    ref_grad = oracle.evaluate_adjoint(spec, e.astype(np.float64))
    assert normwise_rel(_np(grad), ref_grad) <= TOL32

    # NURBS variant: weights U[0.5, 2] on the finest grid
    w = rng.uniform(0.5, 2.0, tuple(finest.shape[:-1]))
    ng = sg.NURBSGrid(g.spline_dimensions, 1)
    ng.weights.copy_(torch.as_tensor(w))
    sg.obtain(ng.control_points).copy_(finest)
    sg.evaluate_(ng)
    ref_n = oracle.evaluate(spec, ref_cp, weights=w)
    assert normwise_rel(_np(ng.eval), ref_n) <= TOL32
