"""The oracle against the reference's own golden vectors and known-answer tests.

The reference (Julia) cannot run here; its test files' literal values are committed in
tests/golden/reference_kats.json (made by tests/golden/make_golden.py).  These tests
pin the CPU restatement before it is used to check the CUDA library.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import normwise_rel

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def _grid(O, n_cp, deg, ns, dtype, max_deriv=0):
    dims = [O.default_dimension(n, d, s, max_deriv, dtype=dtype) for n, d, s in zip(n_cp, deg, ns)]
    spec = O.GridSpec([x["sidx"] for x in dims], [x["basis"] for x in dims], deg, n_cp)
    return dims, spec


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-15), (np.float32, 5e-7)])
def test_forward_golden_vector(oracle, dtype, tol):
    """test/test_spline_grid.jl:29-53: 5x6x2 control points -> 7x9x2 eval, degrees (3,2)."""
    k = KATS["spline_grid_nin2_nout2"]
    _, spec = _grid(oracle, k["n_control_points"], k["degree"], k["n_sample_points"], dtype)
    cp = np.array(k["control_points"]).reshape(5, 6, 2, order="F")
    ref = np.array(k["eval"]).reshape(7, 9, 2, order="F")
    ev = oracle.evaluate(spec, cp.astype(dtype))
    assert np.abs(ev - ref).max() <= tol


def test_knot_vector_kat(oracle):
    """test/test_knot_vector.jl:26-36."""
    k = KATS["knot_vector_5_2"]
    d = oracle.default_dimension(k["n_basis"], k["degree"], 10)
    assert list(d["multiplicities"]) == k["multiplicities"]
    assert np.allclose(d["knots_all"], k["knots_all"], rtol=0, atol=1e-15)
    d2 = oracle.default_dimension(k["n_basis"], k["degree"], 10, extent=tuple(k["extent2"]))
    assert np.allclose(d2["knots_all"], 2 * np.array(k["knots_all"]) + 5.0, atol=1e-14)


def test_nurbs_circle(oracle):
    """test/test_nurbs_grid.jl:25-52: a degree-2 NURBS with weights 1/sqrt(2) at the odd
    control points is the unit circle."""
    k = KATS["nurbs_circle"]
    kv = np.array([0, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi], dtype=np.float32)
    knots = oracle.expand_knots(kv, k["multiplicities"])
    samples = oracle.julia_range(float(kv[0]), float(kv[-1]), k["n_sample_points"]).astype(
        np.float32)
    sidx = oracle.sample_indices(samples, knots, k["degree"])
    b = oracle.basis(knots, samples, sidx, k["degree"], 0)
    spec = oracle.GridSpec([sidx], [b], [k["degree"]], [k["n_control_points"]])
    w = np.ones(9, dtype=np.float32)
    w[1::2] = np.float32(k["weight_even_index"])
    cp = np.array(k["control_points"], dtype=np.float32)
    ev = oracle.evaluate(spec, np.asfortranarray(cp), weights=w)
    r2 = ev[:, 0].astype(np.float64) ** 2 + ev[:, 1].astype(np.float64) ** 2
    assert np.allclose(r2, 1.0, rtol=1e-5)
    assert len({tuple(p) for p in ev[1:].tolist()}) == ev.shape[0] - 1


@pytest.mark.parametrize("degree", range(6))
def test_partition_of_unity(oracle, degree):
    """test/test_spline_dimension.jl:10-29 (equispaced knots)."""
    d = oracle.default_dimension(25, degree, 500, dtype=np.float32)
    B = d["basis"][:, :, 0].astype(np.float64)
    assert B.shape == (500, degree + 1)
    assert np.all(B >= 0)
    assert np.allclose(B.sum(axis=1), 1.0, rtol=1e-5)


def test_derivatives_vs_finite_differences(oracle):
    """test/test_spline_dimension.jl:31-66: FP64, degree 3, max derivative 2, 5000 samples."""
    d = oracle.default_dimension(10, 3, 5000, max_deriv=2, dtype=np.float64)
    t = d["samples"]
    dt = np.diff(t)
    data = oracle.decompress(d["basis"], d["sidx"], 3, 0, 10)
    d1 = oracle.decompress(d["basis"], d["sidx"], 3, 1, 10)
    d2 = oracle.decompress(d["basis"], d["sidx"], 3, 2, 10)
    fd = np.diff(data, axis=0) / dt[:, None]
    fd2 = np.diff(fd, axis=0) / dt[1:, None]
    assert np.allclose(d1[:-1], fd, rtol=1e-2, atol=1e-2 * np.abs(fd).max())
    assert np.allclose(d2[2:], fd2, rtol=1e-2, atol=1e-2 * np.abs(fd2).max())


def test_sample_points_hit_knots_exactly(oracle):
    """Samples l/(n-1) that equal a knot k/m must coincide bit for bit (then the span
    search puts them right of the knot, as the reference's scan does)."""
    # 1024 samples, 62 spans: 33/1023 == 2/62
    d = oracle.default_dimension(64, 2, 1024, dtype=np.float32)
    assert d["samples"][33] == d["knots_all"][2 + 2]
    assert d["sidx"][33] == 2 + 2 + 1  # 1-based index of that knot
    # the reference README example, dim 2: 50 samples, degree 3, 7 spans: 7k/49 == k/7
    d = oracle.default_dimension(10, 3, 50, dtype=np.float64)
    assert d["samples"][7] == d["knots_all"][3 + 1]
    assert d["sidx"][7] == 3 + 1 + 1


def test_adjoint_is_transpose(oracle):
    """<M p, e> == <p, M' e> for the oracle's forward and adjoint (FP64)."""
    rng = np.random.default_rng(3)
    _, spec = _grid(oracle, (7, 6, 5), (2, 3, 1), (11, 13, 9), np.float64)
    p = rng.standard_normal((7, 6, 5, 2))
    e = rng.standard_normal((11, 13, 9, 2))
    Mp = oracle.evaluate(spec, np.asfortranarray(p))
    Mte = oracle.evaluate_adjoint(spec, np.asfortranarray(e))
    assert abs((Mp * e).sum() - (p * Mte).sum()) < 1e-12 * np.abs(Mp * e).sum()


def test_constant_control_points_give_one(oracle):
    """test/test_spline_grid.jl:11-27: Nin=1, every degree up to n-1, eval == 1."""
    for n in range(2, 11):
        for deg in range(1, n):
            _, spec = _grid(oracle, (n,), (deg,), (100,), np.float32)
            ev = oracle.evaluate(spec, np.ones((n, 1), dtype=np.float32, order="F"))
            assert np.allclose(ev, 1.0, rtol=1e-5)


def test_refinement_keeps_geometry(oracle):
    """test/test_refinement.jl:43-58 on explicit (random-draw) knots: refining a dimension
    and applying the refinement matrix to the control points leaves eval unchanged.
    Exercises the package's host knot algebra against the oracle's mult! and evaluate!."""
    import splinegrids as sg
    rng = np.random.default_rng(1)
    n_cp, deg, ns, nout = (5, 8, 6), (4, 2, 3), (15, 20, 25), 2
    dims = []
    for n, d, s in zip(n_cp, deg, ns):
        nv = n - d + 1
        kv = np.cumsum(rng.random(nv))
        kv = (kv - kv[0]) / (kv[-1] - kv[0])
        mult = np.ones(nv, dtype=np.int32)
        mult[0] = mult[-1] = d + 1
        dims.append((kv, mult, d, s))

    def spec_of(ds):
        sidx, bs = [], []
        for kv, mult, d, s in ds:
            knots = oracle.expand_knots(kv, mult)
            samples = oracle.julia_range(kv[0], kv[-1], s)
            si = oracle.sample_indices(samples, knots, d)
            sidx.append(si)
            bs.append(oracle.basis(knots, samples, si, d, 0))
        return oracle.GridSpec(sidx, bs, [x[2] for x in ds],
                               [int(x[1].sum()) - x[2] - 1 for x in ds])

    cp = np.asfortranarray(rng.random(n_cp + (nout,)))
    ref = oracle.evaluate(spec_of(dims), cp)
    for k in range(3):
        kv, mult, d, s = dims[k]
        kv2, mult2, R = sg.refine_knots(kv, mult, d)
        new_shape = list(cp.shape)
        new_shape[k] = R.m
        cp = oracle.mult(new_shape, [R], cp, [k])
        dims[k] = (kv2, mult2, d, s)
        ev = oracle.evaluate(spec_of(dims), cp)
        assert normwise_rel(ev, ref) < 1e-13
