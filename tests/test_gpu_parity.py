"""Parity of the CUDA library (through its C ABI, via the Python mirror) with the oracle.

Bars: bit-exact sample indices; FP64 results within 1e-12 and FP32 within 1e-5
normwise relative error (max|gpu - oracle| / max|oracle|) against the FP64 oracle on
the same inputs.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))
TOL = {"f64": 1e-12, "f32": 1e-5}


def _torch():
    import torch
    return torch


def julia_isapprox(a, b, rtol=float(np.sqrt(np.finfo(np.float32).eps))):
    """Julia's `a ≈ b` on arrays (Float32 default rtol): norm(a-b) <= rtol*max(norm a, norm b)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def _np(t):
    """Column-major CUDA tensor -> numpy array with the same (Julia) shape."""
    return np.asfortranarray(t.detach().cpu().numpy())


def make_grid(sg, n_cp, deg, ns, dtype, nout, max_deriv=0, seed=0):
    torch = _torch()
    tdt = torch.float64 if dtype == "f64" else torch.float32
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=min(max_deriv, d), float_type=tdt)
                 for n, d, s in zip(n_cp, deg, ns))
    g = sg.SplineGrid(dims, nout)
    rng = np.random.default_rng(seed)
    cp = rng.standard_normal(tuple(n_cp) + (nout,))
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp))
    return g


def oracle_spec(O, g):
    """Oracle grid on the same knots and sample points, with its own span search and
    FP64 basis tables."""
    sidx, bs = [], []
    for d in g.spline_dimensions:
        knots = d.knot_vector.knots_all.cpu().numpy().astype(np.float64)
        samples = d.sample_points.cpu().numpy().astype(np.float64)
        si = O.sample_indices(samples, knots, d.degree)
        sidx.append(si)
        bs.append(O.basis(knots, samples, si, d.degree, d.max_derivative_order))
    return O.GridSpec(sidx, bs, [d.degree for d in g.spline_dimensions],
                      [d.n_basis_functions for d in g.spline_dimensions])


# ------------------------------------------------------------------ per dimension
@pytest.mark.parametrize("dtype", ["f32", "f64"])
@pytest.mark.parametrize("n,deg,ns", [(10, 2, 50), (10, 3, 50), (5, 2, 25), (256, 3, 4096),
                                      (64, 2, 1024), (8, 1, 1000), (128, 3, 64), (25, 5, 500),
                                      (12, 9, 333), (2, 1, 7), (4, 0, 13)])
def test_sample_indices_bit_exact(sg, oracle, dtype, n, deg, ns):
    torch = _torch()
    tdt = torch.float64 if dtype == "f64" else torch.float32
    d = sg.SplineDimension(n, deg, ns, float_type=tdt, max_derivative_order=min(deg, 2))
    knots = d.knot_vector.knots_all.cpu().numpy()
    samples = d.sample_points.cpu().numpy()
    ref = oracle.sample_indices(samples, knots, deg)
    assert np.array_equal(d.sample_indices.cpu().numpy(), ref)
    # the basis table against the oracle run in the same value type
    bref = oracle.basis(knots, samples, ref, deg, min(deg, 2))
    assert normwise_rel(_np(d.eval), bref) <= (1e-12 if dtype == "f64" else 1e-6)


def test_sample_indices_random_and_special_points(sg, oracle):
    """Random samples (unsorted), samples on knots, outside the extent, and NaN."""
    torch = _torch()
    rng = np.random.default_rng(11)
    kv = np.sort(rng.random(9)).astype(np.float32)
    kv[0], kv[-1] = 0, 1
    mult = np.ones(9, dtype=np.int32)
    mult[0] = mult[-1] = 4
    knots = oracle.expand_knots(kv, mult)
    pts = np.concatenate([rng.random(1000), kv, [-0.5, 1.5, np.nan, 0.0, 1.0]]).astype(np.float32)
    kvec = sg.KnotVector(torch.as_tensor(kv), torch.as_tensor(mult))
    assert np.array_equal(kvec.knots_all.cpu().numpy(), knots)
    d = sg.SplineDimension(len(knots) - 4, 3, len(pts), knot_vector=kvec, sample_points=pts)
    assert np.array_equal(d.sample_indices.cpu().numpy(), oracle.sample_indices(pts, knots, 3))


def test_decompress(sg, oracle):
    d = sg.SplineDimension(10, 3, 200, max_derivative_order=2, float_type=_torch().float64)
    for o in range(3):
        ref = oracle.decompress(_np(d.eval), d.sample_indices.cpu().numpy(), 3, o, 10)
        assert np.array_equal(_np(sg.decompress(d, o)), ref)


# ------------------------------------------------------------------ forward
def test_forward_golden_vector(sg):
    """test/test_spline_grid.jl:29-53 through the CUDA library (Float32, as the reference)."""
    torch = _torch()
    k = KATS["spline_grid_nin2_nout2"]
    dims = tuple(sg.SplineDimension(n, d, s) for n, d, s in
                 zip(k["n_control_points"], k["degree"], k["n_sample_points"]))
    g = sg.SplineGrid(dims, 2)
    cp = np.array(k["control_points"]).reshape(5, 6, 2, order="F")
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp))
    sg.evaluate_(g)
    ref = np.array(k["eval"]).reshape(7, 9, 2, order="F")
    assert np.abs(_np(g.eval) - ref).max() < 1e-6


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", [
    dict(n_cp=(10, 10, 5), deg=(2, 3, 2), ns=(50, 50, 25), nout=4),       # the reference README example grid
    dict(n_cp=(12,), deg=(3,), ns=(1000,), nout=3),
    dict(n_cp=(7, 9), deg=(1, 2), ns=(33, 61), nout=1),
    dict(n_cp=(6, 5, 4, 3), deg=(2, 1, 3, 0), ns=(9, 8, 7, 6), nout=2),
    dict(n_cp=(30, 11), deg=(5, 7), ns=(123, 45), nout=3),              # generic degrees
    dict(n_cp=(40, 40), deg=(3, 3), ns=(256, 512), nout=5),             # vector path
    dict(n_cp=(9, 40), deg=(3, 3), ns=(6, 13), nout=2),                 # fewer samples than spans
])
def test_forward_matches_oracle(sg, oracle, dtype, case):
    g = make_grid(sg, case["n_cp"], case["deg"], case["ns"], dtype, case["nout"], seed=1)
    sg.evaluate_(g)
    spec = oracle_spec(oracle, g)
    ref = oracle.evaluate(spec, _np(sg.obtain(g.control_points)).astype(np.float64))
    assert normwise_rel(_np(g.eval), ref) <= TOL[dtype]


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_forward_derivatives(sg, oracle, dtype):
    g = make_grid(sg, (20, 17, 9), (3, 2, 2), (40, 30, 20), dtype, 2, max_deriv=2, seed=2)
    spec = oracle_spec(oracle, g)
    cp = _np(sg.obtain(g.control_points)).astype(np.float64)
    for order in [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 2), (2, 2, 1)]:
        sg.evaluate_(g, derivative_order=order)
        ref = oracle.evaluate(spec, cp, order=list(order))
        assert normwise_rel(_np(g.eval), ref) <= TOL[dtype], order


def test_constant_control_points_give_one(sg):
    """test/test_spline_grid.jl:11-27 (Nin=1, n 2..10, all degrees)."""
    for n in range(2, 11):
        for deg in range(1, n):
            d = sg.SplineDimension(n, deg, 100)
            g = sg.SplineGrid(d, 1)
            sg.obtain(g.control_points).fill_(1)
            sg.evaluate_(g)
            assert np.allclose(_np(g.eval), 1.0, rtol=1e-5), (n, deg)


def test_nurbs_circle(sg):
    """test/test_nurbs_grid.jl:25-52 through the CUDA library."""
    torch = _torch()
    k = KATS["nurbs_circle"]
    kv = torch.tensor([0, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi], dtype=torch.float32)
    kvec = sg.KnotVector(kv, torch.tensor(k["multiplicities"], dtype=torch.int32))
    d = sg.SplineDimension(9, 2, 500, knot_vector=kvec)
    g = sg.NURBSGrid(d, 2)
    g.weights[1::2] = 1 / math.sqrt(2)
    g.control_points.copy_(torch.tensor(k["control_points"], dtype=torch.float32))
    sg.evaluate_(g)
    ev = _np(g.eval).astype(np.float64)
    assert np.allclose(ev[:, 0] ** 2 + ev[:, 1] ** 2, 1.0, rtol=1e-5)
    assert len({tuple(p) for p in ev[1:].tolist()}) == ev.shape[0] - 1
    with pytest.raises(Exception, match="Computing derivatives of NURBS is currently not"):
        d1 = sg.SplineDimension(4, 2, 100, max_derivative_order=1)
        sg.evaluate_(sg.NURBSGrid(d1, 1), derivative_order=(1,))


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", [
    dict(n_cp=(10,), deg=(2,), ns=(77,), nout=3),
    dict(n_cp=(10, 8), deg=(2, 3), ns=(40, 31), nout=1),
    dict(n_cp=(10, 8), deg=(2, 3), ns=(40, 32), nout=3),
    dict(n_cp=(8, 7, 6), deg=(2, 2, 2), ns=(16, 12, 10), nout=1),
    dict(n_cp=(8, 9), deg=(2, 5), ns=(20, 21), nout=2),   # generic-degree rational pass
    dict(n_cp=(8, 9), deg=(2, 3), ns=(20, 21), nout=6),   # more channels than in-thread
])
def test_nurbs_matches_oracle(sg, oracle, dtype, case):
    torch = _torch()
    g = make_grid(sg, case["n_cp"], case["deg"], case["ns"], dtype, case["nout"], seed=4)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.5, 2.0, case["n_cp"])
    g.weights = sg.arrays.from_any(torch.as_tensor(w), g.dtype)
    sg.evaluate_(g)
    ref = oracle.evaluate(oracle_spec(oracle, g),
                          _np(sg.obtain(g.control_points)).astype(np.float64), weights=w)
    assert normwise_rel(_np(g.eval), ref) <= TOL[dtype]


def test_bf16_control_points(sg, oracle):
    """BF16-stored control points, FP32 accumulation: against the oracle on the
    BF16-rounded inputs (1e-5) and, for the record, on the unrounded ones."""
    torch = _torch()
    g = make_grid(sg, (64, 48), (3, 2), (300, 257), "f32", 3, seed=6)
    cp32 = sg.obtain(g.control_points)
    cpb = sg.arrays.empty(tuple(cp32.shape), torch.bfloat16)
    cpb.copy_(cp32)
    sg.evaluate_(g, control_points=cpb)
    spec = oracle_spec(oracle, g)
    ref_rounded = oracle.evaluate(spec, _np(cpb.float()).astype(np.float64))
    ref_orig = oracle.evaluate(spec, _np(cp32).astype(np.float64))
    assert normwise_rel(_np(g.eval), ref_rounded) <= 1e-5
    assert normwise_rel(_np(g.eval), ref_orig) <= 2e-2


def test_unsorted_samples(sg, oracle):
    """Custom unsorted sample points (the reference's inner constructor allows them):
    forward and adjoint still match."""
    torch = _torch()
    rng = np.random.default_rng(9)
    d0 = sg.SplineDimension(12, 3, 0, sample_points=rng.random(97), float_type=torch.float64)
    d1 = sg.SplineDimension(9, 2, 40, float_type=torch.float64)
    g = sg.SplineGrid((d0, d1), 2)
    cp = rng.standard_normal((12, 9, 2))
    sg.obtain(g.control_points).copy_(torch.as_tensor(cp))
    sg.evaluate_(g)
    spec = oracle_spec(oracle, g)
    assert normwise_rel(_np(g.eval), oracle.evaluate(spec, cp)) <= 1e-12
    e = sg.arrays.from_any(torch.as_tensor(rng.standard_normal((97, 40, 2))), torch.float64)
    out = sg.arrays.zeros((12, 9, 2), torch.float64)
    sg.evaluate_adjoint_(g, eval=e, control_points=out)
    assert normwise_rel(_np(out), oracle.evaluate_adjoint(spec, _np(e))) <= 1e-12


def test_empty_sample_dimension(sg):
    torch = _torch()
    g = make_grid(sg, (5, 6), (2, 2), (0, 10), "f32", 2)
    sg.evaluate_(g)
    assert g.eval.numel() == 0
    out = sg.arrays.ones((5, 6, 2), torch.float32)
    sg.evaluate_adjoint_(g, eval=g.eval, control_points=out)
    assert float(out.abs().max()) == 0.0


# ------------------------------------------------------------------ adjoint
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", [
    dict(n_cp=(10, 10, 5), deg=(2, 3, 2), ns=(50, 50, 25), nout=4),
    dict(n_cp=(64, 64), deg=(2, 2), ns=(1024, 1024), nout=1),          # adjoint heightfield
    dict(n_cp=(12,), deg=(3,), ns=(1000,), nout=3),
    dict(n_cp=(30, 11), deg=(5, 7), ns=(123, 45), nout=3),
    dict(n_cp=(9, 40), deg=(3, 3), ns=(6, 13), nout=2),
    dict(n_cp=(6, 5, 4, 3), deg=(2, 1, 3, 0), ns=(9, 8, 7, 6), nout=2),
])
def test_adjoint_matches_oracle(sg, oracle, dtype, case):
    torch = _torch()
    g = make_grid(sg, case["n_cp"], case["deg"], case["ns"], dtype, case["nout"], seed=3)
    rng = np.random.default_rng(8)
    e = rng.standard_normal(tuple(case["ns"]) + (case["nout"],))
    et = sg.arrays.from_any(torch.as_tensor(e), g.dtype)
    out = sg.arrays.zeros(tuple(case["n_cp"]) + (case["nout"],), g.dtype)
    sg.evaluate_adjoint_(g, eval=et, control_points=out)
    ref = oracle.evaluate_adjoint(oracle_spec(oracle, g), _np(et).astype(np.float64))
    assert normwise_rel(_np(out), ref) <= TOL[dtype]
    # bitwise deterministic: a second run gives identical bits
    out2 = sg.arrays.zeros(tuple(out.shape), g.dtype)
    sg.evaluate_adjoint_(g, eval=et, control_points=out2)
    assert torch.equal(out, out2)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("offset", [0, 1, 3])
@pytest.mark.parametrize("case", [
    # rows of 1031 values: misaligned row starts, three tiles along m with a ragged last
    dict(n_cp=(40, 12), deg=(3, 2), ns=(1031, 37), nout=2),
    # 4D with odd extents: several adjoint passes over strided rows, array tail < 16 B
    dict(n_cp=(7, 6, 5, 4), deg=(3, 2, 1, 3), ns=(13, 11, 9, 7), nout=1),
    # many columns per tile and long sample ranges (several basis batches per column)
    dict(n_cp=(8, 300), deg=(1, 3), ns=(64, 2000), nout=3),
])
def test_adjoint_ragged_and_unaligned(sg, oracle, dtype, offset, case):
    """Adjoint passes with every row alignment: eval_bar starting `offset` values into
    its allocation makes the passes' input rows start at any 4-byte (f32) or 8-byte
    (f64) boundary, and offset 0 with odd extents gives misaligned later rows."""
    torch = _torch()
    g = make_grid(sg, case["n_cp"], case["deg"], case["ns"], dtype, case["nout"], seed=5)
    shape = tuple(case["ns"]) + (case["nout"],)
    rng = np.random.default_rng(offset + 11)
    e = rng.standard_normal(shape)
    flat = torch.zeros(int(np.prod(shape)) + offset, dtype=g.dtype, device="cuda")
    et = flat[offset:].view(tuple(reversed(shape))).permute(*reversed(range(len(shape))))
    et.copy_(torch.as_tensor(e))
    out = sg.arrays.zeros(tuple(case["n_cp"]) + (case["nout"],), g.dtype)
    sg.evaluate_adjoint_(g, eval=et, control_points=out)
    ref = oracle.evaluate_adjoint(oracle_spec(oracle, g), e)
    assert normwise_rel(_np(out), ref) <= TOL[dtype]
    out2 = sg.arrays.zeros(tuple(out.shape), g.dtype)
    sg.evaluate_adjoint_(g, eval=et, control_points=out2)
    assert torch.equal(out, out2)
    g.plan(g.dtype).check()  # no bounded device wait gave up


def test_adjoint_derivative_order_and_transpose(sg):
    torch = _torch()
    g = make_grid(sg, (20, 17), (3, 2), (64, 50), "f64", 2, max_deriv=1, seed=2)
    rng = np.random.default_rng(1)
    p = sg.arrays.from_any(torch.as_tensor(rng.standard_normal((20, 17, 2))), torch.float64)
    e = sg.arrays.from_any(torch.as_tensor(rng.standard_normal((64, 50, 2))), torch.float64)
    for order in [(0, 0), (1, 0), (0, 1), (1, 1)]:
        sg.evaluate_(g, derivative_order=order, control_points=p)
        mte = sg.arrays.zeros((20, 17, 2), torch.float64)
        sg.evaluate_adjoint_(g, derivative_order=order, control_points=mte, eval=e)
        lhs = float((g.eval * e).sum())
        rhs = float((p * mte).sum())
        assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs)), order


def test_adjoint_vs_central_finite_differences(sg, oracle):
    """Adjoint heightfield at full size: n_control (64, 64), degree (2, 2), samples
    (1024, 1024), Nout 1.  The gradient of L = <eval(P), E> (E ~ N(0,1)) from the adjoint
    against FP64 central differences (h = 1e-6) on 64 random control points; the FP32
    adjoint against the FP64 one and the oracle."""
    torch = _torch()
    g = make_grid(sg, (64, 64), (2, 2), (1024, 1024), "f64", 1, seed=2)
    rng = np.random.default_rng(3)
    e = rng.standard_normal((1024, 1024, 1))
    E = sg.arrays.from_any(torch.as_tensor(e), torch.float64)
    grad = sg.arrays.zeros((64, 64, 1), torch.float64)
    sg.evaluate_adjoint_(g, eval=E, control_points=grad)
    P = sg.obtain(g.control_points)
    pick = np.random.default_rng(4).integers(0, 64, size=(64, 2))
    h = 1e-6
    for i, j in pick:
        P[i, j, 0] += h
        sg.evaluate_(g)
        lp = float((g.eval * E).sum())
        P[i, j, 0] -= 2 * h
        sg.evaluate_(g)
        lm = float((g.eval * E).sum())
        P[i, j, 0] += h
        fd = (lp - lm) / (2 * h)
        assert abs(fd - float(grad[i, j, 0])) <= 1e-5 * max(1.0, abs(fd))
    # the FP32 grid (control points and cotangent in FP32)
    g32 = make_grid(sg, (64, 64), (2, 2), (1024, 1024), "f32", 1, seed=2)
    E32 = sg.arrays.from_any(torch.as_tensor(e), torch.float32)
    grad32 = sg.arrays.zeros((64, 64, 1), torch.float32)
    sg.evaluate_adjoint_(g32, eval=E32, control_points=grad32)
    g32.plan(torch.float32).check()
    assert normwise_rel(_np(grad32), _np(grad)) <= TOL["f32"]
    ref = oracle.evaluate_adjoint(oracle_spec(oracle, g32), _np(E32).astype(np.float64))
    assert normwise_rel(_np(grad32), ref) <= TOL["f32"]


# ------------------------------------------------------------------ refinement
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_mult_and_adjoint_match_oracle(sg, oracle, dtype):
    torch = _torch()
    tdt = torch.float64 if dtype == "f64" else torch.float32
    npdt = np.float64 if dtype == "f64" else np.float32
    rng = np.random.default_rng(12)
    mats, dims = [], [0, 2]
    for k, (n, deg) in enumerate([(7, 2), (5, 3)]):
        kv = np.linspace(0, 1, n - deg + 1).astype(npdt)
        mult = np.ones(len(kv), dtype=np.int32)
        mult[0] = mult[-1] = deg + 1
        _, _, R = sg.refine_knots(kv, mult, deg)
        mats.append(R)
    B = rng.standard_normal((7, 4, 5, 2)).astype(npdt)
    Yshape = (mats[0].m, 4, mats[1].m, 2)
    Bt = sg.arrays.from_any(torch.as_tensor(B), tdt)
    Yt = sg.arrays.zeros(Yshape, tdt)
    sg.mult_(Yt, mats, Bt, dims)
    refY = oracle.mult(Yshape, mats, np.asfortranarray(B), dims)
    assert normwise_rel(_np(Yt), refY) <= TOL[dtype]
    Ybar = rng.standard_normal(Yshape).astype(npdt)
    Bbar = sg.arrays.zeros(B.shape, tdt)
    sg.mult_adjoint_(Bbar, mats, sg.arrays.from_any(torch.as_tensor(Ybar), tdt), dims)
    refB = oracle.mult_adjoint(B.shape, mats, np.asfortranarray(Ybar), dims)
    assert normwise_rel(_np(Bbar), refB) <= TOL[dtype]


def test_local_refinement_keeps_geometry(sg):
    """test/test_local_refinement.jl:11-46: 63 active control points, geometry unchanged."""
    k = KATS["local_refinement_ranges"]
    dims = tuple(sg.SplineDimension(n, d, s) for n, d, s in
                 zip(k["n_control_points"], k["degree"], k["n_sample_points"]))
    g = sg.SplineGrid(dims, k["nout"])
    assert g.n_control_points() == 36
    g = sg.add_default_local_refinement(g)
    assert isinstance(g.control_points, sg.LocallyRefinedControlPoints)
    assert g.control_points.shape[:-1] == tuple(k["finest_grid"])
    before = _np(sg.obtain(g.control_points)).copy()
    for (a0, a1), (b0, b1) in k["ranges_1based"]:
        sg.activate_local_control_point_range_(g, range(a0 - 1, a1), range(b0 - 1, b1))
    sg.deactivate_overwritten_control_points_(g.control_points)
    sg.evaluate_control_points_(g.control_points)
    assert g.n_control_points() == k["n_control_points_after"]
    assert julia_isapprox(_np(sg.obtain(g.control_points)), before)


def test_error_informed_refinement_kat(sg):
    """test/test_local_refinement.jl:48-67: the adjoint of an error box selects exactly the
    18 control points of the reference."""
    torch = _torch()
    k = KATS["error_informed_refinement"]
    dims = tuple(sg.SplineDimension(n, d, s) for n, d, s in
                 zip(k["n_control_points"], k["degree"], k["n_sample_points"]))
    g = sg.add_default_local_refinement(sg.SplineGrid(dims, k["nout"]))
    err = sg.arrays.zeros(tuple(g.eval.shape), torch.float32)
    a0, a1, b0, b1, o = k["error_box_1based"]
    err[a0 - 1:a1, b0 - 1:b1, o - 1] = 1
    sg.error_informed_local_refinement_(g, err)
    got = g.control_points.local_refinements[-1].refinement_indices.cpu().numpy().tolist()
    assert got == k["refinement_indices_1based"]


def test_lrcp_adjoint_is_transpose(sg):
    """evaluate!(LRCP) and evaluate_adjoint!(LRCP) are transposes (FP64)."""
    torch = _torch()
    dims = tuple(sg.SplineDimension(n, 2, 40, float_type=torch.float64) for n in (6, 7))
    g = sg.add_default_local_refinement(sg.SplineGrid(dims, 2))
    sg.activate_local_control_point_range_(g, range(0, 4), range(2, 6))
    g = sg.add_default_local_refinement(g)
    sg.activate_local_control_point_range_(g, range(3, 9), range(0, 5))
    cps = g.control_points
    rng = np.random.default_rng(0)
    n = cps.n_control_points()
    x = torch.as_tensor(rng.standard_normal((n, 2)))
    cps.copy_(x)
    sg.evaluate_control_points_(cps)
    y = sg.obtain(cps).clone()
    ybar = torch.as_tensor(rng.standard_normal(tuple(y.shape))).to(y.device)
    sg.obtain(cps).copy_(ybar)
    sg.evaluate_adjoint_control_points_(cps)
    xbar = cps.values_matrix().cpu()
    lhs = float((y.cpu() * ybar.cpu()).sum())
    rhs = float((x * xbar).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))


def test_knot_insertion_and_refine_keep_geometry(sg):
    """test/test_refinement.jl:29-58 (3D, random interior knots)."""
    torch = _torch()
    gen = torch.Generator().manual_seed(1)
    dims = tuple(sg.SplineDimension(n, d, s, distribution="random", generator=gen)
                 for n, d, s in zip((5, 8, 6), (4, 2, 3), (15, 20, 25)))
    g0 = sg.SplineGrid(dims, 2)
    sg.obtain(g0.control_points).copy_(torch.rand((5, 8, 6, 2), generator=gen))
    sg.evaluate_(g0)
    ref = _np(g0.eval)
    g = g0
    for dim in range(3):
        g, R = sg.insert_knot_grid(g, dim, 0.25)
        sg.evaluate_(g)
        assert julia_isapprox(_np(g.eval), ref)
        assert R.shape == (g.control_points.shape[dim], g.control_points.shape[dim] - 1)
    g = g0
    for dim in range(3):
        old = g.control_points.shape[dim]
        g, R = sg.refine(g, dim)
        sg.evaluate_(g)
        assert julia_isapprox(_np(g.eval), ref)
        assert R.shape == (g.control_points.shape[dim], old)


@pytest.mark.parametrize("shape", [((128, 128), (1024, 1024), 6), ((90, 100), (537, 611), 5),
                                   ((20, 16, 12), (200, 150, 100), 2)])
@pytest.mark.parametrize("strategy", ["separable", "auto"])
def test_tuned_adjoint_is_bitwise_the_heuristic_one(sg, shape, strategy):
    """sg_grid_plan_tune picks, by timing, a stream chunk size per axis (separable
    passes) or the axis-1 block of the fused tiles (Nin = 2); the results do not depend
    on it (every control point sums its samples in the same order)."""
    torch = _torch()
    ncp, ns, nout = shape
    dims = tuple(sg.SplineDimension(n, 3, s) for n, s in zip(ncp, ns))
    g = sg.SplineGrid(dims, nout)
    plan = g.plan(torch.float32)
    if strategy == "separable":
        plan.set_strategy("separable")
    rng = np.random.default_rng(7)
    e = sg.arrays.from_any(torch.as_tensor(rng.standard_normal(tuple(ns) + (nout,))), torch.float32)
    ref = sg.arrays.empty(tuple(ncp) + (nout,), torch.float32)
    sg.evaluate_adjoint_(g, eval=e, control_points=ref)
    chosen = sg.tune_adjoint_(g, eval=e)
    if plan.paths()[1] == "fused":
        assert chosen[0] == 0 and 1 <= chosen[1] <= ncp[1]
    else:
        assert chosen[0] == 0 and all(c in (0, 8, 12, 16, 24, 32, 48, 64) for c in chosen[1:])
    got = sg.arrays.empty(tuple(ncp) + (nout,), torch.float32)
    sg.evaluate_adjoint_(g, eval=e, control_points=got)
    plan.check()
    assert torch.equal(got, ref)
    plan.untune()
    plan.set_strategy("auto")
