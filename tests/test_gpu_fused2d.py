"""The fused Nin = 2 path (both axes in one launch) against the separable passes (bit for
bit) and the FP64 oracle, per grid and in the batch.

Reference: spline_eval_kernel (src/spline_grid.jl:119-183) and
spline_eval_adjoint_kernel (src/adjoint.jl:1-40); the fused path computes the same
linear map with the separable passes' operation order."""
import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu

# (n_control, degree, n_samples, nout): sparse and dense sampling, axis-0 rows longer
# than one warp task or adjoint tile, degree 0, many channels, a single sample
SHAPES = [
    ((12, 9), (3, 2), (70, 41), 3),
    ((7, 15), (1, 3), (33, 90), 2),
    ((40, 30), (2, 2), (25, 20), 1),        # fewer samples than control points
    ((20, 16), (3, 3), (1500, 37), 2),      # axis 0 over several warp tasks
    ((64, 8), (3, 1), (2500, 300), 1),      # long axis 0 (separable adjoint)
    ((30, 40), (2, 3), (1000, 500), 2),     # axis 0 whole in one adjoint tile
    ((9, 11), (0, 2), (50, 61), 5),         # degree 0
    ((10, 10), (2, 3), (64, 64), 48),       # channel groups
    ((5, 6), (1, 1), (1, 1), 1),            # one sample
    ((128, 128), (3, 3), (1024, 1024), 1),  # the batched configuration's largest grids
    ((64, 64), (2, 2), (700, 1024), 17),    # channel groups of odd size, halo along axis 1
    ((300, 20), (3, 2), (4096, 50), 2),     # adjoint in axis-0 chunks (one channel per tile)
    ((3000, 10), (1, 1), (2048, 40), 1),    # chunks of a sparse axis (more control points than samples)
    ((90, 12), (2, 3), (1027, 30), 2),      # too long for a tile, rows not 16-byte multiples
]


def _grid(sg, torch, shape, dtype, seed, max_deriv=1):
    n_cp, deg, ns, nout = shape
    rng = np.random.default_rng(seed)
    ft = torch.float64 if dtype == torch.float64 else torch.float32
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=min(max_deriv, d), float_type=ft)
                 for n, d, s in zip(n_cp, deg, ns))
    g = sg.SplineGrid(dims, nout)
    cp = rng.standard_normal(n_cp + (nout,))
    cot = rng.standard_normal(ns + (nout,))
    return g, cp, cot


def _orders(shape):
    _, deg, _, _ = shape
    out = [(0, 0)]
    if deg[0] >= 1:
        out.append((1, 0))
    if deg[1] >= 1:
        out.append((0, 1))
    return out


@pytest.mark.parametrize("dtype_name", ["f32", "f64"])
@pytest.mark.parametrize("si", range(len(SHAPES)))
def test_fused_equals_separable_and_oracle(sg, oracle, dtype_name, si):
    import torch
    from test_gpu_parity import oracle_spec
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    tol = 1e-12 if dtype_name == "f64" else 1e-5
    shape = SHAPES[si]
    g, cp_h, cot_h = _grid(sg, torch, shape, dtype, 10 + si)
    cp = sg.arrays.from_any(torch.as_tensor(cp_h), dtype)
    cot = sg.arrays.from_any(torch.as_tensor(cot_h), dtype)
    plan = g.plan(dtype)
    # adjoint tiles span axis 0 whole, or chunks of it when its rows are 16-byte multiples;
    # other long axes take the separable adjoint
    ns0 = shape[2][0]
    fits = ns0 <= (512 if dtype_name == "f64" else 1024) or ns0 % (2 if dtype_name == "f64" else 4) == 0
    assert plan.paths() == ("fused", "fused" if fits else "separable")
    spec = oracle_spec(oracle, g)
    for order in _orders(shape):
        ev, gr = {}, {}
        for strat in ("separable", "fused"):
            plan.set_strategy(strat)
            e = sg.arrays.empty(tuple(g.eval.shape), dtype)
            e.fill_(float("nan"))
            sg.evaluate_(g, derivative_order=order, control_points=cp, eval=e)
            c = sg.arrays.empty(tuple(cp.shape), dtype)
            c.fill_(float("nan"))
            sg.evaluate_adjoint_(g, derivative_order=order, eval=cot, control_points=c)
            plan.check()
            ev[strat], gr[strat] = e, c
        plan.set_strategy("auto")
        assert torch.equal(ev["fused"], ev["separable"]), f"forward {order} differs"
        assert torch.equal(gr["fused"], gr["separable"]), f"adjoint {order} differs"
        ref = oracle.evaluate(spec, np.asfortranarray(cp.cpu().numpy().astype(np.float64)), order=list(order))
        assert normwise_rel(ev["fused"].cpu().numpy(), ref) <= tol
        refg = oracle.evaluate_adjoint(spec, np.asfortranarray(cot.cpu().numpy().astype(np.float64)),
                                       order=list(order))
        assert normwise_rel(gr["fused"].cpu().numpy(), refg) <= tol


def test_fused_bf16_control_points(sg):
    import torch
    g, cp_h, _ = _grid(sg, torch, ((30, 20), (3, 2), (300, 200), 3), torch.float32, 3)
    cp = sg.arrays.from_any(torch.as_tensor(cp_h), torch.float32)
    cpb = sg.arrays.empty(tuple(cp.shape), torch.bfloat16)
    cpb.copy_(cp)
    plan = g.plan(torch.bfloat16)
    out = {}
    for strat in ("separable", "fused"):
        plan.set_strategy(strat)
        e = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
        sg.evaluate_(g, control_points=cpb, eval=e)
        out[strat] = e
    plan.set_strategy("auto")
    assert torch.equal(out["fused"], out["separable"])


def test_fused_adjoint_tuning_is_bitwise_neutral(sg):
    import torch
    g, _, cot_h = _grid(sg, torch, ((96, 80), (3, 3), (900, 700), 4), torch.float32, 5)
    cot = sg.arrays.from_any(torch.as_tensor(cot_h), torch.float32)
    ref = sg.arrays.empty((96, 80, 4), torch.float32)
    sg.evaluate_adjoint_(g, eval=cot, control_points=ref)
    scratch = sg.arrays.empty((96, 80, 4), torch.float32)
    chosen = sg.tune_adjoint_(g, eval=cot, control_points=scratch)
    assert 1 <= chosen[1] <= 80
    got = sg.arrays.empty((96, 80, 4), torch.float32)
    sg.evaluate_adjoint_(g, eval=cot, control_points=got)
    assert torch.equal(got, ref)
    g.plan(torch.float32).untune()


def test_separable_only_grids_keep_their_path(sg):
    """Grids outside the fused path (Nin = 3, NURBS, degree > 3) report the separable
    path; forcing the fused strategy on them is refused."""
    import torch
    dims3 = tuple(sg.SplineDimension(n, 2, s) for n, s in zip((6, 7, 5), (11, 12, 9)))
    g3 = sg.SplineGrid(dims3, 1)
    assert g3.plan(torch.float32).paths() == ("separable", "separable")
    with pytest.raises(sg.SplineGridsError):
        g3.plan(torch.float32).set_strategy("fused")
    dims4 = tuple(sg.SplineDimension(n, 4, s) for n, s in zip((9, 8), (20, 21)))
    g4 = sg.SplineGrid(dims4, 1)
    assert g4.plan(torch.float32).paths() == ("separable", "separable")
    dimsn = tuple(sg.SplineDimension(n, 2, s) for n, s in zip((6, 7), (11, 12)))
    gn = sg.NURBSGrid(dimsn, 2)
    assert gn.plan(torch.float32).paths()[0] == "separable"


@pytest.mark.parametrize("dtype_name", ["f32", "f64"])
def test_batch_fused_equals_separable(sg, dtype_name):
    import torch
    from test_gpu_batch import _random_grids
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 20, 300, dtype, sets=4, nin=2)
    orders = [tuple(int(o) for o in np.random.default_rng(i).integers(0, 2, size=2))
              for i in range(len(grids))]
    batch = sg.GridBatch(grids, orders)
    batch.set_arrays(cps, evals, cots, grads)
    assert batch.fused_grids() == len(grids)
    res = {}
    for strat in ("separable", "auto"):
        batch.set_strategy(strat)
        for e in evals:
            e.fill_(float("nan"))
        for gr in grads:
            gr.fill_(float("nan"))
        batch.run(forward=True, adjoint=True)
        batch.check()
        res[strat] = ([e.clone() for e in evals], [gr.clone() for gr in grads])
    assert batch.fused_grids() == len(grids)
    for a, b in zip(res["auto"][0], res["separable"][0]):
        assert torch.equal(a, b)
    for a, b in zip(res["auto"][1], res["separable"][1]):
        assert torch.equal(a, b)
    # forward-only and adjoint-only launches of the fused lists
    for e in evals:
        e.fill_(float("nan"))
    batch.run(forward=True, adjoint=False)
    for gr in grads:
        gr.fill_(float("nan"))
    batch.run(forward=False, adjoint=True)
    batch.check()
    for a, b in zip(evals, res["separable"][0]):
        assert torch.equal(a, b)
    for a, b in zip(grads, res["separable"][1]):
        assert torch.equal(a, b)


def test_batch_mixed_fused_and_separable_grids(sg, oracle):
    """2D grids run fused, 3D and 1D grids run the pass queue, in the same batch run."""
    import torch
    from test_gpu_batch import _random_grids
    from test_gpu_parity import oracle_spec
    g2, c2, e2, t2, r2 = _random_grids(sg, torch, 6, 900, torch.float64, nin=2)
    g3, c3, e3, t3, r3 = _random_grids(sg, torch, 3, 950, torch.float64, nin=3)
    g1, c1, e1, t1, r1 = _random_grids(sg, torch, 3, 990, torch.float64, nin=1)
    grids, cps, evals, cots, grads = (g2 + g3 + g1, c2 + c3 + c1, e2 + e3 + e1, t2 + t3 + t1,
                                      r2 + r3 + r1)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    assert batch.fused_grids() == 6
    batch.run(forward=True, adjoint=True)
    batch.check()
    for g, cp, ev, cot, gr in zip(grids, cps, evals, cots, grads):
        spec = oracle_spec(oracle, g)
        ref = oracle.evaluate(spec, np.asfortranarray(cp.cpu().numpy()))
        assert normwise_rel(ev.cpu().numpy(), ref) <= 1e-12
        refg = oracle.evaluate_adjoint(spec, np.asfortranarray(cot.cpu().numpy()))
        assert normwise_rel(gr.cpu().numpy(), refg) <= 1e-12


def test_batch_tuning_is_bitwise_neutral(sg):
    """sg_batch_tune times fused unit sizes on the plan's arrays and keeps the fastest;
    every size gives the same bits."""
    import torch
    from test_gpu_batch import _random_grids
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 12, 700, torch.float32, sets=4, nin=2)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.run(forward=True, adjoint=True)
    batch.check()
    ref_ev = [e.clone() for e in evals]
    ref_gr = [g.clone() for g in grads]
    fwd, adj = batch.tune()
    assert fwd > 0 and adj >= 0
    for sizes in ((fwd, adj), (1 << 13, 1 << 16), (0, 0)):
        batch.set_unit_sizes(*sizes)
        for e in evals:
            e.fill_(float("nan"))
        for gr in grads:
            gr.fill_(float("nan"))
        batch.run(forward=True, adjoint=True)
        batch.check()
        for a, b in zip(evals, ref_ev):
            assert torch.equal(a, b)
        for a, b in zip(grads, ref_gr):
            assert torch.equal(a, b)
