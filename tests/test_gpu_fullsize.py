"""Parity at the full sizes the benchmark times, against the FP64 oracle.

* The large 2D surface: n_control (256, 256), degree (3, 3), n_samples (4096, 4096),
  Nout 3, derivative orders (0,0), (1,0), (0,1); FP64 forward <= 1e-12, FP32 forward
  and adjoint <= 1e-5, bfloat16-stored control points <= 1e-5 against the oracle on the
  rounded inputs; on both strategies (fused, and the separable passes with their
  4096-wide stream rows).
* The batched configuration at the benchmark's exact draws: all 256 grids x 16 sets,
  forward + adjoint in one GridBatch run, every grid against the FP64 oracle at 1e-5,
  and the fused and separable strategies bit for bit.

Reference kernels: spline_eval_kernel (src/spline_grid.jl:119-183) and
spline_eval_adjoint_kernel (src/adjoint.jl:1-40)."""
import sys

import numpy as np
import pytest

from conftest import ROOT, normwise_rel

pytestmark = pytest.mark.gpu

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ORDERS = ((0, 0), (1, 0), (0, 1))


@pytest.fixture(scope="module")
def large2d(sg, oracle):
    """The large grid's control points and cotangent and the oracle's results per order
    (on the knots and samples of FP64 and of FP32 dimensions), computed once."""
    import bench
    import torch
    from test_gpu_parity import oracle_spec
    c = bench.LARGE2D

    def spec_of(ft):  # the oracle on the knots and samples of a grid of this type
        dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=1, float_type=ft)
                     for n, d, s in zip(c["n_cp"], c["deg"], c["ns"]))
        return oracle_spec(oracle, sg.SplineGrid(dims, c["nout"]))

    spec64, spec32 = spec_of(torch.float64), spec_of(torch.float32)
    cp = np.random.default_rng(c["seed"]).standard_normal(c["n_cp"] + (c["nout"],))
    cot = np.random.default_rng(c["seed"] + 1).standard_normal(c["ns"] + (c["nout"],))
    cp32 = np.asfortranarray(cp.astype(np.float32).astype(np.float64))
    cot32 = np.asfortranarray(cot.astype(np.float32).astype(np.float64))
    cpb = np.asfortranarray(torch.as_tensor(cp).to(torch.bfloat16).to(torch.float64).numpy())
    refs = {}
    for o in ORDERS:
        refs[("f64", o)] = oracle.evaluate(spec64, np.asfortranarray(cp), order=list(o))
        refs[("f32", o)] = oracle.evaluate(spec32, cp32, order=list(o))
        refs[("bf16", o)] = oracle.evaluate(spec32, cpb, order=list(o))
        refs[("adj", o)] = oracle.evaluate_adjoint(spec32, cot32, order=list(o))
    return dict(c=c, cp=cp, cot=cot, refs=refs)


@pytest.mark.parametrize("strategy", ["fused", "separable"])
@pytest.mark.parametrize("mode", ["f64", "f32", "bf16"])
def test_large2d_fullsize(sg, large2d, mode, strategy):
    import torch
    c = large2d["c"]
    ft = torch.float64 if mode == "f64" else torch.float32
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=1, float_type=ft)
                 for n, d, s in zip(c["n_cp"], c["deg"], c["ns"]))
    g = sg.SplineGrid(dims, c["nout"])
    cp_dtype = torch.bfloat16 if mode == "bf16" else ft
    cp = sg.arrays.empty(c["n_cp"] + (c["nout"],), cp_dtype)
    cp.copy_(torch.as_tensor(large2d["cp"]))
    plan = g.plan(cp_dtype)
    plan.set_strategy(strategy)
    tol = 1e-12 if mode == "f64" else 1e-5
    ev = sg.arrays.empty(c["ns"] + (c["nout"],), ft)
    for o in ORDERS:
        ev.fill_(float("nan"))
        sg.evaluate_(g, derivative_order=o, control_points=cp, eval=ev)
        err = normwise_rel(ev.cpu().numpy(), large2d["refs"][(mode, o)])
        assert err <= tol, (o, err)
    if mode == "f32":  # the adjoint of each order
        cot = sg.arrays.empty(c["ns"] + (c["nout"],), ft)
        cot.copy_(torch.as_tensor(large2d["cot"]))
        gr = sg.arrays.empty(c["n_cp"] + (c["nout"],), ft)
        for o in ORDERS:
            gr.fill_(float("nan"))
            sg.evaluate_adjoint_(g, derivative_order=o, eval=cot, control_points=gr)
            err = normwise_rel(gr.cpu().numpy(), large2d["refs"][("adj", o)])
            assert err <= 1e-5, (o, err)
    plan.check()
    plan.set_strategy("auto")


def test_batched_config_fullsize(sg, oracle):
    """All 256 grids x 16 sets of the benchmarked batch, forward + adjoint in one run,
    against the FP64 oracle; then the separable strategy must give the same bits."""
    import bench
    import torch
    from test_gpu_parity import oracle_spec
    specs, grids, cps, evals, cots, grads = bench.build_batched(sg, torch, torch.float32)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    assert batch.fused_grids() == len(grids)
    batch.run(forward=True, adjoint=True)
    batch.check()
    fe = ae = 0.0
    for g, cp, ev, cot, gr in zip(grids, cps, evals, cots, grads):
        spec = oracle_spec(oracle, g)
        ref = oracle.evaluate(spec, np.asfortranarray(cp.cpu().numpy().astype(np.float64)))
        fe = max(fe, normwise_rel(ev.cpu().numpy(), ref))
        refg = oracle.evaluate_adjoint(spec, np.asfortranarray(cot.cpu().numpy().astype(np.float64)))
        ae = max(ae, normwise_rel(gr.cpu().numpy(), refg))
        del ref, refg
    assert fe <= 1e-5 and ae <= 1e-5, (fe, ae)
    # the separable passes (pass queue, intermediates) on the same arrays: same bits
    fused_ev = [e.clone() for e in evals]
    fused_gr = [g_.clone() for g_ in grads]
    batch.set_strategy("separable")
    batch.run(forward=True, adjoint=True)
    batch.check()
    for a, b in zip(evals, fused_ev):
        assert torch.equal(a, b)
    for a, b in zip(grads, fused_gr):
        assert torch.equal(a, b)
