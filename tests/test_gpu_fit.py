"""The device-side fit loop (forward, loss, adjoint, update) per grid and per GridBatch:
its loss and update against a float64 torch restatement, a captured CUDA graph whose
replay gives the bits of the eager steps, and a decreasing loss.

Reference loop: docs/src/examples_optics.md:184-191 (evaluate! of (0,0), (1,0), (0,1)
then a loss and its Enzyme gradient, which runs evaluate_adjoint!, src/adjoint.jl:42-83)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORDERS = [(0, 0), (1, 0), (0, 1)]


def _grid_problem(sg, torch, dtype, seed=0, n_cp=(24, 20), deg=(3, 2), ns=(300, 257), nout=2):
    rng = np.random.default_rng(seed)
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=1, float_type=dtype)
                 for n, d, s in zip(n_cp, deg, ns))
    g = sg.SplineGrid(dims, nout)
    cp = sg.arrays.from_any(torch.as_tensor(rng.standard_normal(n_cp + (nout,))), dtype)
    # targets: the evals of other control points, so the fit has a reachable optimum
    cp_true = sg.arrays.from_any(torch.as_tensor(rng.standard_normal(n_cp + (nout,))), dtype)
    targets = sg.evaluate_multi_(g, ORDERS, control_points=cp_true)
    return g, cp, targets


def _torch_step(sg, g, cp, targets, weights, step):
    """One step restated with float64 torch ops on the library's forward/adjoint results:
    returns (loss, control points after the update)."""
    import torch
    evals = sg.evaluate_multi_(g, ORDERS, control_points=cp)
    loss = 0.0
    grad = torch.zeros(tuple(cp.shape), dtype=torch.float64, device=cp.device)
    for o, e, t, w in zip(ORDERS, evals, targets, weights):
        r = e.double() - t.double()
        loss += 0.5 * w * float((r * r).sum())
        cot = sg.arrays.empty(tuple(e.shape), e.dtype)
        cot.copy_((w * r).to(e.dtype))
        gr = sg.arrays.empty(tuple(cp.shape), cp.dtype)
        sg.evaluate_adjoint_(g, derivative_order=o, eval=cot, control_points=gr)
        grad += gr.double()
    return loss, cp.double() - step * grad


@pytest.mark.parametrize("dtype_name", ["f32", "f64"])
def test_grid_fit_step_matches_torch(sg, dtype_name):
    import torch
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    g, cp, targets = _grid_problem(sg, torch, dtype)
    weights = (1.0, 0.25, 0.5)
    step = 1e-4
    cp0 = cp.clone()
    ref_loss, ref_cp = _torch_step(sg, g, cp0, targets, weights, step)
    fit = sg.grid_fit(g, ORDERS, targets, step, weights=weights, control_points=cp)
    fit.step()
    tol = 1e-12 if dtype_name == "f64" else 1e-5
    assert abs(fit.loss() - ref_loss) <= tol * abs(ref_loss)
    err = float((cp.double() - ref_cp).abs().max() / ref_cp.abs().max())
    assert err <= tol, err
    # the cotangents the loss stage wrote
    for e, t, c, w in zip(fit.evals, targets, fit.cotangents, weights):
        assert torch.allclose(c.double(), w * (e.double() - t.double()), rtol=tol, atol=tol)


def test_grid_fit_graph_replay_is_bitwise_eager(sg):
    import torch
    g, cp, targets = _grid_problem(sg, torch, torch.float32, seed=1)
    step = 1e-7  # well below 2 / the Lipschitz constant of the derivative terms' gradient
    cp_eager = cp.clone()
    fit_e = sg.grid_fit(g, ORDERS, targets, step, control_points=cp_eager)
    for _ in range(6):
        fit_e.step()
    eager_losses = fit_e.losses()
    cp_graph = cp.clone()
    fit_g = sg.grid_fit(g, ORDERS, targets, step, control_points=cp_graph)
    fit_g.capture(steps=3)
    torch.cuda.synchronize()
    assert torch.equal(cp_graph, cp)  # capturing runs nothing
    fit_g.replay()
    fit_g.replay()
    assert fit_g.losses() == eager_losses
    assert torch.equal(cp_graph, cp_eager)
    assert eager_losses[-1] < eager_losses[0]


def test_batch_fit_graph_replay_is_bitwise_eager(sg):
    import torch
    from test_gpu_batch import _random_grids
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 10, 500, torch.float32, sets=2, nin=2)
    targets = []
    for g, cp in zip(grids, cps):
        t = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
        t.copy_(torch.randn(tuple(t.shape), generator=torch.Generator(device="cuda").manual_seed(7),
                            device="cuda"))
        targets.append(t)
    start = [c.clone() for c in cps]
    step = 1e-3

    def run(mode):
        for c, s0 in zip(cps, start):
            c.copy_(s0)
        batch = sg.GridBatch(grids)
        batch.set_arrays(cps, evals, cots, grads)
        fit = sg.batch_fit(batch, targets, step)
        if mode == "eager":
            for _ in range(4):
                fit.step()
        else:
            fit.capture(steps=2)
            fit.replay()
            fit.replay()
        batch.check()
        return fit.losses(), [c.clone() for c in cps]

    le, ce = run("eager")
    lg, cg = run("graph")
    assert le == lg
    for a, b in zip(ce, cg):
        assert torch.equal(a, b)
    assert le[-1] < le[0]
    # the first loss equals the float64 restatement at the starting control points
    ref = 0.0
    for g, s0, t in zip(grids, start, targets):
        e = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
        sg.evaluate_(g, control_points=s0, eval=e)
        ref += 0.5 * float(((e.double() - t.double()) ** 2).sum())
    assert abs(le[0] - ref) <= 1e-6 * ref


def test_fit_rejects_mismatched_arrays(sg):
    import torch
    g, cp, targets = _grid_problem(sg, torch, torch.float32, seed=2)
    with pytest.raises(ValueError):
        sg.grid_fit(g, ORDERS, targets[:2], 1e-3, control_points=cp)
    bad = [t.double() for t in targets]
    with pytest.raises(TypeError):
        sg.grid_fit(g, ORDERS, bad, 1e-3, control_points=cp)
