"""Failure paths, made on purpose without faulting or hanging the GPU.

* Allocation failure: a host-side hook makes the library's device allocations fail after
  a given count, as cudaMalloc does on a full device.  Every create entry point returns
  SG_ERR_OUT_OF_MEMORY and releases what it had allocated (the count of live
  allocations is unchanged), and works again once the hook is cleared.
* Bounded waits: the batch pass queue's dependency waits and the fused adjoint's stage
  waits are given a short limit and a wait that can never complete (a dependency that
  asks for one tile more than its pass has; a producer that withholds its arrival on
  the first stage).  The kernels return, the checks report SG_ERR_TIMEOUT, and a normal
  run afterwards gives the same bits as before.

Error convention of the reference: src/validation.jl:17-49 (errors are raised to the
caller, never swallowed); the C ABI returns the codes and the Python layer raises."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SG_ERR_TIMEOUT = 4
SG_ERR_OUT_OF_MEMORY = 5


@pytest.fixture
def lib(sg):
    lib = sg.load_library()
    yield lib
    lib.sg_test_fail_allocations(-1)
    lib.sg_test_set_wait_limits(0, 0)
    lib.sg_test_block_waits(0, 0)


def _grid(sg, torch, n_cp=(30, 22), deg=(3, 2), ns=(200, 150), nout=3, nin=2, dtype=None):
    dtype = dtype or torch.float32
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=1, float_type=dtype)
                 for n, d, s in zip(n_cp[:nin], deg[:nin], ns[:nin]))
    return sg.SplineGrid(dims, nout)


def _expect_oom(sg, lib, make, max_allocs=64):
    """make() under every failure point 0, 1, ... until it succeeds: each failing call
    raises with SG_ERR_OUT_OF_MEMORY and leaves the live-allocation count unchanged."""
    import gc

    import torch
    failures = 0
    for after in range(max_allocs):
        torch.cuda.synchronize()
        live = lib.sg_test_live_allocations()
        lib.sg_test_fail_allocations(after)
        try:
            obj = make()
        except sg.SplineGridsError as e:
            code, msg = e.code, str(e)
        else:
            lib.sg_test_fail_allocations(-1)
            assert failures >= 1
            return obj
        lib.sg_test_fail_allocations(-1)
        gc.collect()  # the half-built Python object, held by the traceback until here
        assert code == SG_ERR_OUT_OF_MEMORY, msg
        assert "allocation" in msg
        assert lib.sg_test_live_allocations() == live, f"leak after {after} allocations"
        failures += 1
    raise AssertionError("the create never succeeded")


def test_grid_plan_create_out_of_memory(sg, lib):
    import torch
    g = _grid(sg, torch)
    live0 = lib.sg_test_live_allocations()
    plan = _expect_oom(sg, lib, lambda: sg.spline_grid._Plan(g, sg.arrays.dtype_code(torch.float32)))
    assert lib.sg_test_live_allocations() > live0
    del plan
    import gc
    gc.collect()
    assert lib.sg_test_live_allocations() == live0


def test_batch_plan_create_out_of_memory(sg, lib):
    import torch
    from test_gpu_batch import _random_grids
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 6, 40, torch.float32, nin=2)
    grids3, *_ = _random_grids(sg, torch, 2, 41, torch.float32, nin=3)
    b = _expect_oom(sg, lib, lambda: sg.GridBatch(grids + grids3))
    del b


def test_fit_and_lsqr_create_out_of_memory(sg, lib):
    import torch
    g = _grid(sg, torch)
    cp = sg.arrays.zeros(tuple(sg.obtain(g.control_points).shape), torch.float32)
    tgt = [sg.arrays.zeros(tuple(g.eval.shape), torch.float32)]
    f = _expect_oom(sg, lib, lambda: sg.grid_fit(g, [(0, 0)], tgt, 1e-3, control_points=cp))
    del f
    A = sg.LinearMap(g)
    # the grid's plan first, so that the solver's own allocations are the ones that fail
    A.mul_(torch.zeros(A.shape[0], device="cuda"), torch.zeros(A.shape[1], device="cuda"))
    s = _expect_oom(sg, lib, lambda: sg.LSQRSolver(A, graph=False))
    del s


def _batch_arrays(sg, torch):
    from test_gpu_batch import _random_grids
    return _random_grids(sg, torch, 8, 60, torch.float32, sets=2, nin=2)


def test_batch_dependency_wait_times_out_and_recovers(sg, lib):
    """The separable pass queue: every pass that reads another's output waits for a
    count that can never be reached; the waits give up after the test's limit."""
    import torch
    grids, cps, evals, cots, grads = _batch_arrays(sg, torch)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.set_strategy("separable")
    batch.run(forward=True, adjoint=True)
    batch.check()
    ref_e = [e.clone() for e in evals]
    ref_g = [g.clone() for g in grads]
    lib.sg_test_set_wait_limits(2000, 0)  # ~0.2 ms of polling per wait
    lib.sg_test_block_waits(1, 0)
    batch.run(forward=True, adjoint=True)
    with pytest.raises(sg.SplineGridsError) as ei:
        batch.check()
    assert ei.value.code == SG_ERR_TIMEOUT
    lib.sg_test_block_waits(0, 0)
    lib.sg_test_set_wait_limits(0, 0)
    for e in evals:
        e.fill_(float("nan"))
    for g in grads:
        g.fill_(float("nan"))
    batch.run(forward=True, adjoint=True)
    batch.check()
    for a, b in zip(evals, ref_e):
        assert torch.equal(a, b)
    for a, b in zip(grads, ref_g):
        assert torch.equal(a, b)


@pytest.mark.parametrize("where", ["grid", "batch"])
def test_fused_adjoint_stage_wait_times_out_and_recovers(sg, lib, where):
    """The fused adjoint: the producer withholds its arrival on every CTA's first stage,
    the consumers' stage waits run out (short budget), the CTAs drain their copies and
    return; the plan's or batch's check reports SG_ERR_TIMEOUT."""
    import torch
    if where == "grid":
        g = _grid(sg, torch, n_cp=(20, 12), ns=(120, 60))  # a few adjoint tiles
        plan = g.plan(torch.float32)
        assert plan.paths()[1] == "fused"
        cot = sg.arrays.from_any(torch.as_tensor(np.random.default_rng(3).standard_normal(
            tuple(g.eval.shape))), torch.float32)
        out = sg.arrays.empty(tuple(sg.obtain(g.control_points).shape), torch.float32)

        def run():
            sg.evaluate_adjoint_(g, eval=cot, control_points=out)

        check = plan.check
        results = [out]
    else:
        grids, cps, evals, cots, grads = _batch_arrays(sg, torch)
        batch = sg.GridBatch(grids)
        batch.set_arrays(cps, evals, cots, grads)
        assert batch.fused_grids() == len(grids)

        def run():
            batch.run(forward=False, adjoint=True)

        check = batch.check
        results = grads
    run()
    check()
    ref = [r.clone() for r in results]
    lib.sg_test_set_wait_limits(0, 200000)  # ~0.1 ms per stage wait
    lib.sg_test_block_waits(0, 1)
    run()
    with pytest.raises(sg.SplineGridsError) as ei:
        check()
    assert ei.value.code == SG_ERR_TIMEOUT
    lib.sg_test_block_waits(0, 0)
    lib.sg_test_set_wait_limits(0, 0)
    for r in results:
        r.fill_(float("nan"))
    run()
    check()
    for a, b in zip(results, ref):
        assert torch.equal(a, b)
