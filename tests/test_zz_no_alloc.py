"""The allocation-free evaluate entry point (sg_evaluate_noalloc) against the plan-based
sg_evaluate, both called through the C ABI.

sg_evaluate_noalloc exists for host code that must not allocate device memory (a fixed
device budget, or a loop that may never wait on the allocator).  It keeps the separable
passes' intermediates in a static per-device array instead of a plan's scratch.  This
file is collected last so that, if it fails, a stop-at-first-failure run has already
run every other test; it passes both alone in a fresh process and after the others.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu


def _grid(sg, torch, n_cp, deg, ns, nout, dtype, seed, max_deriv=1):
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=min(max_deriv, d),
                                    float_type=dtype) for n, d, s in zip(n_cp, deg, ns))
    g = sg.SplineGrid(dims, nout)
    rng = np.random.default_rng(seed)
    sg.obtain(g.control_points).copy_(torch.as_tensor(rng.standard_normal(n_cp + (nout,))))
    return g


@pytest.mark.parametrize("dtype_name,case", [
    ("f32", dict(n_cp=(64, 48), deg=(3, 2), ns=(512, 300), nout=3, order=(1, 0))),
    ("f64", dict(n_cp=(10, 10, 5), deg=(2, 3, 2), ns=(50, 50, 25), nout=4, order=(0, 1, 0))),
    ("f32", dict(n_cp=(20, 9), deg=(2, 2), ns=(70, 33), nout=2, order=(0, 0), nurbs=True)),
    # one axis: the only pass writes eval, no scratch is used
    ("f32", dict(n_cp=(40,), deg=(3,), ns=(1000,), nout=2, order=(1,))),
    # bfloat16-stored control points: axis 0 reads them, later passes use 4-byte scratch
    ("bf16", dict(n_cp=(30, 12, 6), deg=(3, 2, 1), ns=(90, 40, 20), nout=2, order=(0, 1, 0))),
    # the largest intermediate [8192, 256, 4] x 4 bytes is exactly one 32 MiB half
    ("f32", dict(n_cp=(64, 256), deg=(2, 3), ns=(8192, 300), nout=4, order=(0, 0))),
])
def test_noalloc_matches_plan_path_twice(sg, dtype_name, case):
    import torch
    from splinegrids import _lib
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    tol = 1e-12 if dtype_name == "f64" else 1e-5
    lib = _lib.load()
    g = _grid(sg, torch, case["n_cp"], case["deg"], case["ns"], case["nout"], dtype, seed=5)
    if case.get("nurbs"):
        w = np.random.default_rng(6).uniform(0.5, 2.0, case["n_cp"])
        g.weights = sg.arrays.from_any(torch.as_tensor(w), dtype)
    order = case["order"]
    cp = sg.obtain(g.control_points)
    cp_dtype = dtype
    if dtype_name == "bf16":
        cp_dtype = torch.bfloat16
        cpb = sg.arrays.empty(tuple(cp.shape), torch.bfloat16)
        cpb.copy_(cp)
        cp = cpb
    wptr = g.weights.data_ptr() if g.weights is not None else None
    # existing entry point (plan-based) through the C ABI
    ref = sg.arrays.empty(tuple(g.eval.shape), dtype)
    plan = g.plan(cp_dtype)
    _lib.check(lib.sg_evaluate(plan.handle, _lib.i32_array(order), cp.data_ptr(), wptr,
                               ref.data_ptr(), _lib.stream_handle()))
    # the allocation-free entry point, twice in a row with different control points in
    # between, into a buffer holding garbage
    desc = plan.desc
    for call in range(2):
        if call == 1:
            cp.mul_(-0.5).add_(0.25)
            _lib.check(lib.sg_evaluate(plan.handle, _lib.i32_array(order), cp.data_ptr(), wptr,
                                       ref.data_ptr(), _lib.stream_handle()))
        out = sg.arrays.empty(tuple(g.eval.shape), dtype)
        out.fill_(float("nan"))
        _lib.check(lib.sg_evaluate_noalloc(C.byref(desc), _lib.i32_array(order), cp.data_ptr(),
                                           wptr, out.data_ptr(), _lib.stream_handle()))
        torch.cuda.synchronize()
        assert not torch.isnan(out).any()
        assert normwise_rel(out.cpu().numpy(), ref.cpu().numpy()) <= tol


def test_noalloc_rejects_oversized_intermediate(sg):
    """A grid whose intermediate exceeds the static scratch is refused with a clear
    error (before any launch)."""
    import torch
    from splinegrids import _lib
    desc = _lib.GridDesc()
    desc.nin, desc.nout, desc.dtype, desc.has_weights = 2, 4, _lib.SG_F32, 0
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    for k, (ns, n) in enumerate([(1 << 20, 64), (64, 64)]):
        desc.n_samples[k], desc.n_basis[k] = ns, n
        desc.degree[k], desc.max_derivative_order[k] = 3, 0
        desc.sample_indices[k] = dummy.data_ptr()
        desc.basis_eval[k] = dummy.data_ptr()
    rc = _lib.load().sg_evaluate_noalloc(C.byref(desc), _lib.i32_array((0, 0)),
                                         dummy.data_ptr(), None, dummy.data_ptr(),
                                         _lib.stream_handle())
    assert rc == _lib.SG_ERR_UNSUPPORTED
    assert "scratch" in _lib.last_error()


def test_noalloc_rejects_one_row_over_the_half(sg):
    """One axis-0 sample more than the exactly-fitting case: the intermediate is 16 KiB
    over the 32 MiB half and the call is refused before any launch."""
    import torch
    from splinegrids import _lib
    g = _grid(sg, torch, (64, 256), (2, 3), (8193, 300), 4, torch.float32, seed=7)
    out = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
    rc = _lib.load().sg_evaluate_noalloc(C.byref(g.plan(torch.float32).desc), _lib.i32_array((0, 0)),
                                         sg.obtain(g.control_points).data_ptr(), None,
                                         out.data_ptr(), _lib.stream_handle())
    assert rc == _lib.SG_ERR_UNSUPPORTED
    assert "scratch" in _lib.last_error()


@pytest.mark.parametrize("nurbs,order", [(True, (1, 0)), (False, (2, 0)), (False, (0, -1))])
def test_noalloc_rejects_orders_like_sg_evaluate(sg, nurbs, order):
    """Unavailable derivative orders get the same status and message from both entry
    points (the reference's validate_partial_derivatives, src/validation.jl:76-102)."""
    import torch
    from splinegrids import _lib
    lib = _lib.load()
    g = _grid(sg, torch, (12, 10), (2, 2), (30, 20), 1, torch.float32, seed=8)
    wptr = None
    if nurbs:
        g.weights = sg.arrays.from_any(torch.ones(12, 10, dtype=torch.float64), torch.float32)
        wptr = g.weights.data_ptr()
    plan = g.plan(torch.float32)
    out = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
    cp = sg.obtain(g.control_points)
    rc1 = lib.sg_evaluate(plan.handle, _lib.i32_array(order), cp.data_ptr(), wptr, out.data_ptr(),
                          _lib.stream_handle())
    m1 = _lib.last_error()
    rc2 = lib.sg_evaluate_noalloc(C.byref(plan.desc), _lib.i32_array(order), cp.data_ptr(), wptr,
                                  out.data_ptr(), _lib.stream_handle())
    m2 = _lib.last_error()
    assert rc1 != 0 and rc1 == rc2
    assert m1 == m2
    assert rc1 == (_lib.SG_ERR_UNSUPPORTED if nurbs else _lib.SG_ERR_INVALID_ARGUMENT)
