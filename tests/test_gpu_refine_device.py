"""Device local-refinement selection against host restatements of the reference.

error_informed_local_refinement! (src/control_points.jl:555-578) and
deactivate_overwritten_control_points! (:584-680) run on the device (sg_sum_outputs,
sg_select_above, sg_select_rows and the structural adjoint).  Here they are checked
against numpy restatements of the reference's steps on the same inputs: sum over
outputs, threshold_factor * mean, findall in column-major order, unique against the
level's indices; the `Flag` adjoint as a Boolean OR over the bands.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(sg, torch, dtype, seed):
    dims = tuple(sg.SplineDimension(n, 2, s, float_type=dtype) for n, s in zip((7, 6), (61, 53)))
    g = sg.add_default_local_refinement(sg.SplineGrid(dims, 2))
    sg.activate_local_control_point_range_(g, range(1, 5), range(2, 7))
    g = sg.add_default_local_refinement(g)
    sg.activate_local_control_point_range_(g, range(3, 10), range(0, 5))
    sg.activate_local_control_point_range_(g, range(12, 20), range(6, 14))
    return g


def _host_error_refinement(sg, g, err, factor):
    """The reference's steps on the host (the adjoint itself is the GPU's, checked elsewhere)."""
    import torch
    finest = sg.obtain(g.control_points)
    cp_err = sg.arrays.zeros(tuple(finest.shape), g.dtype)
    sg.evaluate_adjoint_(g, eval=err, control_points=cp_err)
    e = np.asfortranarray(cp_err.cpu().numpy())
    ge = e[..., 0].copy()
    for o in range(1, e.shape[-1]):
        ge = ge + e[..., o]
    thr = factor * float(ge.astype(np.float64).sum()) / ge.size
    lin = np.nonzero(ge.flatten(order="F").astype(np.float64) > thr)[0]
    new = np.stack(np.unravel_index(lin, ge.shape, order="F"), axis=1) + 1
    lr = g.control_points.local_refinements[-1]
    old = lr.refinement_indices.cpu().numpy()
    seen = {tuple(r) for r in old}
    add = np.array([r for r in new if tuple(r) not in seen], dtype=np.int32).reshape(-1, ge.ndim)
    fin = np.asfortranarray(finest.cpu().numpy())
    add_vals = np.array([fin[tuple(r - 1)] for r in add]).reshape(-1, fin.shape[-1])
    return (np.concatenate([old, add], 0),
            np.concatenate([lr.refinement_values.cpu().numpy(), add_vals], 0))


@pytest.mark.parametrize("dt,factor", [("float32", 1.0), ("float64", 0.5), ("float32", 2.5)])
def test_error_informed_refinement_matches_host_steps(sg, dt, factor):
    import torch
    dtype = getattr(torch, dt)
    g = _grid(sg, torch, dtype, 0)
    rng = np.random.default_rng(1)
    err = sg.arrays.from_any(torch.as_tensor(np.abs(rng.standard_normal(tuple(g.eval.shape))) ** 3),
                             dtype)
    ref_idx, ref_vals = _host_error_refinement(sg, g, err, factor)
    sg.error_informed_local_refinement_(g, err, threshold_factor=factor)
    lr = g.control_points.local_refinements[-1]
    assert lr.refinement_indices.cpu().numpy().tolist() == ref_idx.tolist()
    assert np.array_equal(lr.refinement_values.cpu().numpy(), ref_vals)
    # activating again with the same error selects nothing new
    n = lr.n_refined
    sg.error_informed_local_refinement_(g, err, threshold_factor=factor)
    assert g.control_points.local_refinements[-1].n_refined == n


def _host_flags(lr_next, size_next, size_cur):
    flags = np.ones(size_next, dtype=np.int64)
    nxt = lr_next.refinement_indices.cpu().numpy() - 1
    if nxt.shape[0]:
        flags[tuple(nxt[:, d] for d in range(nxt.shape[1]))] = 0
    cur = flags
    for A, d in zip(lr_next.refinement_matrices, lr_next.dims_refinement):
        inc = np.zeros((A.m, A.n), dtype=np.int64)
        for i in range(A.m):
            c0, c1, _ = A.row_range(i)
            inc[i, c0:c1 + 1] = 1
        cur = (np.moveaxis(np.tensordot(inc.T, cur, axes=([1], [d])), 0, d) > 0).astype(np.int64)
    assert cur.shape == size_cur
    return cur


def test_deactivation_matches_host_flag_propagation(sg):
    import torch
    g = _grid(sg, torch, torch.float64, 0)
    cps = g.control_points
    # overwrite most of level 1 at level 2 so that some level-1 points lose all effect
    sg.activate_local_control_point_range_(g, range(0, 22), range(0, 18))
    lrs = cps.local_refinements
    expect, dropped = [], 0
    for lev in range(len(lrs) - 2, -1, -1):
        size_next = tuple(cps.control_points_refined[lev + 1].shape[:-1])
        size_cur = tuple(cps.control_points_refined[lev].shape[:-1])
        cur = _host_flags(lrs[lev + 1], size_next, size_cur)
        idx = lrs[lev].refinement_indices.cpu().numpy() - 1
        keep = cur[tuple(idx[:, d] for d in range(idx.shape[1]))] > 0 if idx.shape[0] else \
            np.zeros(0, bool)
        expect.append((lev, (idx[keep] + 1).tolist(), lrs[lev].refinement_values.cpu().numpy()[keep]))
        dropped += int((~keep).sum())
        # apply the host result level by level, as the reference's loop does
        sg.deactivate_overwritten_control_points_(cps, lev)
        got = lrs[lev]
        assert got.refinement_indices.cpu().numpy().tolist() == expect[-1][1]
        assert np.array_equal(got.refinement_values.cpu().numpy(), expect[-1][2])
    assert dropped > 0  # the case exercises the deactivation


@pytest.mark.parametrize("dt", ["float32", "float64"])
@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_device_refinement_matrix_bit_identical_to_composed_products(sg, dt, deg):
    """sg_refine_matrix (one launch for all knots) against composing the single-knot
    matrices with the banded product on the host, knot by knot as the reference does
    (src/refinement.jl:256-284): identical row pointers, column starts and values."""
    import torch
    npdt = np.float32 if dt == "float32" else np.float64
    rng = np.random.default_rng(deg)
    for trial in range(4):
        nv = int(rng.integers(3, 40))
        kv = np.sort(rng.random(nv)).astype(npdt)
        kv[0], kv[-1] = 0, 1
        kv = np.unique(kv)
        mult = np.ones(len(kv), np.int32)
        mult[0] = mult[-1] = deg + 1
        if trial == 1 and len(kv) > 4:
            mult[2] = deg  # an interior knot of multiplicity degree
        knots_new = None if trial != 2 else np.sort(
            rng.uniform(kv[0], kv[-1], 25).astype(npdt))
        if knots_new is not None:
            knots_new = np.setdiff1d(knots_new, kv)
        kv2, mult2, R = sg.refine_knots(kv, mult, deg, knots_new)
        _, _, knots, spans = sg.knot_span_sequence(kv, mult, knots_new)
        knots_all = torch.as_tensor(sg.expand_knots(kv, mult)).cuda()
        Rd = sg.refinement_matrix_device(knots_all, deg, knots, spans)
        assert (Rd.m, Rd.n) == (R.m, R.n)
        assert np.array_equal(Rd.row_pointer, R.row_pointer)
        assert np.array_equal(Rd.column_start, R.column_start)
        assert Rd.nzval.dtype == R.nzval.dtype
        assert np.array_equal(Rd.nzval.view(np.uint8), R.nzval.view(np.uint8))
    # a single insertion is the single-knot matrix itself
    kv = np.array([0, 0.25, 0.6, 1], dtype=npdt)
    mult = np.array([deg + 1, 1, 1, deg + 1], np.int32)
    kv2, mult2, ksi = sg.insert_knot_values(kv, mult, npdt(0.4))
    ref = sg.knot_insertion_matrix(sg.expand_knots(kv, mult), deg, ksi, npdt(0.4))
    one = sg.refinement_matrix_device(torch.as_tensor(sg.expand_knots(kv, mult)).cuda(), deg,
                                      [npdt(0.4)], [ksi])
    assert np.array_equal(one.collect(), ref.collect())
