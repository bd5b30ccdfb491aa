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
