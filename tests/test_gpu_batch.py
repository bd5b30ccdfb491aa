"""The batched persistent path (one launch for many uneven grids) against the per-grid
entry points and the oracle."""
import numpy as np
import pytest

from conftest import normwise_rel

pytestmark = pytest.mark.gpu


def _random_grids(sg, torch, count, seed, dtype, sets=2, nin=2):
    grids, cps, evals, cots, grads = [], [], [], [], []
    for gi in range(count):
        rng = np.random.default_rng(seed + gi)
        n_cp = tuple(int(x) for x in rng.integers(4, 40, size=nin))
        deg = int(rng.integers(1, 4))
        deg = min(deg, min(n_cp) - 1)
        ns = tuple(int(x) for x in rng.integers(5, 120, size=nin))
        nout = int(rng.choice([1, 3])) * sets
        dims = tuple(sg.SplineDimension(n, deg, s, max_derivative_order=1, float_type=dtype)
                     for n, s in zip(n_cp, ns))
        g = sg.SplineGrid(dims, nout)
        cp = sg.arrays.from_any(torch.as_tensor(rng.standard_normal(n_cp + (nout,))), dtype)
        cot = sg.arrays.from_any(torch.as_tensor(rng.standard_normal(ns + (nout,))), dtype)
        grids.append(g)
        cps.append(cp)
        evals.append(sg.arrays.empty(ns + (nout,), dtype))
        cots.append(cot)
        grads.append(sg.arrays.empty(n_cp + (nout,), dtype))
    return grids, cps, evals, cots, grads


@pytest.mark.parametrize("dtype_name", ["f32", "f64"])
@pytest.mark.parametrize("nin", [1, 2, 3])
def test_batch_matches_per_grid(sg, dtype_name, nin):
    import torch
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    tol = 1e-12 if dtype_name == "f64" else 1e-5
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 24 if nin < 3 else 8, 100 * nin,
                                                   dtype, nin=nin)
    orders = [tuple(int(o) for o in np.random.default_rng(i).integers(0, 2, size=nin))
              for i in range(len(grids))]
    batch = sg.GridBatch(grids, orders)
    batch.set_arrays(cps, evals, cots, grads)
    for rep in range(2):  # two runs in a row: counters and queue are reset per run
        for e in evals:
            e.fill_(float("nan"))
        for gr in grads:
            gr.fill_(float("nan"))
        batch.run(forward=True, adjoint=True)
        batch.check()
        for g, o, cp, ev, cot, gr in zip(grids, orders, cps, evals, cots, grads):
            ref = sg.arrays.empty(tuple(ev.shape), dtype)
            sg.evaluate_(g, derivative_order=o, control_points=cp, eval=ref)
            refg = sg.arrays.empty(tuple(gr.shape), dtype)
            sg.evaluate_adjoint_(g, derivative_order=o, eval=cot, control_points=refg)
            assert normwise_rel(ev.cpu().numpy(), ref.cpu().numpy()) <= tol
            assert normwise_rel(gr.cpu().numpy(), refg.cpu().numpy()) <= tol
            # the adjoint is deterministic: identical bits to the per-grid path
            assert torch.equal(gr, refg)


def test_batch_forward_only_and_adjoint_only(sg, oracle):
    import torch
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 10, 7, torch.float64)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.run(forward=True, adjoint=False)
    batch.run(forward=False, adjoint=True)
    batch.check()
    from test_gpu_parity import oracle_spec
    for g, cp, ev, cot, gr in zip(grids, cps, evals, cots, grads):
        spec = oracle_spec(oracle, g)
        ref = oracle.evaluate(spec, np.asfortranarray(cp.cpu().numpy()))
        assert normwise_rel(ev.cpu().numpy(), ref) <= 1e-12
        refg = oracle.evaluate_adjoint(spec, np.asfortranarray(cot.cpu().numpy()))
        assert normwise_rel(gr.cpu().numpy(), refg) <= 1e-12


def test_batch_in_cuda_graph(sg):
    """The batch run is capturable: replaying the graph reproduces the eager results."""
    import torch
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 12, 55, torch.float32)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.run(forward=True, adjoint=True)
    torch.cuda.synchronize()
    ref_e = [e.clone() for e in evals]
    ref_g = [g.clone() for g in grads]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            batch.run(forward=True, adjoint=True)
    for e in evals:
        e.zero_()
    for gr in grads:
        gr.zero_()
    graph.replay()
    graph.replay()
    torch.cuda.synchronize()
    batch.check()
    for a, b in zip(evals + grads, ref_e + ref_g):
        assert torch.equal(a, b)


def test_pipeline_with_host_arrays_matches_batch(sg):
    """GridBatchPipeline (sub-batches, uploads and downloads overlapped on three streams)
    gives per grid the bits of one GridBatch launch, over repeated calls."""
    import torch
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 20, 900, torch.float32)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.run(forward=True, adjoint=True)
    batch.check()
    ref_ev = [e.clone() for e in evals]
    ref_gr = [g.clone() for g in grads]

    def pinned(t):
        base = torch.empty(tuple(reversed(t.shape)), dtype=t.dtype, pin_memory=True)
        return base.permute(*reversed(range(t.dim())))

    h_cp = [pinned(c) for c in cps]
    h_cot = [pinned(c) for c in cots]
    for h, c in zip(h_cp, cps):
        h.copy_(c)
    for h, c in zip(h_cot, cots):
        h.copy_(c)
    h_ev = [pinned(e) for e in evals]
    h_gr = [pinned(g) for g in grads]
    d_cp = [sg.arrays.zeros(tuple(c.shape), torch.float32) for c in cps]
    d_cot = [sg.arrays.zeros(tuple(c.shape), torch.float32) for c in cots]
    d_ev = [sg.arrays.empty(tuple(e.shape), torch.float32) for e in evals]
    d_gr = [sg.arrays.empty(tuple(g.shape), torch.float32) for g in grads]
    pipe = sg.GridBatchPipeline(grids, d_cp, d_ev, d_cot, d_gr, n_chunks=4)
    assert len(pipe.batches) == 4
    for rep in range(2):
        for h in h_ev + h_gr:
            h.fill_(float("nan"))
        pipe.run(h_cp, h_ev, h_cot, h_gr)
        torch.cuda.synchronize()
        pipe.check()
        for h, r in zip(h_ev, ref_ev):
            assert torch.equal(h, r.cpu())
        for h, r in zip(h_gr, ref_gr):
            assert torch.equal(h, r.cpu())


def test_pipeline_capture_replay_matches_run(sg):
    """GridBatchPipeline.capture records one host-data step (uploads, sub-batch launches,
    downloads) as a CUDA graph; each replay copies the host arrays' current contents, so
    negating the inputs in place negates the outputs bit for bit (both passes are linear
    and a sign flip is exact), and a replay equals run()."""
    import torch
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 12, 700, torch.float32)

    def pinned(t):
        base = torch.empty(tuple(reversed(t.shape)), dtype=t.dtype, pin_memory=True)
        return base.permute(*reversed(range(t.dim())))

    h_cp = [pinned(c) for c in cps]
    h_cot = [pinned(c) for c in cots]
    for h, c in zip(h_cp + h_cot, cps + cots):
        h.copy_(c)
    h_ev = [pinned(e) for e in evals]
    h_gr = [pinned(g) for g in grads]
    d_cp = [sg.arrays.zeros(tuple(c.shape), torch.float32) for c in cps]
    d_cot = [sg.arrays.zeros(tuple(c.shape), torch.float32) for c in cots]
    d_ev = [sg.arrays.empty(tuple(e.shape), torch.float32) for e in evals]
    d_gr = [sg.arrays.empty(tuple(g.shape), torch.float32) for g in grads]
    pipe = sg.GridBatchPipeline(grids, d_cp, d_ev, d_cot, d_gr, n_chunks=3)
    pipe.run(h_cp, h_ev, h_cot, h_gr)
    torch.cuda.synchronize()
    pipe.check()
    ref = [h.clone() for h in h_ev + h_gr]
    pipe.capture(h_cp, h_ev, h_cot, h_gr)
    sign = 1.0
    for flip in (False, True, True):
        if flip:  # new host inputs for the next replay: the current ones negated
            for h in h_cp + h_cot:
                h.neg_()
            sign = -sign
        for h in h_ev + h_gr:
            h.fill_(float("nan"))
        pipe.replay()
        torch.cuda.synchronize()
        pipe.check()
        for h, r in zip(h_ev + h_gr, ref):
            assert torch.equal(h, r * sign)


def test_pipeline_capture_refuses_pageable_host_arrays(sg):
    """A captured copy needs page-locked host memory: capture() refuses a pageable array
    before any capture starts."""
    import torch
    grids, cps, evals, cots, grads = _random_grids(sg, torch, 3, 300, torch.float32)
    h_cp = [c.cpu() for c in cps]  # pageable
    pipe = sg.GridBatchPipeline(grids, cps, evals, cots, grads, n_chunks=1)
    with pytest.raises(ValueError, match="not pinned"):
        pipe.capture(h_cp, None, None, None, forward=True, adjoint=False)
    pipe.run(None, None, None, None, forward=True, adjoint=False)  # the pipeline still runs
    torch.cuda.synchronize()
    pipe.check()
