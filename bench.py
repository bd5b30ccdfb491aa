"""Benchmark of the grid-evaluation hot path on one GB300 (replicas on N > 1).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batched|large2d] [--mode bench|profile|align [--ns0 N]]

Workload "batched" (default; the batched uneven-grids configuration): 256 grids with
Nin = 2; grid g draws, from numpy default_rng(5 + g), n_control per dimension uniform
in [8, 128], one degree in {1, 2, 3}, n_samples per dimension uniform in [64, 1024] and
Nout in {1, 3}; each grid has 16 control-point sets (N(0,1) FP32), folded into the
channel axis.  One step is forward + adjoint of every grid and set through one
sg_batch_run call (the fused forward tiles in one launch, then the fused adjoint tiles in
one persistent launch), replayed from a CUDA graph, with unit sizes tuned on the plan's
own arrays first; units are output values (each written once by the forward and its
cotangent read once by the adjoint).  The eval and cotangent arrays (9.7 GB each)
exceed the 126 MB L2 many times, so no flush is needed.  Side lines: the same step on
the separable pass queue, forward and adjoint alone, the captured fit loop, e2e.

Workload "large2d" (the Large-2D surface configuration): n_control (256, 256), degree
(3, 3), n_samples (4096, 4096), Nout 3, derivative orders (0,0), (1,0), (0,1); one step
is forward + adjoint of the three orders through the per-grid entry points.  The
batched run also measures this grid's plain FP64 forward and forward+adjoint (the
single-grid FP64 path the batched FP32 throughput is compared with) and its per-step
rooflines.

Prints one JSON line (rank 0).  `value` = output values/s with inputs resident in HBM;
`e2e` = the same through the public API from pinned host buffers (inputs copied in and
results copied out inside the timed region, 10 steps, min/median/max; the captured
GridBatchPipeline step, with the uncaptured `run` beside it).  `--impl
reference` times the CPU oracle (a C/OpenMP restatement of the reference's kernels; the
reference itself is Julia, which is not installed) on the whole batched configuration
with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "splinegrids.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "output values/s fwd & fwd+adjoint, batched FP32 vs plain FP64 at ≤1e-5 rel err"
UNIT = "output values/s"

BATCHED = dict(n_grids=256, seed0=5, ncp=(8, 128), deg=(1, 3), ns=(64, 1024), nout=(1, 3),
               sets=16)
LARGE2D = dict(n_cp=(256, 256), deg=(3, 3), ns=(4096, 4096), nout=3, seed=1,
               orders=((0, 0), (1, 0), (0, 1)), max_deriv=1)


# ------------------------------------------------------------------ ranks
def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(ws, v: float) -> float:
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=10)
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _time_region(torch, fn, steps, warmup, ws):
    """W untimed steps, then K steps bracketed by barrier + synchronize, timed with CUDA
    events on the current stream.  Returns seconds."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    _barrier(ws)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        fn()
    stop.record()
    torch.cuda.synchronize()
    _barrier(ws)
    return start.elapsed_time(stop) / 1e3


def _load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def _peak_hbm():
    p = _load_peaks().get("hbm_gbs")
    return (p, "measured") if p else (6800.0, "fallback")


def _load_traffic(key):
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(key)
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------------ batched workload
def batched_specs(n_grids=None):
    """The per-grid draws of the batched configuration (host only)."""
    c = BATCHED
    out = []
    for g in range(n_grids or c["n_grids"]):
        rng = np.random.default_rng(c["seed0"] + g)
        n_cp = tuple(int(x) for x in rng.integers(c["ncp"][0], c["ncp"][1] + 1, size=2))
        deg = int(rng.integers(c["deg"][0], c["deg"][1] + 1))
        ns = tuple(int(x) for x in rng.integers(c["ns"][0], c["ns"][1] + 1, size=2))
        nout = int(rng.choice(list(c["nout"])))
        out.append(dict(n_cp=n_cp, deg=deg, ns=ns, nout=nout, ch=nout * c["sets"], rng=rng))
    return out


def batched_bytes(specs, itemsize=4):
    """Algorithmic bytes of one forward and one adjoint of every grid (per-unit model:
    forward V*s_out + |P|*s_cp + sum ns_k (d_k+1) s_b; adjoint V*s_out + |P_bar|*s_cp)."""
    fwd = adj = vals = 0
    for s in specs:
        V = s["ns"][0] * s["ns"][1] * s["ch"]
        P = s["n_cp"][0] * s["n_cp"][1] * s["ch"]
        basis = sum(n * (s["deg"] + 1) for n in s["ns"])
        fwd += (V + P + basis) * itemsize
        adj += (V + P) * itemsize
        vals += V
    return fwd, adj, vals


def build_batched(sg, torch, dtype, n_grids=None):
    specs = batched_specs(n_grids)
    grids, cps, evals, cots, grads = [], [], [], [], []
    gen = torch.Generator(device="cuda").manual_seed(3)
    for s in specs:
        dims = tuple(sg.SplineDimension(n, s["deg"], m, float_type=dtype)
                     for n, m in zip(s["n_cp"], s["ns"]))
        ev = sg.arrays.empty(s["ns"] + (s["ch"],), dtype)
        cp = sg.arrays.empty(s["n_cp"] + (s["ch"],), dtype)
        cp.copy_(torch.as_tensor(s["rng"].standard_normal(s["n_cp"] + (s["ch"],))))
        g = sg.SplineGrid(dims, control_points=cp, eval=ev)
        cot = sg.arrays.empty(s["ns"] + (s["ch"],), dtype)
        cot.copy_(torch.randn(tuple(cot.shape), generator=gen, device="cuda", dtype=dtype))
        grids.append(g)
        cps.append(cp)
        evals.append(ev)
        cots.append(cot)
        grads.append(sg.arrays.empty(s["n_cp"] + (s["ch"],), dtype))
    return specs, grids, cps, evals, cots, grads


def _capture(torch, fn):
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        fn()  # warm the stream once outside the capture
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=s):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    return graph


def batched_accuracy(oracle, grids, cps, evals, cots, grads, count=6):
    """Normwise relative error of the first `count` grids against the FP64 oracle."""
    fe = ae = 0.0
    for g, cp, ev, cot, gr in list(zip(grids, cps, evals, cots, grads))[:count]:
        sidx, bs = [], []
        for d in g.spline_dimensions:
            kn = d.knot_vector.knots_all.cpu().numpy().astype(np.float64)
            sp = d.sample_points.cpu().numpy().astype(np.float64)
            si = oracle.sample_indices(sp, kn, d.degree)
            sidx.append(si)
            bs.append(oracle.basis(kn, sp, si, d.degree, 0))
        spec = oracle.GridSpec(sidx, bs, [d.degree for d in g.spline_dimensions],
                               [d.n_basis_functions for d in g.spline_dimensions])
        ref = oracle.evaluate(spec, np.asfortranarray(cp.cpu().numpy().astype(np.float64)))
        fe = max(fe, float(np.abs(ev.cpu().numpy() - ref).max() / np.abs(ref).max()))
        refg = oracle.evaluate_adjoint(spec, np.asfortranarray(cot.cpu().numpy().astype(np.float64)))
        ae = max(ae, float(np.abs(gr.cpu().numpy() - refg).max() / np.abs(refg).max()))
    return fe, ae


def reference_workload(O, n_grids=None, dtype=np.float32):
    """Host inputs and output buffers of the batched configuration for the oracle: the
    same per-grid draws (sizes, degree, Nout, control points) as the device arrays;
    cotangents uniform in [-0.5, 0.5) (their values do not change the CPU's work)."""
    specs = batched_specs(n_grids)
    work = []
    crng = np.random.default_rng(1)
    for s in specs:
        dims = [O.default_dimension(n, s["deg"], m, 0, dtype=dtype)
                for n, m in zip(s["n_cp"], s["ns"])]
        spec = O.GridSpec([x["sidx"] for x in dims], [x["basis"] for x in dims],
                          [s["deg"]] * 2, s["n_cp"])
        cp = np.asfortranarray(s["rng"].standard_normal(s["n_cp"] + (s["ch"],)).astype(dtype))
        cot = np.asfortranarray(crng.random(s["ns"] + (s["ch"],), dtype=np.float32) - 0.5,
                                dtype=dtype)
        ev = np.empty(s["ns"] + (s["ch"],), dtype=dtype, order="F")
        gr = np.empty(s["n_cp"] + (s["ch"],), dtype=dtype, order="F")
        work.append((spec, cp, cot, ev, gr))
    vals = sum(s["ns"][0] * s["ns"][1] * s["ch"] for s in specs)
    return work, vals


def reference_step(O, work):
    """evaluate! then evaluate_adjoint! of every grid, in place (src/spline_grid.jl:200-230,
    src/adjoint.jl:42-83), each call on all the oracle's threads."""
    for spec, cp, cot, ev, gr in work:
        O.evaluate(spec, cp, out=ev)
        O.evaluate_adjoint(spec, cot, out=gr)


def cpu_sample_batched(oracle, steps=2, dtype=np.float32):
    """The oracle's forward + adjoint of the whole batched configuration (256 grids x 16
    sets), all host threads, one untimed step then `steps` timed ones:
    (values/s, threads, description)."""
    work, vals = reference_workload(oracle, dtype=dtype)
    reference_step(oracle, work)
    t0 = time.perf_counter()
    for _ in range(steps):
        reference_step(oracle, work)
    dt = time.perf_counter() - t0
    desc = (f"oracle {np.dtype(dtype).name} forward+adjoint of all {BATCHED['n_grids']} grids "
            f"x {BATCHED['sets']} sets of the batched configuration ({vals} values per step), "
            f"{steps} steps after one untimed step")
    return vals * steps / dt, oracle.num_threads(), desc


def pinned_like(torch, t):
    """Pinned host tensor with the same (column-major) layout as the device tensor `t`,
    so host<->device copies are single contiguous transfers."""
    base = torch.empty(tuple(reversed(t.shape)), dtype=t.dtype, pin_memory=True)
    return base.permute(*reversed(range(t.dim())))


def e2e_host_buffers(sg, torch, grids):
    """Pinned host arrays of the e2e step (control points and cotangents in, evals and
    gradients out), allocated right before the e2e measurement (per-tensor pinned
    allocations, 20.4 GB in all)."""
    dev = [(sg.obtain(g.control_points), g.eval) for g in grids]
    h_cp = [pinned_like(torch, cp) for cp, _ in dev]
    h_ev = [pinned_like(torch, ev) for _, ev in dev]
    h_cot = [pinned_like(torch, ev) for _, ev in dev]
    h_gr = [pinned_like(torch, cp) for cp, _ in dev]
    for h, (cp, _) in zip(h_cp, dev):
        h.copy_(cp)
    for h in h_cot:
        h.normal_()
    return h_cp, h_ev, h_cot, h_gr


def measure_e2e_batched(sg, torch, batch, specs, grids, args, ws, host=None, steps=10,
                        n_chunks=16):
    """Forward+adjoint of every grid through the public API with host data
    (GridBatchPipeline): H2D of all control points and cotangents, D2H of all evals and
    gradients, each step, from/to pinned host memory, overlapped with the launches.
    The headline is the captured pipeline (`capture` once, then one graph replay per
    step: every copy and launch of the step, the host issuing nothing per array); the
    same step through `run` (about a thousand copy calls per step from the host) is
    reported beside it.  Each: `steps` timed steps after 3 untimed ones, each bracketed
    by its own events."""
    dev = [(sg.obtain(g.control_points), g.eval) for g in grids]
    h_cp, h_ev, h_cot, h_gr = host if host is not None else e2e_host_buffers(sg, torch, grids)
    d_cot = batch._arrays[2]
    d_gr = batch._arrays[3]
    # the public host-data entry point: sub-batches with uploads, launches and downloads
    # overlapped on three streams
    pipe = sg.GridBatchPipeline(grids, [cp for cp, _ in dev], [ev for _, ev in dev], d_cot,
                                d_gr, n_chunks=n_chunks)
    _, _, vals = batched_bytes(specs)
    h2d = sum(h.numel() * 4 for h in h_cp) + sum(h.numel() * 4 for h in h_cot)
    d2h = sum(h.numel() * 4 for h in h_ev) + sum(h.numel() * 4 for h in h_gr)

    def timed(step):
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        _barrier(ws)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record()
        for i in range(steps):
            step()
            ev[i + 1].record()
        torch.cuda.synchronize()
        _barrier(ws)
        pipe.check()
        per = [ev[i].elapsed_time(ev[i + 1]) / 1e3 for i in range(steps)]
        t = _max_over_ranks(ws, ev[0].elapsed_time(ev[steps]) / 1e3)
        rates = sorted(vals * ws / x for x in per)
        return {"value": vals * ws * steps / t, "unit": UNIT, "steps": steps,
                "per_step": {"min": rates[0], "median": statistics.median(rates), "max": rates[-1],
                             "ms_in_order": [round(x * 1e3, 2) for x in per]},
                "host_link_gbs": (h2d + d2h) * steps / t / 1e9}

    uncaptured = timed(lambda: pipe.run(h_cp, h_ev, h_cot, h_gr, forward=True, adjoint=True))
    uncaptured["call"] = "GridBatchPipeline.run per step"
    pipe.capture(h_cp, h_ev, h_cot, h_gr, forward=True, adjoint=True)
    res = timed(pipe.replay)
    res.update({"h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "call": "GridBatchPipeline.capture once, then GridBatchPipeline.replay per step "
                        f"(one CUDA graph: the {len(pipe.batches)} sub-batches' uploads from pinned host memory, "
                        "launches and downloads to pinned host memory, overlapped on three "
                        "streams)",
                "uncaptured": uncaptured})
    return res


# ------------------------------------------------------------------ large2d workload
def build_large2d(sg, torch, dtype, n_orders=3):
    c = LARGE2D
    dims = tuple(sg.SplineDimension(n, d, s, max_derivative_order=c["max_deriv"], float_type=dtype)
                 for n, d, s in zip(c["n_cp"], c["deg"], c["ns"]))
    ev0 = sg.arrays.empty(c["ns"] + (c["nout"],), dtype)
    cp = sg.arrays.empty(c["n_cp"] + (c["nout"],), dtype)
    cp.copy_(torch.as_tensor(np.random.default_rng(c["seed"]).standard_normal(
        c["n_cp"] + (c["nout"],))))
    g = sg.SplineGrid(dims, control_points=cp, eval=ev0)
    evals = [ev0] + [sg.arrays.empty(c["ns"] + (c["nout"],), dtype) for _ in range(n_orders - 1)]
    gen = torch.Generator(device="cuda").manual_seed(3)
    cots = []
    for _ in range(n_orders):
        e = sg.arrays.empty(c["ns"] + (c["nout"],), dtype)
        e.copy_(torch.randn(tuple(e.shape), generator=gen, device="cuda", dtype=dtype))
        cots.append(e)
    grads = [sg.arrays.empty(c["n_cp"] + (c["nout"],), dtype) for _ in range(n_orders)]
    return g, cp, evals, cots, grads


def _timed_fit(torch, fit, steps, ws, vals, nbytes, call):
    """A captured fit step (forward, loss, adjoint, update), one graph replay per step."""
    fit.capture(steps=1)
    t = _max_over_ranks(ws, _time_region(torch, fit.replay, steps, 3, ws))
    peak, _ = _peak_hbm()
    return {"value": vals * ws * steps / t, "unit": UNIT, "ms_per_step": t / steps * 1e3,
            "algorithmic_bytes": nbytes, "achieved_gbs": nbytes * steps / t / 1e9,
            "frac": nbytes * steps / t / 1e9 / peak, "loss_last": fit.loss(), "call": call,
            "graph": "one CUDA graph replay per step; replay is bitwise the eager loop (tested)"}


def measure_captured_loop(sg, torch, batch, grids, cps, evals, cots, specs, steps, ws):
    """The fit loop over the batched configuration: forward of every grid, loss against a
    target per grid (writes the cotangents), adjoint, update of every control-point
    array; units = output values (each written by the forward once per step)."""
    targets = [sg.arrays.empty(tuple(e.shape), torch.float32) for e in evals]
    gen = torch.Generator(device="cuda").manual_seed(11)
    for t in targets:
        t.copy_(torch.randn(tuple(t.shape), generator=gen, device="cuda"))
    saved = [c.clone() for c in cps]
    fit = sg.batch_fit(batch, targets, 1e-4)
    fwd, adj, vals = batched_bytes(specs)
    P = sum(s["n_cp"][0] * s["n_cp"][1] * s["ch"] for s in specs)
    nbytes = fwd + adj + 3 * vals * 4 + 3 * P * 4  # + loss (eval, target, cotangent), update
    out = _timed_fit(torch, fit, steps, ws, vals, nbytes, "batch_fit(GridBatch): forward, "
                     "sg_fit_loss, adjoint, sg_fit_update")
    batch.check()
    for c, s0 in zip(cps, saved):
        c.copy_(s0)
    del targets, fit
    return out


NURBS_LR = dict(base=(16, 16, 8), degree=2, levels=3, box=0.25, ns=(512, 512, 256), seed=6)


def measure_nurbs_lr(sg, torch, steps, ws):
    """NURBS + 3-level local refinement in 3D (FP32 forward): the refinement chain
    (evaluate!(::LocallyRefinedControlPoints)) then the NURBS evaluation of the finest
    grid with weights U[0.5, 2]; plus the plain variant's forward+adjoint."""
    c = NURBS_LR
    rng = np.random.default_rng(c["seed"])
    dims = tuple(sg.SplineDimension(n, c["degree"], s) for n, s in zip(c["base"], c["ns"]))
    g = sg.SplineGrid(dims, 1)
    sg.obtain(g.control_points).copy_(torch.as_tensor(rng.standard_normal(c["base"] + (1,))))
    for _ in range(c["levels"]):
        g = sg.add_default_local_refinement(g)
        ranges = []
        for n in sg.obtain(g.control_points).shape[:-1]:
            ln = max(1, int(round(n * c["box"] ** (1 / 3))))
            s0 = int(rng.integers(0, n - ln + 1))
            ranges.append(range(s0, s0 + ln))
        sg.activate_local_control_point_range_(g, *ranges)
    cps = g.control_points
    sg.evaluate_control_points_(cps)
    finest = sg.obtain(cps)
    ng = sg.NURBSGrid(g.spline_dimensions, 1)
    ng.weights.copy_(torch.as_tensor(rng.uniform(0.5, 2.0, tuple(finest.shape[:-1]))))
    V = int(np.prod(c["ns"]))

    def nurbs_step():
        sg.evaluate_control_points_(cps)
        sg.obtain(ng.control_points).copy_(finest)
        sg.evaluate_(ng)

    cot = sg.arrays.empty(tuple(g.eval.shape), torch.float32)
    cot.normal_()
    grad = sg.arrays.empty(tuple(finest.shape), torch.float32)

    def plain_step():
        sg.evaluate_(g)
        sg.evaluate_adjoint_(g, eval=cot, control_points=grad)

    t_n = _max_over_ranks(ws, _time_region(torch, nurbs_step, steps, 3, ws))
    t_p = _max_over_ranks(ws, _time_region(torch, plain_step, steps, 3, ws))
    g.plan(torch.float32).check()
    return {"workload": "nurbs_3level_local_refinement_16x16x8_d2_512x512x256_nout1",
            "finest_control_grid": list(finest.shape[:-1]),
            "nurbs_fp32_forward": {"value": V * ws * steps / t_n, "unit": UNIT,
                                   "ms_per_step": t_n / steps * 1e3,
                                   "eval_write_gbs": V * 4 * steps / t_n / 1e9},
            "plain_fp32_fwd_adj": {"value": V * ws * steps / t_p, "unit": UNIT,
                                   "ms_per_step": t_p / steps * 1e3}}


def large2d_bytes(itemsize=4, cp_itemsize=None):
    """Algorithmic bytes of one order's forward and adjoint on the Large-2D grid:
    eval written (or cotangent read) once, control points read (or gradient written)
    once, each axis's basis values (d + 1 per sample) and sample indices read once."""
    c = LARGE2D
    cp_itemsize = cp_itemsize or itemsize
    V1 = int(np.prod(c["ns"])) * c["nout"]
    P = int(np.prod(c["n_cp"])) * c["nout"]
    tables = sum(n * (d + 1) * itemsize + n * 4 for n, d in zip(c["ns"], c["deg"]))
    return V1 * itemsize + P * cp_itemsize + tables, V1 * itemsize + P * itemsize + tables


def _roof(nbytes, seconds, peak, what, kernels):
    gbs = nbytes / seconds / 1e9
    return {"kernels": kernels, "what": what, "bytes": nbytes, "ms": seconds * 1e3,
            "achieved": gbs, "peak": peak, "frac": gbs / peak}


def measure_large2d(sg, torch, steps, ws):
    """The per-grid entry points on the Large-2D grid: FP32 forward+adjoint of the three
    orders (the fused path, and the separable passes for comparison), FP32 forward,
    the multi-order forward, BF16-stored control points, FP64 forward and
    forward+adjoint; per-step rooflines (three orders back to back, 1.2 GB per step, far
    above L2) and single-launch timings."""
    c = LARGE2D
    orders = c["orders"]
    no = len(orders)
    V = int(np.prod(c["ns"])) * c["nout"] * no
    g, cp, evals, cots, grads = build_large2d(sg, torch, torch.float32)
    plan = g.plan(torch.float32)
    paths = plan.paths()
    # the plan's adjoint tiling measured on its own arrays (bitwise neutral), as the batch
    tuned = sg.tune_adjoint_(g, derivative_order=orders[0], eval=cots[0], control_points=grads[0])

    def fwd_adj():
        for o, ev, e, gr in zip(orders, evals, cots, grads):
            sg.evaluate_(g, derivative_order=o, eval=ev)
            sg.evaluate_adjoint_(g, derivative_order=o, eval=e, control_points=gr)

    def fwd():
        for o, ev in zip(orders, evals):
            sg.evaluate_(g, derivative_order=o, eval=ev)

    def adj():
        for o, e, gr in zip(orders, cots, grads):
            sg.evaluate_adjoint_(g, derivative_order=o, eval=e, control_points=gr)

    def fwd_multi():
        sg.evaluate_multi_(g, orders, evals=evals)

    t_fa = _max_over_ranks(ws, _time_region(torch, fwd_adj, steps, 3, ws))
    t_f = _max_over_ranks(ws, _time_region(torch, fwd, steps, 3, ws))
    t_a = _max_over_ranks(ws, _time_region(torch, adj, steps, 3, ws))
    t_fm = _max_over_ranks(ws, _time_region(torch, fwd_multi, steps, 3, ws))
    plan.set_strategy("separable")
    t_fa_sep = _max_over_ranks(ws, _time_region(torch, fwd_adj, steps, 3, ws))
    plan.set_strategy("auto")
    # the captured fit step of the optics example's shape: three orders, loss, adjoints,
    # update (targets: the current evals plus noise)
    fb, ab = large2d_bytes(4)
    V1 = int(np.prod(c["ns"])) * c["nout"]
    P1 = int(np.prod(c["n_cp"])) * c["nout"]
    targets = [e.clone().add_(0.1) for e in evals]
    cfit = cp.clone()
    fit = sg.grid_fit(g, orders, targets, 1e-8, control_points=cfit)
    fit_line = _timed_fit(torch, fit, steps, ws, V, no * (fb + ab + 3 * V1 * 4) + 5 * P1 * 4,
                          "grid_fit: evaluate_multi_ of 3 orders, sg_fit_loss, 3 adjoints, "
                          "sg_fit_update")
    del targets, cfit, fit
    plan.enable_timing(True)
    fp, ap = [], []
    for _ in range(max(5, steps)):
        sg.evaluate_(g, derivative_order=orders[0], eval=evals[0])
        fp.append(plan.pass_times())
        sg.evaluate_adjoint_(g, derivative_order=orders[0], eval=cots[0], control_points=grads[0])
        ap.append(plan.pass_times())
    plan.enable_timing(False)
    plan.check()
    fwd_ms = [statistics.median(x) for x in zip(*fp)]
    adj_ms = [statistics.median(x) for x in zip(*ap)]
    cpb = sg.arrays.empty(tuple(cp.shape), torch.bfloat16)
    cpb.copy_(cp)

    def fwdbf():
        for o, ev in zip(orders, evals):
            sg.evaluate_(g, derivative_order=o, eval=ev, control_points=cpb)
    t_bf = _max_over_ranks(ws, _time_region(torch, fwdbf, steps, 3, ws))
    del g, cp, evals, cots, grads, cpb, plan
    torch.cuda.empty_cache()
    g64, _, ev64, cot64, gr64 = build_large2d(sg, torch, torch.float64, n_orders=3)

    def fwd64():
        for o, ev in zip(orders, ev64):
            sg.evaluate_(g64, derivative_order=o, eval=ev)

    def fwd_adj64():  # the plain single-grid FP64 path on the same step as the batch
        for o, ev, e, gr in zip(orders, ev64, cot64, gr64):
            sg.evaluate_(g64, derivative_order=o, eval=ev)
            sg.evaluate_adjoint_(g64, derivative_order=o, eval=e, control_points=gr)
    s64 = max(3, steps // 2)
    t64 = _max_over_ranks(ws, _time_region(torch, fwd64, s64, 3, ws))
    t64fa = _max_over_ranks(ws, _time_region(torch, fwd_adj64, s64, 3, ws))
    del g64, ev64, cot64, gr64
    torch.cuda.empty_cache()
    peak, src = _peak_hbm()
    fb64, ab64 = large2d_bytes(8)
    fk = "k_f2_fwdt_grid" if paths[0] == "fused" else "forward passes"
    ak = "k_f2_adj_grid" if paths[1] == "fused" else "adjoint passes"
    return {
        "workload": "large2d_256x256_d3_4096x4096_nout3_3orders",
        "paths": {"forward": paths[0], "adjoint": paths[1]},
        "tuned_adjoint_blocks": [int(x) for x in tuned],
        "fp32_fwd_adj": {"value": V * ws * steps / t_fa, "unit": UNIT,
                         "ms_per_step": t_fa / steps * 1e3},
        "fp32_fwd_adj_separable": {"value": V * ws * steps / t_fa_sep, "unit": UNIT,
                                   "ms_per_step": t_fa_sep / steps * 1e3,
                                   "call": "the same step with the plan's strategy 'separable'"},
        "fp32_forward": {"value": V * ws * steps / t_f, "unit": UNIT},
        "fp32_adjoint": {"value": V * ws * steps / t_a, "unit": UNIT},
        "fp32_forward_multi_order": {"value": V * ws * steps / t_fm, "unit": UNIT,
                                     "call": "evaluate_multi_"},
        "bf16_cp_forward": {"value": V * ws * steps / t_bf, "unit": UNIT},
        "captured_fit_step": fit_line,
        "fp64_forward": {"value": V * ws * s64 / t64, "unit": UNIT},
        "fp64_fwd_adj": {"value": V * ws * s64 / t64fa, "unit": UNIT},
        "roofline_step": _roof(no * (fb + ab), t_fa / steps, peak,
                               "FP32 forward+adjoint of the 3 orders back to back",
                               f"{fk} + {ak}"),
        "roofline_forward_step": _roof(no * fb, t_f / steps, peak,
                                       "FP32 forward of the 3 orders back to back", fk),
        "roofline_adjoint_step": _roof(no * ab, t_a / steps, peak,
                                       "FP32 adjoint of the 3 orders back to back", ak),
        "roofline_fp64_step": _roof(no * (fb64 + ab64), t64fa / s64, peak,
                                    "FP64 forward+adjoint of the 3 orders back to back",
                                    f"{fk} + {ak} (FP64)"),
        "peak_source": src,
        "single_launch_ms": {
            "forward": fwd_ms, "adjoint": adj_ms,
            "note": "order (0,0) timed one launch at a time; part of a launch's eval writes "
                    "can still sit in the 126 MB L2 when it ends, so these are not HBM "
                    "rates"},
    }


# ------------------------------------------------------------------ our arm
def run_ours(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    import build as sg_build
    if rank == 0:
        sg_build.build()
    _barrier(ws)
    import splinegrids as sg
    sg.load_library()
    if args.workload == "large2d":
        return run_ours_large2d(sg, torch, args, ws, rank, local)

    specs, grids, cps, evals, cots, grads = build_batched(sg, torch, torch.float32)
    fwd_bytes, adj_bytes, vals = batched_bytes(specs)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    n_fused = batch.fused_grids()
    # the separable pass queue on the same arrays (the comparison line)
    batch.set_strategy("separable")
    g_sep = _capture(torch, lambda: batch.run(forward=True, adjoint=True))
    t_sep = _max_over_ranks(ws, _time_region(torch, g_sep.replay, args.steps, args.warmup, ws))
    batch.check()
    del g_sep
    batch.set_strategy("auto")
    # measured unit sizes on the plan's own arrays, kept in the plan
    tuned = batch.tune()
    g_fa = _capture(torch, lambda: batch.run(forward=True, adjoint=True))
    g_f = _capture(torch, lambda: batch.run(forward=True, adjoint=False))
    g_a = _capture(torch, lambda: batch.run(forward=False, adjoint=True))

    clocks = ClockSampler(local)
    clocks.start()
    t_fa = _time_region(torch, g_fa.replay, args.steps, args.warmup, ws)
    clk = clocks.stop()
    batch.check()
    t_fa = _max_over_ranks(ws, t_fa)
    t_f = _max_over_ranks(ws, _time_region(torch, g_f.replay, args.steps, args.warmup, ws))
    t_a = _max_over_ranks(ws, _time_region(torch, g_a.replay, args.steps, args.warmup, ws))
    batch.check()
    value = vals * ws * args.steps / t_fa
    step_s = t_fa / args.steps

    out = {}
    if rank == 0:
        import oracle
        oracle.build()
        fe, ae = batched_accuracy(oracle, grids, cps, evals, cots, grads)
        out["accuracy"] = {"forward_max_rel_err_vs_fp64_oracle": fe,
                           "adjoint_max_rel_err_vs_fp64_oracle": ae,
                           "sample": "grids 0..5, all sets, against the FP64 oracle (all 256 "
                                     "grids are checked by the full-size GPU test)"}
    e2e = measure_e2e_batched(sg, torch, batch, specs, grids, args, ws)
    loop = measure_captured_loop(sg, torch, batch, grids, cps, evals, cots, specs,
                                 max(5, args.steps // 2), ws)
    del batch, g_fa, g_f, g_a, grids, cps, evals, cots, grads
    torch.cuda.empty_cache()
    plain = measure_large2d(sg, torch, max(5, args.steps // 2), ws)
    torch.cuda.empty_cache()
    nurbs = measure_nurbs_lr(sg, torch, max(5, args.steps // 2), ws)

    if rank != 0:
        return 0
    import oracle
    cpu_v, cpu_threads, cpu_desc = cpu_sample_batched(oracle)
    peak, src = _peak_hbm()
    launch_bytes = fwd_bytes + adj_bytes
    achieved = launch_bytes / step_s / 1e9
    traffic = None
    tf, ta = _load_traffic("batched/k_f2_fwdt_batch"), _load_traffic("batched/k_f2_adj_batch")
    if tf and ta:
        traffic = tf + ta
    kernels = f"k_f2_fwdt_batch + k_f2_adj_batch ({n_fused} grids fused"
    kernels += ")" if n_fused == len(specs) else f"; k_batch for {len(specs) - n_fused} more)"
    launches = 2 + (0 if n_fused == len(specs) else 1)
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded draws of grid sizes/degrees; N(0,1) control points and "
                "cotangents)",
        "config": {"workload": "batched_256_uneven_2d_grids_x16_sets_fwd_adj",
                   "n_grids": len(specs), "sets_per_grid": BATCHED["sets"],
                   "values_per_step": vals, "eval_bytes": vals * 4,
                   "fused_grids": n_fused, "launches_per_step": launches, "cuda_graph": True,
                   "tuned_unit_values": {"forward": tuned[0], "adjoint": tuned[1]},
                   "l2": "eval and cotangent 9.7 GB each > 126 MB L2, no flush",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "forward_only": {"value": vals * ws * args.steps / t_f, "unit": UNIT,
                         "kernel": "k_f2_fwdt_batch", "ms_per_step": t_f / args.steps * 1e3,
                         "achieved_gbs": fwd_bytes / (t_f / args.steps) / 1e9,
                         "frac": fwd_bytes / (t_f / args.steps) / 1e9 / peak},
        "adjoint_only": {"value": vals * ws * args.steps / t_a, "unit": UNIT,
                         "kernel": "k_f2_adj_batch", "ms_per_step": t_a / args.steps * 1e3,
                         "achieved_gbs": adj_bytes / (t_a / args.steps) / 1e9,
                         "frac": adj_bytes / (t_a / args.steps) / 1e9 / peak},
        "separable_passes": {"value": vals * ws * args.steps / t_sep, "unit": UNIT,
                             "ms_per_step": t_sep / args.steps * 1e3,
                             "kernel": "k_batch (dependency-ordered pass queue)"},
        "captured_loop": loop,
        "plain_single_grid": plain,
        "nurbs_local_refinement_3d": nurbs,
        # batched FP32 forward+adjoint against the plain single-grid FP64 path on the same
        # kind of step (forward+adjoint); and against its FP64 forward alone
        "batched_fp32_vs_plain_fp64": value / plain["fp64_fwd_adj"]["value"],
        "batched_fp32_vs_plain_fp64_forward_only": value / plain["fp64_forward"]["value"],
        "roofline": {"bound": "hbm", "kernel": kernels,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": src, "algorithmic_bytes_per_launch": launch_bytes,
                     "per": "step (the forward launch then the adjoint launch)",
                     "launch_ms": step_s * 1e3, "traffic": traffic},
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                         "sample": cpu_desc},
        "e2e": e2e,
        "gpu_launches": args.steps * launches,
        "clocks": clk,
    }
    res.update(out)
    print(json.dumps(res))
    return 0


def run_ours_large2d(sg, torch, args, ws, rank, local):
    clocks = ClockSampler(local)
    clocks.start()
    plain = measure_large2d(sg, torch, args.steps, ws)
    clk = clocks.stop()
    if rank != 0:
        return 0
    r = plain["roofline_step"]
    v = plain["fp32_fwd_adj"]["value"]
    fused = plain["paths"]["forward"] == "fused" and plain["paths"]["adjoint"] == "fused"
    tf, ta = _load_traffic("large2d/k_f2_fwdt_grid"), _load_traffic("large2d/k_f2_adj_grid")
    traffic = 3 * (tf + ta) if (fused and tf and ta) else None
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": plain["fp32_fwd_adj"]["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": plain["workload"] + "_fwd_adj",
                   "l2": "eval/cotangent 201 MB per order > 126 MB L2"},
        "detail": plain,
        "roofline": {"bound": "hbm", "kernel": r["kernels"], "achieved": r["achieved"],
                     "peak": r["peak"], "unit": "GB/s", "frac": r["frac"],
                     "per": "step (3 orders, forward then adjoint each)",
                     "algorithmic_bytes_per_launch": r["bytes"], "traffic": traffic},
        "gpu_launches": args.steps * 6 if fused else None,
        "clocks": clk,
    }))
    return 0


# ------------------------------------------------------------------ reference arm
def run_reference(args, ws, rank):
    """The reference's CPU path for the same workload, timed on the host cores through
    the oracle (its C/OpenMP restatement): every step is the whole batched
    configuration (256 grids x 16 sets, forward then adjoint of each grid)."""
    if rank != 0:
        return 0
    import oracle as O
    O.build()
    work, vals = reference_workload(O)
    for _ in range(args.warmup):
        reference_step(O, work)
    per = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        reference_step(O, work)
        per.append(time.perf_counter() - t0)
    dt = sum(per)
    v = vals * args.steps / dt
    sample = (f"Float32 forward+adjoint of all {BATCHED['n_grids']} grids x {BATCHED['sets']} "
              f"sets of the batched configuration per step ({vals} values)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "step_ms": {"min": min(per) * 1e3, "median": statistics.median(per) * 1e3,
                    "max": max(per) * 1e3},
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "batched_256_uneven_2d_grids_x16_sets_fwd_adj",
                   "n_grids": BATCHED["n_grids"], "sets_per_grid": BATCHED["sets"],
                   "values_per_step": vals, "same_config": True,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Julia (SplineGrids.jl, KernelAbstractions); julia is not "
                "installed, so its CPU() path is timed through the oracle's C/OpenMP "
                "restatement of its kernels",
    }))
    return 0


# ------------------------------------------------------------------ profiling run
def run_profile(args, local):
    """A small run for ncu: the first 32 grids of the batched configuration at the unit
    sizes the full configuration tunes to (forward tiles of 64K values, adjoint tiles
    over axis 1 whole): two forward-only, two adjoint-only and one forward+adjoint run
    (k_f2_fwdt_batch, k_f2_adj_batch), plus two forward+adjoint of the Large-2D grid's
    order (0,0) through the per-grid kernels (~3 GB on the device)."""
    import torch
    torch.cuda.set_device(local)
    import build as sg_build
    sg_build.build()
    import splinegrids as sg
    specs, grids, cps, evals, cots, grads = build_batched(sg, torch, torch.float32, n_grids=32)
    batch = sg.GridBatch(grids)
    batch.set_arrays(cps, evals, cots, grads)
    batch.set_unit_sizes(1 << 16, 0)
    for _ in range(2):  # launches 1-2: forward only
        batch.run(forward=True, adjoint=False)
    for _ in range(2):  # launches 3-4: adjoint only
        batch.run(forward=False, adjoint=True)
    batch.run(forward=True, adjoint=True)  # launch 5: both
    batch.check()
    g, cp, ev, cot, gr = build_large2d(sg, torch, torch.float32, n_orders=1)
    for _ in range(2):
        sg.evaluate_(g, derivative_order=(0, 0), eval=ev[0])
        sg.evaluate_adjoint_(g, derivative_order=(0, 0), eval=cot[0], control_points=gr[0])
    torch.cuda.synchronize()
    print("profile run done")
    return 0


def run_align(args, local):
    """A small run for ncu: the fused forward of one (ns0, 4096) x 3 grid, degree 3,
    (256, 256) control points, launched four times (k_f2_fwdt_grid), for comparing row
    starts on and off 128-byte lines (ns0 = 4096 against 4100, 4104, 4097)."""
    import torch
    torch.cuda.set_device(local)
    import build as sg_build
    sg_build.build()
    import splinegrids as sg
    ns0 = args.ns0
    dims = tuple(sg.SplineDimension(256, 3, m, float_type=torch.float32) for m in (ns0, 4096))
    ev = sg.arrays.empty((ns0, 4096, 3), torch.float32)
    cp = sg.arrays.empty((256, 256, 3), torch.float32)
    cp.normal_()
    g = sg.SplineGrid(dims, control_points=cp, eval=ev)
    for _ in range(4):
        sg.evaluate_(g, eval=ev)
    torch.cuda.synchronize()
    print("align run done", ns0, g.plan(torch.float32).paths())
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="batched", choices=["batched", "large2d"])
    ap.add_argument("--mode", default="bench", choices=["bench", "profile", "align"])
    ap.add_argument("--ns0", type=int, default=4096, help="axis-0 samples of the --mode align grid")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = _dist()
    if args.mode == "profile":
        return run_profile(args, local)
    if args.mode == "align":
        return run_align(args, local)
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
