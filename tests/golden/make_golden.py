"""Extract the reference's known-answer values from its test files into a JSON fixture.

The reference (SplineGrids.jl) is Julia and cannot run here, so its golden vectors
are read from its test sources as text and committed as ``reference_kats.json``.
Run from the repository root with the reference checked out at ``REF`` (default
``/root/reference``):

    python tests/golden/make_golden.py [REF]

Nothing at test time reads the reference; tests load the committed JSON.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np


def _parse_julia_array(text: str) -> np.ndarray:
    """Parse a Julia array literal ``[a b; c d;;; e f; g h]`` (rows ``;``, columns by
    whitespace, 3rd dimension ``;;;``) into a numpy array of the Julia shape."""
    body = text.strip()
    assert body[0] == "[" and body[-1] == "]"
    body = body[1:-1]
    slices = [s for s in body.split(";;;")]
    mats = []
    for s in slices:
        rows = [r.strip() for r in s.split(";") if r.strip()]
        mats.append(np.array([[float(x) for x in r.split()] for r in rows]))
    if len(mats) == 1:
        return mats[0]
    return np.stack(mats, axis=2)


def _between(src: str, start_pat: str, end_pat: str) -> str:
    i = src.index(start_pat)
    j = src.index(end_pat, i + len(start_pat))
    return src[i + len(start_pat): j]


def main(ref: str) -> None:
    out = {}

    # test/test_spline_grid.jl:29-53 -- forward golden vector, Nin=2, Nout=2
    sg = open(os.path.join(ref, "test", "test_spline_grid.jl")).read()
    block = sg[sg.index('@testset "Nin = 2, Nout = 2"'):]
    cp_txt = _between(block, "spline_grid.control_points,\n", "\n    )\n    evaluate!")
    ev_txt = _between(block, "adapt(backend,\n", "\n    )\nend")
    cp = _parse_julia_array(cp_txt)
    ev = _parse_julia_array(ev_txt)
    assert cp.shape == (5, 6, 2) and ev.shape == (7, 9, 2), (cp.shape, ev.shape)
    out["spline_grid_nin2_nout2"] = dict(
        source="test/test_spline_grid.jl:29-53",
        n_control_points=[5, 6], degree=[3, 2], n_sample_points=[7, 9], nout=2,
        float_type="Float32",
        control_points=cp.flatten(order="F").tolist(),
        eval=ev.flatten(order="F").tolist())

    # test/test_knot_vector.jl:26-36 -- default clamped knot vector
    out["knot_vector_5_2"] = dict(
        source="test/test_knot_vector.jl:26-36",
        n_basis=5, degree=2, multiplicities=[3, 1, 1, 3],
        knots_all=[0.0, 0.0, 0.0, 1 / 3, 2 / 3, 1.0, 1.0, 1.0],
        extent2=[5.0, 7.0])

    # test/test_nurbs_grid.jl:25-52 -- NURBS circle
    nb = open(os.path.join(ref, "test", "test_nurbs_grid.jl")).read()
    mult = [int(x) for x in re.search(r"Int32\[([0-9, ]+)\]", nb).group(1).split(",")]
    cps_txt = _between(nb, "copyto!(nurbs_grid.control_points, ", ")\n    evaluate!")
    rows = [r.strip() for r in cps_txt.strip()[1:-1].split(";") if r.strip()]
    circle_cp = [[float(x) for x in r.split()] for r in rows]
    out["nurbs_circle"] = dict(
        source="test/test_nurbs_grid.jl:25-52",
        knot_values=["0", "pi/2", "pi", "3pi/2", "2pi"], multiplicities=mult,
        n_control_points=9, degree=2, n_sample_points=500, nout=2,
        weight_even_index=1 / np.sqrt(2.0), control_points=circle_cp)

    # test/test_local_refinement.jl:48-67 -- error-informed refinement indices
    lr = open(os.path.join(ref, "test", "test_local_refinement.jl")).read()
    idx_txt = re.search(r"Int32\[(.*?)\]", lr, re.S).group(1)
    pairs = [[int(v) for v in p.split()] for p in idx_txt.replace("\n", " ").split(";")
             if p.strip()]
    rng = re.search(r"error\[(\d+):(\d+), (\d+):(\d+), (\d+)\] \.= 1", lr)
    out["error_informed_refinement"] = dict(
        source="test/test_local_refinement.jl:48-67",
        n_control_points=[6, 6], degree=[2, 2], n_sample_points=[50, 50], nout=3,
        error_box_1based=[int(x) for x in rng.groups()],
        refinement_indices_1based=pairs)

    # test/test_local_refinement.jl:11-46 -- local refinement keeps geometry
    out["local_refinement_ranges"] = dict(
        source="test/test_local_refinement.jl:11-46",
        n_control_points=[6, 6], degree=[2, 2], n_sample_points=[500, 500], nout=3,
        ranges_1based=[[[1, 4], [1, 6]], [[1, 6], [1, 2]], [[9, 10], [7, 10]]],
        n_control_points_after=63, finest_grid=[10, 10])

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
