"""ctypes wrapper around the CPU oracle (``sg_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's KernelAbstractions
kernels on the CPU (see the citations in ``sg_oracle.c``).  It is loaded by
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (CPU baseline and reference
arm) as the checker; the product package never imports it.

Array convention: Julia column-major arrays are numpy arrays with ``order='F'`` and
the Julia shape, e.g. ``eval`` of a 2D grid is ``(ns1, ns2, Nout)``.  Sample
indices are 1-based ``int32`` as in the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libsg_oracle.so")
_lib = None

_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_vp = C.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle shared library with ``make`` (gcc, OpenMP)."""
    src = os.path.join(_HERE, "sg_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "libsg_oracle.so"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
    return _lib


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float64:
        return "f64"
    if dt == np.float32:
        return "f32"
    raise TypeError(f"oracle supports float32/float64, got {dt}")


def _p(a: np.ndarray):
    assert a.flags["F_CONTIGUOUS"] or a.ndim <= 1, "oracle arrays must be column-major"
    return a.ctypes.data_as(_vp)


def _i64(vals):
    return (C.c_int64 * len(vals))(*[int(v) for v in vals])


def _i32(vals):
    return (C.c_int32 * len(vals))(*[int(v) for v in vals])


def num_threads() -> int:
    return int(lib().or_num_threads())


def set_num_threads(n: int) -> None:
    lib().or_set_num_threads(C.c_int(int(n)))


# ---------------------------------------------------------------- per dimension
def expand_knots(knot_values: np.ndarray, multiplicities) -> np.ndarray:
    """expand_knot_vector_kernel (src/util_kernels.jl:1-20)."""
    kv = np.ascontiguousarray(knot_values)
    m = np.ascontiguousarray(multiplicities, dtype=np.int32)
    out = np.zeros(int(m.sum()), dtype=kv.dtype)
    getattr(lib(), "or_expand_knots_" + _sfx(kv.dtype))(_p(kv), _p(m), C.c_int64(len(kv)), _p(out))
    return out


def sample_indices(samples: np.ndarray, knots_all: np.ndarray, degree: int) -> np.ndarray:
    """set_sample_indices_kernel (src/util_kernels.jl:22-49); 1-based int32."""
    s = np.ascontiguousarray(samples)
    k = np.ascontiguousarray(knots_all, dtype=s.dtype)
    out = np.zeros(len(s), dtype=np.int32)
    getattr(lib(), "or_sample_indices_" + _sfx(s.dtype))(
        _p(s), C.c_int64(len(s)), _p(k), C.c_int64(len(k)), C.c_int(degree), _p(out))
    return out


def basis(knots_all, samples, sidx, degree: int, max_deriv: int) -> np.ndarray:
    """spline_dimension_kernel (src/spline_dimension.jl:160-215) -> [ns, d+1, maxd+1]."""
    s = np.ascontiguousarray(samples)
    k = np.ascontiguousarray(knots_all, dtype=s.dtype)
    i = np.ascontiguousarray(sidx, dtype=np.int32)
    out = np.zeros((len(s), degree + 1, max_deriv + 1), dtype=s.dtype, order="F")
    getattr(lib(), "or_basis_" + _sfx(s.dtype))(
        _p(k), _p(s), _p(i), C.c_int64(len(s)), C.c_int(degree), C.c_int(max_deriv), _p(out))
    return out


def decompress(eval_: np.ndarray, sidx, degree: int, order: int, n_basis: int) -> np.ndarray:
    """decompress (src/spline_dimension.jl:251-272), FP64."""
    e = np.asfortranarray(eval_, dtype=np.float64)
    i = np.ascontiguousarray(sidx, dtype=np.int32)
    out = np.zeros((len(i), n_basis), dtype=np.float64, order="F")
    lib().or_decompress_f64(_p(e), _p(i), C.c_int64(len(i)), C.c_int(degree), C.c_int(order),
                            C.c_int64(n_basis), _p(out))
    return out


# ---------------------------------------------------------------- grid
class GridSpec:
    """The per-dimension arrays a grid evaluation reads (one entry per input dim)."""

    def __init__(self, sidx, basis_tables, degrees, n_basis):
        self.sidx = [np.ascontiguousarray(s, dtype=np.int32) for s in sidx]
        self.basis = [np.asfortranarray(b) for b in basis_tables]
        self.degrees = [int(d) for d in degrees]
        self.n_basis = [int(n) for n in n_basis]
        self.ns = [len(s) for s in self.sidx]
        self.nin = len(self.sidx)

    def _ptrs(self, dtype):
        bs = [np.asfortranarray(b, dtype=dtype) for b in self.basis]
        self._keep = bs
        sp = (_vp * self.nin)(*[s.ctypes.data for s in self.sidx])
        bp = (_vp * self.nin)(*[b.ctypes.data for b in bs])
        return sp, bp


def _out(out, shape, dtype):
    if out is None:
        return np.zeros(shape, dtype=dtype, order="F")
    assert out.shape == shape and out.dtype == dtype and out.flags["F_CONTIGUOUS"], "bad out"
    return out


def evaluate(spec: GridSpec, control_points: np.ndarray, weights=None, order=None,
             dtype=None, out=None) -> np.ndarray:
    """spline_eval_kernel (src/spline_grid.jl:119-183); eval [ns..., Nout].  `out`: an
    eval array to overwrite (the reference's evaluate! writes in place)."""
    dtype = np.dtype(dtype or control_points.dtype)
    cp = np.asfortranarray(control_points, dtype=dtype)
    nout = cp.shape[-1]
    order = order or [0] * spec.nin
    w = None if weights is None else np.asfortranarray(weights, dtype=dtype)
    out = _out(out, tuple(spec.ns) + (nout,), dtype)
    sp, bp = spec._ptrs(dtype)
    getattr(lib(), "or_eval_" + _sfx(dtype))(
        C.c_int(spec.nin), C.c_int(nout), _i64(spec.ns), _i64(spec.n_basis), _i32(spec.degrees),
        _i32([b.shape[2] - 1 for b in spec.basis]), sp, bp, _i32(order), _p(cp),
        None if w is None else _p(w), _p(out))
    return out


def evaluate_adjoint(spec: GridSpec, eval_bar: np.ndarray, order=None, dtype=None,
                     out=None) -> np.ndarray:
    """spline_eval_adjoint_kernel + evaluate_adjoint! (src/adjoint.jl:1-83).  `out`: a
    control-point array to overwrite."""
    dtype = np.dtype(dtype or eval_bar.dtype)
    e = np.asfortranarray(eval_bar, dtype=dtype)
    nout = e.shape[-1]
    order = order or [0] * spec.nin
    out = _out(out, tuple(spec.n_basis) + (nout,), dtype)
    sp, bp = spec._ptrs(dtype)
    getattr(lib(), "or_eval_adjoint_" + _sfx(dtype))(
        C.c_int(spec.nin), C.c_int(nout), _i64(spec.ns), _i64(spec.n_basis), _i32(spec.degrees),
        sp, bp, _i32(order), _p(e), _p(out))
    return out


# ---------------------------------------------------------------- refinement
def _refmat_args(mats, dims_refinement, ndims):
    r_of_d = [-1] * ndims
    for r, d in enumerate(dims_refinement):
        r_of_d[d] = r
    rps = [np.ascontiguousarray(m.row_pointer, dtype=np.int32) for m in mats]
    css = [np.ascontiguousarray(m.column_start, dtype=np.int32) for m in mats]
    return r_of_d, rps, css


def mult(Y_shape, mats, B: np.ndarray, dims_refinement, dtype=None) -> np.ndarray:
    """refinement_matrix_array_mul_kernel / mult! (src/refinement_matrix.jl:365-445).

    ``mats`` are objects with ``row_pointer``, ``column_start``, ``nzval`` (1-based
    banded format), ``m`` and ``n``; ``dims_refinement`` are 0-based dims of ``B``."""
    dtype = np.dtype(dtype or B.dtype)
    B = np.asfortranarray(B, dtype=dtype)
    nd = B.ndim
    r_of_d, rps, css = _refmat_args(mats, dims_refinement, nd)
    nzs = [np.ascontiguousarray(m.nzval, dtype=dtype) for m in mats]
    Y = np.zeros(tuple(Y_shape), dtype=dtype, order="F")
    nm = max(len(mats), 1)
    getattr(lib(), "or_mult_" + _sfx(dtype))(
        C.c_int(nd), _i64(Y.shape), _i64(B.shape), _i32(r_of_d),
        (_vp * nm)(*[a.ctypes.data for a in rps]), (_vp * nm)(*[a.ctypes.data for a in css]),
        (_vp * nm)(*[a.ctypes.data for a in nzs]), _i64([m.m for m in mats] or [0]),
        _i64([len(a) for a in nzs] or [0]), _p(B), _p(Y))
    return Y


def mult_adjoint(B_shape, mats, Y: np.ndarray, dims_refinement, dtype=None) -> np.ndarray:
    """refinement_matrix_array_mul_adjoint_kernel / mult_adjoint! (src/adjoint.jl:85-152)."""
    dtype = np.dtype(dtype or Y.dtype)
    Y = np.asfortranarray(Y, dtype=dtype)
    nd = Y.ndim
    r_of_d, rps, css = _refmat_args(mats, dims_refinement, nd)
    nzs = [np.ascontiguousarray(m.nzval, dtype=dtype) for m in mats]
    B = np.zeros(tuple(B_shape), dtype=dtype, order="F")
    nm = max(len(mats), 1)
    getattr(lib(), "or_mult_adjoint_" + _sfx(dtype))(
        C.c_int(nd), _i64(Y.shape), _i64(B.shape), _i32(r_of_d),
        (_vp * nm)(*[a.ctypes.data for a in rps]), (_vp * nm)(*[a.ctypes.data for a in css]),
        (_vp * nm)(*[a.ctypes.data for a in nzs]), _i64([m.m for m in mats] or [0]),
        _i64([len(a) for a in nzs] or [0]), _p(Y), _p(B))
    return B


def local_refinement(cp: np.ndarray, ridx: np.ndarray, vals: np.ndarray) -> None:
    """local_refinement_kernel (src/control_points.jl:296-311), in place on ``cp``."""
    nin = cp.ndim - 1
    r = np.asfortranarray(ridx, dtype=np.int32)
    v = np.asfortranarray(vals, dtype=cp.dtype)
    if r.shape[0] == 0:
        return
    getattr(lib(), "or_local_refinement_" + _sfx(cp.dtype))(
        C.c_int(nin), C.c_int(cp.shape[-1]), _i64(cp.shape[:-1]), C.c_int64(r.shape[0]),
        _p(r), _p(v), _p(cp))


def local_refinement_adjoint(cp: np.ndarray, ridx: np.ndarray) -> np.ndarray:
    """local_refinement_adjoint_kernel (src/adjoint.jl:154-170): returns the gathered
    values and zeroes them in ``cp`` (in place)."""
    nin = cp.ndim - 1
    r = np.asfortranarray(ridx, dtype=np.int32)
    vals = np.zeros((r.shape[0], cp.shape[-1]), dtype=cp.dtype, order="F")
    if r.shape[0] == 0:
        return vals
    getattr(lib(), "or_local_refinement_adjoint_" + _sfx(cp.dtype))(
        C.c_int(nin), C.c_int(cp.shape[-1]), _i64(cp.shape[:-1]), C.c_int64(r.shape[0]),
        _p(r), _p(vals), _p(cp))
    return vals


def validate_refinement_matrix(row_pointer, column_start, nnz: int, n_columns: int) -> np.ndarray:
    """validate_refinement_matrix_kernel (src/refinement_matrix.jl:127-181)."""
    rp = np.ascontiguousarray(row_pointer, dtype=np.int32)
    cs = np.ascontiguousarray(column_start, dtype=np.int32)
    out = np.zeros(len(rp), dtype=np.uint8)
    lib().or_validate_refinement_matrix(_p(rp), _p(cs), C.c_int64(len(rp)), C.c_int64(nnz),
                                        C.c_int64(n_columns), _p(out))
    return out.astype(bool)


# ---------------------------------------------------------------- set-up helpers
def julia_range(a: float, b: float, n: int) -> np.ndarray:
    """``collect(range(a, b; length=n))`` in Float64, as the reference builds its sample
    points and equispaced knots (src/spline_dimension.jl:121-128,
    src/knot_vector.jl:95-100): Julia's ``LinRange``-free ``StepRangeLen`` rounds each
    element correctly, which for the unit interval is ``l / (n-1)``."""
    if n == 1:
        return np.array([a], dtype=np.float64)
    if a == 0.0 and b == 1.0:
        return np.arange(n, dtype=np.float64) / float(n - 1)
    ls = np.arange(n, dtype=np.float64)
    return (a * (n - 1 - ls) + b * ls) / float(n - 1)


def default_dimension(n_basis: int, degree: int, n_samples: int, max_deriv: int = 0,
                      dtype=np.float64, extent=(0.0, 1.0)):
    """Oracle-side SplineDimension with the default clamped equispaced knot vector
    (src/knot_vector.jl:75-113, src/spline_dimension.jl:97-156)."""
    nv = n_basis - degree + 1
    kv = julia_range(extent[0], extent[1], nv).astype(dtype)
    mult = np.ones(nv, dtype=np.int32)
    mult[0] = degree + 1
    mult[-1] = degree + 1
    knots = expand_knots(kv, mult)
    samples = julia_range(float(kv[0]), float(kv[-1]), n_samples).astype(dtype)
    sidx = sample_indices(samples, knots, degree)
    b = basis(knots, samples, sidx, degree, max_deriv)
    return dict(knot_values=kv, multiplicities=mult, knots_all=knots, samples=samples,
                sidx=sidx, basis=b, degree=degree, n_basis=n_basis, max_deriv=max_deriv)


# ---------------------------------------------------------------- least squares
def lsqr(matvec, rmatvec, b: np.ndarray, n: int, damp: float = 0.0, atol=None, btol=None,
         conlim=None, maxiter=None, eps=None):
    """LSQR of Paige & Saunders (ACM TOMS 8(1), 1982), restated in numpy: the solver the
    reference hands ``LinearMap(spline_grid)`` to (IterativeSolvers.jl ``lsqr``,
    Project.toml compat 0.9, not part of the reference tree; used in
    test/test_LinearMapsExt.jl:14-61).  Defaults as that solver: atol = btol = sqrt(eps),
    conlim = 1/sqrt(eps), maxiter = max(m, n), x0 = 0.

    ``matvec(x) -> A x`` and ``rmatvec(y) -> A' y`` act on 1-D float64 arrays.  Returns
    ``(x, istop, itn, dict(anorm, acond, rnorm, arnorm, xnorm))`` with the paper's istop
    codes (0 x = 0 exact, 1 / 2 converged, 3 cond > conlim, 4-6 machine precision, 7
    maxiter).  ``eps`` is the machine epsilon of the tests "1 + t <= 1" (float64 by
    default; the device solver uses its vector type's)."""
    b = np.asarray(b, dtype=np.float64).ravel()
    m = b.size
    eps_t = np.finfo(np.float64).eps if eps is None else eps
    one_plus = (lambda t: 1.0 + t <= 1.0) if eps is None else \
        (lambda t: np.float32(1.0) + np.float32(t) <= np.float32(1.0))
    atol = np.sqrt(eps_t) if atol is None else atol
    btol = np.sqrt(eps_t) if btol is None else btol
    conlim = 1.0 / np.sqrt(eps_t) if conlim is None else conlim
    maxiter = max(m, n) if maxiter is None else maxiter
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    feps = np.finfo(np.float64).eps if eps is None else eps

    x = np.zeros(n)
    u = b.copy()
    beta = np.linalg.norm(u)
    bnorm = beta
    if beta > 0:
        u = u / beta
    v = rmatvec(u) if beta > 0 else np.zeros(n)
    alpha = np.linalg.norm(v)
    if alpha > 0:
        v = v / alpha
    w = v.copy()
    rhobar, phibar = alpha, beta
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = sn2 = 0.0
    cs2 = -1.0
    rnorm, arnorm = beta, alpha * beta
    dampsq = damp * damp
    info = lambda: dict(anorm=anorm, acond=acond, rnorm=rnorm, arnorm=arnorm, xnorm=xnorm)
    if arnorm == 0:
        return x, 0, 0, info()
    itn, istop = 0, 0
    while True:
        itn += 1
        u = matvec(v) - alpha * u
        beta = np.linalg.norm(u)
        if beta > 0:
            u = u / beta
            anorm = np.sqrt(anorm ** 2 + alpha ** 2 + beta ** 2 + dampsq)
            v = rmatvec(u) - beta * v
            alpha = np.linalg.norm(v)
            if alpha > 0:
                v = v / alpha
        rhobar1 = np.sqrt(rhobar ** 2 + dampsq)
        cs1, sn1 = rhobar / rhobar1, damp / rhobar1
        psi = sn1 * phibar
        phibar = cs1 * phibar
        rho = np.sqrt(rhobar1 ** 2 + beta ** 2)
        cs, sn = rhobar1 / rho, beta / rho
        theta = sn * alpha
        rhobar = -cs * alpha
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        t1, t2 = phi / rho, -theta / rho
        ddnorm += np.dot(w, w) / rho ** 2
        x = x + t1 * w
        w = v + t2 * w
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = np.sqrt(xxnorm + zbar ** 2)
        gamma = np.sqrt(gambar ** 2 + theta ** 2)
        cs2, sn2 = gambar / gamma, theta / gamma
        z = rhs / gamma
        xxnorm += z * z
        acond = anorm * np.sqrt(ddnorm)
        res2 += psi * psi
        rnorm = np.sqrt(phibar ** 2 + res2)
        arnorm = alpha * abs(tau)
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm + feps)
        test3 = 1.0 / (acond + feps)
        t1s = test1 / (1.0 + anorm * xnorm / bnorm)
        rtol = btol + atol * anorm * xnorm / bnorm
        if itn >= maxiter:
            istop = 7
        if one_plus(test3):
            istop = 6
        if one_plus(test2):
            istop = 5
        if one_plus(t1s):
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        if istop != 0:
            return x, istop, itn, info()
