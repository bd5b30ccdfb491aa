"""KnotVector and SplineDimension (src/knot_vector.jl, src/spline_dimension.jl).

Construction-time host logic (knot values, sample points) follows the reference; the
device work (knot expansion, knot-span search, Cox-de Boor tables) runs through the
library.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, arrays


def julia_range(a: float, b: float, n: int) -> np.ndarray:
    """Float64 elements of Julia's ``range(a, b; length=n)``.

    Julia evaluates ``StepRangeLen`` elements in twice precision, i.e. correctly
    rounded; for the endpoints used by the reference (integers and (0, 1)) that is the
    correctly rounded ``(a*(n-1-l) + b*l) / (n-1)`` computed here, whose numerator is
    exact.  Sample points landing exactly on knots (``l/(n-1) == k/m``) therefore
    coincide bit for bit, as in the reference (src/spline_dimension.jl:121-128,
    src/knot_vector.jl:95-100)."""
    if n == 1:
        return np.array([float(a)])
    ls = np.arange(n, dtype=np.float64)
    if a == 0.0:
        return (b * ls) / float(n - 1)
    return (a * (n - 1 - ls) + b * ls) / float(n - 1)


def _stream():
    return _lib.stream_handle()


class KnotVector:
    """A knot vector (src/knot_vector.jl:11-50).

    ``KnotVector(knot_values, multiplicities)`` expands the strictly increasing
    ``knot_values`` by their multiplicities into ``knots_all`` on the device.
    """

    def __init__(self, knot_values, multiplicities, *, device="cuda"):
        kv_host = torch.as_tensor(knot_values).detach().cpu()
        m_host = torch.as_tensor(multiplicities).detach().cpu()
        assert kv_host.numel() == m_host.numel(), \
            "knot_values and multiplicities must be of the same length."
        assert bool(torch.all(kv_host[1:] >= kv_host[:-1])), "knot_values must be sorted."
        assert bool(torch.all(kv_host[1:] != kv_host[:-1])), "knot_values must be unique."
        if not kv_host.is_floating_point():
            kv_host = kv_host.to(torch.float64)
        dev = torch.device(knot_values.device if isinstance(knot_values, torch.Tensor)
                           and knot_values.is_cuda else device)
        self.knot_values = kv_host.to(dev)
        self.multiplicities = m_host.to(torch.int32).to(dev)
        n_knots = int(m_host.sum())
        self.knots_all = torch.empty(n_knots, dtype=self.knot_values.dtype, device=dev)
        self.extent = (float(kv_host[0]), float(kv_host[-1]))
        _lib.check(_lib.load().sg_expand_knots(
            arrays.dtype_code(self.knot_values.dtype), self.knot_values.data_ptr(),
            self.multiplicities.data_ptr(), kv_host.numel(), n_knots,
            self.knots_all.data_ptr(), _stream()))

    @classmethod
    def default(cls, n_basis_functions: int, degree: int, *, extent=(0, 1),
                distribution: str = "equispaced", device="cuda",
                float_type=torch.float32, int_type=torch.int32, generator=None):
        """Clamped knot vector (src/knot_vector.jl:75-113): multiplicity degree+1 at
        both ends, 1 inside; interior knots equispaced or random."""
        assert n_basis_functions - degree >= 1
        nv = n_basis_functions - degree + 1
        if distribution == "random":
            g = generator if generator is not None else torch.Generator().manual_seed(0)
            kv = torch.cumsum(torch.rand(nv, generator=g, dtype=torch.float64), 0)
            kv = kv - kv[0]
            kv = kv / (kv[-1] - kv[0])
            kv = kv * (extent[1] - extent[0]) + extent[0]
            kv = kv.numpy()
        elif distribution == "equispaced":
            kv = julia_range(float(extent[0]), float(extent[1]), nv)
        else:
            raise ValueError(f"Unsupported knot distribution type {distribution}.")
        mult = np.ones(nv, dtype=np.int32)
        mult[0] = degree + 1
        mult[-1] = degree + 1
        return cls(torch.as_tensor(kv).to(float_type), torch.as_tensor(mult), device=device)

    @property
    def dtype(self):
        return self.knot_values.dtype


class SplineDimension:
    """One spline dimension: knots, samples, knot-span indices and the basis table
    ``eval[n_samples, degree+1, max_derivative_order+1]`` (src/spline_dimension.jl:25-156).

    ``SplineDimension(n_basis_functions, degree, n_sample_points; ...)`` as in the
    reference; ``knot_vector=`` supplies a custom knot vector, other keyword arguments
    go to ``KnotVector.default``.  ``sample_points=`` (an extension) supplies custom
    sample points, as the reference's inner constructor allows.
    """

    def __init__(self, n_basis_functions: int, degree: int, n_sample_points: int, *,
                 max_derivative_order: int = 0, knot_vector: KnotVector | None = None,
                 device="cuda", float_type=torch.float32, int_type=torch.int32,
                 sample_points=None, **kwargs):
        assert 0 <= max_derivative_order <= degree, (
            "The max_degree must be positive and derivatives order higher than `degree` "
            "are all 0.")
        if int_type not in (torch.int32,):
            raise TypeError("sample indices are Int32 (the reference default int_type)")
        if knot_vector is None:
            knot_vector = KnotVector.default(n_basis_functions, degree, device=device,
                                             float_type=float_type, **kwargs)
        else:
            assert knot_vector.knots_all.numel() == n_basis_functions + degree + 1, \
                "Incompatible knot vector supplied."
            float_type = knot_vector.dtype
        dev = knot_vector.knots_all.device
        self.degree = int(degree)
        self.max_derivative_order = int(max_derivative_order)
        self.knot_vector = knot_vector
        if sample_points is None:
            pts = julia_range(knot_vector.extent[0], knot_vector.extent[1], n_sample_points)
            self.sample_points = torch.as_tensor(pts).to(float_type).to(dev)
        else:
            self.sample_points = torch.as_tensor(sample_points).to(float_type).to(dev)
            n_sample_points = self.sample_points.numel()
        self.sample_indices = torch.zeros(n_sample_points, dtype=torch.int32, device=dev)
        self.eval = arrays.zeros((n_sample_points, degree + 1, max_derivative_order + 1),
                                 float_type, dev)
        set_sample_indices_(self)
        evaluate_dimension_(self)

    @property
    def dtype(self):
        return self.eval.dtype

    @property
    def n_basis_functions(self) -> int:
        return self.knot_vector.knots_all.numel() - self.degree - 1

    def __len__(self):
        return self.sample_points.numel()


def set_sample_indices_(dim: SplineDimension) -> None:
    """set_sample_indices! (src/utils.jl:19-29)."""
    kn = dim.knot_vector.knots_all
    _lib.check(_lib.load().sg_sample_indices(
        arrays.dtype_code(dim.sample_points.dtype), dim.sample_points.data_ptr(),
        dim.sample_points.numel(), kn.data_ptr(), kn.numel(), dim.degree,
        dim.sample_indices.data_ptr(), _stream()))


def evaluate_dimension_(dim: SplineDimension) -> None:
    """evaluate!(::SplineDimension) (src/spline_dimension.jl:231-243)."""
    kn = dim.knot_vector.knots_all
    _lib.check(_lib.load().sg_basis_eval(
        arrays.dtype_code(dim.eval.dtype), kn.data_ptr(), kn.numel(),
        dim.sample_points.data_ptr(), dim.sample_indices.data_ptr(), dim.sample_points.numel(),
        dim.degree, dim.max_derivative_order, arrays.ptr(dim.eval, "eval"), _stream()))


def decompress(dim: SplineDimension, derivative_order: int = 0) -> torch.Tensor:
    """decompress (src/spline_dimension.jl:251-272): dense [n_samples, n_basis] matrix."""
    assert derivative_order <= dim.max_derivative_order
    out = arrays.empty((dim.sample_points.numel(), dim.n_basis_functions), dim.dtype,
                       dim.eval.device)
    _lib.check(_lib.load().sg_decompress(
        arrays.dtype_code(dim.dtype), arrays.ptr(dim.eval), dim.sample_indices.data_ptr(),
        dim.sample_points.numel(), dim.degree, dim.max_derivative_order, derivative_order,
        dim.n_basis_functions,
        arrays.ptr(out), _stream()))
    return out
