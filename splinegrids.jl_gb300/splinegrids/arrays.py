"""Julia-layout (column-major) torch tensors.

The library takes the reference's memory layout: first index fastest.  A tensor
created here has the Julia shape and Julia (column-major) strides, so `eval[j1, j2, o]`
indexes the same element as the reference's `eval[j1+1, j2+1, o+1]` and
`data_ptr()` is the start of a dense column-major block.
"""
from __future__ import annotations

import math

import torch

from . import _lib

_DTYPE_CODE = {torch.float64: _lib.SG_F64, torch.float32: _lib.SG_F32}


def dtype_code(dtype: torch.dtype) -> int:
    if dtype not in _DTYPE_CODE:
        raise TypeError(f"float_type must be torch.float32 or torch.float64, got {dtype}")
    return _DTYPE_CODE[dtype]


def colmajor_strides(shape) -> tuple:
    st, acc = [], 1
    for s in shape:
        st.append(acc)
        acc *= max(int(s), 1)
    return tuple(st)


def empty(shape, dtype=torch.float32, device="cuda") -> torch.Tensor:
    shape = tuple(int(s) for s in shape)
    base = torch.empty(tuple(reversed(shape)), dtype=dtype, device=device)
    return base.permute(*reversed(range(len(shape)))) if shape else base


def zeros(shape, dtype=torch.float32, device="cuda") -> torch.Tensor:
    t = empty(shape, dtype, device)
    t.zero_()
    return t


def ones(shape, dtype=torch.float32, device="cuda") -> torch.Tensor:
    t = empty(shape, dtype, device)
    t.fill_(1)
    return t


def from_any(x, dtype=None, device="cuda") -> torch.Tensor:
    """Copy an array-like with Julia indexing semantics into a column-major tensor."""
    t = torch.as_tensor(x)
    out = empty(tuple(t.shape), dtype or t.dtype, device)
    out.copy_(t)
    return out


def is_colmajor(t: torch.Tensor) -> bool:
    if t.numel() <= 1:
        return True
    exp = colmajor_strides(t.shape)
    return all(st == e for st, e, n in zip(t.stride(), exp, t.shape) if n > 1)


def ptr(t: torch.Tensor | None, what: str = "array") -> int | None:
    """Device pointer of a column-major CUDA tensor (the library's calling convention)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor (this package has no CPU path)")
    if not is_colmajor(t):
        raise ValueError(f"{what} must be column-major (Julia layout); use splinegrids.arrays")
    return t.data_ptr()


def vec(t: torch.Tensor) -> torch.Tensor:
    """Julia `vec`: the column-major flattening, as a view when possible."""
    if is_colmajor(t):
        return t.permute(*reversed(range(t.dim()))).reshape(-1) if t.dim() > 1 else t.reshape(-1)
    return t.permute(*reversed(range(t.dim()))).reshape(-1)


def reshape(flat: torch.Tensor, shape) -> torch.Tensor:
    """Julia `reshape` of a column-major flat vector into `shape` (a view)."""
    shape = tuple(int(s) for s in shape)
    assert flat.numel() == math.prod(shape)
    return flat.reshape(tuple(reversed(shape))).permute(*reversed(range(len(shape))))
