"""Device plumbing: tensors, dtypes and streams handed to the C ABI."""

from __future__ import annotations

import torch

from . import _lib


def default_device() -> torch.device:
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def require_cuda(*tensors: torch.Tensor) -> None:
    """Compute calls run on the GPU only: fail loudly for host tensors."""
    for t in tensors:
        if t is not None and not t.is_cuda:
            raise RuntimeError(
                "tatva_gb300 compute kernels need CUDA tensors (got a tensor on "
                f"{t.device}); there is no CPU fallback"
            )


def prec_of(dtype: torch.dtype) -> int:
    if dtype == torch.float32:
        return _lib.TG_F32
    if dtype == torch.float64:
        return _lib.TG_F64
    raise TypeError(f"unsupported floating dtype {dtype}; use float32 or float64")


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return t.data_ptr()


def aligned16(t: torch.Tensor) -> torch.Tensor:
    """``t`` itself when its data starts on a 16-byte boundary, else a fresh copy (the
    solver and dot kernels read vectors four entries at a time)."""
    return t if t.data_ptr() % 16 == 0 else t.clone()


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)
