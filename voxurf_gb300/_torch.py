"""Torch-side plumbing for the C ABI: pointers, streams, input checks.

PyTorch provides device memory (caching allocator) and the current stream;
all arithmetic happens in the library.
"""
from __future__ import annotations

import torch

from . import _native


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_ptr(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def check_input(t: torch.Tensor, name: str, dtype: torch.dtype | None = None) -> None:
    """CHECK_INPUT of the reference (render_utils.cpp:46-48) plus a dtype check."""
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a tensor")
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise RuntimeError(f"{name} must be {dtype}, got {t.dtype}")


def scratch(nbytes: int, device: torch.device) -> torch.Tensor:
    """Scratch bytes from the caching allocator (the library never allocates)."""
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


def call(name: str, *args) -> None:
    _native.call(name, *args)
