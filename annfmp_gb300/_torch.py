"""Small torch plumbing: device placement, raw pointers, current stream."""
from __future__ import annotations

import numpy as np
import torch

_NP_TO_TORCH = {
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.float64): torch.float64,
}


def require_cuda(device) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("annfmp_gb300 needs a CUDA device (the GPU path has no CPU fallback)")
    dev = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)
    if dev.type != "cuda":
        raise ValueError("device must be a CUDA device")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def to_device(x, dtype: torch.dtype, device: torch.device, non_blocking: bool = False) -> torch.Tensor:
    """Contiguous tensor of the given dtype on the device (numpy arrays are copied in)."""
    if isinstance(x, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(x))
        if t.dtype != dtype:
            t = t.to(dtype)
        return t.to(device, non_blocking=non_blocking)
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=device).contiguous()


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_ptr(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def is_numpy(x) -> bool:
    return isinstance(x, np.ndarray) or not isinstance(x, torch.Tensor)
