"""Device helpers: torch tensors as plumbing for device memory and streams."""

import numpy as np
import torch


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required: this library has no CPU path")


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes_void(s.cuda_stream)


def ctypes_void(v):
    import ctypes
    return ctypes.c_void_p(int(v))


def ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr())


def to_device_f64(a, device=None):
    """Contiguous float64 CUDA tensor from a numpy array / list / tensor."""
    if isinstance(a, torch.Tensor):
        t = a
        if t.device.type != "cuda":
            t = t.cuda(device)
        return t.to(torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).cuda(device)


def to_device(a, dtype, device=None, pinned=False):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda" if device is None else device, dtype=dtype).contiguous()
    t = torch.as_tensor(np.ascontiguousarray(a))
    if pinned:
        t = t.pin_memory()
    return t.to(device="cuda" if device is None else device, dtype=dtype,
                non_blocking=pinned).contiguous()
