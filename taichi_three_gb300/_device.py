"""Device selection and tensor helpers."""
import numpy as np
import torch


def default_device():
    return torch.device('cuda') if torch.cuda.is_available() else torch.device('cpu')


def require_cuda(what):
    if not torch.cuda.is_available():
        raise RuntimeError(f'{what} runs on the CUDA device only (no CUDA device is visible)')


def as_f32(x, device=None):
    """float32 contiguous tensor on `device` (default: the CUDA device if present)."""
    device = device or default_device()
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float32).contiguous()
    return torch.as_tensor(np.asarray(x, dtype=np.float32), device=device).contiguous()


def as_i32(x, device=None):
    device = device or default_device()
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.int32).contiguous()
    return torch.as_tensor(np.asarray(x, dtype=np.int32), device=device).contiguous()


def ptr(t, device, keep):
    """Address of `t` on `device` (copying it there if needed; the copy is kept
    alive in `keep`)."""
    if t is None:
        return None
    dev = torch.device(device)
    same = t.device.type == dev.type and (dev.index is None or t.device.index == dev.index)
    if not same or not t.is_contiguous():
        t = t.to(device).contiguous()
    keep.append(t)
    return t.data_ptr()
