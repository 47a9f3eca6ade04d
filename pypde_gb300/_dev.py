"""Device-tensor helpers: every field lives in a float64 CUDA tensor."""
import numpy as np
import torch

from . import _lib

DTYPE = torch.float64


def device():
    if not torch.cuda.is_available():
        raise _lib.PgxError("pypde_gb300 needs a CUDA GPU (GB300, sm_103a); no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def to_dev(x):
    """float64 CUDA tensor view of x (numpy array, scalar or tensor)."""
    if isinstance(x, torch.Tensor):
        if x.is_cuda and x.dtype == DTYPE:
            return x
        return x.to(device=device(), dtype=DTYPE)
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=device())


def to_host(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def stream():
    return torch.cuda.current_stream().cuda_stream


def geom(t, axis):
    """(ptr, s0, s1, n_axis, nlines) for a 1-D or 2-D tensor seen along ``axis``.

    A 1-D tensor is an (n, 1) array: one line along axis 0.
    """
    if t.dim() == 1:
        if axis != 0:
            raise ValueError("axis must be 0 for a 1-D array")
        return t.data_ptr(), t.stride(0), 1, t.shape[0], 1
    if t.dim() != 2:
        raise NotImplementedError("ndim must be less than 3")
    n = t.shape[axis]
    return t.data_ptr(), t.stride(0), t.stride(1), n, t.shape[1 - axis]


def empty_like_axis(t, axis, n):
    """New tensor shaped like t with extent n along axis."""
    shape = list(t.shape)
    shape[axis] = n
    return torch.empty(shape, dtype=DTYPE, device=t.device)
