"""Array interchange at the Python boundary.

The reference passes JAX arrays (solver/lanczos.py:239-250, solver/usbs.py:436).
Here any array that speaks DLPack (``__dlpack__`` / ``__dlpack_device__``: JAX,
CuPy, torch, ...) enters as a torch view of the same memory
(``torch.from_dlpack``), so a device array of the right dtype reaches the
kernels without a copy.  NumPy arrays and Python sequences are copied to the
device once.  Nothing here computes.
"""
import numpy as np


def as_torch(x):
    """A torch tensor sharing x's memory (torch tensors and DLPack producers),
    or None for NumPy arrays, sequences and scalars."""
    import torch
    if isinstance(x, torch.Tensor):
        return x
    if isinstance(x, np.ndarray) or not hasattr(x, "__dlpack__"):
        return None
    return torch.from_dlpack(x)


def to_device(x, dtype, device):
    """x as a contiguous `dtype` tensor on `device`: the same memory when x
    already is one (directly or through DLPack), else one copy."""
    import torch
    t = as_torch(x)
    if t is not None:
        return t.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=device)


def to_host(x):
    """x as a NumPy array (device arrays are copied to the host)."""
    if x is None:
        return None
    t = as_torch(x)
    if t is not None:
        return t.detach().cpu().numpy()
    return x


def shape_of(x):
    """The shape of a NumPy array, torch tensor or DLPack producer."""
    t = as_torch(x)
    return tuple(t.shape) if t is not None else np.shape(x)
