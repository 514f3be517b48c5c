"""The DLPack boundary on the host (no GPU): producers other than NumPy are
taken as views of the same memory; NumPy arrays and sequences are copied."""
import numpy as np

from usbs_gb300.arrays import as_torch, to_device, to_host


class Foreign:
    def __init__(self, t):
        self._t = t

    def __dlpack__(self, **kw):
        return self._t.__dlpack__(**kw)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_dlpack_producer_is_viewed_not_copied():
    import torch
    t = torch.arange(6, dtype=torch.float64)
    v = as_torch(Foreign(t))
    assert v.data_ptr() == t.data_ptr()
    assert to_device(Foreign(t), torch.float64, "cpu").data_ptr() == t.data_ptr()
    np.testing.assert_array_equal(to_host(Foreign(t)), np.arange(6.0))


def test_numpy_and_sequences_are_copied():
    import torch
    a = np.arange(4.0)
    assert as_torch(a) is None
    d = to_device(a, torch.float32, "cpu")
    assert d.dtype == torch.float32 and d.tolist() == [0.0, 1.0, 2.0, 3.0]
    assert to_device([1, 2], torch.float64, "cpu").tolist() == [1.0, 2.0]
    assert to_host(None) is None and to_host(a) is a
