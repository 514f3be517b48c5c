"""Arrays cross the Python boundary by DLPack: a device array from another
framework (anything with __dlpack__ / __dlpack_device__, e.g. a JAX array) is
used in place, with no copy to or from the host."""
import numpy as np
import pytest

from oracle import maxcut as omaxcut
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


class Foreign:
    """A device array of another framework: exposes only the DLPack protocol."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, **kw):
        return self._t.__dlpack__(**kw)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_dlpack_device_array_is_used_in_place(cuda):
    import torch
    from usbs_gb300.arrays import to_device
    t = torch.arange(1000, dtype=torch.float64, device=cuda)
    got = to_device(Foreign(t), torch.float64, cuda)
    assert got.data_ptr() == t.data_ptr()            # no copy
    host = to_device(Foreign(torch.arange(10.0, dtype=torch.float64)), torch.float64, cuda)
    assert host.is_cuda and host.cpu().tolist() == list(np.arange(10.0))


def test_eigsh_and_usbs_take_dlpack_inputs(cuda):
    import torch
    from usbs_gb300 import api, solver
    from usbs_gb300.problem import DeviceProblem, layout
    from usbs_gb300.rng import default_q0
    st = omaxcut.initialize_state(wl.er_graph(200, 1500, 5), 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    y = torch.as_tensor(np.random.default_rng(1).standard_normal(n) * 0.3, device=cuda)
    q0 = torch.as_tensor(default_q0(n), device=cuda)
    ref, _ = api.eigsh_smallest(n, prob, None, None, y, q0, 4, 32, 10, 1e-9, c_scale=-1.0)
    got, _ = api.eigsh_smallest(n, prob, None, None, Foreign(y), Foreign(q0), 4, 32, 10, 1e-9,
                                c_scale=-1.0)
    assert torch.equal(ref, got)
    # a whole solve whose state arrives as foreign device arrays
    dev_state = st._replace(y=Foreign(torch.as_tensor(st.y, device=cuda)),
                            z=Foreign(torch.as_tensor(st.z, device=cuda)),
                            P=Foreign(torch.as_tensor(st.P, device=cuda)),
                            Omega=Foreign(torch.as_tensor(st.Omega, device=cuda)))
    kw = dict(q0=default_q0(n), precision=64)
    a = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 3, np.inf, -1.0, -1.0, -1.0, 32, 10,
                    1e-7, 100, **kw)
    b = solver.usbs(dev_state, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 3, np.inf, -1.0, -1.0, -1.0,
                    32, 10, 1e-7, 100, **kw)
    assert torch.equal(a.y, b.y) and a.primal_obj == b.primal_obj
