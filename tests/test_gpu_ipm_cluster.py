"""The interior-point subproblems on a thread-block cluster (USBS_IPM_CTAS CTAs,
4 by default) against the single-CTA kernel: the cluster splits only the Newton
matrix's columns, the LU's trailing updates and the line search's grid points,
with the single-CTA arithmetic, so whole solves are bit-identical."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, %r)
from oracle import maxcut as omaxcut
from usbs_gb300 import solver, workloads as wl
from usbs_gb300.problems import qap
out = {}
for name, st, kw in [
        ("maxcut", omaxcut.initialize_state(wl.er_graph(300, 3000, 4), 10),
         dict(k_curr=10, k_past=1, rho=0.01)),
        ("maxcut_k12", omaxcut.initialize_state(wl.er_graph(200, 2000, 5), 4),
         dict(k_curr=10, k_past=2, rho=0.01))]:
    n = st.C.shape[0]
    for prec in (64, 32):
        res, tr, info = solver.usbs(st, n, n, 2.0 * n, 2.0, kw["rho"], 0.25, kw["k_curr"],
                                    kw["k_past"], 6, np.inf, -1.0, -1.0, -1.0, 32, 10, 1e-7, 100,
                                    precision=prec, return_trace=True)
        out[f"{name}_{prec}"] = {"trace": [[r[k].hex() if isinstance(r[k], float) else r[k]
                                            for k in sorted(r)] for r in tr],
                                 "y": res.y.cpu().numpy().tobytes().hex()}
D, W = wl.qap_instance(6, 1)
st = qap.initialize_state(D, W, 6)
n, m = st.C.shape[0], st.b.shape[0]
res, tr, info = solver.usbs(st, n, m, 2.0 * 7 * st.SCALE_X, 2.0, 0.005, 0.25, 2, 0, 4, np.inf,
                            -1.0, -1.0, -1.0, 32, 10, 1e-7, 100, precision=64, return_trace=True)
out["qap"] = {"trace": [[r[k].hex() if isinstance(r[k], float) else r[k] for k in sorted(r)]
                        for r in tr], "y": res.y.cpu().numpy().tobytes().hex()}
print(json.dumps(out))
""" % ROOT


def _run(ctas, cl_ls=1):
    env = dict(os.environ, USBS_IPM_CTAS=str(ctas), USBS_IPM_CL_LS=str(cl_ls))
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("ctas", [2, 4])
def test_cluster_ipm_is_bit_identical_to_one_cta(cuda, ctas):
    one, many = _run(1), _run(ctas)
    assert one.keys() == many.keys()
    for key in one:
        assert one[key]["trace"] == many[key]["trace"], key
        assert one[key]["y"] == many[key]["y"], key


def test_cluster_ipm_with_the_one_cta_line_search_is_bit_identical(cuda):
    one, many = _run(1), _run(4, cl_ls=0)
    for key in one:
        assert one[key]["trace"] == many[key]["trace"], key
        assert one[key]["y"] == many[key]["y"], key
