"""Writes oracle_solves.json: full FP64 oracle solves, run to the reference's
stop test (solver/usbs.py:533-540: obj_gap, infeas_gap and max_infeas all at
or below eps), that the device solves are compared with.  The oracle is the
NumPy restatement of the reference's usbs(); each record keeps the instance,
the settings, the iteration at which the stop test fired and the final
values (primal objective, dual objective b.y, gaps, the last candidate's
smallest eigenvalue).  The device path and the oracle share the instance
generators and the start vector (splitmix64 + Box-Muller).

Instances (MaxCut, the reference's README settings: k_curr 10, k_past 1,
sketch 10, rho 0.01, beta 0.25, trace bound 2n, 32 Lanczos vectors x 10
restarts, IPM tolerance 1e-7 x 100):
  er60_1e-4        Erdos-Renyi G(60, 300), seed 3, to eps = 1e-4;
  torus6_1e-4      the 6 x 6 torus with unit weights (bipartite; its SDP
                   value is |E| = 72 in closed form), to eps = 1e-4;
  er800_1e-2       the ER(800, 19176) graph of seed 0 (the README's G1
                   scale), to eps = 1e-2.

Run:  python tests/golden/make_oracle_solves.py   (a few minutes on 8 cores)
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import maxcut as omaxcut  # noqa: E402
from oracle import usbs as ousbs  # noqa: E402
from usbs_gb300 import workloads as wl  # noqa: E402

SETTINGS = dict(trace_factor=2.0, rho=0.01, beta=0.25, k_curr=10, k_past=1, sketch_dim=10,
                lanczos_max_restarts=10, subprob_eps=1e-7, subprob_max_iters=100)
INSTANCES = {
    "er60_1e-4": dict(graph=("er", 60, 300, 3), eps=1e-4, max_iters=6000),
    "torus6_1e-4": dict(graph=("torus_unit", 6), eps=1e-4, max_iters=6000),
    "er800_1e-2": dict(graph=("er", 800, 19176, 0), eps=1e-2, max_iters=3000),
}


def graph(spec):
    if spec[0] == "er":
        return wl.er_graph(spec[1], spec[2], spec[3])
    return wl.torus_graph(spec[1], 0, weights="unit")


def solve(name):
    inst = INSTANCES[name]
    S = SETTINGS
    st = omaxcut.initialize_state(graph(inst["graph"]), S["sketch_dim"])
    n = st.C.shape[0]
    eps = inst["eps"]
    tr = []
    t0 = time.perf_counter()
    out, fin = ousbs.usbs(st, n, n, S["trace_factor"] * n, S["trace_factor"], S["rho"], S["beta"],
                          S["k_curr"], S["k_past"], inst["max_iters"], np.inf, eps, eps, eps,
                          min(n, 32), S["lanczos_max_restarts"], S["subprob_eps"],
                          S["subprob_max_iters"], trace=tr)
    sec = time.perf_counter() - t0
    last = tr[-1]
    return dict(graph=list(inst["graph"]), n=int(n), eps=eps, max_iters=inst["max_iters"],
                iterations=int(fin["t"]), seconds_here=sec,
                primal_obj=float(out.primal_obj), dual_obj=float(np.asarray(st.b) @ out.y),
                obj_gap=float(last["obj_gap"]), infeas_gap=float(last["infeas_gap"]),
                max_infeas=float(last["max_infeas"]), obj_ub=float(last["obj_ub"]),
                cand_eig0=float(last["cand_eig0"]))


def main():
    out = {"settings": SETTINGS, "solves": {}}
    for name in INSTANCES:
        out["solves"][name] = solve(name)
        print(name, out["solves"][name], flush=True)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_solves.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
