"""Writes known_answers.json: closed-form answers the oracle (and, through it,
the device path) is checked against.  The reference ships no golden vectors and
its JAX implementation cannot run here, so these come from mathematics, not
from any implementation:

* Laplacian spectra: path P_n, lambda_j = 2 - 2 cos(pi j / n); cycle C_n,
  lambda_j = 2 - 2 cos(2 pi j / n) (each j and n - j), sorted ascending.
* MaxCut SDP values  max <L/4, X> s.t. diag X = 1, X psd:
  - complete graph K_n, unit weights: n^2 / 4;
  - even side x side torus, unit weights (bipartite, 4-regular): the bound
    (n/4) lambda_max(L) = 2n is met by the bipartition, so the value is |E| = 2n.
  - vertex-transitive graphs, unit weights: the value is (n/4) lambda_max(L)
    (Delorme and Poljak, "Laplacian eigenvalues and the maximum cut problem",
    Math. Programming 62, 1993: the eigenvalue bound with the optimal diagonal
    correction, which is zero for a vertex-transitive graph, equals the SDP
    value).  Non-bipartite cases, where the value lies strictly above the
    maximum cut:
    - odd cycle C_n: lambda_max(L) = 2 + 2 cos(pi / n), value (n/2)(1 + cos(pi/n));
    - Petersen graph: adjacency spectrum {3, 1, -2}, so lambda_max(L) = 5 and
      the value is 12.5 (its maximum cut is 12);
    - odd side x side torus: lambda_max(L) = 2 (2 + 2 cos(pi / side)), value
      side^2 (1 + cos(pi / side)).

Run:  python tests/golden/make_known_answers.py
"""
import json
import math
import os


def path_spectrum(n, count):
    return [2.0 - 2.0 * math.cos(math.pi * j / n) for j in range(count)]


def cycle_spectrum(n, count):
    vals = sorted(2.0 - 2.0 * math.cos(2.0 * math.pi * j / n) for j in range(n))
    return vals[:count]


def main():
    out = {
        "path_laplacian": {"n": 200, "smallest": path_spectrum(200, 5)},
        "cycle_laplacian": {"n": 150, "smallest": cycle_spectrum(150, 5)},
        "maxcut_sdp_complete_graph": {"n": 12, "value": 12 * 12 / 4.0},
        "maxcut_sdp_even_torus": {"side": 6, "n": 36, "edges": 72, "value": 72.0},
        "maxcut_sdp_vertex_transitive": [
            {"graph": ["cycle", 7], "n": 7, "value": 3.5 * (1.0 + math.cos(math.pi / 7))},
            {"graph": ["cycle", 9], "n": 9, "value": 4.5 * (1.0 + math.cos(math.pi / 9))},
            {"graph": ["petersen"], "n": 10, "value": 12.5},
            {"graph": ["torus_unit", 5], "n": 25, "value": 25.0 * (1.0 + math.cos(math.pi / 5))},
        ],
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
