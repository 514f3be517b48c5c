"""Instance files of the reference's experiments, read on the host.

* MaxCut graphs from SuiteSparse ``.mat`` files (Gset and DIMACS10), as
  ``scripts/warm_start_maxcut_usbs.py:81-95`` reads them; the adjacency is
  cut to its leading ``int(N * warm_start_frac)`` nodes.
* QAPLIB ``.dat`` files (``utils/qap_helpers.py:26-45``): n, then the two n x n
  matrices; the sparser one becomes the flow matrix W.
* TSPLIB ``.tsp`` files posed as QAPs (``utils/qap_helpers.py:48-154``): D is
  the distance matrix (explicit edge weights or coordinates with the GEO, ATT,
  EUC_2D or CEIL_2D rule of the TSPLIB95 format description), W the canonical
  tour with weight 1/2 per direction.

The QAP readers return (l, D, W); ``usbs_gb300.problems.qap.initialize_state``
builds the relaxation from them.  MATLAB v7.3 (HDF5) files need the ``mat73``
package, which this environment lacks: they raise an error naming it.
"""
import numpy as np
import scipy.io
import scipy.sparse as sp
from scipy.spatial.distance import pdist, squareform


def load_maxcut_mat(path, warm_start_frac=1.0):
    """(W, num_drop): the graph's adjacency (CSC) cut to its leading
    n = N - num_drop nodes, num_drop = N - int(N * warm_start_frac)."""
    try:
        problem = scipy.io.loadmat(path)
    except NotImplementedError as e:      # v7.3 files are HDF5
        raise ValueError(f"{path}: MATLAB v7.3 file; reading it needs the mat73 package") from e
    name = str(path)
    if "Gset" in name:
        W = problem["Problem"][0][0][1]
    elif "DIMACS" in name:
        W = problem["Problem"][0][0][2]
    else:
        raise ValueError("Unknown path type")
    W = sp.csc_matrix(W)
    num_drop = W.shape[0] - int(W.shape[0] * warm_start_frac)
    n = W.shape[0] - num_drop
    return W.tolil()[:n, :n].tocsc(), num_drop


def load_qaplib(path, num_drop=0):
    """(l, D, W) of a QAPLIB instance, the last num_drop facilities dropped."""
    with open(path) as f:
        tokens = f.read().strip().split()
    n = int(tokens[0])
    M = np.array([float(v) for v in tokens[1:1 + 2 * n * n]]).reshape(2 * n, n)
    D, W = M[:n], M[n:]
    if np.count_nonzero(D) < np.count_nonzero(W):   # W is the sparser one by convention
        D, W = W, D
    l = n - num_drop
    return l, D[:l, :l].copy(), W[:l, :l].copy()


def _geo(p1, p2):
    PI, RRR = 3.141592, 6378.388
    deg = np.round(p1[0]); lat1 = PI * (deg + 5.0 * (p1[0] - deg) / 3.0) / 180.0
    deg = np.round(p1[1]); long1 = PI * (deg + 5.0 * (p1[1] - deg) / 3.0) / 180.0
    deg = np.round(p2[0]); lat2 = PI * (deg + 5.0 * (p2[0] - deg) / 3.0) / 180.0
    deg = np.round(p2[1]); long2 = PI * (deg + 5.0 * (p2[1] - deg) / 3.0) / 180.0
    q1 = np.cos(long1 - long2)
    q2 = np.cos(lat1 - lat2)
    q3 = np.cos(lat1 + lat2)
    return int(RRR * np.arccos(0.5 * (q2 * (1.0 + q1) - q3 * (1.0 - q1))) + 1.0)


def _att(p1, p2):
    xd, yd = p1[0] - p2[0], p1[1] - p2[1]
    return np.ceil(np.sqrt((xd * xd + yd * yd) / 10.0))


def load_tsplib(path, num_drop=0):
    """(l, D, W) of a TSPLIB instance posed as a QAP."""
    spec, D, coords = {}, None, None
    with open(path) as f:
        lines = iter(f.read().splitlines())
        for line in lines:
            parts = [p.strip() for p in line.split(":")]
            if len(parts) == 2:
                spec[parts[0]] = parts[1]
                continue
            if len(parts) != 1:
                raise ValueError("Something went wrong when reading file.")
            key = parts[0]
            n = int(spec["DIMENSION"])
            if key == "NODE_COORD_SECTION":
                coords = []
                for row in lines:
                    row = row.strip()
                    if row == "EOF":
                        break
                    _, x, y = row.split()
                    coords.append([float(x), float(y)])
                if len(coords) != n:
                    raise ValueError(f"{path}: {len(coords)} coordinates for DIMENSION {n}")
                break
            if key == "EDGE_WEIGHT_SECTION":
                vals = []
                for row in lines:
                    row = row.strip()
                    if row in ("EOF", "DISPLAY_DATA_SECTION"):
                        break
                    vals += [int(v) for v in row.split()]
                vals = np.array(vals, dtype=float)
                fmt = spec["EDGE_WEIGHT_FORMAT"]
                D = np.zeros((n, n))
                if fmt == "FULL_MATRIX":
                    D[:] = vals.reshape(n, n)
                elif fmt in ("UPPER_ROW", "LOWER_COL"):
                    D[np.triu_indices(n, k=1)] = vals
                    D = D + D.T
                elif fmt in ("UPPER_DIAG_ROW", "LOWER_DIAG_COL"):
                    D[np.triu_indices(n, k=0)] = vals
                    D = D + D.T
                elif fmt in ("LOWER_DIAG_ROW", "UPPER_DIAG_COL"):
                    D[np.tril_indices(n, k=0)] = vals
                    D = D + D.T
                elif fmt in ("LOWER_ROW", "UPPER_COL"):
                    raise NotImplementedError("edge weight format type not implemented")
                else:
                    raise ValueError("Unsupported EDGE_WEIGHT_FORMAT.")
                break
    if D is None:
        if coords is None:
            raise ValueError(f"{path}: no NODE_COORD_SECTION or EDGE_WEIGHT_SECTION")
        coords = np.array(coords)
        kind = spec.get("EDGE_WEIGHT_TYPE")
        if kind == "GEO":
            D = squareform(pdist(coords, _geo))
        elif kind == "ATT":
            D = squareform(pdist(coords, _att))
        elif kind == "EUC_2D":
            D = np.round(squareform(pdist(coords, "euclidean")))
        elif kind == "CEIL_2D":
            D = np.ceil(squareform(pdist(coords, "euclidean")))
        else:
            raise ValueError("Unsupported EDGE_WEIGHT_TYPE.")
    l = D.shape[0] - num_drop
    D = D[:l, :l].copy()
    W = np.zeros((l, l))
    i = np.arange(l)
    np.add.at(W, (i, (i + 1) % l), 0.5)      # duplicates add up (l <= 2), as a BCOO does
    np.add.at(W, ((i + 1) % l, i), 0.5)
    return l, D, W
