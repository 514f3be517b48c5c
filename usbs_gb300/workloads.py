"""Seeded synthetic SDP instances with the shapes of the reference's benchmarks.

The reference solves Gset / DIMACS10 MaxCut graphs and QAPLIB / TSPLIB QAPs read
from an external archive.  These generators stand in for them with the same
scales, drawn from ``numpy.random.default_rng(seed)``:

* ``er_graph(800, 19176, 0)``        Erdos-Renyi, unit weights (Gset G1 scale)
* ``torus_graph(100, 1)``            100 x 100 torus, +-1 weights (spin glass)
* ``rgg_knn_graph(10**6, 6, 0)``     random geometric 6-NN graph (rgg_n_2_19 scale)
* ``qap_instance(30, 0)``            QAP with a 10 x 10 Manhattan grid
* ``serving_stream(...)``            Poisson stream of ER MaxCut requests

Each graph is returned as a symmetric ``scipy.sparse.csr_matrix`` adjacency with
a zero diagonal, i.e. the matrix the reference's MaxCut builder reads.
"""
import numpy as np
import scipy.sparse as sp


def _sym_adjacency(n, i, j, w):
    A = sp.coo_matrix((w, (i, j)), shape=(n, n))
    A = (A + A.T).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A


def er_graph(n, num_edges, seed, weights="unit"):
    """G(n, E): E distinct unordered pairs drawn uniformly without replacement."""
    rng = np.random.default_rng(seed)
    total = n * (n - 1) // 2
    pick = rng.choice(total, size=num_edges, replace=False)
    iu, ju = np.triu_indices(n, 1)
    i, j = iu[pick], ju[pick]
    if weights == "unit":
        w = np.ones(num_edges)
    else:
        w = rng.choice(np.array([-1.0, 1.0]), size=num_edges)
    return _sym_adjacency(n, i, j, w)


def torus_graph(side, seed, weights="pm1"):
    """side x side periodic grid, degree 4; weights +-1 i.i.d. with P(+1) = 1/2."""
    rng = np.random.default_rng(seed)
    n = side * side
    idx = np.arange(n).reshape(side, side)
    right = np.roll(idx, -1, axis=1)
    down = np.roll(idx, -1, axis=0)
    i = np.concatenate([idx.ravel(), idx.ravel()])
    j = np.concatenate([right.ravel(), down.ravel()])
    if weights == "pm1":
        w = np.where(rng.random(i.size) < 0.5, 1.0, -1.0)
    else:
        w = np.ones(i.size)
    return _sym_adjacency(n, i, j, w)


def rgg_knn_graph(n, k, seed):
    """n points uniform in the unit square joined to their k nearest neighbours,
    symmetrised, unit weights."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    tree = cKDTree(pts)
    _, nbr = tree.query(pts, k=k + 1)
    i = np.repeat(np.arange(n), k)
    j = nbr[:, 1:].reshape(-1)
    A = sp.coo_matrix((np.ones(i.size), (i, j)), shape=(n, n)).tocsr()
    A = ((A + A.T) > 0).astype(np.float64).tocsr()
    A.setdiag(0)
    A.eliminate_zeros()
    A.sort_indices()
    return A


def qap_instance(l, seed, grid=10):
    """Flow F: symmetric, off-diagonal i.i.d. U{0..10}, zero diagonal.  Distance D:
    Manhattan distances between l distinct random cells of a grid x grid lattice.
    Returns (D, W) in the order the reference's loader returns them (the denser
    matrix first)."""
    rng = np.random.default_rng(seed)
    F = np.triu(rng.integers(0, 11, size=(l, l)).astype(np.float64), 1)
    F = F + F.T
    cells = rng.choice(grid * grid, size=l, replace=False)
    xy = np.stack([cells // grid, cells % grid], 1).astype(np.float64)
    Dm = np.abs(xy[:, None, :] - xy[None, :, :]).sum(-1)
    D, W = Dm, F
    if np.count_nonzero(D) < np.count_nonzero(W):
        D, W = W, D
    return D, W


def serving_stream(num_requests=1024, rate=20.0, seed=4, n_lo=200, n_hi=50000, deg_lo=4.0,
                   deg_hi=40.0, warm_frac=0.3, resample_frac=0.01):
    """Poisson arrivals of ER MaxCut requests.  Returns a list of dicts with
    ``arrival`` (s), ``n``, ``edges`` (i, j arrays) and ``warm_from`` (index of an
    earlier request whose graph was perturbed, or -1)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=num_requests))
    reqs = []
    for r in range(num_requests):
        if r > 0 and rng.random() < warm_frac:
            src = int(rng.integers(0, r))
            base = reqs[src]
            n = base["n"]
            i, j = base["i"].copy(), base["j"].copy()
            nre = max(1, int(resample_frac * i.size))
            pos = rng.choice(i.size, size=nre, replace=False)
            a = rng.integers(0, n, size=nre)
            b = (a + 1 + rng.integers(0, n - 1, size=nre)) % n
            i[pos], j[pos] = np.minimum(a, b), np.maximum(a, b)
            reqs.append(dict(arrival=float(t[r]), n=n, i=i, j=j, warm_from=src))
            continue
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        deg = rng.uniform(deg_lo, deg_hi)
        ne = int(round(deg * n / 2))
        a = rng.integers(0, n, size=ne)
        b = (a + 1 + rng.integers(0, n - 1, size=ne)) % n
        reqs.append(dict(arrival=float(t[r]), n=n, i=np.minimum(a, b), j=np.maximum(a, b),
                         warm_from=-1))
    return reqs


def cycle_graph(n):
    """The n-cycle, unit weights."""
    i = np.arange(n)
    A = sp.coo_matrix((np.ones(n), (i, (i + 1) % n)), shape=(n, n))
    return (A + A.T).tocsr()


def petersen_graph():
    """The Petersen graph: outer 5-cycle, spokes i -- i+5, inner pentagram."""
    e = ([(i, (i + 1) % 5) for i in range(5)] + [(i, i + 5) for i in range(5)]
         + [(5 + i, 5 + (i + 2) % 5) for i in range(5)])
    i, j = (np.array(v) for v in zip(*e))
    A = sp.coo_matrix((np.ones(i.size), (i, j)), shape=(10, 10))
    return (A + A.T).tocsr()


def graph_from_spec(spec):
    """("er", n, edges, seed), ("torus_unit", side), ("cycle", n) or
    ("petersen",): the graphs named in recorded solves and known answers."""
    if spec[0] == "er":
        return er_graph(int(spec[1]), int(spec[2]), int(spec[3]))
    if spec[0] == "torus_unit":
        return torus_graph(int(spec[1]), 0, weights="unit")
    if spec[0] == "cycle":
        return cycle_graph(int(spec[1]))
    if spec[0] == "petersen":
        return petersen_graph()
    raise ValueError(f"unknown graph spec {spec!r}")


def stream_adjacency(req):
    n = req["n"]
    A = sp.coo_matrix((np.ones(req["i"].size), (req["i"], req["j"])), shape=(n, n)).tocsr()
    A = ((A + A.T) > 0).astype(np.float64).tocsr()
    A.setdiag(0)
    A.eliminate_zeros()
    A.sort_indices()
    return A


# the benchmark instances, by what they are
INSTANCES = {
    "maxcut_er800_19176": dict(kind="maxcut", gen=lambda: er_graph(800, 19176, 0)),
    "maxcut_torus100_pm1": dict(kind="maxcut", gen=lambda: torus_graph(100, 1)),
    "maxcut_rgg1m_knn6": dict(kind="maxcut", gen=lambda: rgg_knn_graph(10 ** 6, 6, 0)),
    "qap30_grid10": dict(kind="qap", gen=lambda: qap_instance(30, 0)),
}

# USBS settings of the MaxCut configs (README example command of the reference)
MAXCUT_SETTINGS = dict(trace_factor=2.0, rho=0.01, beta=0.25, k_curr=10, k_past=1,
                       sketch_dim=10, obj_gap_eps=1e-7, infeas_gap_eps=1e-7,
                       max_infeas_eps=1e-7, subprob_eps=1e-7, subprob_max_iters=100,
                       lanczos_max_restarts=10, lanczos_inner_iterations=32)
QAP_SETTINGS = dict(trace_factor=2.0, rho=0.005, beta=0.25, k_curr=2, k_past=0,
                    obj_gap_eps=1e-7, infeas_gap_eps=1e-7, max_infeas_eps=1e-7,
                    subprob_eps=1e-7, subprob_max_iters=100, lanczos_max_restarts=10,
                    lanczos_inner_iterations=32)
