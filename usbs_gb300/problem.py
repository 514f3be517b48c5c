"""Device layout of an SDP's problem data (built once on the host, kept in HBM).

The reference stores C as a JAX BCOO matrix and the constraint tensor A as the
triples ``A_indices`` (c, i, j) with values ``A_data`` (utils/common.py:11-26).
Here the same data is laid out for the kernels:

* ``rowptr/col``      union CSR pattern of C and of the triples' (i, j)
                      positions: the Lanczos operator C + A*(w) lives on it;
* ``c_val``           C's values on that pattern (0.0 where only A has an entry);
* ``slot_ptr/slot_tid`` for every pattern position, the triples that land on it
                      (operator assembly without atomics);
* ``con_ptr, t_row, t_col, t_a``  triples sorted by constraint (A(.));
* ``row_ptr, r_con, r_col, r_a``  triples sorted by row (A*(.));
* ``t_con, t_a0``     the triples' constraint ids / values in the caller's order
                      (indexed by slot_tid).

All integer arrays are int32, values float64.
"""
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


@dataclass
class HostProblemLayout:
    n: int
    m: int
    nnz: int
    num_triples: int
    rowptr: np.ndarray
    col: np.ndarray
    c_val: np.ndarray
    slot_ptr: np.ndarray
    slot_tid: np.ndarray
    t_con: np.ndarray
    t_a0: np.ndarray
    con_ptr: np.ndarray
    t_row: np.ndarray
    t_col: np.ndarray
    t_a: np.ndarray
    row_ptr: np.ndarray
    r_con: np.ndarray
    r_col: np.ndarray
    r_a: np.ndarray
    diag_constraints: bool      # every triple is (c, c, c): MaxCut-style diag(X) = b


def _ptr(keys, size):
    cnt = np.bincount(keys, minlength=size) if keys.size else np.zeros(size, dtype=np.int64)
    out = np.zeros(size + 1, dtype=np.int64)
    np.cumsum(cnt, out=out[1:])
    return out.astype(np.int32)


def layout(C, A_data, A_indices, m=None):
    """Build the device layout from a SciPy sparse C (n x n) and the triples."""
    C = sp.csr_matrix(C, dtype=np.float64)
    n = C.shape[0]
    A_indices = np.asarray(A_indices, dtype=np.int64).reshape(-1, 3)
    A_data = np.asarray(A_data, dtype=np.float64).reshape(-1)
    con, ti, tj = A_indices[:, 0], A_indices[:, 1], A_indices[:, 2]
    if m is None:
        m = int(con.max()) + 1 if con.size else 0
    if con.size and (con.min() < 0 or con.max() >= m or ti.min() < 0 or ti.max() >= n
                     or tj.min() < 0 or tj.max() >= n):
        raise ValueError("constraint triple index out of range")
    Cc = C.tocoo()
    ckey = Cc.row.astype(np.int64) * n + Cc.col.astype(np.int64)
    tkey = ti * n + tj
    keys = np.unique(np.concatenate([ckey, tkey]))
    nnz = keys.size
    if nnz > np.iinfo(np.int32).max:
        raise ValueError("pattern too large for int32 indices")
    prow = keys // n
    pcol = keys % n
    rowptr = _ptr(prow, n)
    c_val = np.zeros(nnz)
    np.add.at(c_val, np.searchsorted(keys, ckey), Cc.data)
    tslot = np.searchsorted(keys, tkey)
    o = np.argsort(tslot, kind="stable")
    slot_ptr = _ptr(tslot, nnz)
    slot_tid = o.astype(np.int32)
    oc = np.argsort(con, kind="stable")
    orow = np.argsort(ti, kind="stable")
    return HostProblemLayout(
        n=n, m=m, nnz=nnz, num_triples=A_data.size, rowptr=rowptr, col=pcol.astype(np.int32),
        c_val=c_val, slot_ptr=slot_ptr, slot_tid=slot_tid, t_con=con.astype(np.int32),
        t_a0=A_data.copy(), con_ptr=_ptr(con, m), t_row=ti[oc].astype(np.int32),
        t_col=tj[oc].astype(np.int32), t_a=A_data[oc].copy(), row_ptr=_ptr(ti, n),
        r_con=con[orow].astype(np.int32), r_col=tj[orow].astype(np.int32),
        r_a=A_data[orow].copy(),
        diag_constraints=bool(con.size == n and np.all(con == ti) and np.all(ti == tj)))


class DeviceProblem:
    """The layout uploaded to one CUDA device as torch tensors (HBM resident)."""

    FIELDS = ("rowptr", "col", "c_val", "slot_ptr", "slot_tid", "t_con", "t_a0", "con_ptr",
              "t_row", "t_col", "t_a", "row_ptr", "r_con", "r_col", "r_a")

    def __init__(self, host: HostProblemLayout, device="cuda"):
        import torch
        self.host = host
        self.n, self.m, self.nnz, self.num_triples = host.n, host.m, host.nnz, host.num_triples
        self.diag_constraints = host.diag_constraints
        self.device = torch.device(device)
        for f in self.FIELDS:
            a = getattr(host, f)
            t = torch.from_numpy(np.ascontiguousarray(a))
            if t.numel() == 0:
                t = torch.zeros(1, dtype=t.dtype)
            setattr(self, f, t.to(self.device, non_blocking=False))

    def h2d_bytes(self):
        return sum(getattr(self.host, f).nbytes for f in self.FIELDS)


SELL_WINDOW = 256   # rows per window (one CUDA block)
SELL_SLICE = 32     # rows per slice (one warp)


def sell_layout(rowptr, col):
    """Sliced-ELL layout of a CSR pattern for usbs_operator_apply_sell.

    Rows are taken in windows of 256, sorted by length (longest first, stable)
    inside their window and cut into 32-row slices; slice s stores its entries
    column-major from ``sl_ptr[s]``, padded to its longest row.  Returns a dict
    of int32 ``sl_ptr`` (slices + 1), int32 ``sl_col`` and ``sl_src`` (the CSR
    position of every stored entry, -1 for padding), and uint8 ``sl_row`` (each
    sorted row's position inside its window; padding lanes get their own,
    unused position)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col)
    n = rowptr.size - 1
    lens = np.diff(rowptr)
    nsl = (n + SELL_SLICE - 1) // SELL_SLICE
    npos = nsl * SELL_SLICE
    # sorted order inside each window
    win = np.arange(n) // SELL_WINDOW
    order = np.lexsort((np.arange(n), -lens, win))          # window, then length desc, then row
    srows = np.full(npos, -1, dtype=np.int64)
    srows[:n] = order
    slens = np.zeros(npos, dtype=np.int64)
    slens[:n] = lens[order]
    widths = slens.reshape(nsl, SELL_SLICE).max(axis=1)
    sl_ptr = np.zeros(nsl + 1, dtype=np.int64)
    np.cumsum(widths * SELL_SLICE, out=sl_ptr[1:])
    total = int(sl_ptr[-1])
    if total > np.iinfo(np.int32).max:
        raise ValueError("sliced-ELL layout exceeds 2^31 entries")
    sl_col = np.zeros(total, dtype=np.int32)
    sl_src = np.full(total, -1, dtype=np.int32)
    pos = np.arange(n)
    rep = np.repeat(pos, slens[:n])                           # sorted position of each entry
    first = np.repeat(np.cumsum(slens[:n]) - slens[:n], slens[:n])
    k = np.arange(rep.size) - first                           # entry index inside its row
    dst = sl_ptr[rep // SELL_SLICE] + SELL_SLICE * k + (rep % SELL_SLICE)
    src = rowptr[srows[rep]] + k
    sl_col[dst] = col[src]
    sl_src[dst] = src
    sl_row = np.empty(npos, dtype=np.uint8)
    sl_row[:n] = order - (np.arange(n) // SELL_WINDOW) * SELL_WINDOW
    sl_row[n:] = np.arange(n, npos) % SELL_WINDOW
    return dict(sl_ptr=sl_ptr.astype(np.int32), sl_col=sl_col, sl_src=sl_src, sl_row=sl_row,
                stored=total)
