"""Benchmark of the USBS hot path on GB300 (one JSON line on rank 0).

Workload (N=1): the 100 x 100 toroidal +-1 spin-glass MaxCut SDP (n = 10,000,
degree 4), solved with the reference's MaxCut settings (k_curr 10, k_past 1,
sketch 10, rho 0.01, beta 0.25, trace bound 2n, tolerances 1e-7, 32 Lanczos
vectors x 10 restarts, IPM <= 100 steps) in the mixed-precision mode (FP32
Lanczos, FP64 bundle subproblems / gaps / Rayleigh refinement).  Synthetic data
(seeded generator with the benchmark's shape); no dataset is read.

A step is one ``usbs()`` call from the cold start that runs ``--iters-per-step``
outer iterations (the stop tolerance is the metric's 1e-4, which this instance
does not reach within a step, so every step does the same work).  ``value`` is
outer iterations per second of the whole job (all ranks; each rank solves its
own instance: replicas, weak scaling).  The 1e-4 solve itself takes thousands of
iterations on this instance for the reference algorithm as well (the oracle is
at relative gap 0.95 after 300 iterations), so solves/s is not a per-step
quantity here.  Solves to the reference's stop test are measured in the
``solves`` leg instead: instances that reach a stated gap within a few
thousand iterations, solved to that gap on the device in FP64 and in mixed
precision, their final values compared with full FP64 oracle solves recorded
in tests/golden/oracle_solves.json, beside the oracle's own solve rate.

Extra measurements on the same line: ``fp64`` (the same steps on the plain
FP64 device path, for a precision-matched comparison with the FP64 reference
arm), ``errors_vs_oracle`` (the final state of a 10-iteration solve against
the FP64 oracle on the same instance and start vector), ``roofline`` of the
Lanczos kernel
(CUDA events around every launch inside the timed region, algorithmic bytes
from the kernel's own counters), the standalone Lanczos SpMV GB/s on the
10^6-node random geometric graph, ``cpu_baseline`` (the NumPy oracle on this
host), ``e2e`` through the public API from pinned host buffers, and SM clocks
sampled with nvidia-smi during the timed region.

``--impl reference`` times the reference algorithm on the CPU (the oracle
restatement; JAX is not installed) with the same metric and unit.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
# the serving legs run up to 32 solves at once, two streams each: give CUDA
# enough hardware queues that their streams do not share queue heads (8 by
# default; read when the CUDA context is created, so set before any CUDA use)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

METRIC = "SDP solves/s and p50/p99 latency at 1e-4 rel gap; Lanczos SpMV HBM GB/s"
UNIT = "USBS outer iterations/s"
LANCZOS_CLUSTER_TRAFFIC_TORUS100 = 653312   # bytes per launch (ncu, GB300)
SETTINGS = dict(k_curr=10, k_past=1, sketch_dim=10, rho=0.01, beta=0.25, trace_factor=2.0,
                subprob_eps=1e-7, subprob_max_iters=100, lanczos_inner_iterations=32,
                lanczos_max_restarts=10, gap_eps=1e-4)


def workload(rank=0):
    from usbs_gb300 import workloads as wl
    return wl.torus_graph(100, 1 + 1000 * rank)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms (the recipe's query)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def run_usbs(st, n, iters, inst, device, precision=32, q0=None):
    from usbs_gb300 import solver
    S = SETTINGS
    return solver.usbs(st, n, n, S["trace_factor"] * n * st.SCALE_X, S["trace_factor"], S["rho"],
                       S["beta"], S["k_curr"], S["k_past"], iters, np.inf, S["gap_eps"],
                       S["gap_eps"], S["gap_eps"], S["lanczos_inner_iterations"],
                       S["lanczos_max_restarts"], S["subprob_eps"], S["subprob_max_iters"], 1.0,
                       None, None, None, q0=q0, precision=precision, device=device,
                       return_info=True, instance=inst)


def lanczos_step_chain(inst, st, n, precision=32):
    """The cluster Lanczos kernel's own cycle counters for one eigsh call on the
    benchmark operator (-C + A*(y) at the initial y, the solver's settings):
    where the cycles of its step chain go.  The kernel keeps its basis in shared
    memory, so this, not DRAM traffic, is its bound."""
    from usbs_gb300 import api
    from usbs_gb300.rng import default_q0
    S = SETTINGS
    info = None
    for _ in range(3):
        _, _, info = api.eigsh_smallest(n, inst.problem, None, None, np.asarray(st.y),
                                        default_q0(n), S["k_curr"], S["lanczos_inner_iterations"],
                                        S["lanczos_max_restarts"], S["subprob_eps"],
                                        c_scale=-1.0, precision=precision, return_info=True)
    bar, red, a, b, c = info.phase_kcycles
    steps = max(info.matvecs, 1)
    per = lambda kc: round(1024.0 * kc / steps)
    return {"kernel": f"lanczos_cluster_kernel<{'float' if precision == 32 else 'double'}>",
            "call_kcycles": info.total_kcycles, "steps": info.matvecs,
            "restarts": info.restarts,
            "cycles_per_step": per(bar + red + a + b + c),
            "per_step": {"spmv_and_first_dots": per(a), "second_projection": per(b),
                         "norm_pass": per(c), "cluster_reductions": per(red),
                         "barrier_waits": per(bar)},
            "restart_eigensolve_cycles_per_restart":
                round(1024.0 * info.eig_kcycles / max(info.restarts, 1)),
            "note": "clock64 counters of CTA 0 (1 kcycle = 1024 cycles); the phases are "
                    "latency chains (shared and distributed shared memory loads, FP64 "
                    "reductions, one cluster barrier each), not DRAM streams"}


def cpu_oracle_iterations(st, n, iters):
    """Oracle (NumPy FP64 restatement) outer iterations; returns (iterations, seconds)."""
    from oracle import usbs as ousbs
    S = SETTINGS
    t0 = time.perf_counter()
    out, fin = ousbs.usbs(st, n, n, S["trace_factor"] * n * st.SCALE_X, S["trace_factor"],
                          S["rho"], S["beta"], S["k_curr"], S["k_past"], iters, np.inf,
                          S["gap_eps"], S["gap_eps"], S["gap_eps"],
                          S["lanczos_inner_iterations"], S["lanczos_max_restarts"],
                          S["subprob_eps"], S["subprob_max_iters"])
    return int(fin["t"]), time.perf_counter() - t0


def spmv_gbs(device, reps=20):
    """Standalone Lanczos operator apply (FP32) on the 10^6-node RGG, L2 flushed
    before every launch: the CSR kernel and the sliced-ELL kernel on the graph
    as generated (random node order), and the sliced-ELL kernel after a
    reverse Cuthill-McKee renumbering (a host pre-pass, once per problem).
    Bytes are the CSR algorithmic bytes in every case."""
    import ctypes
    import torch
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    from usbs_gb300 import api, workloads as wl
    from usbs_gb300.problem import DeviceProblem, layout, sell_layout
    from usbs_gb300.problems import maxcut
    lib = api._lib.load()
    W = wl.rgg_knn_graph(10 ** 6, 6, 0)
    st = maxcut.initialize_state(W, 1)
    n = st.C.shape[0]
    host = layout(st.C, st.A_data, st.A_indices, m=n)
    prob = DeviceProblem(host, device)
    w = torch.zeros(n, device=device, dtype=torch.float64)
    op = torch.empty(prob.nnz, dtype=torch.float32, device=device)
    lib.usbs_assemble_operator(prob.nnz, api._p(prob.c_val), -1.0, api._p(prob.slot_ptr),
                               api._p(prob.slot_tid), api._p(prob.t_con), api._p(prob.t_a0),
                               api._p(w), api._p(op), 32, api._stream())
    x = torch.randn(n, device=device, dtype=torch.float32)
    y = torch.empty(n, dtype=torch.float32, device=device)
    # L2 flush between launches: write a 256 MB buffer (larger than the 129 MB
    # L2), then read another, so the timed kernel starts with an L2 of clean
    # lines and pays no write-back of the flush's dirty data
    flush = torch.empty(256 * 2 ** 20, dtype=torch.uint8, device=device)
    flush_rd = torch.ones(64 * 2 ** 20, dtype=torch.float32, device=device)
    p = api._p
    nnz = prob.nnz
    alg = 8.0 * nnz + 4.0 * (n + 1) + 4.0 * n + 4.0 * n

    def timed(fn):
        fn()                                   # warm-up
        ms = []
        for _ in range(reps):
            flush.zero_()
            flush_rd.sum()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    def sell_case(rowptr, col, vals_dev):
        L = sell_layout(rowptr, col)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), device=device, dtype=dt)
        slp, slc, slr = t(L["sl_ptr"], torch.int32), t(L["sl_col"], torch.int32), \
            t(L["sl_row"], torch.uint8)
        src = t(L["sl_src"], torch.int32)
        slv = torch.empty(L["stored"], dtype=torch.float32, device=device)
        lib.usbs_gather_values(L["stored"], p(src), p(vals_dev), p(slv), 32, api._stream())
        ms = timed(lambda: lib.usbs_operator_apply_sell(n, p(slp), p(slc), p(slv), p(slr), p(x),
                                                         p(y), 32, api._stream()))
        return ms, L["stored"], slc, slv

    ms_csr = timed(lambda: lib.usbs_operator_apply(n, nnz, p(prob.rowptr), p(prob.col), p(op),
                                                   p(x), p(y), 32, api._stream()))
    ms_sell, stored, _, _ = sell_case(host.rowptr, host.col, op)
    # renumbered copy of the same operator
    Cop = sp.csr_matrix((op.cpu().numpy(), host.col, host.rowptr), shape=(n, n))
    perm = reverse_cuthill_mckee(Cop, symmetric_mode=True)
    Cr = Cop[perm][:, perm].tocsr()
    Cr.sort_indices()
    ms_rcm, _, slc, slv = sell_case(Cr.indptr, Cr.indices,
                                    torch.as_tensor(Cr.data, device=device, dtype=torch.float32))
    # what a kernel of this size reaches: one coalesced 16-byte pass over the same
    # column and value arrays (no gathers), timed the same way
    pb = (slc.numel() * 4) // 16 * 16
    sums = torch.empty(4 * 152 * 8, dtype=torch.float32, device=device)
    xors = torch.empty(4 * 152 * 8, dtype=torch.int32, device=device)
    ms_stream = {}
    for blocks in (152 * 8, 152 * 32):
        ms_stream[blocks] = timed(lambda: lib.usbs_stream_probe(
            p(slc), pb, p(slv), pb, blocks, p(sums), p(xors), api._stream()))
    ms_probe = min(ms_stream.values())
    gbs = lambda ms: alg / (ms * 1e-3) / 1e9
    return {"graph": "rgg n=1e6 k=6", "nnz": int(nnz), "alg_bytes": alg,
            "kernel": "sell_spmv_kernel<float>", "ms": ms_sell, "gbs": gbs(ms_sell),
            "stored_over_nnz": stored / nnz,
            "csr_kernel": {"ms": ms_csr, "gbs": gbs(ms_csr)},
            "sell_after_rcm_renumbering": {"ms": ms_rcm, "gbs": gbs(ms_rcm)},
            "stream_probe_same_arrays": {
                "bytes": 2 * pb, "ms": ms_probe, "gbs": 2 * pb / (ms_probe * 1e-3) / 1e9,
                "note": "one coalesced pass over the renumbered operator's column and value "
                        "arrays (no gathers, x and y not touched), one launch after the L2 "
                        "flush: the bandwidth a kernel of this size reaches here",
                "sell_after_rcm_gbs_over_probe_gbs": gbs(ms_rcm) / (2 * pb / (ms_probe * 1e-3) / 1e9)},
            "eigsh": eigsh_leg(device, prob, n, flush, flush_rd),
            "eigsh_after_rcm_renumbering": eigsh_renumbered(device, st, n, flush, flush_rd),
            "usbs_solve": rgg_solve_leg(device, st, n)}


def rgg_solve_leg(device, st, n, iters=4):
    """usbs() on the 10^6-node random geometric graph (mixed precision, the
    reference's MaxCut settings): outer iterations per second from the cold
    start after a one-iteration warm-up, with the Lanczos share (the stream
    path), as generated and after the RCM renumbering."""
    import torch
    from usbs_gb300 import solver
    from usbs_gb300.rng import default_q0
    S = SETTINGS
    out = {"workload": "maxcut rgg n=1e6 k=6, mixed precision, reference settings",
           "iterations": iters}
    from usbs_gb300 import renumber
    for ren in (False, True):
        # the problem layout (and the renumbering) are set up once, outside
        # the timed calls, as a caller that solves the problem repeatedly does
        stp, q0 = st, default_q0(n)
        if ren:
            perm = renumber.rcm_permutation(st.C, st.A_indices, n)
            stp, q0 = renumber.permute_state(st, perm), q0[perm]
        inst = solver.DeviceInstance(stp, device)

        def run(k):
            return solver.usbs(stp, n, n, S["trace_factor"] * n, S["trace_factor"], S["rho"],
                               S["beta"], S["k_curr"], S["k_past"], k, np.inf, S["gap_eps"],
                               S["gap_eps"], S["gap_eps"], S["lanczos_inner_iterations"],
                               S["lanczos_max_restarts"], S["subprob_eps"],
                               S["subprob_max_iters"], q0=q0, precision=32, device=device,
                               return_info=True, instance=inst)
        run(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, info = run(iters)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["after_rcm_renumbering" if ren else "as_generated"] = {
            "outer_iterations_per_s": info["iterations"] / dt, "seconds": dt,
            "lanczos_ms_per_call": info["lanczos_ms"] / max(info["lanczos_launches"], 1),
            "lanczos_share": info["lanczos_ms"] * 1e-3 / dt, "obj_gap": info["obj_gap"],
            "kernel_launches": info["kernel_launches"], "status": info["status"]}
    return out


def eigsh_renumbered(device, st, n, flush, flush_rd):
    """eigsh_leg on the RCM-renumbered problem (usbs_gb300.renumber), the start
    vector permuted with it."""
    from usbs_gb300 import renumber
    from usbs_gb300.problem import DeviceProblem, layout
    from usbs_gb300.rng import default_q0
    perm = renumber.rcm_permutation(st.C, st.A_indices, n)
    Cp, idx = renumber.permute_problem(st.C, st.A_indices, perm)
    prob = DeviceProblem(layout(Cp, st.A_data, idx, m=n), device)
    return eigsh_leg(device, prob, n, flush, flush_rd, q0=default_q0(n)[perm])


LANCZOS_KERNELS = {0: "lanczos_team_kernel<float>", 1: "lanczos_cluster_kernel<float>",
                   2: "stream path (st_sell_spmv, st_dot, st_update_* kernels, float)"}


def eigsh_leg(device, prob, n, flush, flush_rd, q0=None):
    """One eigsh_smallest call on the same 10^6-node operator (FP32, 10
    eigenpairs, 32 inner vectors, 10 restarts, tolerance 1e-7; at this size the
    library takes the stream path), L2 flushed first, timed with CUDA events on
    the launching stream, with its algorithmic bytes from the kernel's own
    counters."""
    import torch
    from usbs_gb300 import api
    from usbs_gb300.rng import default_q0
    y = torch.zeros(n, dtype=torch.float64, device=device)
    q0 = torch.as_tensor(default_q0(n) if q0 is None else q0, dtype=torch.float64,
                         device=device)
    call = lambda: api.eigsh_smallest(n, prob, None, None, y, q0, 10, 32, 10, 1e-7,
                                      c_scale=-1.0, precision=32, return_info=True)
    call()                                          # warm-up
    flush.zero_()
    flush_rd.sum()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    _, _, inf = call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    b, m = 4.0, 32
    steps, restarts = inf.matvecs, inf.restarts
    spmv = (4.0 + b) * prob.nnz + 4.0 * (n + 1) + 2.0 * b * n
    cgs = 3.0 * b * n * inf.sum_active_columns + 6.0 * b * n * steps
    rot = restarts * b * n * m + b * n * (inf.sum_saved + 2.0 * restarts)
    alg = steps * spmv + cgs + rot
    peak, kind = peaks()
    vals, _, _ = call()
    from usbs_gb300 import _lib as ulib
    path = ulib.load().usbs_lanczos_kernel(n, 32, 32)
    out = {"kernel": LANCZOS_KERNELS[path], "ms": ms, "matvecs": steps,
           "restarts": restarts, "eigenvalues_first3": [float(v) for v in vals[:3]],
           "alg_bytes": alg, "gbs": alg / (ms * 1e-3) / 1e9,
           "frac_of_" + kind: alg / (ms * 1e-3) / 1e9 / peak}
    if path != 2:
        out["phase_kcycles_bar_red_A_B_C"] = inf.phase_kcycles
    return out


def serving_stream(count, seed, n_lo=200, n_hi=2000):
    """A scaled-down version of the serving workload: `count` Erdos-Renyi MaxCut
    requests, n log-uniform in [n_lo, n_hi], mean degree uniform in [4, 40],
    unit weights, Poisson arrivals (20 per second)."""
    from usbs_gb300 import workloads as wl
    from usbs_gb300.problems import maxcut
    rs = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(count):
        n = int(round(np.exp(rs.uniform(np.log(n_lo), np.log(n_hi)))))
        deg = rs.uniform(4.0, 40.0)
        e = min(int(deg * n / 2), n * (n - 1) // 2)
        st = maxcut.initialize_state(wl.er_graph(n, e, 100 + i), SETTINGS["sketch_dim"])
        t += rs.exponential(1.0 / 20.0)
        out.append((t, n, st))
    return out


def qap_leg(device, iters=10):
    """The QAP relaxation with l = 30 facilities (lifted order 901, about 3.4e5
    constraints; synthetic flow U{0..10}, Manhattan distances on a 10 x 10
    grid) at the reference's QAP settings: outer iterations per second of the
    device solver in each precision, after one warm-up call."""
    import torch
    from usbs_gb300 import solver, workloads as wl
    from usbs_gb300.problems import qap
    D, W = wl.qap_instance(30, 0)
    st = qap.initialize_state(D, W, 30)
    n, m = st.C.shape[0], st.b.shape[0]
    trace_ub = 2.0 * float(30 + 1) * st.SCALE_X
    out = {"workload": "qap l=30 (n=901)", "m": int(m), "nnz_C": int(st.C.nnz),
           "settings": {"k_curr": 2, "k_past": 0, "rho": 0.005, "trace_factor": 2.0,
                        "sketch_dim": 30, "subprob_eps": 1e-7, "lanczos_max_restarts": 10}}
    inst = solver.DeviceInstance(st, device)
    for prec in (32, 64):
        def run(k):
            return solver.usbs(st, n, m, trace_ub, 2.0, 0.005, 0.25, 2, 0, k, np.inf, -1.0, -1.0,
                               -1.0, 32, 10, 1e-7, 100, precision=prec, instance=inst,
                               return_trace=True)
        run(2)
        torch.cuda.synchronize()
        t = time.perf_counter()
        _, recs, info = run(iters)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        out[f"fp{prec}"] = {"outer_iterations_per_s": iters / dt, "status": info["status"],
                            "obj_gap": recs[-1]["obj_gap"], "infeas_gap": recs[-1]["infeas_gap"]}
    return out


def eigsh_batched_leg(device, count=48, seed=9, reps=3):
    """Lanczos for many instances in one launch: `count` MaxCut operators of
    uneven size (the serving stream's generator, n log-uniform in [500, 5000])
    solved by eigsh_smallest_batched (one launch, one cluster per instance)
    against the same calls one after another (one launch each), 10 eigenpairs,
    32 inner vectors, 10 restarts, tolerance 1e-7, in each precision, and
    again after usbs_lanczos_autotune has chosen the batch's cluster size.
    Problems are resident; each timing is the best of `reps` after a warm-up."""
    import torch
    from usbs_gb300 import api
    from usbs_gb300.problem import DeviceProblem, layout
    from usbs_gb300.rng import default_q0
    reqs = serving_stream(count, seed, n_lo=500, n_hi=5000)
    probs = []
    for _, n, st in reqs:
        p = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), device)
        y = torch.as_tensor(np.random.default_rng(n).standard_normal(n) * 0.5, device=device)
        probs.append((p, y, torch.as_tensor(default_q0(n), device=device)))
    out = {"instances": count, "n_total": int(sum(p.n for p, _, _ in probs)),
           "nnz_total": int(sum(p.nnz for p, _, _ in probs)), "num_desired": 10,
           "inner_iterations": 32, "max_restarts": 10, "tolerance": 1e-7}

    def timed(fn):
        fn()
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            best = dt if best is None or dt < best else best
        return best, r

    for prec in (32, 64):
        tb, rb = timed(lambda: api.eigsh_smallest_batched(probs, 10, 32, 10, 1e-7, c_scale=-1.0,
                                                          precision=prec))
        ts, rs = timed(lambda: [api.eigsh_smallest(p.n, p, None, None, y, q0, 10, 32, 10, 1e-7,
                                                   c_scale=-1.0, precision=prec)
                                for p, y, q0 in probs])
        # the smallest eigenvalue converges; the trailing returned values need
        # not (10 restarts), and which ones the restart keeps depends on rounding
        dev0 = max(float(abs(a[0][0] - b[0][0]) / abs(b[0][0])) for a, b in zip(rb, rs))
        dev = max(float((a[0] - b[0]).abs().max() / b[0].abs().max()) for a, b in zip(rb, rs))
        # the autotuner's choice for this batch class, then the batch again
        tune = api.lanczos_autotune(probs, 10, 32, 10, 1e-7, c_scale=-1.0, precision=prec)
        tt, _ = timed(lambda: api.eigsh_smallest_batched(probs, 10, 32, 10, 1e-7, c_scale=-1.0,
                                                          precision=prec))
        api.set_lanczos_tuning([], clear=True)
        out[f"fp{prec}"] = {"batched_solves_per_s": count / tb, "serial_solves_per_s": count / ts,
                            "speedup": ts / tb, "max_rel_diff_smallest_eigenvalue": dev0,
                            "max_rel_diff_all_returned": dev,
                            "autotuned": {"rows_per_cta": tune["rows_per_cta"],
                                          "candidate_ms": tune["ms"],
                                          "batched_solves_per_s": count / tt}}
    return out


def replica_throughput(ms, units, world, device):
    """Whole-job throughput of `world` independent replicas: the units all
    ranks processed over the slowest rank's time.  Returns (max ms, units/s)."""
    import torch
    import torch.distributed as dist
    t_max = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u_tot = torch.tensor([float(units)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
        dist.all_reduce(u_tot, op=dist.ReduceOp.SUM)
    ms_max = float(t_max.item())
    return ms_max, float(u_tot.item()) / (ms_max * 1e-3)


def blas_threads():
    """Threads the oracle's NumPy/SciPy linear algebra runs on (its dense
    kernels are multithreaded BLAS; the rest of the port is one thread)."""
    try:
        import threadpoolctl
        n = [i["num_threads"] for i in threadpoolctl.threadpool_info() if i["user_api"] == "blas"]
        if n:
            return max(n)
    except Exception:
        pass
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        if os.environ.get(var, "").isdigit():
            return int(os.environ[var])
    return os.cpu_count() or 1


def serving_leg(device, count=16, iters=30, slots=8, seed=4):
    """Requests of `serving_stream` solved (a fixed `iters` outer iterations
    each, reference settings) through SolverService in mixed precision, released
    at their arrival times, against the same requests run one after another on
    the plain FP64 single-instance path.  Returns throughput and latencies, with
    the service's cluster Lanczos at the library's single-solve spread (0) and
    packed at 640 rows per CTA."""
    import torch
    from usbs_gb300 import solver
    from usbs_gb300.serving import SolveRequest, SolverService
    S = SETTINGS
    stream = serving_stream(count, seed)

    def kw(n):
        return dict(n=n, m=n, trace_ub=S["trace_factor"] * n, trace_factor=S["trace_factor"],
                    rho=S["rho"], beta=S["beta"], k_curr=S["k_curr"], k_past=S["k_past"],
                    max_iters=iters, max_time=np.inf, obj_gap_eps=-1.0, infeas_gap_eps=-1.0,
                    max_infeas_eps=-1.0, lanczos_inner_iterations=S["lanczos_inner_iterations"],
                    lanczos_max_restarts=S["lanczos_max_restarts"],
                    subprob_eps=S["subprob_eps"], subprob_max_iters=S["subprob_max_iters"])

    solver.usbs(stream[0][2], precision=64, device=device, **kw(stream[0][1]))   # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _, n, st in stream:
        solver.usbs(st, precision=64, device=device, **kw(n))
    torch.cuda.synchronize()
    serial = time.perf_counter() - t0
    def served(nslots, paced, rows):
        with SolverService(device=device, max_slots=nslots, reserve_bytes=4 << 30,
                           lanczos_rows_per_cta=rows) as svc:
            t0 = time.perf_counter()
            handles = []
            for arr, n, st in stream:
                while paced and time.perf_counter() - t0 < arr:
                    time.sleep(0.001)
                handles.append(svc.submit(SolveRequest(st, precision=32, **kw(n))))
            for h in handles:
                h.wait(3600)
            wall = time.perf_counter() - t0
        return wall, np.array([h.latency for h in handles])

    # capacity: every request queued at once (the service admits them as slots free up)
    sat = {(q, r): served(q, False, r)[0] for q in (slots, 2 * slots) for r in (0, 640)}
    best = min(sat, key=sat.get)
    paced = {r: served(slots, True, r) for r in (0, 640)}
    rows = min(paced, key=lambda r: paced[r][0])
    wall, lat = paced[rows]
    return {"requests": count, "outer_iterations_each": iters, "slots": slots,
            "n_range": [200, 2000], "arrivals": "Poisson 20/s", "lanczos_rows_per_cta": rows,
            "served_requests_per_s": count / wall, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "paced_requests_per_s_by_rows_per_cta": {str(r): count / w for r, (w, _) in
                                                     paced.items()},
            "serial_fp64_requests_per_s": count / serial,
            "throughput_ratio_vs_serial_fp64": (count / wall) / (count / serial),
            "saturated": {"slots": best[0], "lanczos_rows_per_cta": best[1],
                          "requests_per_s": count / sat[best],
                          "by_slots_and_rows_per_cta": {f"{q}/{r}": count / w
                                                        for (q, r), w in sat.items()},
                          "ratio_vs_serial_fp64": serial / sat[best]}}


def main_config(it_step):
    """The workload of the main line; both arms report exactly this."""
    return {"workload": "maxcut torus 100x100 +-1 (n=10000, nnz=50000), reference settings",
            "iters_per_step": it_step, "settings": SETTINGS, "parallelism": "replicas",
            "l2": "device arm: flushed before every timed step (256 MB write); the ~3 MB "
                  "working set is reloaded within the step"}


def oracle_trace(st, n, iters, eps=-1.0, q0=None):
    """FP64 oracle run of `iters` outer iterations (or to `eps`): (trace, final
    state, b.y of the final y, seconds)."""
    from oracle import usbs as ousbs
    S = SETTINGS
    tr = []
    t0 = time.perf_counter()
    out, fin = ousbs.usbs(st, n, n, S["trace_factor"] * n * st.SCALE_X, S["trace_factor"],
                          S["rho"], S["beta"], S["k_curr"], S["k_past"], iters, np.inf, eps, eps,
                          eps, min(n, S["lanczos_inner_iterations"]), S["lanczos_max_restarts"],
                          S["subprob_eps"], S["subprob_max_iters"], q0=q0, trace=tr)
    sec = time.perf_counter() - t0
    return tr, out, float(np.asarray(st.b) @ out.y), sec


def errors_vs_oracle(g, o):
    """Final-state errors of a device solve against the FP64 oracle: relative
    for the primal and dual objectives and the smallest candidate eigenvalue,
    absolute for the gaps (themselves relative quantities)."""
    rel = lambda a, b: abs(a - b) / max(abs(b), 1e-300)
    return {"primal_obj_rel": rel(g["primal_obj"], o["primal_obj"]),
            "dual_obj_rel": rel(g["dual_obj"], o["dual_obj"]),
            "lambda_min_abs": abs(g["cand_eig0"] - o["cand_eig0"]),
            "obj_gap_abs": abs(g["obj_gap"] - o["obj_gap"]),
            "infeas_gap_abs": abs(g["infeas_gap"] - o["infeas_gap"]),
            "max_infeas_abs": abs(g["max_infeas"] - o["max_infeas"])}


def device_final(st, n, iters, device, precision, eps=-1.0, q0=None):
    """A device solve of `iters` outer iterations (or to `eps`) with its last
    trace record: (record with dual_obj, info, seconds)."""
    import torch
    from usbs_gb300 import solver
    S = SETTINGS
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out, tr, info = solver.usbs(st, n, n, S["trace_factor"] * n * st.SCALE_X, S["trace_factor"],
                                S["rho"], S["beta"], S["k_curr"], S["k_past"], iters, np.inf,
                                eps, eps, eps, min(n, S["lanczos_inner_iterations"]),
                                S["lanczos_max_restarts"], S["subprob_eps"],
                                S["subprob_max_iters"], q0=q0, precision=precision,
                                device=device, return_trace=True)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    rec = dict(tr[-1])
    rec["dual_obj"] = float(np.asarray(st.b) @ out.y.cpu().numpy())
    return rec, info, sec


TRACE_KEYS = ("primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj",
              "cand_eig0", "obj_gap", "infeas_gap", "max_infeas", "tr_X")


def trajectory_vs_oracle(st, n, device, q0, iters):
    """Per outer iteration t < iters, the largest of |dev - oracle| / max(1,
    |oracle|) over the traced values, FP64 and mixed precision."""
    import torch
    from oracle import usbs as ousbs
    from usbs_gb300 import solver
    S = SETTINGS
    args = (n, n, S["trace_factor"] * n * st.SCALE_X, S["trace_factor"], S["rho"], S["beta"],
            S["k_curr"], S["k_past"], iters, np.inf, -1.0, -1.0, -1.0,
            S["lanczos_inner_iterations"], S["lanczos_max_restarts"], S["subprob_eps"],
            S["subprob_max_iters"])
    otr = []
    ousbs.usbs(st, *args, q0=q0, trace=otr)
    out = {}
    for prec in (64, 32):
        _, gtr, _ = solver.usbs(st, *args, q0=q0, precision=prec, device=device,
                                return_trace=True)
        torch.cuda.synchronize()
        out[f"fp{prec}"] = [max(abs(a[k] - b[k]) / max(1.0, abs(a[k])) for k in TRACE_KEYS)
                            for a, b in zip(otr, gtr)]
    return out


def golden_solves():
    with open(os.path.join(ROOT, "tests", "golden", "oracle_solves.json")) as f:
        return json.load(f)


def oracle_solve_rates():
    """The FP64 oracle's outer iterations per second on each instance of the
    recorded oracle solves (a bounded sample of the same solve from its cold
    start), and the solves/s they give with the recorded iteration count."""
    from usbs_gb300 import workloads as wl
    from usbs_gb300.problems import maxcut
    out = {}
    for name, rec in golden_solves()["solves"].items():
        st = maxcut.initialize_state(wl.graph_from_spec(rec["graph"]), SETTINGS["sketch_dim"])
        n = st.C.shape[0]
        it = min(rec["iterations"], 40 if n <= 100 else 20)
        _, _, _, sec = oracle_trace(st, n, it)              # the solve's first `it` iterations
        rate = it / sec
        out[name] = {"iterations_per_s": rate, "sample_iterations": it,
                     "iterations_to_eps": rec["iterations"],
                     "solves_per_s": rate / rec["iterations"]}
    return out


def solves_leg(device):
    """Solves to the reference's stop test (obj_gap, infeas_gap and max_infeas
    all <= eps) on the device, FP64 and mixed precision, from the cold start,
    for the instances of tests/golden/oracle_solves.json; each with its
    solves/s, iterations and final values, and the final values' errors
    against the recorded FP64 oracle solve of the same instance."""
    from usbs_gb300 import workloads as wl
    from usbs_gb300.problems import maxcut
    g = golden_solves()
    out = {}
    for name, rec in g["solves"].items():
        st = maxcut.initialize_state(wl.graph_from_spec(rec["graph"]), SETTINGS["sketch_dim"])
        n = st.C.shape[0]
        eps = rec["eps"]
        o = dict(rec)
        r = {"n": n, "eps": eps, "oracle_iterations": rec["iterations"]}
        device_final(st, n, 3, device, 32)                  # warm-up
        for prec in (64, 32):
            fin, info, sec = device_final(st, n, rec["max_iters"], device, prec, eps=eps)
            reached = (fin["obj_gap"] <= eps and fin["infeas_gap"] <= eps
                       and fin["max_infeas"] <= eps)
            r[f"fp{prec}"] = {"solves_per_s": 1.0 / sec, "seconds": sec,
                              "iterations": info["iterations"], "reached_eps": bool(reached),
                              "final": {k: fin[k] for k in ("primal_obj", "dual_obj", "obj_gap",
                                                            "infeas_gap", "max_infeas",
                                                            "cand_eig0")},
                              "errors_vs_oracle": errors_vs_oracle(fin, o)}
        out[name] = r
    return out


def serving_stream_leg(device, count=1024, iters=20, slots=32, serial_sample=32):
    """The serving workload: `count` Erdos-Renyi MaxCut requests with Poisson
    arrivals at 20/s, n log-uniform in [200, 50000], mean degree uniform in
    [4, 40], unit weights; 30% are variants of an earlier request (1% of its
    edges re-sampled) warm-started from that request's result on the device
    (implicit warm start).  Each request runs `iters` outer iterations in mixed
    precision through SolverService (the 1e-4 stop is thousands of iterations
    away at the reference's settings), released at its arrival time.  Reported
    beside the plain FP64 single-instance path run one request after another on
    the first `serial_sample` cold requests."""
    import torch
    from usbs_gb300 import solver, workloads as wl
    from usbs_gb300.problems import maxcut
    from usbs_gb300.serving import SolveRequest, SolverService
    S = SETTINGS
    reqs = wl.serving_stream(count, 20.0, 4, 200, 50000, 4.0, 40.0, 0.3, 0.01)
    prep = []
    for r in reqs:                               # host set-up, before the clock starts
        W = wl.stream_adjacency(r)
        st = maxcut.initialize_state(W, S["sketch_dim"])
        prep.append((r, W, st, solver.host_problem_layout(st)))

    def kw(n):
        return dict(n=n, m=n, trace_ub=S["trace_factor"] * n, trace_factor=S["trace_factor"],
                    rho=S["rho"], beta=S["beta"], k_curr=S["k_curr"], k_past=S["k_past"],
                    max_iters=iters, max_time=np.inf, obj_gap_eps=-1.0, infeas_gap_eps=-1.0,
                    max_infeas_eps=-1.0, lanczos_inner_iterations=S["lanczos_inner_iterations"],
                    lanczos_max_restarts=S["lanczos_max_restarts"],
                    subprob_eps=S["subprob_eps"], subprob_max_iters=S["subprob_max_iters"])

    # serial FP64 single-instance path on a sample of cold requests
    cold = [(r, st) for r, _, st, _ in prep if r["warm_from"] < 0][:serial_sample]
    solver.usbs(cold[0][1], precision=64, device=device, **kw(cold[0][0]["n"]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r, st in cold:
        solver.usbs(st, precision=64, device=device, **kw(r["n"]))
    torch.cuda.synchronize()
    serial = (time.perf_counter() - t0) / len(cold)
    with SolverService(device=device, max_slots=slots, reserve_bytes=8 << 30) as svc:
        handles = []
        t0 = time.perf_counter()
        for r, W, st, lay in prep:
            while time.perf_counter() - t0 < r["arrival"]:
                time.sleep(0.0005)
            warm = r["warm_from"] >= 0
            req = SolveRequest(
                st, precision=32, host_layout=lay,
                warm_from=handles[r["warm_from"]] if warm else None,
                warm_start=(lambda res, cold_st, W=W: maxcut.implicit_warm_start(
                    res, W, S["sketch_dim"])) if warm else None,
                **kw(r["n"]))
            handles.append(svc.submit(req))
        for h in handles:
            h.wait(7200)
        wall = time.perf_counter() - t0
    lat = np.array([h.latency for h in handles])
    gaps = np.array([h.info["obj_gap"] for h in handles])
    ns = np.array([r["n"] for r in reqs])
    big = ns > 20000
    return {"requests": count, "arrivals": "Poisson 20/s", "n_range": [200, 50000],
            "degree_range": [4, 40], "warm_fraction": 0.3,
            "warm_started": int(sum(h.warmed for h in handles)),
            "outer_iterations_each": iters, "slots": slots, "precision": "mixed",
            "solves_per_s": count / wall, "wall_s": wall,
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "p99_latency_s_n_over_20000": float(np.percentile(lat[big], 99)) if big.any()
            else None,
            "median_obj_gap_reached": float(np.median(gaps)),
            "serial_fp64_solves_per_s": 1.0 / serial,
            "serial_sample": len(cold),
            "ratio_vs_serial_fp64": (count / wall) * serial,
            "note": "the serial FP64 rate is measured on the first cold requests, whose sizes "
                    "follow the same distribution"}


def profile_case(args):
    """One untimed run of a single piece of the workload, for profiler captures."""
    import torch
    device = torch.device("cuda:0")
    torch.cuda.set_device(device)
    if args.profile_case == "spmv":
        r = spmv_gbs(device, reps=1)
        print(json.dumps({"profile_case": "spmv", "kernel_launches_timed": 1, **r}))
        return 0
    if args.profile_case == "eigsh-rgg":
        from usbs_gb300 import api, workloads as wl
        from usbs_gb300.problem import DeviceProblem, layout
        from usbs_gb300.problems import maxcut
        from usbs_gb300.rng import default_q0
        W = wl.rgg_knn_graph(10 ** 6, 6, 0)
        st = maxcut.initialize_state(W, 1)
        n = st.C.shape[0]
        prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), device)
        out = []
        for nd in (10, 10):
            t0 = time.perf_counter()
            _, _, inf = api.eigsh_smallest(n, prob, None, None, np.zeros(n), default_q0(n), nd, 32,
                                           10, 1e-7, c_scale=-1.0, precision=32, return_info=True)
            torch.cuda.synchronize()
            out.append({"ms": 1e3 * (time.perf_counter() - t0), "matvecs": inf.matvecs,
                        "phase_kcycles": inf.phase_kcycles})
        print(json.dumps({"profile_case": "eigsh-rgg", "calls": out}))
        return 0
    from usbs_gb300 import solver
    from usbs_gb300.problems import maxcut
    from usbs_gb300.rng import default_q0
    W = workload(0)
    st = maxcut.initialize_state(W, SETTINGS["sketch_dim"])
    n = st.C.shape[0]
    inst = solver.DeviceInstance(st, device)
    out, info = run_usbs(st, n, args.iters_per_step, inst, device, q0=default_q0(n))
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "usbs", "iterations": info["iterations"],
                      "lanczos_launches": info["lanczos_launches"],
                      "kernel_launches": info["kernel_launches"]}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--iters-per-step", type=int, default=10)
    ap.add_argument("--cpu-iters", type=int, default=24)
    ap.add_argument("--no-spmv", action="store_true")
    ap.add_argument("--no-solves", action="store_true",
                    help="skip the solves-to-a-gap leg (the main line is unchanged)")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving, QAP and batched-eigsh legs (the main line is unchanged)")
    ap.add_argument("--profile-case", choices=["usbs", "spmv", "eigsh-rgg"], default=None,
                    help="run one piece of the workload once, untimed (for ncu captures): "
                         "'usbs' = --iters-per-step outer iterations on the torus instance, "
                         "'spmv' = the RGG operator apply, "
                         "'eigsh-rgg' = two FP32 eigsh calls (team kernel) on the 10^6-node RGG")
    args = ap.parse_args()
    if args.profile_case:
        return profile_case(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from usbs_gb300.problems import maxcut
    S = SETTINGS

    if args.impl == "reference":
        if rank != 0:
            return 0
        W = workload(0)
        st = maxcut.initialize_state(W, S["sketch_dim"])
        n = st.C.shape[0]
        per = args.iters_per_step
        for _ in range(args.warmup):
            cpu_oracle_iterations(st, n, per)
        tot_it, tot_s = 0, 0.0
        for _ in range(args.steps):
            it, sec = cpu_oracle_iterations(st, n, per)
            tot_it += it
            tot_s += sec
        v = tot_it / tot_s
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": main_config(per),
                "solves": {"oracle": oracle_solve_rates()},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": blas_threads(),
                                 "kind": "port",
                                 "sample": f"{args.steps} x {per} outer iterations of the NumPy "
                                           "oracle restatement (JAX reference not installed; "
                                           "BLAS multithreaded, the rest one thread)"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    from usbs_gb300 import solver
    from usbs_gb300.problem import DeviceProblem, layout
    from usbs_gb300.rng import default_q0

    W = workload(rank)
    st = maxcut.initialize_state(W, S["sketch_dim"])
    n = st.C.shape[0]
    q0 = default_q0(n)
    inst = solver.DeviceInstance(st, device)
    # device-resident state for the value leg
    st_dev = st._replace(y=torch.as_tensor(st.y, device=device),
                         z=torch.as_tensor(st.z, device=device),
                         P=torch.as_tensor(st.P, device=device),
                         Omega=torch.as_tensor(st.Omega, device=device))
    q0_dev = torch.as_tensor(q0, device=device)
    it_step = args.iters_per_step
    # L2 flush before every timed step: a 256 MB write (the L2 holds 129 MB),
    # on the solver's stream, inside the timed region (about 40 us a step)
    l2_flush = torch.empty(256 * 2 ** 20, dtype=torch.uint8, device=device)
    for _ in range(args.warmup):
        run_usbs(st_dev, n, it_step, inst, device, q0=q0_dev)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    infos = []
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            l2_flush.zero_()
            out, info = run_usbs(st_dev, n, it_step, inst, device, q0=q0_dev)
            infos.append(info)
        e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    iters_done = sum(i["iterations"] for i in infos)
    ms_max, value = replica_throughput(ms, iters_done, world, device)
    lz_ms = sum(i["lanczos_ms"] for i in infos)
    lz_n = sum(i["lanczos_launches"] for i in infos)
    lz_bytes = sum(i["lanczos_bytes"] for i in infos)
    launches = sum(i["kernel_launches"] for i in infos)
    peak, peak_kind = peaks()
    from usbs_gb300 import _lib as ulib
    on_cluster = ulib.load().usbs_lanczos_kernel(n, S["lanczos_inner_iterations"], 32) == 1
    lz_kernel = LANCZOS_KERNELS[ulib.load().usbs_lanczos_kernel(n, S["lanczos_inner_iterations"], 32)]
    # DRAM bytes per launch of that kernel on this workload, from one ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum of the first outer iteration's
    # launch; the summary and command are kept with the profiles)
    lz_traffic = LANCZOS_CLUSTER_TRAFFIC_TORUS100 if on_cluster else None
    achieved = (lz_bytes / max(lz_n, 1)) / ((lz_ms / max(lz_n, 1)) * 1e-3) / 1e9 if lz_n else 0.0
    step_chain = None
    if on_cluster:
        try:
            step_chain = lanczos_step_chain(inst, st, n)
        except Exception as exc:  # the main line is still reported
            step_chain = {"error": str(exc)[:200]}

    # e2e: public API from pinned host buffers (problem layout + state in, result out)
    host = inst.problem.host
    pinned = {f: torch.from_numpy(np.ascontiguousarray(getattr(host, f))).pin_memory()
              for f in DeviceProblem.FIELDS}
    st_pin = st._replace(y=torch.from_numpy(st.y).pin_memory(),
                         z=torch.from_numpy(st.z).pin_memory(),
                         P=torch.from_numpy(st.P).pin_memory(),
                         Omega=torch.from_numpy(st.Omega).pin_memory())
    for f in ("b", "mask", "scale_a"):
        pinned[f] = getattr(inst, f).cpu().pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in pinned.values())
    h2d += sum(t.numel() * t.element_size() for t in (st_pin.y, st_pin.z, st_pin.P, st_pin.Omega))
    d2h = 0
    torch.cuda.synchronize()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    e2e_iters = 0
    for _ in range(args.steps):
        l2_flush.zero_()
        inst_e = solver.DeviceInstance.__new__(solver.DeviceInstance)
        inst_e.__dict__.update(inst.__dict__)
        prob = DeviceProblem.__new__(DeviceProblem)
        prob.__dict__.update({k: v for k, v in inst.problem.__dict__.items()
                              if k not in DeviceProblem.FIELDS})
        for f in DeviceProblem.FIELDS:
            setattr(prob, f, pinned[f].to(device, non_blocking=True))
        for f in ("b", "mask", "scale_a"):
            setattr(inst_e, f, pinned[f].to(device, non_blocking=True))
        inst_e.problem = prob
        out, info = run_usbs(st_pin, n, it_step, inst_e, device, q0=q0)
        y_h, z_h, P_h = out.y.cpu(), out.z.cpu(), out.P.cpu()
        d2h = (y_h.numel() + z_h.numel() + P_h.numel()) * 8
        e2e_iters += info["iterations"]
    e3.record()
    torch.cuda.synchronize()
    e2e_ms = e2.elapsed_time(e3)
    _, e2e_value = replica_throughput(e2e_ms, e2e_iters, world, device)

    spmv = None
    if rank == 0 and not args.no_spmv:
        try:
            spmv = spmv_gbs(device)
            spmv["frac_of_" + peak_kind] = spmv["gbs"] / peak
        except Exception as exc:  # the main line is still reported
            spmv = {"error": str(exc)[:200]}

    qapl = None
    if rank == 0 and not args.no_serving:
        try:
            qapl = qap_leg(device)
        except Exception as exc:  # the main line is still reported
            qapl = {"error": str(exc)[:200]}

    batched = None
    if rank == 0 and not args.no_serving:
        try:
            batched = eigsh_batched_leg(device)
        except Exception as exc:  # the main line is still reported
            batched = {"error": str(exc)[:200]}

    serving = None
    if rank == 0 and not args.no_serving:
        try:
            serving = serving_leg(device)
        except Exception as exc:  # the main line is still reported
            serving = {"error": str(exc)[:200]}

    # the same steps on the plain FP64 device path (precision-matched with the
    # FP64 reference arm), timed the same way
    for _ in range(args.warmup):
        run_usbs(st_dev, n, it_step, inst, device, precision=64, q0=q0_dev)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e4.record()
    fp64_iters = 0
    for _ in range(args.steps):
        l2_flush.zero_()
        _, info = run_usbs(st_dev, n, it_step, inst, device, precision=64, q0=q0_dev)
        fp64_iters += info["iterations"]
    e5.record()
    torch.cuda.synchronize()
    _, fp64_value = replica_throughput(e4.elapsed_time(e5), fp64_iters, world, device)

    solves = errors = None
    if rank == 0 and not args.no_solves:
        try:
            solves = {"device": solves_leg(device), "oracle": oracle_solve_rates()}
        except Exception as exc:  # the main line is still reported
            solves = {"error": str(exc)[:200]}
    trajectory = None
    if rank == 0:
        # the first outer iterations on this instance (same start vector) against
        # the FP64 oracle: largest relative difference over the traced values
        trajectory = trajectory_vs_oracle(st, n, device, q0, 3)
        # the solution's errors against the FP64 oracle's, on an instance that
        # both solve to the reference's stop test at 1e-4
        if solves and "device" in solves:
            rec = solves["device"].get("er60_1e-4", {})
            errors = {"instance": "er60 to 1e-4 (tests/golden/oracle_solves.json)",
                      **{p: rec[p]["errors_vs_oracle"] for p in ("fp64", "fp32") if p in rec}}

    stream_serving = None
    if rank == 0 and not args.no_serving:
        try:
            stream_serving = serving_stream_leg(device)
        except Exception as exc:  # the main line is still reported
            stream_serving = {"error": str(exc)[:200]}

    cpu = None
    if rank == 0:
        it, sec = cpu_oracle_iterations(st, n, args.cpu_iters)
        cpu = {"value": it / sec, "unit": UNIT, "cores": blas_threads(), "kind": "port",
               "sample": f"{it} outer iterations of the NumPy oracle restatement on the "
                         f"100x100 torus ({sec:.1f} s; JAX reference not installed; BLAS "
                         f"multithreaded, the rest one thread)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 Lanczos / f64 subproblems", "data": "synthetic",
            "config": main_config(it_step),
            "fp64": {"value": fp64_value, "unit": UNIT, "dtype": "f64",
                     "note": "the same timed steps on the plain FP64 device path"},
            "errors_vs_oracle": errors,
            "trajectory_vs_oracle": trajectory,
            "solves": solves,
            "roofline": {"kernel": lz_kernel, "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "launches": lz_n, "ms_per_launch": lz_ms / max(lz_n, 1),
                         "alg_bytes_per_launch": lz_bytes / max(lz_n, 1),
                         "traffic": lz_traffic,
                         "step_chain": step_chain,
                         "note": "the cluster kernel keeps the basis, work vectors and operator "
                                 "in shared memory, so the algorithmic (streaming) bytes never "
                                 "reach DRAM; it is bound by the latency of its step chain"
                         if lz_kernel.startswith("lanczos_cluster") else None},
            "lanczos_spmv_rgg1m": spmv,
            "qap_l30": qapl,
            "eigsh_batched_48": batched,
            "serving": serving,
            "serving_stream_1024": stream_serving,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "wall_s": wall,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
