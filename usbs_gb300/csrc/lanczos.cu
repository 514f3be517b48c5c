// Thick-restart Lanczos (smallest eigenpairs) as one cooperative launch.
//
// Reference: solver/lanczos.py:80-236 (restart loop, CGS2 full
// reorthogonalisation, arrowhead projected matrix, gap-ratio restart choice).
//
// Layout and schedule.  The CTAs of the launch are split into teams, one team
// per problem.  A team owns a contiguous range of 256-row tiles of its problem;
// every phase below walks the same tiles, so a CTA only ever reads and writes
// its own rows of Q and of the work vectors, except for the SpMV gathers of x
// (read through L2 with ld.global.cg after a team barrier).  One Lanczos step i
// is three phases separated by team barriers:
//   A  y = Op x  (CSR, `lanes` threads per row) fused with h1 = Q[:, :i+1]^T y
//   B  q1 = y - Q h1, fused with h2 = Q^T q1
//   C  q2 = q1 - Q h2, fused with ||q2||^2
// The normalisation q2 / beta is folded into the next phase A (x = v * 1/beta),
// which also stores Q[:, i+1] for its rows.  Partial sums go to a per-team
// [pass][cta][column] buffer and every CTA reduces them in the same fixed order,
// so all CTAs hold bit-identical alpha/beta and take identical branches.
// At a restart CTA 0 builds the arrowhead matrix and runs the FP64 warp
// eigensolver; after a barrier every CTA rotates its rows of Q by the saved
// Ritz vectors.
#include <stdlib.h>
#include <map>
#include <mutex>
#include "common.cuh"
#include "dense.cuh"
#include "internal.h"

namespace usbs {

constexpr int LZ_BLOCK = 256;
constexpr int LZ_NW = LZ_BLOCK / 32;
constexpr int MAX_TEAMS = 48;
constexpr int MP1 = MAXM + 1;

constexpr int LZ_XS_BYTES = 160 * 1024;   // dynamic shared memory for a staged x

template <typename VT>
struct TeamDesc {
  int n, ld, m, num_desired, max_restarts, lanes, first_cta, nctas, xsmem;
  int stages;            // non-zero: phases stream Q tiles through shared memory (bulk copies)
  int stage_csr;         // the stages also carry each tile's CSR slice (phase A)
  int stg_budget;        // bytes of the stage area (a multiple of 128)
  int stg_cap;           // CSR slice capacity (entries, a multiple of 64)
  long long nnz;
  double tol;
  const int* rowptr;
  const int* col;
  const VT* val;
  VT* Q;                 // the caller's basis, ld x (m+1) column-major
  // working basis: element (c, row) at Qw[qix(c, row)].  Staged teams keep it
  // tile-major in the workspace (each 256-row tile's m+1 columns contiguous,
  // so one bulk copy moves a tile's active columns); otherwise it is Q.
  VT* Qw;
  long long qts, qcs;    // tile and column strides (elements)
  VT* vbuf;              // 3 flat vectors: two work vectors, then Q[:, k] of the cycle
  double* part;
  double* Ybuf;
  double* alpha;
  double* beta;
  int* ctl;
  unsigned int* bar;
  int* status;
};

template <typename VT>
__device__ __forceinline__ size_t qix(const TeamDesc<VT>& P, int c, int row) {
  return (size_t)(row / LZ_BLOCK) * (size_t)P.qts + (size_t)c * (size_t)P.qcs +
         (size_t)(row % LZ_BLOCK);
}

template <typename VT>
struct TeamBatch {
  int count;
  TeamDesc<VT> t[MAX_TEAMS];
};

template <typename VT>
struct LzShared {
  union {
    struct {                     // Lanczos step phases
      double ys[LZ_BLOCK];
      double wred[LZ_NW][MP1];
    } st;
    struct {                     // restart on CTA 0 (T, X, R, S, W row-major, ld MP1)
      double T[MAXM * MP1];
      double X[MAXM * MP1];
      double R[MAXM * MP1];      // float copy of T during the Jacobi sweeps
      double S[MAXM * MP1];      // float eigenvectors during the Jacobi sweeps
      double W[MAXM * MP1];
    } rs;
    VT Ys[MAXM * MAXM];          // saved Ritz vectors, every CTA, after the restart barrier
  } u;
  double h[MP1];
  VT hv[MP1];                    // h in the vector type, converted once per reduction
  double alpha[MAXM];
  double beta[MAXM];
  double ritz[MAXM];
  double red[LZ_NW];
  float wf[MAXM], rc[MAXM / 2], rsn[MAXM / 2], redf[32];
  int pidx[MAXM];
  int order[MAXM];
  int k_next, nconv;
  long long eig_cycles;          // cycles in the projected eigensolver (thread 0)
};

// acc[c] (c < nv) summed over the CTA, written to out[c * R] (column-major
// [column][cta] partial layout, so the team reduction reads each column in one
// coalesced load).  Columns 0..31 are reduced across each warp by one
// butterfly reduce-scatter (lane c ends with column c), column 32 by a warp sum.
template <typename VT, typename AT>
__device__ __forceinline__ void block_reduce_cols(AT* acc, int nv, LzShared<VT>& sh, double* out,
                                                  int R) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (nv == 1) {
    const AT v = warp_sum(acc[0]);
    if (lane == 0) sh.u.st.wred[wid][0] = (double)v;
  } else {
    const AT extra = (nv > 32) ? warp_sum(acc[32]) : (AT)0;
    const AT v = warp_reduce_scatter32(acc);
    sh.u.st.wred[wid][lane] = (double)v;
    if (lane == 0 && nv > 32) sh.u.st.wred[wid][32] = (double)extra;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < LZ_NW; ++w) s += sh.u.st.wred[w][c];
    out[(size_t)c * R] = s;
  }
}

// h[c] = sum over the team's CTAs of part_pass[c][r], identical order in every
// CTA.  Warp 0 issues all loads (lane l takes CTAs l, l+32, ...), then one
// butterfly reduce-scatter leaves column c in lane c.
template <typename VT>
__device__ __forceinline__ void reduce_part(const double* part_pass, int R, int nv,
                                            LzShared<VT>& sh) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    if (nv == 1) {
      double a = 0.0;
      for (int r = lane; r < R; r += 32) a += __ldcg(part_pass + r);
      a = warp_sum(a);
      if (lane == 0) { sh.h[0] = a; sh.hv[0] = (VT)a; }
    } else {
      double acc[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) acc[c] = 0.0;
      double extra = 0.0;
      for (int r = lane; r < R; r += 32) {
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c < nv) acc[c] += __ldcg(part_pass + (size_t)c * R + r);
        if (nv > 32) extra += __ldcg(part_pass + (size_t)32 * R + r);
      }
      extra = warp_sum(extra);
      const double v = warp_reduce_scatter32(acc);
      if (lane < nv) { sh.h[lane] = v; sh.hv[lane] = (VT)v; }
      if (lane == 0 && nv > 32) { sh.h[32] = extra; sh.hv[32] = (VT)extra; }
    }
  }
  __syncthreads();
}

// SpMV of one 256-row tile, L lanes per row: sh.u.st.ys[r] = (Op x)[base + r].
// Groups of up to 4 passes issue their rowptr loads, then their first col/val
// loads, before any result is used: two dependent L2 round trips per group
// instead of two per pass.
template <typename VT, int L>
__device__ __forceinline__ void spmv_tile(const TeamDesc<VT>& P, LzShared<VT>& sh, int base,
                                          const VT* xsrc, const VT* xs, bool use_xs) {
  typedef typename Acc<VT>::type AT;
  constexpr int GPP = LZ_BLOCK / L;
  constexpr int CH = L < 4 ? L : 4;          // passes whose loads are issued together
  const int tid = threadIdx.x, g = tid / L, lig = tid - (tid / L) * L;
#pragma unroll 1
  for (int q0 = 0; q0 < L; q0 += CH) {
    int pb[CH], pe[CH];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      const int row = base + (q0 + q) * GPP + g;
      pb[q] = 0; pe[q] = 0;
      if (row < P.n) { pb[q] = P.rowptr[row] + lig; pe[q] = P.rowptr[row + 1]; }
    }
    int c0[CH];
    VT v0[CH];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      c0[q] = 0; v0[q] = (VT)0;
      if (pb[q] < pe[q]) { c0[q] = P.col[pb[q]]; v0[q] = P.val[pb[q]]; }
    }
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      AT s = (AT)v0[q] * (AT)(use_xs ? xs[c0[q]] : __ldcg(xsrc + c0[q]));
      for (int p = pb[q] + L; p < pe[q]; p += L)
        s += (AT)P.val[p] * (AT)(use_xs ? xs[P.col[p]] : __ldcg(xsrc + P.col[p]));
#pragma unroll
      for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lig == 0) sh.u.st.ys[(q0 + q) * GPP + g] = (double)s;
    }
  }
}

// Phase A: y = Op (xsrc * xscale) for own rows -> vout, acc[c] = Q[:, c] . y (c <= i).
// If wq, also stores Q[:, i] = xsrc * xscale for own rows.
template <typename VT>
__device__ void phase_spmv(const TeamDesc<VT>& P, LzShared<VT>& sh, int t0, int t1, int i,
                           const VT* xsrc, VT xscale, bool wq, VT* vout, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const int tid = threadIdx.x, L = P.lanes, gpp = LZ_BLOCK / L;
  const int g = tid / L, lig = tid - g * L;
  const size_t ld = (size_t)P.ld;
  // small vectors: stage x once in shared memory so the gathers skip L2
  extern __shared__ __align__(16) unsigned char lz_dyn[];
  VT* xs = (VT*)lz_dyn;
  const bool use_xs = P.xsmem != 0;
  if (use_xs) {
    // 16-byte loads, several in flight per thread (xsrc is a 256-byte aligned
    // vector buffer or a column of Q with ld a multiple of 32)
    constexpr int VE = 16 / (int)sizeof(VT);
    const int n16 = P.n / VE;
    const uint4* src = (const uint4*)xsrc;
    uint4* dst = (uint4*)xs;
    int j = tid;
    for (; j + 3 * LZ_BLOCK < n16; j += 4 * LZ_BLOCK) {
      const uint4 a = __ldcg(src + j), b = __ldcg(src + j + LZ_BLOCK),
                  c = __ldcg(src + j + 2 * LZ_BLOCK), d = __ldcg(src + j + 3 * LZ_BLOCK);
      dst[j] = a; dst[j + LZ_BLOCK] = b; dst[j + 2 * LZ_BLOCK] = c; dst[j + 3 * LZ_BLOCK] = d;
    }
    for (; j < n16; j += LZ_BLOCK) dst[j] = __ldcg(src + j);
    for (int r = n16 * VE + tid; r < P.n; r += LZ_BLOCK) xs[r] = __ldcg(xsrc + r);
    __syncthreads();
  }
  (void)gpp; (void)g; (void)lig;
  for (int tile = t0; tile < t1; ++tile) {
    const int base = tile * LZ_BLOCK;
    switch (L) {
      case 1: spmv_tile<VT, 1>(P, sh, base, xsrc, xs, use_xs); break;
      case 2: spmv_tile<VT, 2>(P, sh, base, xsrc, xs, use_xs); break;
      case 4: spmv_tile<VT, 4>(P, sh, base, xsrc, xs, use_xs); break;
      case 8: spmv_tile<VT, 8>(P, sh, base, xsrc, xs, use_xs); break;
      case 16: spmv_tile<VT, 16>(P, sh, base, xsrc, xs, use_xs); break;
      default: spmv_tile<VT, 32>(P, sh, base, xsrc, xs, use_xs); break;
    }
    __syncthreads();
    const int row = base + tid;
    if (row < P.n) {
      const VT y = (VT)sh.u.st.ys[tid] * xscale;
      vout[row] = y;
      VT xn = (VT)0;
      if (wq) {
        xn = __ldcg(xsrc + row) * xscale;
        P.Qw[qix(P, i, row)] = xn;
      }
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c <= i) {
          const VT qc = (wq && c == i) ? xn : P.Qw[qix(P, c, row)];
          acc[c] += (AT)qc * (AT)y;
        }
      }
    }
    __syncthreads();
  }
  block_reduce_cols(acc, i + 1, sh, part_out, P.nctas);
}

// ---------------------------------------------------------------- staged tiles
// Large problems (x not staged in shared memory): each phase streams its
// tiles' rows of the needed Q columns and of one work vector into shared
// memory with bulk async copies issued by thread 0, `stages` tiles ahead, so
// a CTA reads its rows of the basis at streaming rate instead of one DRAM
// round trip per tile.  The stage layout is planned per phase: the staged Q
// columns, then the work vector, then (phase A, FP32) the tile's CSR slice,
// so a phase that streams few columns keeps more tiles in flight.
constexpr int STG_MAXS = 8;     // mbarriers, i.e. the deepest pipeline
constexpr int STG_CAP = 4096;   // largest CSR slice (entries) a stage can carry
struct StgHdr {
  int rcnt;       // staged rowptr entries (from the tile's first row)
  int p0;         // first entry of the tile
  int ca0, ca1;   // staged col range [ca0, ca1)
  int va0, va1;   // staged val range [va0, va1)
  int pad[2];
};
// bytes of a stage's CSR slice part (rowptr, col, val, header) for `cap` entries
template <typename VT>
__host__ __device__ constexpr unsigned stg_csr_bytes(int cap) {
  return (unsigned)(((LZ_BLOCK + 4) * 4 + (cap + 8) * 4 + (cap + 8) * (int)sizeof(VT) +
                     (int)sizeof(StgHdr) + 127) / 128 * 128);
}
// bytes of the Q part of a stage: `cols` columns of LZ_BLOCK values
template <typename VT>
__host__ __device__ constexpr unsigned stg_q_bytes(int cols) {
  return (unsigned)cols * LZ_BLOCK * (unsigned)sizeof(VT);
}

template <typename VT>
struct Stager {
  unsigned char* base;   // the stage area, `budget` bytes
  uint64_t* bar;         // STG_MAXS mbarriers
  unsigned budget;
  int cap;               // CSR slice capacity (entries) of a phase-A stage
  int csr;               // phase A stages carry the tile's CSR slice
  // plan of the running phase (identical in every thread)
  unsigned bytes;        // bytes per stage
  int S;                 // stages (tiles in flight)
  int vcol;              // stage column of the work vector (= staged Q columns)
  unsigned rp, col, val, hdr;   // CSR slice offsets inside a stage
  int nx_p0, nx_p1;      // thread 0: entry range of the next tile to issue (prefetched)
  unsigned ph;           // parity of each mbarrier's next phase (identical in every thread)
  __device__ VT* stage(int s) const { return (VT*)(base + (size_t)s * bytes); }
  __device__ unsigned char* raw(int s) const { return base + (size_t)s * bytes; }
};

// stage layout and depth of a phase streaming `ncols` Q columns (+ the work
// vector, + the CSR slice); the host sizes `budget` for two of the largest
template <typename VT>
__device__ __forceinline__ void stg_plan(Stager<VT>& G, int ncols, bool vec, bool csr) {
  G.vcol = ncols;
  const unsigned qb = stg_q_bytes<VT>(ncols + (vec ? 1 : 0));
  G.rp = qb;
  G.col = G.rp + (LZ_BLOCK + 4) * 4;
  G.val = G.col + (unsigned)(G.cap + 8) * 4;
  G.hdr = G.val + (unsigned)(G.cap + 8) * (unsigned)sizeof(VT);
  G.bytes = csr ? qb + stg_csr_bytes<VT>(G.cap) : qb;
  int S = (int)(G.budget / G.bytes);
  G.S = S > STG_MAXS ? STG_MAXS : (S < 1 ? 1 : S);
}

// warp 0: rows of tile `tile` of Q[:, 0:ncols] and, if vec, of vec into stage
// s; lane 0 arms the stage's mbarrier with the byte count, then the lanes
// issue the copies in parallel (copy j by lane j mod 32)
template <typename VT>
__device__ void stg_issue(const TeamDesc<VT>& P, Stager<VT>& G, int s, int tile, int ncols,
                          const VT* vec, bool csr = false) {
  constexpr int E16 = 16 / (int)sizeof(VT);
  const int lane = threadIdx.x & 31;
  const int r0 = tile * LZ_BLOCK;
  const int rows = min(LZ_BLOCK, P.n - r0);
  // ld is a multiple of 32 >= n, so the padded rows stay inside each column
  const unsigned bytes = (unsigned)(((rows + E16 - 1) / E16) * E16 * (int)sizeof(VT));
  VT* st = G.stage(s);
  unsigned tx = stg_q_bytes<VT>(ncols) + (vec ? bytes : 0u);
  // CSR slice of the tile (phase A of FP32 stages): rowptr[r0 ..], col and val
  // over [p0, p1), each widened to 16-byte boundaries inside its array; the
  // few elements past an array's last full 16-byte block, and every entry of
  // a tile larger than STG_CAP, are read from global memory by the consumers
  unsigned rb = 0, cb = 0, vb = 0;
  StgHdr h;
  if (csr) {
    const int p0 = __shfl_sync(0xffffffffu, G.nx_p0, 0);
    const int p1 = __shfl_sync(0xffffffffu, G.nx_p1, 0);
    int rcnt = (rows + 1 + 3) & ~3;
    const int rmax = ((P.n + 1) & ~3) - r0;
    if (rcnt > rmax) rcnt = rmax > 0 ? rmax : 0;
    const long long nnz = P.nnz;
    const bool fits = (p1 - p0) <= G.cap;
    int ca0 = p0 & ~3, ca1 = (p1 + 3) & ~3;
    const int cfull = (int)(nnz & ~3LL);
    if (ca1 > cfull) ca1 = cfull;
    if (!fits || ca1 < ca0) ca1 = ca0;
    int va0 = p0 & ~(E16 - 1), va1 = (p1 + E16 - 1) & ~(E16 - 1);
    const int vfull = (int)(nnz & ~(long long)(E16 - 1));
    if (va1 > vfull) va1 = vfull;
    if (!fits || va1 < va0) va1 = va0;
    h.rcnt = rcnt; h.p0 = p0; h.ca0 = ca0; h.ca1 = ca1; h.va0 = va0; h.va1 = va1;
    if (lane == 0) *(StgHdr*)(G.raw(s) + G.hdr) = h;
    rb = (unsigned)rcnt * 4u;
    cb = (unsigned)(ca1 - ca0) * 4u;
    vb = (unsigned)(va1 - va0) * (unsigned)sizeof(VT);
    tx += rb + cb + vb;
  }
  // the stage's earlier generic accesses (header, products written over the
  // values) before the async copies into it; the global data the copies read
  // was fenced by its writers before the team barrier that precedes the phase
  fence_proxy_async_smem();
  if (lane == 0) mbar_arrive_expect_tx(&G.bar[s], tx);
  __syncwarp();
  // streamed once per phase: evict_first, so the copies do not push the SpMV's
  // x (gathered with evict_last) out of L2
  const uint64_t pol = l2_evict_first_policy();
  // the tile's first ncols columns are contiguous in the tile-major basis
  // (full 256-row columns; the last tile is padded): one copy
  const int nq = ncols > 0 ? 1 : 0;
  const int ncopies = nq + (vec ? 1 : 0) + (csr ? 3 : 0);
  if (lane < ncopies) {
    const int j = lane;
    if (j < nq) {
      bulk_g2s_hint(st, P.Qw + (size_t)tile * (size_t)P.qts, stg_q_bytes<VT>(ncols), &G.bar[s],
                    pol);
    } else if (vec && j == nq) {
      bulk_g2s_hint(st + (size_t)G.vcol * LZ_BLOCK, vec + r0, bytes, &G.bar[s], pol);
    } else {
      const int k = j - nq - (vec ? 1 : 0);   // 0 rowptr, 1 col, 2 val
      if (k == 0 && rb) bulk_g2s_hint(G.raw(s) + G.rp, P.rowptr + r0, rb, &G.bar[s], pol);
      if (k == 1 && cb) bulk_g2s_hint(G.raw(s) + G.col, P.col + h.ca0, cb, &G.bar[s], pol);
      if (k == 2 && vb) bulk_g2s_hint(G.raw(s) + G.val, P.val + h.va0, vb, &G.bar[s], pol);
    }
  }
}

// thread 0: entry range of tile `tile` (loads left in flight until the next issue)
template <typename VT>
__device__ __forceinline__ void stg_prefetch_range(const TeamDesc<VT>& P, Stager<VT>& G, int tile) {
  const int r0 = tile * LZ_BLOCK;
  G.nx_p0 = P.rowptr[r0];
  G.nx_p1 = P.rowptr[min(r0 + LZ_BLOCK, P.n)];
}

// body(tile, stage) for tiles [t0, t1), copies pipelined `stages` deep.  On a
// wait that runs past its limit: records ST_BARRIER_TIMEOUT, waits (bounded)
// for the copies still in flight and returns false; the CTA then leaves at
// its next team barrier.
template <typename VT, typename F>
__device__ bool stg_loop(const TeamDesc<VT>& P, Stager<VT>& G, int t0, int t1, int ncols,
                         const VT* vec, F&& body, bool csr = false) {
  const uint64_t LIMIT = 1000000000ull;
  stg_plan(G, ncols, vec != nullptr, csr);
  const int S = G.S;
  if (threadIdx.x < 32) {
    for (int j = 0; j < S && t0 + j < t1; ++j) {
      if (csr && threadIdx.x == 0) stg_prefetch_range(P, G, t0 + j);
      stg_issue(P, G, j, t0 + j, ncols, vec, csr);
    }
    if (csr && threadIdx.x == 0 && t0 + S < t1) stg_prefetch_range(P, G, t0 + S);
  }
  for (int t = t0; t < t1; ++t) {
    const int s = (t - t0) % S;
    const unsigned par = (G.ph >> s) & 1u;
    const bool ok = mbar_wait(&G.bar[s], par, LIMIT);
    if (__syncthreads_or(!ok)) {
      // drain: this tile's copies and those of the later tiles already issued
      mbar_wait(&G.bar[s], par, LIMIT);
      G.ph ^= (1u << s);
      for (int tt = t + 1; tt < t1 && tt < t + S; ++tt) {
        const int s2 = (tt - t0) % S;
        mbar_wait(&G.bar[s2], (G.ph >> s2) & 1u, LIMIT);
        G.ph ^= (1u << s2);
      }
      if (threadIdx.x == 0) atomicOr(P.status, ST_BARRIER_TIMEOUT);
      __syncthreads();
      return false;
    }
    G.ph ^= (1u << s);
    body(t, s);
    __syncthreads();
    if (threadIdx.x < 32 && t + S < t1) {
      stg_issue(P, G, s, t + S, ncols, vec, csr);
      if (csr && threadIdx.x == 0 && t + S + 1 < t1) stg_prefetch_range(P, G, t + S + 1);
    }
  }
  return true;
}

// SpMV of one 256-row tile from its staged CSR slice (rowptr, col, val in
// shared memory; x gathered from global memory), L lanes per row, groups of up
// to 4 passes as in spmv_tile
template <typename VT, int L>
__device__ __forceinline__ void spmv_tile_stg(const TeamDesc<VT>& P, LzShared<VT>& sh,
                                              const Stager<VT>& G, int base,
                                              const unsigned char* stg, const VT* xsrc) {
  typedef typename Acc<VT>::type AT;
  constexpr int GPP = LZ_BLOCK / L;
  constexpr int CH = L < 4 ? L : 4;
  const StgHdr h = *(const StgHdr*)(stg + G.hdr);
  const int* rp = (const int*)(stg + G.rp);
  const int* cs = (const int*)(stg + G.col);
  VT* vs = (VT*)(stg + G.val);
  const int tid = threadIdx.x, g = tid / L, lig = tid - (tid / L) * L;
  const int rows = min(LZ_BLOCK, P.n - base);
  // fully staged tile: every product v x[c] of the tile at once (about nnz /
  // 256 independent gathers per thread), written over its own value in the
  // stage, then one thread per row sums its row's products
  if (rows + 1 <= h.rcnt) {
    const int p0 = rp[0], p1 = rp[rows];
    if (p1 <= h.ca1 && p1 <= h.va1) {
      const uint64_t keep = l2_evict_last_policy();
      constexpr int U = 16;   // one round of gathers for slices up to STG_CAP entries
      for (int pb = p0 + tid; pb < p1; pb += U * LZ_BLOCK) {
        int c[U];
        VT xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int p = pb + u * LZ_BLOCK;
          c[u] = (p < p1) ? cs[p - h.ca0] : 0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = ldcg_pol(xsrc + c[u], keep);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int p = pb + u * LZ_BLOCK;
          if (p < p1) vs[p - h.va0] = vs[p - h.va0] * xv[u];
        }
      }
      fence_proxy_async_smem();   // the stage is refilled by bulk copies later
      __syncthreads();
      if (tid < rows) {
        AT sacc = (AT)0;
        const int e = rp[tid + 1];
        for (int p = rp[tid]; p < e; ++p) sacc += (AT)vs[p - h.va0];
        sh.u.st.ys[tid] = (double)sacc;
      }
      return;
    }
  }
  auto colv = [&](int p, int& c, VT& v) {
    c = (p < h.ca1) ? cs[p - h.ca0] : P.col[p];
    v = (p < h.va1) ? vs[p - h.va0] : P.val[p];
  };
#pragma unroll 1
  for (int q0 = 0; q0 < L; q0 += CH) {
    int pb[CH], pe[CH];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      const int lr = (q0 + q) * GPP + g;
      const int row = base + lr;
      pb[q] = 0; pe[q] = 0;
      if (row < P.n) {
        pb[q] = ((lr < h.rcnt) ? rp[lr] : P.rowptr[row]) + lig;
        pe[q] = (lr + 1 < h.rcnt) ? rp[lr + 1] : P.rowptr[row + 1];
      }
    }
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      AT s = (AT)0;
      for (int p = pb[q]; p < pe[q]; p += L) {
        int c;
        VT v;
        colv(p, c, v);
        s += (AT)v * (AT)__ldcg(xsrc + c);
      }
#pragma unroll
      for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lig == 0) sh.u.st.ys[(q0 + q) * GPP + g] = (double)s;
    }
  }
}

// staged phase A: as phase_spmv, with Q[:, c] (and xsrc's own rows) from the stage
template <typename VT>
__device__ void stg_phase_spmv(const TeamDesc<VT>& P, LzShared<VT>& sh, Stager<VT>& G, int t0,
                               int t1, int i, const VT* xsrc, VT xscale, bool wq, VT* vout,
                               double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const int tid = threadIdx.x, L = P.lanes;
  const size_t ld = (size_t)P.ld;
  const int ncols = wq ? i : i + 1;
  const bool csr = G.csr != 0;
  stg_loop(P, G, t0, t1, ncols, wq ? xsrc : nullptr, [&](int tile, int sidx) {
    const VT* stq = G.stage(sidx);
    const int base = tile * LZ_BLOCK;
    if (csr) {
      const unsigned char* stg = G.raw(sidx);
      switch (L) {
        case 1: spmv_tile_stg<VT, 1>(P, sh, G, base, stg, xsrc); break;
        case 2: spmv_tile_stg<VT, 2>(P, sh, G, base, stg, xsrc); break;
        case 4: spmv_tile_stg<VT, 4>(P, sh, G, base, stg, xsrc); break;
        case 8: spmv_tile_stg<VT, 8>(P, sh, G, base, stg, xsrc); break;
        case 16: spmv_tile_stg<VT, 16>(P, sh, G, base, stg, xsrc); break;
        default: spmv_tile_stg<VT, 32>(P, sh, G, base, stg, xsrc); break;
      }
    } else {
      switch (L) {
        case 1: spmv_tile<VT, 1>(P, sh, base, xsrc, nullptr, false); break;
        case 2: spmv_tile<VT, 2>(P, sh, base, xsrc, nullptr, false); break;
        case 4: spmv_tile<VT, 4>(P, sh, base, xsrc, nullptr, false); break;
        case 8: spmv_tile<VT, 8>(P, sh, base, xsrc, nullptr, false); break;
        case 16: spmv_tile<VT, 16>(P, sh, base, xsrc, nullptr, false); break;
        default: spmv_tile<VT, 32>(P, sh, base, xsrc, nullptr, false); break;
      }
    }
    __syncthreads();
    const int row = base + tid;
    if (row < P.n) {
      const VT y = (VT)sh.u.st.ys[tid] * xscale;
      vout[row] = y;
      VT xn = (VT)0;
      if (wq) {
        xn = stq[(size_t)G.vcol * LZ_BLOCK + tid] * xscale;
        P.Qw[qix(P, i, row)] = xn;
      }
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c <= i) {
          const VT qc = (wq && c == i) ? xn : stq[(size_t)c * LZ_BLOCK + tid];
          acc[c] += (AT)qc * (AT)y;
        }
      }
    }
  }, csr);
  block_reduce_cols(acc, i + 1, sh, part_out, P.nctas);
}

// staged phase B: buf -= Q h (c < nv); acc[c] = Q[:, c] . buf
template <typename VT>
__device__ void stg_phase_update_dot(const TeamDesc<VT>& P, LzShared<VT>& sh, Stager<VT>& G,
                                     int t0, int t1, int nv, VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const int tid = threadIdx.x;
  stg_loop(P, G, t0, t1, nv, buf, [&](int tile, int sidx) {
    const VT* stq = G.stage(sidx);
    const int row = tile * LZ_BLOCK + tid;
    if (row < P.n) {
      VT qr[MP1];
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c < nv) {
          qr[c] = stq[(size_t)c * LZ_BLOCK + tid];
          s += qr[c] * sh.hv[c];
        }
      }
      const VT q1 = stq[(size_t)G.vcol * LZ_BLOCK + tid] - s;
      buf[row] = q1;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) acc[c] += (AT)qr[c] * (AT)q1;
    }
  });
  block_reduce_cols(acc, nv, sh, part_out, P.nctas);
}

// staged phase C: buf -= Q h (c < nv); part_out[0] = sum buf^2 over own rows
template <typename VT>
__device__ void stg_phase_update_norm(const TeamDesc<VT>& P, LzShared<VT>& sh, Stager<VT>& G,
                                      int t0, int t1, int nv, VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT nrm = (AT)0;
  const int tid = threadIdx.x;
  stg_loop(P, G, t0, t1, nv, buf, [&](int tile, int sidx) {
    const VT* stq = G.stage(sidx);
    const int row = tile * LZ_BLOCK + tid;
    if (row < P.n) {
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) s += stq[(size_t)c * LZ_BLOCK + tid] * sh.hv[c];
      const VT q2 = stq[(size_t)G.vcol * LZ_BLOCK + tid] - s;
      buf[row] = q2;
      nrm += (AT)q2 * (AT)q2;
    }
  });
  AT one[MP1];
  one[0] = nrm;
  block_reduce_cols(one, 1, sh, part_out, P.nctas);
}

// Breakdown pass a: buf = hash_normal(key) for own rows, acc[c] = Q[:, c] . buf (c < nv)
template <typename VT>
__device__ void phase_random(const TeamDesc<VT>& P, LzShared<VT>& sh, int t0, int t1, int nv,
                             uint64_t key, VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      const VT r = (VT)hash_normal(key, (uint64_t)row);
      buf[row] = r;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) acc[c] += (AT)P.Qw[qix(P, c, row)] * (AT)r;
    }
  }
  block_reduce_cols(acc, nv, sh, part_out, P.nctas);
}

// Phase B: buf -= Q h (c < nv); acc[c] = Q[:, c] . buf
template <typename VT>
__device__ void phase_update_dot(const TeamDesc<VT>& P, LzShared<VT>& sh, int t0, int t1, int nv,
                                 VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      VT qr[MP1];
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c < nv) {
          qr[c] = P.Qw[qix(P, c, row)];
          s += qr[c] * sh.hv[c];
        }
      }
      const VT q1 = buf[row] - s;
      buf[row] = q1;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) acc[c] += (AT)qr[c] * (AT)q1;
    }
  }
  block_reduce_cols(acc, nv, sh, part_out, P.nctas);
}

// Phase C: buf -= Q h (c < nv); part_out[0] = sum buf^2 over own rows
template <typename VT>
__device__ void phase_update_norm(const TeamDesc<VT>& P, LzShared<VT>& sh, int t0, int t1, int nv,
                                  VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT nrm = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) s += P.Qw[qix(P, c, row)] * sh.hv[c];
      const VT q2 = buf[row] - s;
      buf[row] = q2;
      nrm += (AT)q2 * (AT)q2;
    }
  }
  AT one[MP1];
  one[0] = nrm;
  block_reduce_cols(one, 1, sh, part_out, P.nctas);
}

// CTA 0 of a team: projected eigenproblem and thick-restart selection
// (solver/lanczos.py:128-168, 202-221).  k = number of saved vectors of the
// finished cycle, beta_last = beta[m-1].
// LOCAL_YS: every CTA of a cluster runs this redundantly (identical inputs give
// identical results) and keeps the saved Ritz vectors in sh.u.Ys; only the CTA
// with write_out set stores alpha/beta/ctl.  Otherwise (team kernel) the Ritz
// vectors go through P.Ybuf.
template <bool LOCAL_YS, typename VT, typename D>
__device__ void restart_select(const D& P, LzShared<VT>& sh, int k, bool write_out = true) {
  const int m = P.m, tid = threadIdx.x;
  double* T = sh.u.rs.T;
  double* X = sh.u.rs.X;
  float* Tf = (float*)sh.u.rs.R;
  float* Zf = (float*)sh.u.rs.S;
  for (int e = tid; e < m * m; e += LZ_BLOCK) {
    const int r = e / m, c = e - r * m;
    double v = 0.0;
    if (r == c) v = sh.alpha[r];
    else if (c == k && r < k) v = sh.beta[r];
    else if (r == k && c < k) v = sh.beta[c];
    else if (c == r + 1 && r >= k) v = sh.beta[r];
    else if (r == c + 1 && c >= k) v = sh.beta[c];
    T[r * MP1 + c] = v;
    Tf[r * MP1 + c] = (float)v;
  }
  __syncthreads();
  // eigh(T) (solver/lanczos.py:203): FP32 parallel Jacobi by the CTA ...
  {
    const long long c0 = clock64();
    const bool ok = cta_jacobi_f32<32>(Tf, MP1, m, sh.wf, Zf, MP1, sh.pidx, sh.rc, sh.rsn, sh.redf);
    if (tid == 0) sh.eig_cycles += clock64() - c0;
    if (!ok && tid == 0) atomicOr(P.status, ST_SMALL_DENSE_FAIL);
  }
  for (int e = tid; e < m * m; e += LZ_BLOCK) {
    const int r = e / m, c = e - r * m;
    X[r * MP1 + c] = (double)Zf[r * MP1 + c];
  }
  if (tid < m) sh.ritz[tid] = (double)sh.wf[tid];
  __syncthreads();
  if (sizeof(VT) == 8) {
    // ... refined to FP64 accuracy by two Ogita-Aishima steps, then re-sorted
    cta_refine_eig(T, X, sh.u.rs.R, sh.u.rs.S, sh.u.rs.W, sh.ritz, sh.red, m, MP1);
    cta_refine_eig(T, X, sh.u.rs.R, sh.u.rs.S, sh.u.rs.W, sh.ritz, sh.red, m, MP1);
    if (tid == 0) {
      for (int i = 0; i < m; ++i) sh.order[i] = i;
      for (int i = 0; i < m - 1; ++i) {
        int kmin = i;
        for (int j = i + 1; j < m; ++j)
          if (sh.ritz[sh.order[j]] < sh.ritz[sh.order[kmin]]) kmin = j;
        const int t = sh.order[i]; sh.order[i] = sh.order[kmin]; sh.order[kmin] = t;
      }
    }
    __syncthreads();
    double* Sx = sh.u.rs.S;
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int r = e / m, c = e - r * m;
      Sx[r * MP1 + c] = X[r * MP1 + sh.order[c]];
    }
    double rv = (tid < m) ? sh.ritz[sh.order[tid]] : 0.0;
    __syncthreads();
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int r = e / m, c = e - r * m;
      X[r * MP1 + c] = Sx[r * MP1 + c];
    }
    if (tid < m) sh.ritz[tid] = rv;
    __syncthreads();
  }
  const double* Z = X;
  if (tid == 0) {
    const double bl = sh.beta[m - 1];
    int nconv = m;
    for (int c = 0; c < m; ++c) {
      if (!(bl * fabs(Z[(m - 1) * MP1 + c]) < P.tol)) { nconv = c; break; }
    }
    const int delta = min(m - P.num_desired, 2 * (m - nconv) / 5);
    const double lt = sh.ritz[min(nconv, m - 1)];
    int kl = 0;
    double bv = 0.0;
    for (int c = 0; c < m; ++c) {
      const int kr = c + delta;
      double g = 0.0;
      if (kr <= m) g = (sh.ritz[c] - lt) / (sh.ritz[min(kr, m - 1)] - lt);
      if (c == 0) { bv = g; kl = 0; if (isnan(g)) break; continue; }
      if (isnan(g)) { kl = c; break; }
      if (g > bv) { bv = g; kl = c; }
    }
    const int kright = kl + delta;
    int kn = 0;
    for (int c = 0; c < m; ++c)
      if (kl >= c || kright < c) sh.order[kn++] = c;
    int pos = kn;
    for (int c = 0; c < m; ++c)
      if (!(kl >= c || kright < c)) sh.order[pos++] = c;
    sh.k_next = kn;
    sh.nconv = nconv;
  }
  __syncthreads();
  const int kn = sh.k_next;
  const double bl = sh.beta[m - 1];
  if constexpr (LOCAL_YS) {
    // sh.u.Ys overlays sh.u.rs.T only (T is no longer needed; Z lives in X)
    for (int e = tid; e < m * MAXM; e += LZ_BLOCK) {
      const int j = e / MAXM, c = e - j * MAXM;
      sh.u.Ys[e] = (c < kn) ? (VT)Z[j * MP1 + sh.order[c]] : (VT)0;
    }
  } else {
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int j = e / m, c = e - j * m;
      P.Ybuf[j * m + c] = Z[j * MP1 + sh.order[c]];
    }
  }
  __syncthreads();
  if (tid < m) {
    const int c = tid;
    const double a = (c < kn) ? sh.ritz[sh.order[c]] : 0.0;
    const double b = (c < kn) ? bl * Z[(m - 1) * MP1 + sh.order[c]] : 0.0;
    sh.alpha[c] = a;
    sh.beta[c] = b;
    if (write_out) {
      P.alpha[c] = a;
      P.beta[c] = b;
    }
  }
  if (tid == 0 && write_out) {
    P.ctl[0] = kn;
    P.ctl[1] = sh.nconv;
  }
  __syncthreads();
}

template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 1)
lanczos_team_kernel(const __grid_constant__ TeamBatch<VT> batch) {
  __shared__ LzShared<VT> sh;
  int team = 0;
  for (int t = 1; t < batch.count; ++t)
    if ((int)blockIdx.x >= batch.t[t].first_cta) team = t;
  const TeamDesc<VT>& P = batch.t[team];
  const int rank = (int)blockIdx.x - P.first_cta, R = P.nctas;
  const int tid = threadIdx.x;
  TeamBarrier bar{P.bar, R, P.status};
  // staged phases read Q and the work vectors with bulk copies (async proxy):
  // every thread fences its generic global stores before each team barrier
  const bool staged = P.stages != 0;
  auto team_sync = [&]() -> bool {
    if (staged) fence_proxy_async_global();
    return bar.sync();
  };
  const int n = P.n, m = P.m;
  const size_t ld = (size_t)P.ld;
  const int ntiles = (n + LZ_BLOCK - 1) / LZ_BLOCK;
  const int t0 = (int)((long long)ntiles * rank / R);
  const int t1 = (int)((long long)ntiles * (rank + 1) / R);
  // [pass][column][cta] partial sums
  double* part0 = P.part;
  double* part1 = P.part + (size_t)R * MP1;
  double* part2 = P.part + (size_t)2 * R * MP1;

  int k = 0, nconv = 0, restart = 0, breakdowns = 0, steps = 0, sum_nv = 0, sum_kn = 0;
  long long clk_start = clock64(), clk_restart = 0;
  // rank-0 phase accounting: [0] barrier waits, [1] team reductions, [2..4] phases A..C
  long long tp[5] = {0, 0, 0, 0, 0}, tmark = clock64();
  const bool timing = (rank == 0 && tid == 0);
#define LZ_MARK(slot)                                   \
  do {                                                  \
    if (timing) {                                       \
      const long long _c = clock64();                   \
      tp[slot] += _c - tmark;                           \
      tmark = _c;                                       \
    }                                                   \
  } while (0)
  if (rank == 0 && tid < MAXM) { sh.alpha[tid] = 0.0; sh.beta[tid] = 0.0; }
  if (tid == 0) sh.eig_cycles = 0;
  // staged tiles (large problems): the stage area (laid out per phase), then
  // STG_MAXS mbarriers, in the dynamic shared memory
  extern __shared__ __align__(16) unsigned char lz_dyn[];
  Stager<VT> G;
  G.budget = (unsigned)P.stg_budget;
  G.cap = P.stg_cap;
  G.csr = P.stage_csr;
  G.S = 0;
  G.bytes = 0;
  G.vcol = 0;
  G.ph = 0u;
  G.nx_p0 = G.nx_p1 = 0;
  G.base = lz_dyn;
  G.bar = (uint64_t*)(lz_dyn + (size_t)G.budget);
  if (P.stages && tid == 0) {
    for (int j = 0; j < STG_MAXS; ++j) mbar_init(&G.bar[j], 1);
    mbar_init_fence();
  }
  // the start vector Q[:, 0]: flat copy for the first cycle's gathers and, for
  // a tile-major working basis, its column 0 (own rows)
  VT* xk = P.vbuf + 2 * ld;
  const bool tiled = P.Qw != P.Q;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + tid;
    if (row < n) {
      const VT v = P.Q[row];
      xk[row] = v;
      if (tiled) P.Qw[qix(P, 0, row)] = v;
    }
  }
  __syncthreads();
  if (!team_sync()) return;
  int prev = 0;          // vbuf slot holding the latest unnormalised vector
  VT invb = (VT)1;       // its normalisation
  while (nconv < P.num_desired && restart < P.max_restarts) {
    int cur = 0;
    for (int i = k; i < m; ++i) {
      const VT* xsrc;
      bool wq;
      if (i == k) {
        xsrc = xk;       // = Q[:, k]
        invb = (VT)1;
        wq = false;
      } else {
        reduce_part(part2, R, 1, sh);
        const double b = sqrt(sh.h[0]);
        if (rank == 0 && tid == 0) sh.beta[i - 1] = b;
        if (b < 1e-15) {
          // Krylov space exhausted: random vector orthogonalised twice
          // against Q[:, :i] (solver/lanczos.py:107-117)
          ++breakdowns;
          VT* buf = P.vbuf + (size_t)prev * ld;
          phase_random(P, sh, t0, t1, i, (uint64_t)i, buf, part0 + rank);
          if (!team_sync()) return;
          reduce_part(part0, R, i, sh);
          phase_update_dot(P, sh, t0, t1, i, buf, part1 + rank);
          if (!team_sync()) return;
          reduce_part(part1, R, i, sh);
          phase_update_norm(P, sh, t0, t1, i, buf, part2 + rank);
          if (!team_sync()) return;
          reduce_part(part2, R, 1, sh);
          invb = (VT)(1.0 / sqrt(sh.h[0]));
        } else {
          invb = (VT)(1.0 / b);
        }
        xsrc = P.vbuf + (size_t)prev * ld;
        wq = true;
      }
      VT* vout = P.vbuf + (size_t)cur * ld;
      LZ_MARK(1);
      if (P.stages) stg_phase_spmv(P, sh, G, t0, t1, i, xsrc, invb, wq, vout, part0 + rank);
      else phase_spmv(P, sh, t0, t1, i, xsrc, invb, wq, vout, part0 + rank);
      LZ_MARK(2);
      if (!team_sync()) return;
      LZ_MARK(0);
      reduce_part(part0, R, i + 1, sh);
      LZ_MARK(1);
      const double h1i = sh.h[i];
      if (P.stages) stg_phase_update_dot(P, sh, G, t0, t1, i + 1, vout, part1 + rank);
      else phase_update_dot(P, sh, t0, t1, i + 1, vout, part1 + rank);
      LZ_MARK(3);
      if (!team_sync()) return;
      LZ_MARK(0);
      reduce_part(part1, R, i + 1, sh);
      LZ_MARK(1);
      if (rank == 0 && tid == 0) sh.alpha[i] = h1i + sh.h[i];
      if (P.stages) stg_phase_update_norm(P, sh, G, t0, t1, i + 1, vout, part2 + rank);
      else phase_update_norm(P, sh, t0, t1, i + 1, vout, part2 + rank);
      LZ_MARK(4);
      if (!team_sync()) return;
      LZ_MARK(0);
      prev = cur;
      cur ^= 1;
      ++steps;
      sum_nv += i + 1;
    }
    // ---- restart ----
    const bool stepped = (k < m);
    if (stepped) {
      reduce_part(part2, R, 1, sh);
      const double b = sqrt(sh.h[0]);
      if (rank == 0 && tid == 0) sh.beta[m - 1] = b;
      if (b < 1e-15) {
        ++breakdowns;
        VT* buf = P.vbuf + (size_t)prev * ld;
        phase_random(P, sh, t0, t1, m, (uint64_t)m, buf, part0 + rank);
        if (!team_sync()) return;
        reduce_part(part0, R, m, sh);
        phase_update_dot(P, sh, t0, t1, m, buf, part1 + rank);
        if (!team_sync()) return;
        reduce_part(part1, R, m, sh);
        phase_update_norm(P, sh, t0, t1, m, buf, part2 + rank);
        if (!team_sync()) return;
        reduce_part(part2, R, 1, sh);
        invb = (VT)(1.0 / sqrt(sh.h[0]));
      } else {
        invb = (VT)(1.0 / b);
      }
    }
    __syncthreads();
    if (rank == 0) {
      const long long c0 = clock64();
      restart_select<false>(P, sh, k);
      clk_restart += clock64() - c0;
    }
    if (!team_sync()) return;
    const int kn = __ldcg(P.ctl + 0);
    nconv = __ldcg(P.ctl + 1);
    for (int e = tid; e < m * MAXM; e += LZ_BLOCK) {
      const int j = e / MAXM, c = e - j * MAXM;
      sh.u.Ys[e] = (c < kn) ? (VT)__ldcg(P.Ybuf + j * m + c) : (VT)0;
    }
    __syncthreads();
    const VT* lastv = P.vbuf + (size_t)prev * ld;
    for (int tile = t0; tile < t1; ++tile) {
      const int row = tile * LZ_BLOCK + tid;
      if (row < n) {
        VT qr[MAXM];
#pragma unroll
        for (int j = 0; j < MAXM; ++j) qr[j] = (j < m) ? P.Qw[qix(P, j, row)] : (VT)0;
        const VT xl = stepped ? lastv[row] * invb : P.Qw[qix(P, m, row)];
        for (int c = 0; c < kn; ++c) {
          if (c >= m) break;
          VT s = (VT)0;
#pragma unroll
          for (int j = 0; j < MAXM; ++j)
            if (j < m) s += qr[j] * sh.u.Ys[j * MAXM + c];
          P.Qw[qix(P, c, row)] = s;
        }
        P.Qw[qix(P, kn, row)] = xl;
        if (kn != m) P.Qw[qix(P, m, row)] = xl;
        xk[row] = xl;
      }
    }
    k = kn;
    sum_kn += kn;
    ++restart;
    if (!team_sync()) return;
    if (timing) tmark = clock64();   // restart time is reported separately (ctl[6])
  }
  // a tile-major working basis back to the caller's column-major Q (own rows)
  if (tiled && restart > 0) {
    for (int c = 0; c <= m; ++c)
      for (int tile = t0; tile < t1; ++tile) {
        const int row = tile * LZ_BLOCK + tid;
        if (row < n) P.Q[(size_t)c * ld + row] = P.Qw[qix(P, c, row)];
      }
  }
  if (rank == 0 && tid == 0) {
    P.ctl[2] = restart;
    P.ctl[3] = breakdowns;
    P.ctl[4] = steps;
    P.ctl[6] = (int)(clk_restart >> 10);
    P.ctl[7] = (int)((clock64() - clk_start) >> 10);
    for (int j = 0; j < 5; ++j) P.ctl[8 + j] = (int)(tp[j] >> 10);
    P.ctl[13] = sum_nv;
    P.ctl[14] = sum_kn;
    P.ctl[15] = (int)(sh.eig_cycles >> 10);
    if (restart == 0) P.ctl[0] = 0;
  }
}

// ---------------------------------------------------------------- cluster path
// A problem of at most CL_MAX_CTAS x rc rows runs as one thread-block cluster.
// CTA r of the cluster owns rows [r rc, (r+1) rc) and keeps, for the whole
// eigsh call, its rows of the basis Q (column-major, stride rc), the two work
// vectors and, when it fits, its slice of the operator (CSR with the column
// pre-split into owner CTA and local row) in shared memory.  The SpMV gathers
// x straight from the owner CTAs' shared memory (distributed shared memory,
// mapa + ld.shared::cluster); each phase's per-CTA partial sums are written to
// the CTA's own shared memory and, after a hardware cluster barrier, summed by
// every CTA over the cluster in the same fixed order, so all CTAs hold
// bit-identical coefficients and take identical branches.  The restart's
// projected eigenproblem is solved redundantly by every CTA (identical inputs,
// identical results), which needs no broadcast.  A cluster is co-scheduled by
// the hardware, so there is no software barrier and no spin-wait.
constexpr int CL_MAX_CTAS = 16;

template <typename VT>
struct ClusterDesc {
  int n, ld, m, num_desired, max_restarts, lanes, rc, csr_cap;
  long long nnz;
  double tol;
  const int* rowptr;
  const int* col;
  const VT* val;
  VT* Q;
  double* alpha;
  double* beta;
  int* ctl;
  int* status;
};

template <typename VT>
struct ClusterBatch {
  int count, csize;
  ClusterDesc<VT> t[MAX_TEAMS];
};

__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cl_map(const void* p, unsigned rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float cl_ld(uint32_t a, float) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double cl_ld(uint32_t a, double) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}

// per-CTA shared-memory layout of the cluster kernel (byte offsets)
struct ClLayout {
  size_t q, vb, part, rp, cg, val, total;
};
__host__ __device__ inline size_t cl_al(size_t b) { return (b + 15) & ~(size_t)15; }
template <typename VT>
__host__ __device__ inline ClLayout cl_layout(int m, int rc, int csr_cap) {
  ClLayout L;
  L.q = 0;
  L.vb = L.q + cl_al((size_t)(m + 1) * rc * sizeof(VT));
  L.part = L.vb + cl_al((size_t)2 * rc * sizeof(VT));
  L.rp = L.part + cl_al((size_t)3 * MP1 * sizeof(double));
  L.cg = L.rp + cl_al((size_t)(rc + 1) * sizeof(int));
  L.val = L.cg + cl_al((size_t)csr_cap * sizeof(int));
  L.total = L.val + cl_al((size_t)csr_cap * sizeof(VT));
  return L;
}

// h[c] = sum over the cluster's CTAs r = 0..C-1 of part_r[c], c < nv, summed
// as a fixed pairwise tree (FP64 adds are ~64 cycles dependent on this part).
template <typename VT>
__device__ __forceinline__ void cl_reduce(const double* part, int C, int nv, LzShared<VT>& sh) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    for (int c = lane; c < nv; c += 32) {
      double v[CL_MAX_CTAS];
#pragma unroll
      for (int r = 0; r < CL_MAX_CTAS; ++r) v[r] = (r < C) ? cl_ld(cl_map(part + c, r), 0.0) : 0.0;
#pragma unroll
      for (int h = CL_MAX_CTAS / 2; h >= 1; h >>= 1)
#pragma unroll
        for (int r = 0; r < h; ++r) v[r] = v[r] + v[r + h];
      sh.h[c] = v[0];
      sh.hv[c] = (VT)v[0];
    }
  }
  __syncthreads();
}

template <typename VT>
struct ClCtx {
  const ClusterDesc<VT>* P;
  int rank, C, r0, rows;
  bool staged;          // CSR slice in shared memory
  int p0;               // first entry of the slice
  VT* Qs;               // (m+1) x rc
  VT* vb;               // 2 x rc
  double* part;         // 3 x MP1
  int* rp;              // rows+1, relative to p0
  int* cg;              // (owner << 24) | local row
  VT* vs;
};

// Phase A: y = Op (x * xscale) for own rows -> vout, partial Q[:, c] . y (c <= i).
// x is column `xcol` of the cluster's vectors: xq selects Qs (else vb); the
// gathers read the owner CTA's copy.  If wq, Qs[:, i] = x * xscale (own rows).
template <typename VT, int L>
__device__ void cl_phase_spmv(const ClCtx<VT>& X, LzShared<VT>& sh, int i, const VT* xbase,
                              VT xscale, bool wq, VT* vout, double* part_out) {
  typedef typename Acc<VT>::type AT;
  const ClusterDesc<VT>& P = *X.P;
  const int tid = threadIdx.x, rc = P.rc;
  constexpr int GPP = LZ_BLOCK / L;
  const int g = tid / L, lig = tid - (tid / L) * L;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int base = 0; base < X.rows; base += LZ_BLOCK) {
    // SpMV of rows base..base+255 (L lanes per row) into sh.u.st.ys; groups of
    // up to 4 passes load their row bounds and first entries before any gather
    constexpr int CH = L < 4 ? L : 4;
#pragma unroll 1
    for (int q0 = 0; q0 < L; q0 += CH) {
      int pb[CH], pe[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        const int lr = base + (q0 + q) * GPP + g;
        pb[q] = 0; pe[q] = 0;
        if (lr < X.rows) {
          if (X.staged) { pb[q] = X.rp[lr] + lig; pe[q] = X.rp[lr + 1]; }
          else { pb[q] = P.rowptr[X.r0 + lr] + lig; pe[q] = P.rowptr[X.r0 + lr + 1]; }
        }
      }
      AT sacc[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        sacc[q] = (AT)0;
        if (X.staged) {
          for (int p = pb[q]; p < pe[q]; p += L) {
            const int w = X.cg[p];
            sacc[q] += (AT)X.vs[p] * (AT)cl_ld(cl_map(xbase + (w & 0xffffff), (unsigned)w >> 24), (VT)0);
          }
        } else {
          for (int p = pb[q]; p < pe[q]; p += L) {
            const int gc = P.col[p];
            const int o = gc / rc;
            sacc[q] += (AT)P.val[p] * (AT)cl_ld(cl_map(xbase + (gc - o * rc), (unsigned)o), (VT)0);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < CH; ++q) {
#pragma unroll
        for (int o = L >> 1; o > 0; o >>= 1) sacc[q] += __shfl_xor_sync(0xffffffffu, sacc[q], o);
        if (lig == 0) sh.u.st.ys[(q0 + q) * GPP + g] = (double)sacc[q];
      }
    }
    __syncthreads();
    const int lr = base + tid;
    if (lr < X.rows) {
      const VT y = (VT)sh.u.st.ys[tid] * xscale;
      vout[lr] = y;
      VT xn = (VT)0;
      if (wq) {
        xn = xbase[lr] * xscale;
        X.Qs[(size_t)i * rc + lr] = xn;
      }
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c <= i) {
          const VT qc = (wq && c == i) ? xn : X.Qs[(size_t)c * rc + lr];
          acc[c] += (AT)qc * (AT)y;
        }
      }
    }
    __syncthreads();
  }
  block_reduce_cols(acc, i + 1, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_random(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, uint64_t key,
                                VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    const VT r = (VT)hash_normal(key, (uint64_t)(X.r0 + lr));
    buf[lr] = r;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) acc[c] += (AT)X.Qs[(size_t)c * rc + lr] * (AT)r;
  }
  block_reduce_cols(acc, nv, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_update_dot(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, VT* buf,
                                    double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    VT qr[MP1];
    VT s = (VT)0;
#pragma unroll
    for (int c = 0; c < MP1; ++c) {
      if (c < nv) {
        qr[c] = X.Qs[(size_t)c * rc + lr];
        s += qr[c] * sh.hv[c];
      }
    }
    const VT q1 = buf[lr] - s;
    buf[lr] = q1;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) acc[c] += (AT)qr[c] * (AT)q1;
  }
  block_reduce_cols(acc, nv, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_update_norm(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, VT* buf,
                                     double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT nrm = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    VT s = (VT)0;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) s += X.Qs[(size_t)c * rc + lr] * sh.hv[c];
    const VT q2 = buf[lr] - s;
    buf[lr] = q2;
    nrm += (AT)q2 * (AT)q2;
  }
  AT one[MP1];
  one[0] = nrm;
  block_reduce_cols(one, 1, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_spmv_dispatch(const ClCtx<VT>& X, LzShared<VT>& sh, int i, const VT* xbase,
                                 VT xscale, bool wq, VT* vout, double* part_out) {
  switch (X.P->lanes) {
    case 1: cl_phase_spmv<VT, 1>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 2: cl_phase_spmv<VT, 2>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 4: cl_phase_spmv<VT, 4>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 8: cl_phase_spmv<VT, 8>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 16: cl_phase_spmv<VT, 16>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    default: cl_phase_spmv<VT, 32>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
  }
}

template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 1)
lanczos_cluster_kernel(const __grid_constant__ ClusterBatch<VT> batch) {
  __shared__ LzShared<VT> sh;
  extern __shared__ __align__(16) unsigned char cl_dyn[];
  const int C = batch.csize;
  const ClusterDesc<VT>& P = batch.t[blockIdx.x / C];
  const int rank = (int)cl_rank();
  const int tid = threadIdx.x;
  const int n = P.n, m = P.m, rc = P.rc;
  const size_t ld = (size_t)P.ld;
  const ClLayout Lo = cl_layout<VT>(m, rc, P.csr_cap);
  ClCtx<VT> X;
  X.P = &P;
  X.rank = rank;
  X.C = C;
  X.r0 = rank * rc;
  X.rows = max(0, min(rc, n - X.r0));
  X.Qs = (VT*)(cl_dyn + Lo.q);
  X.vb = (VT*)(cl_dyn + Lo.vb);
  X.part = (double*)(cl_dyn + Lo.part);
  X.rp = (int*)(cl_dyn + Lo.rp);
  X.cg = (int*)(cl_dyn + Lo.cg);
  X.vs = (VT*)(cl_dyn + Lo.val);
  double* part0 = X.part;
  double* part1 = X.part + MP1;
  double* part2 = X.part + 2 * MP1;
  // stage Q[:, 0] (the start vector) and, if it fits, the operator slice
  for (int lr = tid; lr < X.rows; lr += LZ_BLOCK) X.Qs[lr] = P.Q[X.r0 + lr];
  X.p0 = (X.rows > 0) ? P.rowptr[X.r0] : 0;
  const int p1 = (X.rows > 0) ? P.rowptr[X.r0 + X.rows] : 0;
  X.staged = (p1 - X.p0) <= P.csr_cap;
  if (X.staged) {
    for (int lr = tid; lr <= X.rows; lr += LZ_BLOCK) X.rp[lr] = P.rowptr[X.r0 + lr] - X.p0;
    for (int p = X.p0 + tid; p < p1; p += LZ_BLOCK) {
      const int gc = P.col[p];
      const int o = gc / rc;
      X.cg[p - X.p0] = (o << 24) | (gc - o * rc);
      X.vs[p - X.p0] = P.val[p];
    }
  }
  int k = 0, nconv = 0, restart = 0, breakdowns = 0, steps = 0, sum_nv = 0, sum_kn = 0;
  long long clk_start = clock64(), clk_restart = 0;
  long long tp[5] = {0, 0, 0, 0, 0}, tmark = clock64();
  const bool timing = (rank == 0 && tid == 0);
  if (tid < MAXM) { sh.alpha[tid] = 0.0; sh.beta[tid] = 0.0; }
  if (tid == 0) sh.eig_cycles = 0;
  __syncthreads();
  cl_sync();
  int prev = 0;
  VT invb = (VT)1;
  while (nconv < P.num_desired && restart < P.max_restarts) {
    int cur = 0;
    for (int i = k; i < m; ++i) {
      const VT* xbase;
      bool wq;
      if (i == k) {
        xbase = X.Qs + (size_t)k * rc;
        invb = (VT)1;
        wq = false;
      } else {
        cl_reduce(part2, C, 1, sh);
        const double b = sqrt(sh.h[0]);
        if (tid == 0) sh.beta[i - 1] = b;
        if (b < 1e-15) {
          // Krylov space exhausted: random vector orthogonalised twice
          // against Q[:, :i] (solver/lanczos.py:107-117)
          ++breakdowns;
          VT* buf = X.vb + (size_t)prev * rc;
          cl_phase_random(X, sh, i, (uint64_t)i, buf, part0);
          cl_sync();
          cl_reduce(part0, C, i, sh);
          cl_phase_update_dot(X, sh, i, buf, part1);
          cl_sync();
          cl_reduce(part1, C, i, sh);
          cl_phase_update_norm(X, sh, i, buf, part2);
          cl_sync();
          cl_reduce(part2, C, 1, sh);
          invb = (VT)(1.0 / sqrt(sh.h[0]));
        } else {
          invb = (VT)(1.0 / b);
        }
        xbase = X.vb + (size_t)prev * rc;
        wq = true;
      }
      VT* vout = X.vb + (size_t)cur * rc;
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      cl_spmv_dispatch(X, sh, i, xbase, invb, wq, vout, part0);
      if (timing) { const long long c = clock64(); tp[2] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      cl_reduce(part0, C, i + 1, sh);
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      const double h1i = sh.h[i];
      cl_phase_update_dot(X, sh, i + 1, vout, part1);
      if (timing) { const long long c = clock64(); tp[3] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      cl_reduce(part1, C, i + 1, sh);
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      if (tid == 0) sh.alpha[i] = h1i + sh.h[i];
      cl_phase_update_norm(X, sh, i + 1, vout, part2);
      if (timing) { const long long c = clock64(); tp[4] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      prev = cur;
      cur ^= 1;
      ++steps;
      sum_nv += i + 1;
    }
    // ---- restart ----
    const bool stepped = (k < m);
    if (stepped) {
      cl_reduce(part2, C, 1, sh);
      const double b = sqrt(sh.h[0]);
      if (tid == 0) sh.beta[m - 1] = b;
      if (b < 1e-15) {
        ++breakdowns;
        VT* buf = X.vb + (size_t)prev * rc;
        cl_phase_random(X, sh, m, (uint64_t)m, buf, part0);
        cl_sync();
        cl_reduce(part0, C, m, sh);
        cl_phase_update_dot(X, sh, m, buf, part1);
        cl_sync();
        cl_reduce(part1, C, m, sh);
        cl_phase_update_norm(X, sh, m, buf, part2);
        cl_sync();
        cl_reduce(part2, C, 1, sh);
        invb = (VT)(1.0 / sqrt(sh.h[0]));
      } else {
        invb = (VT)(1.0 / b);
      }
    }
    __syncthreads();
    const long long c0 = clock64();
    restart_select<true>(P, sh, k, /*write_out=*/rank == 0);
    if (timing) clk_restart += clock64() - c0;
    const int kn = sh.k_next;
    nconv = sh.nconv;
    const VT* last = stepped ? (X.vb + (size_t)prev * rc) : (X.Qs + (size_t)m * rc);
    const VT lscale = stepped ? invb : (VT)1;
    for (int lr = tid; lr < X.rows; lr += LZ_BLOCK) {
      VT qr[MAXM];
#pragma unroll
      for (int j = 0; j < MAXM; ++j) qr[j] = (j < m) ? X.Qs[(size_t)j * rc + lr] : (VT)0;
      const VT xl = last[lr] * lscale;
      for (int c = 0; c < kn; ++c) {
        if (c >= m) break;
        VT s = (VT)0;
#pragma unroll
        for (int j = 0; j < MAXM; ++j)
          if (j < m) s += qr[j] * sh.u.Ys[j * MAXM + c];
        X.Qs[(size_t)c * rc + lr] = s;
      }
      X.Qs[(size_t)kn * rc + lr] = xl;
      if (kn != m) X.Qs[(size_t)m * rc + lr] = xl;
    }
    k = kn;
    sum_kn += kn;
    ++restart;
    __syncthreads();
    cl_sync();   // rotated rows visible to the next cycle's gathers
    if (timing) tmark = clock64();
  }
  // the basis back to global memory (own rows; untouched if no cycle ran)
  if (restart > 0) {
    for (int c = 0; c <= m; ++c)
      for (int lr = tid; lr < X.rows; lr += LZ_BLOCK)
        P.Q[(size_t)c * ld + X.r0 + lr] = X.Qs[(size_t)c * rc + lr];
  }
  if (rank == 0 && tid == 0) {
    P.ctl[2] = restart;
    P.ctl[3] = breakdowns;
    P.ctl[4] = steps;
    P.ctl[6] = (int)(clk_restart >> 10);
    P.ctl[7] = (int)((clock64() - clk_start) >> 10);
    for (int j = 0; j < 5; ++j) P.ctl[8 + j] = (int)(tp[j] >> 10);
    P.ctl[13] = sum_nv;
    P.ctl[14] = sum_kn;
    P.ctl[15] = (int)(sh.eig_cycles >> 10);
    if (restart == 0) P.ctl[0] = 0;
  }
  cl_sync();   // no CTA leaves while a peer may still read its shared memory
}

// ---------------------------------------------------------------- host side

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// tile-major working basis of a staged team (x too large for shared memory)
static size_t team_basis_bytes(int n, int m, size_t vt) {
  if ((size_t)n * vt <= (size_t)LZ_XS_BYTES) return 0;
  const size_t tiles = ((size_t)n + LZ_BLOCK - 1) / LZ_BLOCK;
  return align256(tiles * (size_t)(m + 1) * LZ_BLOCK * vt);
}

size_t lanczos_workspace_bytes(int n, int ld, int m, int prec, int nctas) {
  const size_t vt = (prec == 64) ? 8 : 4;
  size_t b = align256(3 * (size_t)ld * vt);
  b += align256((size_t)3 * nctas * MP1 * sizeof(double));
  b += align256((size_t)MAXM * MAXM * sizeof(double));
  b += 256;  // barrier counters
  b += team_basis_bytes(n, m, vt);
  return b;
}

int lanczos_lanes(int n, long long nnz) {
  const double avg = n > 0 ? (double)nnz / n : 1.0;
  int L = 1;
  while (L < 32 && L * 2 <= avg * 0.75 + 1) L *= 2;
  return L;
}

int lanczos_team_size(const DeviceInfo& di, int n, int prec) {
  const int occ = (prec == 64) ? di.lanczos_occ64 : di.lanczos_occ32;
  // two SMs stay free for the single-CTA kernels that run beside the team
  const int maxc = (di.sm_count > 4 ? di.sm_count - 2 : di.sm_count) * (occ > 0 ? occ : 1);
  const int tiles = (n + LZ_BLOCK - 1) / LZ_BLOCK;
  // at least 4 tiles per CTA: small problems are latency bound, and every
  // extra CTA costs barrier arrivals and partial sums on each phase
  int want = (tiles + 3) / 4;
  // USBS_LANCZOS_CTAS overrides the team size (tuning experiments)
  static const int forced = [] {
    const char* e = getenv("USBS_LANCZOS_CTAS");
    return e ? atoi(e) : 0;
  }();
  if (forced > 0) want = forced;
  if (want > tiles) want = tiles;
  if (want > maxc) want = maxc;
  if (want < 1) want = 1;
  return want;
}

// team kernel: dynamic shared memory it may use (x staged, or the stage area
// plus its mbarriers) and the stage area itself
template <typename VT>
constexpr size_t tm_dyn_max() {
  return (227 * 1024 - sizeof(LzShared<VT>) - 1024) / 128 * 128;
}
template <typename VT>
constexpr unsigned tm_budget() {
  return (unsigned)((tm_dyn_max<VT>() - STG_MAXS * sizeof(uint64_t)) / 128 * 128);
}
static_assert(tm_dyn_max<double>() >= (size_t)LZ_XS_BYTES, "staged x must fit");

template <typename VT>
static int run_typed(const DeviceInfo& di, const LanczosProblem* probs, int count,
                     cudaStream_t stream) {
  const int occ = (sizeof(VT) == 8) ? di.lanczos_occ64 : di.lanczos_occ32;
  const int maxc = (di.sm_count > 4 ? di.sm_count - 2 : di.sm_count) * (occ > 0 ? occ : 1);
  for (int base = 0; base < count; base += MAX_TEAMS) {
    const int cnt = (count - base < MAX_TEAMS) ? (count - base) : MAX_TEAMS;
    TeamBatch<VT> batch;
    batch.count = cnt;
    int total = 0;
    int want[MAX_TEAMS];   // cnt <= MAX_TEAMS; no heap allocation on the launch path
    for (int i = 0; i < cnt; ++i) {
      want[i] = lanczos_team_size(di, probs[base + i].n, sizeof(VT) == 8 ? 64 : 32);
      total += want[i];
    }
    if (total > maxc) {
      // shrink teams proportionally so that every CTA is co-resident
      int tot2 = 0;
      for (int i = 0; i < cnt; ++i) {
        want[i] = (int)((long long)want[i] * maxc / total);
        if (want[i] < 1) want[i] = 1;
        tot2 += want[i];
      }
      if (tot2 > maxc) {
        set_error("lanczos: %d problems need more co-resident CTAs (%d) than the device holds (%d)",
                  cnt, tot2, maxc);
        return -3;
      }
      total = tot2;
    }
    int first = 0;
    size_t dyn = 0;
    for (int i = 0; i < cnt; ++i) {
      const LanczosProblem& p = probs[base + i];
      if (p.m > MAXM || p.m < 1 || p.n < 1 || p.ld < p.n) {
        set_error("lanczos: unsupported sizes n=%d ld=%d m=%d (m must be in [1, %d])", p.n,
                  p.ld, p.m, MAXM);
        return -2;
      }
      TeamDesc<VT>& t = batch.t[i];
      t.n = p.n; t.ld = p.ld; t.m = p.m; t.num_desired = p.num_desired;
      t.max_restarts = p.max_restarts; t.tol = p.tol;
      t.lanes = lanczos_lanes(p.n, p.nnz);
      t.xsmem = ((size_t)p.n * sizeof(VT) <= (size_t)LZ_XS_BYTES) ? 1 : 0;
      if (t.xsmem && (size_t)p.n * sizeof(VT) > dyn) dyn = (size_t)p.n * sizeof(VT);
      // staged tiles when x is not staged: bulk copies from the workspace (the
      // work vectors and the tile-major basis) need it 16-byte aligned
      t.stages = 0;
      t.stage_csr = 0;
      t.stg_budget = 0;
      t.stg_cap = 0;
      if (!t.xsmem && p.ld % 32 == 0 && ((uintptr_t)p.work & 15u) == 0) {
        // the stage area takes the shared memory the kernel leaves; every
        // phase keeps at least two of its largest stages in flight.  FP32
        // stages also carry the tile's CSR slice, sized for 1.5x the mean
        // tile (bulk copies of rowptr / col / val need 16-byte aligned arrays)
        const unsigned budget = tm_budget<VT>();
        const long long mean_tile = p.nnz * LZ_BLOCK / (p.n > 0 ? p.n : 1);
        long long cap = (mean_tile * 3 / 2 + 63) / 64 * 64;
        cap = cap < 512 ? 512 : (cap > STG_CAP ? STG_CAP : cap);
        const unsigned qmax = stg_q_bytes<VT>(MP1 + 1);
        const bool csr_ok = sizeof(VT) == 4 && ((((uintptr_t)p.rowptr) | ((uintptr_t)p.col) |
                                                 ((uintptr_t)p.val)) & 15u) == 0 &&
                            2 * (qmax + stg_csr_bytes<VT>((int)cap)) <= budget;
        if (2 * qmax <= budget) {
          t.stages = 1;
          t.stage_csr = csr_ok ? 1 : 0;
          t.stg_budget = (int)budget;
          t.stg_cap = (int)cap;
          const size_t need = (size_t)budget + STG_MAXS * sizeof(uint64_t);
          if (need > dyn) dyn = need;
        }
      }
      t.first_cta = first;
      t.nctas = want[i];
      t.rowptr = p.rowptr; t.col = p.col; t.val = (const VT*)p.val;
      t.nnz = p.nnz;
      t.Q = (VT*)p.Q;
      char* w = (char*)p.work;
      t.vbuf = (VT*)w; w += align256(3 * (size_t)p.ld * sizeof(VT));
      t.part = (double*)w; w += align256((size_t)3 * want[i] * MP1 * sizeof(double));
      t.Ybuf = (double*)w; w += align256((size_t)MAXM * MAXM * sizeof(double));
      t.bar = (unsigned int*)w; w += 256;
      // staged teams work on a tile-major copy of the basis (workspace)
      if (t.stages) {
        t.Qw = (VT*)w;
        t.qts = (long long)(p.m + 1) * LZ_BLOCK;
        t.qcs = LZ_BLOCK;
      } else {
        t.Qw = t.Q;
        t.qts = LZ_BLOCK;
        t.qcs = p.ld;
      }
      t.alpha = p.alpha; t.beta = p.beta; t.ctl = p.ctl; t.status = p.status;
      first += want[i];
      if (cudaMemsetAsync(t.bar, 0, 2 * sizeof(unsigned int), stream) != cudaSuccess ||
          cudaMemsetAsync(p.ctl, 0, 16 * sizeof(int), stream) != cudaSuccess) {
        set_error("lanczos: memset failed");
        return -4;
      }
    }
    void* args[] = {(void*)&batch};
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute((const void*)lanczos_team_kernel<VT>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<VT>());
      attr_set = true;
    }
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)lanczos_team_kernel<VT>,
                                                dim3(total), dim3(LZ_BLOCK), args, dyn, stream);
    if (e != cudaSuccess) {
      set_error("lanczos: cooperative launch of %d CTAs failed: %s", total,
                cudaGetErrorString(e));
      return -5;
    }
  }
  return 0;
}

// shared memory left for the cluster kernel's dynamic layout
template <typename VT>
constexpr size_t cl_budget() { return 227 * 1024 - sizeof(LzShared<VT>) - 1024; }
// ---- cluster-size policy and its autotuner ----
// A launch's cluster size is ceil(n_max / target) CTAs (at most 16), for a
// target number of rows per CTA.  Each step's phases scale with the rows per
// CTA and its cluster reductions with the CTAs, and clusters of one launch
// (or of concurrent solves) compete for the SMs: on GB300 a lone problem runs
// fastest spread over 16 CTAs (FP32 n = 5000: 4.8 ms at 16 CTAs, 8.7 ms at 8),
// while 48 problems in one launch run fastest packed at 640 rows per CTA
// (17 ms against 27 ms spread).  A caller that knows its launch shares the
// GPU (a solve service) passes its own rows per CTA in the problem; otherwise
// the class's measured choice is used (usbs_lanczos_autotune times the
// candidates on a caller's batch and records the fastest for its precision,
// batch and size class), else 64 rows per CTA for one problem and 640 for a
// batch.
constexpr int TUNE_NCAND = 5;
constexpr int TUNE_CAND[TUNE_NCAND] = {64, 128, 256, 640, 1280};
static std::mutex g_tune_mu;
static std::map<long long, int> g_tune;            // class key -> rows per CTA
static thread_local int t_forced_target = 0;       // set by the tuner while it measures

static int log2_bucket(long long v) {
  int b = 0;
  while (v > 1) { v >>= 1; ++b; }
  return b;
}
// class key: precision << 32 | floor(log2(problems)) << 16 | floor(log2(largest n))
static long long tune_key(int prec, int count, int nmax) {
  return ((long long)prec << 32) | ((long long)log2_bucket(count < 1 ? 1 : count) << 16) |
         log2_bucket(nmax);
}
static int cl_target(int prec, int count, int nmax, int requested) {
  if (t_forced_target) return t_forced_target;
  if (requested > 0) return requested;
  if (const char* e = getenv(prec == 64 ? "USBS_CL_TARGET64" : "USBS_CL_TARGET32"))
    if (atoi(e) >= 32) return atoi(e);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(prec, count, nmax));
    if (it != g_tune.end()) return it->second;
  }
  return count <= 1 ? 64 : 640;
}
static int cl_csize_for(int n, int target) {
  const int c = (n + target - 1) / target;
  return c < 1 ? 1 : (c > CL_MAX_CTAS ? CL_MAX_CTAS : c);
}
template <typename VT>
inline int cl_csize(int n) {
  return cl_csize_for(n, cl_target(sizeof(VT) == 8 ? 64 : 32, 1, n, 0));
}
template <typename VT>
static bool cl_fits(int n, int m) {
  const int csize = cl_csize<VT>(n);
  if (csize > CL_MAX_CTAS || m > MAXM || m < 1 || n < 1) return false;
  const int rc = (n + csize - 1) / csize;
  return cl_layout<VT>(m, rc, 0).total <= cl_budget<VT>();
}

int lanczos_kernel_kind(int n, int m, int prec) {
  static const int enabled = [] {
    const char* e = getenv("USBS_LANCZOS_CLUSTER");
    return e ? atoi(e) : 1;
  }();
  if (!enabled) return 0;
  return (prec == 64 ? cl_fits<double>(n, m) : cl_fits<float>(n, m)) ? 1 : 0;
}

// Cluster path: every problem of the launch as one cluster of `csize` CTAs.
// Returns 1 if the problems do not fit (the caller then runs the team kernel),
// 0 on success, negative on a launch error.
template <typename VT>
static int run_cluster(const LanczosProblem* probs, int count, cudaStream_t stream) {
  static const int enabled = [] {
    const char* e = getenv("USBS_LANCZOS_CLUSTER");   // 0 forces the team kernel
    return e ? atoi(e) : 1;
  }();
  if (!enabled || count < 1 || count > MAX_TEAMS) return 1;
  constexpr size_t BUDGET = cl_budget<VT>();
  int nmax = 1, req = 0;
  for (int i = 0; i < count; ++i) {
    nmax = probs[i].n > nmax ? probs[i].n : nmax;
    req = probs[i].rows_per_cta > req ? probs[i].rows_per_cta : req;
  }
  const int csize = cl_csize_for(nmax, cl_target(sizeof(VT) == 8 ? 64 : 32, count, nmax, req));
  if (csize > CL_MAX_CTAS) return 1;
  ClusterBatch<VT> batch;
  batch.count = count;
  size_t dyn = 0;
  for (int i = 0; i < count; ++i) {
    const LanczosProblem& p = probs[i];
    if (p.m > MAXM || p.m < 1 || p.n < 1 || p.ld < p.n) return 1;
    const int rc = (p.n + csize - 1) / csize;
    const ClLayout base = cl_layout<VT>(p.m, rc, 0);
    if (base.total > BUDGET) return 1;
    // whatever is left holds the operator slice (else it is read from L2)
    const int cap = (int)((BUDGET - base.total) / (sizeof(int) + sizeof(VT))) - 8;
    ClusterDesc<VT>& t = batch.t[i];
    t.n = p.n; t.ld = p.ld; t.m = p.m; t.num_desired = p.num_desired;
    t.max_restarts = p.max_restarts; t.tol = p.tol; t.nnz = p.nnz;
    t.lanes = lanczos_lanes(p.n, p.nnz);
    t.rc = rc;
    t.csr_cap = cap > 0 ? cap : 0;
    t.rowptr = p.rowptr; t.col = p.col; t.val = (const VT*)p.val;
    t.Q = (VT*)p.Q; t.alpha = p.alpha; t.beta = p.beta; t.ctl = p.ctl; t.status = p.status;
    const size_t tot = cl_layout<VT>(p.m, rc, t.csr_cap).total;
    dyn = tot > dyn ? tot : dyn;
  }
  batch.csize = csize;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute((const void*)lanczos_cluster_kernel<VT>,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)lanczos_cluster_kernel<VT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BUDGET);
    attr_set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(csize * count));
  cfg.blockDim = dim3(LZ_BLOCK);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  cudaLaunchConfig_t qcfg = cfg;     // the query needs no stream (this one may be capturing)
  qcfg.stream = nullptr;
  if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)lanczos_cluster_kernel<VT>, &qcfg) !=
          cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return 1;
  }
  for (int i = 0; i < count; ++i) {
    if (cudaMemsetAsync(probs[i].ctl, 0, 16 * sizeof(int), stream) != cudaSuccess) {
      set_error("lanczos: memset failed");
      return -4;
    }
  }
  cudaError_t e = cudaLaunchKernelEx(&cfg, lanczos_cluster_kernel<VT>, batch);
  if (e != cudaSuccess) {
    set_error("lanczos: cluster launch (%d x %d CTAs) failed: %s", count, csize,
              cudaGetErrorString(e));
    return -5;
  }
  return 0;
}

int lanczos_run(const DeviceInfo& di, const LanczosProblem* probs, int count, int prec,
                cudaStream_t stream) {
  if (prec == 64) {
    const int rc = run_cluster<double>(probs, count, stream);
    if (rc <= 0) return rc;
    return run_typed<double>(di, probs, count, stream);
  }
  if (prec == 32) {
    const int rc = run_cluster<float>(probs, count, stream);
    if (rc <= 0) return rc;
    return run_typed<float>(di, probs, count, stream);
  }
  set_error("lanczos: precision must be 32 or 64");
  return -2;
}

int lanczos_tune_candidates(int i) { return (i >= 0 && i < TUNE_NCAND) ? TUNE_CAND[i] : 0; }

void lanczos_force_target(int target) { t_forced_target = target; }

// cluster size a launch of `count` problems of at most nmax rows gets with `target`
int lanczos_cluster_size(int nmax, int target) { return cl_csize_for(nmax, target); }

void lanczos_tune_record(int prec, int count, int nmax, int target) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (target > 0) g_tune[tune_key(prec, count, nmax)] = target;
  else g_tune.erase(tune_key(prec, count, nmax));
}

int lanczos_tune_entries(long long* keys, int* targets, int cap) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int i = 0;
  for (const auto& kv : g_tune) {
    if (i < cap) { keys[i] = kv.first; targets[i] = kv.second; }
    ++i;
  }
  return i;
}

void lanczos_tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

int lanczos_occupancy(int prec) {
  // occupancy with the largest staged x, so any launch stays co-resident
  int occ = 0;
  if (prec == 64) {
    cudaFuncSetAttribute((const void*)lanczos_team_kernel<double>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<double>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lanczos_team_kernel<double>, LZ_BLOCK,
                                                  tm_dyn_max<double>());
  } else {
    cudaFuncSetAttribute((const void*)lanczos_team_kernel<float>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<float>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lanczos_team_kernel<float>, LZ_BLOCK,
                                                  tm_dyn_max<float>());
  }
  return occ;
}

}  // namespace usbs
