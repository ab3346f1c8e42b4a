// Numeric engine: launch schedules for the multifrontal factorisation, the
// forward/backward solves and the Takahashi selected inversion, and their
// execution on one stream.
//
// Replaces the CHOLMOD calls of the reference: cholesky(Q) + Factor.logdet()
// (spdes/advection_diffusion2D.py:117,193,198), Factor.solve_A
// (:194,201-202; model.py:126), Factor.solve_Lt + apply_Pt (model.py:80) and the
// R-INLA selected inverse (model.py:89-118, rqinv.R:18-205).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "engine.cuh"

namespace spde {

#define CUDA_TRY(x)                                                   \
  do {                                                                \
    cudaError_t e_ = (x);                                             \
    if (e_ != cudaSuccess) {                                          \
      p->last_error = std::string(#x) + ": " + cudaGetErrorString(e_); \
      return 2;                                                       \
    }                                                                 \
  } while (0)

constexpr int kNbk = 64;  // diagonal block size (kMaxNbk in dense.cu)
constexpr int kTcMinK = 128;  // shortest K routed to the tensor-core product
constexpr int kTcMinKUpdate = 64;  // ... for the rank-64 updates inside a factor panel
// shortest K of a cluster-pair task: below it the pair's per-task set-up and
// pipeline fill outweigh its throughput, and the single-CTA kernel is faster
constexpr int kPairMinK = 256;
enum { KT_NONE = 0, KT_A_UPPER, KT_B_LOWER, KT_BOTH_UPPER };
constexpr int kPanel = 512;   // panel width of the two-level blocked factorisation

// ----------------------------------------------------------- upload helpers
template <typename X>
static X* upload_vec(const std::vector<X>& v) {
  if (v.empty()) return nullptr;
  X* d = nullptr;
  if (cudaMalloc(&d, v.size() * sizeof(X)) != cudaSuccess) return nullptr;
  cudaMemcpy(d, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice);
  return d;
}

void Schedule::upload() {
  d_gemm = upload_vec(gemm);
  d_diag = upload_vec(diag);
  d_ext = upload_vec(ext);
  d_rows = upload_vec(rows);
  d_mirror = upload_vec(mirror);
}
void Schedule::release() {
  cudaFree(d_gemm); cudaFree(d_diag); cudaFree(d_ext); cudaFree(d_rows); cudaFree(d_mirror); cudaFree(d_maps);
  d_gemm = nullptr; d_diag = nullptr; d_ext = nullptr; d_rows = nullptr; d_mirror = nullptr; d_maps = nullptr;
}

// ----------------------------------------------------------- schedule helpers
struct Builder {
  Schedule& s;
  int TM, TN;
  bool pair_ok;   // products of at least 128 x 128 x kPairMinK may take 256 x 256 cluster-pair tiles (FP32 plan)
  int depth = 0;  // tree depth of the ops begun next
  explicit Builder(Schedule& sc, int tm, int tn, bool pairs = false) : s(sc), TM(tm), TN(tn), pair_ok(pairs) {}

  // TMA source of a row-major operand starting at element `off` of buffer `buf`,
  // inside the region [base, ...) with row stride ld: the map index and the
  // (column, row) coordinates, or -1 where TMA cannot address it (alignment)
  int tma_source(int buf, int64_t base, int64_t off, int ld, int* x, int* y) {
    if (buf == B_NONE || base < 0 || (ld & 3) != 0 || (base & 3) != 0 || off < base) return -1;
    const int64_t d = off - base, col = d % ld, row = d / ld;
    if ((col & 3) != 0 || row > int64_t(1) << 30) return -1;
    const auto key = std::make_tuple(buf, base, ld);
    auto it = s.map_index.find(key);
    int idx;
    if (it == s.map_index.end()) {
      idx = int(s.maps.size());
      s.maps.push_back({buf, base, ld});
      s.map_index.emplace(key, idx);
    } else {
      idx = it->second;
    }
    *x = int(col);
    *y = int(row);
    return idx;
  }

  Op& begin(int kind) {
    s.ops.push_back(Op());
    Op& o = s.ops.back();
    o.kind = kind;
    o.depth = depth;
    switch (kind) {
      case OP_GEMM: o.off = int64_t(s.gemm.size()); break;
      case OP_DIAG: o.off = int64_t(s.diag.size()); break;
      case OP_EXTEND: o.off = int64_t(s.ext.size()); break;
      case OP_MIRROR: o.off = int64_t(s.mirror.size()); break;
      default: o.off = int64_t(s.rows.size()); break;
    }
    return o;
  }
  void end() {
    if (s.ops.back().kind == OP_GEMM) split_by_k();
    finish(s.ops.back());
  }
  // Tiles with a short K (panel solves, rank-64 updates) run on the SIMT kernel,
  // the others on the tensor-core kernel: split one GEMM launch into two, the
  // first (already complete) and the second left for finish().
  void split_by_k() {
    {
      // cluster-pair tasks go first, in a launch of their own
      Op& o = s.ops.back();
      const int64_t beg = o.off, end = int64_t(s.gemm.size());
      auto mid = std::stable_partition(s.gemm.begin() + beg, s.gemm.begin() + end,
                                       [](const GemmTask& t) { return t.pair != 0; });
      const int64_t npair = int64_t(mid - s.gemm.begin()) - beg;
      if (npair > 0) {
        o.tc = kPathPair;
        if (beg + npair == end) return;
        Op rest = o;
        o.flops = 0;
        for (int64_t i = beg; i < beg + npair; ++i) o.flops += 2.0 * s.gemm[i].m * s.gemm[i].n * s.gemm[i].k;
        o.count = int(npair);
        ++s.launches;
        rest.off = beg + npair;
        rest.flops = 0;
        for (int64_t i = beg + npair; i < end; ++i) rest.flops += 2.0 * s.gemm[i].m * s.gemm[i].n * s.gemm[i].k;
        s.ops.push_back(rest);
      }
    }
    Op& o = s.ops.back();
    const int64_t beg = o.off, end = int64_t(s.gemm.size());
    int nmax = 0;
    for (int64_t i = beg; i < end; ++i) nmax = std::max(nmax, s.gemm[i].n);
    if (end > beg && nmax <= kNarrowMaxN) {
      o.tc = kPathNarrow;
      o.nmax = nmax;
      return;
    }
    // panel solves, and look-ahead updates of one block column: m <= TM, n <= 64, k <= 64
    bool panel = (o.site == S_F_TRSM || o.site == S_F_UPD) && end > beg;
    for (int64_t i = beg; i < end && panel; ++i) panel = s.gemm[i].n <= kNbk && s.gemm[i].k <= kNbk;
    if (panel) {
      o.tc = kPathPanel;
      return;
    }
    const int mink = o.site == S_F_UPD ? kTcMinKUpdate : kTcMinK;
    auto mid = std::stable_partition(s.gemm.begin() + beg, s.gemm.begin() + end,
                                     [mink](const GemmTask& t) { return t.k >= mink; });
    const int64_t nlong = int64_t(mid - s.gemm.begin()) - beg;
    if (nlong == 0 || beg + nlong == end) {
      o.tc = nlong > 0 ? 1 : 0;
      return;
    }
    Op second = o;
    o.tc = 1;
    o.flops = 0;
    for (int64_t i = beg; i < beg + nlong; ++i) o.flops += 2.0 * s.gemm[i].m * s.gemm[i].n * s.gemm[i].k;
    o.count = int(nlong);
    ++s.launches;
    second.off = beg + nlong;
    second.tc = 0;
    second.flops = 0;
    for (int64_t i = beg + nlong; i < end; ++i) second.flops += 2.0 * s.gemm[i].m * s.gemm[i].n * s.gemm[i].k;
    s.ops.push_back(second);
  }
  void finish(Op& o) {
    switch (o.kind) {
      case OP_GEMM: o.count = int(int64_t(s.gemm.size()) - o.off); break;
      case OP_DIAG: o.count = int(int64_t(s.diag.size()) - o.off); break;
      case OP_EXTEND: o.count = int(int64_t(s.ext.size()) - o.off); break;
      case OP_MIRROR: o.count = int(int64_t(s.mirror.size()) - o.off); break;
      case OP_MEMSET: o.count = 1; break;
      default: o.count = int(int64_t(s.rows.size()) - o.off); break;
    }
    if (o.count == 0) s.ops.pop_back();
    else ++s.launches;
  }
  // C[m x n] (op)= A B' tiled; A row i at a + i*arow_step, B row j at b + j*brow_step,
  // C(i, j) at c + i*ldc + j.  lower: only tiles with row tile >= column tile.
  // kt: skip structurally zero K ranges of triangular row-layout operands whose
  // K index shares the origin of their row index (KT_A_UPPER: A[i,k] = 0 for
  // k < i; KT_B_LOWER: B[j,k] = 0 for k > j; KT_BOTH_UPPER: both upper).
  // abase / bbase: start of the row-major region the operand lies in (for its
  // TMA map); with both given, a product of at least 128 x 128 x kPairMinK in the FP32
  // plan takes 256 x 256 tiles for the cluster-pair tensor-core kernel.
  void gemm_tiles(int64_t a, int lda, int64_t arow, int64_t b, int ldb, int64_t brow, int64_t c, int ldc, int m, int n,
                  int k, bool lower = false, int i_start = 0, int kt = KT_NONE, int64_t abase = -1,
                  int64_t bbase = -1) {
    if (m <= 0 || n <= 0 || k <= 0) return;
    const Op& op = s.ops.back();
    const bool pair = pair_ok && abase >= 0 && bbase >= 0 && arow == lda && brow == ldb && op.al == kRow &&
                      op.bl == kRow && m >= 128 && n >= 128 && k >= kPairMinK && i_start == 0;
    const int tm = pair ? kPairTile : TM, tn = pair ? kPairTile : TN;
    for (int j0 = 0; j0 < n; j0 += tn)
      for (int i0 = lower ? std::max(j0, i_start) : i_start; i0 < m; i0 += tm) {
        int klo = 0, khi = k;
        if (kt == KT_A_UPPER) klo = std::min(i0, k);
        else if (kt == KT_B_LOWER) khi = std::min(k, j0 + tn);
        else if (kt == KT_BOTH_UPPER) klo = std::min(std::max(i0, j0), k);
        if (khi <= klo) { klo = 0; khi = std::min(k, 1); }
        GemmTask t;
        t.a = a + int64_t(i0) * arow + klo;
        t.b = b + int64_t(j0) * brow + klo;
        t.c = c + int64_t(i0) * ldc + j0;
        t.lda = lda; t.ldb = ldb; t.ldc = ldc;
        t.m = std::min(tm, m - i0);
        t.n = std::min(tn, n - j0);
        t.k = khi - klo;
        if (pair) {
          t.pair = 1;
          t.amap = tma_source(op.abuf, abase, t.a, lda, &t.ax, &t.ay);
          t.bmap = tma_source(op.bbuf, bbase, t.b, ldb, &t.bx, &t.by);
        }
        s.gemm.push_back(t);
        s.ops.back().flops += 2.0 * t.m * t.n * t.k;
      }
  }
  // dst (ldd) <- src (lds), rows x cols of src, transposed or not, 32 x 32 per task
  void copy_tiles(int64_t src, int lds, int64_t dst, int ldd, int rows, int cols, bool trans) {
    for (int i0 = 0; i0 < rows; i0 += 32)
      for (int j0 = 0; j0 < cols; j0 += 32) {
        MirrorTask t;
        t.src = src + int64_t(i0) * lds + j0;
        t.dst = trans ? dst + int64_t(j0) * ldd + i0 : dst + int64_t(i0) * ldd + j0;
        t.lds = lds;
        t.ldd = ldd;
        t.rows = std::min(32, rows - i0);
        t.cols = std::min(32, cols - j0);
        t.trans = trans ? 1 : 0;
        s.mirror.push_back(t);
      }
  }
  void mirror_tiles(int64_t src, int64_t dst, int ld, int rows, int cols) { copy_tiles(src, ld, dst, ld, rows, cols, true); }
};

static inline int nblocks(int ns) { return (ns + kNbk - 1) / kNbk; }

static void build_factor_schedule(const Symbolic& S, Schedule& sc, int TM, int TN, bool pairs) {
  Builder b(sc, TM, TN, pairs);
  const auto& F = S.fronts;
  for (int d = S.max_depth; d >= 0; --d) {
    const auto& fr = S.by_depth[d];
    b.depth = d;
    const int pd = d & 1, pc = (d + 1) & 1;
    // zero this depth's update blocks
    int64_t used = 0;
    for (int f : fr) used = std::max(used, F[f].u_off + int64_t(F[f].nb) * F[f].ldu);
    if (used > 0) {
      Op& o = b.begin(OP_MEMSET);
      o.cbuf = pd == 0 ? B_P0 : B_P1;
      o.elems = used;
      b.end();
    }
    // extend-add of the children's update blocks, one launch per child rank
    for (int rank = 0; rank < 2; ++rank) {
      Op& o = b.begin(OP_EXTEND);
      o.abuf = pc == 0 ? B_P0 : B_P1;
      o.cbuf = pd == 0 ? B_P0 : B_P1;
      o.depth = d;
      for (int f : fr) {
        int c = F[f].child[rank];
        if (c < 0 || F[c].nb == 0) continue;
        // about 16k elements per block (row r holds r + 1): 8 rows of the long
        // rows, up to 128 of the short ones
        for (int r0 = 0; r0 < F[c].nb;) {
          const int rows = std::max(8, std::min(128, (16384 / (r0 + 1)) & ~7));
          const int r1 = std::min(F[c].nb, r0 + rows);
          sc.ext.push_back({c, r0, r1});
          o.nmax = std::max(o.nmax, r1);
          r0 = r1;
        }
      }
      b.end();
    }
    int steps = 0;
    for (int f : fr) steps = std::max(steps, nblocks(F[f].ns));
    for (int kb = 0; kb < steps; ++kb) {
      Op& od = b.begin(OP_DIAG);
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        DiagTask t;
        t.w = std::min(kNbk, x.ns - kb * kNbk);
        t.a = x.p_off + int64_t(kb) * kNbk * x.ld + kb * kNbk;
        t.dinv = x.d_off + int64_t(kb) * kNbk * kNbk;
        t.lda = x.ld;
        t.front = f;
        sc.diag.push_back(t);
      }
      b.end();
      // panel below the diagonal block: X = A Linv^T (in place)
      Op& ot = b.begin(OP_GEMM);
      ot.site = S_F_TRSM; ot.mode = kStore; ot.al = kRow; ot.bl = kRow;
      ot.abuf = B_L; ot.bbuf = B_DINV; ot.cbuf = B_L;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int r0 = kb * kNbk + w, rows = x.ns + x.nb - r0;
        int64_t a = x.p_off + int64_t(r0) * x.ld + kb * kNbk;
        b.gemm_tiles(a, x.ld, x.ld, x.d_off + int64_t(kb) * kNbk * kNbk, kNbk, kNbk, a, x.ld, rows, w, w);
      }
      b.end();
      // Updates inside this 512-column panel, by pairs of diagonal blocks (the
      // panel holds an even number of them): after the first block of a pair only
      // the next block column is updated (rank 64, look-ahead), after the second
      // the rest of the panel at once (rank 128).
      const int pstart = (kb * kNbk) / kPanel * kPanel, pend = pstart + kPanel;
      const bool first_of_pair = ((kb * kNbk - pstart) / kNbk) % 2 == 0;
      Op& ou = b.begin(OP_GEMM);
      ou.site = S_F_UPD; ou.mode = kSub; ou.al = kRow; ou.bl = kRow;
      ou.abuf = B_L; ou.bbuf = B_L; ou.cbuf = B_L;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int c0 = kb * kNbk + w, c1 = std::min(x.ns, pend);
        if (first_of_pair) c1 = std::min(c1, c0 + kNbk);
        if (c0 >= c1) continue;
        const int k0 = first_of_pair ? kb * kNbk : (kb - 1) * kNbk;  // first column of the update's K range
        int rows = x.ns + x.nb - c0, cols = c1 - c0;
        int64_t a = x.p_off + int64_t(c0) * x.ld + k0;
        b.gemm_tiles(a, x.ld, x.ld, a, x.ld, x.ld, x.p_off + int64_t(c0) * x.ld + c0, x.ld, rows, cols,
                     kb * kNbk + w - k0, true, 0, KT_NONE, x.p_off, x.p_off);
      }
      b.end();
      // at the end of a panel: one update of all later separator columns with K = panel width
      if ((kb + 1) * kNbk == pend) {
        Op& op = b.begin(OP_GEMM);
        op.site = S_F_UPD; op.mode = kSub; op.al = kRow; op.bl = kRow;
        op.abuf = B_L; op.bbuf = B_L; op.cbuf = B_L;
        for (int f : fr) {
          const Front& x = F[f];
          if (x.ns <= pend) continue;
          int rows = x.ns + x.nb - pend, cols = x.ns - pend;
          int64_t a = x.p_off + int64_t(pend) * x.ld + pstart;
          b.gemm_tiles(a, x.ld, x.ld, a, x.ld, x.ld, x.p_off + int64_t(pend) * x.ld + pend, x.ld, rows, cols,
                       kPanel, true, 0, KT_NONE, x.p_off, x.p_off);
        }
        b.end();
      }
    }
    // Schur complement of the rows below the separator: U -= P_B P_B^T
    Op& os = b.begin(OP_GEMM);
    os.site = S_F_SYRK; os.mode = kSub; os.al = kRow; os.bl = kRow;
    os.abuf = B_L; os.bbuf = B_L; os.cbuf = pd == 0 ? B_P0 : B_P1;
    for (int f : fr) {
      const Front& x = F[f];
      if (x.nb == 0) continue;
      int64_t a = x.p_off + int64_t(x.ns) * x.ld;
      b.gemm_tiles(a, x.ld, x.ld, a, x.ld, x.ld, x.u_off, x.ldu, x.nb, x.nb, x.ns, true, 0, KT_NONE, x.p_off, x.p_off);
    }
    b.end();
  }
}

// First completion flag of every front's 64-row blocks (one-column sweeps).
static std::vector<int64_t> chain_bases(const Symbolic& S, int64_t* total) {
  std::vector<int64_t> base(S.fronts.size());
  int64_t t = 0;
  for (size_t f = 0; f < S.fronts.size(); ++f) {
    base[f] = t;
    t += (S.fronts[f].ns + kNbk - 1) / kNbk;
  }
  if (total) *total = t;
  return base;
}

static void build_fwd_schedule(const Symbolic& S, Schedule& sc, int TM, int TN, int nrhs) {
  Builder b(sc, TM, TN);
  const auto& F = S.fronts;
  const std::vector<int64_t> chain_base = chain_bases(S, nullptr);
  const int chunk = std::max(1, std::min(nrhs, 16));
  for (int d = S.max_depth; d >= 0; --d) {
    const auto& fr = S.by_depth[d];
    b.depth = d;
    const int pd = d & 1;
    Op& og = b.begin(OP_SGATHER_FWD);
    og.depth = d;
    for (int f : fr)
      for (int r0 = 0; r0 < nrhs; r0 += chunk) sc.rows.push_back({f, r0, std::min(nrhs, r0 + chunk)});
    b.end();
    int steps = 0;
    for (int f : fr) steps = std::max(steps, nblocks(F[f].ns));
    if (nrhs == 1) {
      // one right-hand side: the level's block chain in one launch, then the
      // border rows in one product: W[B] -= L_B y
      Op& oc = b.begin(OP_FWD_CHAIN);
      oc.depth = d;
      for (int kb = 0; kb < steps; ++kb)
        for (int f : fr)
          if (F[f].ns > kb * kNbk) sc.rows.push_back({f, kb, int(chain_base[f])});
      b.end();
      Op& ob = b.begin(OP_GEMM);
      ob.site = S_V_FWD_B; ob.mode = kSub; ob.al = kRow; ob.bl = kCol;
      ob.abuf = B_L; ob.bbuf = B_X; ob.cbuf = pd == 0 ? B_W0 : B_W1;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.nb == 0 || x.ns == 0) continue;
        b.gemm_tiles(x.p_off + int64_t(x.ns) * x.ld, x.ld, x.ld, int64_t(x.s0), 1, 1, x.w_base, 1, x.nb, 1, x.ns);
      }
      b.end();
      continue;
    }
    for (int kb = 0; kb < steps; ++kb) {
      Op& o1 = b.begin(OP_GEMM);  // y_k = Linv_k x_k (in place)
      o1.site = S_V_FWD_D; o1.mode = kStore; o1.al = kRow; o1.bl = kCol;
      o1.abuf = B_DINV; o1.bbuf = B_X; o1.cbuf = B_X;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int64_t xo = int64_t(x.s0 + kb * kNbk) * nrhs;
        b.gemm_tiles(x.d_off + int64_t(kb) * kNbk * kNbk, kNbk, kNbk, xo, nrhs, 1, xo, nrhs, w, nrhs, w);
      }
      b.end();
      Op& o2 = b.begin(OP_GEMM);  // x[S below] -= L y_k
      o2.site = S_V_FWD_S; o2.mode = kSub; o2.al = kRow; o2.bl = kCol;
      o2.abuf = B_L; o2.bbuf = B_X; o2.cbuf = B_X;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int r0 = kb * kNbk + w;
        int64_t xo = int64_t(x.s0 + kb * kNbk) * nrhs;
        b.gemm_tiles(x.p_off + int64_t(r0) * x.ld + kb * kNbk, x.ld, x.ld, xo, nrhs, 1,
                     int64_t(x.s0 + r0) * nrhs, nrhs, x.ns - r0, nrhs, w);
      }
      b.end();
      Op& o3 = b.begin(OP_GEMM);  // W[B] -= L_B y_k
      o3.site = S_V_FWD_B; o3.mode = kSub; o3.al = kRow; o3.bl = kCol;
      o3.abuf = B_L; o3.bbuf = B_X; o3.cbuf = pd == 0 ? B_W0 : B_W1;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk || x.nb == 0) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int64_t xo = int64_t(x.s0 + kb * kNbk) * nrhs;
        b.gemm_tiles(x.p_off + int64_t(x.ns) * x.ld + kb * kNbk, x.ld, x.ld, xo, nrhs, 1, x.w_base * nrhs, nrhs,
                     x.nb, nrhs, w);
      }
      b.end();
    }
  }
}

static void build_bwd_schedule(const Symbolic& S, Schedule& sc, int TM, int TN, int nrhs) {
  Builder b(sc, TM, TN);
  const auto& F = S.fronts;
  const std::vector<int64_t> chain_base = chain_bases(S, nullptr);
  const int chunk = std::max(1, std::min(nrhs, 16));
  for (int d = 0; d <= S.max_depth; ++d) {
    const auto& fr = S.by_depth[d];
    b.depth = d;
    const int pd = d & 1;
    Op& og = b.begin(OP_SGATHER_BWD);
    og.depth = d;
    for (int f : fr)
      if (F[f].nb > 0)
        for (int r0 = 0; r0 < nrhs; r0 += chunk) sc.rows.push_back({f, r0, std::min(nrhs, r0 + chunk)});
    b.end();
    int steps = 0;
    for (int f : fr) steps = std::max(steps, nblocks(F[f].ns));
    if (nrhs == 1) {
      // one right-hand side: the level's block chain in one launch, each front's
      // blocks from its last one down; each block first takes its border term
      // -L_BS^T x_B, which depends on no other block
      Op& oc = b.begin(OP_BWD_CHAIN);
      oc.depth = d;
      for (int r = 0; r < steps; ++r)
        for (int f : fr) {
          const int kb = nblocks(F[f].ns) - 1 - r;
          if (kb >= 0) sc.rows.push_back({f, kb, int(chain_base[f])});
        }
      b.end();
      continue;
    }
    Op& o0 = b.begin(OP_GEMM);  // x_S -= L_BS^T x_B
    o0.site = S_V_BWD_0; o0.mode = kSub; o0.al = kCol; o0.bl = kCol;
    o0.abuf = B_L; o0.bbuf = pd == 0 ? B_G0 : B_G1; o0.cbuf = B_X;
    for (int f : fr) {
      const Front& x = F[f];
      if (x.nb == 0) continue;
      b.gemm_tiles(x.p_off + int64_t(x.ns) * x.ld, x.ld, 1, x.w_base * nrhs, nrhs, 1, int64_t(x.s0) * nrhs, nrhs, x.ns,
                   nrhs, x.nb);
    }
    b.end();
    for (int kb = steps - 1; kb >= 0; --kb) {
      Op& o1 = b.begin(OP_GEMM);  // x_k = Linv_k^T x_k
      o1.site = S_V_BWD_D; o1.mode = kStore; o1.al = kCol; o1.bl = kCol;
      o1.abuf = B_DINV; o1.bbuf = B_X; o1.cbuf = B_X;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int64_t xo = int64_t(x.s0 + kb * kNbk) * nrhs;
        b.gemm_tiles(x.d_off + int64_t(kb) * kNbk * kNbk, kNbk, 1, xo, nrhs, 1, xo, nrhs, w, nrhs, w);
      }
      b.end();
      if (kb == 0) continue;
      Op& o2 = b.begin(OP_GEMM);  // x[rows above] -= L[k, rows]^T x_k
      o2.site = S_V_BWD_U; o2.mode = kSub; o2.al = kCol; o2.bl = kCol;
      o2.abuf = B_L; o2.bbuf = B_X; o2.cbuf = B_X;
      for (int f : fr) {
        const Front& x = F[f];
        if (x.ns <= kb * kNbk) continue;
        int w = std::min(kNbk, x.ns - kb * kNbk);
        int64_t xo = int64_t(x.s0 + kb * kNbk) * nrhs;
        b.gemm_tiles(x.p_off + int64_t(kb) * kNbk * x.ld, x.ld, 1, xo, nrhs, 1, int64_t(x.s0) * nrhs, nrhs, kb * kNbk,
                     nrhs, w);
      }
      b.end();
    }
  }
}

// Selected inversion, top-down over depths.  Per front (S = separator rows, B =
// the rows below it, L = [L_SS; L_BS]), with Z_BB gathered from the parent:
//   W   = L_SS^-1                 (recursive halving of the 64-blocks, below)
//   X^T = W^T L_BS^T              (S x B)
//   Z_SB = -X^T Z_BB,             Z_BS = Z_SB^T
//   Z_SS = W^T W - X^T Z_SB^T     (lower tiles, then mirrored)
// i.e. the Takahashi recursion Z_BS = -Z_BB L_BS L_SS^-1,
// Z_SS = (L_SS L_SS^T)^-1 - (L_BS L_SS^-1)^T Z_BS, written so that every product
// reads its operands row by row (K contiguous).  W and W^T are both kept
// (row-major); for a node [a, b) of the halving tree with children [a, m), [m, b):
//   TT = W_11^T L_21^T,  (W^T)_12 = -TT W_22^T,  W_21 = ((W^T)_12)^T.
static void build_selinv_schedule(const Symbolic& S, Schedule& sc, int TM, int TN, int64_t* scratch_elems,
                                  bool pairs) {
  Builder b(sc, TM, TN, pairs);
  const auto& F = S.fronts;
  auto r4 = [](int64_t v) { return (v + 3) / 4 * 4; };
  int64_t scratch = 32;
  for (int d = 0; d <= S.max_depth; ++d) {
    const auto& fr = S.by_depth[d];
    b.depth = d;
    const int pz = (d & 1) ? B_P1 : B_P0;
    // scratch layout of this depth: W, W^T, X^T, TT per front
    struct Sx { int64_t w, wt, xt, tt; int ldw, ldx; std::vector<std::vector<std::array<int, 3>>> levels; };
    std::vector<Sx> sx(fr.size());
    int64_t off = 0;
    int maxlev = 0;
    for (size_t q = 0; q < fr.size(); ++q) {
      const Front& x = F[fr[q]];
      Sx& z = sx[q];
      z.ldw = int(r4(x.ns));
      z.ldx = int(r4(std::max(x.nb, 1)));
      z.w = off; off += int64_t(x.ns) * z.ldw;
      z.wt = off; off += int64_t(x.ns) * z.ldw;
      z.xt = off; off += int64_t(x.ns) * z.ldx;
      // halving tree over the 64-blocks; levels[L] = nodes (a, m, b) at recursion depth L
      const int nblk = nblocks(x.ns);
      std::vector<std::array<int, 4>> stack{{0, nblk, 0, 0}};
      while (!stack.empty()) {
        auto nd = stack.back();
        stack.pop_back();
        const int a = nd[0], e = nd[1], L = nd[2];
        if (e - a < 2) continue;
        const int m = a + (e - a) / 2;
        if (int(z.levels.size()) <= L) z.levels.resize(L + 1);
        z.levels[L].push_back({a, m, e});
        stack.push_back({a, m, L + 1, 0});
        stack.push_back({m, e, L + 1, 0});
      }
      maxlev = std::max(maxlev, int(z.levels.size()));
      int64_t tt_need = 0;
      for (auto& lv : z.levels) {
        int64_t sum = 0;
        for (auto& nd : lv) {
          const int64_t r0 = int64_t(nd[0]) * kNbk, r1 = int64_t(nd[1]) * kNbk;
          const int64_t c0 = r1, c1 = std::min<int64_t>(int64_t(nd[2]) * kNbk, x.ns);
          sum += (r1 - r0) * r4(c1 - c0);
        }
        tt_need = std::max(tt_need, sum);
      }
      z.tt = off; off += tt_need;
      off = (off + 31) / 32 * 32;
    }
    scratch = std::max(scratch, off);
    {
      Op& o = b.begin(OP_ZGATHER);
      o.depth = d;
      for (int f : fr) {
        if (F[f].nb == 0) continue;
        for (int r0 = 0; r0 < F[f].nb; r0 += 8) sc.rows.push_back({f, r0, std::min(F[f].nb, r0 + 8)});
      }
      b.end();
    }
    {  // W, W^T start as zero, then take the inverse diagonal blocks
      Op& o = b.begin(OP_MEMSET);
      o.cbuf = B_SX;
      o.elems = off;
      b.end();
      Op& oc = b.begin(OP_MIRROR);
      oc.abuf = B_DINV; oc.cbuf = B_SX;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        for (int kb = 0; kb < nblocks(x.ns); ++kb) {
          const int w = std::min(kNbk, x.ns - kb * kNbk);
          const int64_t src = x.d_off + int64_t(kb) * kNbk * kNbk;
          const int64_t dw = sx[q].w + int64_t(kb) * kNbk * sx[q].ldw + kb * kNbk;
          const int64_t dwt = sx[q].wt + int64_t(kb) * kNbk * sx[q].ldw + kb * kNbk;
          b.copy_tiles(src, kNbk, dw, sx[q].ldw, w, w, false);
          b.copy_tiles(src, kNbk, dwt, sx[q].ldw, w, w, true);
        }
      }
      b.end();
    }
    for (int L = maxlev - 1; L >= 0; --L) {
      std::vector<int64_t> ttoff(fr.size(), 0);
      Op& o1 = b.begin(OP_GEMM);  // TT = W_11^T L_21^T
      o1.site = S_Z_XSOLVE; o1.mode = kStore; o1.al = kRow; o1.bl = kRow;
      o1.abuf = B_SX; o1.bbuf = B_L; o1.cbuf = B_SX;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (int(sx[q].levels.size()) <= L) continue;
        int64_t to = sx[q].tt;
        for (auto& nd : sx[q].levels[L]) {
          const int r0 = nd[0] * kNbk, r1 = nd[1] * kNbk, c1 = std::min(nd[2] * kNbk, x.ns);
          const int ldt = int(r4(c1 - r1));
          b.gemm_tiles(sx[q].wt + int64_t(r0) * sx[q].ldw + r0, sx[q].ldw, sx[q].ldw,
                       x.p_off + int64_t(r1) * x.ld + r0, x.ld, x.ld, to, ldt, r1 - r0, c1 - r1, r1 - r0, false, 0,
                       KT_A_UPPER);
          to += int64_t(r1 - r0) * ldt;
        }
      }
      b.end();
      Op& o2 = b.begin(OP_GEMM);  // (W^T)_12 = -TT W_22^T
      o2.site = S_Z_XUPD; o2.mode = kNegStore; o2.al = kRow; o2.bl = kRow;
      o2.abuf = B_SX; o2.bbuf = B_SX; o2.cbuf = B_SX;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (int(sx[q].levels.size()) <= L) continue;
        int64_t to = sx[q].tt;
        for (auto& nd : sx[q].levels[L]) {
          const int r0 = nd[0] * kNbk, r1 = nd[1] * kNbk, c1 = std::min(nd[2] * kNbk, x.ns);
          const int ldt = int(r4(c1 - r1));
          b.gemm_tiles(to, ldt, ldt, sx[q].w + int64_t(r1) * sx[q].ldw + r1, sx[q].ldw, sx[q].ldw,
                       sx[q].wt + int64_t(r0) * sx[q].ldw + r1, sx[q].ldw, r1 - r0, c1 - r1, c1 - r1, false, 0,
                       KT_B_LOWER);
          to += int64_t(r1 - r0) * ldt;
        }
      }
      b.end();
      Op& om = b.begin(OP_MIRROR);  // W_21 = ((W^T)_12)^T
      om.abuf = B_SX; om.cbuf = B_SX;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (int(sx[q].levels.size()) <= L) continue;
        for (auto& nd : sx[q].levels[L]) {
          const int r0 = nd[0] * kNbk, r1 = nd[1] * kNbk, c1 = std::min(nd[2] * kNbk, x.ns);
          b.copy_tiles(sx[q].wt + int64_t(r0) * sx[q].ldw + r1, sx[q].ldw, sx[q].w + int64_t(r1) * sx[q].ldw + r0,
                       sx[q].ldw, r1 - r0, c1 - r1, true);
        }
      }
      b.end();
    }
    {  // X^T = W^T L_BS^T
      Op& o = b.begin(OP_GEMM);
      o.site = S_Z_XJ; o.mode = kStore; o.al = kRow; o.bl = kRow;
      o.abuf = B_SX; o.bbuf = B_L; o.cbuf = B_SX;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (x.nb == 0) continue;
        b.gemm_tiles(sx[q].wt, sx[q].ldw, sx[q].ldw, x.p_off + int64_t(x.ns) * x.ld, x.ld, x.ld, sx[q].xt, sx[q].ldx,
                     x.ns, x.nb, x.ns, false, 0, KT_A_UPPER, sx[q].wt, x.p_off);
      }
      b.end();
    }
    {  // Z_SB = -X^T Z_BB
      Op& o = b.begin(OP_GEMM);
      o.site = S_Z_BS; o.mode = kNegStore; o.al = kRow; o.bl = kRow;
      o.abuf = B_SX; o.bbuf = pz; o.cbuf = pz;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (x.nb == 0) continue;
        b.gemm_tiles(sx[q].xt, sx[q].ldx, sx[q].ldx, x.z_off + int64_t(x.ns) * x.ldz + x.ns, x.ldz, x.ldz,
                     x.z_off + x.ns, x.ldz, x.ns, x.nb, x.nb, false, 0, KT_NONE, sx[q].xt, x.z_off);
      }
      b.end();
    }
    {  // Z_SS = W^T W (lower tiles), then -= X^T Z_SB^T
      Op& o = b.begin(OP_GEMM);
      o.site = S_Z_JJ; o.mode = kStore; o.al = kRow; o.bl = kRow;
      o.abuf = B_SX; o.bbuf = B_SX; o.cbuf = pz;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        b.gemm_tiles(sx[q].wt, sx[q].ldw, sx[q].ldw, sx[q].wt, sx[q].ldw, sx[q].ldw, x.z_off, x.ldz, x.ns, x.ns, x.ns,
                     true, 0, KT_BOTH_UPPER, sx[q].wt, sx[q].wt);
      }
      b.end();
      Op& o2 = b.begin(OP_GEMM);
      o2.site = S_Z_SS; o2.mode = kSub; o2.al = kRow; o2.bl = kRow;
      o2.abuf = B_SX; o2.bbuf = pz; o2.cbuf = pz;
      for (size_t q = 0; q < fr.size(); ++q) {
        const Front& x = F[fr[q]];
        if (x.nb == 0) continue;
        b.gemm_tiles(sx[q].xt, sx[q].ldx, sx[q].ldx, x.z_off + x.ns, x.ldz, x.ldz, x.z_off, x.ldz, x.ns, x.ns, x.nb,
                     true, 0, KT_NONE, sx[q].xt, x.z_off);
      }
      b.end();
    }
    {  // upper triangle of Z_SS from the strictly lower tiles; Z_BS = Z_SB^T
      Op& om = b.begin(OP_MIRROR);
      om.abuf = pz; om.cbuf = pz;
      for (int f : fr) {
        const Front& x = F[f];
        for (int j0 = 0; j0 < x.ns; j0 += TN)
          for (int i0 = j0 + TM; i0 < x.ns; i0 += TM) {
            const int rows = std::min(TM, x.ns - i0), cols = std::min(TN, x.ns - j0);
            b.copy_tiles(x.z_off + int64_t(i0) * x.ldz + j0, x.ldz, x.z_off + int64_t(j0) * x.ldz + i0, x.ldz, rows,
                         cols, true);
          }
        if (x.nb > 0)
          b.copy_tiles(x.z_off + x.ns, x.ldz, x.z_off + int64_t(x.ns) * x.ldz, x.ldz, x.ns, x.nb, true);
      }
      b.end();
    }
    {
      Op& o = b.begin(OP_ZEXTRACT);
      o.depth = d;
      o.cbuf = pz;
      for (int f : fr)
        for (int r0 = 0; r0 < F[f].ns; r0 += 32) sc.rows.push_back({f, r0, std::min(F[f].ns, r0 + 32)});
      b.end();
    }
  }
  *scratch_elems = scratch;
}

// ------------------------------------------------------ one-column sweeps
// The forward and backward substitutions of one tree level for a single right-
// hand side, as one launch each instead of two launches per 64-column block:
// block (front f, block k) of the level is a CTA that takes a ticket (so that
// every block it waits for belongs to a CTA that has already started), folds in
// the blocks it depends on as their completion flags appear, solves with the
// 64 x 64 block inverse and publishes its flag.  Flags carry the sweep's epoch,
// so they need no reset.  A wait gives up after wait_ns (the solve then reports
// an error instead of hanging).
__device__ __forceinline__ unsigned long long chain_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool chain_wait(const unsigned* flag, unsigned epoch, unsigned long long wait_ns) {
  auto done = [&]() {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    return int(v - epoch) >= 0;
  };
  if (done()) return true;
  const unsigned long long t0 = chain_now();
  while (!done()) {
    if (chain_now() - t0 > wait_ns) return false;
    __nanosleep(64);
  }
  return true;
}
__device__ __forceinline__ void chain_publish(unsigned* flag, unsigned epoch) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(flag), "r"(epoch) : "memory");
}
template <typename T>
__device__ __forceinline__ T load_cg(const T* p) {
  return __ldcg(p);
}

// Forward: y_k = Linv_k (x_k - sum_{j<k} L_kj y_j) in place in X (tasks: front,
// block k, flag base of the front; sorted by k).  Thread (row i, quarter q).
template <typename T>
__global__ void __launch_bounds__(256) fwd_chain_kernel(const RowTask* __restrict__ tasks,
                                                        const DevFront* __restrict__ fronts, const T* __restrict__ L,
                                                        const T* __restrict__ dinv, T* __restrict__ X,
                                                        unsigned* __restrict__ flags, unsigned* __restrict__ counter,
                                                        unsigned epoch, int* __restrict__ err,
                                                        unsigned long long wait_ns) {
  __shared__ T sD[64][65];
  __shared__ T ys[64], acc[64];
  __shared__ int ticket, fail;
  const int tid = threadIdx.x, i = tid >> 2, q = tid & 3;
  if (tid == 0) {
    ticket = int(atomicAdd(counter, 1u));
    fail = 0;
  }
  __syncthreads();
  const RowTask tk = tasks[ticket];
  const DevFront f = fronts[tk.front];
  const int k = tk.r0, r0 = k * 64, w = min(64, f.ns - r0);
  const T* Lrow = L + f.p_off + int64_t(r0 + (i < w ? i : 0)) * f.ld + q * 16;
  for (int e = tid; e < 64 * 64; e += 256) {
    const int a = e >> 6, b = e & 63;
    sD[a][b] = (a < w && b < w) ? dinv[f.d_off + int64_t(k) * 64 * 64 + e] : T(0);
  }
  T part = 0;
  for (int j = 0; j < k; ++j) {
    if (tid == 0 && !chain_wait(flags + tk.r1 + j, epoch, wait_ns)) {
      fail = 1;
      atomicExch(err, 1);
    }
    __syncthreads();
    if (tid < 64) ys[tid] = load_cg(X + f.s0 + j * 64 + tid);
    __syncthreads();
    if (fail) break;
#pragma unroll
    for (int c = 0; c < 16; ++c) part += Lrow[j * 64 + c] * ys[q * 16 + c];
  }
  part += __shfl_xor_sync(0xffffffffu, part, 1);
  part += __shfl_xor_sync(0xffffffffu, part, 2);
  if (q == 0) acc[i] = i < w ? X[f.s0 + r0 + i] - part : T(0);
  __syncthreads();
  T y = 0;
#pragma unroll
  for (int c = 0; c < 16; ++c) y += sD[i][q * 16 + c] * acc[q * 16 + c];
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  if (q == 0 && i < w) {
    X[f.s0 + r0 + i] = y;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) chain_publish(flags + tk.r1 + k, epoch);
}

// Backward: x_k = Linv_k^T (x_k - L_Bk^T x_B - sum_{j>k} L_jk^T x_j) in place in
// X (tasks sorted by the distance of k from the front's last block; x_B, the
// border rows' solution from the parent, in G).  Thread (column c, row group g
// of eight): the border term, which depends on no other block, comes first.
template <typename T>
__global__ void __launch_bounds__(512) bwd_chain_kernel(const RowTask* __restrict__ tasks,
                                                        const DevFront* __restrict__ fronts, const T* __restrict__ L,
                                                        const T* __restrict__ dinv, T* __restrict__ X,
                                                        const T* __restrict__ G, unsigned* __restrict__ flags,
                                                        unsigned* __restrict__ counter, unsigned epoch,
                                                        int* __restrict__ err, unsigned long long wait_ns) {
  __shared__ T sD[64][65];
  __shared__ T xs[64], acc[64], red[8][64];
  __shared__ int ticket, fail;
  const int tid = threadIdx.x, c = tid & 63, g = tid >> 6;
  if (tid == 0) {
    ticket = int(atomicAdd(counter, 1u));
    fail = 0;
  }
  __syncthreads();
  const RowTask tk = tasks[ticket];
  const DevFront f = fronts[tk.front];
  const int k = tk.r0, c0 = k * 64, w = min(64, f.ns - c0);
  const int nbk = (f.ns + 63) / 64;
  for (int e = tid; e < 64 * 64; e += 512) {
    const int a = e >> 6, b = e & 63;
    sD[a][b] = (a < w && b < w) ? dinv[f.d_off + int64_t(k) * 64 * 64 + e] : T(0);
  }
  // border rows: FP32 rows with 16-byte aligned columns and the block's 64
  // columns inside the row are read as float4 (thread: 4 columns, row group of
  // 32, four rows in flight), the others one column per thread (row group of 8,
  // eight rows in flight); either way a block sum per column lands in bsum
  __shared__ T bsum[64];
  T part = 0;
  const T* xb = G + f.w_base;
  const bool vec = sizeof(T) == 4 && ((f.p_off | f.ld) & 3) == 0 && c0 + 64 <= f.ld;
  if (f.nb > 0 && vec) {
    __shared__ float red32[32][65];
    const int cq = tid & 15, g2 = tid >> 4;
    const float* Lb = reinterpret_cast<const float*>(L) + f.p_off + int64_t(f.ns) * f.ld + c0 + 4 * cq;
    const float* xf = reinterpret_cast<const float*>(xb);
    float4 s4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    int b = g2;
    for (; b + 96 < f.nb; b += 128) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 l = *reinterpret_cast<const float4*>(Lb + int64_t(b + 32 * u) * f.ld);
        const float xv = xf[b + 32 * u];
        s4[u].x += l.x * xv; s4[u].y += l.y * xv; s4[u].z += l.z * xv; s4[u].w += l.w * xv;
      }
    }
    for (; b < f.nb; b += 32) {
      const float4 l = *reinterpret_cast<const float4*>(Lb + int64_t(b) * f.ld);
      const float xv = xf[b];
      s4[0].x += l.x * xv; s4[0].y += l.y * xv; s4[0].z += l.z * xv; s4[0].w += l.w * xv;
    }
    red32[g2][4 * cq + 0] = (s4[0].x + s4[1].x) + (s4[2].x + s4[3].x);
    red32[g2][4 * cq + 1] = (s4[0].y + s4[1].y) + (s4[2].y + s4[3].y);
    red32[g2][4 * cq + 2] = (s4[0].z + s4[1].z) + (s4[2].z + s4[3].z);
    red32[g2][4 * cq + 3] = (s4[0].w + s4[1].w) + (s4[2].w + s4[3].w);
    __syncthreads();
    if (tid < 64) {
      float t = 0.f;
#pragma unroll 8
      for (int h = 0; h < 32; ++h) t += red32[h][tid];
      bsum[tid] = T(t);
    }
  } else if (f.nb > 0) {
    if (c < w) {
      const T* Lb = L + f.p_off + int64_t(f.ns) * f.ld + c0 + c;
      T s8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      int b = g;
      for (; b + 56 < f.nb; b += 64) {
#pragma unroll
        for (int u = 0; u < 8; ++u) s8[u] += Lb[int64_t(b + 8 * u) * f.ld] * xb[b + 8 * u];
      }
      for (; b < f.nb; b += 8) s8[0] += Lb[int64_t(b) * f.ld] * xb[b];
      part = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
    }
    if (tid < 64) bsum[tid] = T(0);
  } else if (tid < 64) {
    bsum[tid] = T(0);
  }
  for (int j = nbk - 1; j > k; --j) {
    const int wj = min(64, f.ns - j * 64);
    if (tid == 0 && !chain_wait(flags + tk.r1 + j, epoch, wait_ns)) {
      fail = 1;
      atomicExch(err, 1);
    }
    __syncthreads();
    if (tid < 64) xs[tid] = tid < wj ? load_cg(X + f.s0 + j * 64 + tid) : T(0);
    __syncthreads();
    if (fail) break;
    if (c < w) {
      const T* Lj = L + f.p_off + int64_t(j * 64 + g * 8) * f.ld + c0 + c;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (g * 8 + i < wj) part += Lj[int64_t(i) * f.ld] * xs[g * 8 + i];
    }
  }
  red[g][c] = part;
  __syncthreads();
  if (tid < 64) {
    T t = bsum[tid];
#pragma unroll
    for (int h = 0; h < 8; ++h) t += red[h][tid];
    acc[tid] = tid < w ? X[f.s0 + c0 + tid] - t : T(0);
  }
  __syncthreads();
  T x = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) x += sD[g * 8 + i][c] * acc[g * 8 + i];
  red[g][c] = x;
  __syncthreads();
  if (tid < w) {
    T t = 0;
#pragma unroll
    for (int h = 0; h < 8; ++h) t += red[h][tid];
    X[f.s0 + c0 + tid] = t;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) chain_publish(flags + tk.r1 + k, epoch);
}

// ------------------------------------------------------------ small kernels
template <typename T>
__global__ void sgather_fwd_kernel(const RowTask* __restrict__ tasks, const DevFront* __restrict__ F,
                                   const int* __restrict__ rmap, T* __restrict__ X, T* __restrict__ Wd,
                                   const T* __restrict__ Wc, int nrhs) {
  const RowTask tk = tasks[blockIdx.x];
  const DevFront f = F[tk.front];
  const int nr = tk.r1 - tk.r0;
  T* W = Wd + f.w_base * nrhs;
  for (int e = threadIdx.x; e < f.nb * nr; e += blockDim.x) W[int64_t(e / nr) * nrhs + tk.r0 + e % nr] = T(0);
  __syncthreads();
  for (int ci = 0; ci < 2; ++ci) {
    if (f.child[ci] < 0) continue;
    const DevFront c = F[f.child[ci]];
    const int* rm = rmap + c.b_off;
    const T* Wch = Wc + c.w_base * nrhs;
    for (int e = threadIdx.x; e < c.nb * nr; e += blockDim.x) {
      int bi = e / nr, r = tk.r0 + e % nr;
      int pos = rm[bi];
      T v = Wch[int64_t(bi) * nrhs + r];
      if (pos < f.ns) X[int64_t(f.s0 + pos) * nrhs + r] += v;
      else W[int64_t(pos - f.ns) * nrhs + r] += v;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void sgather_bwd_kernel(const RowTask* __restrict__ tasks, const DevFront* __restrict__ F,
                                   const int* __restrict__ blist, const T* __restrict__ X, T* __restrict__ G,
                                   int nrhs) {
  const RowTask tk = tasks[blockIdx.x];
  const DevFront f = F[tk.front];
  const int nr = tk.r1 - tk.r0;
  const int* bl = blist + f.b_off;
  T* Gf = G + f.w_base * nrhs;
  for (int e = threadIdx.x; e < f.nb * nr; e += blockDim.x) {
    int bi = e / nr, r = tk.r0 + e % nr;
    Gf[int64_t(bi) * nrhs + r] = X[int64_t(bl[bi]) * nrhs + r];
  }
}

template <typename T>
__global__ void zgather_kernel(const RowTask* __restrict__ tasks, const DevFront* __restrict__ F,
                               const int* __restrict__ rmap, const T* __restrict__ Zp, T* __restrict__ Zc) {
  const RowTask tk = tasks[blockIdx.x];
  const DevFront f = F[tk.front];
  const DevFront p = F[f.parent];
  const int* rm = rmap + f.b_off;
  // one warp per row (up to 8 rows per task), four independent elements in
  // flight per lane: the gather is latency-bound otherwise
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = tk.r0 + warp;
  if (a >= tk.r1) return;
  const T* src = Zp + p.z_off + int64_t(rm[a]) * p.ldz;
  T* dst = Zc + f.z_off + int64_t(f.ns + a) * f.ldz + f.ns;
  int bcol = lane;
  for (; bcol + 96 < f.nb; bcol += 128) {
    const int c0 = rm[bcol], c1 = rm[bcol + 32], c2 = rm[bcol + 64], c3 = rm[bcol + 96];
    const T v0 = src[c0], v1 = src[c1], v2 = src[c2], v3 = src[c3];
    dst[bcol] = v0;
    dst[bcol + 32] = v1;
    dst[bcol + 64] = v2;
    dst[bcol + 96] = v3;
  }
  for (; bcol < f.nb; bcol += 32) dst[bcol] = src[rm[bcol]];
}

// 32 x 32 block copies, kMirrorTiles tasks per CTA: all their loads first, then
// all their stores, so that a CTA keeps several tiles in flight (the tasks of one
// launch never read what another writes)
constexpr int kMirrorTiles = 4;
template <typename T>
__global__ void mirror_kernel(const MirrorTask* __restrict__ tasks, int ntasks, const T* src, T* dst) {
  __shared__ T tile[kMirrorTiles][32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int t0 = blockIdx.x * kMirrorTiles;
#pragma unroll
  for (int u = 0; u < kMirrorTiles; ++u) {
    if (t0 + u >= ntasks) break;
    const MirrorTask tk = tasks[t0 + u];
    for (int i = ty; i < 32; i += 8)
      if (i < tk.rows && tx < tk.cols) tile[u][i][tx] = src[tk.src + int64_t(i) * tk.lds + tx];
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kMirrorTiles; ++u) {
    if (t0 + u >= ntasks) break;
    const MirrorTask tk = tasks[t0 + u];
    if (tk.trans) {
      for (int j = ty; j < 32; j += 8)
        if (j < tk.cols && tx < tk.rows) dst[tk.dst + int64_t(j) * tk.ldd + tx] = tile[u][tx][j];
    } else {
      for (int i = ty; i < 32; i += 8)
        if (i < tk.rows && tx < tk.cols) dst[tk.dst + int64_t(i) * tk.ldd + tx] = tile[u][i][tx];
    }
  }
}

template <typename T>
__global__ void zextract_kernel(const RowTask* __restrict__ tasks, const DevFront* __restrict__ F,
                                const int* __restrict__ iperm, const int* __restrict__ amap, int nslots,
                                const T* __restrict__ Z, double* __restrict__ zq) {
  const RowTask tk = tasks[blockIdx.x];
  const DevFront f = F[tk.front];
  const int cnt = (tk.r1 - tk.r0) * nslots;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    int v = f.s0 + tk.r0 + e / nslots, s = e % nslots;
    int k = iperm[v];
    int off = amap[int64_t(k) * nslots + s];
    if (off < 0) continue;
    int row = off / f.ld, col = off - row * f.ld;
    zq[int64_t(k) * nslots + s] = double(Z[f.z_off + int64_t(row) * f.ldz + col]);
  }
}

__global__ void zsym_kernel(int Mx, int Ny, int T, int nslots, const int* __restrict__ amap, double* __restrict__ zq) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = int64_t(Mx) * Ny * T;
  if (e >= n * nslots) return;
  if (amap[e] >= 0) return;
  const int k = int(e / nslots), s = int(e % nslots);
  int dx, dy, dt;
  stencil_slot(nslots, s, &dx, &dy, &dt);
  const int t = k / (Mx * Ny), c = k - t * Mx * Ny, y = c / Mx, x = c - y * Mx;
  if (x + dx < 0 || x + dx >= Mx || y + dy < 0 || y + dy >= Ny || t + dt < 0 || t + dt >= T) {
    zq[e] = 0.0;
    return;
  }
  const int64_t nb = (int64_t(t + dt) * Ny + y + dy) * Mx + x + dx;
  const int opp = nslots - 1 - s;  // every layout is symmetric under (dx, dy, dt) -> -(dx, dy, dt)
  zq[e] = zq[nb * nslots + opp];
}

// Sum of the log pivots (FP64, fixed order: strided per thread, then a warp
// shuffle tree, then the eight warp sums in order), one block of 256 threads.
__global__ void sum_kernel(const double* __restrict__ v, int64_t n, double* __restrict__ out) {
  __shared__ double warp_sum[8];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += v[i];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += warp_sum[w];
    *out = t;
  }
}

// r = b - r (in place on r), and partial sums of |r|^2 and |b|^2
__global__ void resid_kernel(const double* __restrict__ b, double* __restrict__ r, int64_t n,
                             double* __restrict__ part) {
  __shared__ double s1[256], s2[256];
  double a1 = 0.0, a2 = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * 256 + threadIdx.x; i < n; i += int64_t(gridDim.x) * 256) {
    double v = b[i] - r[i];
    r[i] = v;
    a1 += v * v;
    a2 += b[i] * b[i];
  }
  s1[threadIdx.x] = a1;
  s2[threadIdx.x] = a2;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) { s1[threadIdx.x] += s1[threadIdx.x + k]; s2[threadIdx.x] += s2[threadIdx.x + k]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = s1[0]; part[2 * blockIdx.x + 1] = s2[0]; }
}

// -------------------------------------------------------- per-launch timing
static void prof_begin(Plan* p, cudaStream_t st) {
  if (p->ev_used + 2 > p->ev_pool.size()) {
    for (int i = 0; i < 512; ++i) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      p->ev_pool.push_back(e);
    }
  }
  cudaEventRecord(p->ev_pool[p->ev_used], st);
}
static void prof_end(Plan* p, cudaStream_t st, int kind, double flops, int site, int tiles) {
  cudaEventRecord(p->ev_pool[p->ev_used + 1], st);
  p->ev_pending.push_back({kind, flops});
  p->ev_site.push_back(site | (tiles << 8));
  p->ev_used += 2;
}
// Fold the recorded event pairs into the per-kind totals (synchronises).
void prof_collect(Plan* p) {
  if (p->ev_pending.empty()) return;
  cudaStreamSynchronize(p->stream);
  for (size_t i = 0; i < p->ev_pending.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev_pool[2 * i], p->ev_pool[2 * i + 1]);
    int k = p->ev_pending[i].first;
    p->prof_ms[k] += ms;
    p->prof_flops[k] += p->ev_pending[i].second;
    p->prof_count[k] += 1;
    const int site = p->ev_site[i] & 255;
    if (site > 0 && site < S_COUNT) {
      p->site_ms[site] += ms;
      p->site_flops[site] += p->ev_pending[i].second;
      p->site_tiles[site] += p->ev_site[i] >> 8;
    }
  }
  p->ev_pending.clear();
  p->ev_site.clear();
  p->ev_used = 0;
}

// Optional launch log of the tensor-core tiled product: with SPDE_LAUNCH_LOG set
// to a file name, one line per launch (process-wide launch number, call site,
// tasks, algorithmic flops, path: 1 single-CTA tiles, 4 cluster pairs), so that
// a profiler capture of the n-th launch can be matched with the work it did.
// Host-side bookkeeping only.
static void tc_launch_log(const Op& o) {
  static std::mutex mu;
  static FILE* fh = nullptr;
  static bool opened = false;
  static int64_t seq = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (!opened) {
    opened = true;
    const char* path = std::getenv("SPDE_LAUNCH_LOG");
    if (path && *path) fh = std::fopen(path, "w");
    if (fh) std::fprintf(fh, "launch site tiles flops path\n");
  }
  if (fh) {
    std::fprintf(fh, "%lld %d %d %.0f %d\n", static_cast<long long>(seq), o.site, o.count, o.flops, o.tc);
    std::fflush(fh);
  }
  ++seq;
}

// ------------------------------------------------------------------ executor
template <typename T>
struct Exec {
  Plan* p;
  const Schedule& s;
  int nrhs;
  double* zq;
  T* buf(int id) const {
    switch (id) {
      case B_L: return static_cast<T*>(p->d_L);
      case B_DINV: return static_cast<T*>(p->d_dinv);
      case B_P0: return static_cast<T*>(p->d_pool[0]);
      case B_P1: return static_cast<T*>(p->d_pool[1]);
      case B_X: return static_cast<T*>(p->d_X);
      case B_W0: return static_cast<T*>(p->d_W[0]);
      case B_W1: return static_cast<T*>(p->d_W[1]);
      case B_G0: return static_cast<T*>(p->d_G[0]);
      case B_G1: return static_cast<T*>(p->d_G[1]);
      case B_SX: return static_cast<T*>(p->d_sx);
      default: return nullptr;
    }
  }
  void run() {
    cudaStream_t st = p->stream;
    // optional per-depth timeline (SPDE_PHASE_LOG): an event at every change of depth
    static const bool depth_log = std::getenv("SPDE_PHASE_LOG") != nullptr;
    std::vector<std::pair<int, cudaEvent_t>> dmarks;
    auto dmark = [&](int d) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      cudaEventRecord(e, st);
      dmarks.emplace_back(d, e);
    };
    for (const Op& o : s.ops) {
      if (depth_log && (dmarks.empty() || dmarks.back().first != o.depth)) dmark(o.depth);
      const bool on_tc = o.kind == OP_GEMM && sizeof(T) == sizeof(float) &&
                         ((o.tc == kPathTensor && tc_gemm_enabled()) || o.tc == kPathPair);
      const bool timed = p->profile && o.kind != OP_MEMSET && (on_tc || !p->profile_tc_only);
      if (timed) prof_begin(p, st);
      switch (o.kind) {
        case OP_MEMSET: cudaMemsetAsync(buf(o.cbuf), 0, size_t(o.elems) * sizeof(T), st); break;
        case OP_EXTEND:
          launch_extend_add<T>(s.d_ext + o.off, o.count, p->d_fronts, p->d_rmap, buf(o.abuf), buf(B_L), buf(o.cbuf),
                               o.nmax, st);
          break;
        case OP_DIAG:
          launch_potrf<T>(s.d_diag + o.off, o.count, buf(B_L), buf(B_DINV), p->d_logpiv + o.off, p->d_err, st);
          break;
        case OP_GEMM:
          if constexpr (sizeof(T) == sizeof(float)) {
            if (o.tc == kPathPair) {
              launch_gemm_pair(s.d_gemm + o.off, o.count, s.d_maps, buf(o.abuf), buf(o.bbuf), buf(o.cbuf), o.mode, st,
                               p->tc_wait_ns);
              tc_launch_log(o);
              break;
            }
          }
          launch_gemm<T>(s.d_gemm + o.off, o.count, buf(o.abuf), buf(o.bbuf), buf(o.cbuf), o.mode, o.al, o.bl, st,
                         o.tc, o.nmax, p->tc_wait_ns);
          if (on_tc) tc_launch_log(o);
          break;
        case OP_SGATHER_FWD: {
          int pd = o.depth & 1;
          sgather_fwd_kernel<T><<<o.count, 256, 0, st>>>(s.d_rows + o.off, p->d_fronts, p->d_rmap, buf(B_X),
                                                         buf(pd ? B_W1 : B_W0), buf(pd ? B_W0 : B_W1), nrhs);
          break;
        }
        case OP_SGATHER_BWD: {
          int pd = o.depth & 1;
          sgather_bwd_kernel<T><<<o.count, 256, 0, st>>>(s.d_rows + o.off, p->d_fronts, p->d_blist, buf(B_X),
                                                         buf(pd ? B_G1 : B_G0), nrhs);
          break;
        }
        case OP_ZGATHER: {
          int pd = o.depth & 1;
          zgather_kernel<T><<<o.count, 256, 0, st>>>(s.d_rows + o.off, p->d_fronts, p->d_rmap, buf(pd ? B_P0 : B_P1),
                                                     buf(pd ? B_P1 : B_P0));
          break;
        }
        case OP_MIRROR:
          mirror_kernel<T><<<(o.count + kMirrorTiles - 1) / kMirrorTiles, 256, 0, st>>>(s.d_mirror + o.off, o.count,
                                                                                         buf(o.abuf), buf(o.cbuf));
          break;
        case OP_FWD_CHAIN:
        case OP_BWD_CHAIN: {
          cudaMemsetAsync(p->d_chain, 0, sizeof(unsigned), st);
          if (++p->chain_epoch == 0) ++p->chain_epoch;
          if (o.kind == OP_FWD_CHAIN)
            fwd_chain_kernel<T><<<o.count, 256, 0, st>>>(s.d_rows + o.off, p->d_fronts, buf(B_L), buf(B_DINV),
                                                         buf(B_X), p->d_chain + 64, p->d_chain, p->chain_epoch,
                                                         p->d_chain_err, p->tc_wait_ns);
          else
            bwd_chain_kernel<T><<<o.count, 512, 0, st>>>(s.d_rows + o.off, p->d_fronts, buf(B_L), buf(B_DINV),
                                                         buf(B_X), buf((o.depth & 1) == 0 ? B_G0 : B_G1),
                                                         p->d_chain + 64, p->d_chain, p->chain_epoch,
                                                         p->d_chain_err, p->tc_wait_ns);
          break;
        }
        case OP_ZEXTRACT:
          zextract_kernel<T><<<o.count, 256, 0, st>>>(s.d_rows + o.off, p->d_fronts, p->d_iperm, p->d_amap,
                                                      p->sym.nslots, buf(o.cbuf), zq);
          break;
      }
      if (timed)
        prof_end(p, st, on_tc ? kProfTensorCore : (o.kind >= OP_FWD_CHAIN ? int(OP_GEMM) : o.kind), o.flops, o.site,
                 o.kind == OP_GEMM ? o.count : 0);
    }
    if (depth_log && !dmarks.empty()) {
      dmark(-1);
      const char* what = &s == &p->sched_factor ? "factor" : &s == &p->sched_selinv ? "inverse" : "solve";
      std::string line = std::string(what) + " ms by depth:";
      for (size_t i = 0; i + 1 < dmarks.size(); ++i) {
        float ms = 0.0f;
        cudaEventSynchronize(dmarks[i + 1].second);
        cudaEventElapsedTime(&ms, dmarks[i].second, dmarks[i + 1].second);
        char buf[48];
        std::snprintf(buf, sizeof(buf), " %d:%.2f", dmarks[i].first, ms);
        line += buf;
      }
      for (auto& m : dmarks) cudaEventDestroy(m.second);
      std::fprintf(stderr, "%s\n", line.c_str());
    }
    p->launches_total += s.launches;
  }
};

// ------------------------------------------------------------- TMA maps
// cuTensorMapEncodeTiled, the CUDA driver API entry point obtained through the runtime (no libcuda link)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return PFN_cuTensorMapEncodeTiled_v12000(nullptr);
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// Encode the schedule's TMA maps over the plan's FP32 buffers (sizes in
// elements: factor, pool 0, pool 1, inverse scratch) and upload them.  A map
// that cannot be encoded leaves its operands on the cp.async path.
static void encode_maps(Plan* p, Schedule& sc, const int64_t* sizes) {
  if (sc.maps.empty()) return;
  const auto encode = tensor_map_encoder();
  std::vector<CUtensorMap> host(sc.maps.size());
  std::vector<char> ok(sc.maps.size(), 0);
  for (size_t i = 0; i < sc.maps.size() && encode; ++i) {
    const MapReq& r = sc.maps[i];
    void* buf = nullptr;
    int64_t size = 0;
    switch (r.buf) {
      case B_L: buf = p->d_L; size = sizes[0]; break;
      case B_P0: buf = p->d_pool[0]; size = sizes[1]; break;
      case B_P1: buf = p->d_pool[1]; size = sizes[2]; break;
      case B_SX: buf = p->d_sx; size = sizes[3]; break;
      default: break;
    }
    const int64_t rows = buf ? (size - r.base) / r.ld : 0;
    if (rows < 1) continue;
    const cuuint64_t dims[2] = {cuuint64_t(r.ld), cuuint64_t(rows)};
    const cuuint64_t strides[1] = {cuuint64_t(r.ld) * sizeof(float)};
    const cuuint32_t box[2] = {32, 128};
    const cuuint32_t estr[2] = {1, 1};
    ok[i] = encode(&host[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, static_cast<float*>(buf) + r.base, dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  for (GemmTask& t : sc.gemm) {
    if (t.amap >= 0 && !ok[t.amap]) t.amap = -1;
    if (t.bmap >= 0 && !ok[t.bmap]) t.bmap = -1;
  }
  if (cudaMalloc(&sc.d_maps, host.size() * sizeof(CUtensorMap)) != cudaSuccess) {
    sc.d_maps = nullptr;
    for (GemmTask& t : sc.gemm) t.amap = t.bmap = -1;
    return;
  }
  cudaMemcpy(sc.d_maps, host.data(), host.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
}

// ------------------------------------------------------ nested dissection
// The fill-reducing ordering on the device: every lattice node descends the
// geometric dissection tree of the (x, y, t) box by itself, with the splitting
// rule of the symbolic analysis (symbolic.cpp, NDBuilder::build): the cheapest of
// a thickness-2 cut across x or y and a thickness-1 cut across t, a box of at
// most leaf_max nodes or with no admissible cut being a leaf.  A box's nodes are
// numbered after both children's (post-order): child 1, child 2, then its own
// separator, each box x-fastest.  The numbering of a node follows from the box
// volumes alone, so no tree is stored.
__global__ void nd_perm_kernel(int Mx, int Ny, int T, int leaf_max, int* __restrict__ perm,
                               int* __restrict__ iperm) {
  const int64_t n = int64_t(Mx) * Ny * T;
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int x = int(k % Mx), y = int((k / Mx) % Ny), t = int(k / (int64_t(Mx) * Ny));
  int box[6] = {0, Mx, 0, Ny, 0, T};
  int64_t base = 0;
  const int64_t kInf = INT64_MAX;
  for (int level = 0; level < 256; ++level) {
    const int a = box[1] - box[0], b = box[3] - box[2], c = box[5] - box[4];
    const int64_t vol = int64_t(a) * b * c;
    const int64_t cx = a >= 4 ? int64_t(2) * b * c : kInf;
    const int64_t cy = b >= 4 ? int64_t(2) * a * c : kInf;
    const int64_t ct = (T > 1 && c >= 3) ? int64_t(a) * b : kInf;
    const int64_t cmin = min(cx, min(cy, ct));
    int sp[6] = {box[0], box[1], box[2], box[3], box[4], box[5]};
    if (vol <= leaf_max || cmin == kInf) break;  // leaf: numbered below as a whole
    int k1[6] = {box[0], box[1], box[2], box[3], box[4], box[5]};
    int k2[6] = {box[0], box[1], box[2], box[3], box[4], box[5]};
    if (cmin == cx) {
      const int m = box[0] + (a - 2) / 2;
      k1[1] = m; sp[0] = m; sp[1] = m + 2; k2[0] = m + 2;
    } else if (cmin == cy) {
      const int m = box[2] + (b - 2) / 2;
      k1[3] = m; sp[2] = m; sp[3] = m + 2; k2[2] = m + 2;
    } else {
      const int m = box[4] + (c - 1) / 2;
      k1[5] = m; sp[4] = m; sp[5] = m + 1; k2[4] = m + 1;
    }
    auto inside = [&](const int* q) {
      return x >= q[0] && x < q[1] && y >= q[2] && y < q[3] && t >= q[4] && t < q[5];
    };
    const int64_t v1 = int64_t(k1[1] - k1[0]) * (k1[3] - k1[2]) * (k1[5] - k1[4]);
    const int64_t v2 = int64_t(k2[1] - k2[0]) * (k2[3] - k2[2]) * (k2[5] - k2[4]);
    if (inside(k1)) {
      for (int e = 0; e < 6; ++e) box[e] = k1[e];
      continue;
    }
    if (inside(k2)) {
      base += v1;
      for (int e = 0; e < 6; ++e) box[e] = k2[e];
      continue;
    }
    base += v1 + v2;  // the separator, after both children
    for (int e = 0; e < 6; ++e) box[e] = sp[e];
    break;
  }
  const int wa = box[1] - box[0], wb = box[3] - box[2];
  const int64_t v = base + (int64_t(t - box[4]) * wb + (y - box[2])) * wa + (x - box[0]);
  perm[k] = int(v);
  iperm[v] = int(k);
}

// ------------------------------------------------------------------- plan API
int plan_build(Plan* p) {
  Symbolic& S = p->sym;
  const int TM = p->precision == 0 ? 64 : 128;
  p->tile_m = TM;
  p->tile_n = TM;
  std::vector<DevFront> df(S.fronts.size());
  p->w_elems_per_rhs[0] = std::max<int64_t>(S.w_pool[0], 1);
  p->w_elems_per_rhs[1] = std::max<int64_t>(S.w_pool[1], 1);
  for (size_t f = 0; f < S.fronts.size(); ++f) {
    const Front& x = S.fronts[f];
    DevFront& d = df[f];
    d.p_off = x.p_off; d.u_off = x.u_off; d.z_off = x.z_off; d.b_off = x.b_off; d.d_off = x.d_off;
    d.w_base = x.w_base;
    d.s0 = x.s0; d.ns = x.ns; d.nb = x.nb; d.ld = x.ld; d.ldu = x.ldu; d.ldz = x.ldz;
    d.parent = x.parent; d.depth = x.depth;
    d.child[0] = x.child[0]; d.child[1] = x.child[1];
  }
  p->d_fronts = upload_vec(df);
  // the permutations come from the device ordering, checked against the
  // symbolic analysis that laid out the fronts
  CUDA_TRY(cudaMalloc(&p->d_perm, size_t(S.n) * sizeof(int)));
  CUDA_TRY(cudaMalloc(&p->d_iperm, size_t(S.n) * sizeof(int)));
  nd_perm_kernel<<<int((int64_t(S.n) + 255) / 256), 256>>>(S.Mx, S.Ny, S.T, S.leaf_max, p->d_perm, p->d_iperm);
  CUDA_TRY(cudaGetLastError());
  {
    std::vector<int> dev(S.n);
    CUDA_TRY(cudaMemcpy(dev.data(), p->d_perm, size_t(S.n) * sizeof(int), cudaMemcpyDeviceToHost));
    if (dev != S.perm) {
      p->last_error = "device nested-dissection ordering differs from the symbolic analysis";
      return 2;
    }
  }
  p->d_front_of = upload_vec(S.front_of);
  p->d_blist = upload_vec(S.blist);
  p->d_rmap = upload_vec(S.rmap);
  p->d_amap = upload_vec(S.amap);
  if (!p->d_fronts || !p->d_perm || !p->d_amap) { p->last_error = "device allocation failed (symbolic)"; return 4; }
  const size_t es = p->esize();
  CUDA_TRY(cudaMalloc(&p->d_L, size_t(S.l_size) * es));
  CUDA_TRY(cudaMalloc(&p->d_dinv, size_t(std::max<int64_t>(S.dinv_size, 1)) * es));
  for (int k = 0; k < 2; ++k) {
    p->pool_elems[k] = std::max<int64_t>(std::max(S.u_pool[k], S.z_pool[k]), 32);
    CUDA_TRY(cudaMalloc(&p->d_pool[k], size_t(p->pool_elems[k]) * es));
  }
  const bool pairs = p->precision == 1 && tc_gemm_enabled();
  build_factor_schedule(S, p->sched_factor, TM, TM, pairs);
  int64_t sx_elems = 0;
  build_selinv_schedule(S, p->sched_selinv, TM, TM, &sx_elems, pairs);
  CUDA_TRY(cudaMalloc(&p->d_sx, size_t(sx_elems) * es));
  if (pairs) {
    const int64_t sizes[] = {S.l_size, p->pool_elems[0], p->pool_elems[1], sx_elems};
    encode_maps(p, p->sched_factor, sizes);
    encode_maps(p, p->sched_selinv, sizes);
  }
  p->sched_factor.upload();
  p->sched_selinv.upload();
  CUDA_TRY(cudaMalloc(&p->d_logpiv, std::max<size_t>(p->sched_factor.diag.size(), 1) * sizeof(double)));
  CUDA_TRY(cudaMalloc(&p->d_err, sizeof(int)));
  CUDA_TRY(cudaMalloc(&p->d_scalar, 64 * sizeof(double)));
  CUDA_TRY(cudaMalloc(&p->d_part, 1024 * sizeof(double)));
  CUDA_TRY(cudaMallocHost(&p->h_pin, 2048 * sizeof(double)));
  int64_t nflags = 0;
  chain_bases(S, &nflags);
  CUDA_TRY(cudaMalloc(&p->d_chain, size_t(64 + nflags) * sizeof(unsigned)));
  CUDA_TRY(cudaMemset(p->d_chain, 0, size_t(64 + nflags) * sizeof(unsigned)));
  CUDA_TRY(cudaMalloc(&p->d_chain_err, sizeof(int)));
  CUDA_TRY(cudaMemset(p->d_chain_err, 0, sizeof(int)));
  p->chain_epoch = 0;
  return 0;
}

template <typename T>
static int factor_t(Plan* p, int with_obs, double tau) {
  const Symbolic& S = p->sym;
  cudaStream_t st = p->stream;
  CUDA_TRY(cudaMemsetAsync(p->d_L, 0, size_t(S.l_size) * sizeof(T), st));
  CUDA_TRY(cudaMemsetAsync(p->d_err, 0xFF, sizeof(int), st));  // -1: no failed pivot
  launch_scatter<T>(p->qstencil(), S.nslots, p->d_amap, p->d_perm, p->d_front_of, p->d_fronts,
                    with_obs ? p->d_obs_cnt : nullptr, tau, static_cast<T*>(p->d_L), st);
  Exec<T>{p, p->sched_factor, 0, nullptr}.run();
  sum_kernel<<<1, 256, 0, st>>>(p->d_logpiv, int64_t(p->sched_factor.diag.size()), p->d_scalar);
  CUDA_TRY(cudaMemcpyAsync(p->h_pin + 1024, p->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(p->pin_int(), p->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(cudaGetLastError());
  const double sum = p->h_pin[1024];
  const int err = p->pin_int()[0];
  if (tc_gemm_take_error(p->stream, p->pin_int() + 1)) { p->last_error = "tensor-core product timed out"; p->factored = 0; return 2; }
  if (err >= 0) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "matrix is not positive definite (front %d)", err);
    p->last_error = buf;
    p->factored = 0;
    return 3;
  }
  p->logdet = 2.0 * sum;
  p->launches_total += 2;  // scatter, log-pivot sum
  if (p->profile) prof_collect(p);
  p->factored = with_obs ? 2 : 1;
  p->factored_tau = tau;
  return 0;
}

int plan_factor(Plan* p, int with_obs, double tau) {
  if (!p->assembled) { p->last_error = "no assembled model"; return 5; }
  if (with_obs && !p->d_obs_cnt) { p->last_error = "no observations set"; return 5; }
  return p->precision == 0 ? factor_t<double>(p, with_obs, tau) : factor_t<float>(p, with_obs, tau);
}

static int ensure_solve_buffers(Plan* p, int nrhs) {
  if (nrhs <= p->solve_cap) return 0;
  const size_t es = p->esize();
  cudaFree(p->d_X);
  for (int k = 0; k < 2; ++k) { cudaFree(p->d_W[k]); cudaFree(p->d_G[k]); }
  CUDA_TRY(cudaMalloc(&p->d_X, size_t(p->sym.n) * nrhs * es));
  for (int k = 0; k < 2; ++k) {
    CUDA_TRY(cudaMalloc(&p->d_W[k], size_t(p->w_elems_per_rhs[k]) * nrhs * es));
    CUDA_TRY(cudaMalloc(&p->d_G[k], size_t(p->w_elems_per_rhs[k]) * nrhs * es));
  }
  p->solve_cap = nrhs;
  return 0;
}

static int ensure_refine_buffers(Plan* p, int64_t elems) {
  if (elems <= p->r_cap) return 0;
  cudaFree(p->d_r); cudaFree(p->d_x64); cudaFree(p->d_b64);
  CUDA_TRY(cudaMalloc(&p->d_r, size_t(elems) * sizeof(double)));
  CUDA_TRY(cudaMalloc(&p->d_x64, size_t(elems) * sizeof(double)));
  CUDA_TRY(cudaMalloc(&p->d_b64, size_t(elems) * sizeof(double)));
  p->r_cap = elems;
  return 0;
}

template <typename T>
static void tri_solve(Plan* p, int nrhs) {
  auto& fw = p->sched_fwd[nrhs];
  if (!fw) {
    fw.reset(new Schedule());
    build_fwd_schedule(p->sym, *fw, p->tile_m, p->tile_n, nrhs);
    fw->upload();
  }
  auto& bw = p->sched_bwd[nrhs];
  if (!bw) {
    bw.reset(new Schedule());
    build_bwd_schedule(p->sym, *bw, p->tile_m, p->tile_n, nrhs);
    bw->upload();
  }
  Exec<T>{p, *fw, nrhs, nullptr}.run();
  Exec<T>{p, *bw, nrhs, nullptr}.run();
}

// Reads and clears the one-column sweeps' wait-failure flag (page-locked read-back).
static int chain_take_error(Plan* p) {
  int* h = p->pin_int() + 2;
  *h = 0;
  cudaMemcpyAsync(h, p->d_chain_err, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
  cudaStreamSynchronize(p->stream);
  const int e = *h;
  if (e) {
    cudaMemsetAsync(p->d_chain_err, 0, sizeof(int), p->stream);
    cudaStreamSynchronize(p->stream);
  }
  return e;
}

template <typename T>
static int solve_t(Plan* p, const double* b, double* x, int nrhs, int iters, double tol, double* resid) {
  const int n = p->sym.n;
  const int64_t ne = int64_t(n) * nrhs;
  cudaStream_t st = p->stream;
  if (ensure_solve_buffers(p, nrhs)) return 2;
  if (ensure_refine_buffers(p, ne)) return 2;
  const double* obs = p->factored == 2 ? p->d_obs_cnt : nullptr;
  const double tau = p->factored_tau;
  // first solve straight from b
  launch_to_new<T>(b, p->d_perm, n, nrhs, static_cast<T*>(p->d_X), st);
  tri_solve<T>(p, nrhs);
  launch_from_new<T>(static_cast<const T*>(p->d_X), p->d_perm, n, nrhs, x, 0, st);
  p->launches_total += 2;
  const int nblk = 512;
  // relative residual ||b - A x|| / ||b|| of the current x (partial sums read
  // through the plan's page-locked buffer)
  auto residual = [&]() -> double {
    launch_spmv(p->qstencil(), obs, tau, x, p->d_r, nrhs, st);
    resid_kernel<<<nblk, 256, 0, st>>>(b, p->d_r, ne, p->d_part);
    p->launches_total += 2;
    if (cudaMemcpyAsync(p->h_pin, p->d_part, 2 * nblk * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return -1.0;
    double r2 = 0.0, b2 = 0.0;
    for (int k = 0; k < nblk; ++k) { r2 += p->h_pin[2 * k]; b2 += p->h_pin[2 * k + 1]; }
    return b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
  };
  double rel = -1.0;
  bool fresh = false;  // rel belongs to the current x
  for (int it = 0; it < iters; ++it) {
    rel = residual();
    if (rel < 0) { p->last_error = "residual read-back failed"; return 2; }
    fresh = true;
    if (rel <= tol) break;
    p->launches_total += 2;
    launch_to_new<T>(p->d_r, p->d_perm, n, nrhs, static_cast<T*>(p->d_X), st);
    tri_solve<T>(p, nrhs);
    launch_from_new<T>(static_cast<const T*>(p->d_X), p->d_perm, n, nrhs, x, 1, st);
    fresh = false;
  }
  if (resid) {
    if (!fresh) {
      rel = residual();
      if (rel < 0) { p->last_error = "residual read-back failed"; return 2; }
    }
    *resid = rel;
  }
  CUDA_TRY(cudaGetLastError());
  if (p->profile) prof_collect(p);
  if (tc_gemm_take_error(p->stream, p->pin_int() + 1)) { p->last_error = "tensor-core product timed out"; return 2; }
  if (chain_take_error(p)) { p->last_error = "triangular sweep timed out"; return 2; }
  return 0;
}

template <typename T>
static int sample_t(Plan* p, const double* z, double* x, int nrhs) {
  const int n = p->sym.n;
  cudaStream_t st = p->stream;
  if (ensure_solve_buffers(p, nrhs)) return 2;
  auto& bw = p->sched_bwd[nrhs];
  if (!bw) {
    bw.reset(new Schedule());
    build_bwd_schedule(p->sym, *bw, p->tile_m, p->tile_n, nrhs);
    bw->upload();
  }
  launch_to_new<T>(z, p->d_perm, n, nrhs, static_cast<T*>(p->d_X), st);
  Exec<T>{p, *bw, nrhs, nullptr}.run();
  launch_from_new<T>(static_cast<const T*>(p->d_X), p->d_perm, n, nrhs, x, 0, st);
  p->launches_total += 2;
  CUDA_TRY(cudaGetLastError());
  if (p->profile) prof_collect(p);
  if (nrhs == 1 && chain_take_error(p)) { p->last_error = "triangular sweep timed out"; return 2; }
  return 0;
}

int plan_sample(Plan* p, const double* z, double* x, int nrhs) {
  if (!p->factored) { p->last_error = "no valid factor"; return 5; }
  return p->precision == 0 ? sample_t<double>(p, z, x, nrhs) : sample_t<float>(p, z, x, nrhs);
}

int plan_solve(Plan* p, const double* b, double* x, int nrhs, int iters, double tol, double* resid) {
  if (!p->factored) { p->last_error = "no valid factor (factor first; selinv consumes it)"; return 5; }
  if (nrhs < 1) { p->last_error = "nrhs must be >= 1"; return 1; }
  return p->precision == 0 ? solve_t<double>(p, b, x, nrhs, iters, tol, resid)
                           : solve_t<float>(p, b, x, nrhs, iters, tol, resid);
}

template <typename T>
static int selinv_t(Plan* p, double* zq) {
  cudaStream_t st = p->stream;
  const Symbolic& S = p->sym;
  Exec<T>{p, p->sched_selinv, 0, zq}.run();
  int64_t tot = int64_t(S.n) * S.nslots;
  zsym_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(S.Mx, S.Ny, S.T, S.nslots, p->d_amap, zq);
  p->launches_total += 1;
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(cudaGetLastError());
  if (tc_gemm_take_error(p->stream, p->pin_int() + 1)) {
    p->last_error = "tensor-core product timed out";
    p->factored = 0;
    return 2;
  }
  if (p->profile) prof_collect(p);
  p->factored = 0;  // the factor's panels now hold intermediate products
  return 0;
}

int plan_selinv(Plan* p, double* zq) {
  if (!p->factored) { p->last_error = "no valid factor"; return 5; }
  return p->precision == 0 ? selinv_t<double>(p, zq) : selinv_t<float>(p, zq);
}

}  // namespace spde
