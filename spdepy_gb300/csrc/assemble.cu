// Q(theta) assembly: fields -> 9-point operator A -> compact per-cell stencils
// of Q -> values scattered straight into the dense fronts of the factorisation.
//
// Reference path being replaced: makeQ (spdes/advection_diffusion2D.py:86-117,
// spdes/var_advection_var_diffusion2D.py:83-116, spatial models e.g.
// spdes/whittle_matern_anisotropic2D.py:59-75) with the stencils built by the
// ccode/*.cpp libraries through ctypes and scipy sparse products.
//
// Because the coefficients are time-invariant (all interior time blocks are
// identical), Q is held as four spatial stencils per cell (the first diagonal
// block's 25 values, the interior diagonal block's 25, the off-diagonal 9 and the
// kappa^2 diagonal), i.e. O(Ns) memory, and node values are formed on the fly.
#include <cuda_runtime.h>
#include <math.h>

#include "assemble.cuh"
#include "stencil.cuh"

namespace spde {

__device__ __forceinline__ double dotb(const double* b, const double* c, int nb) {
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s = fma(b[i], c[i], s);
  return s;
}

// H = gamma I (iso), gamma I + v v^T (ani), or the half-angle form
// gamma (cosh|v| I + sinh|v|/|v| [[vx, vy], [vy, -vx]]) (whittle_matern_ha2D.py:73-82);
// out = {H00, H01, H10, H11}.  At |v| = 0 the half-angle ratio takes its limit 1.
__device__ __forceinline__ void h_tensor(int diff, double g, double vx, double vy, double* out) {
  if (diff == 0) {
    out[0] = g; out[1] = 0.0; out[2] = 0.0; out[3] = g;
  } else if (diff == 1) {
    out[0] = g + vx * vx; out[1] = vx * vy; out[2] = vx * vy; out[3] = g + vy * vy;
  } else {
    double a = sqrt(vx * vx + vy * vy);
    double ea = exp(a), eb = exp(-a);
    double ch = (ea + eb) / 2, sh = (ea - eb) / 2;
    double r = a > 0.0 ? sh / a : 1.0;
    out[0] = g * (ch + r * vx); out[1] = g * r * vy; out[2] = g * r * vy; out[3] = g * (ch - r * vx);
  }
}

// Field values of cell c (kappa, per-face H, per-face w) from the canonical theta.
__device__ void cell_fields(const DevModel& m, int c, double* kappa, double* Hf /*16*/, double* wf /*4*/) {
  const double* th = m.theta;
  const int nk = m.nk, nb = m.nbasis;
  if (m.var_h) {
    *kappa = exp(dotb(m.bs + int64_t(c) * nb, th, nb));
    for (int f = 0; f < 4; ++f) {
      const double* b = m.bsH + (int64_t(c) * 4 + f) * nb;
      double g = exp(dotb(b, th + nk, nb));
      double vx = m.diff ? dotb(b, th + 2 * nk, nb) : 0.0;
      double vy = m.diff ? dotb(b, th + 3 * nk, nb) : 0.0;
      h_tensor(m.diff, g, vx, vy, Hf + 4 * f);
    }
  } else {
    *kappa = exp(th[0]);
    h_tensor(m.diff, exp(th[nk]), m.diff ? th[2 * nk] : 0.0, m.diff ? th[3 * nk] : 0.0, Hf);
  }
  const double* tw = th + 4 * nk;
  if (m.adv == 1) {
    wf[0] = tw[0]; wf[1] = tw[1];
  } else if (m.adv == 2) {
    for (int f = 0; f < 4; ++f) {
      const double* b = m.bsA + (int64_t(c) * 4 + f) * nb;
      wf[f] = dotb(b, tw + ((f & 1) ? nb : 0), nb);
    }
  } else if (m.adv == 3) {
    for (int f = 0; f < 4; ++f) wf[f] = tw[0] * m.ww[int64_t(c) * 4 + f];
  }
}

// A = V(1 + dt kappa) I - dt A_H + dt A_w (spatio-temporal) or V kappa I - A_H
// (spatial), accumulated into the geometric 3x3 slots of each cell; A0 of the
// initial-field model likewise.  Also Qs = V kappa^2.
__global__ void fields_kernel(DevModel m, double* __restrict__ Ageo, double* __restrict__ A0geo,
                              double* __restrict__ kap, double* __restrict__ qs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.Ns) return;
  const int M = m.Mx, N = m.Ny;
  const int j = c / M, i = c - j * M;
  double kappa, Hf[16], wf[4];
  cell_fields(m, c, &kappa, Hf, wf);
  double a[9];
  for (int p = 0; p < 9; ++p) a[p] = 0.0;
  const bool st = m.T > 1;
  const double sc = st ? m.dt : 1.0;
  a[4] = st ? m.V + m.V * kappa * m.dt : m.V * kappa;
  double v[9];
  int col[9];
  bool keep[9];
  CellH h = cell_h(Hf, m.var_h != 0, c, i, j, M, N, m.bc);
  diffusion_cell(h, m.hx, m.hy, i, j, M, N, m.bc, v, col, keep);
  for (int p = 0; p < 9; ++p)
    if (keep[p]) a[geo9(col[p], i, j, M)] -= sc * v[p];
  if (m.adv) {
    advection_cell(wf, nullptr, m.adv != 1, m.hx, m.hy, i, j, M, N, m.bc, 3, v, col, keep);
    for (int p = 0; p < 5; ++p)
      if (keep[p]) a[geo9(col[p], i, j, M)] += m.dt * v[p];
  }
  for (int p = 0; p < 9; ++p) Ageo[int64_t(c) * 9 + p] = a[p];
  kap[c] = kappa;
  qs[c] = m.V * kappa * kappa;
  if (st) {
    const double* t0 = m.theta + 4 * m.nk + m.nw + 1;
    double H0[4];
    h_tensor(m.mod0_diff, exp(t0[1]), m.mod0_diff ? t0[2] : 0.0, m.mod0_diff ? t0[3] : 0.0, H0);
    for (int p = 0; p < 9; ++p) a[p] = 0.0;
    a[4] = m.V * exp(t0[0]);
    CellH h0 = cell_h(H0, false, c, i, j, M, N, m.mod0_bc);
    diffusion_cell(h0, m.hx, m.hy, i, j, M, N, m.mod0_bc, v, col, keep);
    for (int p = 0; p < 9; ++p)
      if (keep[p]) a[geo9(col[p], i, j, M)] -= v[p];
    for (int p = 0; p < 9; ++p) A0geo[int64_t(c) * 9 + p] = a[p];
  }
}

// (A^T D A)[k, k+d] over the 25 offsets d: sum over rows m of A in the 3x3
// neighbourhood of k of A[m,k] D[m] A[m,l].
__device__ void ata_row(const double* Ag, const double* D, double dscale, int c, int M, int N, double* out) {
  for (int s = 0; s < 25; ++s) out[s] = 0.0;
  const int j = c / M, i = c - j * M;
  for (int dy1 = -1; dy1 <= 1; ++dy1)
    for (int dx1 = -1; dx1 <= 1; ++dx1) {
      // row m = k - (dx1, dy1); A[m, k] sits in slot (dx1, dy1) of row m
      int mi = i - dx1, mj = j - dy1;
      if (mi < 0 || mi >= M || mj < 0 || mj >= N) continue;
      int mm = mj * M + mi;
      const double* Am = Ag + int64_t(mm) * 9;
      double amk = Am[(dy1 + 1) * 3 + (dx1 + 1)];
      if (amk == 0.0) continue;
      double w = amk * (D ? D[mm] * dscale : dscale);
      for (int dy2 = -1; dy2 <= 1; ++dy2)
        for (int dx2 = -1; dx2 <= 1; ++dx2) {
          // column l = m + (dx2, dy2); offset from k = (dx2 - dx1, dy2 - dy1)
          int ox = dx2 - dx1, oy = dy2 - dy1;
          out[(oy + 2) * 5 + (ox + 2)] += w * Am[(dy2 + 1) * 3 + (dx2 + 1)];
        }
    }
}

__global__ void qstencil_kernel(DevModel m, const double* __restrict__ Ageo, const double* __restrict__ A0geo,
                                const double* __restrict__ kap, const double* __restrict__ qs, double* __restrict__ Q0,
                                double* __restrict__ QA, double* __restrict__ QO, double* __restrict__ cQs,
                                double cfac) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.Ns) return;
  double r[25];
  if (m.T == 1) {
    ata_row(Ageo, nullptr, 1.0 / m.V, c, m.Mx, m.Ny, r);
    for (int s = 0; s < 25; ++s) QA[int64_t(c) * 25 + s] = r[s];
    return;
  }
  // interior diagonal block: A^T (Qs / V^2) A, scaled by c = 1/(dt sigma)
  // (spdes/advection_diffusion2D.py:103,112-116)
  ata_row(Ageo, qs, 1.0 / (m.V * m.V), c, m.Mx, m.Ny, r);
  for (int s = 0; s < 25; ++s) QA[int64_t(c) * 25 + s] = cfac * r[s];
  ata_row(A0geo, nullptr, 1.0 / m.V, c, m.Mx, m.Ny, r);
  for (int s = 0; s < 25; ++s) Q0[int64_t(c) * 25 + s] = r[s];
  const double* Ac = Ageo + int64_t(c) * 9;
  for (int p = 0; p < 9; ++p) QO[int64_t(c) * 9 + p] = -cfac * qs[c] / m.V * Ac[p];
  cQs[c] = cfac * qs[c];
}

// Q in stencil layout (natural order, nslots values per node), FP64.
__global__ void qexport_kernel(QStencil q, int nslots, const double* __restrict__ obs_cnt, double tau,
                               double* __restrict__ out) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = int64_t(q.Ns) * q.T;
  if (e >= n * nslots) return;
  const int k = int(e / nslots), s = int(e % nslots);
  const int t = k / q.Ns, c = k - t * q.Ns;
  const int y = c / q.Mx, x = c - y * q.Mx;
  int dx, dy, dt;
  stencil_slot(nslots, s, &dx, &dy, &dt);
  double v = 0.0;
  if (x + dx >= 0 && x + dx < q.Mx && y + dy >= 0 && y + dy < q.Ny && t + dt >= 0 && t + dt < q.T) {
    v = qval(q, c, t, dx, dy, dt);
    if (obs_cnt && dx == 0 && dy == 0 && dt == 0) v += tau * obs_cnt[k];
  }
  out[e] = v;
}

// Scatter Q (or Q + tau S^T S) into the zeroed front panels.
template <typename T>
__global__ void scatter_kernel(QStencil q, int nslots, const int* __restrict__ amap, const int* __restrict__ perm,
                               const int* __restrict__ front_of, const DevFront* __restrict__ fronts,
                               const double* __restrict__ obs_cnt, double tau, T* __restrict__ L) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = int64_t(q.Ns) * q.T;
  if (e >= n * nslots) return;
  const int off = amap[e];
  if (off < 0) return;
  const int k = int(e / nslots), s = int(e % nslots);
  const int t = k / q.Ns, c = k - t * q.Ns;
  int dx, dy, dt;
  stencil_slot(nslots, s, &dx, &dy, &dt);
  double v = qval(q, c, t, dx, dy, dt);
  if (obs_cnt && dx == 0 && dy == 0 && dt == 0) v += tau * obs_cnt[k];
  const DevFront f = fronts[front_of[perm[k]]];
  L[f.p_off + off] = T(v);
}

// ---------------------------------------------------- stencil triplets (B3)
__global__ void diffusion_triplet_kernel(int M, int N, const double* __restrict__ H, int field, double hx, double hy,
                                         int bc, int* __restrict__ row, int* __restrict__ col,
                                         double* __restrict__ val) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M * N) return;
  const int j = c / M, i = c - j * M;
  CellH h = cell_h(field ? H + int64_t(c) * 16 : H, field != 0, c, i, j, M, N, bc);
  double v[9];
  int cl[9];
  bool keep[9];
  diffusion_cell(h, hx, hy, i, j, M, N, bc, v, cl, keep);
  for (int p = 0; p < 9; ++p) {
    row[int64_t(c) * 9 + p] = keep[p] ? c : M * N;
    col[int64_t(c) * 9 + p] = cl[p];
    val[int64_t(c) * 9 + p] = v[p];
  }
}

__global__ void advection_triplet_kernel(int M, int N, const double* __restrict__ G, const double* __restrict__ dG,
                                         int field, double hx, double hy, int bc, int diff, int* __restrict__ row,
                                         int* __restrict__ col, double* __restrict__ val) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M * N) return;
  const int j = c / M, i = c - j * M;
  double v[5];
  int cl[5];
  bool keep[5];
  const double* g = field ? G + int64_t(c) * 4 : G;
  const double* d = (field && dG) ? dG + int64_t(c) * 4 : nullptr;
  advection_cell(g, d, field != 0, hx, hy, i, j, M, N, bc, diff, v, cl, keep);
  for (int p = 0; p < 5; ++p) {
    row[int64_t(c) * 5 + p] = keep[p] ? c : M * N;
    col[int64_t(c) * 5 + p] = cl[p];
    val[int64_t(c) * 5 + p] = v[p];
  }
}

// ------------------------------------------------------------ permutations
template <typename T>
__global__ void to_new_kernel(const double* __restrict__ src, const int* __restrict__ perm, int n, int nrhs,
                              T* __restrict__ dst) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * nrhs) return;
  const int k = int(e / nrhs), r = int(e % nrhs);
  dst[int64_t(perm[k]) * nrhs + r] = T(src[e]);
}

template <typename T>
__global__ void from_new_kernel(const T* __restrict__ src, const int* __restrict__ perm, int n, int nrhs,
                                double* __restrict__ dst, int accumulate) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * nrhs) return;
  const int k = int(e / nrhs), r = int(e % nrhs);
  double v = double(src[int64_t(perm[k]) * nrhs + r]);
  dst[e] = accumulate ? dst[e] + v : v;
}

// ------------------------------------------------------------------ launchers
static inline int nblk(int64_t n, int b) { return int((n + b - 1) / b); }

void launch_fields(const DevModel& m, double* Ageo, double* A0geo, double* kap, double* qs, cudaStream_t st) {
  fields_kernel<<<nblk(m.Ns, 128), 128, 0, st>>>(m, Ageo, A0geo, kap, qs);
}
void launch_qstencil(const DevModel& m, const double* Ageo, const double* A0geo, const double* kap, const double* qs,
                     double* Q0, double* QA, double* QO, double* cQs, double cfac, cudaStream_t st) {
  qstencil_kernel<<<nblk(m.Ns, 128), 128, 0, st>>>(m, Ageo, A0geo, kap, qs, Q0, QA, QO, cQs, cfac);
}
void launch_qexport(const QStencil& q, int nslots, const double* obs, double tau, double* out, cudaStream_t st) {
  int64_t tot = int64_t(q.Ns) * q.T * nslots;
  qexport_kernel<<<nblk(tot, 256), 256, 0, st>>>(q, nslots, obs, tau, out);
}
template <typename T>
void launch_scatter(const QStencil& q, int nslots, const int* amap, const int* perm, const int* front_of,
                    const DevFront* fronts, const double* obs, double tau, T* L, cudaStream_t st) {
  int64_t tot = int64_t(q.Ns) * q.T * nslots;
  scatter_kernel<T><<<nblk(tot, 256), 256, 0, st>>>(q, nslots, amap, perm, front_of, fronts, obs, tau, L);
}
template void launch_scatter<double>(const QStencil&, int, const int*, const int*, const int*, const DevFront*,
                                     const double*, double, double*, cudaStream_t);
template void launch_scatter<float>(const QStencil&, int, const int*, const int*, const int*, const DevFront*,
                                    const double*, double, float*, cudaStream_t);
// y = (Q + tau S^T S) x with one thread per (spatial cell, column) sweeping the
// time axis: the cell's time-invariant coefficients (25 in-block values, 9 to
// t + 1 and the 9 mirrored from the neighbours to t - 1) are loaded once and
// reused for all T blocks.
__global__ void __launch_bounds__(128) spmv_cells_kernel(QStencil q, const double* __restrict__ obs, double tau,
                                                         const double* __restrict__ x, double* __restrict__ y,
                                                         int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(q.Ns) * nrhs) return;
  const int c = int(e / nrhs), r = int(e - int64_t(c) * nrhs);
  const int cy = c / q.Mx, cx = c - cy * q.Mx;
  double qa[25], qf[9], qb[9];
  uint32_t m25 = 0, m9 = 0;
#pragma unroll
  for (int s = 0; s < 25; ++s) {
    const int dx = s % 5 - 2, dy = s / 5 - 2;
    const bool in = cx + dx >= 0 && cx + dx < q.Mx && cy + dy >= 0 && cy + dy < q.Ny;
    m25 |= uint32_t(in) << s;
    qa[s] = q.QA[int64_t(c) * 25 + s];
  }
  if (q.T > 1) {
#pragma unroll
    for (int s = 0; s < 9; ++s) {
      const int dx = s % 3 - 1, dy = s / 3 - 1;
      const bool in = cx + dx >= 0 && cx + dx < q.Mx && cy + dy >= 0 && cy + dy < q.Ny;
      m9 |= uint32_t(in) << s;
      qf[s] = q.QO[int64_t(c) * 9 + s];
      qb[s] = in ? q.QO[int64_t(c + dy * q.Mx + dx) * 9 + (8 - s)] : 0.0;
    }
  }
  const double cqs = q.T > 1 ? q.cQs[c] : 0.0;
  for (int t = 0; t < q.T; ++t) {
    const int64_t k = int64_t(t) * q.Ns + c;
    const double* xt = x + k * nrhs + r;
    double acc = 0.0;
    if (t == 0 && q.T > 1) {
#pragma unroll
      for (int s = 0; s < 25; ++s)
        if (m25 >> s & 1u) {
          const int off = (s / 5 - 2) * q.Mx + (s % 5 - 2);
          acc = fma(q.Q0[int64_t(c) * 25 + s], xt[int64_t(off) * nrhs], acc);
        }
    } else {
#pragma unroll
      for (int s = 0; s < 25; ++s)
        if (m25 >> s & 1u) {
          const int off = (s / 5 - 2) * q.Mx + (s % 5 - 2);
          acc = fma(qa[s], xt[int64_t(off) * nrhs], acc);
        }
    }
    if (q.T > 1) {
      if (t < q.T - 1 || t == 0) acc = fma(cqs, xt[0], acc);
      if (t + 1 < q.T) {
        const double* xn = xt + int64_t(q.Ns) * nrhs;
#pragma unroll
        for (int s = 0; s < 9; ++s)
          if (m9 >> s & 1u) acc = fma(qf[s], xn[int64_t((s / 3 - 1) * q.Mx + (s % 3 - 1)) * nrhs], acc);
      }
      if (t > 0) {
        const double* xp = xt - int64_t(q.Ns) * nrhs;
#pragma unroll
        for (int s = 0; s < 9; ++s)
          if (m9 >> s & 1u) acc = fma(qb[s], xp[int64_t((s / 3 - 1) * q.Mx + (s % 3 - 1)) * nrhs], acc);
      }
    }
    if (obs) acc = fma(tau * obs[k], xt[0], acc);
    y[k * nrhs + r] = acc;
  }
}

// Separable Q = Qt (x) Qs: one thread per spatial cell and right-hand side forms
// the spatial product u_t = sum_s Qs[c, s] x_t(c + off_s) once per time slice and
// combines y_t = Qt_tt u_t + Qt_off (u_(t-1) + u_(t+1)).
__global__ void __launch_bounds__(128) spmv_sep_kernel(QStencil q, const double* __restrict__ obs, double tau,
                                                       const double* __restrict__ x, double* __restrict__ y,
                                                       int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(q.Ns) * nrhs) return;
  const int c = int(e / nrhs), r = int(e - int64_t(c) * nrhs);
  const int cy = c / q.Mx, cx = c - cy * q.Mx;
  double qa[25];
  uint32_t m25 = 0;
#pragma unroll
  for (int s = 0; s < 25; ++s) {
    const int dx = s % 5 - 2, dy = s / 5 - 2;
    const bool in = cx + dx >= 0 && cx + dx < q.Mx && cy + dy >= 0 && cy + dy < q.Ny;
    m25 |= uint32_t(in) << s;
    qa[s] = q.QA[int64_t(c) * 25 + s];
  }
  auto spatial = [&](int t) {
    const double* xt = x + (int64_t(t) * q.Ns + c) * nrhs + r;
    double acc = 0.0;
#pragma unroll
    for (int s = 0; s < 25; ++s)
      if (m25 >> s & 1u) acc = fma(qa[s], xt[int64_t((s / 5 - 2) * q.Mx + (s % 5 - 2)) * nrhs], acc);
    return acc;
  };
  double up = 0.0, uc = spatial(0);
  for (int t = 0; t < q.T; ++t) {
    const double un = t + 1 < q.T ? spatial(t + 1) : 0.0;
    const int64_t k = int64_t(t) * q.Ns + c;
    double acc = (t == 0 || t == q.T - 1 ? q.qt_end : q.qt_mid) * uc + q.qt_off * (up + un);
    if (obs) acc = fma(tau * obs[k], x[k * nrhs + r], acc);
    y[k * nrhs + r] = acc;
    up = uc;
    uc = un;
  }
}

void launch_spmv(const QStencil& q, const double* obs, double tau, const double* x, double* y, int nrhs,
                 cudaStream_t st) {
  const int64_t tot = int64_t(q.Ns) * nrhs;
  if (q.sep) spmv_sep_kernel<<<nblk(tot, 128), 128, 0, st>>>(q, obs, tau, x, y, nrhs);
  else spmv_cells_kernel<<<nblk(tot, 128), 128, 0, st>>>(q, obs, tau, x, y, nrhs);
}
void launch_diffusion_triplets(int M, int N, const double* H, int field, double hx, double hy, int bc, int* row,
                               int* col, double* val, cudaStream_t st) {
  diffusion_triplet_kernel<<<nblk(int64_t(M) * N, 128), 128, 0, st>>>(M, N, H, field, hx, hy, bc, row, col, val);
}
void launch_advection_triplets(int M, int N, const double* G, const double* dG, int field, double hx, double hy,
                               int bc, int diff, int* row, int* col, double* val, cudaStream_t st) {
  advection_triplet_kernel<<<nblk(int64_t(M) * N, 128), 128, 0, st>>>(M, N, G, dG, field, hx, hy, bc, diff, row,
                                                                       col, val);
}
template <typename T>
void launch_to_new(const double* src, const int* perm, int n, int nrhs, T* dst, cudaStream_t st) {
  to_new_kernel<T><<<nblk(int64_t(n) * nrhs, 256), 256, 0, st>>>(src, perm, n, nrhs, dst);
}
template <typename T>
void launch_from_new(const T* src, const int* perm, int n, int nrhs, double* dst, int acc, cudaStream_t st) {
  from_new_kernel<T><<<nblk(int64_t(n) * nrhs, 256), 256, 0, st>>>(src, perm, n, nrhs, dst, acc);
}
template void launch_to_new<double>(const double*, const int*, int, int, double*, cudaStream_t);
template void launch_to_new<float>(const double*, const int*, int, int, float*, cudaStream_t);
template void launch_from_new<double>(const double*, const int*, int, int, double*, int, cudaStream_t);
template void launch_from_new<float>(const float*, const int*, int, int, double*, int, cudaStream_t);

}  // namespace spde
