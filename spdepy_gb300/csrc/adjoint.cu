// Adjoint of the assembly: given a symmetric cotangent Gbar on the stencil of Q
// (natural order, nslots per node), compute d/dtheta <Gbar, Q(theta)> for every
// canonical parameter except log tau.
//
// The reference materialises one n x n matrix dQ_i per parameter and contracts
// it with Hutchinson probes (spdes/advection_diffusion2D.py:119-183,200-207;
// spdes/var_advection_var_diffusion2D.py:118-197).  Here the contraction is run
// backwards once: the time blocks of Gbar are summed (the coefficients are
// time-invariant), pushed through Q = blocks(A, Qs, Q0) to the 9-point operator A,
// through the stencil formulas to the per-face H and w and per-cell kappa, and
// through the B-spline bases to the coefficients.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "engine.cuh"
#include "stencil.cuh"

namespace spde {

constexpr int kCW = 22;  // per-cell partial gradient width

// --- time reduction: per cell, G0/Gmid/Glast (25) and Goff (9); T == 1: G (25)
__global__ void time_reduce_kernel(int Ns, int T, int nslots, const double* __restrict__ gbar,
                                   double* __restrict__ red /* Ns x 84 */) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(Ns) * 34) return;
  const int c = int(e / 34), s = int(e % 34);
  double* r = red + int64_t(c) * 84;
  if (T == 1) {
    if (s < 25) r[s] = gbar[int64_t(c) * nslots + s];
    return;
  }
  if (s < 25) {
    const int slot = 9 + s;
    double g0 = gbar[int64_t(c) * nslots + slot];
    double gm = 0.0;
    for (int t = 1; t < T - 1; ++t) gm += gbar[(int64_t(t) * Ns + c) * nslots + slot];
    double gl = gbar[(int64_t(T - 1) * Ns + c) * nslots + slot];
    r[s] = g0; r[25 + s] = gm; r[50 + s] = gl;
  } else {
    const int p = s - 25;  // dt = +1 slot p
    double go = 0.0;
    for (int t = 0; t < T - 1; ++t) go += gbar[(int64_t(t) * Ns + c) * nslots + 34 + p];
    r[75 + p] = go;
  }
}

// (A G)[m, m + d] for the 9 offsets d, G a symmetric 25-point field per cell at
// stride `gs` with offset `go` inside each cell's record.
__device__ void a_times_g(const double* Ag, const double* G, int gs, int go, int m, int M, int N, double* out,
                          const double* G2 = nullptr, int go2 = 0) {
  const int j = m / M, i = m - j * M;
  const double* Am = Ag + int64_t(m) * 9;
  for (int d = 0; d < 9; ++d) out[d] = 0.0;
  for (int d1 = 0; d1 < 9; ++d1) {
    const int dx1 = d1 % 3 - 1, dy1 = d1 / 3 - 1;
    const int ki = i + dx1, kj = j + dy1;
    if (ki < 0 || ki >= M || kj < 0 || kj >= N) continue;
    const double a = Am[d1];
    if (a == 0.0) continue;
    const int k = kj * M + ki;
    const double* Gk = G + int64_t(k) * gs + go;
    const double* Gk2 = G2 ? G2 + int64_t(k) * gs + go2 : nullptr;
    for (int d = 0; d < 9; ++d) {
      const int ox = (d % 3 - 1) - dx1, oy = (d / 3 - 1) - dy1;  // l - k
      const int s = (oy + 2) * 5 + (ox + 2);
      double g = Gk[s];
      if (Gk2) g += Gk2[s];
      out[d] += a * g;
    }
  }
}

// d/d(eight face coefficients) of the diffusion stencil, given the gradient of
// every raw entry (folded entries take the centre's gradient, dropped ones 0).
struct FaceGrad {
  double W00, E00, N01, S01, N11, S11, E10, W10;
};
__device__ FaceGrad diffusion_adjoint(const double* gA /*geo 9*/, double hx, double hy, int i, int j, int M, int N,
                                      int bc) {
  CellH h{};
  double v[9];
  int col[9];
  bool keep[9];
  diffusion_cell(h, hx, hy, i, j, M, N, bc, v, col, keep);  // only the pattern is used
  double g[9];
  g[0] = gA[4];
  for (int p = 1; p < 9; ++p) {
    if (keep[p]) g[p] = gA[geo9(col[p], i, j, M)];
    else g[p] = bc == 1 ? gA[4] : 0.0;
  }
  const double ha = hy / hx, hb = hx / hy;
  FaceGrad r;
  r.E00 = -ha * g[0] + ha * g[1];
  r.W00 = -ha * g[0] + ha * g[2];
  r.N11 = -hb * g[0] + hb * g[3];
  r.S11 = -hb * g[0] + hb * g[4];
  r.N01 = 0.25 * (g[1] - g[2] + g[5] - g[7]);
  r.S01 = 0.25 * (-g[1] + g[2] + g[6] - g[8]);
  r.E10 = 0.25 * (g[3] - g[4] + g[5] - g[8]);
  r.W10 = 0.25 * (-g[3] + g[4] + g[6] - g[7]);
  return r;
}

// d/d(log gamma, vx, vy) of H given dL/dH = {g00, g01, g10, g11}.
__device__ void h_adjoint(int diff, double gamma, double vx, double vy, const double* gH, double* out) {
  const double gsum = gH[1] + gH[2];
  if (diff == 0) {
    out[0] = gamma * (gH[0] + gH[3]); out[1] = 0.0; out[2] = 0.0;
  } else if (diff == 1) {
    out[0] = gamma * (gH[0] + gH[3]);
    out[1] = 2.0 * vx * gH[0] + vy * gsum;
    out[2] = 2.0 * vy * gH[3] + vx * gsum;
  } else {
    const double a2 = vx * vx + vy * vy, a = sqrt(a2);
    double ch, r, shoa, q;  // cosh a, sinh(a)/a, sinh(a)/a again, (cosh a - sinh(a)/a)/a^2
    if (a > 1e-4) {
      double ea = exp(a), eb = exp(-a);
      ch = (ea + eb) / 2;
      shoa = (ea - eb) / 2 / a;
      q = (ch - shoa) / a2;
    } else {
      ch = 1.0 + a2 / 2;
      shoa = 1.0 + a2 / 6;
      q = 1.0 / 3.0 + a2 / 30;
    }
    r = shoa;
    const double H00 = gamma * (ch + r * vx), H01 = gamma * r * vy, H11 = gamma * (ch - r * vx);
    out[0] = gH[0] * H00 + gsum * H01 + gH[3] * H11;  // dH/dlog gamma = H
    // d ch/dv = shoa * v ; d r/dv = q * v
    const double drx = q * vx, dry = q * vy;
    const double d00x = gamma * (shoa * vx + drx * vx + r), d01x = gamma * drx * vy, d11x = gamma * (shoa * vx - drx * vx - r);
    const double d00y = gamma * (shoa * vy + dry * vx), d01y = gamma * (dry * vy + r), d11y = gamma * (shoa * vy - dry * vx);
    out[1] = gH[0] * d00x + gsum * d01x + gH[3] * d11x;
    out[2] = gH[0] * d00y + gsum * d01y + gH[3] * d11y;
  }
}

__device__ __forceinline__ double sgn0(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

__device__ double dotb2(const double* b, const double* c, int nb) {
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s = fma(b[i], c[i], s);
  return s;
}

__global__ void cell_adjoint_kernel(DevModel m, const double* __restrict__ red, const double* __restrict__ Ageo,
                                    const double* __restrict__ A0geo, const double* __restrict__ kap,
                                    const double* __restrict__ qs, double cfac, double* __restrict__ cg) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.Ns) return;
  const int M = m.Mx, N = m.Ny;
  const int j = c / M, i = c - j * M;
  const bool st = m.T > 1;
  const double V = m.V;
  double* out = cg + int64_t(c) * kCW;
  for (int k = 0; k < kCW; ++k) out[k] = 0.0;
  const double* rc = red + int64_t(c) * 84;
  const double* Am = Ageo + int64_t(c) * 9;
  double gA[9], ag[9];
  double gQs = 0.0, lsig = 0.0;
  if (st) {
    // G2 = Gmid + Glast
    a_times_g(Ageo, red, 84, 25, c, M, N, ag, red, 50);
    const double Dm = qs[c] / (V * V);
    double aga = 0.0, goa = 0.0;
    for (int d = 0; d < 9; ++d) {
      gA[d] = cfac * (2.0 * Dm * ag[d] - 2.0 * (qs[c] / V) * rc[75 + d]);
      aga += ag[d] * Am[d];
      goa += rc[75 + d] * Am[d];
    }
    gQs = cfac * (rc[12] + rc[25 + 12]) + cfac / (V * V) * aga - 2.0 * cfac / V * goa;
    lsig = -(cfac * (rc[12] + rc[25 + 12]) * qs[c] + cfac * Dm * aga - 2.0 * cfac * (qs[c] / V) * goa);
  } else {
    a_times_g(Ageo, red, 84, 0, c, M, N, ag);
    for (int d = 0; d < 9; ++d) gA[d] = 2.0 / V * ag[d];
  }
  const double kc = kap[c];
  // kappa: A's centre and (spatio-temporal) Qs = V kappa^2; per log kappa
  double gk = st ? (m.dt * V * gA[4] + gQs * 2.0 * V * kc) : V * gA[4];
  out[0] = gk * kc;
  // diffusion: A_H enters with -dt (or -1)
  double gAH[9];
  const double sc = st ? m.dt : 1.0;
  for (int d = 0; d < 9; ++d) gAH[d] = -sc * gA[d];
  FaceGrad fgr = diffusion_adjoint(gAH, m.hx, m.hy, i, j, M, N, m.bc);
  // per-face dL/dH {00, 01, 10, 11}, faces W,E,S,N
  double gH[4][4] = {{fgr.W00, 0.0, fgr.W10, 0.0}, {fgr.E00, 0.0, fgr.E10, 0.0},
                     {0.0, fgr.S01, 0.0, fgr.S11}, {0.0, fgr.N01, 0.0, fgr.N11}};
  if (m.var_h) {
    if (m.bc == 1 && c == 0) { gH[0][0] = 0.0; gH[0][2] = 0.0; gH[2][3] = 0.0; gH[2][1] = 0.0; }
    const double* th = m.theta;
    for (int f = 0; f < 4; ++f) {
      const double* b = m.bsH + (int64_t(c) * 4 + f) * m.nbasis;
      double gamma = exp(dotb2(b, th + m.nk, m.nbasis));
      double vx = m.diff ? dotb2(b, th + 2 * m.nk, m.nbasis) : 0.0;
      double vy = m.diff ? dotb2(b, th + 3 * m.nk, m.nbasis) : 0.0;
      double o3[3];
      h_adjoint(m.diff, gamma, vx, vy, gH[f], o3);
      out[1 + f] = o3[0]; out[5 + f] = o3[1]; out[9 + f] = o3[2];
    }
  } else {
    // constant H: zero the current boundary faces (bc 1) and fold onto one 2x2
    if (m.bc == 1) {
      if (i == 0) { gH[0][0] = 0.0; gH[0][2] = 0.0; }
      else if (i == M - 1) { gH[1][0] = 0.0; gH[1][2] = 0.0; }
      if (j == 0) { gH[2][3] = 0.0; gH[2][1] = 0.0; }
      else if (j == N - 1) { gH[3][3] = 0.0; gH[3][1] = 0.0; }
    }
    double g2[4] = {gH[0][0] + gH[1][0], 0.0, 0.0, gH[2][3] + gH[3][3]};
    const double cross = gH[2][1] + gH[3][1] + gH[0][2] + gH[1][2];
    if (m.bc == 1) { g2[2] = cross; }
    else { g2[1] = gH[2][1] + gH[3][1]; g2[2] = gH[0][2] + gH[1][2]; }
    const double* th = m.theta;
    double o3[3];
    h_adjoint(m.diff, exp(th[m.nk]), m.diff ? th[2 * m.nk] : 0.0, m.diff ? th[3 * m.nk] : 0.0, g2, o3);
    out[1] = o3[0]; out[5] = o3[1]; out[9] = o3[2];
  }
  // advection: A_w enters with +dt
  if (m.adv) {
    double gAw[9];
    for (int d = 0; d < 9; ++d) gAw[d] = m.dt * gA[d];
    double v[5];
    int col[5];
    bool keep[5];
    double wf[4] = {0.0, 0.0, 0.0, 0.0};
    const double* tw = m.theta + 4 * m.nk;
    if (m.adv == 1) { wf[0] = tw[0]; wf[1] = tw[1]; }
    else if (m.adv == 2) {
      for (int f = 0; f < 4; ++f)
        wf[f] = dotb2(m.bsA + (int64_t(c) * 4 + f) * m.nbasis, tw + ((f & 1) ? m.nbasis : 0), m.nbasis);
    } else {
      for (int f = 0; f < 4; ++f) wf[f] = tw[0] * m.ww[int64_t(c) * 4 + f];
    }
    advection_cell(wf, nullptr, m.adv != 1, m.hx, m.hy, i, j, M, N, m.bc, 3, v, col, keep);
    double g[5];
    for (int p = 0; p < 5; ++p) g[p] = keep[p] ? gAw[geo9(col[p], i, j, M)] : 0.0;
    const double hx = m.hx, hy = m.hy;
    if (m.adv == 1) {
      const double s0 = sgn0(wf[0]), s1 = sgn0(wf[1]);
      double cx = 1.0, cy = 1.0;
      if (m.bc == 1) {
        if (i == 0 || i == M - 1) cx = 0.5;
        if (j == 0 || j == N - 1) cy = 0.5;
      }
      out[13] = s0 * hy * cx * g[0] - (s0 - 1.0) * hy / 2 * g[1] - (s0 + 1.0) * hy / 2 * g[2];
      out[14] = s1 * hx * cy * g[0] - (s1 - 1.0) * hx / 2 * g[3] - (s1 + 1.0) * hx / 2 * g[4];
    } else {
      double gw[4];
      double gg[4] = {wf[0], wf[1], wf[2], wf[3]};
      bool zero[4] = {false, false, false, false};
      if (m.bc == 1) {
        zero[0] = !keep[1]; zero[2] = !keep[2]; zero[1] = !keep[3]; zero[3] = !keep[4];
        for (int f = 0; f < 4; ++f) if (zero[f]) gg[f] = 0.0;
      }
      const double s0 = sgn0(gg[0]), s1 = sgn0(gg[1]), s2 = sgn0(gg[2]), s3 = sgn0(gg[3]);
      gw[0] = (s0 + 1.0) * hy / 2 * g[0] - (s0 - 1.0) * hy / 2 * g[1];
      gw[2] = (s2 - 1.0) * hy / 2 * g[0] - (s2 + 1.0) * hy / 2 * g[2];
      gw[1] = (s1 + 1.0) * hx / 2 * g[0] - (s1 - 1.0) * hx / 2 * g[3];
      gw[3] = (s3 - 1.0) * hx / 2 * g[0] - (s3 + 1.0) * hx / 2 * g[4];
      for (int f = 0; f < 4; ++f) {
        if (zero[f]) gw[f] = 0.0;
        out[13 + f] = (m.adv == 3) ? gw[f] * m.ww[int64_t(c) * 4 + f] : gw[f];
      }
    }
  }
  if (st) {
    out[17] = lsig;
    // initial field Q0 = A0^T V^-1 A0
    double a0g[9];
    a_times_g(A0geo, red, 84, 0, c, M, N, a0g);
    double gA0[9];
    for (int d = 0; d < 9; ++d) gA0[d] = 2.0 / V * a0g[d];
    const double* t0 = m.theta + 4 * m.nk + m.nw + 1;
    out[18] = V * exp(t0[0]) * gA0[4];
    double gAH0[9];
    for (int d = 0; d < 9; ++d) gAH0[d] = -gA0[d];
    FaceGrad f0 = diffusion_adjoint(gAH0, m.hx, m.hy, i, j, M, N, m.mod0_bc);
    double h0[4][4] = {{f0.W00, 0.0, f0.W10, 0.0}, {f0.E00, 0.0, f0.E10, 0.0},
                       {0.0, f0.S01, 0.0, f0.S11}, {0.0, f0.N01, 0.0, f0.N11}};
    if (m.mod0_bc == 1) {
      if (i == 0) { h0[0][0] = 0.0; h0[0][2] = 0.0; }
      else if (i == M - 1) { h0[1][0] = 0.0; h0[1][2] = 0.0; }
      if (j == 0) { h0[2][3] = 0.0; h0[2][1] = 0.0; }
      else if (j == N - 1) { h0[3][3] = 0.0; h0[3][1] = 0.0; }
    }
    double g2[4] = {h0[0][0] + h0[1][0], 0.0, 0.0, h0[2][3] + h0[3][3]};
    if (m.mod0_bc == 1) g2[2] = h0[2][1] + h0[3][1] + h0[0][2] + h0[1][2];
    else { g2[1] = h0[2][1] + h0[3][1]; g2[2] = h0[0][2] + h0[1][2]; }
    double o3[3];
    h_adjoint(m.mod0_diff, exp(t0[1]), m.mod0_diff ? t0[2] : 0.0, m.mod0_diff ? t0[3] : 0.0, g2, o3);
    out[19] = o3[0]; out[20] = o3[1]; out[21] = o3[2];
  }
}

// One block per canonical parameter: reduce the per-cell partials through the bases.
__global__ void coef_reduce_kernel(DevModel m, const double* __restrict__ cg, double* __restrict__ grad) {
  __shared__ double red[256];
  const int p = blockIdx.x;
  const int nk = m.nk, nb = m.nbasis;
  int kind, idx;  // kind: 0 kappa 1 gamma 2 vx 3 vy 4 w 5 sigma 6 mod0
  if (p < 4 * nk) { kind = p / nk; idx = p % nk; }
  else if (p < 4 * nk + m.nw) { kind = 4; idx = p - 4 * nk; }
  else if (p == 4 * nk + m.nw) { kind = 5; idx = 0; }
  else { kind = 6; idx = p - (4 * nk + m.nw + 1); }
  double s = 0.0;
  for (int c = threadIdx.x; c < m.Ns; c += 256) {
    const double* o = cg + int64_t(c) * kCW;
    switch (kind) {
      case 0: s += m.var_h ? m.bs[int64_t(c) * nb + idx] * o[0] : o[0]; break;
      case 1: case 2: case 3: {
        const int base = kind == 1 ? 1 : (kind == 2 ? 5 : 9);
        for (int f = 0; f < 4; ++f) s += (m.var_h ? m.bsH[(int64_t(c) * 4 + f) * nb + idx] : 1.0) * o[base + f];
        break;
      }
      case 4:
        if (m.adv == 1) s += o[13 + idx];
        else if (m.adv == 2) {
          const int comp = idx / nb, ii = idx % nb;  // 0: wx (faces E, W), 1: wy (faces N, S)
          for (int f = comp; f < 4; f += 2) s += m.bsA[(int64_t(c) * 4 + f) * nb + ii] * o[13 + f];
        } else {
          for (int f = 0; f < 4; ++f) s += o[13 + f];
        }
        break;
      case 5: s += o[17]; break;
      default: s += o[18 + idx]; break;
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bool used = true;
    if ((kind == 2 || kind == 3) && m.diff == 0) used = false;
    if ((kind == 5 || kind == 6) && m.T == 1) used = false;
    grad[p] = used ? red[0] : 0.0;
  }
}

int64_t adjoint_work_elems(const Plan* p) { return int64_t(p->sym.Mx) * p->sym.Ny * kAdjointCellElems; }
static_assert(kAdjointCellElems == 84 + kCW, "adjoint work per cell: 84 reduced stencil values + kCW partials");

// ---------------------------------------------------------------------------
// Fixed scratch of the allocation-free adjoint entry point (spde_adjoint_noalloc).
// It lives in the module's static device memory: every GPU that loads this
// library holds these 8 MiB until the process exits.  In host code the symbol is
// only a stand-in, so its device address is looked up once per device, with that
// device current, and cached.
constexpr int64_t kNoAllocElems = int64_t(1) << 20;  // doubles
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocElems];

int noalloc_scratch(int dev, double** ptr, int64_t* elems) {
  static std::mutex mu;
  static double* cache[64] = {nullptr};
  if (dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if (!cache[dev]) {
    // the lookup must run with `dev` current: switch to it and back
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return 1;
    if (cur != dev && cudaSetDevice(dev) != cudaSuccess) return 1;
    void* addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (cur != dev) cudaSetDevice(cur);
    if (e != cudaSuccess || !addr) return 1;
    cache[dev] = static_cast<double*>(addr);
  }
  *ptr = cache[dev];
  *elems = kNoAllocElems;
  return 0;
}

// --- separable models Q = Qt (x) Qs.  Per cell c: the spatial cotangent
// Gs(c, s) = sum_t sum_dt Qt(t, t + dt) Gbar(t, c, dt, s) into red[c 84 + s]
// (the spatial adjoint then gives every Qs parameter), and the partial sums
// sum_s Gbar-class(c, s) Qs(c, s) for the end-diagonal, interior-diagonal and
// off-diagonal classes of Qt into red[c 84 + 25 .. 27].
__global__ void sep_reduce_kernel(int Ns, int T, double qe, double qm, double qo, const double* __restrict__ gbar,
                                  const double* __restrict__ Qs, double* __restrict__ red) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= Ns) return;
  double* r = red + int64_t(c) * 84;
  double pe = 0.0, pm = 0.0, po = 0.0;
  for (int s = 0; s < 25; ++s) {
    double ee = 0.0, em = 0.0, eo = 0.0;
    for (int t = 0; t < T; ++t) {
      const double* g = gbar + (int64_t(t) * Ns + c) * 75;
      if (t == 0 || t == T - 1) ee += g[25 + s];
      else em += g[25 + s];
      eo += g[s] + g[50 + s];  // slots outside the lattice hold zero
    }
    r[s] = qe * ee + qm * em + qo * eo;
    const double q = Qs[int64_t(c) * 25 + s];
    pe += ee * q;
    pm += em * q;
    po += eo * q;
  }
  r[25] = pe;
  r[26] = pm;
  r[27] = po;
}

// Gradient of the two temporal parameters: sum_c of the partials, weighted by
// the derivatives of (end, interior, off) of Qt; one block.
__global__ void sep_temporal_kernel(int Ns, const double* __restrict__ red, double a0, double a1, double a2,
                                    double b0, double b1, double b2, double* __restrict__ grad) {
  __shared__ double sh[3][256];
  double e0 = 0.0, e1 = 0.0, e2 = 0.0;
  for (int c = threadIdx.x; c < Ns; c += 256) {
    const double* r = red + int64_t(c) * 84;
    e0 += r[25];
    e1 += r[26];
    e2 += r[27];
  }
  sh[0][threadIdx.x] = e0;
  sh[1][threadIdx.x] = e1;
  sh[2][threadIdx.x] = e2;
  __syncthreads();
  for (int q = 128; q > 0; q >>= 1) {
    if (threadIdx.x < q)
      for (int i = 0; i < 3; ++i) sh[i][threadIdx.x] += sh[i][threadIdx.x + q];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    grad[0] = a0 * sh[0][0] + a1 * sh[1][0] + a2 * sh[2][0];
    grad[1] = b0 * sh[0][0] + b1 * sh[1][0] + b2 * sh[2][0];
  }
}

void launch_adjoint(const Plan* p, const double* gbar, double* grad_dev, double* work, cudaStream_t st) {
  const int Ns = p->sym.Mx * p->sym.Ny;
  double* red = work;
  double* cg = work + int64_t(Ns) * 84;
  if (p->temporal) {
    const DevModel ms = spatial_view(p->model);
    const int to = 4 * ms.nk + ms.nw;
    double qt[3], d1[3], d2[3];
    separable_qt(p->temporal, p->theta[to], p->theta[to + 1], qt, d1, d2);
    sep_reduce_kernel<<<(Ns + 127) / 128, 128, 0, st>>>(Ns, p->sym.T, qt[0], qt[1], qt[2], gbar, p->d_QA, red);
    cell_adjoint_kernel<<<(Ns + 127) / 128, 128, 0, st>>>(ms, red, p->d_Ageo, p->d_A0geo, p->d_kap, p->d_qs, 1.0,
                                                           cg);
    coef_reduce_kernel<<<4 * ms.nk + ms.nw + 5, 256, 0, st>>>(ms, cg, grad_dev);
    sep_temporal_kernel<<<1, 256, 0, st>>>(Ns, red, d1[0], d1[1], d1[2], d2[0], d2[1], d2[2], grad_dev + to);
    return;
  }
  int64_t tot = int64_t(Ns) * 34;
  time_reduce_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(Ns, p->sym.T, p->sym.nslots, gbar, red);
  cell_adjoint_kernel<<<(Ns + 127) / 128, 128, 0, st>>>(p->model, red, p->d_Ageo, p->d_A0geo, p->d_kap, p->d_qs,
                                                         p->cfac, cg);
  const int ntheta = 4 * p->model.nk + p->model.nw + 5;  // all but log tau
  coef_reduce_kernel<<<ntheta, 256, 0, st>>>(p->model, cg, grad_dev);
}

}  // namespace spde
