// Learned space-time preconditioner and preconditioned conjugate gradients for
// A = Q (+ tau S^T S) on grids too large to factor.
//
// The preconditioner is a factorised sparse approximate inverse M^-1 = G^T G.
// G is a 27-point stencil on the (x, y, t) lattice (dx, dy, dt in {-1, 0, 1})
// whose per-node weights come from a small network that reads the node's own
// row of A: w_o(p) = (delta_o,centre + N(f_p)_o) / sqrt(A_pp), with
// f_p = A_p,. / A_pp over the 43-slot stencil (centre dropped) and N a
// 42-32-32-27 perceptron with tanh activations.  A zero last layer gives the
// Jacobi preconditioner.  Training minimises
//   L = E_z || z - G A G^T z ||^2 / (n k)
// over probe blocks z (n x k), i.e. drives G A G^T towards the identity; the
// gradient with respect to the weights is
//   dL/dw_o(p) = -2/(n k) sum_r (e_pr u_(p+o)r + z_pr g_(p+o)r)
// with y = G^T z, u = A y, e = z - G u, g = A G^T e, and flows into the network
// through its own backward kernel.  Parameters live in caller-owned FP32
// device memory; every reduction is a fixed-order two-pass sum, so results are
// deterministic.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "engine.cuh"

namespace spde {

namespace {

constexpr int kFeat = kPcFeat, kHid = kPcHidden, kOff = kPcOffsets;
constexpr int kW1 = 0, kB1 = kW1 + kHid * kFeat, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kOff * kHid, kNP = kB3 + kOff;
static_assert(kNP == kPcParams, "parameter layout");
constexpr int kAct = kFeat + 2 * kHid + 1;  // per node: f, h1, h2, 1 / sqrt(A_pp)
constexpr int kCentre43 = 21;               // centre slot of the 43-slot layout

__device__ __forceinline__ void off27(int o, int* dx, int* dy, int* dt) {
  *dt = o / 9 - 1;
  *dy = (o / 3) % 3 - 1;
  *dx = o % 3 - 1;
}

// 43-slot layout offsets (dt = -1: 3 x 3, dt = 0: 5 x 5, dt = +1: 3 x 3)
__device__ __forceinline__ void off43(int s, int* dx, int* dy, int* dt) {
  if (s < 9) { *dt = -1; *dy = s / 3 - 1; *dx = s % 3 - 1; }
  else if (s < 34) { *dt = 0; *dy = (s - 9) / 5 - 2; *dx = (s - 9) % 5 - 2; }
  else { *dt = 1; *dy = (s - 34) / 3 - 1; *dx = (s - 34) % 3 - 1; }
}

__device__ __forceinline__ bool inside(const QStencil& q, int x, int y, int t) {
  return x >= 0 && x < q.Mx && y >= 0 && y < q.Ny && t >= 0 && t < q.T;
}

// Features, network forward and the 27 G weights of the row of A at (cell c,
// time t), whose diagonal carries the observation term `obs_term`; `act`
// (optional) receives the activations a gradient step needs.
__device__ __forceinline__ void pc_network(const QStencil& q, int c, int t, double obs_term, const float* sp,
                                           float* wout, float* act) {
  const int y = c / q.Mx, x = c - y * q.Mx;
  double diag = qval(q, c, t, 0, 0, 0) + obs_term;
  if (!(diag > 0.0)) diag = 1.0;
  const double rd = 1.0 / diag;
  float f[kFeat];
#pragma unroll
  for (int s = 0; s < 43; ++s) {
    if (s == kCentre43) continue;
    int dx, dy, dt;
    off43(s, &dx, &dy, &dt);
    double v = 0.0;
    if ((q.T > 1 || dt == 0) && inside(q, x + dx, y + dy, t + dt)) v = qval(q, c, t, dx, dy, dt) * rd;
    f[s < kCentre43 ? s : s - 1] = float(v);
  }
  float h1[kHid], h2[kHid];
#pragma unroll 4
  for (int i = 0; i < kHid; ++i) {
    float a = sp[kB1 + i];
#pragma unroll
    for (int j = 0; j < kFeat; ++j) a = fmaf(sp[kW1 + i * kFeat + j], f[j], a);
    h1[i] = tanhf(a);
  }
#pragma unroll 4
  for (int i = 0; i < kHid; ++i) {
    float a = sp[kB2 + i];
#pragma unroll
    for (int j = 0; j < kHid; ++j) a = fmaf(sp[kW2 + i * kHid + j], h1[j], a);
    h2[i] = tanhf(a);
  }
  const float s = float(rsqrt(diag));
  for (int o = 0; o < kOff; ++o) {
    float a = sp[kB3 + o];
#pragma unroll
    for (int j = 0; j < kHid; ++j) a = fmaf(sp[kW3 + o * kHid + j], h2[j], a);
    int dx, dy, dt;
    off27(o, &dx, &dy, &dt);
    const bool in = inside(q, x + dx, y + dy, t + dt);
    wout[o] = in ? ((o == 13 ? 1.f : 0.f) + a) * s : 0.f;
  }
  if (act) {
#pragma unroll
    for (int j = 0; j < kFeat; ++j) act[j] = f[j];
#pragma unroll
    for (int j = 0; j < kHid; ++j) act[kFeat + j] = h1[j];
#pragma unroll
    for (int j = 0; j < kHid; ++j) act[kFeat + kHid + j] = h2[j];
    act[kAct - 1] = s;
  }
}

// G weights of every node, offset-major (w[o n + p]), one thread per node.
__global__ void __launch_bounds__(128) pc_forward_kernel(QStencil q, const double* __restrict__ obs, double tau,
                                                         const float* __restrict__ prm, float* __restrict__ w,
                                                         float* __restrict__ act) {
  __shared__ float sp[kNP];
  for (int i = threadIdx.x; i < kNP; i += blockDim.x) sp[i] = prm[i];
  __syncthreads();
  const int64_t n = int64_t(q.Ns) * q.T;
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int t = int(p / q.Ns), c = int(p - int64_t(t) * q.Ns);
  float wo[kOff];
  pc_network(q, c, t, obs ? tau * obs[p] : 0.0, sp, wo, act ? act + p * kAct : nullptr);
#pragma unroll
  for (int o = 0; o < kOff; ++o) w[int64_t(o) * n + p] = wo[o];
}

// Compact weights.  A node's row of A depends on its time only through three
// classes (first step, interior steps, last step: the stencil coefficients are
// time-invariant) unless the node is observed, so G has one row per (class,
// cell) and one per distinct observed node: w[(k 27 + o) Ns + c] for class k,
// then w[27 3 Ns + o nob + j] for the j-th observed node.  One thread per row.
__global__ void __launch_bounds__(128) pc_forward_compact_kernel(QStencil q, const double* __restrict__ obs,
                                                                 double tau, const int* __restrict__ obs_nodes,
                                                                 int nob, const float* __restrict__ prm,
                                                                 float* __restrict__ w) {
  __shared__ float sp[kNP];
  for (int i = threadIdx.x; i < kNP; i += blockDim.x) sp[i] = prm[i];
  __syncthreads();
  const int64_t ncls = int64_t(3) * q.Ns;
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= ncls + nob) return;
  float wo[kOff];
  if (e < ncls) {
    const int k = int(e / q.Ns), c = int(e - int64_t(k) * q.Ns);
    const int t = k == 0 ? 0 : (k == 1 ? (q.T > 2 ? 1 : 0) : q.T - 1);
    pc_network(q, c, t, 0.0, sp, wo, nullptr);
#pragma unroll
    for (int o = 0; o < kOff; ++o) w[(int64_t(k) * kOff + o) * q.Ns + c] = wo[o];
  } else {
    const int j = int(e - ncls);
    const int p = obs_nodes[j];
    const int t = p / q.Ns, c = p - t * q.Ns;
    pc_network(q, c, t, obs ? tau * obs[p] : 0.0, sp, wo, nullptr);
#pragma unroll
    for (int o = 0; o < kOff; ++o) w[ncls * kOff + int64_t(o) * nob + j] = wo[o];
  }
}

// out = G x (transpose = 0) or G^T x (transpose = 1); x, out n x nrhs row-major;
// weights offset-major (w[o n + p]), so every offset's read is coalesced.  The
// 27 offsets are unrolled (compile-time displacements, loads issued together);
// node indices fit in 32 bits (checked by the caller).
template <int TRANS, typename TIn, typename TOut>
__global__ void pc_apply_kernel(QStencil q, const float* __restrict__ w, const TIn* __restrict__ x,
                                TOut* __restrict__ out, int nrhs) {
  const int n = q.Ns * q.T;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int p = nrhs == 1 ? e : e / nrhs;
  const int r = e - p * nrhs;
  const int t = p / q.Ns, c = p - t * q.Ns;
  const int y = c / q.Mx, xx = c - y * q.Mx;
  const int sy = q.Mx, st = q.Ns;
  // FP32 arithmetic: a preconditioner only has to be a fixed SPD operator, and
  // FP64 is a narrow pipe on this part
  float acc = 0.f;
#pragma unroll
  for (int o = 0; o < kOff; ++o) {
    const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dt = o / 9 - 1;
    const int sgn = TRANS ? -1 : 1;
    const int x2 = xx + sgn * dx, y2 = y + sgn * dy, t2 = t + sgn * dt;
    if (x2 < 0 || x2 >= q.Mx || y2 < 0 || y2 >= q.Ny || t2 < 0 || t2 >= q.T) continue;
    const int nb = p + sgn * (dt * st + dy * sy + dx);
    const float wv = TRANS ? w[int64_t(o) * n + nb] : w[int64_t(o) * n + p];
    acc = fmaf(wv, float(x[int64_t(nb) * nrhs + r]), acc);
  }
  out[e] = TOut(acc);
}

__global__ void pc_sub_kernel(const double* __restrict__ z, double* __restrict__ v, int64_t len) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < len) v[i] = z[i] - v[i];
}

// dL/d(network output) per node: (sum_r e_pr u_(p+o)r + z_pr g_(p+o)r) * scale * s_p
__global__ void pc_wgrad_kernel(QStencil q, const double* __restrict__ z, const double* __restrict__ e,
                                const double* __restrict__ u, const double* __restrict__ g, int nrhs, double scale,
                                const float* __restrict__ act, float* __restrict__ dout) {
  const int64_t n = int64_t(q.Ns) * q.T;
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int t = int(p / q.Ns), c = int(p - int64_t(t) * q.Ns);
  const int y = c / q.Mx, x = c - y * q.Mx;
  const double s = act[p * kAct + kAct - 1];
  for (int o = 0; o < kOff; ++o) {
    int dx, dy, dt;
    off27(o, &dx, &dy, &dt);
    double acc = 0.0;
    if (inside(q, x + dx, y + dy, t + dt)) {
      const int64_t nb = p + (int64_t(dt) * q.Ny + dy) * q.Mx + dx;
      for (int r = 0; r < nrhs; ++r)
        acc += e[p * nrhs + r] * u[nb * nrhs + r] + z[p * nrhs + r] * g[nb * nrhs + r];
    }
    dout[p * kOff + o] = float(acc * scale * s);
  }
}

// Network backward: per block of kBwNodes nodes, the parameter gradient of the
// block's nodes into its own row of `part` (nblocks x kNP).
constexpr int kBwNodes = 64;
__global__ void __launch_bounds__(128) pc_backward_kernel(int64_t n, const float* __restrict__ prm,
                                                          const float* __restrict__ act,
                                                          const float* __restrict__ dout, float* __restrict__ part) {
  extern __shared__ float sm[];
  float* sW2 = sm;                              // kHid * kHid
  float* sW3 = sW2 + kHid * kHid;               // kOff * kHid
  float* sf = sW3 + kOff * kHid;                // kBwNodes * kFeat
  float* sh1 = sf + kBwNodes * kFeat;           // kBwNodes * kHid
  float* sh2 = sh1 + kBwNodes * kHid;
  float* sdo = sh2 + kBwNodes * kHid;           // kBwNodes * kOff
  float* sd2 = sdo + kBwNodes * kOff;           // kBwNodes * kHid
  float* sd1 = sd2 + kBwNodes * kHid;
  const int tid = threadIdx.x;
  for (int i = tid; i < kHid * kHid; i += blockDim.x) sW2[i] = prm[kW2 + i];
  for (int i = tid; i < kOff * kHid; i += blockDim.x) sW3[i] = prm[kW3 + i];
  const int64_t p0 = int64_t(blockIdx.x) * kBwNodes;
  const int cnt = n - p0 < kBwNodes ? int(n - p0) : kBwNodes;
  for (int i = tid; i < kBwNodes * kFeat; i += blockDim.x) {
    const int a = i / kFeat, j = i - a * kFeat;
    sf[i] = a < cnt ? act[(p0 + a) * kAct + j] : 0.f;
  }
  for (int i = tid; i < kBwNodes * kHid; i += blockDim.x) {
    const int a = i / kHid, j = i - a * kHid;
    sh1[i] = a < cnt ? act[(p0 + a) * kAct + kFeat + j] : 0.f;
    sh2[i] = a < cnt ? act[(p0 + a) * kAct + kFeat + kHid + j] : 0.f;
  }
  for (int i = tid; i < kBwNodes * kOff; i += blockDim.x) {
    const int a = i / kOff;
    sdo[i] = a < cnt ? dout[(p0 + a) * kOff + (i - a * kOff)] : 0.f;
  }
  __syncthreads();
  // dh2 = W3^T dout (1 - h2^2), then dh1 = W2^T dh2 (1 - h1^2)
  for (int i = tid; i < kBwNodes * kHid; i += blockDim.x) {
    const int a = i / kHid, j = i - a * kHid;
    float acc = 0.f;
    for (int o = 0; o < kOff; ++o) acc = fmaf(sW3[o * kHid + j], sdo[a * kOff + o], acc);
    const float h = sh2[i];
    sd2[i] = acc * (1.f - h * h);
  }
  __syncthreads();
  for (int i = tid; i < kBwNodes * kHid; i += blockDim.x) {
    const int a = i / kHid, j = i - a * kHid;
    float acc = 0.f;
    for (int k = 0; k < kHid; ++k) acc = fmaf(sW2[k * kHid + j], sd2[a * kHid + k], acc);
    const float h = sh1[i];
    sd1[i] = acc * (1.f - h * h);
  }
  __syncthreads();
  float* out = part + int64_t(blockIdx.x) * kNP;
  for (int e = tid; e < kNP; e += blockDim.x) {
    float acc = 0.f;
    if (e < kB1) {
      const int i = e / kFeat, j = e - i * kFeat;
      for (int a = 0; a < kBwNodes; ++a) acc = fmaf(sd1[a * kHid + i], sf[a * kFeat + j], acc);
    } else if (e < kW2) {
      const int i = e - kB1;
      for (int a = 0; a < kBwNodes; ++a) acc += sd1[a * kHid + i];
    } else if (e < kB2) {
      const int i = (e - kW2) / kHid, j = (e - kW2) - i * kHid;
      for (int a = 0; a < kBwNodes; ++a) acc = fmaf(sd2[a * kHid + i], sh1[a * kHid + j], acc);
    } else if (e < kW3) {
      const int i = e - kB2;
      for (int a = 0; a < kBwNodes; ++a) acc += sd2[a * kHid + i];
    } else if (e < kB3) {
      const int o = (e - kW3) / kHid, j = (e - kW3) - o * kHid;
      for (int a = 0; a < kBwNodes; ++a) acc = fmaf(sdo[a * kOff + o], sh2[a * kHid + j], acc);
    } else {
      const int o = e - kB3;
      for (int a = 0; a < kBwNodes; ++a) acc += sdo[a * kOff + o];
    }
    out[e] = acc;
  }
}

// grad[e] = sum over blocks of part[b][e] (fixed order)
__global__ void pc_colsum_kernel(const float* __restrict__ part, int nb, float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kNP) return;
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) acc += part[int64_t(b) * kNP + e];
  grad[e] = float(acc);
}

// Column-wise dot products of a and b (n x nrhs row-major): two-pass, fixed order.
constexpr int kDotBlocks = 256;
__global__ void pc_dot_partial_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n, int nrhs,
                                      double* __restrict__ part) {
  __shared__ double red[256];
  for (int r = 0; r < nrhs; ++r) {
    double acc = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
      acc += a[i * nrhs + r] * b[i * nrhs + r];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
      if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[int64_t(r) * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}
// The same for many columns: lane = column within a 32-column chunk
// (blockIdx.y), warps stride over the rows, so each row segment is read
// contiguously; part[r * gridDim.x + block] as in pc_dot_partial_kernel.
__global__ void pc_dot_wide_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n, int nrhs,
                                   double* __restrict__ part) {
  __shared__ double red[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = blockIdx.y * 32 + lane;
  double acc = 0.0;
  if (r < nrhs)
    for (int64_t i = int64_t(blockIdx.x) * 8 + warp; i < n; i += int64_t(gridDim.x) * 8)
      acc += a[i * nrhs + r] * b[i * nrhs + r];
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && r < nrhs) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w][lane];
    part[int64_t(r) * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void pc_dot_final_kernel(const double* __restrict__ part, int nblocks, int nrhs, double* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs) return;
  double acc = 0.0;
  for (int b = 0; b < nblocks; ++b) acc += part[int64_t(r) * nblocks + b];
  out[r] = acc;
}

// z -= omega D^-1 (A z) for one damped-Jacobi sweep (az = A z)
__global__ void jacobi_sweep_kernel(QStencil q, const double* __restrict__ obs, double tau, double omega,
                                    const double* __restrict__ az, double* __restrict__ z, int nrhs) {
  const int64_t n = int64_t(q.Ns) * q.T;
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t p = e / nrhs;
  const int t = int(p / q.Ns), c = int(p - int64_t(t) * q.Ns);
  const double d = qval(q, c, t, 0, 0, 0) + (obs ? tau * obs[p] : 0.0);
  z[e] -= omega * az[e] / d;
}
// z[:, r] *= 1 / sqrt(ss[r] / n)
__global__ void col_scale_kernel(double* __restrict__ z, const double* __restrict__ ss, int64_t n, int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int r = int(e % nrhs);
  const double ms = ss[r] / double(n);
  if (ms > 0.0) z[e] *= 1.0 / sqrt(ms);
}

__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  prm[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

inline int nblk(int64_t n, int b = 256) { return int((n + b - 1) / b); }

double* scratch(Plan* p, size_t elems) {
  if (elems > p->pc_cap) {
    cudaFree(p->d_pc);
    p->d_pc = nullptr;
    p->pc_cap = 0;
    if (cudaMalloc(&p->d_pc, elems * sizeof(double)) != cudaSuccess) return nullptr;
    p->pc_cap = elems;
  }
  return static_cast<double*>(p->d_pc);
}

void col_dots(Plan* p, const double* a, const double* b, int nrhs, double* part, double* out) {
  if (nrhs == 1) {
    pc_dot_partial_kernel<<<kDotBlocks, 256, 0, p->stream>>>(a, b, p->sym.n, 1, part);
  } else {
    const dim3 grid(kDotBlocks, (nrhs + 31) / 32);
    pc_dot_wide_kernel<<<grid, 256, 0, p->stream>>>(a, b, p->sym.n, nrhs, part);
  }
  pc_dot_final_kernel<<<nblk(nrhs, 64), 64, 0, p->stream>>>(part, kDotBlocks, nrhs, out);
}

// Square root of Q: Q = B^T B with B (n x n) stacking, for the initial field,
// V^-1/2 A0 (rows (c, 0)) and, for each step t -> t + 1, sqrt(c qs_c) (A x_(t+1)
// / V - x_t) (rows (c, t + 1)); for a spatial model (T = 1) B = V^-1/2 A.  A and
// A0 are the 9-point implicit-Euler and initial-field operators (A_geo[c 9 + p]
// = A[c, c + off_p], off_p = (p % 3 - 1, p / 3 - 1)), qs = V kappa^2, c =
// 1 / (dt sigma) (spdes/advection_diffusion2D.py:101-116 written as a sum of squares).
// out = B x (TRANS = 0) or B^T x (TRANS = 1), n x nrhs row-major.
template <int TRANS>
__global__ void qsqrt_kernel(int Mx, int Ny, int T, const double* __restrict__ Ag, const double* __restrict__ A0g,
                             const double* __restrict__ qs, double V, double cfac, const double* __restrict__ x,
                             double* __restrict__ out, int nrhs) {
  const int Ns = Mx * Ny, n = Ns * T;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int k = nrhs == 1 ? e : e / nrhs;
  const int r = e - k * nrhs;
  const int t = k / Ns, c = k - t * Ns;
  const int cy = c / Mx, cx = c - cy * Mx;
  const double rv = 1.0 / sqrt(V);
  double acc = 0.0;
  if (!TRANS) {
    // row (c, t)
    const double* Ar = (T > 1 && t == 0 ? A0g : Ag) + int64_t(c) * 9;
    double sum = 0.0;
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      const int x2 = cx + p % 3 - 1, y2 = cy + p / 3 - 1;
      if (x2 < 0 || x2 >= Mx || y2 < 0 || y2 >= Ny) continue;
      sum = fma(Ar[p], x[int64_t(t * Ns + y2 * Mx + x2) * nrhs + r], sum);
    }
    if (T == 1 || t == 0) acc = rv * sum;
    else acc = sqrt(cfac * qs[c]) * (sum / V - x[int64_t((t - 1) * Ns + c) * nrhs + r]);
  } else {
    // column (c, t): rows (c', t) with c = c' + off_p, and the -1 of row (c, t + 1)
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      const int x2 = cx - (p % 3 - 1), y2 = cy - (p / 3 - 1);
      if (x2 < 0 || x2 >= Mx || y2 < 0 || y2 >= Ny) continue;
      const int c2 = y2 * Mx + x2;
      const double xe = x[int64_t(t * Ns + c2) * nrhs + r];
      if (T == 1 || t == 0) acc = fma(rv * (T > 1 ? A0g : Ag)[int64_t(c2) * 9 + p], xe, acc);
      else acc = fma(sqrt(cfac * qs[c2]) * Ag[int64_t(c2) * 9 + p] / V, xe, acc);
    }
    if (T > 1 && t + 1 < T) acc -= sqrt(cfac * qs[c]) * x[int64_t((t + 1) * Ns + c) * nrhs + r];
  }
  out[e] = acc;
}

// ------------------------------------------------------------ FP32 PCG
// The iteration runs in FP32 (stencil product, vectors, preconditioner): FP64
// is a narrow pipe on this part, and an FP64 stencil product is bound by it.
// The solution is accumulated and the residual recomputed in FP64 whenever
// the recursive FP32 residual has fallen by kReplaceDrop (reliable updates),
// so the reported tolerance is always met by the true FP64 residual.
// Inside the solver every vector is stored column by column (column r of an
// FP32 vector at v + r n), and each kernel takes its column from blockIdx.y or
// blockIdx.z.

// FP32 copies of the stencil coefficients, slot-major (cf[s Ns + c]): slots
// 0-24 first diagonal block (T > 1), 25-49 interior diagonal block, 50-58 the
// block to t + 1, 59-67 the neighbours' blocks to t - 1 mirrored onto this
// cell, 68 c Qs.
constexpr int kCoef32 = 69;
__global__ void coef32_kernel(QStencil q, float* __restrict__ cf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= q.Ns) return;
  const int cy = c / q.Mx, cx = c - cy * q.Mx;
  const int64_t Ns = q.Ns;
  const bool st = q.T > 1 && !q.sep;
  for (int s = 0; s < 25; ++s) {
    cf[s * Ns + c] = st ? float(q.Q0[int64_t(c) * 25 + s]) : 0.f;
    cf[(25 + s) * Ns + c] = float(q.QA[int64_t(c) * 25 + s]);
  }
  for (int s = 0; s < 9; ++s) {
    const int dx = s % 3 - 1, dy = s / 3 - 1;
    const bool in = cx + dx >= 0 && cx + dx < q.Mx && cy + dy >= 0 && cy + dy < q.Ny;
    cf[(50 + s) * Ns + c] = st ? float(q.QO[int64_t(c) * 9 + s]) : 0.f;
    cf[(59 + s) * Ns + c] = (st && in) ? float(q.QO[int64_t(c + dy * q.Mx + dx) * 9 + (8 - s)]) : 0.f;
  }
  cf[68 * Ns + c] = st ? float(q.cQs[c]) : 0.f;
}

// obs32[k] = tau obs[k] in FP32 (the observation term of the diagonal)
__global__ void obs32_kernel(const double* __restrict__ obs, double tau, float* __restrict__ o32, int64_t n) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) o32[k] = float(tau * obs[k]);
}

// row-major FP64 (n x nrhs) -> column-major FP32, and x += xc back (xc = 0)
__global__ void to32cm_kernel(const double* __restrict__ v, float* __restrict__ o, int64_t n, int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t k = e / nrhs;
  o[(e - k * nrhs) * n + k] = float(v[e]);
}
__global__ void acc64cm_kernel(double* __restrict__ x, float* __restrict__ xc, int64_t n, int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int64_t k = e / nrhs;
  const int64_t f = (e - k * nrhs) * n + k;
  x[e] += double(xc[f]);
  xc[f] = 0.f;
}

// Fixed-order block sum of one float per thread into part[] (thread 0 writes)
__device__ __forceinline__ double block_sum(float v, float* red) {
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// ap = A p in FP32 for column blockIdx.y, one thread per node (the cell's
// coefficients, shared by all its time steps, come from L1 / L2), and the
// block's partial sum of p . ap into part[col gridDim.x + block].  Node and
// coefficient offsets fit in 32 bits (checked by the caller).
__global__ void __launch_bounds__(256, 4) spmv32n_kernel(int Mx, int Ny, int T, int sep, float qe, float qm,
                                                         float qo, const float* __restrict__ cf,
                                                         const float* __restrict__ o32, const float* __restrict__ pv,
                                                         float* __restrict__ apv, double* __restrict__ part) {
  __shared__ float red[8];
  const int Ns = Mx * Ny, n = Ns * T;
  const int col = blockIdx.y;
  const float* x = pv + int64_t(col) * n;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  float dot = 0.f;
  if (k < n) {
    const int t = k / Ns, c = k - t * Ns;
    const int cy = c / Mx, cx = c - cy * Mx;
    // bit (dx + 2) of vx: cx + dx inside the grid; likewise vy
    const uint32_t vx = (cx >= 2 ? 1u : 0u) | (cx >= 1 ? 2u : 0u) | 4u | (cx + 1 < Mx ? 8u : 0u) | (cx + 2 < Mx ? 16u : 0u);
    const uint32_t vy = (cy >= 2 ? 1u : 0u) | (cy >= 1 ? 2u : 0u) | 4u | (cy + 1 < Ny ? 8u : 0u) | (cy + 2 < Ny ? 16u : 0u);
    const float* cc = cf + c;
    const float* xt = x + k;
    const int sb = (t == 0 && T > 1 && !sep) ? 0 : 25;
    auto block25 = [&](const float* xs) {
      float acc = 0.f;
#pragma unroll
      for (int s = 0; s < 25; ++s) {
        const int dx = s % 5 - 2, dy = s / 5 - 2;
        if ((vx >> (dx + 2)) & (vy >> (dy + 2)) & 1u) acc = fmaf(cc[(sb + s) * Ns], xs[dy * Mx + dx], acc);
      }
      return acc;
    };
    float acc;
    if (sep) {
      // Q = Qt (x) Qs: Qt_tt (Qs x_t) + Qt_off (Qs x_(t-1) + Qs x_(t+1))
      acc = (t == 0 || t == T - 1 ? qe : qm) * block25(xt);
      if (t > 0) acc = fmaf(qo, block25(xt - Ns), acc);
      if (t + 1 < T) acc = fmaf(qo, block25(xt + Ns), acc);
    } else {
      acc = block25(xt);
      if (T > 1) {
        if (t < T - 1) acc = fmaf(cc[68 * Ns], xt[0], acc);
        if (t + 1 < T) {
#pragma unroll
          for (int s = 0; s < 9; ++s) {
            const int dx = s % 3 - 1, dy = s / 3 - 1;
            if ((vx >> (dx + 2)) & (vy >> (dy + 2)) & 1u) acc = fmaf(cc[(50 + s) * Ns], xt[Ns + dy * Mx + dx], acc);
          }
        }
        if (t > 0) {
#pragma unroll
          for (int s = 0; s < 9; ++s) {
            const int dx = s % 3 - 1, dy = s / 3 - 1;
            if ((vx >> (dx + 2)) & (vy >> (dy + 2)) & 1u) acc = fmaf(cc[(59 + s) * Ns], xt[-Ns + dy * Mx + dx], acc);
          }
        }
      }
    }
    if (o32) acc = fmaf(o32[k], xt[0], acc);
    apv[int64_t(col) * n + k] = acc;
    dot = xt[0] * acc;
  }
  const double bs = block_sum(dot, red);
  if (threadIdx.x == 0) part[int64_t(col) * gridDim.x + blockIdx.x] = bs;
}

// Diagonal of A at node (cell c, time t) from the FP32 coefficients
__device__ __forceinline__ float diag32(const float* __restrict__ cf, int Ns, int T, int sep, float qe, float qm,
                                        int c, int t) {
  if (sep) return (t == 0 || t == T - 1 ? qe : qm) * cf[int64_t(25 + 12) * Ns + c];
  if (T == 1) return cf[int64_t(25 + 12) * Ns + c];
  if (t == 0) return cf[int64_t(12) * Ns + c] + cf[int64_t(68) * Ns + c];
  return cf[int64_t(25 + 12) * Ns + c] + (t < T - 1 ? cf[int64_t(68) * Ns + c] : 0.f);
}

// Elementwise step of column blockIdx.y (grid-stride over the nodes):
//   xc += alpha p, r -= alpha Ap   (alpha 0: no update)
//   mode 0: z = r;  mode 1: z = r / A_pp;  mode 2: z left to the G^T G kernel
// and the block's partial sums of r . z (mode < 2) into partA[col G + b] and of
// r . r into partB[col G + b].
constexpr int kElemBlocks = 1216;  // 8 per SM
__global__ void __launch_bounds__(256) update32c_kernel(int Ns, int T, int sep, float qe, float qm, int mode,
                                                        const float* __restrict__ cf, const float* __restrict__ o32,
                                                        float* __restrict__ xc, float* __restrict__ rv,
                                                        const float* __restrict__ pv, const float* __restrict__ apv,
                                                        float* __restrict__ zv, const float* __restrict__ alpha,
                                                        double* __restrict__ partA, double* __restrict__ partB) {
  __shared__ float red[8];
  const int64_t n = int64_t(Ns) * T;
  const int col = blockIdx.y;
  const float a = alpha[col];
  float* r = rv + col * n;
  float srz = 0.f, srr = 0.f;
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x) {
    float rk = r[k];
    if (a != 0.f) {
      xc[col * n + k] = fmaf(a, pv[col * n + k], xc[col * n + k]);
      rk = fmaf(-a, apv[col * n + k], rk);
      r[k] = rk;
    }
    srr = fmaf(rk, rk, srr);
    if (mode < 2) {
      float zk = rk;
      if (mode == 1) {
        const int t = int(k) / Ns, c = int(k) - t * Ns;  // node indices fit in 32 bits
        zk = __fdividef(rk, diag32(cf, Ns, T, sep, qe, qm, c, t) + (o32 ? o32[k] : 0.f));
      }
      zv[col * n + k] = zk;
      srz = fmaf(rk, zk, srz);
    }
  }
  const double b1 = block_sum(srz, red);
  if (threadIdx.x == 0 && mode < 2) partA[int64_t(col) * gridDim.x + blockIdx.x] = b1;
  const double b2 = block_sum(srr, red);
  if (threadIdx.x == 0) partB[int64_t(col) * gridDim.x + blockIdx.x] = b2;
}

// Weights of G: compact (rows per cell and time class, observed rows through
// the bitmask and per-word ranks) or per node
struct GWeights {
  const float* w;
  const uint32_t* mask;  // compact, with observations: observed nodes have their own rows
  const int* rank;
  const uint32_t* near;  // with mask: bit p set when one of the 27 nodes p - d is observed
  int nob, Ns, T, compact;
};

// Bits of the nodes whose G^T row gathers from an observed node: p = q + d for
// every observed q and offset d inside the grid.
__global__ void near_obs_kernel(const int* __restrict__ nodes, int nob, int Mx, int Ny, int T,
                                uint32_t* __restrict__ near) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nob) return;
  const int Ns = Mx * Ny, q = nodes[j];
  const int t = q / Ns, c = q - t * Ns, y = c / Mx, x = c - y * Mx;
  for (int o = 0; o < kOff; ++o) {
    const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dt = o / 9 - 1;
    const int xp = x + dx, yp = y + dy, tp = t + dt;
    if (xp < 0 || xp >= Mx || yp < 0 || yp >= Ny || tp < 0 || tp >= T) continue;
    const int p = (tp * Ny + yp) * Mx + xp;
    atomicOr(&near[p >> 5], 1u << (p & 31));
  }
}

// u = G r (TRANS 0) or z = G^T u with the block's partial sum of r . z
// (TRANS 1) for column blockIdx.y, one thread per node; the rows of G come
// from the compact (COMPACT 1) or per-node weights through L1 / L2.  Offsets
// fit in 32 bits (checked by the caller).
template <int TRANS, int COMPACT>
__global__ void __launch_bounds__(256, 4) g32n_kernel(int Mx, int Ny, int T, GWeights gw,
                                                      const float* __restrict__ xv, float* __restrict__ outv,
                                                      const float* __restrict__ rv, double* __restrict__ part) {
  __shared__ float red[8];
  const int Ns = Mx * Ny, n = Ns * T;
  const int col = blockIdx.y;
  const float* x = xv + int64_t(col) * n;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  float dot = 0.f;
  if (p < n) {
    const int t = p / Ns, c = p - t * Ns;
    const int y = c / Mx, xx = c - y * Mx;
    // bit (d + 1) set: the neighbour at +-d (sign of the direction used) is inside
    const int sg = TRANS ? -1 : 1;
    auto bits = [](int v, int lim, int sgn) {
      return (v - sgn >= 0 && v - sgn < lim ? 1u : 0u) | 2u | (v + sgn >= 0 && v + sgn < lim ? 4u : 0u);
    };
    const uint32_t bx = bits(xx, Mx, sg), by = bits(y, Ny, sg), bt = bits(t, T, sg);
    const float* w = gw.w;
    // the weight row of node q (time tq, cell cq) for offset o
    auto wrow = [&](int q, int tq, int cq, int o) -> float {
      if (!COMPACT) return w[o * n + q];
      if (gw.mask) {
        const uint32_t m = gw.mask[q >> 5], bit = 1u << (q & 31);
        if (m & bit) return w[3 * kOff * Ns + o * gw.nob + gw.rank[q >> 5] + __popc(m & (bit - 1u))];
      }
      const int kc = tq == 0 ? 0 : (tq == T - 1 ? 2 : 1);
      return w[(kc * kOff + o) * Ns + cq];
    };
    float acc = 0.f;
    // interior node (all 27 neighbours exist and, for G^T, lie in the interior
    // time class): no validity tests, rows found without per-offset lookups
    const bool inner = xx >= 1 && xx + 1 < Mx && y >= 1 && y + 1 < Ny && t >= 1 + TRANS && t + 1 + TRANS < T &&
                       (!TRANS || !COMPACT || !gw.mask || !((gw.near[p >> 5] >> (p & 31)) & 1u));
    if (inner && !TRANS) {
      const float* wr;
      int stride;
      if (!COMPACT) {
        wr = w + p;
        stride = n;
      } else {
        wr = w + kOff * Ns + c;
        stride = Ns;
        if (gw.mask) {
          const uint32_t m = gw.mask[p >> 5], bit = 1u << (p & 31);
          if (m & bit) {
            wr = w + 3 * kOff * Ns + gw.rank[p >> 5] + __popc(m & (bit - 1u));
            stride = gw.nob;
          }
        }
      }
#pragma unroll
      for (int o = 0; o < kOff; ++o) {
        const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dt = o / 9 - 1;
        acc = fmaf(wr[o * stride], x[p + dt * Ns + dy * Mx + dx], acc);
      }
    } else if (inner) {
#pragma unroll
      for (int o = 0; o < kOff; ++o) {
        const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dt = o / 9 - 1;
        const int d = dt * Ns + dy * Mx + dx;
        const float wv = COMPACT ? w[(kOff + o) * Ns + c - dy * Mx - dx] : w[o * n + p - d];
        acc = fmaf(wv, x[p - d], acc);
      }
    } else {
#pragma unroll
      for (int o = 0; o < kOff; ++o) {
        const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dt = o / 9 - 1;
        if (!((bx >> (dx + 1)) & (by >> (dy + 1)) & (bt >> (dt + 1)) & 1u)) continue;
        const int d = dt * Ns + dy * Mx + dx;
        const int q = TRANS ? p - d : p + d;
        const float wv = TRANS ? wrow(q, t - dt, c - dy * Mx - dx, o) : wrow(p, t, c, o);
        acc = fmaf(wv, x[q], acc);
      }
    }
    outv[int64_t(col) * n + p] = acc;
    if (TRANS) dot = rv[int64_t(col) * n + p] * acc;
  }
  if (TRANS) {
    const double bs = block_sum(dot, red);
    if (threadIdx.x == 0) part[int64_t(col) * gridDim.x + blockIdx.x] = bs;
  }
}

// ------------------------------------------------------------ IC(0)
// Incomplete Cholesky with the pattern of A's lower triangle in the natural
// node order (the baseline preconditioner of the PCG comparison).  The 21 lower
// neighbours of a node, ordered by increasing node index: dt = -1 (3 x 3),
// then dt = 0 with dy = -2, dy = -1 (dx -2..2 each) and dy = 0 (dx -2, -1).
// Every lower neighbour of node (x, y, t) lies on an earlier level of
// x + 3 y + 5 t, so the factorisation and the forward solve run level by
// level (one launch per level, the backward solve in reverse).  L is FP32, 22
// values per node: the 21 lower entries, then the diagonal.
constexpr int kIcLow = 21, kIcRow = 22;
struct IcTables {
  int dx[kIcLow], dy[kIcLow], dt[kIcLow];
  // for lower entry a: the common lower neighbours k of node i and of j = i + o_a
  // with k < j, as (index b of k in i's row, index c of k in j's row)
  int cstart[kIcLow + 1];
  int cb[512], cc[512];
};
__constant__ IcTables c_ic;

void ic_tables(IcTables* tb) {
  int m = 0;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) { tb->dx[m] = dx; tb->dy[m] = dy; tb->dt[m] = -1; ++m; }
  for (int dy = -2; dy <= -1; ++dy)
    for (int dx = -2; dx <= 2; ++dx) { tb->dx[m] = dx; tb->dy[m] = dy; tb->dt[m] = 0; ++m; }
  for (int dx = -2; dx <= -1; ++dx) { tb->dx[m] = dx; tb->dy[m] = 0; tb->dt[m] = 0; ++m; }
  auto find = [&](int dx, int dy, int dt) {
    for (int i = 0; i < kIcLow; ++i)
      if (tb->dx[i] == dx && tb->dy[i] == dy && tb->dt[i] == dt) return i;
    return -1;
  };
  int e = 0;
  for (int a = 0; a < kIcLow; ++a) {
    tb->cstart[a] = e;
    for (int b = 0; b < kIcLow; ++b) {
      // k = i + o_b must precede j = i + o_a and be a lower neighbour of j: o_b - o_a lower
      const int c = find(tb->dx[b] - tb->dx[a], tb->dy[b] - tb->dy[a], tb->dt[b] - tb->dt[a]);
      if (c >= 0) { tb->cb[e] = b; tb->cc[e] = c; ++e; }
    }
  }
  tb->cstart[kIcLow] = e;
}

// A(i, i + o) in FP32 from the coefficient copies (spatio-temporal layout)
__device__ __forceinline__ float aval32(const float* __restrict__ cf, const float* __restrict__ o32, int Ns, int T,
                                        int k, int c, int t, int dx, int dy, int dt) {
  if (dt == -1) return cf[(59 + (dy + 1) * 3 + dx + 1) * Ns + c];
  if (dt == 1) return cf[(50 + (dy + 1) * 3 + dx + 1) * Ns + c];
  const int sb = (t == 0 && T > 1) ? 0 : 25;
  float v = cf[(sb + (dy + 2) * 5 + dx + 2) * Ns + c];
  if (dx == 0 && dy == 0) {
    if (T > 1 && t < T - 1) v += cf[68 * Ns + c];
    if (o32) v += o32[k];
  }
  return v;
}

// Node on level lev handled by thread e = (t, y): x = lev - 3 y - 5 t
__device__ __forceinline__ int ic_node(int lev, int e, int Mx, int Ny, int T, int* x, int* y, int* t) {
  if (e >= Ny * T) return -1;
  *t = e / Ny;
  *y = e - *t * Ny;
  *x = lev - 3 * *y - 5 * *t;
  if (*x < 0 || *x >= Mx) return -1;
  return (*t * Ny + *y) * Mx + *x;
}

// One level of the factorisation of A + shift diag(A); *bad counts pivots <= 0
__global__ void ic0_factor_kernel(int lev, int Mx, int Ny, int T, const float* __restrict__ cf,
                                  const float* __restrict__ o32, float shift, float* __restrict__ L,
                                  int* __restrict__ bad) {
  int x, y, t;
  const int i = ic_node(lev, blockIdx.x * blockDim.x + threadIdx.x, Mx, Ny, T, &x, &y, &t);
  if (i < 0) return;
  const int Ns = Mx * Ny, c = i - t * Ns;
  float* Li = L + int64_t(i) * kIcRow;
  bool in[kIcLow];
  float dsum = 0.f;
  for (int a = 0; a < kIcLow; ++a) {
    const int dx = c_ic.dx[a], dy = c_ic.dy[a], dt = c_ic.dt[a];
    in[a] = x + dx >= 0 && x + dx < Mx && y + dy >= 0 && y + dy < Ny && t + dt >= 0;
    if (!in[a]) { Li[a] = 0.f; continue; }
    const int j = i + dt * Ns + dy * Mx + dx;
    const float* Lj = L + int64_t(j) * kIcRow;
    float v = aval32(cf, o32, Ns, T, i, c, t, dx, dy, dt);
    for (int e = c_ic.cstart[a]; e < c_ic.cstart[a + 1]; ++e) {
      const int b = c_ic.cb[e];
      if (in[b]) v = fmaf(-Li[b], Lj[c_ic.cc[e]], v);  // b < a: Li[b] is final
    }
    const float lij = v / Lj[kIcLow];
    Li[a] = lij;
    dsum = fmaf(lij, lij, dsum);
  }
  float d = aval32(cf, o32, Ns, T, i, c, t, 0, 0, 0);
  d = d * (1.f + shift) - dsum;
  if (!(d > 0.f)) {
    atomicAdd(bad, 1);
    d = 1.f;
  }
  Li[kIcLow] = sqrtf(d);
}

// One level of L y = r (FWD) or L^T z = y (backward), column blockIdx.y
template <int FWD>
__global__ void ic0_solve_kernel(int lev, int Mx, int Ny, int T, const float* __restrict__ L,
                                 const float* __restrict__ in, float* __restrict__ out) {
  int x, y, t;
  const int i = ic_node(lev, blockIdx.x * blockDim.x + threadIdx.x, Mx, Ny, T, &x, &y, &t);
  if (i < 0) return;
  const int Ns = Mx * Ny, n = Ns * T;
  const int64_t off = int64_t(blockIdx.y) * n;
  float v = in[off + i];
#pragma unroll
  for (int a = 0; a < kIcLow; ++a) {
    const int dx = c_ic.dx[a], dy = c_ic.dy[a], dt = c_ic.dt[a];
    if (FWD) {
      if (x + dx < 0 || x + dx >= Mx || y + dy < 0 || y + dy >= Ny || t + dt < 0) continue;
      const int j = i + dt * Ns + dy * Mx + dx;
      v = fmaf(-L[int64_t(i) * kIcRow + a], out[off + j], v);
    } else {
      // upper neighbour j = i - o_a, whose row holds L(j, i) at index a
      if (x - dx < 0 || x - dx >= Mx || y - dy < 0 || y - dy >= Ny || t - dt >= T) continue;
      const int j = i - (dt * Ns + dy * Mx + dx);
      v = fmaf(-L[int64_t(j) * kIcRow + a], out[off + j], v);
    }
  }
  out[off + i] = v / L[int64_t(i) * kIcRow + kIcLow];
}

// partial sums of a . b per block and column (column blockIdx.y)
__global__ void __launch_bounds__(256) dot32c_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                     int n, double* __restrict__ part) {
  __shared__ float red[8];
  const int64_t off = int64_t(blockIdx.y) * n;
  float s = 0.f;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    s = fmaf(a[off + k], b[off + k], s);
  const double bs = block_sum(s, red);
  if (threadIdx.x == 0) part[int64_t(blockIdx.y) * gridDim.x + blockIdx.x] = bs;
}

// Per-column scalars from block partials (one block per column, fixed order):
//   mode 0: pap = sum partA;  alpha = rz / pap (0 if done or pap <= 0)
//   mode 1: rzn = sum partA, rr = sum partB;  beta = rzn / rz, rz = rzn
//   mode 2: rz = sum partA, rr = sum partB, beta = 0 (a new or replaced residual)
__global__ void scal32_kernel(const double* __restrict__ partA, int na, const double* __restrict__ partB, int nb,
                              int mode, const int* __restrict__ done, double* __restrict__ rz,
                              double* __restrict__ rr, double* __restrict__ pap, float* __restrict__ alpha,
                              float* __restrict__ beta) {
  __shared__ double sh[2][256];
  const int col = blockIdx.x;
  double s1 = 0.0, s2 = 0.0;
  for (int i = threadIdx.x; i < na; i += 256) s1 += partA[int64_t(col) * na + i];
  if (mode != 0)
    for (int i = threadIdx.x; i < nb; i += 256) s2 += partB[int64_t(col) * nb + i];
  sh[0][threadIdx.x] = s1;
  sh[1][threadIdx.x] = s2;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + k];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double a = sh[0][0], b = sh[1][0];
  if (mode == 0) {
    pap[col] = a;
    alpha[col] = (!done[col] && a > 0.0) ? float(rz[col] / a) : 0.f;
  } else if (mode == 1) {
    beta[col] = (!done[col] && rz[col] != 0.0) ? float(a / rz[col]) : 0.f;
    rz[col] = a;
    rr[col] = b;
  } else {
    rz[col] = a;
    rr[col] = b;
    beta[col] = 0.f;
  }
}

//   p = z + beta p (finished columns unchanged)
__global__ void p32c_kernel(float* __restrict__ pv, const float* __restrict__ zv, const float* __restrict__ beta,
                            const int* __restrict__ done, int64_t n) {
  const int col = blockIdx.y;
  if (done[col]) return;
  const float b = beta[col];
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x)
    pv[col * n + k] = fmaf(b, pv[col * n + k], zv[col * n + k]);
}

}  // namespace

int qsqrt_apply(Plan* p, int transpose, const double* x, double* y, int nrhs) {
  const int64_t len = int64_t(p->sym.n) * nrhs;
  if (len >= (int64_t(1) << 31)) return 1;
  const int Mx = p->sym.Mx, Ny = p->sym.Ny, T = p->sym.T;
  if (transpose)
    qsqrt_kernel<1><<<nblk(len), 256, 0, p->stream>>>(Mx, Ny, T, p->d_Ageo, p->d_A0geo, p->d_qs, p->model.V, p->cfac,
                                                      x, y, nrhs);
  else
    qsqrt_kernel<0><<<nblk(len), 256, 0, p->stream>>>(Mx, Ny, T, p->d_Ageo, p->d_A0geo, p->d_qs, p->model.V, p->cfac,
                                                      x, y, nrhs);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pc_weights(Plan* p, int with_obs, double tau, const float* prm, float* w, float* act) {
  const int64_t n = p->sym.n;
  pc_forward_kernel<<<nblk(n, 128), 128, 0, p->stream>>>(p->qstencil(), with_obs ? p->d_obs_cnt : nullptr, tau, prm,
                                                          w, act);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pc_grad(Plan* p, int with_obs, double tau, const float* prm, const float* w, const float* act, const double* z,
            int k, double* loss, float* grad) {
  const int64_t n = p->sym.n, len = n * k;
  if (len >= (int64_t(1) << 31)) return 1;  // the stencil kernels index entries in 32 bits
  const int nbw = int((n + kBwNodes - 1) / kBwNodes);
  // y, u, e, g1, g2 (n x k doubles each) + partial sums + per-node dout and block partials (as floats)
  const size_t dbl = size_t(5 * len) + size_t(kDotBlocks) * k + 8;
  const size_t flt = size_t(n) * kOff + size_t(nbw) * kNP;
  double* base = scratch(p, dbl + (flt + 1) / 2);
  if (!base) return 4;
  double *y = base, *u = y + len, *e = u + len, *g1 = e + len, *g2 = g1 + len, *part = g2 + len;
  double* sums = part + size_t(kDotBlocks) * k;
  float* dout = reinterpret_cast<float*>(sums + 8);
  float* bpart = dout + size_t(n) * kOff;
  const QStencil q = p->qstencil();
  const double* obs = with_obs ? p->d_obs_cnt : nullptr;
  cudaStream_t st = p->stream;
  pc_apply_kernel<1, double, double><<<nblk(len), 256, 0, st>>>(q, w, z, y, k);           // y = G^T z
  launch_spmv(q, obs, tau, y, u, k, st);                                   // u = A y
  pc_apply_kernel<0, double, double><<<nblk(len), 256, 0, st>>>(q, w, u, e, k);           // v = G u
  pc_sub_kernel<<<nblk(len), 256, 0, st>>>(z, e, len);                     // e = z - v
  pc_apply_kernel<1, double, double><<<nblk(len), 256, 0, st>>>(q, w, e, g1, k);          // G^T e
  launch_spmv(q, obs, tau, g1, g2, k, st);                                 // g = A G^T e
  // loss = ||e||^2 / (n k): one column of length n k
  pc_dot_partial_kernel<<<kDotBlocks, 256, 0, st>>>(e, e, len, 1, part);
  pc_dot_final_kernel<<<1, 64, 0, st>>>(part, kDotBlocks, 1, sums);
  const double scale = -2.0 / double(len);
  pc_wgrad_kernel<<<nblk(n, 128), 128, 0, st>>>(q, z, e, u, g2, k, scale, act, dout);
  const size_t smem = sizeof(float) * (kHid * kHid + kOff * kHid + kBwNodes * (kFeat + 4 * kHid + kOff));
  static const bool attr = [smem] {  // once, thread-safely
    cudaFuncSetAttribute(pc_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    return true;
  }();
  (void)attr;
  pc_backward_kernel<<<nbw, 128, smem, st>>>(n, prm, act, dout, bpart);
  pc_colsum_kernel<<<nblk(kNP, 128), 128, 0, st>>>(bpart, nbw, grad);
  double h = 0.0;
  cudaMemcpyAsync(&h, sums, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
  *loss = h / double(len);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int pc_adam(const float* g, float* prm, float* m, float* v, int n, float lr, float b1, float b2, float eps, int t,
            cudaStream_t st) {
  const float c1 = 1.f - powf(b1, float(t)), c2 = 1.f - powf(b2, float(t));
  adam_kernel<<<nblk(n), 256, 0, st>>>(prm, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int jacobi_smooth(Plan* p, int with_obs, double tau, double omega, int sweeps, double* z, int nrhs) {
  const int64_t n = p->sym.n, len = n * nrhs;
  double* base = scratch(p, size_t(len) + size_t(kDotBlocks) * nrhs + size_t(nrhs));
  if (!base) return 4;
  double *az = base, *part = az + len, *ss = part + size_t(kDotBlocks) * nrhs;
  const QStencil q = p->qstencil();
  const double* obs = with_obs ? p->d_obs_cnt : nullptr;
  for (int it = 0; it < sweeps; ++it) {
    launch_spmv(q, obs, tau, z, az, nrhs, p->stream);
    jacobi_sweep_kernel<<<nblk(len), 256, 0, p->stream>>>(q, obs, tau, omega, az, z, nrhs);
  }
  col_dots(p, z, z, nrhs, part, ss);
  col_scale_kernel<<<nblk(len), 256, 0, p->stream>>>(z, ss, n, nrhs);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

float* scratch32(Plan* p, size_t elems) {
  if (elems > p->pc32_cap) {
    cudaFree(p->d_pc32);
    p->d_pc32 = nullptr;
    p->pc32_cap = 0;
    if (cudaMalloc(&p->d_pc32, elems * sizeof(float)) != cudaSuccess) return nullptr;
    p->pc32_cap = elems;
  }
  return static_cast<float*>(p->d_pc32);
}

// Compact weights start with a 4-int header (magic, observed rows included,
// observation-set version, number of observed rows) so that a solve can check
// that they belong to its observation set; the rows follow.
constexpr int kCompactHeader = 4;
constexpr int kCompactMagic = 0x53504345;

int64_t pc_compact_floats(const Plan* p) {
  return kCompactHeader + int64_t(kOff) * (3 * int64_t(p->sym.Mx) * p->sym.Ny + p->nob);
}

int pc_weights_compact(Plan* p, int with_obs, double tau, const float* prm, float* w) {
  const int Ns = p->sym.Mx * p->sym.Ny;
  const int nob = with_obs ? p->nob : 0;
  const int64_t rows = 3 * int64_t(Ns) + nob;
  static thread_local int head[kCompactHeader];
  head[0] = kCompactMagic;
  head[1] = with_obs ? 1 : 0;
  head[2] = p->obs_version;
  head[3] = nob;
  cudaMemcpyAsync(w, head, sizeof(head), cudaMemcpyHostToDevice, p->stream);
  pc_forward_compact_kernel<<<nblk(rows, 128), 128, 0, p->stream>>>(p->qstencil(), with_obs ? p->d_obs_cnt : nullptr,
                                                                    tau, p->d_obs_nodes, nob, prm,
                                                                    w + kCompactHeader);
  // the header copy reads host memory asynchronously: finish before it can change
  return cudaStreamSynchronize(p->stream) == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Reliable-update PCG: the recursive FP32 residual is replaced by the true
// FP64 one (and the FP32 correction added into the FP64 solution) whenever it
// has fallen by this factor since the last replacement, reaches the tolerance,
// or kReplaceEvery iterations have passed.
constexpr double kReplaceDrop = 0.1;
constexpr int kReplaceEvery = 64;

int pcg_solve(Plan* p, int with_obs, double tau, int kind, const float* w, const double* b, double* x, int nrhs,
              double tol, int maxit, int check_every, int* iters, double* relres) {
  const int64_t n = p->sym.n, len = n * nrhs;
  // the stencil kernels index nodes, weights (27 n) and coefficients (69 Ns) in 32 bits
  if (len >= (int64_t(1) << 31) || int64_t(p->sym.n) * kOff >= (int64_t(1) << 31) || nrhs > 65535) return 1;
  const int Mx = p->sym.Mx, Ny = p->sym.Ny, Ns = Mx * Ny, T = p->sym.T;
  cudaStream_t st = p->stream;
  const int nsp = nblk(n, 256);  // blocks of the per-node kernels (stencil product, G, G^T)
  const int na_max = std::max(nsp, int(kElemBlocks));
  // FP64: true residual (row-major), block partials, per-column scalars
  const size_t need64 = size_t(len) + size_t(nrhs) * (na_max + kElemBlocks) + size_t(kDotBlocks) * nrhs +
                        size_t(8 * nrhs) + size_t(nrhs);
  double* base = scratch(p, need64);
  // FP32 (column-major): r, z, p, Ap, x correction, G r; coefficients; observation term; alpha, beta
  const bool near_bits = kind == 3 && with_obs;  // G^T needs the nodes next to observed ones
  const size_t nwords = size_t((n + 31) / 32);
  const size_t need32 = size_t(6 * len) + size_t(kCoef32) * Ns + size_t(n) + size_t(2 * nrhs) +
                        (kind == 4 ? size_t(kIcRow) * n : 0) + (near_bits ? nwords : 0);
  float* b32 = scratch32(p, need32);
  if (!base || !b32) return 4;
  double* r64 = base;
  double* partA = r64 + len;
  double* partB = partA + size_t(nrhs) * na_max;
  double* part64 = partB + size_t(nrhs) * kElemBlocks;
  double* sc = part64 + size_t(kDotBlocks) * nrhs;
  double *rz = sc, *pap = sc + nrhs, *rr = sc + 2 * nrhs, *bb = sc + 3 * nrhs, *rrt = sc + 4 * nrhs;
  int* done = reinterpret_cast<int*>(sc + 8 * nrhs);
  float *r32 = b32, *z32 = r32 + len, *p32 = z32 + len, *ap32 = p32 + len, *xc32 = ap32 + len, *u32 = xc32 + len;
  float* cf = u32 + len;
  float* o32 = cf + size_t(kCoef32) * Ns;
  float* alpha = o32 + n;
  float* beta = alpha + nrhs;
  float* Lic = beta + nrhs;  // IC(0) factor (kind 4)
  uint32_t* near = reinterpret_cast<uint32_t*>(Lic + (kind == 4 ? size_t(kIcRow) * n : 0));
  const QStencil q = p->qstencil();
  const double* obs = with_obs ? p->d_obs_cnt : nullptr;
  const int sep = q.sep;
  const float qe = float(q.qt_end), qm = float(q.qt_mid), qo = float(q.qt_off);
  const int mode = kind == 0 ? 0 : (kind == 1 ? 1 : 2);  // 2: z from a separate preconditioner pass
  // IC(0) of the spatio-temporal stencil; its lower-neighbour order needs Mx >= 5, Ny >= 4
  if (kind == 4 && (q.sep || T < 2 || Mx < 5 || Ny < 4)) return 8;
  if (kind == 3) {
    // compact weights hold observed rows for the observation set they were computed with
    int head[kCompactHeader] = {0, 0, 0, 0};
    if (cudaMemcpyAsync(head, w, sizeof(head), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return 2;
    const bool ok = head[0] == kCompactMagic && head[1] == (with_obs ? 1 : 0) &&
                    (!with_obs || (head[2] == p->obs_version && head[3] == p->nob));
    if (!ok) return 7;
    w += kCompactHeader;
  }
  GWeights gw{w, near_bits ? p->d_obs_mask : nullptr, p->d_obs_rank, near_bits ? near : nullptr, p->nob, Ns, T,
              kind == 3 ? 1 : 0};
  if (near_bits) {
    cudaMemsetAsync(near, 0, nwords * sizeof(uint32_t), st);
    if (p->nob > 0) near_obs_kernel<<<nblk(p->nob), 256, 0, st>>>(p->d_obs_nodes, p->nob, Mx, Ny, T, near);
  }
  coef32_kernel<<<nblk(Ns, 128), 128, 0, st>>>(q, cf);
  if (obs) obs32_kernel<<<nblk(n), 256, 0, st>>>(obs, tau, o32, n);
  const float* o = obs ? o32 : nullptr;
  const dim3 gsp(nsp, nrhs), gel(kElemBlocks, nrhs);
  const int nlev = (Mx - 1) + 3 * (Ny - 1) + 5 * (T - 1) + 1;
  const dim3 glev(nblk(int64_t(Ny) * T, 128), nrhs);
  if (kind == 4) {
    // IC(0) of A + shift diag(A), the shift raised until no pivot breaks down
    static IcTables tables;
    static const bool tables_ready = (ic_tables(&tables), true);
    (void)tables_ready;
    if (cudaMemcpyToSymbolAsync(c_ic, &tables, sizeof(IcTables), 0, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return 2;
    int* bad = reinterpret_cast<int*>(alpha);  // alpha is set before its first use
    const float shifts[] = {0.f, 1e-3f, 1e-2f, 1e-1f, 1.f};
    bool ok = false;
    for (float sh : shifts) {
      cudaMemsetAsync(bad, 0, sizeof(int), st);
      for (int lev = 0; lev < nlev; ++lev)
        ic0_factor_kernel<<<nblk(int64_t(Ny) * T, 128), 128, 0, st>>>(lev, Mx, Ny, T, cf, o, sh, Lic, bad);
      int hb = 0;
      if (cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return 2;
      if (hb == 0) { ok = true; break; }
    }
    if (!ok) return 9;
  }
  // z = M r with the partial sums of r . z and r . r, after the update of r by alpha
  auto update_precond = [&]() {
    update32c_kernel<<<gel, 256, 0, st>>>(Ns, T, sep, qe, qm, mode, cf, o, xc32, r32, p32, ap32, z32, alpha, partA,
                                          partB);
    if (mode == 2 && kind == 3) {
      g32n_kernel<0, 1><<<gsp, 256, 0, st>>>(Mx, Ny, T, gw, r32, u32, nullptr, nullptr);
      g32n_kernel<1, 1><<<gsp, 256, 0, st>>>(Mx, Ny, T, gw, u32, z32, r32, partA);
    } else if (kind == 4) {
      for (int lev = 0; lev < nlev; ++lev)
        ic0_solve_kernel<1><<<glev, 128, 0, st>>>(lev, Mx, Ny, T, Lic, r32, u32);
      for (int lev = nlev - 1; lev >= 0; --lev)
        ic0_solve_kernel<0><<<glev, 128, 0, st>>>(lev, Mx, Ny, T, Lic, u32, z32);
      dot32c_kernel<<<gsp, 256, 0, st>>>(r32, z32, int(n), partA);
    } else if (mode == 2) {
      g32n_kernel<0, 0><<<gsp, 256, 0, st>>>(Mx, Ny, T, gw, r32, u32, nullptr, nullptr);
      g32n_kernel<1, 0><<<gsp, 256, 0, st>>>(Mx, Ny, T, gw, u32, z32, r32, partA);
    }
  };
  const int na = mode == 2 ? nsp : int(kElemBlocks);
  // a new residual r32: z = M r, rz = r . z (p unchanged)
  auto restart = [&]() {
    cudaMemsetAsync(alpha, 0, size_t(nrhs) * sizeof(float), st);
    update_precond();
    scal32_kernel<<<nrhs, 256, 0, st>>>(partA, na, partB, kElemBlocks, 2, done, rz, rr, pap, alpha, beta);
  };
  auto true_residual = [&]() {
    launch_spmv(q, obs, tau, x, r64, nrhs, st);
    pc_sub_kernel<<<nblk(len), 256, 0, st>>>(b, r64, len);
    col_dots(p, r64, r64, nrhs, part64, rrt);
  };
  cudaMemsetAsync(x, 0, size_t(len) * sizeof(double), st);
  cudaMemsetAsync(xc32, 0, size_t(len) * sizeof(float), st);
  cudaMemsetAsync(p32, 0, size_t(len) * sizeof(float), st);
  col_dots(p, b, b, nrhs, part64, bb);
  std::vector<double> hb(nrhs), hr(nrhs), href(nrhs);
  std::vector<int> hd(nrhs, 0);
  cudaMemcpyAsync(hb.data(), bb, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
  for (int c = 0; c < nrhs; ++c)
    if (!(hb[c] > 0.0)) hd[c] = 1;  // a zero right-hand side is solved by x = 0
  cudaMemcpyAsync(done, hd.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, st);
  href = hb;
  to32cm_kernel<<<nblk(len), 256, 0, st>>>(b, r32, n, nrhs);
  restart();
  p32c_kernel<<<gel, 256, 0, st>>>(p32, z32, beta, done, n);  // p = z
  const double tol2 = tol * tol;
  const int every = std::max(1, std::min(check_every, 4));
  int it = 0, last_rep = 0;
  bool all_done = false, fresh = false;  // fresh: x holds every correction and rrt is its true residual
  for (int c = 0; c < nrhs; ++c) all_done = (c == 0 || all_done) && hd[c];
  while (it < maxit && !all_done) {
    spmv32n_kernel<<<gsp, 256, 0, st>>>(Mx, Ny, T, sep, qe, qm, qo, cf, o, p32, ap32, partA);
    scal32_kernel<<<nrhs, 256, 0, st>>>(partA, nsp, partB, 0, 0, done, rz, rr, pap, alpha, beta);
    update_precond();
    scal32_kernel<<<nrhs, 256, 0, st>>>(partA, na, partB, kElemBlocks, 1, done, rz, rr, pap, alpha, beta);
    p32c_kernel<<<gel, 256, 0, st>>>(p32, z32, beta, done, n);
    ++it;
    fresh = false;
    if (it % every != 0 && it != maxit) continue;
    cudaMemcpyAsync(hr.data(), rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
    bool replace = it == maxit || it - last_rep >= kReplaceEvery;
    for (int c = 0; c < nrhs && !replace; ++c)
      if (!hd[c] && (hr[c] <= kReplaceDrop * kReplaceDrop * href[c] || hr[c] <= tol2 * hb[c])) replace = true;
    if (!replace) continue;
    acc64cm_kernel<<<nblk(len), 256, 0, st>>>(x, xc32, n, nrhs);
    true_residual();
    cudaMemcpyAsync(hr.data(), rrt, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
    fresh = true;
    last_rep = it;
    all_done = true;
    for (int c = 0; c < nrhs; ++c) {
      if (!hd[c] && hr[c] <= tol2 * hb[c]) hd[c] = 1;
      all_done = all_done && hd[c];
      href[c] = hr[c];
    }
    if (all_done) break;
    cudaMemcpyAsync(done, hd.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, st);
    // continue from the true residual (p kept)
    to32cm_kernel<<<nblk(len), 256, 0, st>>>(r64, r32, n, nrhs);
    restart();
  }
  if (!fresh) {
    acc64cm_kernel<<<nblk(len), 256, 0, st>>>(x, xc32, n, nrhs);
    true_residual();
    cudaMemcpyAsync(hr.data(), rrt, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
  }
  double worst = 0.0;
  for (int c = 0; c < nrhs; ++c) worst = std::max(worst, hb[c] > 0.0 ? sqrt(hr[c] / hb[c]) : 0.0);
  *iters = it;
  *relres = worst;
  return cudaGetLastError() == cudaSuccess ? (worst <= tol ? 0 : 6) : 2;
}

}  // namespace spde
