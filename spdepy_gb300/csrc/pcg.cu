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

// Features, network forward and G weights, one thread per node.
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
  const int y = c / q.Mx, x = c - y * q.Mx;
  double diag = qval(q, c, t, 0, 0, 0) + (obs ? tau * obs[p] : 0.0);
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
    w[int64_t(o) * n + p] = in ? ((o == 13 ? 1.f : 0.f) + a) * s : 0.f;
  }
  if (act) {
    float* ap = act + p * kAct;
#pragma unroll
    for (int j = 0; j < kFeat; ++j) ap[j] = f[j];
#pragma unroll
    for (int j = 0; j < kHid; ++j) ap[kFeat + j] = h1[j];
#pragma unroll
    for (int j = 0; j < kHid; ++j) ap[kFeat + kHid + j] = h2[j];
    ap[kAct - 1] = s;
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

// FP32 copy of a vector: the preconditioner reads every entry from 27 nodes,
// so converting once here keeps FP64 -> FP32 conversions (on the narrow FP64
// pipe of this part) out of the stencil passes.
__global__ void pc_to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t len) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < len) y[i] = float(x[i]);
}

// Jacobi: out = x / A_pp
__global__ void pc_jacobi_kernel(QStencil q, const double* __restrict__ obs, double tau, const double* __restrict__ x,
                                 double* __restrict__ out, int nrhs) {
  const int n = q.Ns * q.T;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int p = nrhs == 1 ? e : e / nrhs;
  const int t = p / q.Ns, c = p - t * q.Ns;
  const double d = qval(q, c, t, 0, 0, 0) + (obs ? tau * obs[p] : 0.0);
  out[e] = double(__fdividef(float(x[e]), float(d)));  // FP32: see pc_apply_kernel
}

// e = z - v (in place into v)
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

// CG updates with per-column scalars kept on the device.
//   x += alpha p, r -= alpha Ap with alpha = rz / pAp (0 where pAp <= 0 or done)
__global__ void pcg_xr_kernel(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                              const double* __restrict__ ap, const double* __restrict__ rz,
                              const double* __restrict__ pap, const int* __restrict__ done, int64_t n, int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int c = nrhs == 1 ? 0 : int(e % nrhs);
  if (done[c]) return;
  const double alpha = pap[c] > 0.0 ? rz[c] / pap[c] : 0.0;
  x[e] = fma(alpha, p[e], x[e]);
  r[e] = fma(-alpha, ap[e], r[e]);
}
//   p = z + beta p with beta = rz_new / rz_old
__global__ void pcg_p_kernel(double* __restrict__ p, const double* __restrict__ z, const double* __restrict__ rzn,
                             const double* __restrict__ rzo, const int* __restrict__ done, int64_t n, int nrhs) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * nrhs) return;
  const int c = nrhs == 1 ? 0 : int(e % nrhs);
  if (done[c]) return;
  const double beta = rzo[c] != 0.0 ? rzn[c] / rzo[c] : 0.0;
  p[e] = fma(beta, p[e], z[e]);
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

void apply_precond(Plan* p, int kind, const float* w, const double* obs, double tau, const double* r, double* z,
                   double* tmp, int nrhs) {
  const QStencil q = p->qstencil();
  const int64_t len = int64_t(p->sym.n) * nrhs;
  if (kind == 0) {
    cudaMemcpyAsync(z, r, size_t(len) * sizeof(double), cudaMemcpyDeviceToDevice, p->stream);
  } else if (kind == 1) {
    pc_jacobi_kernel<<<nblk(len), 256, 0, p->stream>>>(q, obs, tau, r, z, nrhs);
  } else {
    // FP32 copy of r and the FP32 intermediate G r share tmp (len doubles)
    float* r32 = reinterpret_cast<float*>(tmp);
    float* t32 = r32 + len;
    pc_to_f32_kernel<<<nblk(len), 256, 0, p->stream>>>(r, r32, len);
    pc_apply_kernel<0, float, float><<<nblk(len), 256, 0, p->stream>>>(q, w, r32, t32, nrhs);
    pc_apply_kernel<1, float, double><<<nblk(len), 256, 0, p->stream>>>(q, w, t32, z, nrhs);
  }
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

int pcg_solve(Plan* p, int with_obs, double tau, int kind, const float* w, const double* b, double* x, int nrhs,
              double tol, int maxit, int check_every, int* iters, double* relres) {
  const int64_t n = p->sym.n, len = n * nrhs;
  if (len >= (int64_t(1) << 31)) return 1;  // the stencil kernels index entries in 32 bits
  const size_t need = size_t(5 * len) + size_t(kDotBlocks) * nrhs + size_t(8 * nrhs) + size_t(nrhs);
  double* base = scratch(p, need);
  if (!base) return 4;
  double *r = base, *z = r + len, *pp = z + len, *ap = pp + len, *tmp = ap + len, *part = tmp + len;
  double* sc = part + size_t(kDotBlocks) * nrhs;  // rz, rzn, pap, rr, bb (nrhs each)
  double *rz = sc, *rzn = sc + nrhs, *pap = sc + 2 * nrhs, *rr = sc + 3 * nrhs, *bb = sc + 4 * nrhs;
  int* done = reinterpret_cast<int*>(sc + 8 * nrhs);
  const QStencil q = p->qstencil();
  const double* obs = with_obs ? p->d_obs_cnt : nullptr;
  cudaStream_t st = p->stream;
  cudaMemsetAsync(x, 0, size_t(len) * sizeof(double), st);
  cudaMemcpyAsync(r, b, size_t(len) * sizeof(double), cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(done, 0, size_t(nrhs) * sizeof(int), st);
  col_dots(p, b, b, nrhs, part, bb);
  apply_precond(p, kind, w, obs, tau, r, z, tmp, nrhs);
  cudaMemcpyAsync(pp, z, size_t(len) * sizeof(double), cudaMemcpyDeviceToDevice, st);
  col_dots(p, r, z, nrhs, part, rz);
  std::vector<double> hb(nrhs), hr(nrhs);
  std::vector<int> hd(nrhs, 0);
  cudaMemcpyAsync(hb.data(), bb, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
  int it = 0;
  double worst = 0.0;
  bool all_done = false;
  while (it < maxit && !all_done) {
    launch_spmv(q, obs, tau, pp, ap, nrhs, st);
    col_dots(p, pp, ap, nrhs, part, pap);
    pcg_xr_kernel<<<nblk(len), 256, 0, st>>>(x, r, pp, ap, rz, pap, done, n, nrhs);
    apply_precond(p, kind, w, obs, tau, r, z, tmp, nrhs);
    col_dots(p, r, z, nrhs, part, rzn);
    pcg_p_kernel<<<nblk(len), 256, 0, st>>>(pp, z, rzn, rz, done, n, nrhs);
    cudaMemcpyAsync(rz, rzn, nrhs * sizeof(double), cudaMemcpyDeviceToDevice, st);
    ++it;
    if (it % check_every == 0 || it == maxit) {
      col_dots(p, r, r, nrhs, part, rr);
      cudaMemcpyAsync(hr.data(), rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
      all_done = true;
      worst = 0.0;
      for (int c = 0; c < nrhs; ++c) {
        const double rel = hb[c] > 0.0 ? sqrt(hr[c] / hb[c]) : 0.0;
        if (!hd[c] && rel <= tol) hd[c] = 1;
        all_done = all_done && hd[c];
        worst = std::max(worst, rel);
      }
      cudaMemcpyAsync(done, hd.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, st);
    }
  }
  // true residual of the returned x
  launch_spmv(q, obs, tau, x, ap, nrhs, st);
  pc_sub_kernel<<<nblk(len), 256, 0, st>>>(b, ap, len);
  col_dots(p, ap, ap, nrhs, part, rr);
  cudaMemcpyAsync(hr.data(), rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
  worst = 0.0;
  for (int c = 0; c < nrhs; ++c) worst = std::max(worst, hb[c] > 0.0 ? sqrt(hr[c] / hb[c]) : 0.0);
  *iters = it;
  *relres = worst;
  return cudaGetLastError() == cudaSuccess ? (worst <= tol ? 0 : 6) : 2;
}

}  // namespace spde
