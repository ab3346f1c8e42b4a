// Assembly-side structures and launchers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace spde {

// Model description on the device.  Canonical parameter layout (theta):
//   [0, nk)            log kappa (one value, or nbasis B-spline coefficients)
//   [nk, 2nk)          log gamma
//   [2nk, 3nk)         vx      (ignored for iso)
//   [3nk, 4nk)         vy      (ignored for iso)
//   [4nk, 4nk+nw)      advection: (wx, wy) | wx coefs, wy coefs | lambda | none
//   4nk+nw             log sigma
//   4nk+nw+1 .. +4     initial field: log kappa0, log gamma0, vx0, vy0
//   4nk+nw+5           log tau
struct DevModel {
  int Mx, Ny, T, Ns, bc, mod0_bc;
  double hx, hy, dt, V;
  int diff, mod0_diff, var_h, adv, nbasis, nk, nw;
  const double* bs;   // Ns x nbasis
  const double* bsH;  // Ns x 4 x nbasis (faces W,E,S,N)
  const double* bsA;  // Ns x 4 x nbasis (faces E,N,W,S, boundary extension applied)
  const double* ww;   // Ns x 4 given face velocities
  const double* theta;
};

// Compact Q: per-cell spatial stencils (see assemble.cu).
struct QStencil {
  const double* Q0;   // Ns x 25: first diagonal block minus c*Qs (mod0's A0^T V^-1 A0)
  const double* QA;   // Ns x 25: c * A^T (Qs/V^2) A   (T == 1 or separable: A^T V^-1 A)
  const double* QO;   // Ns x 9 : -c Qs V^-1 A, block (t, t+1)
  const double* cQs;  // Ns     : c * V kappa^2
  int Mx, Ny, T, Ns;
  // separable space-time models, Q = Qt (x) Qs with Qs = QA and the tridiagonal
  // Qt given by its end and interior diagonal and its off-diagonal
  int sep = 0;
  double qt_end = 0.0, qt_mid = 0.0, qt_off = 0.0;
};

#ifdef __CUDACC__
// Offset (dx, dy, dt) of slot s in the layout with `nslots` slots (25: spatial,
// 43: spatio-temporal, 75: separable; see spde_internal.h).
__device__ __forceinline__ void stencil_slot(int nslots, int s, int* dx, int* dy, int* dt) {
  if (nslots == 25) { *dt = 0; *dy = s / 5 - 2; *dx = s % 5 - 2; return; }
  if (nslots == 75) { *dt = s / 25 - 1; const int r = s % 25; *dy = r / 5 - 2; *dx = r % 5 - 2; return; }
  if (s < 9) { *dt = -1; *dy = s / 3 - 1; *dx = s % 3 - 1; }
  else if (s < 34) { *dt = 0; *dy = (s - 9) / 5 - 2; *dx = (s - 9) % 5 - 2; }
  else { *dt = 1; *dy = (s - 34) / 3 - 1; *dx = (s - 34) % 3 - 1; }
}

// Value of Q at node (cell c, time t), stencil offset (dx, dy, dt).
__device__ __forceinline__ double qval(const QStencil& q, int c, int t, int dx, int dy, int dt) {
  if (q.sep) {
    const double w = dt != 0 ? q.qt_off : (t == 0 || t == q.T - 1 ? q.qt_end : q.qt_mid);
    return w * q.QA[int64_t(c) * 25 + (dy + 2) * 5 + dx + 2];
  }
  if (q.T == 1) return q.QA[int64_t(c) * 25 + (dy + 2) * 5 + dx + 2];
  if (dt == 0) {
    const int s = (dy + 2) * 5 + dx + 2;
    const bool ctr = dx == 0 && dy == 0;
    if (t == 0) return q.Q0[int64_t(c) * 25 + s] + (ctr ? q.cQs[c] : 0.0);
    double v = q.QA[int64_t(c) * 25 + s];
    if (t < q.T - 1 && ctr) v += q.cQs[c];
    return v;
  }
  if (dt == 1) return q.QO[int64_t(c) * 9 + (dy + 1) * 3 + dx + 1];
  const int mcell = c + dy * q.Mx + dx;
  return q.QO[int64_t(mcell) * 9 + (1 - dy) * 3 + (1 - dx)];
}
#endif

void launch_fields(const DevModel& m, double* Ageo, double* A0geo, double* kap, double* qs, cudaStream_t st);
void launch_qstencil(const DevModel& m, const double* Ageo, const double* A0geo, const double* kap, const double* qs,
                     double* Q0, double* QA, double* QO, double* cQs, double cfac, cudaStream_t st);
void launch_qexport(const QStencil& q, int nslots, const double* obs, double tau, double* out, cudaStream_t st);
template <typename T>
void launch_scatter(const QStencil& q, int nslots, const int* amap, const int* perm, const int* front_of,
                    const DevFront* fronts, const double* obs, double tau, T* L, cudaStream_t st);
void launch_spmv(const QStencil& q, const double* obs, double tau, const double* x, double* y, int nrhs,
                 cudaStream_t st);
void launch_diffusion_triplets(int M, int N, const double* H, int field, double hx, double hy, int bc, int* row,
                               int* col, double* val, cudaStream_t st);
void launch_advection_triplets(int M, int N, const double* G, const double* dG, int field, double hx, double hy,
                               int bc, int diff, int* row, int* col, double* val, cudaStream_t st);
template <typename T>
void launch_to_new(const double* src, const int* perm, int n, int nrhs, T* dst, cudaStream_t st);
template <typename T>
void launch_from_new(const T* src, const int* perm, int n, int nrhs, double* dst, int acc, cudaStream_t st);

}  // namespace spde
