// Batched dense kernels of the multifrontal factorisation, selected inversion
// and solves.  Every launch walks a task list prepared once per lattice by the
// symbolic phase, so fronts of very different sizes share one launch.
//
// This file holds the SIMT kernels (FP64 "plain" path, and the FP32 path on
// tiles the tensor-core kernel does not take).
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>

#include "kernels.cuh"

namespace spde {

// --------------------------------------------------------------------- GEMM
template <typename T>
struct GemmCfg;
template <>
struct GemmCfg<double> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};
template <>
struct GemmCfg<float> {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8;
};

// A, B and C may alias (in-place triangular solves): every block reads all of
// its A and B tiles before its epilogue writes C, and blocks own disjoint C tiles.
template <typename T, int MODE, int AL, int BL>
__global__ void __launch_bounds__(256) gemm_kernel(const GemmTask* __restrict__ tasks, const T* Ab, const T* Bb,
                                                   T* Cb) {
  using C = GemmCfg<T>;
  constexpr int BM = C::BM, BN = C::BN, BK = C::BK, TM = C::TM, TN = C::TN;
  __shared__ T As[BK][BM + 4];
  __shared__ T Bs[BK][BN + 4];
  const GemmTask tk = tasks[blockIdx.x];
  const T* A = Ab + tk.a;
  const T* B = Bb + tk.b;
  T* Cp = Cb + tk.c;
  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN);  // column group
  const int ty = tid / (BN / TN);  // row group
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < tk.k; k0 += BK) {
    // A tile: BM x BK
    for (int e = tid; e < BM * BK; e += 256) {
      int i, kk;
      if (AL == kRow) { kk = e % BK; i = e / BK; } else { i = e % BM; kk = e / BM; }
      T v = T(0);
      if (i < tk.m && k0 + kk < tk.k)
        v = (AL == kRow) ? A[int64_t(i) * tk.lda + k0 + kk] : A[int64_t(k0 + kk) * tk.lda + i];
      As[kk][i] = v;
    }
    for (int e = tid; e < BN * BK; e += 256) {
      int j, kk;
      if (BL == kRow) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
      T v = T(0);
      if (j < tk.n && k0 + kk < tk.k)
        v = (BL == kRow) ? B[int64_t(j) * tk.ldb + k0 + kk] : B[int64_t(k0 + kk) * tk.ldb + j];
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int r = ty * TM + i;
    if (r >= tk.m) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int c = tx * TN + j;
      if (c >= tk.n) continue;
      T* dst = Cp + int64_t(r) * tk.ldc + c;
      if (MODE == kSub) *dst -= acc[i][j];
      else if (MODE == kStore) *dst = acc[i][j];
      else if (MODE == kNegStore) *dst = -acc[i][j];
      else *dst += acc[i][j];
    }
  }
}

template <typename T, int MODE>
static void gemm_mode(const GemmTask* t, int n, const T* A, const T* B, T* C, int al, int bl, cudaStream_t st) {
  if (al == kRow && bl == kRow) gemm_kernel<T, MODE, kRow, kRow><<<n, 256, 0, st>>>(t, A, B, C);
  else if (al == kRow && bl == kCol) gemm_kernel<T, MODE, kRow, kCol><<<n, 256, 0, st>>>(t, A, B, C);
  else if (al == kCol && bl == kRow) gemm_kernel<T, MODE, kCol, kRow><<<n, 256, 0, st>>>(t, A, B, C);
  else gemm_kernel<T, MODE, kCol, kCol><<<n, 256, 0, st>>>(t, A, B, C);
}

// ------------------------------------------------------------ narrow GEMM
// Products with at most 8 output columns (solves with few right-hand sides) are
// bandwidth work: one CTA per task (m <= 128 rows) streams its A once,
// coalesced, against B staged in shared memory.  Each thread keeps 16 to 32
// independent loads in flight, and the CTA holds only 8 KB of shared memory
// (FP32), so that it fits on an SM beside a resident tensor-core CTA.  NB (1 or
// 8) bounds the task's columns.  Every CTA reads all of its A and B before it
// writes C (in-place solves stay valid).
constexpr int kNarrowN = 8;
constexpr int kNarrowBEnt = 2048;  // shared entries: staged B (NB x k chunk), then the k-split partial sums

// Sum of v[r] over the 32 lanes of the warp for the eight rows r: lanes with
// (lane >> 2) == r receive row r (a butterfly that halves the rows each lane
// carries at every step: 9 shuffles instead of 8 x 5).
template <typename T>
__device__ __forceinline__ T warp_sum8(const T (&v)[8], int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  T w[4], x[2];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const T send = b4 ? v[r] : v[r + 4], keep = b4 ? v[r + 4] : v[r];
    w[r] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const T send = b3 ? w[r] : w[r + 2], keep = b3 ? w[r + 2] : w[r];
    x[r] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  T y = (b2 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, b2 ? x[0] : x[1], 4);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  return y;
}

template <int MODE, typename T>
__device__ __forceinline__ void narrow_store(T* dst, T v) {
  if (MODE == kSub) *dst -= v;
  else if (MODE == kStore) *dst = v;
  else if (MODE == kNegStore) *dst = -v;
  else *dst += v;
}

template <typename T, int MODE, int AL, int NB>
__global__ void __launch_bounds__(256) gemv_kernel(const GemmTask* __restrict__ tasks, const T* Ab, const T* Bb,
                                                   T* Cb, int bl) {
  constexpr int kc = kNarrowBEnt / NB;  // k values per staged chunk (a multiple of 64)
  __shared__ T sh[kNarrowBEnt];         // Bs[j * kc + kk] while streaming, partial sums after
  const GemmTask tk = tasks[blockIdx.x];
  const T* A = Ab + tk.a;
  const T* B = Bb + tk.b;
  T* C = Cb + tk.c;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = tk.n, m = tk.m;
  if (AL == kRow) {
    // rows in batches of 8; warp w owns batches w and w + 8 (m <= 128); lanes
    // stride along k, 64 k values per step
    constexpr int BAT = NB == 1 ? 2 : 1;  // batches loaded together
    T res[2][NB];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int j = 0; j < NB; ++j) res[q][j] = T(0);
    for (int k0 = 0; k0 < tk.k; k0 += kc) {
      const int kn = min(kc, tk.k - k0);
      const int kp = (kn + 63) & ~63;
      __syncthreads();
      for (int e = tid; e < kp * NB; e += 256) {
        const int j = e / kp, kk = e - j * kp;
        T v = T(0);
        if (kk < kn && j < n) v = bl == kRow ? B[int64_t(j) * tk.ldb + k0 + kk] : B[int64_t(k0 + kk) * tk.ldb + j];
        sh[j * kc + kk] = v;
      }
      __syncthreads();
#pragma unroll
      for (int b0 = 0; b0 < 2; b0 += BAT) {
        if (8 * (warp + 8 * b0) >= m) break;
        T v[BAT][8][NB];
#pragma unroll
        for (int q = 0; q < BAT; ++q)
#pragma unroll
          for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int j = 0; j < NB; ++j) v[q][r][j] = T(0);
        for (int kk0 = 0; kk0 < kn; kk0 += 64) {
          T a[BAT][8][2];
#pragma unroll
          for (int q = 0; q < BAT; ++q)
#pragma unroll
            for (int r = 0; r < 8; ++r) {
              const int i = 8 * (warp + 8 * (b0 + q)) + r;
              const T* ar = A + int64_t(i) * tk.lda + k0 + kk0 + lane;
#pragma unroll
              for (int u = 0; u < 2; ++u)
                a[q][r][u] = (i < m && kk0 + lane + 32 * u < kn) ? ar[32 * u] : T(0);
            }
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            T bv[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) bv[j] = sh[j * kc + kk0 + lane + 32 * u];
#pragma unroll
            for (int q = 0; q < BAT; ++q)
#pragma unroll
              for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int j = 0; j < NB; ++j) v[q][r][j] = fma(a[q][r][u], bv[j], v[q][r][j]);
          }
        }
#pragma unroll
        for (int q = 0; q < BAT; ++q)
#pragma unroll
          for (int j = 0; j < NB; ++j) {
            T col[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) col[r] = v[q][r][j];
            res[b0 + q][j] += warp_sum8(col, lane);
          }
      }
    }
    __syncthreads();
    if ((lane & 3) == 0) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int i = 8 * (warp + 8 * q) + (lane >> 2);
        if (i < m) {
#pragma unroll
          for (int j = 0; j < NB; ++j)
            if (j < n) narrow_store<MODE>(C + int64_t(i) * tk.ldc + j, res[q][j]);
        }
      }
    }
  } else {
    // thread (h, i): row i, every H-th k value starting at h; 8 loads in flight
    const int rsh = m <= 32 ? 5 : (m <= 64 ? 6 : 7);
    const int i = tid & ((1 << rsh) - 1), h = tid >> rsh, H = 256 >> rsh;
    T s[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) s[j] = T(0);
    for (int k0 = 0; k0 < tk.k; k0 += kc) {
      const int kn = min(kc, tk.k - k0);
      __syncthreads();
      for (int e = tid; e < kn * NB; e += 256) {
        const int j = e / kn, kk = e - j * kn;
        T v = T(0);
        if (j < n) v = bl == kRow ? B[int64_t(j) * tk.ldb + k0 + kk] : B[int64_t(k0 + kk) * tk.ldb + j];
        sh[j * kc + kk] = v;
      }
      __syncthreads();
      if (i < m) {
        const T* ac = A + int64_t(k0) * tk.lda + i;
        int kk = h;
        for (; kk + 7 * H < kn; kk += 8 * H) {
          T a[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) a[u] = ac[int64_t(kk + u * H) * tk.lda];
#pragma unroll
          for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int j = 0; j < NB; ++j) s[j] = fma(a[u], sh[j * kc + kk + u * H], s[j]);
        }
        for (; kk < kn; kk += H) {
          const T a = ac[int64_t(kk) * tk.lda];
#pragma unroll
          for (int j = 0; j < NB; ++j) s[j] = fma(a, sh[j * kc + kk], s[j]);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NB; ++j) sh[j * 256 + tid] = s[j];
    __syncthreads();
    for (int e = tid; e < m * n; e += 256) {
      const int ii = e / n, j = e - ii * n;
      T v = T(0);
      for (int hh = 0; hh < H; ++hh) v += sh[j * 256 + (hh << rsh) + ii];
      narrow_store<MODE>(C + int64_t(ii) * tk.ldc + j, v);
    }
  }
}

// ------------------------------------------------------ panel solve (FP32)
// X = A Linv^T for one 64-column diagonal block: tasks with m <= 128 rows,
// n <= 64 columns and k <= 64, both operands in row layout.  The CTA stages its
// whole A tile and the block inverse in shared memory once (no K loop), then
// each thread computes an 8 x 4 block of the output; A may alias C (in-place
// panel solve): every read happens before the first write.
constexpr int kPanelLdA = 129, kPanelLdB = 65;
constexpr int kPanelSmem = (64 * kPanelLdA + 64 * kPanelLdB) * int(sizeof(float));

template <int MODE>
__global__ void __launch_bounds__(256) panel64_kernel(const GemmTask* __restrict__ tasks, const float* Ab,
                                                      const float* Bb, float* Cb) {
  extern __shared__ float psm[];
  float* As = psm;                     // As[k * kPanelLdA + i] = A(i, k)
  float* Bs = psm + 64 * kPanelLdA;    // Bs[k * kPanelLdB + j] = B(j, k)
  const GemmTask tk = tasks[blockIdx.x];
  const float* A = Ab + tk.a;
  const float* B = Bb + tk.b;
  float* C = Cb + tk.c;
  const int tid = threadIdx.x;
  for (int e = tid; e < 128 * 64; e += 256) {
    const int i = e >> 6, k = e & 63;
    As[k * kPanelLdA + i] = (i < tk.m && k < tk.k) ? A[int64_t(i) * tk.lda + k] : 0.f;
  }
  for (int e = tid; e < 64 * 64; e += 256) {
    const int j = e >> 6, k = e & 63;
    Bs[k * kPanelLdB + j] = (j < tk.n && k < tk.k) ? B[int64_t(j) * tk.ldb + k] : 0.f;
  }
  __syncthreads();
  const int ty = tid >> 4, tx = tid & 15;  // rows 8 ty .. + 7, columns 4 tx .. + 3
  float acc[8][4];
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
  for (int kk = 0; kk < tk.k; ++kk) {
    float a[8], b[4];
#pragma unroll
    for (int r = 0; r < 8; ++r) a[r] = As[kk * kPanelLdA + ty * 8 + r];
#pragma unroll
    for (int c = 0; c < 4; ++c) b[c] = Bs[kk * kPanelLdB + tx * 4 + c];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int i = ty * 8 + r;
    if (i >= tk.m) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = tx * 4 + c;
      if (j >= tk.n) continue;
      float* dst = C + int64_t(i) * tk.ldc + j;
      if (MODE == kSub) *dst -= acc[r][c];
      else if (MODE == kStore) *dst = acc[r][c];
      else if (MODE == kNegStore) *dst = -acc[r][c];
      else *dst += acc[r][c];
    }
  }
}

template <int MODE>
static void panel64_launch(const GemmTask* t, int n, const float* A, const float* B, float* C, cudaStream_t st) {
  static const bool attr = [] {  // once, thread-safely (two pipelines launch from two host threads)
    cudaFuncSetAttribute(panel64_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPanelSmem);
    return true;
  }();
  (void)attr;
  panel64_kernel<MODE><<<n, 256, kPanelSmem, st>>>(t, A, B, C);
}

template <typename T, int MODE>
static void gemv_mode(const GemmTask* t, int n, const T* A, const T* B, T* C, int al, int bl, cudaStream_t st,
                      int nmax) {
  if (nmax == 1) {
    if (al == kRow) gemv_kernel<T, MODE, kRow, 1><<<n, 256, 0, st>>>(t, A, B, C, bl);
    else gemv_kernel<T, MODE, kCol, 1><<<n, 256, 0, st>>>(t, A, B, C, bl);
  } else {
    if (al == kRow) gemv_kernel<T, MODE, kRow, kNarrowN><<<n, 256, 0, st>>>(t, A, B, C, bl);
    else gemv_kernel<T, MODE, kCol, kNarrowN><<<n, 256, 0, st>>>(t, A, B, C, bl);
  }
}

// The FP32 products run on the tensor cores unless SPDE_TC=0 is set in the environment.
bool tc_gemm_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("SPDE_TC");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on == 1;
}

template <typename T>
void launch_gemm(const GemmTask* tasks, int ntasks, const T* A, const T* B, T* C, int mode, int alayout, int blayout,
                 cudaStream_t st, int path, int nmax, unsigned long long wait_ns) {
  if (ntasks <= 0) return;
  if (path == kPathNarrow) {
    switch (mode) {
      case kSub: gemv_mode<T, kSub>(tasks, ntasks, A, B, C, alayout, blayout, st, nmax); break;
      case kStore: gemv_mode<T, kStore>(tasks, ntasks, A, B, C, alayout, blayout, st, nmax); break;
      case kNegStore: gemv_mode<T, kNegStore>(tasks, ntasks, A, B, C, alayout, blayout, st, nmax); break;
      default: gemv_mode<T, kAdd>(tasks, ntasks, A, B, C, alayout, blayout, st, nmax); break;
    }
    return;
  }
  if constexpr (sizeof(T) == sizeof(float)) {
    if (path == kPathPanel && alayout == kRow && blayout == kRow) {
      const float* Af = reinterpret_cast<const float*>(A);
      const float* Bf = reinterpret_cast<const float*>(B);
      float* Cf = reinterpret_cast<float*>(C);
      switch (mode) {
        case kSub: panel64_launch<kSub>(tasks, ntasks, Af, Bf, Cf, st); break;
        case kStore: panel64_launch<kStore>(tasks, ntasks, Af, Bf, Cf, st); break;
        case kNegStore: panel64_launch<kNegStore>(tasks, ntasks, Af, Bf, Cf, st); break;
        default: panel64_launch<kAdd>(tasks, ntasks, Af, Bf, Cf, st); break;
      }
      return;
    }
    if (path == kPathTensor && tc_gemm_enabled()) {
      launch_gemm_tc(tasks, ntasks, reinterpret_cast<const float*>(A), reinterpret_cast<const float*>(B),
                     reinterpret_cast<float*>(C), mode, alayout, blayout, st, wait_ns);
      return;
    }
  }
  switch (mode) {
    case kSub: gemm_mode<T, kSub>(tasks, ntasks, A, B, C, alayout, blayout, st); break;
    case kStore: gemm_mode<T, kStore>(tasks, ntasks, A, B, C, alayout, blayout, st); break;
    case kNegStore: gemm_mode<T, kNegStore>(tasks, ntasks, A, B, C, alayout, blayout, st); break;
    default: gemm_mode<T, kAdd>(tasks, ntasks, A, B, C, alayout, blayout, st); break;
  }
}

template void launch_gemm<double>(const GemmTask*, int, const double*, const double*, double*, int, int, int,
                                  cudaStream_t, int, int, unsigned long long);
template void launch_gemm<float>(const GemmTask*, int, const float*, const float*, float*, int, int, int,
                                 cudaStream_t, int, int, unsigned long long);

// --------------------------------------------------- diagonal block POTRF
// Cholesky factor and inverse of one w x w diagonal block (w <= 64) per CTA.
//
// The factorisation runs in FP64 whatever the storage type, so the pivots and
// the log-determinant carry FP64 arithmetic (an FP32 sweep measured 1e-6
// relative log-likelihood error against 1e-7 at 960k nodes).  FP64 is a narrow
// pipe on this part, so the sweep is arranged around it: the block lives in the
// registers of 256 threads, thread (ty, tx) = (tid / 16, tid % 16) owning the
// entries (i, k) = (ty + 16 m, tx + 16 n), m, n = 0..3.  Step j reads column j of
// the partly reduced block from a shared buffer, applies
// a_ik -= a_ij a_kj / a_jj (j < k <= i) and publishes column j + 1, one barrier
// per column and one FP64 division per warp; square roots come at the end:
// L_ij = a_ij / sqrt(d_j) and log L_jj = log(d_j) / 2 with d_j the j-th pivot.
// L^-1 (consumed by the panel products as a product operand) then follows by
// forward elimination in the storage type's arithmetic with the same ownership.
constexpr int kMaxNbk = 64;

template <typename T>
__global__ void __launch_bounds__(256) potrf_kernel(const DiagTask* __restrict__ tasks, T* __restrict__ L,
                                                    T* __restrict__ dinv, double* __restrict__ logpiv,
                                                    int* __restrict__ err) {
  __shared__ double colb[2][kMaxNbk];
  __shared__ double dpiv[kMaxNbk];
  __shared__ double sq[kMaxNbk];
  __shared__ T lsh[kMaxNbk][kMaxNbk + 1];
  __shared__ T xrow[2][kMaxNbk];
  __shared__ int bad;
  const DiagTask tk = tasks[blockIdx.x];
  const int w = tk.w;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  T* blk = L + tk.a;
  double r[4][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int i = ty + 16 * m, k = tx + 16 * n;
      r[m][n] = (k <= i && i < w) ? double(blk[int64_t(i) * tk.lda + k]) : 0.0;
    }
  if (tid == 0) bad = 0;
  if (tx == 0) {
#pragma unroll
    for (int m = 0; m < 4; ++m)
      if (ty + 16 * m < w) colb[0][ty + 16 * m] = r[m][0];
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const double* c = colb[j & 1];
    double d = c[j];
    if (!(d > 0.0) || !isfinite(d)) {
      d = 1.0;
      if (tid == 0) bad = 1;
    }
    double q = 0.0;
    if ((tid & 31) == 0) q = 1.0 / d;
    const double dv = __shfl_sync(0xffffffffu, q, 0);
    if (tid == 0) dpiv[j] = d;
    double ci[4], ck[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = ty + 16 * m;
      ci[m] = (i > j && i < w) ? c[i] * dv : 0.0;
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int k = tx + 16 * n;
      ck[n] = (k > j && k < w) ? c[k] : 0.0;
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (16 * m + 15 <= j) continue;  // block row finished (uniform over the CTA)
#pragma unroll
      for (int n = 0; n <= m; ++n) {
        if (16 * n + 15 <= j) continue;
        r[m][n] -= ci[m] * ck[n];
      }
    }
    // publish column j + 1 (its owners hold it fully reduced by columns 0..j)
    const int jn = j + 1;
    if (jn < w && tx == (jn & 15)) {
      const int n = jn >> 4;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int i = ty + 16 * m;
        if (i >= jn && i < w) {
#pragma unroll
          for (int nn = 0; nn < 4; ++nn)
            if (nn == n) colb[jn & 1][i] = r[m][nn];
        }
      }
    }
    __syncthreads();
  }
  if (tid < w) sq[tid] = sqrt(dpiv[tid]);
  if (tid < 32) {
    double s = 0.0;
    for (int j = tid; j < w; j += 32) s += 0.5 * log(dpiv[j]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (tid == 0) {
      logpiv[blockIdx.x] = s;
      if (bad) atomicCAS(err, -1, tk.front);
    }
  }
  __syncthreads();
  // L = a_ik / sqrt(d_k) below the diagonal, sqrt(d_k) on it; zero above
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int i = ty + 16 * m, k = tx + 16 * n;
      if (i < w && k < w) {
        const T v = k < i ? T(r[m][n] / sq[k]) : (k == i ? T(sq[k]) : T(0));
        lsh[i][k] = v;
        blk[int64_t(i) * tk.lda + k] = v;
      }
    }
  // X = L^-1: B = I; step j takes the finished row j of X and applies
  // B_ic -= L_ij X_jc (i > j, c <= j); row j + 1 finishes as B_(j+1)c / L_(j+1)(j+1)
  T b[4][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) b[m][n] = (ty + 16 * m == tx + 16 * n) ? T(1) : T(0);
  __syncthreads();
  if (ty == 0 && tx == 0) {
    b[0][0] = T(1) / lsh[0][0];
    xrow[0][0] = b[0][0];
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const T* xr = xrow[j & 1];
    T li[4], xc[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = ty + 16 * m;
      li[m] = (i > j && i < w) ? lsh[i][j] : T(0);
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int cc = tx + 16 * n;
      xc[n] = cc <= j ? xr[cc] : T(0);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (16 * m + 15 <= j) continue;
#pragma unroll
      for (int n = 0; n <= m; ++n) {
        if (16 * n > j) continue;  // columns beyond j of row j of X are zero
        b[m][n] -= li[m] * xc[n];
      }
    }
    const int jn = j + 1;
    if (jn < w && ty == (jn & 15)) {
      const int m = jn >> 4;
      const T inv = T(1) / lsh[jn][jn];
#pragma unroll
      for (int mm = 0; mm < 4; ++mm) {
        if (mm != m) continue;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const int cc = tx + 16 * n;
          if (cc <= jn) {
            b[mm][n] *= inv;
            xrow[jn & 1][cc] = b[mm][n];
          }
        }
      }
    }
    __syncthreads();
  }
  T* dv = dinv + tk.dinv;
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int i = ty + 16 * m, cc = tx + 16 * n;
      if (i < w && cc < w) dv[int64_t(i) * kMaxNbk + cc] = cc <= i ? b[m][n] : T(0);
    }
}

// ---------------------------------------------- double-float diagonal block
// The mixed path's diagonal blocks: the same register-blocked right-looking
// sweep as potrf_kernel, in double-float arithmetic (value = hi + lo, two FP32
// numbers, about 44 significant bits; Dekker/Knuth error-free transformations
// with FMA), which runs on the FP32 pipe instead of the narrow FP64 one.  Pivots
// are converted to FP64 for the log-determinant; L and L^-1 are rounded to FP32
// for storage (L^-1 from the FP32 L, as in potrf_kernel).
struct DF {
  float hi, lo;
};
// The _rn intrinsics keep the compiler from contracting the error-free
// transformations into FMAs.
__device__ __forceinline__ DF df_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}
// b * c
__device__ __forceinline__ DF df_mul(DF b, DF c) {
  const float p = __fmul_rn(b.hi, c.hi);
  float e = fmaf(b.hi, c.hi, -p);
  e = fmaf(b.hi, c.lo, e);
  e = fmaf(b.lo, c.hi, e);
  return df_renorm(p, e);
}
// a - b * c
__device__ __forceinline__ DF df_fms(DF a, DF b, DF c) {
  const float p = __fmul_rn(b.hi, c.hi);
  float e = fmaf(b.hi, c.hi, -p);
  e = fmaf(b.hi, c.lo, e);
  e = fmaf(b.lo, c.hi, e);
  const float s = __fsub_rn(a.hi, p);
  const float v = __fsub_rn(s, a.hi);
  float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(-p, v));
  err = __fadd_rn(err, __fsub_rn(a.lo, e));
  return df_renorm(s, err);
}
// 1 / d: FP32 reciprocal estimate refined by one Newton step with a
// double-float residual (the step squares the estimate's relative error, so
// the hardware approximation is enough)
__device__ __forceinline__ DF df_rcp(DF d) {
  const float r = __fdividef(1.0f, d.hi);
  const DF one_minus = df_fms(DF{1.0f, 0.0f}, d, DF{r, 0.0f});  // 1 - d r
  return df_renorm(r, __fmul_rn(r, one_minus.hi));
}

// 1 / sqrt(d) rounded to FP32 for a double-float pivot, without the (narrow)
// FP64 pipe: the hardware estimate y refined by one Newton-Raphson step
// y + y e / 2 with the residual e = 1 - d y^2 formed from the exact square of y
// (FMA error terms), which leaves an error far below FP32 rounding.
__device__ __forceinline__ float df_rsqrt(DF d) {
  const float y = rsqrtf(d.hi);
  const float p = __fmul_rn(y, y);
  const float pe = fmaf(y, y, -p);        // y^2 = p + pe exactly
  float e = fmaf(-d.hi, p, 1.0f);         // 1 - d_hi p, one rounding
  e = fmaf(-d.hi, pe, e);
  e = fmaf(-d.lo, p, e);
  return fmaf(0.5f * y, e, y);
}

// Blocked double-float factorisation of one diagonal block A = L L^T
// (w <= 64), in 16-column sub-blocks s with the trailing Schur updates written
// as A_ik -= (a_ic / d_c) a_kc, so that the pivots d_c and the columns a_ic
// (at the time column c is eliminated) stay in double-float and L_ic =
// a_ic / sqrt(d_c) is rounded to FP32 once, at the end.  Per sub-block:
//   (1) warp 0 eliminates the 16 x 16 diagonal sub-block column by column
//       (warp-synchronous, each lane holding up to five of its 136 entries);
//   (2) four threads per row below it eliminate that row's 16 columns and
//       record S_ic = a_ic / d_c;
//   (3) the whole CTA applies the rank-16 update S a^T to the trailing lower
//       triangle, 2 x 2 entries per thread.
// Then L^-1 (FP32) by sub-blocks: the four 16 x 16 diagonal inverses (one warp
// each, one lane per column), then the off-diagonal blocks by distance from the
// diagonal, X_ij = -X_ii (sum_{i > k >= j} L_ik X_kj).  About 20 CTA barriers
// in all instead of one per column.
constexpr int kDfSub = 16;

__device__ __forceinline__ int tri_row(int q) {  // largest r with r (r + 1) / 2 <= q
  int r = int((sqrtf(8.0f * float(q) + 1.0f) - 1.0f) * 0.5f);
  while (r * (r + 1) / 2 > q) --r;
  while ((r + 1) * (r + 2) / 2 <= q) ++r;
  return r;
}

__global__ void __launch_bounds__(256) potrf_df_kernel(const DiagTask* __restrict__ tasks, float* __restrict__ L,
                                                       float* __restrict__ dinv, double* __restrict__ logpiv,
                                                       int* __restrict__ err) {
  // Ah/Al: the double-float working matrix (lower triangle); after the
  // factorisation Al holds L (FP32, zero above the diagonal) and Ah holds L^-1.
  __shared__ float Ah[kMaxNbk][kMaxNbk + 1], Al[kMaxNbk][kMaxNbk + 1];
  // S_ic of the current sub-block (double-float); later the inverse's products
  __shared__ float Sh[kMaxNbk][kDfSub + 1], Sl[kMaxNbk][kDfSub + 1];
  __shared__ float dph[kMaxNbk], dpl[kMaxNbk], rsq[kMaxNbk];
  __shared__ float dvh[kDfSub], dvl[kDfSub];
  __shared__ int bad;
  const DiagTask tk = tasks[blockIdx.x];
  const int w = tk.w;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float* blk = L + tk.a;
  for (int e = tid; e < w * w; e += 256) {
    const int i = e / w, k = e - i * w;
    if (k <= i) {
      Ah[i][k] = blk[int64_t(i) * tk.lda + k];
      Al[i][k] = 0.0f;
    }
  }
  if (tid == 0) bad = 0;
  // entries of the 16 x 16 lower triangle held by this lane in (1): e = lane + 32 t
  int eii[5], ekk[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int e = lane + 32 * t;
    const int r = tri_row(e < 136 ? e : 0);
    eii[t] = e < 136 ? r : kDfSub;  // kDfSub: no entry
    ekk[t] = e < 136 ? e - r * (r + 1) / 2 : 0;
  }
  __syncthreads();
  const int nsb = (w + kDfSub - 1) / kDfSub;
  for (int sb = 0; sb < nsb; ++sb) {
    const int c0 = sb * kDfSub, cw = min(kDfSub, w - c0);
    // ---- (1) diagonal sub-block, warp 0; inactive entries are masked, not
    // branched around, so that the five updates of a lane overlap
    if (warp == 0) {
      DF v[5];
#pragma unroll
      for (int t = 0; t < 5; ++t)
        v[t] = eii[t] < cw ? DF{Ah[c0 + eii[t]][c0 + ekk[t]], Al[c0 + eii[t]][c0 + ekk[t]]} : DF{0.0f, 0.0f};
      for (int j = 0; j < cw; ++j) {
        // publish column j (its entries are final from here on)
#pragma unroll
        for (int t = 0; t < 5; ++t)
          if (eii[t] < cw && ekk[t] == j) {
            Ah[c0 + eii[t]][c0 + j] = v[t].hi;
            Al[c0 + eii[t]][c0 + j] = v[t].lo;
          }
        __syncwarp();
        DF d{Ah[c0 + j][c0 + j], Al[c0 + j][c0 + j]};
        const bool nonpos = !(d.hi > 0.0f) || !isfinite(d.hi);
        if (nonpos) d = DF{1.0f, 0.0f};
        const DF dv = df_rcp(d);
        if (lane == 0) {
          if (nonpos) bad = 1;
          dph[c0 + j] = d.hi;
          dpl[c0 + j] = d.lo;
          dvh[j] = dv.hi;
          dvl[j] = dv.lo;
        }
#pragma unroll
        for (int t = 0; t < 5; ++t) {
          const bool act = eii[t] < cw && ekk[t] > j;
          const int ri = c0 + (act ? eii[t] : j), rk = c0 + (act ? ekk[t] : j);  // (j, j) when masked
          DF ci = df_mul(DF{Ah[ri][c0 + j], Al[ri][c0 + j]}, dv);
          DF ck{Ah[rk][c0 + j], Al[rk][c0 + j]};
          if (!act) ci = ck = DF{0.0f, 0.0f};
          v[t] = df_fms(v[t], ci, ck);
        }
      }
    }
    __syncthreads();
    const int b0 = c0 + cw, mt = w - b0;  // rows below the sub-block
    if (mt <= 0) break;
    // ---- (2) panel rows, four threads per row: thread q holds the row's
    // entries in columns q, q + 4, q + 8, q + 12 of the sub-block; the owner of
    // column j forms S_ij and passes it to the other three by shuffle
    const unsigned pmask = __ballot_sync(0xffffffffu, tid < 4 * mt);
    if (tid < 4 * mt) {
      const int i = b0 + (tid >> 2), q = tid & 3;
      DF x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = q + 4 * u;
        x[u] = c < cw ? DF{Ah[i][c0 + c], Al[i][c0 + c]} : DF{0.0f, 0.0f};
      }
      for (int j = 0; j < cw; ++j) {
        const int uj = j >> 2, qj = j & 3;
        DF xj = x[0];
        if (uj == 1) xj = x[1];
        if (uj == 2) xj = x[2];
        if (uj == 3) xj = x[3];
        DF sj = df_mul(xj, DF{dvh[j], dvl[j]});
        const int src = (lane & ~3) | qj;
        sj.hi = __shfl_sync(pmask, sj.hi, src);
        sj.lo = __shfl_sync(pmask, sj.lo, src);
        if (q == qj) {
          Sh[i][j] = sj.hi;
          Sl[i][j] = sj.lo;
          Ah[i][c0 + j] = xj.hi;
          Al[i][c0 + j] = xj.lo;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = q + 4 * u;
          const bool act = c > j && c < cw;
          const int r = c0 + (act ? c : j);  // (j, j) when masked
          const DF nx = df_fms(x[u], sj, DF{Ah[r][c0 + j], Al[r][c0 + j]});
          if (act) x[u] = nx;
        }
      }
    }
    __syncthreads();
    // ---- (3) trailing update A_ik -= sum_c S_ic a_kc, 2 x 2 entries per thread
    const int nb2 = (mt + 1) >> 1, nq = nb2 * (nb2 + 1) / 2;
    for (int q = tid; q < nq; q += 256) {
      const int bi = tri_row(q), bk = q - bi * (bi + 1) / 2;
      const int i0 = b0 + 2 * bi, k0 = b0 + 2 * bk;
      const bool i1ok = i0 + 1 < w, k1ok = k0 + 1 < w;
      DF acc[2][2];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int i = i0 + r, k = k0 + u;
          const bool ok = (r == 0 || i1ok) && (u == 0 || k1ok) && k <= i;
          acc[r][u] = ok ? DF{Ah[i][k], Al[i][k]} : DF{0.0f, 0.0f};
        }
      for (int c = 0; c < cw; ++c) {
        const DF s0{Sh[i0][c], Sl[i0][c]};
        const DF s1 = i1ok ? DF{Sh[i0 + 1][c], Sl[i0 + 1][c]} : DF{0.0f, 0.0f};
        const DF a0{Ah[k0][c0 + c], Al[k0][c0 + c]};
        const DF a1 = k1ok ? DF{Ah[k0 + 1][c0 + c], Al[k0 + 1][c0 + c]} : DF{0.0f, 0.0f};
        acc[0][0] = df_fms(acc[0][0], s0, a0);
        acc[1][0] = df_fms(acc[1][0], s1, a0);
        acc[1][1] = df_fms(acc[1][1], s1, a1);
        if (bi != bk) acc[0][1] = df_fms(acc[0][1], s0, a1);
      }
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int i = i0 + r, k = k0 + u;
          if ((r == 0 || i1ok) && (u == 0 || k1ok) && k <= i) {
            Ah[i][k] = acc[r][u].hi;
            Al[i][k] = acc[r][u].lo;
          }
        }
    }
    __syncthreads();
  }
  // ---- L = a_ik / sqrt(d_k) (FP32) into Al and the block: thread (i, q)
  // holds row i, columns 16 q .. 16 q + 15
  if (tid < w) rsq[tid] = df_rsqrt(DF{dph[tid], dpl[tid]});
  __syncthreads();
  {
    const int i = tid >> 2, kq = (tid & 3) * kDfSub;
    float lv[kDfSub];
#pragma unroll
    for (int u = 0; u < kDfSub; ++u) {
      const int k = kq + u;
      float v = 0.0f;
      if (i < w && k < w) {
        if (k < i) v = (Ah[i][k] + Al[i][k]) * rsq[k];
        else if (k == i) v = 1.0f / rsq[k];
      }
      lv[u] = v;
    }
    __syncthreads();
    if (i < w) {
#pragma unroll
      for (int u = 0; u < kDfSub; ++u) {
        const int k = kq + u;
        if (k < w) {
          Al[i][k] = lv[u];
          blk[int64_t(i) * tk.lda + k] = lv[u];
        }
      }
    }
  }
  __syncthreads();
  // ---- L^-1 into Ah: diagonal 16 x 16 inverses, warp s, lane = column
  if (warp < nsb && lane < kDfSub) {
    const int c0 = warp * kDfSub, cw = min(kDfSub, w - c0), c = lane;
    if (c < cw) {
      float x[kDfSub];
#pragma unroll
      for (int ii = 0; ii < kDfSub; ++ii) {
        float v = 0.0f;
        if (ii == c) v = rsq[c0 + c];
        else if (ii > c && ii < cw) {
          float sum = 0.0f;
#pragma unroll
          for (int k = 0; k < ii; ++k) sum = fmaf(Al[c0 + ii][c0 + k], x[k], sum);
          v = -sum * rsq[c0 + ii];
        }
        x[ii] = v;
      }
#pragma unroll
      for (int ii = 0; ii < kDfSub; ++ii)
        if (ii < cw) Ah[c0 + ii][c0 + c] = x[ii];
    }
  }
  __syncthreads();
  // off-diagonal blocks by distance dd: T = sum_k L_(bi,k) X_(k,bj), then X_(bi,bj) = -X_(bi,bi) T
  float* Tb = &Sh[0][0];  // up to 3 x 256 products
  for (int dd = 1; dd < nsb; ++dd) {
    const int np = nsb - dd;
    for (int e = tid; e < np * 256; e += 256) {
      const int pidx = e >> 8, r = (e >> 4) & 15, c = e & 15;
      const int bi = dd + pidx, bj = pidx;
      const int i = bi * kDfSub + r;
      float sum = 0.0f;
      if (i < w)
        for (int k = bj * kDfSub; k < bi * kDfSub; ++k) sum = fmaf(Al[i][k], Ah[k][bj * kDfSub + c], sum);
      Tb[e] = sum;
    }
    __syncthreads();
    for (int e = tid; e < np * 256; e += 256) {
      const int pidx = e >> 8, r = (e >> 4) & 15, c = e & 15;
      const int bi = dd + pidx, bj = pidx;
      const int i = bi * kDfSub + r;
      if (i < w) {
        float sum = 0.0f;
        for (int rr = 0; rr <= r; ++rr) sum = fmaf(Ah[i][bi * kDfSub + rr], Tb[(pidx << 8) + (rr << 4) + c], sum);
        Ah[i][bj * kDfSub + c] = -sum;
      }
    }
    __syncthreads();
  }
  if (tid < 32) {
    double sum = 0.0;
    for (int j = tid; j < w; j += 32) sum += 0.5 * log(double(dph[j]) + double(dpl[j]));
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (tid == 0) {
      logpiv[blockIdx.x] = sum;
      if (bad) atomicCAS(err, -1, tk.front);
    }
  }
  float* dvp = dinv + tk.dinv;
  for (int e = tid; e < w * w; e += 256) {
    const int i = e / w, c = e - i * w;
    dvp[int64_t(i) * kMaxNbk + c] = c <= i ? Ah[i][c] : 0.0f;
  }
}

template <typename T>
void launch_potrf(const DiagTask* tasks, int ntasks, T* L, T* dinv, double* logpiv, int* err, cudaStream_t st) {
  if (ntasks <= 0) return;
  if constexpr (sizeof(T) == sizeof(float)) {
    potrf_df_kernel<<<ntasks, 256, 0, st>>>(tasks, L, dinv, logpiv, err);
  } else {
    potrf_kernel<T><<<ntasks, 256, 0, st>>>(tasks, L, dinv, logpiv, err);
  }
}
template void launch_potrf<double>(const DiagTask*, int, double*, double*, double*, int*, cudaStream_t);
template void launch_potrf<float>(const DiagTask*, int, float*, float*, double*, int*, cudaStream_t);

// ------------------------------------------------------------- extend-add
// Adds the lower triangle of a child's update block into its parent's front:
// columns inside the parent separator go to the parent panel P, the rest to the
// parent's own update block U.  One launch per child rank, so no two blocks of
// a launch touch the same parent entry.  A task is a range of the child's rows
// [r0, r1) (more rows when they are short); the row map entries rm[0 .. r1) that
// its rows use as column targets are staged in shared memory first (up to
// kExtendSmemRows of them, else read from global memory), so that the
// read-modify-write of each element waits on one global load, not two.
constexpr int kExtendSmemRows = 12288;  // 48 KB of row map per block

template <typename T>
__global__ void __launch_bounds__(256) extend_add_kernel(const ExtendTask* __restrict__ tasks,
                                                         const DevFront* __restrict__ fronts,
                                                         const int* __restrict__ rmap, const T* __restrict__ Uc,
                                                         T* __restrict__ L, T* __restrict__ Up) {
  extern __shared__ int srm[];
  const ExtendTask tk = tasks[blockIdx.x];
  const DevFront c = fronts[tk.child];
  const DevFront p = fronts[c.parent];
  const int* rm = rmap + c.b_off;
  const bool staged = tk.r1 <= kExtendSmemRows;
  if (staged)
    for (int e = threadIdx.x; e < tk.r1; e += blockDim.x) srm[e] = rm[e];
  __syncthreads();
  const int* cm = staged ? srm : rm;
  const T* U = Uc + c.u_off;
  T* P = L + p.p_off;
  T* Upar = Up + p.u_off;
  // one warp per row (rows r0 + warp, r0 + warp + 8, ...), eight elements in
  // flight per lane; row i adds its lower part j <= i into the parent's row rm[i]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = tk.r0 + warp; i < tk.r1; i += 8) {
    const int pi = cm[i];
    const T* urow = U + int64_t(i) * c.ldu;
    T* prow = P + int64_t(pi) * p.ld;
    // pj >= ns implies pi >= ns (rm increases and j <= i): the parent's update block
    T* urw = pi >= p.ns ? Upar + int64_t(pi - p.ns) * p.ldu : nullptr;
    auto target = [&](int pj) -> T* { return pj < p.ns ? prow + pj : urw + (pj - p.ns); };
    int j = lane;
    for (; j + 224 <= i; j += 256) {
      T v[8];
      T* d[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        v[u] = urow[j + 32 * u];
        d[u] = target(cm[j + 32 * u]);
      }
      T o[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) o[u] = *d[u];
#pragma unroll
      for (int u = 0; u < 8; ++u) *d[u] = o[u] + v[u];
    }
    for (; j <= i; j += 32) {
      T* d = target(cm[j]);
      *d += urow[j];
    }
  }
}

template <typename T>
void launch_extend_add(const ExtendTask* tasks, int ntasks, const DevFront* fronts, const int* rmap, const T* U_child,
                       T* L, T* U_parent, int max_r1, cudaStream_t st) {
  if (ntasks <= 0) return;
  const size_t smem = size_t(max_r1 <= kExtendSmemRows ? max_r1 : 0) * sizeof(int);
  extend_add_kernel<T><<<ntasks, 256, smem, st>>>(tasks, fronts, rmap, U_child, L, U_parent);
}
template void launch_extend_add<double>(const ExtendTask*, int, const DevFront*, const int*, const double*, double*,
                                        double*, int, cudaStream_t);
template void launch_extend_add<float>(const ExtendTask*, int, const DevFront*, const int*, const float*, float*,
                                       float*, int, cudaStream_t);

}  // namespace spde
