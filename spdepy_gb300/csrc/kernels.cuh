// Kernel launch interfaces shared by the CUDA translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace spde {

// One output tile of a batched product C (op)= A * B' over K.
// A is addressed as A[i*lda + k] (arow) or A[k*lda + i] (acol);
// B as B[j*ldb + k] (brow) or B[k*ldb + j] (bcol).  Offsets are in elements
// relative to the base pointers passed at launch.
struct GemmTask {
  int64_t a, b, c;
  int lda, ldb, ldc;
  int m, n, k;
  // cluster-pair tasks (256 x 256 tiles, tc_gemm.cu): tensor-map index of the
  // A / B operand (-1: loaded by cp.async) and the TMA coordinates (column,
  // row) of the task's first element in that map
  int amap = -1, bmap = -1;
  int ax = 0, ay = 0, bx = 0, by = 0;
  int pair = 0;
};

enum GemmMode { kSub = 0, kStore = 1, kNegStore = 2, kAdd = 3 };
enum GemmLayout { kRow = 0, kCol = 1 };

// Diagonal-block task: factor the w x w block at `a` (row stride lda) in place,
// write its inverse to `dinv` (row stride nbk), record sum(log pivot).
struct DiagTask {
  int64_t a;
  int64_t dinv;
  int lda;
  int w;
  int front;
};

// Extend-add task: rows [r0, r1) of a child's update block.
struct ExtendTask {
  int child;
  int r0, r1;
};

struct DevFront {
  int64_t p_off, u_off, z_off, b_off, d_off;
  int64_t w_base;  // offset (per right-hand side) of this front's solve vectors in its depth pool
  int s0, ns, nb, ld, ldu, ldz, parent, depth;
  int child[2];
};

// product paths: CUDA-core tiles, tensor-core tiles (FP32 only), narrow (n <= 8
// columns), panel solve (FP32: m <= 128, n <= 64, k <= 64; CUDA-core tiles
// otherwise), 256 x 256 tiles on a cluster pair of tensor-core CTAs (FP32)
enum GemmPath { kPathSimt = 0, kPathTensor = 1, kPathNarrow = 2, kPathPanel = 3, kPathPair = 4 };
constexpr int kPairTile = 256;
// default wall-clock limit of every bounded wait in the tensor-core kernels
constexpr unsigned long long kTcWaitNs = 2000000000ull;
constexpr int kNarrowMaxN = 8;

// nmax bounds the tasks' n on the narrow path (1 selects the one-column kernel).
template <typename T>
void launch_gemm(const GemmTask* tasks, int ntasks, const T* A, const T* B, T* C, int mode, int alayout,
                 int blayout, cudaStream_t st, int path = kPathTensor, int nmax = kNarrowMaxN,
                 unsigned long long wait_ns = kTcWaitNs);

// tcgen05 path for FP32 (tc_gemm.cu); tc_gemm_take_error returns and clears the
// bounded-wait error flag of that kernel, read through `pinned` (page-locked host
// memory, so that the copy does not serialise with other host threads' copies).
void launch_gemm_tc(const GemmTask* tasks, int ntasks, const float* A, const float* B, float* C, int mode, int al,
                    int bl, cudaStream_t st, unsigned long long wait_ns = kTcWaitNs);
// cluster-pair path (row-major A and B): one 2-CTA cluster per 256 x 256 task
void launch_gemm_pair(const GemmTask* tasks, int ntasks, const CUtensorMap* maps, const float* A, const float* B,
                      float* C, int mode, cudaStream_t st, unsigned long long wait_ns = kTcWaitNs);
int tc_gemm_take_error(cudaStream_t st, int* pinned);
bool tc_gemm_enabled();

template <typename T>
void launch_potrf(const DiagTask* tasks, int ntasks, T* L, T* dinv, double* logpiv, int* err, cudaStream_t st);

template <typename T>
void launch_extend_add(const ExtendTask* tasks, int ntasks, const DevFront* fronts, const int* rmap, const T* U_child,
                       T* L, T* U_parent, int max_r1, cudaStream_t st);

}  // namespace spde
