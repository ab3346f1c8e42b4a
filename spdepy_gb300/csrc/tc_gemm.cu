// Tiled product on the 5th-generation tensor cores (tcgen05) for FP32 fronts.
//
// One CTA computes one 128 x 128 output tile of C (op)= A B' (the GemmTask
// contract of dense.cu).  The accumulator lives in tensor memory (128 TMEM
// columns, FP32).  K advances in chunks of 32 FP32 values staged by cp.async
// straight into 128-byte-swizzled K-major shared-memory tiles, two chunks ahead
// of the tensor core (four raw stages).  The tensor core reads a raw FP32 tile as
// TF32 (it drops the 13 low mantissa bits: hi = trunc(x)); the threads write the
// exact residual x - hi, rounded to TF32, into a second plane, and one elected
// thread issues, per 8-wide k step, hi*hi + hi*lo + lo*hi (the lo*lo term,
// ~2^-21 relative, is dropped), which gives FP32-class products.
// Warps 0-3 stage, convert and write back; warp 4 issues the MMAs; they hand
// stages over through mbarriers (tcgen05.commit arrives when MMAs finish).
// Every wait is bounded by a wall-clock limit, after which the CTA records an
// error, frees its tensor memory and returns.
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace spde {

namespace {

constexpr int kTM = 128, kTN = 128, kTK = 32;
constexpr int kConv = 128;                 // loader / converter / epilogue threads (warps 0-3)
constexpr int kThreads = kConv + 32;       // + one MMA warp
constexpr int kPlane = 128 * 32 * 4;       // one 128 x 32 FP32 operand plane (16 KB)
constexpr int kStages = 3;                 // stage = raw A, raw B, residual A, residual B
constexpr int kStageBytes = 4 * kPlane;
constexpr int kSmem = kStages * kStageBytes + 1024;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// The tensor core reads a 32-bit operand as TF32 by dropping its 13 low mantissa
// bits; the residual x - trunc(x) is exact in FP32 and is fed rounded to TF32.
__device__ __forceinline__ float tf32_resid(float x) {
  const float hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  return tf32_rna(x - hi);
}

// byte offset of the 16-byte chunk c4 (k = 4 c4 .. 4 c4 + 3) of row r inside a
// 128 x 32 FP32 K-major tile with the 128-byte swizzle
__device__ __forceinline__ uint32_t sw_chunk(int r, int c4) {
  return uint32_t((r >> 3) * 1024 + (r & 7) * 128 + (((c4 ^ r) & 7) << 4));
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;            // leading byte offset (unused with the 128-byte swizzle)
  d |= uint64_t(1024 >> 4) << 32;    // stride byte offset
  d |= uint64_t(1) << 46;            // descriptor version
  d |= uint64_t(2) << 61;            // 128-byte swizzle
  return d;
}

// instruction descriptor: D F32, A/B TF32, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t(kTN) >> 3) << 17) |
                            ((uint32_t(kTM) >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stage one raw 128 x 32 FP32 chunk of an operand into the swizzled tile `dst`
// (zero outside rows < rows, k < K).  Thread `tid` of the kConv loader threads
// owns the 16-byte chunks q = tid + i * kConv; row layout with 16-byte aligned
// rows goes through cp.async, other layouts through registers.
template <int LAYOUT>
__device__ __forceinline__ void stage_raw(const float* X, int64_t ld, int rows, int k0, int K, bool vec, uint8_t* dst,
                                          int tid) {
  if (LAYOUT == kRow && vec) {
    const uint32_t d0 = smem_u32(dst);
#pragma unroll
    for (int it = 0; it < 1024 / kConv; ++it) {
      const int q = tid + it * kConv;
      const int r = q >> 3, c4 = q & 7;
      const int k = k0 + 4 * c4;
      int bytes = 0;
      const float* src = X;
      if (r < rows && k < K) {
        bytes = 4 * min(4, K - k);
        src = X + int64_t(r) * ld + k;
      }
      cp_async16(d0 + sw_chunk(r, c4), src, bytes);
    }
  } else if (LAYOUT == kRow) {
#pragma unroll 2
    for (int it = 0; it < 1024 / kConv; ++it) {
      const int q = tid + it * kConv;
      const int r = q >> 3, c4 = q & 7;
      const int k = k0 + 4 * c4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < rows) {
        const float* p = X + int64_t(r) * ld + k;
        if (k < K) v.x = p[0];
        if (k + 1 < K) v.y = p[1];
        if (k + 2 < K) v.z = p[2];
        if (k + 3 < K) v.w = p[3];
      }
      *reinterpret_cast<float4*>(dst + sw_chunk(r, c4)) = v;
    }
  } else {
    // column layout: element (row r, k) at X[k*ld + r]; loads along r
#pragma unroll 2
    for (int it = 0; it < 1024 / kConv; ++it) {
      const int q = tid + it * kConv;
      const int i4 = q & 31, kk = q >> 5;
      const int k = k0 + kk;
      const int r0 = 4 * i4;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (k < K) {
        const float* p = X + int64_t(k) * ld + r0;
        if (vec && r0 + 3 < rows) {
          float4 t = *reinterpret_cast<const float4*>(p);
          v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (r0 + e < rows) v[e] = p[e];
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e)
        *reinterpret_cast<float*>(dst + sw_chunk(r0 + e, kk >> 2) + ((kk & 3) << 2)) = v[e];
    }
  }
}

// Residual planes of one stage.  With cp.async staging every thread converts
// exactly the chunks it copied (its own completed copies are all it needs);
// register-staged layouts are followed by a loader-wide barrier first.
__device__ __forceinline__ void split_stage(const uint8_t* raw, uint8_t* lo, int tid) {
#pragma unroll
  for (int plane = 0; plane < 2; ++plane)
#pragma unroll
    for (int it = 0; it < 1024 / kConv; ++it) {
      const int q = tid + it * kConv;
      const int r = q >> 3, c4 = q & 7;
      const uint32_t off = uint32_t(plane * kPlane) + sw_chunk(r, c4);
      float4 v = *reinterpret_cast<const float4*>(raw + off);
      *reinterpret_cast<float4*>(lo + off) =
          make_float4(tf32_resid(v.x), tf32_resid(v.y), tf32_resid(v.z), tf32_resid(v.w));
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Barrier among the loader warps only (id 1, kConv threads) that also ANDs a
// flag, so a failed wait ends the loop for every loader thread together.
__device__ __forceinline__ bool loader_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\tbar.red.and.pred po, 1, %2, pi;\n\t"
      "selp.u32 %0, 1, 0, po;\n\t}\n"
      : "=r"(r)
      : "r"(uint32_t(v)), "n"(kConv)
      : "memory");
  return r != 0;
}

template <int MODE, int AL, int BL>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_kernel(const GemmTask* __restrict__ tasks, const float* Ab,
                                                              const float* Bb, float* Cb) {
  // Warps 0-3 stage chunks (cp.async), write the residual planes and run the
  // epilogue; warp 4 issues the MMAs.  Per stage s: `ready[s]` (kConv arrivals)
  // says the stage is converted, `free_[s]` (tcgen05.commit) says its MMAs are
  // done; `done` follows the last MMA.
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t ready[kStages], free_[kStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const GemmTask tk = tasks[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* A = Ab + tk.a;
  const float* B = Bb + tk.b;
  float* C = Cb + tk.c;
  const bool avec = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && ((tk.lda & 3) == 0);
  const bool bvec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && ((tk.ldb & 3) == 0);
  const bool async_a = AL == kRow && avec, async_b = BL == kRow && bvec;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&ready[s])), "r"(kConv));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&free_[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const int nk = (tk.k + kTK - 1) / kTK;

  auto wait = [&](uint64_t* bar, uint32_t parity) -> bool {
    if (mbar_try(smem_u32(bar), parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_try(smem_u32(bar), parity)) {
      if (*(volatile int*)&abort_flag) return false;
      if (now_ns() - t0 > kWaitNs) {
        atomicExch(&abort_flag, 1);
        return false;
      }
    }
    return true;
  };

  if (warp < 4) {
    // ---------------- loaders / converters
    for (int t = 0; t < 2 && t < nk; ++t) {
      uint8_t* st = smem + t * kStageBytes;
      stage_raw<AL>(A, tk.lda, tk.m, t * kTK, tk.k, avec, st, tid);
      stage_raw<BL>(B, tk.ldb, tk.n, t * kTK, tk.k, bvec, st + kPlane, tid);
      cp_async_commit();
    }
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      uint8_t* st = smem + s * kStageBytes;
      if (t + 1 < nk) cp_async_wait<1>(); else cp_async_wait<0>();
      if (!(async_a && async_b) && !loader_all(true)) break;
      split_stage(st, st + 2 * kPlane, tid);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(smem_u32(&ready[s]));
      if (t + 2 < nk) {
        const int s2 = (t + 2) % kStages;  // last used by chunk t - 1
        const bool ok = t < 1 || wait(&free_[s2], uint32_t(((t - 1) / kStages) & 1));
        if (async_a && async_b) {
          if (!ok) break;
        } else if (!loader_all(ok)) {
          break;
        }
        uint8_t* st2 = smem + s2 * kStageBytes;
        stage_raw<AL>(A, tk.lda, tk.m, (t + 2) * kTK, tk.k, avec, st2, tid);
        stage_raw<BL>(B, tk.ldb, tk.n, (t + 2) * kTK, tk.k, bvec, st2 + kPlane, tid);
      }
      cp_async_commit();
    }
    cp_async_wait<0>();
    const bool ok = nk == 0 || wait(&done, 0u);
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int row = warp * 32 + lane;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int col0 = c * 32;
        uint32_t r[32];
        const uint32_t ta = tmem + (uint32_t(warp * 32) << 16) + uint32_t(col0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < tk.m && nk > 0 && col0 < tk.n) {
          float* dst = C + int64_t(row) * tk.ldc + col0;
          const bool v4 = ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) && col0 + 32 <= tk.n;
          if (v4) {
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
              float4 v = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                                     __uint_as_float(r[j + 3]));
              float4* d4 = reinterpret_cast<float4*>(dst + j);
              if (MODE == kStore) { *d4 = v; }
              else if (MODE == kNegStore) { *d4 = make_float4(-v.x, -v.y, -v.z, -v.w); }
              else {
                float4 o = *d4;
                if (MODE == kSub) *d4 = make_float4(o.x - v.x, o.y - v.y, o.z - v.z, o.w - v.w);
                else *d4 = make_float4(o.x + v.x, o.y + v.y, o.z + v.z, o.w + v.w);
              }
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (col0 + j >= tk.n) break;
              const float v = __uint_as_float(r[j]);
              if (MODE == kSub) dst[j] -= v;
              else if (MODE == kStore) dst[j] = v;
              else if (MODE == kNegStore) dst[j] = -v;
              else dst[j] += v;
            }
          }
        }
      }
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      if (!wait(&ready[s], uint32_t((t / kStages) & 1))) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ra = smem_u32(smem + s * kStageBytes), la = ra + 2 * kPlane;
#pragma unroll
      for (int kk = 0; kk < kTK / 8; ++kk) {
        const uint64_t ah = smem_desc(ra + kk * 32), bh = smem_desc(ra + kPlane + kk * 32);
        const uint64_t al = smem_desc(la + kk * 32), bl = smem_desc(la + kPlane + kk * 32);
        mma_tf32(tmem, ah, bh, (t > 0 || kk > 0) ? 1u : 0u);
        mma_tf32(tmem, ah, bl, 1u);
        mma_tf32(tmem, al, bh, 1u);
      }
      mma_commit(smem_u32(&free_[s]));
    }
    if (nk > 0) mma_commit(smem_u32(&done));
  }
  __syncthreads();
  if (tid == 0 && abort_flag) atomicExch(&g_tc_error, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

template <int MODE, int AL, int BL>
void launch_one(const GemmTask* t, int n, const float* A, const float* B, float* C, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(tc_gemm_kernel<MODE, AL, BL>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    attr = true;
  }
  tc_gemm_kernel<MODE, AL, BL><<<n, kThreads, kSmem, st>>>(t, A, B, C);
}

template <int MODE>
void launch_mode(const GemmTask* t, int n, const float* A, const float* B, float* C, int al, int bl, cudaStream_t st) {
  if (al == kRow && bl == kRow) launch_one<MODE, kRow, kRow>(t, n, A, B, C, st);
  else if (al == kRow) launch_one<MODE, kRow, kCol>(t, n, A, B, C, st);
  else if (bl == kRow) launch_one<MODE, kCol, kRow>(t, n, A, B, C, st);
  else launch_one<MODE, kCol, kCol>(t, n, A, B, C, st);
}

}  // namespace

void launch_gemm_tc(const GemmTask* tasks, int ntasks, const float* A, const float* B, float* C, int mode, int al,
                    int bl, cudaStream_t st) {
  if (ntasks <= 0) return;
  switch (mode) {
    case kSub: launch_mode<kSub>(tasks, ntasks, A, B, C, al, bl, st); break;
    case kStore: launch_mode<kStore>(tasks, ntasks, A, B, C, al, bl, st); break;
    case kNegStore: launch_mode<kNegStore>(tasks, ntasks, A, B, C, al, bl, st); break;
    default: launch_mode<kAdd>(tasks, ntasks, A, B, C, al, bl, st); break;
  }
}

int tc_gemm_take_error() {
  int h = 0, z = 0;
  cudaMemcpyFromSymbol(&h, g_tc_error, sizeof(int));
  if (h) cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
  return h;
}

}  // namespace spde
