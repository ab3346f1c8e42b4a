// Tiled product on the 5th-generation tensor cores (tcgen05) for FP32 fronts.
//
// One CTA computes one 128 x 128 output tile of C (op)= A B' (the GemmTask
// contract of dense.cu).  The accumulator lives in tensor memory (TMEM columns
// 0-127, FP32).  K advances in chunks of 32 FP32 values staged by cp.async into
// 128-byte-swizzled K-major shared-memory tiles, three chunks ahead of the tensor
// core (four stages).  Each product runs as 3xTF32: the tensor core reads
// operands as TF32, so every operand is split (Veltkamp) into an 11-bit hi part
// and the exact remainder lo, and one elected thread issues, per 8-wide k step,
// hi*hi + hi*lo + lo*hi (the lo*lo term, under 2^-24 relative, is dropped),
// which gives FP32-class products.
//
// Operand A goes to the tensor core from TMEM: two threads of the eight
// converter warps own row r of the tile (TMEM lane r), read its 32 raw values of
// the chunk from shared memory and store hi and lo with tcgen05.st into the
// stage's 64-column TMEM slot.  Operand B is read by the tensor core from shared
// memory: its raw plane rewritten as hi, plus a residual plane.
// Roles: four loader warps issue cp.async copies whose completion arrives on an
// mbarrier, eight converter warps split the operands and later run the
// epilogue, one thread issues the MMAs; stages pass between them through
// mbarriers (tcgen05.commit arrives when a stage's MMAs finish), so loads,
// conversions and MMAs of different stages overlap.
// Every wait is bounded by a wall-clock limit, after which the CTA records an
// error, waits for its issued MMAs, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace spde {

namespace {

constexpr int kTM = 128, kTN = 128, kTK = 32;
constexpr int kConv = 256;                 // converter / epilogue threads (warps 0-7)
constexpr int kGroups = 1;                 // converter groups (group g takes chunks t = g mod kGroups)
constexpr int kLoad = 128;                 // loader threads (warps 8-11)
constexpr int kThreads = kGroups * kConv + kLoad + 32;  // + one MMA warp (warp 12)
constexpr int kEpiCols = 128 / (kGroups * kConv / 128);  // accumulator columns per epilogue warp
constexpr int kPlane = 128 * 32 * 4;       // one 128 x 32 FP32 operand plane (16 KB)
constexpr int kStages = 4;                 // stage = raw A, raw B, residual B
constexpr int kStageBytes = 3 * kPlane;
constexpr int kSmem = kStages * kStageBytes + 1024;
constexpr int kASlot0 = 128, kASlotCols = 64;  // TMEM: accumulator 0-127, A slot s at 128 + 64 s
constexpr int kTmemCols = 512;             // power of two >= 128 + kStages * 64
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
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

// D (TMEM) (+)= A (TMEM, lane = row, one column per k) * B (shared memory descriptor)
__device__ __forceinline__ void mma_tf32_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(b), "r"(kIdesc), "r"(acc));
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
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
// the mbarrier receives one arrival when every cp.async this thread issued so far has landed
__device__ __forceinline__ void cp_async_arrive(uint32_t mbar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Stage one raw 128 x 32 FP32 chunk of an operand into the swizzled tile at
// shared address d0 (zero outside rows < rows, k < K) with cp.async: loader
// thread `tid` of NT copies 16-byte chunks q = tid + i NT when rows are 16-byte
// aligned (row layout), single elements otherwise (column layout along r).
template <int LAYOUT, int NT>
__device__ __forceinline__ void stage_async(const float* X, int64_t ld, int rows, int k0, int K, bool vec, uint32_t d0,
                                            int tid) {
  if (LAYOUT == kRow && vec) {
#pragma unroll
    for (int it = 0; it < 1024 / NT; ++it) {
      const int q = tid + it * NT;
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
#pragma unroll 4
    for (int it = 0; it < 4096 / NT; ++it) {
      const int e = tid + it * NT;
      const int r = e >> 5, kk = e & 31, k = k0 + kk;
      const bool ok = r < rows && k < K;
      cp_async4(d0 + sw_chunk(r, kk >> 2) + ((kk & 3) << 2), ok ? X + int64_t(r) * ld + k : X, ok ? 4 : 0);
    }
  } else {
#pragma unroll 4
    for (int it = 0; it < 4096 / NT; ++it) {
      const int e = tid + it * NT;
      const int r = e & 127, kk = e >> 7, k = k0 + kk;
      const bool ok = r < rows && k < K;
      cp_async4(d0 + sw_chunk(r, kk >> 2) + ((kk & 3) << 2), ok ? X + int64_t(k) * ld + r : X, ok ? 4 : 0);
    }
  }
}

// Veltkamp split of an FP32 value for the tensor core: hi = x (2^13 + 1) -
// (x (2^13 + 1) - x) keeps the 11 leading significant bits (round to nearest),
// so it is exact in TF32, and lo = x - hi is exact in FP32 with |lo| <= 2^-12 |x|;
// the tensor core drops lo's bits below TF32, an error under 2^-22 |x|.  Only
// FP32 adds and multiplies (the _rn forms keep them from being contracted).
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  const float t = __fmul_rn(x, 8193.0f);
  hi = __fsub_rn(t, __fsub_rn(t, x));
  lo = __fsub_rn(x, hi);
}

// Operand B of one stage: the raw plane is rewritten as its hi part, the lo
// part goes to the residual plane; converter thread `tid` takes the 16-byte
// chunks q = tid + i * kConv.
__device__ __forceinline__ void split_b(uint8_t* raw, uint8_t* lo, int tid) {
#pragma unroll
  for (int it = 0; it < 1024 / kConv; ++it) {
    const int q = tid + it * kConv;
    const uint32_t off = sw_chunk(q >> 3, q & 7);
    const float4 v = *reinterpret_cast<const float4*>(raw + off);
    float4 h, l;
    split_tf32(v.x, h.x, l.x);
    split_tf32(v.y, h.y, l.y);
    split_tf32(v.z, h.z, l.z);
    split_tf32(v.w, h.w, l.w);
    *reinterpret_cast<float4*>(raw + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]) : "memory");
}

// Half `h` (k = 16 h .. 16 h + 15) of row `row` of the raw A plane into TMEM lane
// `row`: hi = trunc(x) in columns col + 16 h .., lo = rna(x - hi) in col + 32 + 16 h ..
__device__ __forceinline__ void a_to_tmem(const uint8_t* raw, int row, int h, uint32_t taddr) {
  uint32_t hi[16], lo[16];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float4 v = *reinterpret_cast<const float4*>(raw + sw_chunk(row, 4 * h + c));
    const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float h, l;
      split_tf32(x[e], h, l);
      hi[4 * c + e] = __float_as_uint(h);
      lo[4 * c + e] = __float_as_uint(l);
    }
  }
  tmem_st16(taddr + 16 * h, hi);
  tmem_st16(taddr + 32 + 16 * h, lo);
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

template <int MODE, int AL, int BL>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_kernel(const GemmTask* __restrict__ tasks, const float* Ab,
                                                              const float* Bb, float* Cb, unsigned long long wait_ns) {
  // Three roles hand chunk t (stage s = t % kStages) along through mbarriers:
  //   loaders (warps 8-11): wait consumed[s] (MMAs of chunk t - kStages done),
  //     issue the cp.async copies of A and B, arrive on full[s] when they land;
  //   converters (warps 0-7): wait full[s], write A hi/lo into TMEM slot s and
  //     the B hi/lo planes, arrive on ready[s]; afterwards they run the epilogue;
  //   MMA issuer (warp 12, one lane): wait ready[s], issue the chunk's 12 MMAs,
  //     commit to consumed[s]; a final commit arrives on done.
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kStages], ready[kStages], consumed[kStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag, mma_issued;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const GemmTask tk = tasks[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* A = Ab + tk.a;
  const float* B = Bb + tk.b;
  float* C = Cb + tk.c;
  const bool avec = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && ((tk.lda & 3) == 0);
  const bool bvec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && ((tk.ldb & 3) == 0);

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[s])), "r"(kLoad));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&ready[s])), "r"(kConv));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&consumed[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    mma_issued = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const int nk = (tk.k + kTK - 1) / kTK;

  // bounded wait (wait_ns for the pipeline's waits; the clean-up below always
  // allows kWaitNs); with `honor_abort` it also gives up as soon as another
  // thread of the CTA has recorded a failure
  auto wait = [&](uint64_t* bar, uint32_t parity, bool honor_abort, unsigned long long limit) -> bool {
    if (mbar_try(smem_u32(bar), parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_try(smem_u32(bar), parity)) {
      if (honor_abort && *(volatile int*)&abort_flag) return false;
      if (now_ns() - t0 > limit) {
        atomicExch(&abort_flag, 1);
        return false;
      }
    }
    return true;
  };

  if (warp < kGroups * kConv / 32) {
    // ---------------- converters (two groups on alternate chunks), then the epilogue
    const int g = tid / kConv, ct = tid - g * kConv;
    for (int t = g; t < nk; t += kGroups) {
      const int s = t % kStages;
      if (!wait(&full[s], uint32_t((t / kStages) & 1), true, wait_ns)) break;
      uint8_t* st = smem + s * kStageBytes;
      // warp w reaches TMEM lanes 32 (w % 4) ..; the group's warps 0-3 take k 0-15, warps 4-7 k 16-31
      a_to_tmem(st, ct & 127, ct >> 7,
                tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(kASlot0 + s * kASlotCols));
      split_b(st + kPlane, st + 2 * kPlane, ct);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(smem_u32(&ready[s]));
    }
    const bool fin = nk == 0 || wait(&done, 0u, true, wait_ns);
    if (fin) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      // warp w reads lanes 32 (w % 4) .. and accumulator columns kEpiCols (w / 4) ..
      const int row = (warp & 3) * 32 + lane;
#pragma unroll
      for (int c = 0; c < kEpiCols / 32; ++c) {
        const int col0 = (warp >> 2) * kEpiCols + c * 32;
        uint32_t r[32];
        const uint32_t ta = tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(col0);
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
  } else if (warp < (kGroups * kConv + kLoad) / 32) {
    // ---------------- loaders
    const int ltid = tid - kGroups * kConv;
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      // stage s last held chunk t - kStages, read by its MMAs (B) and converters (A)
      if (t >= kStages && !wait(&consumed[s], uint32_t(((t - kStages) / kStages) & 1), true, wait_ns)) break;
      const uint32_t d0 = smem_u32(smem + s * kStageBytes);
      stage_async<AL, kLoad>(A, tk.lda, tk.m, t * kTK, tk.k, avec, d0, ltid);
      stage_async<BL, kLoad>(B, tk.ldb, tk.n, t * kTK, tk.k, bvec, d0 + kPlane, ltid);
      cp_async_arrive(smem_u32(&full[s]));
    }
    cp_async_wait_all();
  } else if (lane == 0) {
    // ---------------- MMA issuer
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      if (!wait(&ready[s], uint32_t((t / kStages) & 1), true, wait_ns)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t rb = smem_u32(smem + s * kStageBytes + kPlane), lb = rb + kPlane;
      const uint32_t ah = tmem + uint32_t(kASlot0 + s * kASlotCols), al = ah + 32;
#pragma unroll
      for (int kk = 0; kk < kTK / 8; ++kk) {
        const uint64_t bh = smem_desc(rb + kk * 32), bl = smem_desc(lb + kk * 32);
        mma_tf32_ts(tmem, ah + kk * 8, bh, (t > 0 || kk > 0) ? 1u : 0u);
        mma_tf32_ts(tmem, ah + kk * 8, bl, 1u);
        mma_tf32_ts(tmem, al + kk * 8, bh, 1u);
      }
      mma_commit(smem_u32(&consumed[s]));
      mma_issued = 1;
    }
    // `done` tracks every MMA issued, also after a failure, so the clean-up can
    // wait for them before the tensor memory is freed
    if (mma_issued) mma_commit(smem_u32(&done));
  }
  __syncthreads();
  if (tid == 0 && abort_flag) {
    atomicExch(&g_tc_error, 1);
    if (mma_issued) wait(&done, 0u, false, kWaitNs);  // the fixed limit: MMAs must finish before dealloc
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
}

// ---------------------------------------------------------------------------
// Pair kernel: a cluster of two CTAs on two SMs computes one 256 x 256 output
// tile with tcgen05.mma.cta_group::2 (M = 256, N = 256).  CTA r of the pair owns
// rows 128 r .. 128 r + 127 of the tile: its slice of A (in its own TMEM, split
// hi / lo by its converters), its half of B (columns 128 r .. of the tile, hi and
// lo planes in its own shared memory) and its half of the accumulator (TMEM
// lanes 0-127, 256 columns).  Each SM therefore converts the same operand bytes
// per k step as a 128 x 128 tile but feeds twice the tensor-core work.
//
// Operands whose rows are 16-byte aligned arrive by TMA (cp.async.bulk.tensor,
// one 32 x 128 FP32 box per plane and stage, 128-byte swizzle) from tensor maps
// built for the task's front; the others by cp.async as in the single-CTA
// kernel.  The converters zero every k >= K of the last chunk, so a box may
// read past the task's K range.
//
// Two groups of eight converter warps take alternate chunks, so that two
// chunks are split at a time (one group's split latency no longer bounds the
// tensor core); both groups then share the epilogue, 64 accumulator columns per
// warp.  Only the even CTA issues MMAs.  The converter warps that took chunk t
// in both CTAs arrive on its ready[s] (16 arrivals: 8 warps x 2 CTAs); its
// tcgen05.commit arrives on
// consumed[s] and, after the last chunk, on done in both CTAs.  Neither CTA
// frees its tensor memory or exits before the pair's MMAs are done (a wait on
// done, then a cluster barrier), also after a failed (timed-out) wait.
constexpr int kPairASlot0 = 256;  // TMEM: accumulator columns 0-255, A slot s at 256 + 64 s
constexpr int kPairGroups = 2;     // converter groups of the pair kernel (group g takes chunks t = g mod 2)
constexpr int kPairThreads = kPairGroups * kConv + kLoad + 32;  // warps 0-15 converters, 16-19 loaders, 20 MMA
constexpr int kPairEpiCols = 256 / (kPairGroups * kConv / 128);  // accumulator columns per epilogue warp
constexpr uint32_t kIdescPair = (1u << 4) | (2u << 7) | (2u << 10) | ((256u >> 3) << 17) | ((256u >> 4) << 24);

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared::cluster address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_shared(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ bool mbar_try_cluster(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// 2-D TMA load of one box at (x, y) into shared memory; completion is counted on mbar
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void mma_tf32_pair(uint32_t tmem_d, uint32_t tmem_a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(b), "r"(kIdescPair), "r"(acc));
}
// arrives on the mbarrier at shared::cluster address `mbar` (this CTA's or the
// peer's) when every MMA this thread issued so far has completed
__device__ __forceinline__ void mma_commit_pair(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// a_to_tmem / split_b with every k >= kvalid of the chunk set to zero (last chunk)
__device__ __forceinline__ void a_to_tmem_masked(const uint8_t* raw, int row, int h, uint32_t taddr, int kvalid) {
  uint32_t hi[16], lo[16];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float4 v = *reinterpret_cast<const float4*>(raw + sw_chunk(row, 4 * h + c));
    const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float xv = (16 * h + 4 * c + e < kvalid) ? x[e] : 0.0f;
      float hh, ll;
      split_tf32(xv, hh, ll);
      hi[4 * c + e] = __float_as_uint(hh);
      lo[4 * c + e] = __float_as_uint(ll);
    }
  }
  tmem_st16(taddr + 16 * h, hi);
  tmem_st16(taddr + 32 + 16 * h, lo);
}
__device__ __forceinline__ void split_b_masked(uint8_t* raw, uint8_t* lo, int tid, int kvalid) {
#pragma unroll
  for (int it = 0; it < 1024 / kConv; ++it) {
    const int q = tid + it * kConv;
    const int c4 = q & 7;
    const uint32_t off = sw_chunk(q >> 3, c4);
    float4 v = *reinterpret_cast<const float4*>(raw + off);
    const int k0 = 4 * c4;
    if (k0 + 0 >= kvalid) v.x = 0.0f;
    if (k0 + 1 >= kvalid) v.y = 0.0f;
    if (k0 + 2 >= kvalid) v.z = 0.0f;
    if (k0 + 3 >= kvalid) v.w = 0.0f;
    float4 h, l;
    split_tf32(v.x, h.x, l.x);
    split_tf32(v.y, h.y, l.y);
    split_tf32(v.z, h.z, l.z);
    split_tf32(v.w, h.w, l.w);
    *reinterpret_cast<float4*>(raw + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

template <int MODE>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kPairThreads, 1)
    tc_pair_kernel(const GemmTask* __restrict__ tasks, const CUtensorMap* __restrict__ maps, const float* Ab,
                   const float* Bb, float* Cb, unsigned long long wait_ns) {
  extern __shared__ uint8_t smem_raw[];
  // full: the loaders' cp.async arrivals; tfull: the TMA boxes (one expect_tx
  // arrival plus their bytes), kept apart so that the issuing thread can wait
  // for its own boxes alone before the CTA exits
  __shared__ uint64_t full[kStages], tfull[kStages], ready[kStages], consumed[kStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t rank = cluster_rank();
  const GemmTask tk = tasks[blockIdx.x >> 1];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = int(rank) * 128;              // this CTA's rows of A and of B within the pair tile
  const int am = tk.m - row0, bn = tk.n - row0;  // of which valid (may be <= 0)
  const float* A = Ab + tk.a + (am > 0 ? int64_t(row0) * tk.lda : 0);
  const float* B = Bb + tk.b + (bn > 0 ? int64_t(row0) * tk.ldb : 0);
  const bool avec = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && ((tk.lda & 3) == 0);
  const bool bvec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && ((tk.ldb & 3) == 0);
  const bool atma = tk.amap >= 0, btma = tk.bmap >= 0;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[s])), "r"(kLoad));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&tfull[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&ready[s])), "r"(2 * kConv / 32));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&consumed[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    // one warp of each CTA of the pair allocates, collectively, the same columns in both
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  __syncthreads();
  cluster_sync_all();  // the peer's barriers are initialised and its tensor memory allocated
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const int nk = (tk.k + kTK - 1) / kTK;

  auto wait = [&](uint64_t* bar, uint32_t parity, bool honor_abort, unsigned long long limit) -> bool {
    if (mbar_try(smem_u32(bar), parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_try(smem_u32(bar), parity)) {
      if (honor_abort && *(volatile int*)&abort_flag) return false;
      if (now_ns() - t0 > limit) {
        atomicExch(&abort_flag, 1);
        return false;
      }
    }
    return true;
  };

  if (warp < kPairGroups * kConv / 32) {
    // ---------------- converters (two groups on alternate chunks), then the epilogue
    const uint32_t lane_base = uint32_t((warp & 3) * 32) << 16;
    const int g = warp / (kConv / 32), ct = tid - g * kConv;
    for (int t = g; t < nk; t += kPairGroups) {
      const int s = t % kStages;
      if (!wait(&full[s], uint32_t((t / kStages) & 1), true, wait_ns)) break;
      if ((atma || btma) && !wait(&tfull[s], uint32_t((t / kStages) & 1), true, wait_ns)) break;
      uint8_t* st = smem + s * kStageBytes;
      const int kvalid = tk.k - t * kTK;
      const uint32_t slot = tmem + lane_base + uint32_t(kPairASlot0 + s * kASlotCols);
      if (kvalid >= kTK) {
        a_to_tmem(st, ct & 127, ct >> 7, slot);
        split_b(st + kPlane, st + 2 * kPlane, ct);
      } else {
        a_to_tmem_masked(st, ct & 127, ct >> 7, slot, kvalid);
        split_b_masked(st + kPlane, st + 2 * kPlane, ct, kvalid);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive_cluster(mapa_shared(smem_u32(&ready[s]), 0));
    }
    const bool fin = nk > 0 && wait(&done, 0u, true, wait_ns);
    if (fin) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      // warp w reads lanes 32 (w % 4) .. and accumulator columns kPairEpiCols (w / 4) ..
      const int row = (warp & 3) * 32 + lane;
      const int grow = row0 + row;
#pragma unroll 1
      for (int c = 0; c < kPairEpiCols / 32; ++c) {
        const int col0 = (warp >> 2) * kPairEpiCols + c * 32;
        uint32_t r[32];
        const uint32_t ta = tmem + lane_base + uint32_t(col0);
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
        if (grow < tk.m && col0 < tk.n) {
          float* dst = Cb + tk.c + int64_t(grow) * tk.ldc + col0;
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
  } else if (warp < (kPairGroups * kConv + kLoad) / 32) {
    // ---------------- loaders: TMA boxes (one elected thread) and / or cp.async
    const int ltid = tid - kPairGroups * kConv;
    int issued = 0;  // chunks whose TMA boxes this thread (ltid 0) issued
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      if (t >= kStages && !wait(&consumed[s], uint32_t(((t - kStages) / kStages) & 1), true, wait_ns)) break;
      const uint32_t d0 = smem_u32(smem + s * kStageBytes);
      if (ltid == 0 && (atma || btma)) {
        const uint32_t tb = smem_u32(&tfull[s]);
        mbar_expect_tx(tb, uint32_t((atma ? kPlane : 0) + (btma ? kPlane : 0)));
        if (atma) tma_load_2d(d0, maps + tk.amap, tk.ax + t * kTK, tk.ay + row0, tb);
        if (btma) tma_load_2d(d0 + kPlane, maps + tk.bmap, tk.bx + t * kTK, tk.by + row0, tb);
        issued = t + 1;
      }
      if (!atma) stage_async<kRow, kLoad>(A, tk.lda, am, t * kTK, tk.k, avec, d0, ltid);
      if (!btma) stage_async<kRow, kLoad>(B, tk.ldb, bn, t * kTK, tk.k, bvec, d0 + kPlane, ltid);
      cp_async_arrive(smem_u32(&full[s]));
    }
    cp_async_wait_all();
    // boxes still in flight (a failed wait ended the loop early) must land before
    // the CTA's shared memory goes away: wait for the last kStages chunks issued
    if (ltid == 0)
      for (int t = issued - kStages > 0 ? issued - kStages : 0; t < issued; ++t)
        wait(&tfull[t % kStages], uint32_t((t / kStages) & 1), false, kWaitNs);
  } else if (lane == 0 && rank == 0) {
    // ---------------- MMA issuer (even CTA of the pair)
    for (int t = 0; t < nk; ++t) {
      const int s = t % kStages;
      const uint32_t rb_ = smem_u32(&ready[s]);
      bool ok = mbar_try_cluster(rb_, uint32_t((t / kStages) & 1));
      if (!ok) {
        const unsigned long long t0 = now_ns();
        while (!(ok = mbar_try_cluster(rb_, uint32_t((t / kStages) & 1)))) {
          if (*(volatile int*)&abort_flag) break;
          if (now_ns() - t0 > wait_ns) {
            atomicExch(&abort_flag, 1);
            break;
          }
        }
      }
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t rb = smem_u32(smem + s * kStageBytes + kPlane), lb = rb + kPlane;
      const uint32_t ah = tmem + uint32_t(kPairASlot0 + s * kASlotCols), al = ah + 32;
#pragma unroll
      for (int kk = 0; kk < kTK / 8; ++kk) {
        const uint64_t bh = smem_desc(rb + kk * 32), bl = smem_desc(lb + kk * 32);
        mma_tf32_pair(tmem, ah + kk * 8, bh, (t > 0 || kk > 0) ? 1u : 0u);
        mma_tf32_pair(tmem, ah + kk * 8, bl, 1u);
        mma_tf32_pair(tmem, al + kk * 8, bh, 1u);
      }
      mma_commit_pair(mapa_shared(smem_u32(&consumed[s]), 0));
      mma_commit_pair(mapa_shared(smem_u32(&consumed[s]), 1));
    }
    // always: both CTAs' `done` track every MMA issued (none issued: it arrives at once)
    mma_commit_pair(mapa_shared(smem_u32(&done), 0));
    mma_commit_pair(mapa_shared(smem_u32(&done), 1));
  }
  __syncthreads();
  if (tid == 0) {
    if (abort_flag) atomicExch(&g_tc_error, 1);
    // the pair's MMAs read this CTA's shared memory and TMEM: wait for them (fixed limit)
    if (!wait(&done, 0u, false, kWaitNs)) atomicExch(&g_tc_error, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  cluster_sync_all();  // both CTAs are past the pair's MMAs before either frees its tensor memory
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
}

template <int MODE>
void launch_pair(const GemmTask* t, int n, const CUtensorMap* maps, const float* A, const float* B, float* C,
                 cudaStream_t st, unsigned long long wait_ns) {
  static const bool attr = [] {  // once per instantiation, thread-safely
    cudaFuncSetAttribute(tc_pair_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    return true;
  }();
  (void)attr;
  tc_pair_kernel<MODE><<<2 * n, kPairThreads, kSmem, st>>>(t, maps, A, B, C, wait_ns);
}

template <int MODE, int AL, int BL>
void launch_one(const GemmTask* t, int n, const float* A, const float* B, float* C, cudaStream_t st,
                unsigned long long wait_ns) {
  // once per instantiation; a function-local static is initialised thread-safely
  // (the second log-likelihood pipeline launches from its own host thread)
  static const bool attr = [] {
    cudaFuncSetAttribute(tc_gemm_kernel<MODE, AL, BL>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    return true;
  }();
  (void)attr;
  tc_gemm_kernel<MODE, AL, BL><<<n, kThreads, kSmem, st>>>(t, A, B, C, wait_ns);
}

template <int MODE>
void launch_mode(const GemmTask* t, int n, const float* A, const float* B, float* C, int al, int bl, cudaStream_t st,
                 unsigned long long w) {
  if (al == kRow && bl == kRow) launch_one<MODE, kRow, kRow>(t, n, A, B, C, st, w);
  else if (al == kRow) launch_one<MODE, kRow, kCol>(t, n, A, B, C, st, w);
  else if (bl == kRow) launch_one<MODE, kCol, kRow>(t, n, A, B, C, st, w);
  else launch_one<MODE, kCol, kCol>(t, n, A, B, C, st, w);
}

}  // namespace

void launch_gemm_tc(const GemmTask* tasks, int ntasks, const float* A, const float* B, float* C, int mode, int al,
                    int bl, cudaStream_t st, unsigned long long wait_ns) {
  if (ntasks <= 0) return;
  switch (mode) {
    case kSub: launch_mode<kSub>(tasks, ntasks, A, B, C, al, bl, st, wait_ns); break;
    case kStore: launch_mode<kStore>(tasks, ntasks, A, B, C, al, bl, st, wait_ns); break;
    case kNegStore: launch_mode<kNegStore>(tasks, ntasks, A, B, C, al, bl, st, wait_ns); break;
    default: launch_mode<kAdd>(tasks, ntasks, A, B, C, al, bl, st, wait_ns); break;
  }
}

void launch_gemm_pair(const GemmTask* tasks, int ntasks, const CUtensorMap* maps, const float* A, const float* B,
                      float* C, int mode, cudaStream_t st, unsigned long long wait_ns) {
  if (ntasks <= 0) return;
  switch (mode) {
    case kSub: launch_pair<kSub>(tasks, ntasks, maps, A, B, C, st, wait_ns); break;
    case kStore: launch_pair<kStore>(tasks, ntasks, maps, A, B, C, st, wait_ns); break;
    case kNegStore: launch_pair<kNegStore>(tasks, ntasks, maps, A, B, C, st, wait_ns); break;
    default: launch_pair<kAdd>(tasks, ntasks, maps, A, B, C, st, wait_ns); break;
  }
}

int tc_gemm_take_error(cudaStream_t st, int* pinned) {
  // stream-ordered, so a second pipeline on another stream is not serialised
  static const int z = 0;
  *pinned = 0;
  cudaMemcpyFromSymbolAsync(pinned, g_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  const int h = *pinned;
  if (h) {
    cudaMemcpyToSymbolAsync(g_tc_error, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  return h;
}

}  // namespace spde
