// umma.cuh -- a BF16 matrix product on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory, operands staged by TMA).
//
// gemm_tc<BN> computes C[M,N] = A[M,K] B[N,K]^T, A and B in BF16 with K
// contiguous, FP32 accumulation, one 128 x BN tile per block of 128 threads:
//   - thread 0 issues the TMA loads of 64-wide K slices of A (128 rows) and B
//     (BN rows) into a ring of STAGES shared-memory stages, in the 128-byte
//     swizzled K-major layout, each stage completing on an mbarrier;
//   - the same thread issues four tcgen05.mma (K = 16 each) per stage into a
//     128 x BN FP32 accumulator in tensor memory and commits them to the
//     stage's "empty" mbarrier, which releases the stage for the next load;
//   - after the last stage's MMAs a final commit signals the accumulator;
//     every warp reads its 32 rows (tensor-memory lanes 32w..32w+31) with
//     tcgen05.ld and applies the epilogue of gemm_tn (bias, ReLU, FP32 and
//     BF16 stores, row-major and transposed).
// Rows and columns past M, N and the K tail read zeros (the tensor maps'
// out-of-bounds fill).  Every mbarrier wait is bounded; a wait that runs
// out sets *err, waits (bounded) for the copies and products in flight,
// frees the tensor memory and leaves without storing.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

namespace cliffs_nn {

namespace umma {

constexpr int BM = 128, BK = 64, STAGES = 4, THREADS = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s: far above any product here

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of the given parity, for at most kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_try(bar, parity))
    if (now_ns() - t0 > kWaitNs) return false;
  return true;
}

// One box of a 2-D tensor map at element coordinates (x, y), completing on bar.
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile in the 128-byte
// swizzled layout: rows of 128 bytes (64 BF16), 8-row groups 1024 bytes apart
// (the stride byte offset); the leading byte offset is unused in this layout.
// Bits: start address >> 4 [0,14), leading offset >> 4 [16,30), stride offset
// >> 4 [32,46), the descriptor version 1 at bit 46, swizzle mode 2 (128 B) in
// [61,64).  The tile's base is 1024-byte aligned (base offset 0).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits [4,6) = 1),
// A and B in BF16 ([7,10) = 1, [10,13) = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in [17,23), M >> 4 in [24,29).
template <int BN>
__device__ __forceinline__ uint32_t idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives on bar once every tcgen05 operation this thread issued before has
// completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace umma

template <int BN>
constexpr uint32_t gemm_tc_smem() {
  return umma::STAGES * (umma::BM + BN) * umma::BK * 2 + 1024;  // + alignment slack
}

template <int BN>
__global__ void __launch_bounds__(umma::THREADS, 1)
    gemm_tc(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N, int K,
            Epi e, unsigned* err) {
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "tcgen05 kind::f16 with M = 128 takes N = 16..256, step 16");
  constexpr uint32_t ABYTES = umma::BM * umma::BK * 2, BBYTES = BN * umma::BK * 2, STAGE = ABYTES + BBYTES;
  constexpr uint32_t TCOLS = BN < 32 ? 32 : BN;  // tensor-memory columns: a power of 2, at least 32
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[umma::STAGES], empty[umma::STAGES], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * umma::BM, n0 = blockIdx.y * BN;
  const int nk = (K + umma::BK - 1) / umma::BK;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(umma::smem_u32(&tmem_base)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < umma::STAGES; ++s) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    umma::mbar_init(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    s_ok = 1;
  }
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tmem = tmem_base;
  if (threadIdx.x == 0) {
    auto issue = [&](int kb) {
      const int s = kb % umma::STAGES;
      uint8_t* a = smem + s * STAGE;
      umma::mbar_expect_tx(&full[s], STAGE);
      umma::tma_2d(a, &ta, &full[s], kb * umma::BK, m0);
      umma::tma_2d(a + ABYTES, &tb, &full[s], kb * umma::BK, n0);
    };
    const int pre = nk < umma::STAGES ? nk : umma::STAGES;
    for (int kb = 0; kb < pre; ++kb) issue(kb);
    int issued = pre, consumed = 0;
    bool ok = true;
    const uint32_t idesc = umma::idesc_bf16<BN>();
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % umma::STAGES;
      const uint32_t ph = (uint32_t)(kb / umma::STAGES) & 1u;
      if (!umma::mbar_wait(&full[s], ph)) {
        ok = false;
        break;
      }
      consumed = kb + 1;
      umma::fence_after();
      const uint32_t a = umma::smem_u32(smem + s * STAGE), b = a + ABYTES;
#pragma unroll
      for (int k = 0; k < umma::BK / 16; ++k)  // K = 16 per MMA: 32 bytes along the swizzled row
        umma::mma_bf16(tmem, umma::sw128_desc(a + 32 * k), umma::sw128_desc(b + 32 * k), idesc, (kb | k) != 0);
      umma::commit(&empty[s]);
      if (kb + umma::STAGES < nk) {
        if (!umma::mbar_wait(&empty[s], ph)) {
          ok = false;
          break;
        }
        issue(kb + umma::STAGES);
        ++issued;
      }
    }
    if (!ok) {
      atomicOr(err, 1u);
      // the copies still in flight land before the block leaves
      for (int kb = consumed; kb < issued; ++kb) umma::mbar_wait(&full[kb % umma::STAGES], (uint32_t)(kb / umma::STAGES) & 1u);
      s_ok = 0;
    }
    umma::commit(&done);  // arrives once every product issued above is done
  }
  __syncthreads();
  // every thread waits for the accumulator; the outcome is the block's, so
  // the warp-wide tensor-memory loads below run in every warp or in none
  const bool fin = __syncthreads_and(umma::mbar_wait(&done, 0)) != 0;
  umma::fence_after();
  if (!fin && threadIdx.x == 0) atomicOr(err, 1u);
  if (s_ok && fin) {
    const int row = m0 + 32 * warp + lane;
    // a thread's 16 consecutive columns go out as 16-byte stores where the
    // rows allow it (the transposed copy is coalesced across the warp as is)
    const bool vf = e.f32 && e.ldf % 4 == 0 && ((uintptr_t)e.f32 & 15) == 0;
    const bool vb = e.b16 && e.ldb % 8 == 0 && ((uintptr_t)e.b16 & 15) == 0;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
      const int cb = n0 + c0;
      if (row < M && cb + 16 <= N) {
        if (e.bias) {
          const float4* b4 = reinterpret_cast<const float4*>(e.bias + cb);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float4 b = __ldg(b4 + q);
            v[4 * q] += b.x;
            v[4 * q + 1] += b.y;
            v[4 * q + 2] += b.z;
            v[4 * q + 3] += b.w;
          }
        }
        if (e.relu)
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.f);
        if (vf) {
          float4* o = reinterpret_cast<float4*>(e.f32 + (size_t)row * e.ldf + cb);
#pragma unroll
          for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else if (e.f32) {
#pragma unroll
          for (int j = 0; j < 16; ++j) e.f32[(size_t)row * e.ldf + cb + j] = v[j];
        }
        if (e.b16 || e.b16t) {
          uint32_t h[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const __nv_bfloat162 t = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);  // .x = low half
            h[q] = *reinterpret_cast<const uint32_t*>(&t);
          }
          if (vb) {
            uint4* o = reinterpret_cast<uint4*>(e.b16 + (size_t)row * e.ldb + cb);
            o[0] = make_uint4(h[0], h[1], h[2], h[3]);
            o[1] = make_uint4(h[4], h[5], h[6], h[7]);
          } else if (e.b16) {
#pragma unroll
            for (int j = 0; j < 16; ++j) e.b16[(size_t)row * e.ldb + cb + j] = __float2bfloat16(v[j]);
          }
          if (e.b16t)
#pragma unroll
            for (int j = 0; j < 16; ++j) e.b16t[(size_t)(cb + j) * e.ldt + row] = __float2bfloat16(v[j]);
        }
      } else if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = cb + j;
          if (col >= N) break;
          float x = v[j];
          if (e.bias) x += e.bias[col];
          if (e.relu) x = fmaxf(x, 0.f);
          if (e.f32) e.f32[(size_t)row * e.ldf + col] = x;
          const __nv_bfloat16 hb = __float2bfloat16(x);
          if (e.b16) e.b16[(size_t)row * e.ldb + col] = hb;
          if (e.b16t) e.b16t[(size_t)col * e.ldt + row] = hb;
        }
      }
    }
  }
  umma::fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS) : "memory");
}

}  // namespace cliffs_nn
