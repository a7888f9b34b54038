// tc_gemm.cuh -- a small tcgen05 (5th-generation tensor core) GEMM for
// sm_103a: C[m][n] (+)= sum_k A[m][k] B[n][k] from FP64 operands, computed
// as three TF32 products with FP32 accumulation in tensor memory
// ("3xTF32": a = a_hi + a_lo with a_hi = tf32(a), a_lo = tf32(a - a_hi);
// a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, ~2^-21 relative), and FP64 output.
//
// One CTA of 128 threads owns one 128-row tile of A and one 64-row tile of B
// and loops over K in steps of 64 (the FP32 accumulator in tensor memory
// is folded into FP64 registers every kFoldTiles tiles):
//   * every thread loads FP64 elements, splits them and stores the TF32
//     halves in shared memory in the canonical no-swizzle K-major layout of
//     the tensor-core descriptors (8-row x 16-byte core matrices, 128 B
//     each; core matrix (row group g, k chunk c) at ((g * 16) + c) * 128 B,
//     so the leading byte offset between K-adjacent core matrices is 128 B
//     and the stride byte offset between 8-row groups is 2 KiB);
//   * thread 0 issues tcgen05.mma.cta_group::1.kind::tf32 (M = 128, N = 64,
//     K = 8) for the eight K steps and the three products, then
//     tcgen05.commit to an mbarrier;
//   * every thread waits on the mbarrier (bounded: after kSpinLimit polls the
//     kernel records an error flag instead of hanging);
// and finally each warp reads its 32 accumulator lanes with tcgen05.ld and
// the CTA writes the FP64 tile through shared memory, coalesced.  Tensor memory (64 columns) is allocated
// and freed by warp 0.  Operand rows past M or N and K past the end read as
// zero.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "narrow.cuh"

namespace neoxc {
namespace tc {

constexpr int kTileM = 128, kTileN = 64, kTileK = 64;
// K tiles accumulated in tensor memory (FP32) between two FP64 folds
constexpr int kFoldTiles = 4;
constexpr int kThreads = 128;
constexpr long long kSpinLimit = 1LL << 26;

// shared-memory bytes of one operand half: rows x 64 TF32 values
constexpr int kABytes = kTileM * kTileK * 4;   // 32 KiB
constexpr int kBBytes = kTileN * kTileK * 4;   // 16 KiB
constexpr int kSmemBytes = 2 * kABytes + 2 * kBBytes + 64;
// the epilogue's FP64 staging tile (kTileM rows of kTileN + 1) reuses the
// operand buffers
static_assert(kTileM * (kTileN + 1) * 8 <= 2 * kABytes + 2 * kBBytes, "epilogue tile");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of (row, k) in the canonical K-major layout above
__device__ __forceinline__ int canon_off(int row, int k) {
  return ((row >> 3) * 16 + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  const uint64_t lbo = 128, sbo = 2048;
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((lbo >> 4) & 0x3FFF) << 16 |
         ((sbo >> 4) & 0x3FFF) << 32 | (uint64_t)1 << 46;   // version 1, no swizzle
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N = 64, M = 128
__host__ __device__ constexpr uint32_t instr_desc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTileN >> 3) << 17) |
         ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// hi + lo carries the 22 leading bits of v, split in FP32 from narrow_f64
// (f - hi is exact in FP32): no FP64-pipe instruction
__device__ __forceinline__ void split_tf32(double v, uint32_t& hi, uint32_t& lo) {
  const float f = narrow_f64(v);
  hi = to_tf32(f);
  lo = to_tf32(f - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
      :
      : "r"(mbar)
      : "memory");
}

// bounded wait for the mbarrier phase; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (long long it = 0; it < kSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
        "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace neoxc
