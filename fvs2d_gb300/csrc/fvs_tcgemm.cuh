// fvs_tcgemm.cuh — BF16 GEMM on the 5th-generation tensor cores (tcgen05),
// FP32 accumulation in tensor memory:  C[m][n] = sum_k A(m,k) B(n,k).
//
// Operands are K-major (row m at A + m*lda) or stored transposed (element
// (m,k) at A + k*lda + m), as in the mma.sync GEMM of fvs_mlp.cu.
//
// CTA tile 128 x 128, K in blocks of 64 (four 128x128x16 MMAs), two shared
// memory stages.  128 threads (one warpgroup):
//   - all threads stage the operand tiles in the canonical K-major layout
//     without swizzle (core matrices of 8 rows x 16 bytes): 16-byte vectors
//     from K-major operands, element by element from transposed ones; then
//     fence.proxy.async makes them visible to the tensor core;
//   - thread 0 issues the MMAs (tcgen05.mma.cta_group::1.kind::f16, M 128,
//     N 128, K 16) and commits them to the stage's mbarrier, which frees the
//     stage for the block two steps later;
//   - after the last block, warp w reads accumulator rows 32w..32w+31
//     (tensor-memory lanes) with tcgen05.ld, 32 columns at a time, transposes
//     them through shared memory and writes whole row segments (coalesced)
//     with the epilogue applied.
// Split K (gridDim.z > 1): CTA z sums its own range of K blocks into the
// partial matrix C + z * split_stride (raw accumulators, no epilogue);
// k_sum_splits adds the partials in order (deterministic).
// Every mbarrier wait is bounded (clock64 budget).  On expiry the kernel sets
// *err, skips the remaining K blocks and the epilogue, waits for the MMAs it
// already issued (bounded, up to 9 budgets in all), frees its tensor memory
// and returns.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tc {

typedef __nv_bfloat16 bf16;

constexpr int BM = 128, BN = 128, BK = 64, THREADS = 128, STAGES = 2;
constexpr int TILE_BYTES = BM * BK * 2;                  // one operand tile: 16 KB
constexpr int SMEM_BYTES = STAGES * 2 * TILE_BYTES;      // 64 KB dynamic shared memory
constexpr uint32_t TMEM_COLS = 128;                      // FP32 accumulator 128 x 128
constexpr long long WAIT_BUDGET = 4000000000ll;          // clock cycles (~2 s at 2 GHz)

// Byte offset of element (r, k) of a 128 x 64 tile: core matrices of 8 rows x
// 8 elements stored as 128 contiguous bytes (row-major, 16 bytes a row); the
// two core matrices of one 16-wide K step 128 bytes apart (leading byte
// offset), 8-row groups 256 bytes apart (stride byte offset), K steps 4 KB apart.
__host__ __device__ constexpr uint32_t tile_offset(int r, int k) {
  return (uint32_t)((k >> 4) * 4096 + (r >> 3) * 256 + ((k >> 3) & 1) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset 128 >> 4 (bits 16-29), stride byte offset 256 >> 4 (bits 32-45),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A BF16 (bits 7-9
// = 1), B BF16 (bits 10-12 = 1), no negation, A and B K-major (bits 15, 16 =
// 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
constexpr uint32_t IDESC =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > WAIT_BUDGET) return false;
  }
}

template <bool KMAJOR>
__device__ __forceinline__ void stage_tile(uint8_t* s, const bf16* g, int ld, int row0, int rows, int k0, int K) {
  const int t = threadIdx.x;
  if (KMAJOR) {
    // 1024 chunks of 8 consecutive k (16 bytes), 8 per thread; 8 threads cover
    // one 128-byte row segment (coalesced)
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = q * THREADS + t;
      const int r = i >> 3, kc = (i & 7) * 8;
      const int gr = row0 + r, gk = k0 + kc;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gr < rows) {
        const bf16* src = g + (size_t)gr * ld + gk;
        if (gk + 8 <= K && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0)) {
          v = *reinterpret_cast<const uint4*>(src);
        } else {
          __align__(16) bf16 e[8];
#pragma unroll
          for (int j = 0; j < 8; j++) e[j] = gk + j < K ? src[j] : __float2bfloat16(0.f);
          v = *reinterpret_cast<const uint4*>(e);
        }
      }
      *reinterpret_cast<uint4*>(s + tile_offset(r, kc)) = v;
    }
  } else {
    // element (r, k) at g + k*ld + r: 8 consecutive r of one k per chunk
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = q * THREADS + t;
      const int k = i >> 4, rc = (i & 15) * 8;
      const int gk = k0 + k, gr = row0 + rc;
      __align__(16) bf16 e[8];
#pragma unroll
      for (int j = 0; j < 8; j++) e[j] = __float2bfloat16(0.f);
      if (gk < K) {
        const bf16* src = g + (size_t)gk * ld + gr;
        if (gr + 8 <= rows && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0)) {
          const uint4 v = *reinterpret_cast<const uint4*>(src);
          *reinterpret_cast<uint4*>(e) = v;
        } else {
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (gr + j < rows) e[j] = src[j];
        }
      }
#pragma unroll
      for (int j = 0; j < 8; j++) *reinterpret_cast<bf16*>(s + tile_offset(rc + j, k)) = e[j];
    }
  }
}

__device__ __forceinline__ float gelu_tc(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

// epi: 0 = C only, 1 = C = acc + bias, 2 = C = acc + bias and Cact = GELU(C)
template <bool A_KM, bool B_KM>
__global__ void __launch_bounds__(THREADS) k_gemm_tc(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B,
                                                     int ldb, int M, int N, int K, int epi,
                                                     const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                                     bf16* __restrict__ Cact, int ldact, int* __restrict__ err,
                                                     size_t split_stride) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar[STAGES];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  uint8_t* sA[STAGES] = {smem, smem + 2 * TILE_BYTES};
  uint8_t* sB[STAGES] = {smem + TILE_BYTES, smem + 3 * TILE_BYTES};

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; s++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_ok = 1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // K blocks of this CTA (all of them without split K)
  const int nk_all = (K + BK - 1) / BK;
  const int per = (nk_all + (int)gridDim.z - 1) / (int)gridDim.z;
  const int kb0 = (int)blockIdx.z * per;
  const int nk = max(0, min(nk_all - kb0, per));
  if (gridDim.z > 1) C += (size_t)blockIdx.z * split_stride;
  int issued = -1;  // last K block whose MMAs thread 0 committed
  for (int kb = 0; kb < nk; kb++) {
    const int s = kb & 1;
    if (kb >= STAGES) {
      // the MMAs of block kb-2 read this stage: wait for their commit
      if (tid == 0 && !mbar_wait(smem_u32(&mbar[s]), (uint32_t)(((kb - STAGES) >> 1) & 1))) s_ok = 0;
      __syncthreads();
      if (!s_ok) break;
    }
    stage_tile<A_KM>(sA[s], A, lda, m0, M, (kb0 + kb) * BK, K);
    stage_tile<B_KM>(sB[s], B, ldb, n0, N, (kb0 + kb) * BK, K);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t a0 = smem_u32(sA[s]), b0 = smem_u32(sB[s]);
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++) {
        const uint64_t ad = smem_desc(a0 + kk * 4096), bd = smem_desc(b0 + kk * 4096);
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(&mbar[s]))
                   : "memory");
      issued = kb;
    }
  }
  // Every MMA this CTA issued must be complete before its tensor memory is
  // read or freed, and before the CTA exits (the MMAs read the operand
  // stages in shared memory).  The commit of the last issued block tracks
  // all earlier MMAs of thread 0, so one wait on it covers them all; this
  // wait also runs after an earlier wait ran out (s_ok == 0, loop left
  // early).  The MMAs' operands are staged and nothing else gates them, so
  // the tensor core completes them; only a GPU stalled for the whole budget
  // makes the wait expire.  Then it is repeated once with 8 times the
  // budget, and the CTA frees its tensor memory only after that: freeing it
  // earlier could let a later CTA's accumulator receive these MMAs' writes.
  if (tid == 0 && issued >= 0) {
    const uint32_t fb = smem_u32(&mbar[issued & 1]), fp = (uint32_t)((issued >> 1) & 1);
    if (!mbar_wait(fb, fp)) {
      s_ok = 0;
      for (int r = 0; r < 8 && !mbar_wait(fb, fp); r++) {
      }
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (s_ok) {
    // transpose staging, one 32 x 33 float tile per warp, in the (now free)
    // operand stages
    float* st = reinterpret_cast<float*>(smem) + warp * (32 * 33);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      // lane = row: v[j] is column c0 + j; write the tile, read it back by
      // column so that each store instruction covers 32 consecutive columns
      if (nk == 0) {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = 0u;  // an empty K range contributes zeros
      }
#pragma unroll
      for (int j = 0; j < 32; j++) st[lane * 33 + j] = __uint_as_float(v[j]);
      __syncwarp();
      const int n = n0 + c0 + lane;
      const float bn = (epi != 0 && bias && n < N) ? bias[n] : 0.f;
#pragma unroll 4
      for (int r = 0; r < 32; r++) {
        const int m = m0 + warp * 32 + r;
        if (m >= M || n >= N) continue;
        const float z = st[r * 33 + lane] + bn;
        if (C) C[(size_t)m * ldc + n] = z;
        if (epi == 2 && Cact) Cact[(size_t)m * ldact + n] = __float2bfloat16(gelu_tc(z));
      }
      __syncwarp();
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// C[m][n] = sum over z of the split partials P[z][m][n] (ldc, stride), in
// order z = 0, 1, ... (deterministic)
__global__ void k_sum_splits(const float* __restrict__ P, int nsplit, size_t stride, int M, int N, int ldc,
                             float* __restrict__ C) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)M * N) return;
  const int m = (int)(i / N), n = (int)(i % N);
  const size_t o = (size_t)m * ldc + n;
  float acc = 0.f;
  for (int z = 0; z < nsplit; z++) acc += P[z * stride + o];
  C[o] = acc;
}

}  // namespace tc
