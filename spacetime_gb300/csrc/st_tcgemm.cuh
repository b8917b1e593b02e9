// st_tcgemm.cuh -- BF16 GEMM on the 5th-generation tensor cores for the
// surrogate's training passes: C[M][256] = A[M][K] . B[256][K]^T, both
// operands K-major bf16, FP32 accumulation in tensor memory, fused epilogue.
//
// One CTA computes a 128 x 256 tile (M = 128 rows of A, all 256 rows of B)
// with one 128-lane x 256-column TMEM accumulator.  K runs in blocks of 64
// elements (128 bytes per row): each block of A (16 KiB) and B (32 KiB) is
// copied with cp.async into a 128-byte-swizzled K-major stage (the layout of
// st_tc.cuh), four stages deep (a K = 256 layer's whole operands in flight
// at once); one thread issues the block's four tcgen05.mma (M = 128, N = 256,
// K = 16) and commits them to an mbarrier, which tells the copy of the block
// four ahead that the stage is free.  gridDim.z splits K (the epilogue then
// accumulates, e.g. with atomics).
//
// Every mbarrier wait is bounded.  A wait that runs out sets *status, the
// issuing thread waits again (bounded) for its last committed MMAs, and the
// CTA frees its TMEM and returns without an epilogue.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "st_tc.cuh"

namespace st {
namespace tcg {

constexpr int TILE_M = 128, TILE_N = 256, KB = 64, STAGES = 4, THREADS = 256;
constexpr uint32_t A_STAGE = TILE_M * 128, B_STAGE = TILE_N * 128;  // bytes per K-block
constexpr size_t SMEM = 1024 + STAGES * (size_t)(A_STAGE + B_STAGE) + 64;
constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr uint32_t IDESC = tc::idesc_bf16_f32(TILE_M, TILE_N);

// 16-byte global -> shared copy (cp.async, L2 only), its group and group wait.
__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(tc::smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Copy the K-block at k0 of A (rows m0..m0+127) and B (rows 0..255) into a
// stage: 16-byte chunk c of row r lands at r * 128 + ((c ^ (r & 7)) << 4).
__device__ __forceinline__ void load_block(unsigned char* As, unsigned char* Bs, const __nv_bfloat16* A, int lda,
                                           const __nv_bfloat16* B, int ldb, int m0, int k0, int tid) {
#pragma unroll
  for (int i = 0; i < (TILE_M * 8) / THREADS; ++i) {
    const int id = tid + i * THREADS, r = id >> 3, c = id & 7;
    cp16(As + r * 128 + ((c ^ (r & 7)) << 4), A + (size_t)(m0 + r) * lda + k0 + c * 8);
  }
#pragma unroll
  for (int i = 0; i < (TILE_N * 8) / THREADS; ++i) {
    const int id = tid + i * THREADS, r = id >> 3, c = id & 7;
    cp16(Bs + r * 128 + ((c ^ (r & 7)) << 4), B + (size_t)r * ldb + k0 + c * 8);
  }
}

// Epilogue contract: epi.store(m, n, v, a) receives C[m][n] and a = epi.pre(m, n),
// the epilogue's own operand at (m, n) (read for a whole block before any of
// its stores), and returns its output value; with epi.T set that value is also
// written transposed, T[n * epi.ldt + m] (bf16).  Each warp moves a 32 x 32
// block of the accumulator (its TMEM lanes = rows, 32 columns) through shared
// memory, so the epilogue runs a row at a time across the warp's lanes and its
// loads, stores and atomics are coalesced along n, and the transposed copy a
// column at a time, coalesced along m.
template <class Epi>
__global__ void __launch_bounds__(THREADS, 1)
    gemm_tc_kernel(const __nv_bfloat16* __restrict__ A, int lda, const __nv_bfloat16* __restrict__ B, int ldb, int K,
                   Epi epi, int* status) {
  extern __shared__ unsigned char tcg_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tcg_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char* Ast = base;                     // STAGES x A_STAGE
  unsigned char* Bst = base + STAGES * A_STAGE;  // STAGES x B_STAGE
  uint64_t* bar = reinterpret_cast<uint64_t*>(Bst + STAGES * B_STAGE);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  int* fail = reinterpret_cast<int*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TILE_M;
  // split-K range of this CTA, in whole K-blocks
  const int nkb_all = K / KB;
  const int per = (nkb_all + (int)gridDim.z - 1) / (int)gridDim.z;
  const int kb0 = blockIdx.z * per;
  const int nkb = min(nkb_all - kb0, per);
  if (nkb <= 0) return;  // uniform over the CTA: nothing allocated yet
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    *fail = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 256);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  int committed = -1;  // thread 0: index of the last K-block whose MMAs were committed
  // prologue: blocks 0 .. STAGES-2
#pragma unroll
  for (int s = 0; s < STAGES - 1; ++s) {
    if (s < nkb) load_block(Ast + s * A_STAGE, Bst + s * B_STAGE, A, lda, B, ldb, m0, (kb0 + s) * KB, tid);
    cp_commit();
  }
  for (int kb = 0; kb < nkb; ++kb) {
    // the stage the copy ahead will fill was read by block kb - 1's MMAs
    if (kb >= 1) {
      if (!tc::mbar_wait(bar, (uint32_t)(kb - 1) & 1u, WAIT_LIMIT)) *fail = 1;
    }
    __syncthreads();
    if (*fail) break;
    const int ahead = kb + STAGES - 1;
    if (ahead < nkb) {
      const int sa = ahead % STAGES;
      load_block(Ast + sa * A_STAGE, Bst + sa * B_STAGE, A, lda, B, ldb, m0, (kb0 + ahead) * KB, tid);
    }
    cp_commit();
    cp_wait<STAGES - 1>();   // block kb's copies have landed
    tc::fence_proxy_async();  // ... and are visible to the tensor cores
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const int st = kb % STAGES;
      const uint32_t a_addr = tc::smem_u32(Ast + st * A_STAGE), b_addr = tc::smem_u32(Bst + st * B_STAGE);
#pragma unroll
      for (int s = 0; s < KB / 16; ++s)
        tc::mma_bf16(tmem, tc::sw128_desc(a_addr + s * 32), tc::sw128_desc(b_addr + s * 32), IDESC,
                     (kb > 0 || s > 0) ? 1u : 0u);
      tc::mma_commit(bar);
      committed = kb;
    }
  }
  cp_wait<0>();
  // the last block's MMAs
  if (!*fail && !tc::mbar_wait(bar, (uint32_t)(nkb - 1) & 1u, WAIT_LIMIT)) *fail = 1;
  __syncthreads();
  const bool failed = *fail != 0;
  if (failed && tid == 0 && committed >= 0) {
    // drain: the last committed phase (returns at once if it has completed)
    (void)tc::mbar_wait(bar, (uint32_t)committed & 1u, WAIT_LIMIT);
  }
  tc::fence_after_sync();
  if (!failed) {
    // warp w: TMEM lanes (rows) 32 (w mod 4).., columns 128 (w div 4)..; the
    // stages are free (every copy and MMA has completed), so each warp turns
    // its blocks around in a padded 32 x 33 float tile there
    const uint32_t q = warp & 3, ch = warp >> 2;
    float* tile = reinterpret_cast<float*>(Ast) + warp * (32 * 33);
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      const int col0 = (int)ch * 128 + c * 32;
      const int mq = m0 + (int)(q * 32);
      float pre[32];
#pragma unroll
      for (int r = 0; r < 32; ++r) pre[r] = epi.pre(mq + r, col0 + lane);
      float v[32];
      tc::tmem_ld32(tmem + ((q * 32u) << 16) + (uint32_t)col0, v);
#pragma unroll
      for (int e = 0; e < 32; ++e) tile[lane * 33 + e] = v[e];
      __syncwarp();
#pragma unroll
      for (int r = 0; r < 32; ++r)
        tile[r * 33 + lane] = epi.store(mq + r, col0 + lane, tile[r * 33 + lane], pre[r]);
      __syncwarp();
      if (epi.T) {
#pragma unroll 8
        for (int c = 0; c < 32; ++c)
          epi.T[(size_t)(col0 + c) * epi.ldt + mq + lane] = __float2bfloat16_rn(tile[lane * 33 + c]);
        __syncwarp();
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 256);
  }
  if (failed && tid == 0 && status) atomicExch(status, 1);
}

// dst[c][r] = src[r][c] for a rows x cols bf16 matrix (both multiples of 32).
__global__ void __launch_bounds__(256) transpose_bf16(const __nv_bfloat16* __restrict__ src,
                                                      __nv_bfloat16* __restrict__ dst, int rows, int cols) {
  __shared__ __nv_bfloat16 t[32][34];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 32; i += 8) t[ty + i][tx] = src[(size_t)(r0 + ty + i) * cols + c0 + tx];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 32; i += 8) dst[(size_t)(c0 + ty + i) * rows + r0 + tx] = t[tx][ty + i];
}

}  // namespace tcg
}  // namespace st
