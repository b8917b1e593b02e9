// st_mlp.cuh -- BF16 tensor-core GEMM (mma.sync m16n8k16, FP32 accumulate)
// with fused epilogues, used by the surrogate MLP's forward and backward.
//
// C[M][N] = sum_k A(m,k) B(k,n); operands staged in shared memory with
// cp.async (double-buffered) and read as fragments with ldmatrix.
//   A_KMAJ: A stored [M][lda] (k contiguous), else [K][lda] (m contiguous)
//   B_KMAJ: B stored [N][ldb] (k contiguous), else [K][ldb] (n contiguous)
// CTA tile 128 x 128 x 32, 256 threads = 8 warps (2 along M x 4 along N),
// warp tile 64 x 32 = 4 x 4 mma tiles.  M, N multiples of 128, K of 32;
// gridDim.z splits K (the epilogue then accumulates).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace st {
namespace mlp {

constexpr int TM = 128, TN = 128, TK = 32;
constexpr int GEMM_THREADS = 256;
constexpr int PAD = 8;  // halfs of row padding: 16-byte aligned rows, fewer ldmatrix bank conflicts

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldsm_x4(uint32_t* r, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t* r, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory tile shapes (halfs): K-contiguous tiles are [rows][TK+PAD],
// row/col-contiguous tiles are [TK][128+PAD].
constexpr int SK = TK + PAD;    // 40
constexpr int SR = 128 + PAD;   // 136
constexpr int TILE_HALFS = (128 * SK > TK * SR) ? 128 * SK : TK * SR;  // 5120 vs 4352

template <bool KMAJ>
__device__ __forceinline__ void load_tile(__nv_bfloat16* s, const __nv_bfloat16* g, int ld, int row0, int k0,
                                          int tid) {
  // 512 chunks of 16 bytes per tile, two per thread
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int id = tid + c * GEMM_THREADS;
    if (KMAJ) {  // 128 rows x 4 chunks
      const int r = id >> 2, q = id & 3;
      cp_async16(s + r * SK + q * 8, g + (size_t)(row0 + r) * ld + k0 + q * 8);
    } else {     // 32 k-rows x 16 chunks
      const int r = id >> 4, q = id & 15;
      cp_async16(s + r * SR + q * 8, g + (size_t)(k0 + r) * ld + row0 + q * 8);
    }
  }
}

// Epilogue contract: epi(m, n, v0, v1) receives C[m][n], C[m][n+1].
template <bool A_KMAJ, bool B_KMAJ, class Epi>
__global__ void __launch_bounds__(GEMM_THREADS) gemm_bf16_kernel(const __nv_bfloat16* __restrict__ A, int lda,
                                                                 const __nv_bfloat16* __restrict__ B, int ldb,
                                                                 int K, Epi epi) {
  __shared__ __align__(16) __nv_bfloat16 As[2][TILE_HALFS];
  __shared__ __align__(16) __nv_bfloat16 Bs[2][TILE_HALFS];
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;          // warp tile origin: (64 wm, 32 wn)
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  // split-K range of this CTA
  const int ksplit = gridDim.z;
  const int kchunk = ((K / TK + ksplit - 1) / ksplit) * TK;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;
  if (kbeg >= kend) {
    return;
  }
  const int nk = (kend - kbeg) / TK;
  load_tile<A_KMAJ>(As[0], A, lda, m0, kbeg, tid);
  load_tile<B_KMAJ>(Bs[0], B, ldb, n0, kbeg, tid);
  cp_async_commit();
  for (int kt = 0; kt < nk; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nk) {
      load_tile<A_KMAJ>(As[buf ^ 1], A, lda, m0, kbeg + (kt + 1) * TK, tid);
      load_tile<B_KMAJ>(Bs[buf ^ 1], B, ldb, n0, kbeg + (kt + 1) * TK, tid);
      cp_async_commit();
      cp_async_wait1();
    } else {
      cp_async_wait0();
    }
    __syncthreads();
    const __nv_bfloat16* as = As[buf];
    const __nv_bfloat16* bs = Bs[buf];
#pragma unroll
    for (int kk = 0; kk < TK; kk += 16) {
      uint32_t af[4][4], bfr[2][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mb = wm * 64 + i * 16;
        if (A_KMAJ) ldsm_x4(af[i], as + (mb + (lane & 15)) * SK + kk + (lane >> 4) * 8);
        else ldsm_x4_t(af[i], as + (kk + (lane & 7) + (lane >> 4) * 8) * SR + mb + ((lane >> 3) & 1) * 8);
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int nb = wn * 32 + j * 16;
        if (B_KMAJ) ldsm_x4(bfr[j], bs + (nb + (lane & 7) + (lane >> 4) * 8) * SK + kk + ((lane >> 3) & 1) * 8);
        else ldsm_x4_t(bfr[j], bs + (kk + (lane & 7) + ((lane >> 3) & 1) * 8) * SR + nb + (lane >> 4) * 8);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j >> 1][(j & 1) * 2], bfr[j >> 1][(j & 1) * 2 + 1]);
    }
    __syncthreads();
  }
  const int g = lane >> 2, t2 = (lane & 3) * 2;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + wm * 64 + i * 16 + g;
      const int n = n0 + wn * 32 + j * 8 + t2;
      epi(m, n, acc[i][j][0], acc[i][j][1]);
      epi(m + 8, n, acc[i][j][2], acc[i][j][3]);
    }
}

// SiLU and its derivative with the fast exponential and division (two MUFU
// operations each); where exp(-z) overflows, the quotient is 0 as it should be.
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = __fdividef(1.f, 1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// Forward of a hidden layer: z = acc + b; stores z (fp32, optional) and silu(z) (bf16).
struct EpiHidden {
  const float* bias;
  float* Z;               // [M][ldc] or null (inference)
  __nv_bfloat16* H;       // [M][ldc]
  int ldc;
  __device__ void operator()(int m, int n, float v0, float v1) const {
    const float z0 = v0 + bias[n], z1 = v1 + bias[n + 1];
    if (Z) *reinterpret_cast<float2*>(Z + (size_t)m * ldc + n) = make_float2(z0, z1);
    *reinterpret_cast<__nv_bfloat162*>(H + (size_t)m * ldc + n) = __floats2bfloat162_rn(silu(z0), silu(z1));
  }
  // one element (the tcgen05 GEMM's row-coalesced epilogue): pre() is read
  // for a whole block before its stores, so no store orders a later load;
  // store() returns the stored value for the transposed copy T (optional,
  // [ldc][ldt]: H^T for the weight gradient)
  __nv_bfloat16* T = nullptr;
  int ldt = 0;
  __device__ float pre(int, int) const { return 0.f; }
  __device__ float store(int m, int n, float v, float) const {
    const float z = v + bias[n];
    if (Z) Z[(size_t)m * ldc + n] = z;
    const __nv_bfloat16 h = __float2bfloat16_rn(silu(z));
    H[(size_t)m * ldc + n] = h;
    return __bfloat162float(h);
  }
};

// Backward through a hidden layer's input: dZ_prev = (dZ W) * silu'(Z_prev), bf16.
struct EpiBackDX {
  const float* Zprev;     // [M][ldc]
  __nv_bfloat16* dZprev;  // [M][ldc]
  int ldc;
  __device__ void operator()(int m, int n, float v0, float v1) const {
    const float2 z = *reinterpret_cast<const float2*>(Zprev + (size_t)m * ldc + n);
    *reinterpret_cast<__nv_bfloat162*>(dZprev + (size_t)m * ldc + n) =
        __floats2bfloat162_rn(v0 * dsilu(z.x), v1 * dsilu(z.y));
  }
  __nv_bfloat16* T = nullptr;  // optional transposed copy [ldc][ldt] (dZ^T for the weight gradient)
  int ldt = 0;
  __device__ float pre(int m, int n) const { return Zprev[(size_t)m * ldc + n]; }
  __device__ float store(int m, int n, float v, float z) const {
    const __nv_bfloat16 d = __float2bfloat16_rn(v * dsilu(z));
    dZprev[(size_t)m * ldc + n] = d;
    return __bfloat162float(d);
  }
};

// Weight gradient (split-K over the batch): dW[m][n] += acc.
struct EpiAccum {
  float* dW;
  int ldc;
  __device__ void operator()(int m, int n, float v0, float v1) const {
    atomicAdd(dW + (size_t)m * ldc + n, v0);
    atomicAdd(dW + (size_t)m * ldc + n + 1, v1);
  }
  __nv_bfloat16* T = nullptr;  // (no transposed copy)
  int ldt = 0;
  __device__ float pre(int, int) const { return 0.f; }
  __device__ float store(int m, int n, float v, float) const {
    atomicAdd(dW + (size_t)m * ldc + n, v);
    return 0.f;
  }
};

}  // namespace mlp
}  // namespace st
