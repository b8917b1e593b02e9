// st_surrogate.cu -- the learned exit-direction surrogate.
//
// MLP 6 -> 256 -> 256 -> 256 -> 256 -> 6 (SiLU), 200,710 parameters.
//   inputs  : camera KS radius r in [4, 50] M, inclination theta in [0, 90] deg,
//             spin a in [0, 0.99], unit ray direction n in the static observer's
//             frame (radial, polar, azimuthal axes), normalised to O(1).
//             Training directions put 80% of the samples in the 75-degree cone
//             around the inward radial direction (the rays of a camera looking
//             at the hole) and 20% on the rest of the sphere.
//   outputs : exit direction in the ray's own plane -- the plane of the unit
//             position xh and the launch direction d0, in which a Schwarzschild
//             ray stays: the in-plane deflection D (radians, wrapped to
//             [-pi/2, 3pi/2)) and the out-of-plane tilt E (radians), with the
//             third output unused; then the first equatorial-crossing radius as
//             10/s - 1 (no crossing is the s -> inf limit, -1), redshift g - 1
//             there, and the log-variance of the two angles.
//             exit = cos E (cos(psi + D) xh + sin(psi + D) et) + sin E (xh x et),
//             with psi the angle from xh to d0 and et the unit part of d0
//             normal to xh.  For a = 0 the angles depend only on r and n . xh,
//             so the network's work is the spin's correction, not the geometry.
// The three 256x256 layers run on the tensor cores in BF16 with FP32
// accumulation (st_mlp.cuh); the 6->256 and 256->6 layers, the loss and AdamW
// run in FP32.  Master weights and optimiser state are FP32.
//
// Training labels come from the FP64 integrator on the GPU (label_kernel):
// Sobol-sampled inputs, the kernel's step rule and kill tests
// (src/metal.jl:1201-1572) with the spin per sample, exit direction on the
// escape radius 2 max(|pos|, 15M) (src/metal.jl:2058-2059).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "st_internal.h"
#include "st_mlp.cuh"
#include "st_tc.cuh"
#include "st_tcgemm.cuh"
#include "st_trace.cuh"

namespace st {
namespace sur {

using mlp::EpiAccum;
using mlp::EpiBackDX;
using mlp::EpiHidden;

constexpr int NIN = 6, NH = 256, NOUT = 6, NT = 8;  // NT: target floats per row
constexpr int NRAW = 15;  // floats per optional raw label row (LabelParams::raw)
// parameter offsets (floats)
constexpr size_t OW0 = 0, OB0 = OW0 + NH * NIN, OW1 = OB0 + NH, OB1 = OW1 + NH * NH, OW2 = OB1 + NH,
                 OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NH * NH, OW4 = OB3 + NH, OB4 = OW4 + NOUT * NH,
                 NPARAM = OB4 + NOUT;
static_assert(NPARAM == 200710, "parameter count");
constexpr size_t OWH[3] = {OW1, OW2, OW3};
constexpr size_t OBH[3] = {OB1, OB2, OB3};

// ---------------------------------------------------------------------------
// small FP32 layers, loss, reductions, AdamW
// ---------------------------------------------------------------------------

// Z0 = X W0^T + b0, H0 = bf16(silu(Z0)): a block of 256 threads (one per
// unit, its weights in registers) takes L0_ROWS rows, whose inputs it stages in
// shared memory; each row's outputs are one coalesced store per array.
constexpr int L0_ROWS = 16;
__global__ void __launch_bounds__(NH) l0_fwd(const float* __restrict__ X, const float* __restrict__ P, float* Z0,
                                             __nv_bfloat16* H0, int B) {
  const int n = threadIdx.x;
  const int b0 = blockIdx.x * L0_ROWS, nb = min(B - b0, L0_ROWS);
  __shared__ float xs[L0_ROWS * NIN];
  if (n < nb * NIN) xs[n] = X[(size_t)b0 * NIN + n];
  float w[NIN];
#pragma unroll
  for (int i = 0; i < NIN; ++i) w[i] = P[OW0 + n * NIN + i];
  const float bias = P[OB0 + n];
  __syncthreads();
#pragma unroll 4
  for (int r = 0; r < nb; ++r) {
    float z = bias;
#pragma unroll
    for (int i = 0; i < NIN; ++i) z += xs[r * NIN + i] * w[i];
    const size_t idx = (size_t)(b0 + r) * NH + n;
    if (Z0) Z0[idx] = z;
    H0[idx] = __float2bfloat16_rn(mlp::silu(z));
  }
}

// one warp per row: out[b][j] = H3[b] . W4[j] + b4[j]
__global__ void l4_fwd(const __nv_bfloat16* __restrict__ H3, const float* __restrict__ P, float* out, int B) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B) return;
  float acc[NOUT] = {0, 0, 0, 0, 0, 0};
  for (int k = lane; k < NH; k += 32) {
    const float h = __bfloat162float(H3[(size_t)warp * NH + k]);
#pragma unroll
    for (int j = 0; j < NOUT; ++j) acc[j] += h * P[OW4 + j * NH + k];
  }
#pragma unroll
  for (int j = 0; j < NOUT; ++j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
  }
  if (lane < NOUT) {
    float v = acc[0];
#pragma unroll
    for (int j = 1; j < NOUT; ++j) if (lane == j) v = acc[j];
    out[(size_t)warp * NOUT + lane] = v + P[OB4 + lane];
  }
}

// Loss per row (targets: t0, t1 the in-plane deflection and out-of-plane
// tilt, t3 crossing radius, t4 g - 1, t5 direction mask, t6 crossing mask):
//   0.5 |o01 - t01|^2 exp(-s) + s   (two angles, heteroscedastic, s = o5)
//   + WR (o3 - t3)^2 + WG m (o4 - t4)^2
// o2 is unused and carries no gradient.
// loss_acc[0..3] += (total, direction MSE, radius MSE, g MSE) / B
constexpr float WR = 1.0f, WG = 1.0f;
__global__ void loss_grad(const float* __restrict__ out, const float* __restrict__ T, float* dout, float* loss_acc,
                          int B, float inv_batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l_tot = 0.f, l_dir = 0.f, l_r = 0.f, l_g = 0.f;
  if (b < B) {
    const float* o = out + (size_t)b * NOUT;
    const float* t = T + (size_t)b * NT;
    const float md = t[5], mc = t[6];
    const float s = fminf(fmaxf(o[5], -30.f), 12.f);
    const float es = __expf(-s);
    float e2 = 0.f, g[NOUT];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const float e = o[k] - t[k];
      e2 += e * e;
      g[k] = md * e * es;
    }
    g[2] = 0.f;
    g[5] = (o[5] > -30.f && o[5] < 12.f) ? md * (-0.5f * e2 * es + 1.f) : 0.f;
    const float er = o[3] - t[3], eg = o[4] - t[4];
    g[3] = 2.f * WR * er;
    g[4] = 2.f * WG * mc * eg;
#pragma unroll
    for (int k = 0; k < NOUT; ++k) dout[(size_t)b * NOUT + k] = g[k] * inv_batch;
    l_dir = md * e2;
    l_r = er * er;
    l_g = mc * eg * eg;
    l_tot = md * (0.5f * e2 * es + s) + WR * l_r + WG * l_g;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    l_tot += __shfl_xor_sync(0xffffffffu, l_tot, o);
    l_dir += __shfl_xor_sync(0xffffffffu, l_dir, o);
    l_r += __shfl_xor_sync(0xffffffffu, l_r, o);
    l_g += __shfl_xor_sync(0xffffffffu, l_g, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(loss_acc + 0, l_tot * inv_batch);
    atomicAdd(loss_acc + 1, l_dir * inv_batch);
    atomicAdd(loss_acc + 2, l_r * inv_batch);
    atomicAdd(loss_acc + 3, l_g * inv_batch);
  }
}

// dZ3 = silu'(Z3) * (dout . W4)
// dZ3 = silu'(Z3) * (dout . W4); a thread takes four adjacent units of one
// row (vector loads and stores), the row's output gradient read once.
__global__ void l4_bwd_dx(const float* __restrict__ dout, const float* __restrict__ P, const float* __restrict__ Z3,
                          __nv_bfloat16* dZ3, int B) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // quad index
  if (q >= B * (NH / 4)) return;
  const int b = q / (NH / 4), k0 = (q - b * (NH / 4)) * 4;
  float d[NOUT];
#pragma unroll
  for (int j = 0; j < NOUT; ++j) d[j] = dout[(size_t)b * NOUT + j];
  const size_t idx = (size_t)b * NH + k0;
  const float4 z = *reinterpret_cast<const float4*>(Z3 + idx);
  float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int j = 0; j < NOUT; ++j) {
    const float4 w = *reinterpret_cast<const float4*>(P + OW4 + j * NH + k0);
    v[0] += d[j] * w.x; v[1] += d[j] * w.y; v[2] += d[j] * w.z; v[3] += d[j] * w.w;
  }
  const __nv_bfloat162 a = __floats2bfloat162_rn(v[0] * mlp::dsilu(z.x), v[1] * mlp::dsilu(z.y));
  const __nv_bfloat162 c = __floats2bfloat162_rn(v[2] * mlp::dsilu(z.z), v[3] * mlp::dsilu(z.w));
  *reinterpret_cast<uint2*>(dZ3 + idx) =
      make_uint2(*reinterpret_cast<const uint32_t*>(&a), *reinterpret_cast<const uint32_t*>(&c));
}

// dW4[j][k] = sum_b dout[b][j] H3[b][k], db4[j] = sum_b dout[b][j], in two
// stages: a block of 256 threads (one per k) sweeps RED_ROWS rows (32: a batch
// of 16384 gives 512 blocks, enough to cover the GPU's SMs) and writes its
// partial sums to its row of `part` ([block][L4_PART]: dW4 row-major, then db4),
// then reduce_parts sums the blocks' rows in a fixed order.  (Atomic adds of
// every block into the same 1.5-1.8 K gradient words serialise on the few L2
// slices those words live in.)
constexpr int RED_ROWS = 32;
constexpr int L4_PART = NOUT * NH + NOUT;  // 1542
constexpr int L0_PART = NH * NIN + NH;     // 1792
__global__ void l4_bwd_w(const float* __restrict__ dout, const __nv_bfloat16* __restrict__ H3, float* part, int B) {
  const int k = threadIdx.x;
  const int b0 = blockIdx.x * RED_ROWS, b1 = min(B, b0 + RED_ROWS);
  // the block's rows of dout, which every thread reads, staged once
  __shared__ float ds[RED_ROWS * NOUT];
  if (k < (b1 - b0) * NOUT) ds[k] = dout[(size_t)b0 * NOUT + k];
  __syncthreads();
  float acc[NOUT] = {0, 0, 0, 0, 0, 0};
#pragma unroll 8
  for (int b = b0; b < b1; ++b) {
    const float h = __bfloat162float(H3[(size_t)b * NH + k]);
#pragma unroll
    for (int j = 0; j < NOUT; ++j) acc[j] += ds[(b - b0) * NOUT + j] * h;
  }
  float* row = part + (size_t)blockIdx.x * L4_PART;
#pragma unroll
  for (int j = 0; j < NOUT; ++j) row[j * NH + k] = acc[j];
  if (k < NOUT) {
    // thread j < 6: the block's db4[j]
    float db = 0.f;
    for (int b = 0; b < b1 - b0; ++b) db += ds[b * NOUT + k];
    row[NOUT * NH + k] = db;
  }
}

// G[base + c] = sum over the nparts rows of part[p][c], c < ncols, in a
// fixed order.  Block: 32 columns (a lane each) x 32 warps, warp w taking rows
// w, w + 32, ... (coalesced 128-byte loads, 16 per warp for 512 rows); the
// warps' sums combine in shared memory.
__global__ void __launch_bounds__(1024) reduce_parts(const float* __restrict__ part, int nparts, int ncols,
                                                     float* G, size_t base) {
  __shared__ float red[32][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  float acc = 0.f;
  if (c < ncols) {
#pragma unroll 8
    for (int p = w; p < nparts; p += 32) acc += part[(size_t)p * ncols + c];
  }
  red[w][lane] = acc;
  __syncthreads();
  if (w == 0 && c < ncols) {
    float t = red[0][lane];
#pragma unroll
    for (int k = 1; k < 32; ++k) t += red[k][lane];
    G[base + c] = t;
  }
}

// column sums of a bf16 [B][256] matrix into G[off + n]
__global__ void colsum_bf16(const __nv_bfloat16* __restrict__ D, float* G, size_t off, int B) {
  const int n = threadIdx.x;
  const int b0 = blockIdx.x * RED_ROWS, b1 = min(B, b0 + RED_ROWS);
  float s = 0.f;
#pragma unroll 8
  for (int b = b0; b < b1; ++b) s += __bfloat162float(D[(size_t)b * NH + n]);
  atomicAdd(G + off + n, s);
}

// dW0[n][i] = sum_b dZ0[b][n] X[b][i], db0[n] = sum_b dZ0[b][n]: the block
// partials of the two-stage reduction above ([block][L0_PART]: dW0 row-major,
// then db0)
__global__ void l0_bwd(const __nv_bfloat16* __restrict__ dZ0, const float* __restrict__ X, float* part, int B) {
  const int n = threadIdx.x;
  const int b0 = blockIdx.x * RED_ROWS, b1 = min(B, b0 + RED_ROWS);
  // the block's rows of X, which every thread reads, staged once
  __shared__ float xs[RED_ROWS * NIN];
  if (n < (b1 - b0) * NIN) xs[n] = X[(size_t)b0 * NIN + n];
  __syncthreads();
  float acc[NIN] = {0, 0, 0, 0, 0, 0}, db = 0.f;
#pragma unroll 8
  for (int b = b0; b < b1; ++b) {
    const float d = __bfloat162float(dZ0[(size_t)b * NH + n]);
    db += d;
#pragma unroll
    for (int i = 0; i < NIN; ++i) acc[i] += d * xs[(b - b0) * NIN + i];
  }
  float* row = part + (size_t)blockIdx.x * L0_PART;
#pragma unroll
  for (int i = 0; i < NIN; ++i) row[n * NIN + i] = acc[i];
  row[NH * NIN + n] = db;
}

__global__ void adamw(float* P, const float* G, float* Mm, float* Vv, size_t n, float lr, float b1, float b2,
                      float eps, float wd, float bc1, float bc2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * Mm[i] + (1.f - b1) * g;
  const float v = b2 * Vv[i] + (1.f - b2) * g * g;
  Mm[i] = m;
  Vv[i] = v;
  // decoupled weight decay on the weight matrices only (biases are exempt)
  const bool is_bias = (i >= OB0 && i < OW1) || (i >= OB1 && i < OW2) || (i >= OB2 && i < OW3) ||
                       (i >= OB3 && i < OW4) || i >= OB4;
  float p = P[i];
  if (!is_bias) p -= lr * wd * p;
  P[i] = p - lr * (m / bc1) / (sqrtf(v / bc2) + eps);
}

__global__ void to_bf16(const float* __restrict__ src, __nv_bfloat16* dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// ---------------------------------------------------------------------------
// Sobol points and FP64 labels
// ---------------------------------------------------------------------------

constexpr int SOBOL_DIMS = 5;
__constant__ uint32_t c_sobol_v[SOBOL_DIMS][32];

// Direction numbers from primitive polynomials (degree s, coefficient bits a,
// initial m_k), Bratley-Fox recurrence; dimension 0 is van der Corput.
static void sobol_directions(uint32_t v[SOBOL_DIMS][32]) {
  struct Poly { int s, a; uint32_t m[4]; };
  const Poly polys[SOBOL_DIMS - 1] = {{1, 0, {1}}, {2, 1, {1, 3}}, {3, 1, {1, 3, 1}}, {3, 2, {1, 1, 1}}};
  for (int k = 0; k < 32; ++k) v[0][k] = 1u << (31 - k);
  for (int d = 1; d < SOBOL_DIMS; ++d) {
    const Poly& P = polys[d - 1];
    uint32_t m[33];
    for (int k = 1; k <= P.s; ++k) m[k] = P.m[k - 1];
    for (int k = P.s + 1; k <= 32; ++k) {
      uint32_t mk = m[k - P.s] ^ (m[k - P.s] << P.s);
      for (int j = 1; j < P.s; ++j)
        if ((P.a >> (P.s - 1 - j)) & 1) mk ^= m[k - j] << j;
      m[k] = mk;
    }
    for (int k = 1; k <= 32; ++k) v[d][k - 1] = m[k] << (32 - k);
  }
}

__device__ __forceinline__ float sobol(uint32_t i, int d) {
  uint32_t x = 0;
#pragma unroll 4
  for (int k = 0; k < 32; ++k)
    if ((i >> k) & 1u) x ^= c_sobol_v[d][k];
  return (float)((x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Static observer's orthonormal frame in Kerr-Schild form at pos (valid
// where f <= 0.72, i.e. r >= 4 M here); Gram-Schmidt of (e1, e2, e3) under g.
template <typename D>
__device__ void static_frame(const D* pos, const D* e1, const D* e2, const D* e3, D M, D a, D* U, D* E1, D* E2,
                             D* E3) {
  D l[3], f;
  if (a != D(0)) {
    const D rk2 = ks_r2(pos[0], pos[1], pos[2], a);
    const D rk = sqrt_(max_(rk2, D(1e-12)));
    const D ira = D(1) / (rk2 + a * a);
    l[0] = (rk * pos[0] + a * pos[1]) * ira;
    l[1] = (rk * pos[1] - a * pos[0]) * ira;
    l[2] = pos[2] / rk;
    f = D(2) * M * rk2 * rk / (rk2 * rk2 + a * a * pos[2] * pos[2]);
  } else {
    const D r = sqrt_(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
    l[0] = pos[0] / r; l[1] = pos[1] / r; l[2] = pos[2] / r;
    f = D(2) * M / r;
  }
  auto gd = [&](const D* A, const D* B) {
    const D la = A[0] + l[0] * A[1] + l[1] * A[2] + l[2] * A[3];
    const D lb = B[0] + l[0] * B[1] + l[1] * B[2] + l[2] * B[3];
    return -A[0] * B[0] + A[1] * B[1] + A[2] * B[2] + A[3] * B[3] + f * la * lb;
  };
  U[0] = D(1) / sqrt_(D(1) - f); U[1] = U[2] = U[3] = D(0);
  D a1[4] = {D(0), e1[0], e1[1], e1[2]}, a2[4] = {D(0), e2[0], e2[1], e2[2]}, a3[4] = {D(0), e3[0], e3[1], e3[2]};
  D c = gd(a1, U);
  for (int k = 0; k < 4; ++k) a1[k] += c * U[k];
  c = sqrt_(gd(a1, a1));
  for (int k = 0; k < 4; ++k) E1[k] = a1[k] / c;
  c = gd(a2, U);
  for (int k = 0; k < 4; ++k) a2[k] += c * U[k];
  c = gd(a2, E1);
  for (int k = 0; k < 4; ++k) a2[k] -= c * E1[k];
  c = sqrt_(gd(a2, a2));
  for (int k = 0; k < 4; ++k) E2[k] = a2[k] / c;
  c = gd(a3, U);
  for (int k = 0; k < 4; ++k) a3[k] += c * U[k];
  const D c1 = gd(a3, E1), c2 = gd(a3, E2);
  for (int k = 0; k < 4; ++k) a3[k] -= c1 * E1[k] + c2 * E2[k];
  c = sqrt_(gd(a3, a3));
  for (int k = 0; k < 4; ++k) E3[k] = a3[k] / c;
}

// Frame axes of a camera at inclination theta (azimuth 0): radial, polar
// (increasing theta) and azimuthal unit vectors of the Cartesian position.
template <typename D>
__device__ __forceinline__ void frame_axes(const D* pos, D* e1, D* e2, D* e3) {
  const D rr = sqrt_(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
  const D ct = pos[2] / rr, st = sqrt_(max_(D(1) - ct * ct, D(0)));
  e1[0] = pos[0] / rr; e1[1] = pos[1] / rr; e1[2] = ct;
  e2[0] = ct; e2[1] = D(0); e2[2] = -st;
  e3[0] = D(0); e3[1] = D(1); e3[2] = D(0);
}

// The ray's own plane: unit position xh, the unit part et of the launch
// direction d0 normal to xh, and en = xh x et; psi is the angle from xh to d0.
// A (near-)radial launch has no plane; any normal serves, its deflection is 0.
template <typename D>
__device__ __forceinline__ void ray_plane(const D* xh, const D* d0, D* et, D* en, D* psi) {
  const D c = xh[0] * d0[0] + xh[1] * d0[1] + xh[2] * d0[2];
  D t[3] = {d0[0] - c * xh[0], d0[1] - c * xh[1], d0[2] - c * xh[2]};
  D sn = sqrt_(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  if (!(sn > D(1e-7))) {
    // any unit normal of xh
    const D ax = fabs_(xh[0]) < D(0.9) ? D(1) : D(0), ay = D(1) - ax;
    const D cc = xh[0] * ax + xh[1] * ay;
    t[0] = ax - cc * xh[0]; t[1] = ay - cc * xh[1]; t[2] = -cc * xh[2];
    const D tn = sqrt_(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    t[0] /= tn; t[1] /= tn; t[2] /= tn;
  } else {
    t[0] /= sn; t[1] /= sn; t[2] /= sn;
  }
  et[0] = t[0]; et[1] = t[1]; et[2] = t[2];
  en[0] = xh[1] * t[2] - xh[2] * t[1];
  en[1] = xh[2] * t[0] - xh[0] * t[2];
  en[2] = xh[0] * t[1] - xh[1] * t[0];
  *psi = atan2_(max_(sn, D(0)), c);
}

// Exit direction d -> (in-plane deflection, out-of-plane tilt); the
// deflection is wrapped to [-pi/2, 3pi/2).
__device__ __forceinline__ void plane_angles(const double* xh, const double* d0, const double* d, double* defl,
                                             double* tilt) {
  double et[3], en[3], psi;
  ray_plane(xh, d0, et, en, &psi);
  const double cx = d[0] * xh[0] + d[1] * xh[1] + d[2] * xh[2];
  const double ct = d[0] * et[0] + d[1] * et[1] + d[2] * et[2];
  const double cn = d[0] * en[0] + d[1] * en[1] + d[2] * en[2];
  const double two_pi = 6.283185307179586;
  double D = atan2(ct, cx) - psi;
  D -= two_pi * floor((D + 1.5707963267948966) / two_pi);
  *defl = D;
  *tilt = asin(fmin(fmax(cn, -1.0), 1.0));
}

struct LabelParams {
  long long n;
  long long offset;   // Sobol index of the first sample
  float* X;           // [n][6] normalised inputs
  float* T;           // [n][8] targets
  float* raw;         // optional [n][15]: r, theta, a, n0, n1, n2, flags, steps, exit dir (3), r_cross,
                      // launch coordinate direction d0 (3)
  double dt;
};

__device__ __forceinline__ void normalise_inputs(float r, float th, float a, const float* n, float* x) {
  x[0] = (r - 27.0f) / 23.0f;
  x[1] = th / 0.78539816f - 1.0f;
  x[2] = a / 0.495f - 1.0f;
  x[3] = n[0];
  x[4] = n[1];
  x[5] = n[2];
}

// FP64 integration of one sample with the kernel's rules (no gas, no disc
// shading): exit direction on r_escape (landed), first z = 0 crossing radius
// and 1/(1+z) of the exact emitter there.
__global__ void label_kernel(const LabelParams lp) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= lp.n) return;
  const uint32_t idx = (uint32_t)(lp.offset + tid + 1);  // skip the origin point
  const float u0 = sobol(idx, 0), u1 = sobol(idx, 1), u2 = sobol(idx, 2), u3 = sobol(idx, 3), u4 = sobol(idx, 4);
  const double r = 4.0 + 46.0 * u0;
  const double th = 1.5707963267948966 * u1;
  const double a = 0.99 * u2;
  // directions: 80% uniform on the 75-degree cone around the inward radial
  // axis (every camera that looks at the hole sees its whole frame inside it),
  // 20% uniform on the rest of the sphere
  const double cmin = 0.25881904510252074;  // cos 75 deg
  const double ca = (u3 < 0.8f) ? 1.0 - (double)(u3 / 0.8f) * (1.0 - cmin)
                                : cmin - (double)((u3 - 0.8f) / 0.2f) * (1.0 + cmin);
  const double sa = sqrt(fmax(1.0 - ca * ca, 0.0)), ph = 6.283185307179586 * u4;
  const double nv[3] = {-ca, sa * cos(ph), sa * sin(ph)};
  const double M = 1.0;
  const double pos[3] = {sqrt(r * r + a * a) * sin(th), 0.0, r * cos(th)};
  double e1[3], e2[3], e3[3], U[4], E1[4], E2[4], E3[4];
  frame_axes(pos, e1, e2, e3);
  static_frame(pos, e1, e2, e3, M, a, U, E1, E2, E3);
  double q[4];
  for (int k = 0; k < 4; ++k) q[k] = nv[0] * E1[k] + nv[1] * E2[k] + nv[2] * E3[k] - U[k];
  double y[6], pt;
  if (a != 0.0) lower_photon<1>(pos, q, M, a, y, &pt);
  else lower_photon<0>(pos, q, M, a, y, &pt);
  bool cap0 = false, graze0 = false;
  if (a != 0.0) bardeen(y, pt, M, a, &cap0, &graze0);
  // initial coordinate direction (the residual's base)
  double k1[6];
  rhs_kerr(y, pt, M, a, k1);
  const double v0n = sqrt(k1[0] * k1[0] + k1[1] * k1[1] + k1[2] * k1[2]);
  const double d0[3] = {k1[0] / v0n, k1[1] / v0n, k1[2] / v0n};
  // rules of the kernel (src/metal.jl:347-357, 1201-1260, 2058-2062)
  const double rph = (a == 0.0) ? 3.0 * M : 2.0 * M * (1.0 + cos((2.0 / 3.0) * acos(-a / M)));
  const float rkf = (float)(0.995 * rph);
  const double rkill2 = (double)(rkf * rkf);
  const double rpos = sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
  const double r_esc = (double)(float)(2.0 * fmax(rpos, 15.0 * M));
  const int nmax = (int)fmin(fmax(1000.0, ceil((75.0 + 6.5 * log(r_esc / M)) * M / lp.dt)), 40000.0);
  double r_isco, E_isco, L_isco;
  {
    auto cb = [](double x) { return exp(log(fmax(x, 1e-12)) / 3.0); };
    const double qq = a / M;
    const double z1 = 1.0 + cb(1.0 - qq * qq) * (cb(1.0 + qq) + cb(1.0 - qq));
    const double z2 = sqrt(3.0 * qq * qq + z1 * z1);
    r_isco = M * (3.0 + z2 - sqrt(fmax((3.0 - z1) * (3.0 + z1 + 2.0 * z2), 0.0)));
    E_isco = sqrt(1.0 - 2.0 * M / (3.0 * r_isco));
    L_isco = (2.0 * M / (3.0 * sqrt(3.0))) * (1.0 + 2.0 * sqrt(3.0 * r_isco / M - 2.0));
  }
  int flags = 0, steps = 0;
  float r_cross = -1.f, g_cross = 0.f;
  bool done = false;
  for (; steps < nmax && !done; ++steps) {
    const double r2 = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
    const double rr = sqrt(r2);
    const double rk2 = ks_r2(y[0], y[1], y[2], a);
    if (rk2 < rkill2) { flags |= ST_RAY_CAPTURED; break; }
    if (rr > r_esc) { flags |= ST_RAY_ESCAPED; break; }
    double h = lp.dt * fmin(fmax(0.16 * rr / M, 1.0), 8.0);
    const double fr = fmin(fmax((rk2 - rkill2) / fmax(rkill2, 1e-6), 0.0), 1.0);
    h *= 0.12 + 0.88 * fr;
    double yp[6], inc[6];
    for (int k = 0; k < 6; ++k) yp[k] = y[k];
    rhs_kerr(y, pt, M, a, k1);
    rk4_inc<1>(y, pt, M, a, h, k1, inc);
    for (int k = 0; k < 6; ++k) y[k] += inc[k];
    if (!(y[0] == y[0]) || !(y[3] == y[3])) { flags |= ST_RAY_CAPTURED; break; }
    if (r_cross < 0.f && yp[2] * y[2] < 0.0) {
      const double cfz = yp[2] / (yp[2] - y[2]);
      const double xh = yp[0] + cfz * (y[0] - yp[0]), yh = yp[1] + cfz * (y[1] - yp[1]);
      const double pxh = yp[3] + cfz * (y[3] - yp[3]), pyh = yp[4] + cfz * (y[4] - yp[4]);
      r_cross = (float)sqrt(xh * xh + yh * yh);
      g_cross = (float)(1.0 / emitter_opz(xh, yh, pxh, pyh, -pt, M, a, r_isco, E_isco, L_isco));
    }
    const double rn = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    if (rn > r_esc) {
      // land on r_escape, as the render path does
      double yt[6];
      land_on_sphere<1>(yp, pt, M, a, h, k1, rr, rn, r_esc, yt);
      for (int k = 0; k < 6; ++k) y[k] = yt[k];
      flags |= ST_RAY_ESCAPED;
      done = true;
    }
  }
  if (!(flags & (ST_RAY_ESCAPED | ST_RAY_CAPTURED))) flags |= ST_RAY_BUDGET;
  if (cap0) flags |= ST_RAY_BCAPT;
  if (graze0) flags |= ST_RAY_GRAZE;
  double vel[6];
  rhs_kerr(y, pt, M, a, vel);
  const double vl = fmax(sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]), 1e-20);
  const bool ok = (flags & ST_RAY_ESCAPED) && !cap0 && !(flags & ST_RAY_BUDGET);
  float x[6];
  const float nf[3] = {(float)nv[0], (float)nv[1], (float)nv[2]};
  normalise_inputs((float)r, (float)th, (float)a, nf, x);
  float* Xo = lp.X + tid * NIN;
  for (int k = 0; k < NIN; ++k) Xo[k] = x[k];
  float* To = lp.T + tid * NT;
  double defl = 0.0, tilt = 0.0;
  if (ok) {
    const double xh[3] = {pos[0] / rpos, pos[1] / rpos, pos[2] / rpos};
    const double dex[3] = {vel[0] / vl, vel[1] / vl, vel[2] / vl};
    plane_angles(xh, d0, dex, &defl, &tilt);
  }
  To[0] = (float)defl;
  To[1] = (float)tilt;
  To[2] = 0.f;
  To[3] = (r_cross > 0.f ? fminf(10.f / r_cross, 5.f) : 0.f) - 1.f;  // 10/s - 1; no crossing = s -> inf
  To[4] = r_cross > 0.f ? g_cross - 1.f : 0.f;
  To[5] = ok ? 1.f : 0.f;
  To[6] = r_cross > 0.f ? 1.f : 0.f;
  To[7] = 0.f;
  if (lp.raw) {
    float* Ro = lp.raw + tid * NRAW;
    Ro[0] = (float)r; Ro[1] = (float)th; Ro[2] = (float)a;
    Ro[3] = nf[0]; Ro[4] = nf[1]; Ro[5] = nf[2];
    Ro[6] = (float)flags; Ro[7] = (float)steps;
    Ro[8] = (float)(vel[0] / vl); Ro[9] = (float)(vel[1] / vl); Ro[10] = (float)(vel[2] / vl);
    Ro[11] = r_cross;
    Ro[12] = (float)d0[0]; Ro[13] = (float)d0[1]; Ro[14] = (float)d0[2];
  }
}

// ---------------------------------------------------------------------------
// Frame pass: camera rays -> network inputs -> MLP -> gate, fused
// ---------------------------------------------------------------------------

// Network inputs of one pixel's camera ray.  The ray is built as the trace
// kernel builds it (init_ray, in FP32: the network input is float, and an
// FP64 pass over every pixel would cost more than the network on GB300's
// FP64 rate), raised to its tangent q = (-p_t + f l, p - f l L) and projected
// on the static observer's frame.  aux = (unit launch coordinate direction,
// camera shift); fl = launch flags (Bardeen capture / graze, Schwarzschild
// critical band).
template <int KERR>
__device__ __forceinline__ void pixel_inputs(const TraceParams& p, const SurFrame& f, int pix, float* x, float4* aux,
                                             int* fl) {
  const int i = pix % p.width, j = pix / p.width;
  RayState<float> st;
  const CamView cam{p.pos, p.Ef, p.Er, p.Eu, p.U, p.r_escape, p.nmax};
  init_ray<ST_PREC_FP32, KERR, ST_SEM_DRAFT>(p, cam, i, j, st);
  const float* y = st.y;
  const float pt = st.pt, a = (float)p.a, M = (float)p.M;
  float L[3], fk;
  if (KERR) {
    const float r2 = fmaxf(ks_r2(y[0], y[1], y[2], a), 1e-12f), r = sqrtf(r2), ira = 1.f / (r2 + a * a);
    L[0] = (r * y[0] + a * y[1]) * ira;
    L[1] = (r * y[1] - a * y[0]) * ira;
    L[2] = y[2] / r;
    fk = 2.f * M * r2 * r / (r2 * r2 + a * a * y[2] * y[2]);
  } else {
    const float r = sqrtf(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    L[0] = y[0] / r; L[1] = y[1] / r; L[2] = y[2] / r;
    fk = 2.f * M / r;
  }
  const float ell = -pt + L[0] * y[3] + L[1] * y[4] + L[2] * y[5];
  const float q[4] = {-pt + fk * ell, y[3] - fk * ell * L[0], y[4] - fk * ell * L[1], y[5] - fk * ell * L[2]};
  auto dot4 = [&](const double* c) {
    return q[0] * (float)c[0] + q[1] * (float)c[1] + q[2] * (float)c[2] + q[3] * (float)c[3];
  };
  const float al = fabsf(dot4(f.Ul));
  const float n[3] = {dot4(f.E1l) / al, dot4(f.E2l) / al, dot4(f.E3l) / al};
  normalise_inputs((float)f.r, (float)f.th, a, n, x);
  const float qn = sqrtf(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  *aux = make_float4(q[1] / qn, q[2] / qn, q[3] / qn, st.scam);
  int flags = st.flags & (ST_RAY_BCAPT | ST_RAY_GRAZE);
  if (!KERR) {
    // Schwarzschild critical band: b = |x cross p| / E against 3 sqrt(3) M
    const float Lx = y[1] * y[5] - y[2] * y[4], Ly = y[2] * y[3] - y[0] * y[5], Lz = y[0] * y[4] - y[1] * y[3];
    const float b = sqrtf(Lx * Lx + Ly * Ly + Lz * Lz) / fabsf(pt);
    const float bc = (float)p.b_crit;
    if (b < bc) flags |= ST_RAY_BCAPT;
    if (fabsf(b - bc) < fmaxf((float)p.crit_band, 0.05f)) flags |= ST_RAY_GRAZE;
  }
  *fl = flags;
}

// Gate of one pixel: serve it from the network when it is not near the
// critical curve, the predicted std-dev of its exit angles is below
// sigma_max and it is predicted not to cross the disc annulus.  A served
// pixel gets its sky colour (exit direction rebuilt from the ray-plane
// angles) in *rgba and its direction in dird.
__device__ __forceinline__ bool gate_pixel(const TraceParams& p, const SurFrame& f, const float* o, float4 a4, int fl,
                                           float4* rgba, double* dird) {
  const float sig = __expf(0.5f * fminf(fmaxf(o[5], -30.f), 12.f));
  bool serve = (fl & (ST_RAY_BCAPT | ST_RAY_GRAZE)) == 0 && sig < (float)f.sigma_max;
  if (serve && p.disc_on) {
    const float u = o[3] + 1.f;  // 10 / s
    const float sc = u > 0.02f ? 10.f / u : 1e9f;
    if (sc > (float)p.disc_inner - 1.5f && sc < (float)p.disc_outer + 3.0f) serve = false;
  }
  if (!serve) return false;
  const float xh[3] = {(float)f.xh[0], (float)f.xh[1], (float)f.xh[2]};
  const float dl[3] = {a4.x, a4.y, a4.z};
  float et[3], en[3], psi;
  ray_plane(xh, dl, et, en, &psi);
  float sc, cc, se, ce;
  __sincosf(psi + o[0], &sc, &cc);
  __sincosf(o[1], &se, &ce);
  const float dx = ce * (cc * xh[0] + sc * et[0]) + se * en[0];
  const float dy = ce * (cc * xh[1] + sc * et[1]) + se * en[1];
  const float dz = ce * (cc * xh[2] + sc * et[2]) + se * en[2];
  const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
  const float d0 = dx * inv, d1 = dy * inv, d2 = dz * inv;
  dird[0] = d0; dird[1] = d1; dird[2] = d2;
  float sky[3];
  sample_sky(p, acosf(fminf(fmaxf(d2, -1.f), 1.f)), atan2f(d1, d0), sky);
  if (p.star_strength > 0.0) {
    float sl[3];
    star_light<ST_SEM_DRAFT>(p, d0, d1, d2, sl);
    const float tw = (float)p.star_tw, ss = (float)p.star_strength;
    for (int c = 0; c < 3; ++c) sky[c] = sky[c] * tw + ss * sl[c];
  }
  const float g = a4.w;
  if (g != 1.f) {
    sky[0] *= 57.4f / (__expf(4.067f / g) - 1.f);
    sky[1] *= 90.2f / (__expf(4.513f / g) - 1.f);
    sky[2] *= 206.5f / (__expf(5.335f / g) - 1.f);
  }
  *rgba = make_float4(p.weight * sky[0], p.weight * sky[1], p.weight * sky[2], 1.f);
  return true;
}

// One CTA = 128 pixels = 128 network rows, 8 warps; warp w owns rows
// 16w..16w+15 through all layers.  Shared memory holds the activation tile
// (bf16, 128 x 256) and one hidden layer's weights (bf16, 256 x 256, loaded
// with cp.async from L2 while the previous layer's epilogue runs), so no
// activation leaves the SM.  Hidden layers: mma.sync m16n8k16 BF16 with FP32
// accumulate, 32 accumulator tiles per warp; the 6 -> 256 and 256 -> 6 edge
// layers run in FP32 (the last one straight from the layer-3 accumulators,
// rounded to bf16 as the unfused forward stores them).
constexpr int FROWS = 128, FTHREADS = 256, FS = NH + 8;
constexpr size_t F_SMEM = (size_t)FROWS * FS * 2      // activations
                          + (size_t)NH * FS * 2       // one hidden layer's weights
                          + (size_t)NOUT * NH * 4     // W4
                          + (size_t)FROWS * NIN * 4   // inputs
                          + (size_t)FROWS * NOUT * 4  // outputs
                          + (size_t)FROWS * 16        // aux
                          + (size_t)FROWS * 4;        // launch flags
static_assert(F_SMEM <= 227 * 1024, "fused surrogate tile exceeds shared memory");

__device__ __forceinline__ void load_hidden_weights(__nv_bfloat16* Ws, const __nv_bfloat16* W, int tid) {
  // 256 rows x 32 chunks of 16 bytes
#pragma unroll 4
  for (int c = tid; c < NH * (NH / 8); c += FTHREADS) {
    const int r = c >> 5, q = c & 31;
    mlp::cp_async16(Ws + r * FS + q * 8, W + (size_t)r * NH + q * 8);
  }
  mlp::cp_async_commit();
}

template <int KERR>
__global__ void __launch_bounds__(FTHREADS, 1)
    sur_frame_kernel(const __grid_constant__ TraceParams p, const __grid_constant__ SurFrame f,
                     const float* __restrict__ P, const __nv_bfloat16* __restrict__ W1,
                     const __nv_bfloat16* __restrict__ W2, const __nv_bfloat16* __restrict__ W3, int* list,
                     int* count) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __nv_bfloat16* Hs = reinterpret_cast<__nv_bfloat16*>(fsm);
  __nv_bfloat16* Ws = Hs + FROWS * FS;
  float* W4s = reinterpret_cast<float*>(Ws + NH * FS);
  float* Xs = W4s + NOUT * NH;
  float* Os = Xs + FROWS * NIN;
  float4* As = reinterpret_cast<float4*>(Os + FROWS * NOUT);
  int* Fs = reinterpret_cast<int*>(As + FROWS);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the CTA's 128 pixels are a 16 x 8 tile; each of the gating warps 0-3
  // holds an 8 x 4 block, the warp shape of the trace kernel, so the list of
  // pixels left to integrate keeps that coherence
  const int tiles_x = (p.width + 15) >> 4;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  int my_pix = -1;
  if (tid < FROWS) {
    const int wq = tid >> 5, l = tid & 31;
    const int i = tx * 16 + (wq & 1) * 8 + (l & 7), j = ty * 8 + (wq >> 1) * 4 + (l >> 3);
    if (i < p.width && j < p.height) my_pix = j * p.width + i;
  }
  load_hidden_weights(Ws, W1, tid);
  for (int c = tid; c < NOUT * NH; c += FTHREADS) W4s[c] = P[OW4 + c];
  if (tid < FROWS) {
    float x[NIN] = {0, 0, 0, 0, 0, 0};
    float4 a4 = make_float4(0.f, 0.f, 1.f, 1.f);
    int fl = ST_RAY_GRAZE;
    if (my_pix >= 0) pixel_inputs<KERR>(p, f, my_pix, x, &a4, &fl);
#pragma unroll
    for (int k = 0; k < NIN; ++k) Xs[tid * NIN + k] = x[k];
    As[tid] = a4;
    Fs[tid] = fl;
  }
  __syncthreads();
  // layer 0 (FP32): thread = hidden unit n, all 128 rows
  {
    const int n = tid;
    float w0[NIN];
#pragma unroll
    for (int i = 0; i < NIN; ++i) w0[i] = P[OW0 + n * NIN + i];
    const float b0 = P[OB0 + n];
    for (int r = 0; r < FROWS; ++r) {
      float z = b0;
#pragma unroll
      for (int i = 0; i < NIN; ++i) z += Xs[r * NIN + i] * w0[i];
      Hs[r * FS + n] = __float2bfloat16_rn(mlp::silu(z));
    }
  }
  mlp::cp_async_wait0();
  __syncthreads();
  const int g = lane >> 2, t2 = (lane & 3) * 2;
  const int row0 = warp * 16;
  float o4[2][NOUT];
#pragma unroll
  for (int l = 1; l <= 3; ++l) {
    float acc[32][4];
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 1
    for (int kk = 0; kk < NH; kk += 16) {
      uint32_t af[4];
      mlp::ldsm_x4(af, Hs + (row0 + (lane & 15)) * FS + kk + (lane >> 4) * 8);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        uint32_t bfr[4];
        mlp::ldsm_x4(bfr, Ws + (j * 16 + (lane & 7) + (lane >> 4) * 8) * FS + kk + ((lane >> 3) & 1) * 8);
        mlp::mma_bf16(acc[2 * j], af, bfr[0], bfr[1]);
        mlp::mma_bf16(acc[2 * j + 1], af, bfr[2], bfr[3]);
      }
    }
    __syncthreads();  // every warp is done with this layer's weights
    if (l < 3) load_hidden_weights(Ws, l == 1 ? W2 : W3, tid);
    const float* bias = P + (l == 1 ? OB1 : l == 2 ? OB2 : OB3);
    if (l < 3) {
      // this warp's rows only: no other warp reads them
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int n = j * 8 + t2;
        const float bn0 = bias[n], bn1 = bias[n + 1];
        *reinterpret_cast<__nv_bfloat162*>(Hs + (row0 + g) * FS + n) =
            __floats2bfloat162_rn(mlp::silu(acc[j][0] + bn0), mlp::silu(acc[j][1] + bn1));
        *reinterpret_cast<__nv_bfloat162*>(Hs + (row0 + g + 8) * FS + n) =
            __floats2bfloat162_rn(mlp::silu(acc[j][2] + bn0), mlp::silu(acc[j][3] + bn1));
      }
      mlp::cp_async_wait0();
      __syncthreads();
    } else {
      // layer 4 from the accumulators: rows g and g+8 of this warp, 64 columns
#pragma unroll
      for (int k = 0; k < NOUT; ++k) o4[0][k] = o4[1][k] = 0.f;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int n = j * 8 + t2;
        const float bn0 = bias[n], bn1 = bias[n + 1];
        const float h00 = __bfloat162float(__float2bfloat16_rn(mlp::silu(acc[j][0] + bn0)));
        const float h01 = __bfloat162float(__float2bfloat16_rn(mlp::silu(acc[j][1] + bn1)));
        const float h10 = __bfloat162float(__float2bfloat16_rn(mlp::silu(acc[j][2] + bn0)));
        const float h11 = __bfloat162float(__float2bfloat16_rn(mlp::silu(acc[j][3] + bn1)));
#pragma unroll
        for (int k = 0; k < NOUT; ++k) {
          const float w0 = W4s[k * NH + n], w1 = W4s[k * NH + n + 1];
          o4[0][k] += h00 * w0 + h01 * w1;
          o4[1][k] += h10 * w0 + h11 * w1;
        }
      }
    }
  }
  // reduce over the quad (the 4 lanes sharing rows g, g+8)
#pragma unroll
  for (int k = 0; k < NOUT; ++k) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      o4[h][k] += __shfl_xor_sync(0xffffffffu, o4[h][k], 1);
      o4[h][k] += __shfl_xor_sync(0xffffffffu, o4[h][k], 2);
    }
  }
  if ((lane & 3) == 0) {
#pragma unroll
    for (int k = 0; k < NOUT; ++k) {
      Os[(row0 + g) * NOUT + k] = o4[0][k] + P[OB4 + k];
      Os[(row0 + g + 8) * NOUT + k] = o4[1][k] + P[OB4 + k];
    }
  }
  __syncthreads();
  if (tid >= FROWS) return;  // warps 0-3 gate the tile (whole warps: ballots stay full)
  const int pix = my_pix;
  float4 rgba = make_float4(0.f, 0.f, 0.f, 1.f);
  double dird[3] = {0, 0, 0};
  const bool serve = pix >= 0 && gate_pixel(p, f, Os + tid * NOUT, As[tid], Fs[tid], &rgba, dird);
  const unsigned want = __ballot_sync(0xffffffffu, pix >= 0 && !serve);
  int base = 0;
  if (lane == 0 && want) base = atomicAdd(count, __popc(want));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (pix < 0) return;
  if (serve) {
    p.out[pix] = rgba;
    if (p.diag) {
      st_ray_diag d;
      d.dir[0] = dird[0]; d.dir[1] = dird[1]; d.dir[2] = dird[2];
      d.r_final = 0.f; d.alpha = 1.f; d.r_cross = -1.f; d.g_cross = 0.f; d.lambda = 0.f;
      d.flags = ST_RAY_SURROGATE | ST_RAY_ESCAPED;
      d.steps = 0; d.fp64_steps = 0; d.pad[0] = d.pad[1] = 0;
      p.diag[pix] = d;
    }
  } else {
    list[base + __popc(want & ((1u << lane) - 1u))] = pix;
  }
}

// ---------------------------------------------------------------------------
// The same frame pass on the 5th-generation tensor cores (tcgen05 + TMEM)
// ---------------------------------------------------------------------------
//
// The network pass on the tensor cores (sur_mlp_tc_kernel): a persistent CTA
// per SM takes 128-row tiles in turn, 16 warps.  All five layers are
// tcgen05.mma (M = 128, FP32 accumulator of 256 TMEM columns) with both
// operands K-major, 128-byte-swizzled bf16 in shared memory:
//  - layer 0 (6 -> 256, FP32 in the unfused forward) as one K = 32 product in
//    split bf16: A row = (x_hi, x_lo, x_hi, 1, 1), B row n = (w_hi, w_hi, w_lo,
//    b_hi, b_lo), so x.w + b is carried to ~2^-16 relative (x_lo.w_lo dropped);
//  - hidden layers 1-3 (256 -> 256, bf16 in the unfused forward too);
//  - layer 4 (256 -> 6, FP32 weights on the bf16-rounded last activations) as
//    N = 16: rows 0-5 w_hi, rows 8-13 w_lo, summed in the epilogue.
// Each layer's weights come by bulk copy into one 128 KB buffer, the next
// layer's while the current epilogue runs (tcgen05.ld, warp w: TMEM lanes
// 32 (w mod 4).., columns 64 (w / 4)..; bias, SiLU, bf16 into the activation
// tile for the next MMA).  Layer 4's 8 KB image stays resident, so the next
// tile's layer-0 weights and inputs are copied as soon as layer 3's MMAs are
// done, behind layer 3's epilogue and layer 4.  The epilogue and the MMAs run
// in turn, not overlapped: schedules that ran the next layer's MMAs under the
// epilogue (two accumulators, the activations handed over by halves or by
// quarters) measured slower.
//
// Every wait on an mbarrier is bounded; a wait that runs out leaves the CTA's
// current and remaining tiles marked failed (the host sets every tile status
// to -1 before the launch, a finished tile writes 0), so their pixels all go
// to the integrator and the frame stays exact, and sets the status word.
// Before the CTA frees its TMEM and exits, the thread that issued the copies
// and the MMAs waits again (bounded) for the one operation of each barrier
// still outstanding -- the last armed copy and the last committed MMA batch --
// so that neither lands in shared memory or TMEM the CTA no longer owns.
constexpr uint32_t TC_ROWS = 128, TC_THREADS = 512;
constexpr uint32_t TC_A_BYTES = TC_ROWS * NH * 2;  // 64 KB activation tile
constexpr uint32_t TC_B_BYTES = NH * NH * 2;       // 128 KB hidden-layer weights
constexpr uint32_t TC_W0_BYTES = NH * 128;         // layer 0: 256 rows x one K-block of 64
constexpr uint32_t TC_W4_ROWS = 16;
constexpr uint32_t TC_W4_BYTES = TC_W4_ROWS * NH * 2;  // layer 4: 16 rows x K = 256
constexpr size_t TC_WSW_BYTES = TC_W0_BYTES + 3 * (size_t)TC_B_BYTES + TC_W4_BYTES;
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 22;
constexpr uint32_t TC_IDESC = tc::idesc_bf16_f32(128, 256);
constexpr uint32_t TC_IDESC4 = tc::idesc_bf16_f32(128, TC_W4_ROWS);

struct TcSmall {
  // hidden biases and the output bias (FP32), in the order of the packed
  // device image Psmall (bulk copy)
  float bh[3][NH];
  float b4[8];
  float X[TC_ROWS * NIN];  // this tile's inputs (bulk copy)
  uint64_t bar_w, bar_mma;
  uint32_t tmem;
  int fail;
};
constexpr uint32_t TC_SMALL_BYTES = (3 * NH + 8) * 4;
constexpr uint32_t TC_X_BYTES = TC_ROWS * NIN * 4;
static_assert(TC_SMALL_BYTES % 16 == 0 && offsetof(TcSmall, X) == TC_SMALL_BYTES && TC_X_BYTES % 16 == 0,
              "bulk-copy sizes and alignment");
constexpr size_t TC_SMEM = 1024 + TC_A_BYTES + TC_B_BYTES + TC_W4_BYTES + sizeof(TcSmall);
static_assert(TC_SMEM <= 227 * 1024, "tensor-core surrogate tile exceeds shared memory");

// SiLU of two pre-activations on the packed FP32x2 path:
// z / (1 + 2^(-z log2 e)), with the hardware base-2 exponential and reciprocal
// approximations (ex2.approx / rcp.approx, relative error ~2^-22), a finite z
// giving a finite result (-0 when 2^(-z log2 e) overflows).  (A reciprocal by
// Newton steps on the FMA pipe, one MUFU operation per value instead of two,
// measured slower: the epilogue is bound by issue, not by the MUFU pipe.)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 silu2(float2 z) {
  const float2 t = __fmul2_rn(z, make_float2(-1.4426950408889634f, -1.4426950408889634f));
  const float2 d = __fadd2_rn(make_float2(ex2_approx(t.x), ex2_approx(t.y)), make_float2(1.f, 1.f));
  return __fmul2_rn(z, make_float2(rcp_approx(d.x), rcp_approx(d.y)));
}

// bf16 pair (hi, lo) of an FP32 value: v = hi + lo to ~2^-16 relative.
__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16* hi, __nv_bfloat16* lo) {
  *hi = __float2bfloat16_rn(v);
  *lo = __float2bfloat16_rn(v - __bfloat162float(*hi));
}

// P (FP32 master weights) -> the weight images of the tcgen05 network pass:
// [layer 0, 32 KB][hidden layers 1-3, 128 KB each][layer 4, 8 KB].
__global__ void pack_sw128(const float* __restrict__ P, unsigned char* __restrict__ Wsw) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int nh = 3 * NH * NH, n0 = NH * 64, n4 = TC_W4_ROWS * NH;
  if (idx < nh) {
    const int l = idx / (NH * NH), rem = idx - l * NH * NH;
    const int n = rem / NH, k = rem - n * NH;
    *reinterpret_cast<__nv_bfloat16*>(Wsw + TC_W0_BYTES + (size_t)l * TC_B_BYTES + tc::sw128_off(n, k, NH)) =
        __float2bfloat16_rn(P[(l == 0 ? OW1 : l == 1 ? OW2 : OW3) + (size_t)n * NH + k]);
  } else if (idx < nh + n0) {
    // layer 0, row n: k 0-5 w_hi, 6-11 w_hi, 12-17 w_lo, 18 b_hi, 19 b_lo, then 0
    const int n = (idx - nh) >> 6, k = (idx - nh) & 63;
    __nv_bfloat16 hi, lo, v = __float2bfloat16_rn(0.f);
    if (k < 18) {
      split_bf16(P[OW0 + n * NIN + k % 6], &hi, &lo);
      v = k < 12 ? hi : lo;
    } else if (k < 20) {
      split_bf16(P[OB0 + n], &hi, &lo);
      v = k == 18 ? hi : lo;
    }
    *reinterpret_cast<__nv_bfloat16*>(Wsw + tc::sw128_off(n, k, NH)) = v;
  } else if (idx < nh + n0 + n4) {
    // layer 4, row n: 0-5 w_hi of output n, 8-13 w_lo of output n - 8, else 0
    const int n = (idx - nh - n0) / NH, k = (idx - nh - n0) % NH;
    __nv_bfloat16 hi, lo, v = __float2bfloat16_rn(0.f);
    const int o = n & 7;
    if (o < NOUT) {
      split_bf16(P[OW4 + o * NH + k], &hi, &lo);
      v = n < 8 ? hi : lo;
    }
    *reinterpret_cast<__nv_bfloat16*>(Wsw + TC_W0_BYTES + 3 * (size_t)TC_B_BYTES + tc::sw128_off(n, k, TC_W4_ROWS)) =
        v;
  }
}
constexpr int TC_PACK_N = 3 * NH * NH + NH * 64 + TC_W4_ROWS * NH;

// Pixel of row `r` (0..127) of tile `t`: each 32-row group is an 8 x 4 block
// of the 16 x 8 tile, the warp shape of the trace kernel; -1 off the frame.
__device__ __forceinline__ int tile_pixel(const TraceParams& p, int t, int r) {
  const int tiles_x = (p.width + 15) >> 4;
  const int tx = t % tiles_x, ty = t / tiles_x;
  const int wq = r >> 5, l = r & 31;
  const int i = tx * 16 + (wq & 1) * 8 + (l & 7), j = ty * 8 + (wq >> 1) * 4 + (l >> 3);
  return (i < p.width && j < p.height) ? j * p.width + i : -1;
}

// The hidden and output biases packed as TcSmall holds them.
__global__ void pack_small(const float* __restrict__ P, float* __restrict__ S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int n1 = 3 * NH, n2 = n1 + 8;
  if (i >= n2) return;
  float v;
  if (i < n1) v = P[(i < NH ? OB1 : i < 2 * NH ? OB2 : OB3) + i % NH];
  else v = (i - n1) < NOUT ? P[OB4 + (i - n1)] : 0.f;
  S[i] = v;
}

// Network inputs of every pixel, row-ordered by tile (one thread per pixel).
template <int KERR>
__global__ void __launch_bounds__(128) sur_inputs_kernel(const __grid_constant__ TraceParams p,
                                                          const __grid_constant__ SurFrame f, float* __restrict__ X,
                                                          float4* __restrict__ aux, int* __restrict__ fl) {
  const int row = blockIdx.x * 128 + threadIdx.x;
  const int pix = tile_pixel(p, blockIdx.x, threadIdx.x);
  float x[NIN] = {0, 0, 0, 0, 0, 0};
  float4 a4 = make_float4(0.f, 0.f, 1.f, 1.f);
  int flags = ST_RAY_GRAZE;
  if (pix >= 0) pixel_inputs<KERR>(p, f, pix, x, &a4, &flags);
#pragma unroll
  for (int k = 0; k < NIN; ++k) X[(size_t)row * NIN + k] = x[k];
  aux[row] = a4;
  fl[row] = flags;
}

// Gate of every pixel from the network's outputs (one thread per pixel).
// Served pixels are written; each warp records which of its pixels are left
// to integrate (mask, count) for the ordered compaction below.
__global__ void __launch_bounds__(128) sur_gate_kernel(const __grid_constant__ TraceParams p,
                                                        const __grid_constant__ SurFrame f,
                                                        const float* __restrict__ O, const float4* __restrict__ aux,
                                                        const int* __restrict__ fl, const int* __restrict__ status,
                                                        unsigned* __restrict__ wmask, int* __restrict__ wcount) {
  const int row = blockIdx.x * 128 + threadIdx.x, lane = threadIdx.x & 31;
  const int pix = tile_pixel(p, blockIdx.x, threadIdx.x);
  float o[NOUT];
#pragma unroll
  for (int k = 0; k < NOUT; ++k) o[k] = O[(size_t)row * NOUT + k];
  float4 rgba = make_float4(0.f, 0.f, 0.f, 1.f);
  double dird[3] = {0, 0, 0};
  // a tile whose network pass failed (status[t] != 0) is integrated whole
  const bool serve = pix >= 0 && status[blockIdx.x] == 0 && gate_pixel(p, f, o, aux[row], fl[row], &rgba, dird);
  const unsigned want = __ballot_sync(0xffffffffu, pix >= 0 && !serve);
  if (lane == 0) {
    wmask[row >> 5] = want;
    wcount[row >> 5] = __popc(want);
  }
  if (pix < 0 || !serve) return;
  p.out[pix] = rgba;
  if (p.diag) {
    st_ray_diag d;
    d.dir[0] = dird[0]; d.dir[1] = dird[1]; d.dir[2] = dird[2];
    d.r_final = 0.f; d.alpha = 1.f; d.r_cross = -1.f; d.g_cross = 0.f; d.lambda = 0.f;
    d.flags = ST_RAY_SURROGATE | ST_RAY_ESCAPED;
    d.steps = 0; d.fp64_steps = 0; d.pad[0] = d.pad[1] = 0;
    p.diag[pix] = d;
  }
}

// Exclusive prefix sum of the per-warp counts in one CTA of 1024 threads,
// and the total into *count.  The counts go through in chunks of 1024 in
// index order (thread t takes entry base + t); each thread first loads its
// entries of eight chunks (coalesced, independent loads), then the chunks are
// scanned one after another: warp scans by shuffle, the 32 warp totals by
// one more warp, and a running carry.
__global__ void __launch_bounds__(1024) sur_scan_kernel(const int* __restrict__ wcount, int* __restrict__ woff,
                                                         int nwarps, int* count) {
  constexpr int U = 8;
  __shared__ int wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  int carry = 0;
  for (int base = 0; base < nwarps; base += 1024 * U) {
    int v[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int idx = base + k * 1024 + t;
      v[k] = idx < nwarps ? wcount[idx] : 0;
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      int x = v[k];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) wsum[w] = x;
      __syncthreads();
      if (w == 0) {
        int s = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, s, o);
          if (lane >= o) s += y;
        }
        wsum[lane] = s;  // inclusive over warps
      }
      __syncthreads();
      const int idx = base + k * 1024 + t;
      if (idx < nwarps) woff[idx] = carry + (w > 0 ? wsum[w - 1] : 0) + x - v[k];
      carry += wsum[31];
      __syncthreads();  // every thread has read wsum before the next chunk writes it
    }
  }
  if (t == 0) *count = carry;
}

// Pixels left to integrate, in tile raster order (warp by warp).
__global__ void __launch_bounds__(128) sur_scatter_kernel(const __grid_constant__ TraceParams p,
                                                           const unsigned* __restrict__ wmask,
                                                           const int* __restrict__ woff, int* __restrict__ list) {
  const int row = blockIdx.x * 128 + threadIdx.x, lane = threadIdx.x & 31;
  const unsigned m = wmask[row >> 5];
  if (!((m >> lane) & 1u)) return;
  list[woff[row >> 5] + __popc(m & ((1u << lane) - 1u))] = tile_pixel(p, blockIdx.x, threadIdx.x);
}

// The network on the tensor cores: X[ntiles*128][6] -> O[ntiles*128][6].
// Persistent: CTA b takes tiles b, b + gridDim.x, ...; a finished tile writes
// tile_status[t] = 0 (the host sets -1 before the launch).  wait_limit bounds
// every mbarrier wait (polls); issue_first = 0 leaves the first copies
// unissued, so the first wait runs out with nothing in flight -- the failure
// path's test.
__global__ void __launch_bounds__(TC_THREADS, 1)
    sur_mlp_tc_kernel(const float* __restrict__ Psmall, const unsigned char* __restrict__ Wsw,
                      const float* __restrict__ X, float* __restrict__ O, int* __restrict__ tile_status, int ntiles,
                      unsigned long long* counters, uint32_t wait_limit, int issue_first) {
  extern __shared__ unsigned char tsm_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tsm_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char* As = base;                // activations, 128 x 256
  unsigned char* Bs = base + TC_A_BYTES;   // the current layer's weights
  unsigned char* W4s = Bs + TC_B_BYTES;    // layer 4, resident
  TcSmall& S = *reinterpret_cast<TcSmall*>(W4s + TC_W4_BYTES);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    tc::mbar_init(&S.bar_w, 1);
    tc::mbar_init(&S.bar_mma, 1);
    S.fail = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, TC_TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const uint32_t a_addr = tc::smem_u32(As), b_addr = tc::smem_u32(Bs), w4_addr = tc::smem_u32(W4s);
  // warp w: TMEM lanes (rows) 32 (w mod 4).., columns 64 (w div 4)..
  const uint32_t q = warp & 3, cq = warp >> 2;
  const int row = (int)(q * 32 + lane);
  const uint32_t t_lane = tmem + ((q * 32u) << 16);
  // parity of the next phase of each barrier (every thread keeps the count);
  // thread 0 also records the last phase it armed / committed and whether it
  // has seen that phase complete
  uint32_t pw = 0, pm = 0, w_par = 0, m_par = 0;
  bool w_out = false, m_out = false;
  int t = blockIdx.x;
  if (tid == 0 && issue_first && t < ntiles) {
    tc::mbar_expect_tx(&S.bar_w, TC_W4_BYTES + TC_SMALL_BYTES + TC_W0_BYTES + TC_X_BYTES);
    tc::bulk_g2s(W4s, Wsw + TC_W0_BYTES + 3 * (size_t)TC_B_BYTES, TC_W4_BYTES, &S.bar_w);
    tc::bulk_g2s(S.bh, Psmall, TC_SMALL_BYTES, &S.bar_w);
    tc::bulk_g2s(Bs, Wsw, TC_W0_BYTES, &S.bar_w);
    tc::bulk_g2s(S.X, X + (size_t)t * TC_ROWS * NIN, TC_X_BYTES, &S.bar_w);
    w_out = true;
    w_par = pw;
  }
  for (; t < ntiles; t += gridDim.x) {
    // this tile's inputs and layer-0 weights (on the first tile also layer 4
    // and the biases); one thread waits, the CTA barrier releases the rest
    if (tid == 0) {
      if (!tc::mbar_wait(&S.bar_w, pw, wait_limit)) S.fail = 1;
      else w_out = false;
    }
    pw ^= 1u;
    __syncthreads();
    if (S.fail) break;
    {
      // layer 0's A tile, K 0..31: thread = (row r, 16-byte chunk c)
      const int r = tid >> 2, c = tid & 3;
      uint32_t pk[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        __nv_bfloat16 h[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int k = c * 8 + 2 * e + u;
          __nv_bfloat16 hi, lo;
          split_bf16(S.X[r * NIN + (k < 18 ? k % 6 : 0)], &hi, &lo);
          h[u] = k < 18 ? ((k >= 6 && k < 12) ? lo : hi) : __float2bfloat16_rn(k < 20 ? 1.f : 0.f);
        }
        pk[e] = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
      }
      *reinterpret_cast<uint4*>(As + tc::sw128_off(r, c * 8, TC_ROWS)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < 2; ++s)
        tc::mma_bf16(tmem, tc::sw128_desc(a_addr + s * 32), tc::sw128_desc(b_addr + s * 32), TC_IDESC,
                     s > 0 ? 1u : 0u);
      tc::mma_commit(&S.bar_mma);
      m_out = true;
      m_par = pm;
    }
    for (int L = 0; L < 5; ++L) {
      // layer L's MMAs are done (one thread waits, as above)
      if (tid == 0) {
        if (!tc::mbar_wait(&S.bar_mma, pm, wait_limit)) S.fail = 1;
        else m_out = false;
      }
      pm ^= 1u;
      __syncthreads();
      if (S.fail) break;
      tc::fence_after_sync();
      if (tid == 0 && L < 4) {
        // the weight buffer is free: the next layer's weights, or after layer
        // 3 the next tile's layer-0 weights and inputs
        if (L < 3) {
          tc::mbar_expect_tx(&S.bar_w, TC_B_BYTES);
#pragma unroll
          for (int c = 0; c < 4; ++c)
            tc::bulk_g2s(Bs + c * 32768, Wsw + TC_W0_BYTES + (size_t)L * TC_B_BYTES + c * 32768, 32768, &S.bar_w);
          w_out = true;
          w_par = pw;
        } else if (t + (int)gridDim.x < ntiles) {
          tc::mbar_expect_tx(&S.bar_w, TC_W0_BYTES + TC_X_BYTES);
          tc::bulk_g2s(Bs, Wsw, TC_W0_BYTES, &S.bar_w);
          tc::bulk_g2s(S.X, X + (size_t)(t + gridDim.x) * TC_ROWS * NIN, TC_X_BYTES, &S.bar_w);
          w_out = true;
          w_par = pw;
        }
      }
      if (L == 4) break;
      // epilogue of layer L: bias (layers 1-3), SiLU, bf16 into the activation tile
      const float2 bm = L > 0 ? make_float2(1.f, 1.f) : make_float2(0.f, 0.f);
#pragma unroll 1
      for (int c = 0; c < 2; ++c) {
        const int col0 = (int)cq * 64 + c * 32;
        const float2* b2 = reinterpret_cast<const float2*>(S.bh[L > 0 ? L - 1 : 0] + col0);
        float v[32];
        tc::tmem_ld32(t_lane + (uint32_t)col0, v);
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          uint32_t pk[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int j = ch * 8 + 2 * e;
            const float2 h = silu2(__ffma2_rn(b2[j / 2], bm, make_float2(v[j], v[j + 1])));
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(h.x, h.y);
            pk[e] = *reinterpret_cast<const uint32_t*>(&h2);
          }
          *reinterpret_cast<uint4*>(As + tc::sw128_off(row, col0 + ch * 8, TC_ROWS)) =
              make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        bool ok = true;
        if (L < 3) {
          // layer L + 1 from the copied weights
          ok = tc::mbar_wait(&S.bar_w, pw, wait_limit);
          if (ok) {
            w_out = false;
#pragma unroll
            for (int s = 0; s < NH / 16; ++s) {
              const uint64_t ad = tc::sw128_desc(a_addr + (s >> 2) * (TC_ROWS * 128) + (s & 3) * 32);
              const uint64_t bd = tc::sw128_desc(b_addr + (s >> 2) * (NH * 128) + (s & 3) * 32);
              tc::mma_bf16(tmem, ad, bd, TC_IDESC, s > 0 ? 1u : 0u);
            }
          }
        } else {
          // layer 4 from the resident image: N = 16
#pragma unroll
          for (int s = 0; s < NH / 16; ++s) {
            const uint64_t ad = tc::sw128_desc(a_addr + (s >> 2) * (TC_ROWS * 128) + (s & 3) * 32);
            const uint64_t bd = tc::sw128_desc(w4_addr + (s >> 2) * (TC_W4_ROWS * 128) + (s & 3) * 32);
            tc::mma_bf16(tmem, ad, bd, TC_IDESC4, s > 0 ? 1u : 0u);
          }
        }
        if (ok) {
          tc::mma_commit(&S.bar_mma);
          m_out = true;
          m_par = pm;
        } else {
          S.fail = 1;
        }
      }
      if (L < 3) pw ^= 1u;
      __syncthreads();
      if (S.fail) break;
    }
    if (S.fail) break;
    // layer 4 epilogue: out = acc[hi] + acc[lo] + b4
    if (warp < 4) {
      float v[16];
      tc::tmem_ld16(t_lane, v);
      float* o = O + ((size_t)t * TC_ROWS + row) * NOUT;
#pragma unroll
      for (int k = 0; k < NOUT; ++k) o[k] = v[k] + v[k + 8] + S.b4[k];
    }
    tc::fence_before_sync();
    __syncthreads();  // the accumulator is read before the next tile's MMAs
    if (tid == 0) tile_status[t] = 0;
  }
  const bool failed = S.fail != 0;
  if (failed && tid == 0) {
    // drain: a parity wait on the last armed / committed phase returns at once
    // if it has completed and otherwise waits for it (each barrier has at most
    // one phase outstanding)
    if (w_out) (void)tc::mbar_wait(&S.bar_w, w_par, wait_limit);
    if (m_out) (void)tc::mbar_wait(&S.bar_mma, m_par, wait_limit);
    if (counters) atomicMax(counters + CNT_STATUS, (unsigned long long)ST_ECUDA);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, TC_TMEM_COLS);
  }
}

// Grid of the persistent network kernel: one CTA per SM, at most one per tile.
inline int tc_grid(int ntiles) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
    nsm = 1;
  return ntiles < nsm ? ntiles : nsm;
}

}  // namespace sur
}  // namespace st

// ---------------------------------------------------------------------------
// Host object and C ABI
// ---------------------------------------------------------------------------

extern "C" void st_surrogate_destroy(st_surrogate* s);

struct st_surrogate {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *P = nullptr, *G = nullptr, *Mm = nullptr, *Vv = nullptr;
  __nv_bfloat16* Wb[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16* Wt[3] = {nullptr, nullptr, nullptr};  // W^T (bf16) for the tcgen05 input-gradient GEMM
  // [256][cap] transposes for the weight gradient: H_0..H_2 (written by the
  // forward epilogues) and dZ (ping-pong, written by the input-gradient epilogues)
  __nv_bfloat16* HT[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16* dZT[2] = {nullptr, nullptr};
  int* d_status = nullptr;                              // tcgen05 GEMM: a bounded wait ran out
  unsigned char* Wsw = nullptr;  // hidden layers as swizzled bf16 images for the tcgen05 frame kernel
  float* Psmall = nullptr;       // FP32 edge layers and biases packed for the same kernel
  // frame-pass buffers, rows in tile order: inputs, launch data, outputs, per-tile status
  float* fX = nullptr;
  float4* fAux = nullptr;
  int* fFl = nullptr;
  float* fO = nullptr;
  int* fStatus = nullptr;
  unsigned* fMask = nullptr;  // per warp of rows: pixels left to integrate
  int* fCount = nullptr;      // per warp: their number
  int* fOff = nullptr;        // per warp: offset in the list
  long long frows = 0;
  int cap = 0;  // rows of the work buffers
  float* X = nullptr;
  float* Z[4] = {nullptr, nullptr, nullptr, nullptr};
  __nv_bfloat16* H[4] = {nullptr, nullptr, nullptr, nullptr};
  __nv_bfloat16 *dZa = nullptr, *dZb = nullptr;
  float* part = nullptr;  // block partials of the layer-0 / layer-4 weight gradients
  float *out = nullptr, *dout = nullptr, *T = nullptr, *loss = nullptr;
  // training set (device)
  float *DX = nullptr, *DT = nullptr;
  long long ndata = 0;
  long long step = 0;
  unsigned long long seed = 0;
};

namespace {

using namespace st::sur;

#define SC(call)                               \
  do {                                         \
    if ((call) != cudaSuccess) return ST_ECUDA; \
  } while (0)

int ensure_work(st_surrogate* s, int rows) {
  if (rows <= s->cap) return ST_OK;
  cudaFree(s->X);
  for (int l = 0; l < 4; ++l) { cudaFree(s->Z[l]); cudaFree(s->H[l]); }
  cudaFree(s->dZa); cudaFree(s->dZb); cudaFree(s->out); cudaFree(s->dout); cudaFree(s->T);
  for (int l = 0; l < 3; ++l) { cudaFree(s->HT[l]); s->HT[l] = nullptr; }
  for (int l = 0; l < 2; ++l) { cudaFree(s->dZT[l]); s->dZT[l] = nullptr; }
  cudaFree(s->part);
  s->part = nullptr;
  s->cap = 0;
  const size_t R = rows;
  if (cudaMalloc(&s->X, R * NIN * 4) != cudaSuccess) return ST_ENOMEM;
  for (int l = 0; l < 4; ++l) {
    if (cudaMalloc(&s->Z[l], R * NH * 4) != cudaSuccess) return ST_ENOMEM;
    if (cudaMalloc(&s->H[l], R * NH * 2) != cudaSuccess) return ST_ENOMEM;
  }
  if (cudaMalloc(&s->dZa, R * NH * 2) != cudaSuccess || cudaMalloc(&s->dZb, R * NH * 2) != cudaSuccess)
    return ST_ENOMEM;
  if (cudaMalloc(&s->out, R * NOUT * 4) != cudaSuccess || cudaMalloc(&s->dout, R * NOUT * 4) != cudaSuccess ||
      cudaMalloc(&s->T, R * NT * 4) != cudaSuccess)
    return ST_ENOMEM;
  for (int l = 0; l < 3; ++l)
    if (cudaMalloc(&s->HT[l], R * NH * 2) != cudaSuccess) return ST_ENOMEM;
  for (int l = 0; l < 2; ++l)
    if (cudaMalloc(&s->dZT[l], R * NH * 2) != cudaSuccess) return ST_ENOMEM;
  if (cudaMalloc(&s->part, (R / RED_ROWS + 1) * (size_t)L0_PART * 4) != cudaSuccess) return ST_ENOMEM;
  s->cap = rows;
  return ST_OK;
}

// The training kernels' bf16 copies of the hidden weights (and W^T), after
// every parameter update.
int sync_bf16(st_surrogate* s) {
  for (int l = 0; l < 3; ++l) {
    to_bf16<<<(NH * NH + 255) / 256, 256, 0, s->stream>>>(s->P + OWH[l], s->Wb[l], NH * NH);
    SC(cudaGetLastError());
    st::tcg::transpose_bf16<<<dim3(NH / 32, NH / 32), 256, 0, s->stream>>>(s->Wb[l], s->Wt[l], NH, NH);
    SC(cudaGetLastError());
  }
  return ST_OK;
}

// The tensor-core network kernel's weight images and packed biases: once the
// parameters are final (creation, st_surrogate_set_params, the end of
// st_surrogate_train), not after every training step.
int sync_tc_images(st_surrogate* s) {
  pack_sw128<<<(TC_PACK_N + 255) / 256, 256, 0, s->stream>>>(s->P, s->Wsw);
  SC(cudaGetLastError());
  pack_small<<<(TC_SMALL_BYTES / 4 + 255) / 256, 256, 0, s->stream>>>(s->P, s->Psmall);
  SC(cudaGetLastError());
  return ST_OK;
}

// The hidden-layer GEMMs of training and of st_surrogate_forward run on
// tcgen05 (st_tcgemm.cuh) unless SPACETIME_GB300_TRAIN_MMA=sync selects the
// mma.sync kernels (st_mlp.cuh), the same computation on the warp-level path.
bool train_on_tcgen05() {
  const char* e = std::getenv("SPACETIME_GB300_TRAIN_MMA");
  return !(e && std::strcmp(e, "sync") == 0);
}

// C[M][256] = A[M][K] B[256][K]^T on tcgen05, K split over gridDim.z.
template <class Epi>
int gemm_tc(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int K, int splits, Epi epi,
            int* status, cudaStream_t st) {
  static bool attr = false;  // one instantiation per epilogue
  if (!attr) {
    SC(cudaFuncSetAttribute(st::tcg::gemm_tc_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)st::tcg::SMEM));
    attr = true;
  }
  st::tcg::gemm_tc_kernel<Epi><<<dim3(1, M / st::tcg::TILE_M, splits), st::tcg::THREADS, st::tcg::SMEM, st>>>(
      A, lda, B, ldb, K, epi, status);
  SC(cudaGetLastError());
  return ST_OK;
}

// forward of B rows (B multiple of 128) from s->X-like input pointer
int forward(st_surrogate* s, const float* X, int B, bool keep_z, cudaStream_t st) {
  l0_fwd<<<(B + L0_ROWS - 1) / L0_ROWS, NH, 0, st>>>(X, s->P, keep_z ? s->Z[0] : nullptr, s->H[0], B);
  SC(cudaGetLastError());
  const bool tc5 = train_on_tcgen05();
  if (tc5 && keep_z) {
    // training: H_0^T for the first layer's weight gradient (the GEMM
    // epilogues write H_1^T and H_2^T themselves)
    st::tcg::transpose_bf16<<<dim3(NH / 32, B / 32), 256, 0, st>>>(s->H[0], s->HT[0], B, NH);
    SC(cudaGetLastError());
  }
  for (int l = 1; l <= 3; ++l) {
    EpiHidden e{s->P + OBH[l - 1], keep_z ? s->Z[l] : nullptr, s->H[l], NH};
    if (tc5) {
      // Z = H W^T: A = H [B][256], B = W [256 out][256 in], both K-major
      if (keep_z && l < 3) { e.T = s->HT[l]; e.ldt = B; }
      const int rc = gemm_tc(s->H[l - 1], NH, s->Wb[l - 1], NH, B, NH, 1, e, s->d_status, st);
      if (rc != ST_OK) return rc;
      continue;
    }
    st::mlp::gemm_bf16_kernel<true, true, EpiHidden>
        <<<dim3(NH / st::mlp::TN, B / st::mlp::TM, 1), st::mlp::GEMM_THREADS, 0, st>>>(s->H[l - 1], NH, s->Wb[l - 1],
                                                                                      NH, NH, e);
    SC(cudaGetLastError());
  }
  l4_fwd<<<(B * 32 + 255) / 256, 256, 0, st>>>(s->H[3], s->P, s->out, B);
  SC(cudaGetLastError());
  return ST_OK;
}

// Layer 0's weight and bias gradients from dZ0: block partials, then their
// ordered sum into G (dW0 and db0 are adjacent in the parameter vector).
int l0_backward(st_surrogate* s, const __nv_bfloat16* dZ0, const float* X, int B, int nred) {
  static_assert(OB0 == OW0 + NH * NIN, "dW0 and db0 adjacent in the parameter vector");
  l0_bwd<<<nred, NH, 0, s->stream>>>(dZ0, X, s->part, B);
  SC(cudaGetLastError());
  reduce_parts<<<(L0_PART + 31) / 32, 1024, 0, s->stream>>>(s->part, nred, L0_PART, s->G, OW0);
  SC(cudaGetLastError());
  return ST_OK;
}

// backward from s->dout (already scaled by 1/B); accumulates into s->G
int backward(st_surrogate* s, const float* X, int B) {
  cudaStream_t st = s->stream;
  SC(cudaMemsetAsync(s->G, 0, NPARAM * 4, st));
  l4_bwd_dx<<<(B * (NH / 4) + 255) / 256, 256, 0, st>>>(s->dout, s->P, s->Z[3], s->dZa, B);
  SC(cudaGetLastError());
  const int nred = (B + RED_ROWS - 1) / RED_ROWS;
  l4_bwd_w<<<nred, NH, 0, st>>>(s->dout, s->H[3], s->part, B);
  SC(cudaGetLastError());
  static_assert(OB4 == OW4 + NOUT * NH, "dW4 and db4 adjacent in the parameter vector");
  reduce_parts<<<(L4_PART + 31) / 32, 1024, 0, st>>>(s->part, nred, L4_PART, s->G, OW4);
  SC(cudaGetLastError());
  __nv_bfloat16* dZ = s->dZa;
  __nv_bfloat16* dZn = s->dZb;
  const int splits = std::max(1, std::min(64, B / 1024));
  if (train_on_tcgen05()) {
    // both weight-gradient operands K-major over the batch: dZ^T and H^T
    // (written transposed by the forward and input-gradient epilogues; dZ_3,
    // from the FP32 output layer, transposed here); K = 1024 per split keeps
    // the atomics few and the pipeline full
    st::tcg::transpose_bf16<<<dim3(NH / 32, B / 32), 256, 0, st>>>(dZ, s->dZT[0], B, NH);
    SC(cudaGetLastError());
    int cur = 0;
    for (int l = 3; l >= 1; --l) {
      // dW_l[o][i] = sum_b dZ[b][o] H_{l-1}[b][i]: A = dZ^T [256][B], B = H^T [256][B]
      EpiAccum ea{s->G + OWH[l - 1], NH};
      int rc = gemm_tc(s->dZT[cur], B, s->HT[l - 1], B, NH, B, splits, ea, s->d_status, st);
      if (rc != ST_OK) return rc;
      colsum_bf16<<<nred, NH, 0, st>>>(dZ, s->G, OBH[l - 1], B);
      SC(cudaGetLastError());
      // dZ_{l-1}[b][i] = (sum_o dZ[b][o] W[o][i]) silu'(Z_{l-1}): A = dZ [B][256], B = W^T [256 in][256 out]
      EpiBackDX eb{s->Z[l - 1], dZn, NH};
      if (l > 1) { eb.T = s->dZT[cur ^ 1]; eb.ldt = B; }
      rc = gemm_tc(dZ, NH, s->Wt[l - 1], NH, B, NH, 1, eb, s->d_status, st);
      if (rc != ST_OK) return rc;
      std::swap(dZ, dZn);
      cur ^= 1;
    }
    return l0_backward(s, dZ, X, B, nred);
  }
  for (int l = 3; l >= 1; --l) {
    // dW_l = dZ_l^T H_{l-1}
    EpiAccum ea{s->G + OWH[l - 1], NH};
    st::mlp::gemm_bf16_kernel<false, false, EpiAccum>
        <<<dim3(NH / st::mlp::TN, NH / st::mlp::TM, splits), st::mlp::GEMM_THREADS, 0, st>>>(dZ, NH, s->H[l - 1], NH,
                                                                                              B, ea);
    SC(cudaGetLastError());
    colsum_bf16<<<nred, NH, 0, st>>>(dZ, s->G, OBH[l - 1], B);
    SC(cudaGetLastError());
    // dZ_{l-1} = (dZ_l W_l) * silu'(Z_{l-1})
    EpiBackDX eb{s->Z[l - 1], dZn, NH};
    st::mlp::gemm_bf16_kernel<true, false, EpiBackDX>
        <<<dim3(NH / st::mlp::TN, B / st::mlp::TM, 1), st::mlp::GEMM_THREADS, 0, st>>>(dZ, NH, s->Wb[l - 1], NH, NH,
                                                                                      eb);
    SC(cudaGetLastError());
    std::swap(dZ, dZn);
  }
  return l0_backward(s, dZ, X, B, nred);
}

int pad128(long long n) { return (int)((n + 127) / 128 * 128); }

// After a sync: ST_ECUDA (and the flag cleared) when a tcgen05 GEMM's bounded
// wait ran out since the last check.
int gemm_status(st_surrogate* s) {
  int h = 0;
  SC(cudaMemcpy(&h, s->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    SC(cudaMemset(s->d_status, 0, sizeof(int)));
    return ST_ECUDA;
  }
  return ST_OK;
}

// Wait bound and first-copy switch of sur_mlp_tc_kernel.  The environment
// variable SPACETIME_GB300_TC_WAIT_OUT=1 makes every CTA's first wait run out
// (its first copies are never issued, short wait bound), so all tiles fail:
// the failure path under test.
struct TcWait {
  uint32_t limit;
  int issue_first;
};
TcWait tc_wait_mode() {
  const char* e = std::getenv("SPACETIME_GB300_TC_WAIT_OUT");
  if (e && std::strcmp(e, "1") == 0) return TcWait{1024u, 0};
  return TcWait{TC_WAIT_LIMIT, 1};
}

// Frame-pass buffers for `rows` network rows (a multiple of 128, one tile of
// the tcgen05 kernel per 128).
int ensure_frame(st_surrogate* s, long long rows) {
  if (s->frows >= rows) return ST_OK;
  cudaFree(s->fX); cudaFree(s->fAux); cudaFree(s->fFl); cudaFree(s->fO); cudaFree(s->fStatus);
  cudaFree(s->fMask); cudaFree(s->fCount); cudaFree(s->fOff);
  s->fX = nullptr; s->fAux = nullptr; s->fFl = nullptr; s->fO = nullptr; s->fStatus = nullptr;
  s->fMask = nullptr; s->fCount = nullptr; s->fOff = nullptr;
  s->frows = 0;
  const size_t nw = (size_t)rows / 32, nb = (size_t)rows / TC_ROWS;
  if (cudaMalloc(&s->fX, rows * NIN * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&s->fAux, rows * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&s->fFl, rows * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->fO, rows * NOUT * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&s->fStatus, nb * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->fMask, nw * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&s->fCount, nw * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->fOff, nw * sizeof(int)) != cudaSuccess)
    return ST_ENOMEM;
  s->frows = rows;
  return ST_OK;
}

}  // namespace

extern "C" {

int st_surrogate_create(st_surrogate** out, int device, unsigned long long seed) {
  if (!out) return ST_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ST_ECUDA;
  if (device < 0 || device >= ndev) return ST_EINVAL;
  st_surrogate* s = new (std::nothrow) st_surrogate();
  if (!s) return ST_ENOMEM;
  s->device = device;
  s->seed = seed;
  auto fail = [&](int c) { st_surrogate_destroy(s); return c; };
  if (cudaSetDevice(device) != cudaSuccess) return fail(ST_ECUDA);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(ST_ECUDA);
  if (cudaMalloc(&s->P, NPARAM * 4) != cudaSuccess || cudaMalloc(&s->G, NPARAM * 4) != cudaSuccess ||
      cudaMalloc(&s->Mm, NPARAM * 4) != cudaSuccess || cudaMalloc(&s->Vv, NPARAM * 4) != cudaSuccess ||
      cudaMalloc(&s->loss, 16 * 4) != cudaSuccess)
    return fail(ST_ENOMEM);
  for (int l = 0; l < 3; ++l)
    if (cudaMalloc(&s->Wb[l], NH * NH * 2) != cudaSuccess || cudaMalloc(&s->Wt[l], NH * NH * 2) != cudaSuccess)
      return fail(ST_ENOMEM);
  if (cudaMalloc(&s->d_status, sizeof(int)) != cudaSuccess || cudaMemset(s->d_status, 0, sizeof(int)) != cudaSuccess)
    return fail(ST_ENOMEM);
  if (cudaMalloc(&s->Wsw, TC_WSW_BYTES) != cudaSuccess) return fail(ST_ENOMEM);
  if (cudaMalloc(&s->Psmall, TC_SMALL_BYTES) != cudaSuccess) return fail(ST_ENOMEM);
  // He-style uniform initialisation from a splitmix64 stream (host)
  std::vector<float> P(NPARAM, 0.f);
  uint64_t z = seed * 0x9e3779b97f4a7c15ull + 12345;
  auto rnd = [&]() {
    z += 0x9e3779b97f4a7c15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  auto fill = [&](size_t off, int fan_out, int fan_in, double gain) {
    const double lim = gain * std::sqrt(3.0 / fan_in);
    for (int i = 0; i < fan_out * fan_in; ++i) P[off + i] = (float)(lim * rnd());
  };
  fill(OW0, NH, NIN, 1.6);
  fill(OW1, NH, NH, 1.6);
  fill(OW2, NH, NH, 1.6);
  fill(OW3, NH, NH, 1.6);
  fill(OW4, NOUT, NH, 0.1);
  P[OB4 + 5] = -6.0f;  // start the log-variance small
  if (cudaMemcpy(s->P, P.data(), NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) return fail(ST_ECUDA);
  if (cudaMemset(s->Mm, 0, NPARAM * 4) != cudaSuccess || cudaMemset(s->Vv, 0, NPARAM * 4) != cudaSuccess)
    return fail(ST_ECUDA);
  uint32_t v[SOBOL_DIMS][32];
  sobol_directions(v);
  if (cudaMemcpyToSymbol(c_sobol_v, v, sizeof v) != cudaSuccess) return fail(ST_ECUDA);
  if (sync_bf16(s) != ST_OK || sync_tc_images(s) != ST_OK || cudaStreamSynchronize(s->stream) != cudaSuccess)
    return fail(ST_ECUDA);
  *out = s;
  return ST_OK;
}

void st_surrogate_destroy(st_surrogate* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaFree(s->P); cudaFree(s->G); cudaFree(s->Mm); cudaFree(s->Vv); cudaFree(s->loss);
  for (int l = 0; l < 3; ++l) { cudaFree(s->Wb[l]); cudaFree(s->Wt[l]); }
  cudaFree(s->d_status);
  for (int l = 0; l < 3; ++l) cudaFree(s->HT[l]);
  for (int l = 0; l < 2; ++l) cudaFree(s->dZT[l]);
  cudaFree(s->part);
  cudaFree(s->Wsw);
  cudaFree(s->Psmall);
  cudaFree(s->fX); cudaFree(s->fAux); cudaFree(s->fFl); cudaFree(s->fO); cudaFree(s->fStatus);
  cudaFree(s->X);
  for (int l = 0; l < 4; ++l) { cudaFree(s->Z[l]); cudaFree(s->H[l]); }
  cudaFree(s->dZa); cudaFree(s->dZb); cudaFree(s->out); cudaFree(s->dout); cudaFree(s->T);
  cudaFree(s->DX); cudaFree(s->DT);

  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

int st_surrogate_num_params(void) { return (int)NPARAM; }

int st_surrogate_get_params(st_surrogate* s, float* host) {
  if (!s || !host) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  SC(cudaMemcpy(host, s->P, NPARAM * 4, cudaMemcpyDeviceToHost));
  return ST_OK;
}

int st_surrogate_set_params(st_surrogate* s, const float* host) {
  if (!s || !host) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  SC(cudaMemcpy(s->P, host, NPARAM * 4, cudaMemcpyHostToDevice));
  if (sync_bf16(s) != ST_OK || sync_tc_images(s) != ST_OK) return ST_ECUDA;
  SC(cudaStreamSynchronize(s->stream));
  return ST_OK;
}

int st_surrogate_forward(st_surrogate* s, const float* X, int n, float* out) {
  if (!s || !X || !out || n <= 0) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  const int B = pad128(n);
  int rc = ensure_work(s, B);
  if (rc != ST_OK) return rc;
  SC(cudaMemsetAsync(s->X, 0, (size_t)B * NIN * 4, s->stream));
  SC(cudaMemcpyAsync(s->X, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice, s->stream));
  if ((rc = forward(s, s->X, B, false, s->stream)) != ST_OK) return rc;
  SC(cudaMemcpyAsync(out, s->out, (size_t)n * NOUT * 4, cudaMemcpyDeviceToHost, s->stream));
  SC(cudaStreamSynchronize(s->stream));
  return gemm_status(s);
}

// The same network on the frame pass's tensor-core kernel (tcgen05 / TMEM,
// sur_mlp_tc_kernel): rows padded to whole 128-row tiles with zeros.
int st_surrogate_forward_tc(st_surrogate* s, const float* X, int n, float* out) {
  if (!s || !X || !out || n <= 0) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  const long long B = pad128(n);
  const int nb = (int)(B / TC_ROWS);
  int rc = ensure_frame(s, B);
  if (rc != ST_OK) return rc;
  cudaStream_t st = s->stream;
  SC(cudaMemsetAsync(s->fX, 0, (size_t)B * NIN * 4, st));
  SC(cudaMemcpyAsync(s->fX, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice, st));
  SC(cudaFuncSetAttribute(sur_mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
  SC(cudaMemsetAsync(s->fStatus, 0xFF, (size_t)nb * sizeof(int), st));  // -1 until a tile finishes
  const TcWait tw = tc_wait_mode();
  sur_mlp_tc_kernel<<<tc_grid(nb), TC_THREADS, TC_SMEM, st>>>(s->Psmall, s->Wsw, s->fX, s->fO, s->fStatus, nb,
                                                               nullptr, tw.limit, tw.issue_first);
  SC(cudaGetLastError());
  std::vector<int> status(nb);
  SC(cudaMemcpyAsync(out, s->fO, (size_t)n * NOUT * 4, cudaMemcpyDeviceToHost, st));
  SC(cudaMemcpyAsync(status.data(), s->fStatus, nb * sizeof(int), cudaMemcpyDeviceToHost, st));
  SC(cudaStreamSynchronize(st));
  for (int t = 0; t < nb; ++t)
    if (status[t]) return ST_ECUDA;  // a bounded wait ran out: that tile has no output
  return ST_OK;
}

// Loss and parameter gradient on n rows (rows beyond n are masked padding).
int st_surrogate_loss_grad(st_surrogate* s, const float* X, const float* T, int n, float* loss4, float* grad) {
  if (!s || !X || !T || n <= 0) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  const int B = pad128(n);
  int rc = ensure_work(s, B);
  if (rc != ST_OK) return rc;
  cudaStream_t st = s->stream;
  SC(cudaMemsetAsync(s->X, 0, (size_t)B * NIN * 4, st));
  SC(cudaMemsetAsync(s->T, 0, (size_t)B * NT * 4, st));
  SC(cudaMemcpyAsync(s->X, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice, st));
  SC(cudaMemcpyAsync(s->T, T, (size_t)n * NT * 4, cudaMemcpyHostToDevice, st));
  if ((rc = forward(s, s->X, B, true, s->stream)) != ST_OK) return rc;
  SC(cudaMemsetAsync(s->loss, 0, 16 * 4, st));
  loss_grad<<<(B + 255) / 256, 256, 0, st>>>(s->out, s->T, s->dout, s->loss, n, 1.0f / n);
  SC(cudaGetLastError());
  // padding rows carry no gradient
  if (B > n) SC(cudaMemsetAsync(s->dout + (size_t)n * NOUT, 0, (size_t)(B - n) * NOUT * 4, st));
  if ((rc = backward(s, s->X, B)) != ST_OK) return rc;
  if (loss4) SC(cudaMemcpyAsync(loss4, s->loss, 4 * 4, cudaMemcpyDeviceToHost, st));
  if (grad) SC(cudaMemcpyAsync(grad, s->G, NPARAM * 4, cudaMemcpyDeviceToHost, st));
  SC(cudaStreamSynchronize(st));
  return gemm_status(s);
}

// Generate n labelled samples (Sobol indices offset..offset+n-1) on the
// device and keep them as the training set; optionally copy to the host.
int st_surrogate_generate(st_surrogate* s, long long n, long long offset, double dt, float* host_x, float* host_t,
                          float* host_raw) {
  if (!s || n <= 0 || !(dt > 0.0)) return ST_EINVAL;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  cudaFree(s->DX);
  cudaFree(s->DT);
  s->DX = s->DT = nullptr;
  s->ndata = 0;
  if (cudaMalloc(&s->DX, (size_t)n * NIN * 4) != cudaSuccess || cudaMalloc(&s->DT, (size_t)n * NT * 4) != cudaSuccess)
    return ST_ENOMEM;
  float* raw = nullptr;
  if (host_raw && cudaMalloc(&raw, (size_t)n * NRAW * 4) != cudaSuccess) return ST_ENOMEM;
  LabelParams lp{n, offset, s->DX, s->DT, raw, dt};
  label_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(lp);
  SC(cudaGetLastError());
  if (host_x) SC(cudaMemcpyAsync(host_x, s->DX, (size_t)n * NIN * 4, cudaMemcpyDeviceToHost, s->stream));
  if (host_t) SC(cudaMemcpyAsync(host_t, s->DT, (size_t)n * NT * 4, cudaMemcpyDeviceToHost, s->stream));
  if (raw) SC(cudaMemcpyAsync(host_raw, raw, (size_t)n * NRAW * 4, cudaMemcpyDeviceToHost, s->stream));
  SC(cudaStreamSynchronize(s->stream));
  cudaFree(raw);
  s->ndata = n;
  return ST_OK;
}

// `steps` AdamW steps on batches drawn (cyclically, in order of a per-epoch
// stride) from the generated set; loss_hist[k] gets each step's loss.
int st_surrogate_train(st_surrogate* s, int steps, int batch, float lr, float weight_decay, float* loss_hist) {
  if (!s || steps <= 0 || batch < 128 || batch % 128 != 0) return ST_EINVAL;
  if (s->ndata < batch) return ST_ESTATE;
  if (cudaSetDevice(s->device) != cudaSuccess) return ST_ECUDA;
  int rc = ensure_work(s, batch);
  if (rc != ST_OK) return rc;
  cudaStream_t st = s->stream;
  const long long nb = s->ndata / batch;
  std::vector<float> lh(steps > 0 ? steps : 1);
  for (int k = 0; k < steps; ++k) {
    const long long bi = (s->step * 7919LL) % nb;  // stride through the batches
    const float* X = s->DX + bi * batch * NIN;
    const float* T = s->DT + bi * batch * NT;
    if ((rc = forward(s, X, batch, true, s->stream)) != ST_OK) return rc;
    SC(cudaMemsetAsync(s->loss, 0, 16 * 4, st));
    loss_grad<<<(batch + 255) / 256, 256, 0, st>>>(s->out, T, s->dout, s->loss, batch, 1.0f / batch);
    SC(cudaGetLastError());
    if ((rc = backward(s, X, batch)) != ST_OK) return rc;
    ++s->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)s->step), bc2 = 1.f - std::pow(b2, (float)s->step);
    adamw<<<(unsigned)((NPARAM + 255) / 256), 256, 0, st>>>(s->P, s->G, s->Mm, s->Vv, NPARAM, lr, b1, b2, 1e-8f,
                                                           weight_decay, bc1, bc2);
    SC(cudaGetLastError());
    if ((rc = sync_bf16(s)) != ST_OK) return rc;
    if (loss_hist) SC(cudaMemcpyAsync(&lh[k], s->loss, 4, cudaMemcpyDeviceToHost, st));
  }
  if ((rc = sync_tc_images(s)) != ST_OK) return rc;
  SC(cudaStreamSynchronize(st));
  if ((rc = gemm_status(s)) != ST_OK) return rc;
  if (loss_hist) std::memcpy(loss_hist, lh.data(), steps * sizeof(float));
  return ST_OK;
}

}  // extern "C"

namespace st {

// Surrogate pass of one frame on `stream` (see st_internal.h).
int surrogate_frame(st_surrogate* s, const TraceParams& p, const Variant& v, const SurFrame& f, int* list, int* count,
                    cudaStream_t stream) {
  const unsigned nb = (unsigned)(((p.width + 15) / 16) * ((p.height + 7) / 8));
  SC(cudaMemsetAsync(count, 0, sizeof(int), stream));
  // tcgen05 / TMEM kernel by default; SPACETIME_GB300_SURROGATE_MMA=sync runs
  // the mma.sync kernel (the same computation on the warp-level tensor-core path)
  const char* mode = std::getenv("SPACETIME_GB300_SURROGATE_MMA");
  if (mode && std::strcmp(mode, "sync") == 0) {
    auto k = v.kerr ? sur::sur_frame_kernel<1> : sur::sur_frame_kernel<0>;
    SC(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sur::F_SMEM));
    k<<<nb, sur::FTHREADS, sur::F_SMEM, stream>>>(p, f, s->P, s->Wb[0], s->Wb[1], s->Wb[2], list, count);
  } else {
    const long long rows = (long long)nb * sur::TC_ROWS;
    const int rc = ensure_frame(s, rows);
    if (rc != ST_OK) return rc;
    if (v.kerr) sur::sur_inputs_kernel<1><<<nb, 128, 0, stream>>>(p, f, s->fX, s->fAux, s->fFl);
    else sur::sur_inputs_kernel<0><<<nb, 128, 0, stream>>>(p, f, s->fX, s->fAux, s->fFl);
    SC(cudaGetLastError());
    SC(cudaFuncSetAttribute(sur::sur_mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)sur::TC_SMEM));
    SC(cudaMemsetAsync(s->fStatus, 0xFF, (size_t)nb * sizeof(int), stream));  // -1 until a tile finishes
    const TcWait tw = tc_wait_mode();
    sur::sur_mlp_tc_kernel<<<sur::tc_grid((int)nb), sur::TC_THREADS, sur::TC_SMEM, stream>>>(
        s->Psmall, s->Wsw, s->fX, s->fO, s->fStatus, (int)nb, p.counters, tw.limit, tw.issue_first);
    SC(cudaGetLastError());
    sur::sur_gate_kernel<<<nb, 128, 0, stream>>>(p, f, s->fO, s->fAux, s->fFl, s->fStatus, s->fMask, s->fCount);
    SC(cudaGetLastError());
    sur::sur_scan_kernel<<<1, 1024, 0, stream>>>(s->fCount, s->fOff, (int)(rows / 32), count);
    SC(cudaGetLastError());
    sur::sur_scatter_kernel<<<nb, 128, 0, stream>>>(p, s->fMask, s->fOff, list);
  }
  SC(cudaGetLastError());
  return ST_OK;
}

}  // namespace st
