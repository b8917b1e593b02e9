// st_fluid.cu -- the live fluid-simulated accretion disc (DiscFluidSim /
// step_sim!, src/disc_sim.jl): a 2-D stable-fluids solver on the gas volume's
// own (log s, phi) grid whose surface density is extruded through the
// vertical envelope into the context's density texture, which the trace
// kernels then sample unchanged.
//
// One step of the reference is ~20 dispatches (src/disc_sim.jl:287-320):
// velocity advection, forcing, divergence, 2 ceil(jacobi / 2) Jacobi sweeps,
// gradient subtraction, forward and backward density advection, the
// MacCormack combine and the extrusion.  Here it is four kernels:
//
//   fluid_velocity_kernel   advection of (vu, vv) under shear + itself, then
//                           the curl-noise forcing, drag and edge taper of the
//                           same cell (pointwise after the advection);
//   fluid_divergence_kernel divergence of the forced field and the first
//                           Jacobi sweep, which from p = 0 is -dv / 4;
//   fluid_pressure_kernel   the remaining sweeps, temporally blocked: a tile
//                           and a halo as wide as the sweeps it runs are
//                           staged in shared memory and every sweep updates
//                           the shrinking valid region there; the last pass
//                           subtracts the pressure gradient on the tile;
//   fluid_density_kernel    MacCormack advection of the surface density: the
//                           forward result at the cell and at the four
//                           corners of its backward point are recomputed in
//                           registers (each is one bilinear sample), so the
//                           forward and backward fields never go through
//                           memory; then the limiter, the relaxation toward
//                           the noise-modulated profile, and the extrusion of
//                           the new value through the nz envelope cells.
//
// Each cell's arithmetic is the reference's, in the same order, in float;
// this unit is compiled without multiply-add contraction so every operation
// rounds as written.  Index arithmetic is 1-based in the formulas, as in the
// reference; field (i, j) lives at (i - 1) + nr (j - 1).
//
// The simulation clock lives on the device (t[parity] is read by the step,
// t[1 - parity] = t[parity] + dt written by it) and the density ping-pongs
// between two buffers by the same parity, so a step's launches are fixed per
// (parity, dt, jacobi) and are captured once into a CUDA graph per parity.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "st_internal.h"

namespace st {
namespace fluid {

// ---- device helpers (src/disc_sim.jl:80-134) ---------------------------------

__device__ __forceinline__ float hash01(int x, int y, int z) {
  uint32_t h = ((uint32_t)x * 0x8da6b343u) ^ ((uint32_t)y * 0xd8163841u) ^ ((uint32_t)z * 0xcb1ab31fu);
  h ^= h >> 13;
  h *= 0x9e3779b9u;
  h ^= h >> 16;
  return (float)(h & 0x00ffffffu) * 5.9604645e-8f;
}

// Value noise on the hashed lattice, smoothstep-weighted trilinear.
__device__ __forceinline__ float noise3(float x, float y, float z) {
  const float flx = floorf(x), fly = floorf(y), flz = floorf(z);
  const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
  float fx = x - flx, fy = y - fly, fz = z - flz;
  fx = fx * fx * (3.0f - 2.0f * fx);
  fy = fy * fy * (3.0f - 2.0f * fy);
  fz = fz * fz * (3.0f - 2.0f * fz);
  const int i1 = ix + 1, j1 = iy + 1, k1 = iz + 1;
  const float h000 = hash01(ix, iy, iz), h100 = hash01(i1, iy, iz);
  const float h010 = hash01(ix, j1, iz), h110 = hash01(i1, j1, iz);
  const float h001 = hash01(ix, iy, k1), h101 = hash01(i1, iy, k1);
  const float h011 = hash01(ix, j1, k1), h111 = hash01(i1, j1, k1);
  const float c00 = h000 + fx * (h100 - h000);
  const float c10 = h010 + fx * (h110 - h010);
  const float c01 = h001 + fx * (h101 - h001);
  const float c11 = h011 + fx * (h111 - h011);
  const float c0 = c00 + fy * (c10 - c00);
  const float c1 = c01 + fy * (c11 - c01);
  return c0 + fz * (c1 - c0);
}

__device__ __forceinline__ int jmod(int a, int n) {
  const int r = a % n;
  return r < 0 ? r + n : r;
}

// jmod for a in [-n, 2n) by compare (the footprints and halos stay there);
// anything else falls back to the division.
__device__ __forceinline__ int jwrap(int a, int n) {
  const int b = a < 0 ? a + n : (a >= n ? a - n : a);
  return (b >= 0 && b < n) ? b : jmod(a, n);
}

// Corners of the bilinear footprint of (x, y): radius clamped, phi periodic.
struct Foot {
  int o00, o10, o01, o11;  // storage offsets of (i0, j0a), (i0+1, j0a), (i0, j1a), (i0+1, j1a)
  int i0, j0a, j1a;        // the corners' 1-based indices
  float tx, ty;
};

__device__ __forceinline__ Foot footprint(float x, float y, int nr, int nphi) {
  x = fminf(fmaxf(x, 1.0f), (float)nr);
  const int i0 = min(max((int)floorf(x), 1), nr - 1);
  Foot f;
  f.tx = x - (float)i0;
  const float yw = y - (float)nphi * floorf((y - 1.0f) / (float)nphi);
  const int j0 = (int)floorf(yw);
  f.ty = yw - (float)j0;
  const int j0a = jwrap(j0 - 1, nphi) + 1;
  const int j1a = jwrap(j0, nphi) + 1;
  f.i0 = i0; f.j0a = j0a; f.j1a = j1a;
  f.o00 = (i0 - 1) + nr * (j0a - 1);
  f.o10 = f.o00 + 1;
  f.o01 = (i0 - 1) + nr * (j1a - 1);
  f.o11 = f.o01 + 1;
  return f;
}

__device__ __forceinline__ float bilerp(const float* __restrict__ f, const Foot& q) {
  const float a = f[q.o00] + q.tx * (f[q.o10] - f[q.o00]);
  const float b = f[q.o01] + q.tx * (f[q.o11] - f[q.o01]);
  return a + q.ty * (b - a);
}

// ---- kernels -------------------------------------------------------------------

struct Fields {
  int nr, nphi, nz;
  float* vu; float* vv;         // velocity after projection (cells / M-time)
  float* vu2; float* vv2;       // advected + forced velocity
  float* dens[2];               // surface density, ping-pong by parity
  const float* base;            // radial profile (relaxation target)
  const float* shear;           // [nr] Keplerian shear, phi cells / M-time
  const float* env;             // [nr][nz] vertical envelope, (nr, nz) column-major
  float* prs[2];                // pressure ping-pong
  float* div;
  float* t;                     // [2] simulation clock by parity
  float* vol;                   // (nr, nphi, nz) density texture of the context
};

// Semi-Lagrangian velocity advection, then forcing + drag + edge taper
// (k_advect_vel!, k_force!: src/disc_sim.jl:136-172).
__global__ void fluid_velocity_kernel(Fields F, int parity, float dt, float amp, float drag) {
  const int nr = F.nr, nphi = F.nphi;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;  // one grid row per phi row
  if (i > nr) return;
  const int idx = (i - 1) + nr * (j - 1);
  const float x = (float)i - dt * F.vu[idx];
  const float y = (float)j - dt * (F.vv[idx] + F.shear[i - 1]);
  const Foot q = footprint(x, y, nr, nphi);
  float u = bilerp(F.vu, q);
  float v = bilerp(F.vv, q);
  // psi on a coarse lattice (~12-cell eddies) drifting in time; F = curl(psi z)
  const float t = F.t[parity];
  const float sc = 0.085f;
  const float px = (float)i * sc, py = (float)j * sc, pz = t * 0.35f;
  const float e = 0.35f;
  const float dpy = noise3(px, py + e, pz) - noise3(px, py - e, pz);
  const float dpx = noise3(px + e, py, pz) - noise3(px - e, py, pz);
  const float fu = dpy / (2.0f * e);
  const float fv = -dpx / (2.0f * e);
  float edge = fminf((float)i - 1.0f, (float)(nr - i)) * 0.125f;
  edge = fminf(fmaxf(edge, 0.0f), 1.0f);
  const float damp = expf(-drag * dt);
  u = (u + dt * amp * fu * edge) * damp * edge;
  v = (v + dt * amp * fv * edge) * damp;
  F.vu2[idx] = u;
  F.vv2[idx] = v;
}

// Divergence (k_div!) and the first Jacobi sweep from p = 0 (k_jacobi!:
// 0.25 ((((0 + 0) + 0) + 0) - dv) = 0.25 (-dv)); with no sweeps p stays 0.
__global__ void fluid_divergence_kernel(Fields F, int first_sweep) {
  const int nr = F.nr, nphi = F.nphi;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  if (i > nr) return;
  const int idx = (i - 1) + nr * (j - 1);
  const int ip = min(i + 1, nr), im = max(i - 1, 1);
  const int jp = jwrap(j, nphi) + 1, jm = jwrap(j - 2, nphi) + 1;
  const float dv = 0.5f * (F.vu2[(ip - 1) + nr * (j - 1)] - F.vu2[(im - 1) + nr * (j - 1)] +
                           F.vv2[(i - 1) + nr * (jp - 1)] - F.vv2[(i - 1) + nr * (jm - 1)]);
  F.div[idx] = dv;
  F.prs[0][idx] = first_sweep ? 0.25f * (0.0f - dv) : 0.0f;
}

constexpr int TI = 32, TJ = 8;     // tile of the blocked sweeps (i fastest)
constexpr int MAX_SWEEPS = 16;     // sweeps per pass; halo = sweeps (+1 on the last pass): <= 33 KB of shared memory

// `sweeps` Jacobi sweeps (k_jacobi!, src/disc_sim.jl:184-192) on one tile,
// reading p from prs[src] and, unless `last`, writing the tile's p to
// prs[1 - src]; the last pass subtracts the gradient (k_subgrad!,
// src/disc_sim.jl:194-203) on the tile: (vu, vv) = (vu2, vv2) - grad p / 2.
// Shared memory: p ping-pong and dv over the tile + halo.
__global__ void __launch_bounds__(256) fluid_pressure_kernel(Fields F, int src, int sweeps, int last) {
  extern __shared__ float sm[];
  const int nr = F.nr, nphi = F.nphi;
  const int H = sweeps + (last ? 1 : 0);
  const int RI = TI + 2 * H, RJ = TJ + 2 * H, RN = RI * RJ;
  float* P0 = sm;
  float* P1 = sm + RN;
  float* D = sm + 2 * RN;
  const int i0 = blockIdx.x * TI + 1 - H;  // global (unclamped) i of local row 0
  const int j0 = blockIdx.y * TJ + 1 - H;
  const float* __restrict__ pin = src ? F.prs[1] : F.prs[0];
  float* __restrict__ pout = src ? F.prs[0] : F.prs[1];
  // blockDim = (32, 8): x runs along i (coalesced), y along phi
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int lj = ty; lj < RJ; lj += 8) {
    const int gj = jwrap(j0 + lj - 1, nphi) + 1;
    for (int li = tx; li < RI; li += 32) {
      const int gi = i0 + li;
      float pv = 0.0f, dv = 0.0f;
      if (gi >= 1 && gi <= nr) {
        const int o = (gi - 1) + nr * (gj - 1);
        pv = pin[o];
        dv = F.div[o];
      }
      P0[li + RI * lj] = pv;
      D[li + RI * lj] = dv;
    }
  }
  __syncthreads();
  float* cur = P0;
  float* nxt = P1;
  for (int k = 1; k <= sweeps; ++k) {
    // valid region after this sweep: margin k from every side of the staged block
    for (int lj = k + ty; lj < RJ - k; lj += 8) {
      for (int li = k + tx; li < RI - k; li += 32) {
        const int gi = i0 + li;
        if (gi < 1 || gi > nr) continue;
        const int lip = gi + 1 <= nr ? li + 1 : li;  // clamped radial neighbours
        const int lim = gi - 1 >= 1 ? li - 1 : li;
        const int l = li + RI * lj;
        const float sum = cur[lip + RI * lj] + cur[lim + RI * lj] + cur[l + RI] + cur[l - RI];
        nxt[l] = 0.25f * (sum - D[l]);
      }
    }
    __syncthreads();
    float* tmp = cur; cur = nxt; nxt = tmp;
  }
  // the tile's own cells
  for (int tj = ty; tj < TJ; tj += 8) {
    const int ti = tx;
    const int gi = blockIdx.x * TI + 1 + ti, gjr = blockIdx.y * TJ + 1 + tj;
    if (gi > nr || gjr > nphi) continue;
    const int li = ti + H, lj = tj + H;
    const int o = (gi - 1) + nr * (gjr - 1);
    if (!last) {
      pout[o] = cur[li + RI * lj];
      continue;
    }
    const int lip = gi + 1 <= nr ? li + 1 : li;
    const int lim = gi - 1 >= 1 ? li - 1 : li;
    F.vu[o] = F.vu2[o] - 0.5f * (cur[lip + RI * lj] - cur[lim + RI * lj]);
    F.vv[o] = F.vv2[o] - 0.5f * (cur[li + RI * (lj + 1)] - cur[li + RI * (lj - 1)]);
  }
}

// Forward semi-Lagrangian density sample at cell (ci, cj) (k_adv_scalar!).
__device__ __forceinline__ float advect_at(const Fields& F, const float* __restrict__ d, int ci, int cj, float dt) {
  const int o = (ci - 1) + F.nr * (cj - 1);
  const float x = (float)ci - dt * F.vu[o];
  const float y = (float)cj - dt * (F.vv[o] + F.shear[ci - 1]);
  return bilerp(d, footprint(x, y, F.nr, F.nphi));
}

// MacCormack density step + relaxation (k_adv_scalar! forward and backward,
// k_maccormack!: src/disc_sim.jl:205-251) and the extrusion of the new value
// through the envelope (k_extrude!, :253-266).  Thread 0 advances the clock.
__global__ void fluid_density_kernel(Fields F, int parity, float dt, float relax) {
  const int nr = F.nr, nphi = F.nphi;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  const float t = F.t[parity];
  if (i == 1 && j == 1) F.t[1 - parity] = t + dt;
  if (i > nr) return;
  const int idx = (i - 1) + nr * (j - 1);
  const float* __restrict__ d = parity ? F.dens[1] : F.dens[0];
  float* __restrict__ dout = parity ? F.dens[0] : F.dens[1];
  // forward: d1 = d at the backtraced point; its corners bound the limiter
  const float x = (float)i - dt * F.vu[idx];
  const float y = (float)j - dt * (F.vv[idx] + F.shear[i - 1]);
  const Foot q = footprint(x, y, nr, nphi);
  const float d1 = bilerp(d, q);
  const float lo = fminf(fminf(d[q.o00], d[q.o10]), fminf(d[q.o01], d[q.o11]));
  const float hi = fmaxf(fmaxf(d[q.o00], d[q.o10]), fmaxf(d[q.o01], d[q.o11]));
  // backward: the forward field re-advected by -dt, sampled at the cell
  const float ndt = -dt;
  const float xb = (float)i - ndt * F.vu[idx];
  const float yb = (float)j - ndt * (F.vv[idx] + F.shear[i - 1]);
  const Foot qb = footprint(xb, yb, nr, nphi);
  const float c00 = advect_at(F, d, qb.i0, qb.j0a, dt), c10 = advect_at(F, d, qb.i0 + 1, qb.j0a, dt);
  const float c01 = advect_at(F, d, qb.i0, qb.j1a, dt), c11 = advect_at(F, d, qb.i0 + 1, qb.j1a, dt);
  const float ea = c00 + qb.tx * (c10 - c00);
  const float eb = c01 + qb.tx * (c11 - c01);
  const float d2 = ea + qb.ty * (eb - ea);
  const float a = fminf(fmaxf(d1 + 0.5f * (d[idx] - d2), lo), hi);
  const float n = noise3((float)i * 0.11f, (float)j * 0.11f, t * 0.25f);
  const float tgt = F.base[idx] * expf(1.2f * (2.0f * n - 1.0f));
  const float dn = fmaxf(a + relax * dt * (tgt - a), 0.0f);
  dout[idx] = dn;
  // the envelope loads of a batch are issued before its stores, so the
  // column's latency is paid once per eight cells rather than per cell
  const size_t plane = (size_t)nr * nphi;
  const float* __restrict__ env = F.env + (i - 1);
  float* __restrict__ vol = F.vol + idx;
  int k = 0;
  for (; k + 8 <= F.nz; k += 8) {
    float e[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) e[q] = __ldg(env + (size_t)nr * (k + q));
#pragma unroll
    for (int q = 0; q < 8; ++q) vol[plane * (k + q)] = dn * e[q];
  }
  for (; k < F.nz; ++k) vol[plane * k] = dn * __ldg(env + (size_t)nr * k);
}

}  // namespace fluid
}  // namespace st

// ---- host side --------------------------------------------------------------

using namespace st::fluid;

struct st_fluid {
  st_context* ctx = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr;
  int nr = 0, nphi = 0, nz = 0;
  float* block = nullptr;  // every field in one allocation
  Fields F{};
  int parity = 0;
  double forcing = 6.0, drag = 0.15, relax = 0.05;
  // graph per parity for the current (dt, jacobi)
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  const float* g_vol = nullptr;  // the density texture the graphs write
  float g_dt = 0.f;
  int g_jacobi = -1;
  long long steps = 0;
};

namespace {

int launch_step(st_fluid* f, int parity, float dt, int jacobi, cudaStream_t s) {
  Fields F = f->F;
  F.vol = nullptr;
  st::CtxVolume cv;
  if (st::context_volume(f->ctx, &cv) != ST_OK || !cv.on || cv.meta.nr != f->nr || cv.meta.nphi != f->nphi ||
      cv.meta.nz != f->nz)
    return ST_ESTATE;
  F.vol = cv.d_vol;
  // one 64-thread block per 64 cells of an s row, one grid row per phi row:
  // the grids are a few tens of thousands of cells, so small blocks spread
  // them over all SMs, and the 2-D grid gives (i, j) without a division
  const int B = 64;
  const dim3 G((f->nr + B - 1) / B, f->nphi);
  fluid_velocity_kernel<<<G, B, 0, s>>>(F, parity, dt, (float)f->forcing, (float)f->drag);
  // 2 ceil(jacobi / 2) sweeps (src/disc_sim.jl:305-308); the first runs in the
  // divergence kernel, the rest in blocked passes of at most MAX_SWEEPS
  const int total = jacobi > 0 ? 2 * ((jacobi + 1) / 2) : 0;
  fluid_divergence_kernel<<<G, B, 0, s>>>(F, total > 0 ? 1 : 0);
  int left = total > 0 ? total - 1 : 0;
  int src = 0;
  const dim3 grid((f->nr + TI - 1) / TI, (f->nphi + TJ - 1) / TJ);
  do {
    const int k = std::min(left, MAX_SWEEPS);
    left -= k;
    const int last = left == 0 ? 1 : 0;
    const int H = k + last;
    const size_t smem = 3 * (size_t)(TI + 2 * H) * (TJ + 2 * H) * sizeof(float);
    fluid_pressure_kernel<<<grid, dim3(32, 8), smem, s>>>(F, src, k, last);
    src = 1 - src;
  } while (left > 0);
  fluid_density_kernel<<<G, B, 0, s>>>(F, parity, dt, (float)f->relax);
  return cudaGetLastError() == cudaSuccess ? ST_OK : ST_ECUDA;
}

void drop_graphs(st_fluid* f) {
  for (auto& e : f->exec)
    if (e) { cudaGraphExecDestroy(e); e = nullptr; }
  f->g_jacobi = -1;
}

}  // namespace

extern "C" {

void st_fluid_params_default(st_fluid_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->M = 1.0;
  p->forcing = 6.0;
  p->drag = 0.15;
  p->relax = 0.05;
  p->scale_height = 0.08;
}

int st_fluid_create(st_fluid** out, st_context* ctx, const st_disc* disc, const st_fluid_params* fp) {
  if (!out || !ctx || !disc || !fp) return ST_EINVAL;
  *out = nullptr;
  if (!(fp->M > 0.0) || !(fp->scale_height > 0.0) || !(disc->outer > disc->inner) || !(disc->inner > 0.0))
    return ST_EINVAL;
  st::CtxVolume cv;
  if (st::context_volume(ctx, &cv) != ST_OK || !cv.on || !cv.d_vol) return ST_ESTATE;
  const int nr = cv.meta.nr, nphi = cv.meta.nphi, nz = cv.meta.nz;
  if (nr < 2 || nphi < 1 || nz < 2) return ST_ESTATE;
  if (nphi > 65535) return ST_EUNSUPPORTED;  // one grid row per phi row
  if (cudaSetDevice(cv.device) != cudaSuccess) return ST_ECUDA;
  const size_t n = (size_t)nr * nphi;
  // initial density: the volume's midplane slice k = (nz + 1) / 2 (1-based),
  // normalised to a peak of 1 (src/disc_sim.jl:45-91)
  std::vector<float> dens0(n);
  const size_t kmid = (size_t)((nz + 1) / 2 - 1);
  if (cudaMemcpyAsync(dens0.data(), cv.d_vol + kmid * n, n * sizeof(float), cudaMemcpyDeviceToHost, cv.stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(cv.stream) != cudaSuccess)
    return ST_ECUDA;
  float peak = dens0[0];
  for (float v : dens0) peak = std::max(peak, v);
  if (peak > 0.0f)
    for (float& v : dens0) v /= peak;
  std::vector<float> base(n), env((size_t)nr * nz), shear(nr);
  const double M = fp->M;
  const float log_in = cv.meta.log_s_in, log_out = cv.meta.log_s_out, zmax = cv.meta.z_max;
  const float hsc = (float)fp->scale_height;
  const float dlog = log_out - log_in;  // a Float32 difference, as the reference forms it
  for (int i = 1; i <= nr; ++i) {
    const double s = std::exp((double)log_in + (double)(i - 1) / (double)(nr - 1) * (double)dlog);
    // _disc_radial_profile, src/disc_volume.jl:274-283
    const double R = s / (2.0 * M), R_in = disc->inner / (2.0 * M), R_out = disc->outer / (2.0 * M);
    const double iscotaper = std::min(std::max((R * R - R_in * R_in) * 0.3, 0.0), 1.0);
    const double T_emit = std::exp(10.034259 - 0.375 * std::log(R * R));
    const double outertaper = std::min(std::max(T_emit / 1000.0, 0.0), 1.0);
    const double dens = std::min(std::max((R_out - R) / (R_out - R_in), 0.0), 1.0);
    const float b = (float)(iscotaper * outertaper * std::pow(dens, disc->falloff));
    for (int j = 0; j < nphi; ++j) base[(size_t)(i - 1) + (size_t)nr * j] = b;
    const double H = (double)hsc * s;
    for (int k = 1; k <= nz; ++k) {
      const double z = -(double)zmax + (double)(k - 1) / (double)(nz - 1) * 2.0 * (double)zmax;
      env[(size_t)(i - 1) + (size_t)nr * (k - 1)] = (float)std::exp(-z * z / (2.0 * H * H));
    }
    shear[i - 1] = (float)(std::sqrt(M / (s * s * s)) * nphi / (2.0 * 3.141592653589793));
  }
  st_fluid* f = new st_fluid;
  f->ctx = ctx;
  f->device = cv.device;
  f->nr = nr; f->nphi = nphi; f->nz = nz;
  f->forcing = fp->forcing; f->drag = fp->drag; f->relax = fp->relax;
  // layout: vu vv vu2 vv2 dens0 dens1 base prs0 prs1 div (n each), env (nr nz), shear (nr), t (2)
  const size_t total = 10 * n + (size_t)nr * nz + nr + 2;
  if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) { delete f; return ST_ECUDA; }
  if (cudaMalloc(&f->block, total * sizeof(float)) != cudaSuccess) {
    cudaStreamDestroy(f->stream);
    delete f;
    return ST_ENOMEM;
  }
  float* b = f->block;
  Fields& F = f->F;
  F.nr = nr; F.nphi = nphi; F.nz = nz;
  F.vu = b; F.vv = b + n; F.vu2 = b + 2 * n; F.vv2 = b + 3 * n;
  F.dens[0] = b + 4 * n; F.dens[1] = b + 5 * n;
  float* base_d = b + 6 * n;
  F.prs[0] = b + 7 * n; F.prs[1] = b + 8 * n; F.div = b + 9 * n;
  float* env_d = b + 10 * n;
  float* shear_d = env_d + (size_t)nr * nz;
  F.t = shear_d + nr;
  F.base = base_d; F.env = env_d; F.shear = shear_d;
  bool ok = cudaMemsetAsync(b, 0, total * sizeof(float), f->stream) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(F.dens[0], dens0.data(), n * sizeof(float), cudaMemcpyHostToDevice, f->stream) ==
                 cudaSuccess;
  ok = ok && cudaMemcpyAsync(base_d, base.data(), n * sizeof(float), cudaMemcpyHostToDevice, f->stream) ==
                 cudaSuccess;
  ok = ok && cudaMemcpyAsync(env_d, env.data(), env.size() * sizeof(float), cudaMemcpyHostToDevice, f->stream) ==
                 cudaSuccess;
  ok = ok && cudaMemcpyAsync(shear_d, shear.data(), nr * sizeof(float), cudaMemcpyHostToDevice, f->stream) ==
                 cudaSuccess;
  ok = ok && cudaStreamSynchronize(f->stream) == cudaSuccess;
  if (!ok) {
    cudaFree(f->block);
    cudaStreamDestroy(f->stream);
    delete f;
    return ST_ECUDA;
  }
  *out = f;
  return ST_OK;
}

int st_fluid_step(st_fluid* f, double dt, int jacobi, int nsteps, int use_graph, float* ms) {
  if (!f || !(std::isfinite(dt)) || jacobi < 0 || jacobi > 4096 || nsteps < 0) return ST_EINVAL;
  if (ms) *ms = 0.f;
  if (cudaSetDevice(f->device) != cudaSuccess) return ST_ECUDA;
  st::CtxVolume cv;
  if (st::context_volume(f->ctx, &cv) != ST_OK || !cv.on || cv.meta.nr != f->nr || cv.meta.nphi != f->nphi ||
      cv.meta.nz != f->nz)
    return ST_ESTATE;
  const float dtf = (float)dt;
  // the steps run on the context's stream, so the next render sees the field
  cudaStream_t s = cv.stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) return ST_ECUDA;
  if (e0 && cudaEventRecord(e0, s) != cudaSuccess) return ST_ECUDA;
  int rc = ST_OK;
  if (use_graph) {
    if (f->g_jacobi != jacobi || f->g_dt != dtf || f->g_vol != cv.d_vol || f->exec[0] == nullptr) {
      drop_graphs(f);
      for (int par = 0; par < 2 && rc == ST_OK; ++par) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { rc = ST_ECUDA; break; }
        const int lr = launch_step(f, par, dtf, jacobi, f->stream);
        const cudaError_t ce = cudaStreamEndCapture(f->stream, &g);
        if (lr != ST_OK || ce != cudaSuccess) { rc = lr != ST_OK ? lr : ST_ECUDA; if (g) cudaGraphDestroy(g); break; }
        if (cudaGraphInstantiate(&f->exec[par], g, 0) != cudaSuccess) rc = ST_ECUDA;
        cudaGraphDestroy(g);
      }
      if (rc != ST_OK) drop_graphs(f);
      else { f->g_dt = dtf; f->g_jacobi = jacobi; f->g_vol = cv.d_vol; }
    }
    for (int k = 0; k < nsteps && rc == ST_OK; ++k) {
      if (cudaGraphLaunch(f->exec[f->parity], s) != cudaSuccess) rc = ST_ECUDA;
      else f->parity ^= 1;
    }
  } else {
    for (int k = 0; k < nsteps && rc == ST_OK; ++k) {
      rc = launch_step(f, f->parity, dtf, jacobi, s);
      if (rc == ST_OK) f->parity ^= 1;
    }
  }
  if (rc == ST_OK) f->steps += nsteps;
  if (e1) {
    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) rc = ST_ECUDA;
    else if (cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) { (void)cudaGetLastError(); *ms = 0.f; }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}

int st_fluid_state(st_fluid* f, float* vu, float* vv, float* dens, float* volume, double* t) {
  if (!f) return ST_EINVAL;
  if (cudaSetDevice(f->device) != cudaSuccess) return ST_ECUDA;
  st::CtxVolume cv;
  if (st::context_volume(f->ctx, &cv) != ST_OK) return ST_ESTATE;
  cudaStream_t s = cv.stream;
  const size_t n = (size_t)f->nr * f->nphi;
  float tt[2] = {0.f, 0.f};
  bool ok = true;
  if (vu) ok = ok && cudaMemcpyAsync(vu, f->F.vu, n * sizeof(float), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  if (vv) ok = ok && cudaMemcpyAsync(vv, f->F.vv, n * sizeof(float), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  if (dens)
    ok = ok && cudaMemcpyAsync(dens, f->F.dens[f->parity], n * sizeof(float), cudaMemcpyDeviceToHost, s) ==
                   cudaSuccess;
  if (volume) {
    if (!cv.on || cv.meta.nr != f->nr || cv.meta.nphi != f->nphi || cv.meta.nz != f->nz) return ST_ESTATE;
    ok = ok && cudaMemcpyAsync(volume, cv.d_vol, n * f->nz * sizeof(float), cudaMemcpyDeviceToHost, s) ==
                   cudaSuccess;
  }
  ok = ok && cudaMemcpyAsync(tt, f->F.t, sizeof tt, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(s) == cudaSuccess;
  if (!ok) return ST_ECUDA;
  if (t) *t = (double)tt[f->parity];
  return ST_OK;
}

void st_fluid_destroy(st_fluid* f) {
  if (!f) return;
  cudaSetDevice(f->device);
  drop_graphs(f);
  if (f->stream) cudaStreamSynchronize(f->stream);
  cudaFree(f->block);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
}

}  // extern "C"
