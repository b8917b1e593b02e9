// st_layered.cu -- the layered engine for Schwarzschild frames
// (src/metal.jl:2394-3147): an exact deflection fan for the sky, the disc /
// gas layer traced only where the fan cannot prove it empty, and a per-pixel
// composite.
//
// By spherical symmetry the sky a static observer at radius r sees is a
// function of one angle, psi, between the ray and the outward radial axis.
// One fan of geodesics over psi in [0, pi] (4096 rays, the work of one image
// column) plus a finer fan across the escape/capture transition replaces
// per-pixel sky integration: each pixel looks its exit direction up by its
// own psi and rebuilds it in its own geodesic plane.  Only the disc and gas,
// which break the symmetry, are integrated per pixel (the trace kernel's
// layer pass), at the display or a lower resolution, and composited over the
// sky.  The fan is indexed by the local angle in the static frame, so the
// camera must be the unboosted static observer (r >= 2.5 M).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "st_internal.h"
#include "st_trace.cuh"

namespace st {
namespace lay {

template <int PREC>
__global__ void __launch_bounds__(128) skyfan_kernel(const __grid_constant__ FanParams fp) {
  using R = typename RealOf<PREC>::T;
  using D = typename std::conditional<PREC == ST_PREC_FP32, float, double>::type;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= fp.n) return;
  const TraceParams& p = fp.p;
  D psi;
  if (fp.band) {
    const D lo = D(fp.band_lohi[0]), hi = D(fp.band_lohi[1]);
    psi = lo + (hi - lo) * D(k) / D(fp.n - 1);
  } else {
    psi = D(3.141592653589793) * D(k) / D(fp.n - 1);
  }
  const CamView cam{p.pos, p.Ef, p.Er, p.Eu, p.U, p.r_escape, p.nmax};
  RayState<R> st;
  init_ray_dir<PREC, 0, ST_SEM_DRAFT>(p, cam, 1, 1, cos_(psi), sin_(psi), D(0), D(0), D(0), st);
  R rmin = sqrt_(st.y[0] * st.y[0] + st.y[1] * st.y[1] + st.y[2] * st.y[2]);
  bool done = false;
  while (!done) {
    done = step_ray<PREC, 0, 0, ST_SEM_DRAFT>(p, st);
    rmin = min_(rmin, sqrt_(st.y[0] * st.y[0] + st.y[1] * st.y[1] + st.y[2] * st.y[2]));
  }
  const R M = PR(M);
  const R rf = max_(sqrt_(st.y[0] * st.y[0] + st.y[1] * st.y[1] + st.y[2] * st.y[2]), R(1e-6));
  // captured, or ended in the strong field: no sky (src/metal.jl:2504-2507)
  if ((st.flags & ST_RAY_CAPTURED) || rf < R(4) * M) {
    fp.out[k] = make_float4(0.f, 1.f, 0.f, (float)rmin);
    return;
  }
  R vel[6];
  rhs<0>(st.y, st.pt, M, R(0), vel);
  const R vl = max_(sqrt_(vel[0] * vel[0] + vel[1] * vel[1]), R(1e-20));
  fp.out[k] = make_float4(1.f, (float)(vel[0] / vl), (float)(vel[1] / vl), (float)rmin);
}

// The escape/capture transition of the coarse fan, padded by `pad` coarse
// spacings each side (src/metal.jl:2888-2898); band stays (0, 0) without one.
__global__ void fanband_kernel(const float4* __restrict__ fan, int n, int pad, float* band) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n - 1) return;
  if (fan[k].x != fan[k + 1].x) {
    const float dpsi = 3.14159265358979f / (float)(n - 1);
    band[0] = (float)max(k - pad, 0) * dpsi;
    band[1] = (float)min(k + 1 + pad, n - 1) * dpsi;
  }
}

// Fan lookup (src/metal.jl:2905-2937): the fine fan inside the band, the
// coarse one elsewhere; linear interpolation where neighbours agree on
// escape and direction, the nearest entry where they do not.
template <typename R>
__device__ __forceinline__ void fan_dir(const float4* __restrict__ fan, int n, const float4* __restrict__ fine,
                                        int nf, R lo, R hi, R psi, R* esc, R* c, R* s) {
  const bool use_fine = hi > lo && lo <= psi && psi <= hi;
  const float4* t = use_fine ? fine : fan;
  const int m = use_fine ? nf : n;
  const R tf = use_fine ? (psi - lo) / (hi - lo) * R(m - 1) : psi * R(m - 1) / R(3.141592653589793);
  const int k0 = min(max((int)tf, 0), m - 2);
  const R fr = tf - R(k0);
  const float4 a = t[k0], b = t[k0 + 1];
  if (a.x == b.x && R(a.y) * R(b.y) + R(a.z) * R(b.z) > R(0.9987)) {
    R cc = R(a.y) + fr * (R(b.y) - R(a.y));
    R ss = R(a.z) + fr * (R(b.z) - R(a.z));
    const R nl = max_(sqrt_(cc * cc + ss * ss), R(1e-6));
    *esc = R(a.x); *c = cc / nl; *s = ss / nl;
    return;
  }
  const float4 q = fr < R(0.5) ? a : b;
  *esc = R(q.x); *c = R(q.y); *s = R(q.z);
}

// Bilinear tap of the premultiplied layer at display pixel (i, j), 1-based
// (src/metal.jl:2670-2690).
__device__ __forceinline__ float4 layer_tap(const float4* __restrict__ L, int i, int j, int W, int H, int lw,
                                            int lh) {
  const float fx = ((float)i - 0.5f) * (float)lw / (float)W + 0.5f;
  const float fy = ((float)j - 0.5f) * (float)lh / (float)H + 0.5f;
  const int x0 = min(max((int)floorf(fx), 1), max(lw - 1, 1));
  const int y0 = min(max((int)floorf(fy), 1), max(lh - 1, 1));
  const float tx = fminf(fmaxf(fx - (float)x0, 0.f), 1.f);
  const float ty = fminf(fmaxf(fy - (float)y0, 0.f), 1.f);
  const int x1 = min(x0 + 1, lw), y1 = min(y0 + 1, lh);
  const float w00 = (1.f - tx) * (1.f - ty), w10 = tx * (1.f - ty), w01 = (1.f - tx) * ty, w11 = tx * ty;
  const float4 a = L[(y0 - 1) * lw + (x0 - 1)], b = L[(y0 - 1) * lw + (x1 - 1)];
  const float4 c = L[(y1 - 1) * lw + (x0 - 1)], d = L[(y1 - 1) * lw + (x1 - 1)];
  return make_float4(a.x * w00 + b.x * w10 + c.x * w01 + d.x * w11, a.y * w00 + b.y * w10 + c.y * w01 + d.y * w11,
                     a.z * w00 + b.z * w10 + c.z * w01 + d.z * w11, a.w * w00 + b.w * w10 + c.w * w01 + d.w * w11);
}

// Per display pixel: the pixel's ray as the trace kernel builds it, its
// local angle to the radial axis, the fan's exit direction rebuilt in the
// ray's own plane, the sky (and stars, and the relativistic tint) along it,
// and the layer composited over it (src/metal.jl:2707-2880).
template <int PREC>
__global__ void __launch_bounds__(128) composite_kernel(const __grid_constant__ TraceParams p,
                                                        const __grid_constant__ CompParams cp) {
  using R = typename RealOf<PREC>::T;
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, j0 = blockIdx.y * blockDim.y + threadIdx.y;
  if (i0 >= p.width || j0 >= p.height) return;
  const CamView cam{p.pos, p.Ef, p.Er, p.Eu, p.U, p.r_escape, p.nmax};
  RayState<R> st;
  init_ray<PREC, 0, ST_SEM_DRAFT>(p, cam, i0, j0, st);
  const R* y = st.y;
  const R pt = st.pt, M = PR(M);
  const R cpsi = clamp_(pt * R(p.er[0]) + y[3] * R(p.er[1]) + y[4] * R(p.er[2]) + y[5] * R(p.er[3]), R(-1), R(1));
  const R psi = acos_(cpsi);
  R esc, ct, sn;
  fan_dir<R>(cp.fan, cp.n, cp.fine, cp.nf, R(cp.band[0]), R(cp.band[1]), psi, &esc, &ct, &sn);
  R sky[3] = {R(0), R(0), R(0)};
  double dird[3] = {0, 0, 0};
  if (esc > R(0.5)) {
    const R r = sqrt_(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]), ir = R(1) / r;
    const R f = R(2) * M * ir;
    const R k0 = (y[0] * y[3] + y[1] * y[4] + y[2] * y[5]) * ir;
    const R c1 = f * (-pt + k0) * ir;
    const R vx = y[3] - c1 * y[0], vy = y[4] - c1 * y[1], vz = y[5] - c1 * y[2];
    const R e1x = y[0] * ir, e1y = y[1] * ir, e1z = y[2] * ir;
    const R vr = vx * e1x + vy * e1y + vz * e1z;
    R lx = vx - vr * e1x, ly = vy - vr * e1y, lz = vz - vr * e1z;
    const R ll = sqrt_(lx * lx + ly * ly + lz * lz);
    if (ll < R(1e-7)) {
      // (anti)radial ray: no deflection plane
      lx = -e1y; ly = e1x; lz = R(0);
      const R lm = max_(sqrt_(lx * lx + ly * ly), R(1e-6));
      lx /= lm; ly /= lm;
    } else {
      lx /= ll; ly /= ll; lz /= ll;
    }
    R dx = ct * e1x + sn * lx, dy = ct * e1y + sn * ly, dz = ct * e1z + sn * lz;
    const R dl = max_(sqrt_(dx * dx + dy * dy + dz * dz), R(1e-20));
    dx /= dl; dy /= dl; dz /= dl;
    dird[0] = (double)dx; dird[1] = (double)dy; dird[2] = (double)dz;
    sample_sky(p, acos_(clamp_(dz, R(-1), R(1))), atan2_(dy, dx), sky);
    if (p.star_strength > 0.0) {
      R sl[3];
      star_light<ST_SEM_DRAFT>(p, dx, dy, dz, sl);
      const R tw = R(p.star_tw), ss = R(p.star_strength);
      for (int c = 0; c < 3; ++c) sky[c] = sky[c] * tw + ss * sl[c];
    }
    const R g = st.scam;
    if (g != R(1)) {
      sky[0] *= R(57.4) / (exp_(R(4.067) / g) - R(1));
      sky[1] *= R(90.2) / (exp_(R(4.513) / g) - R(1));
      sky[2] *= R(206.5) / (exp_(R(5.335) / g) - R(1));
    }
  }
  float4 lay = make_float4(0.f, 0.f, 0.f, 1.f);
  if (cp.layer) lay = layer_tap(cp.layer, i0 + 1, j0 + 1, p.width, p.height, cp.lw, cp.lh);
  if (cp.ring && cp.ring_rmin > 0.f) {
    // foveated ring: toward the finer ring layer where the ray winds near the
    // photon sphere, feathered on the fan periapsis over the top fifth of
    // ring_rmin so the two resolutions never meet at a seam (src/metal.jl:2846-2863)
    const float tpsi = (float)psi * (float)(cp.n - 1) / 3.14159265358979f;
    const int rk0 = min(max((int)tpsi, 0), cp.n - 2);
    const float rfr = tpsi - (float)rk0;
    const float rmin = cp.fan[rk0].w + rfr * (cp.fan[rk0 + 1].w - cp.fan[rk0].w);
    const float rf = 0.8f;
    float t = (rmin - rf * cp.ring_rmin) / fmaxf((1.f - rf) * cp.ring_rmin, 1e-6f);
    t = fminf(fmaxf(t, 0.f), 1.f);
    const float wr = 1.f - t * t * (3.f - 2.f * t);
    if (wr > 0.f) {
      const float4 rg = layer_tap(cp.ring, i0 + 1, j0 + 1, p.width, p.height, cp.rw, cp.rh);
      lay.x += wr * (rg.x - lay.x); lay.y += wr * (rg.y - lay.y);
      lay.z += wr * (rg.z - lay.z); lay.w += wr * (rg.w - lay.w);
    }
  }
  const float w = p.weight;
  float4 o = make_float4(w * (lay.x + lay.w * (float)sky[0]), w * (lay.y + lay.w * (float)sky[1]),
                         w * (lay.z + lay.w * (float)sky[2]), lay.w);
  const int idx = j0 * p.width + i0;
  if (!p.first_pass) {
    const float4 prev = p.out[idx];
    o.x += prev.x; o.y += prev.y; o.z += prev.z;
  }
  p.out[idx] = o;
  if (p.diag) {
    st_ray_diag d;
    d.dir[0] = dird[0]; d.dir[1] = dird[1]; d.dir[2] = dird[2];
    d.flags = esc > R(0.5) ? ST_RAY_ESCAPED : (ST_RAY_CAPTURED | ST_RAY_BLACK);
    d.r_final = 0.f; d.alpha = lay.w; d.r_cross = -1.f; d.g_cross = 0.f; d.lambda = (float)psi;
    d.steps = 0; d.fp64_steps = 0; d.pad[0] = d.pad[1] = 0;
    p.diag[idx] = d;
  }
}

}  // namespace lay

cudaError_t launch_skyfan(int prec, const lay::FanParams& fp, cudaStream_t stream) {
  const unsigned nb = (unsigned)((fp.n + 127) / 128);
  if (prec == ST_PREC_FP64) lay::skyfan_kernel<ST_PREC_FP64><<<nb, 128, 0, stream>>>(fp);
  else lay::skyfan_kernel<ST_PREC_FP32><<<nb, 128, 0, stream>>>(fp);
  return cudaGetLastError();
}

cudaError_t launch_fanband(const float4* fan, int n, int pad, float* band, cudaStream_t stream) {
  lay::fanband_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(fan, n, pad, band);
  return cudaGetLastError();
}

namespace lay {
__global__ void fill_transparent_kernel(float4* __restrict__ L, size_t n) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) L[k] = make_float4(0.f, 0.f, 0.f, 1.f);
}
}  // namespace lay

cudaError_t launch_fill_transparent(float4* layer, size_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  lay::fill_transparent_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(layer, n);
  return cudaGetLastError();
}

cudaError_t launch_composite(int prec, const TraceParams& p, const lay::CompParams& cp, cudaStream_t stream) {
  const dim3 block(16, 8), grid((p.width + 15) / 16, (p.height + 7) / 8);
  if (prec == ST_PREC_FP64) lay::composite_kernel<ST_PREC_FP64><<<grid, block, 0, stream>>>(p, cp);
  else lay::composite_kernel<ST_PREC_FP32><<<grid, block, 0, stream>>>(p, cp);
  return cudaGetLastError();
}

}  // namespace st
