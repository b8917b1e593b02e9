// st_trace.cuh -- device code of the null-geodesic trace (sm_103a).
//
// One ray = one pixel sample, traced backward from the camera in Cartesian
// Kerr-Schild coordinates: tetrad ray generation, radius-adaptive RK4 with
// horizon / escape termination, thin-disc or volumetric-gas shading, and the
// equirectangular sky.  The rules follow SpaceTime.jl's two renderers:
//   SEM = ST_SEM_DRAFT   trace_kernel_mtl!  (src/metal.jl:750-1707)
//   SEM = ST_SEM_RENDER  render / _trace_color (src/raytrace.jl:225-428,
//                        src/callbacks.jl:7-105, src/accretion_disc.jl:19-49)
// Precision:
//   ST_PREC_FP64          all double
//   ST_PREC_FP32          all float (the reference kernel's arithmetic)
//   ST_PREC_FP32_GUARDED  float RHS, float-float (TwoSum) state, FP64 steps
//                         for guarded rays/regions, FP64 null renormalisation
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "st_internal.h"

namespace st {

// ---------------------------------------------------------------------------
// Scalar helpers: the double forms follow the oracle's arithmetic exactly;
// the float forms use the MUFU reciprocal / reciprocal-sqrt.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
// MUFU reciprocal (at most 1 ulp; subnormals flushed, as in the fast-math units)
__device__ __forceinline__ float rcp_(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }
// MUFU base-2 exponential and logarithm (PTX ex2 / lg2 .approx.ftz), for the
// float units' emission terms written in base 2
__device__ __forceinline__ float ex2_(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float lg2_(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// log2(e), for the base-2 forms of exp(c x)
constexpr double kLog2e = 1.4426950408889634;
__device__ __forceinline__ float exp_(float x) { return expf(x); }
__device__ __forceinline__ double exp_(double x) { return exp(x); }
__device__ __forceinline__ float log_(float x) { return logf(x); }
__device__ __forceinline__ double log_(double x) { return log(x); }
__device__ __forceinline__ float atan2_(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double atan2_(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float acos_(float x) { return acosf(x); }
__device__ __forceinline__ double acos_(double x) { return acos(x); }
__device__ __forceinline__ float cos_(float x) { return cosf(x); }
__device__ __forceinline__ double cos_(double x) { return cos(x); }
__device__ __forceinline__ float sin_(float x) { return sinf(x); }
__device__ __forceinline__ double sin_(double x) { return sin(x); }
__device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
__device__ __forceinline__ double fabs_(double x) { return fabs(x); }
__device__ __forceinline__ float floor_(float x) { return floorf(x); }
__device__ __forceinline__ double floor_(double x) { return floor(x); }
// A parameter in the variant's precision: the float copy for float code, the
// double for double code (no conversion either way).
template <typename R> __device__ __forceinline__ R pr(double d, float f);
template <> __device__ __forceinline__ float pr<float>(double, float f) { return f; }
template <> __device__ __forceinline__ double pr<double>(double d, float) { return d; }
#define PR(x) pr<R>(p.x, p.f.x)
template <typename R> __device__ __forceinline__ R min_(R a, R b) { return a < b ? a : b; }
template <typename R> __device__ __forceinline__ R max_(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R clamp_(R x, R lo, R hi) { return x < lo ? lo : (x > hi ? hi : x); }

// r and 1/r from r^2
__device__ __forceinline__ void r_and_inv(float r2, float& r, float& ir) { ir = rsqrtf(r2); r = r2 * ir; }
__device__ __forceinline__ void r_and_inv(double r2, double& r, double& ir) { r = sqrt(r2); ir = 1.0 / r; }

template <typename R> struct IsD { static constexpr bool v = std::is_same<R, double>::value; };

// Integer hash -> [0,1): src/disc_sim.jl:83-91 (bit-exact).
__device__ __forceinline__ float sim_hash(int x, int y, int z) {
  uint32_t h = (uint32_t)x * 0x8da6b343u ^ (uint32_t)y * 0xd8163841u ^ (uint32_t)z * 0xcb1ab31fu;
  h ^= h >> 13;
  h *= 0x9e3779b9u;
  h ^= h >> 16;
  return (float)(h & 0x00ffffffu) * 5.9604645e-8f;
}

// ---------------------------------------------------------------------------
// Geodesic RHS in Cartesian Kerr-Schild coordinates.
// ---------------------------------------------------------------------------

// Schwarzschild, src/gr.jl:85-109 / src/metal.jl:324-340.
template <typename R>
__device__ __forceinline__ void rhs_schw(const R* s, R pt, R M, R* d) {
  const R x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const R r2 = x * x + y * y + z * z;
  R inv_r;
  if constexpr (IsD<R>::v) inv_r = 1.0 / sqrt(r2); else inv_r = rsqrtf(r2);
  const R f = R(2) * M * inv_r;
  const R kap = (x * px + y * py + z * pz) * inv_r;
  const R ell = -pt + kap;
  const R c1 = f * ell * inv_r;
  R c2;
  if constexpr (IsD<R>::v) c2 = f * ell * (R(0.5) * ell + kap) * inv_r * inv_r;
  else c2 = c1 * fmaf(0.5f, ell, kap) * inv_r;  // the same product, sharing c1
  d[0] = px - c1 * x;
  d[1] = py - c1 * y;
  d[2] = pz - c1 * z;
  d[3] = c1 * px - c2 * x;
  d[4] = c1 * py - c2 * y;
  d[5] = c1 * pz - c2 * z;
}

// Kerr-Schild r^2 from the implicit quartic, in float (the form both the
// RHS and the step's kill test use, so a step can pass it to its first RHS).
// With w/2 = (x^2 + y^2 + z^2 - a^2)/2 the root is w/2 + sqrt((w/2)^2 + a^2 z^2).
__device__ __forceinline__ float ks_r2_f32(float x, float y, float z, float a) {
  const float a2 = a * a, z2 = z * z;
  const float wh = fmaf(fmaf(x, x, fmaf(y, y, z2)), 0.5f, -(0.5f * a2));
  return wh + sqrtf(fmaf(wh, wh, a2 * z2));
}

template <typename R>
__device__ __forceinline__ R ks_r2(R x, R y, R z, R a) {
  if constexpr (std::is_same<R, float>::value) return ks_r2_f32(x, y, z, a);
  const R a2 = a * a;
  const R w = x * x + y * y + z * z - a2;
  return R(0.5) * (w + sqrt_(w * w + R(4) * a2 * z * z));
}

// Kerr in float: the same Hamiltonian derivatives regrouped to share their
// products (about a quarter fewer multiplies than the term-by-term form).
// With A = p_x x + p_y y, B = p_x y - p_y x, T = (r A + a B)/(r^2 + a^2) and
// Z = z p_z / r:
//   l = L.p - p_t = T + Z - p_t
//   dl/dr         = (A - 2 r T)/(r^2 + a^2) - Z / r
//   dx_xy         = p_xy - f l / (r^2 + a^2) (r x + a y, r y - a x)
//   dp_xy         = G r^3/Sigma (x, y) + f l / (r^2 + a^2) (r p_x - a p_y, r p_y + a p_x)
//   dp_z          = z/Sigma (G r (r^2 + a^2) - a^2 l (f l)) + f l p_z / r
// where G = l^2/2 df/dr + f l dl/dr collects every term along grad r.  The f
// derivatives come from f itself: df/dr = (f/r)(3 a^2 z^2 - r^4)/Sigma, and
// since Sigma = r^4 + a^2 z^2, (3 a^2 z^2 - r^4)/Sigma = 4 a^2 z^2/Sigma - 1,
// so G = f l (dl/dr + (l/r)(2 a^2 z^2/Sigma - 1/2)); df/dz = -2 a^2 z f/Sigma.
// r2_known: this state's ks_r2_f32 when the caller has it, else negative.
__device__ __forceinline__ void rhs_kerr_f32(const float* s, float pt, float M, float a, float* d,
                                             float r2_known = -1.f) {
  const float x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const float a2 = a * a, z2 = z * z;
  const float q = a2 * z2;
  float r2 = r2_known >= 0.f ? r2_known : ks_r2_f32(x, y, z, a);
  r2 = fmaxf(r2, 1e-12f);
  float r, ir;
  r_and_inv(r2, r, ir);
  const float isig = rcp_(fmaf(r2, r2, q));
  const float r2a = r2 + a2;
  const float ira = rcp_(r2a);
  const float A = fmaf(px, x, py * y);
  const float B = fmaf(px, y, -(py * x));
  const float T = fmaf(r, A, a * B) * ira;
  const float Z = (z * pz) * ir;
  const float ell = (T + Z) - pt;
  const float rsig = (r2 * r) * isig;
  const float fl = ((2.f * M) * rsig) * ell;
  const float Fi = fl * ira;
  const float Fr = Fi * r, Fa = Fi * a;
  const float flir = fl * ir;
  d[0] = fmaf(-Fr, x, fmaf(-Fa, y, px));
  d[1] = fmaf(-Fr, y, fmaf(Fa, x, py));
  d[2] = fmaf(-flir, z, pz);
  const float dldr = fmaf(fmaf(-2.f * r, T, A), ira, -(Z * ir));
  const float inner = fmaf(ell * ir, fmaf(q + q, isig, -0.5f), dldr);
  const float G = fl * inner;
  const float Gr = G * rsig;
  d[3] = fmaf(Gr, x, fmaf(Fr, px, -(Fa * py)));
  d[4] = fmaf(Gr, y, fmaf(Fr, py, Fa * px));
  d[5] = fmaf(z * isig, fmaf(G * r, r2a, -((a2 * ell) * fl)), flir * pz);
}

// The regrouped Kerr RHS above in double, for the FP32_GUARDED path's FP64
// guard steps: the same algebra (r from the half-w quartic root, one
// reciprocal square root for r and 1/r, two reciprocals), so a guard step
// issues about half the FP64 instructions of the term-by-term form.  On GB300
// an FP64 instruction costs tens of FP32 ones; the all-FP64 precision keeps
// the term-by-term form the oracle restates.
__device__ __forceinline__ void rhs_kerr_rg64(const double* s, double pt, double M, double a, double* d) {
  const double x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const double a2 = a * a, z2 = z * z;
  const double q = a2 * z2;
  const double wh = fma(fma(x, x, fma(y, y, z2)), 0.5, -(0.5 * a2));
  const double r2 = fmax(wh + sqrt(fma(wh, wh, q)), 1e-12);
  const double ir = rsqrt(r2), r = r2 * ir;
  const double isig = 1.0 / fma(r2, r2, q);
  const double r2a = r2 + a2;
  const double ira = 1.0 / r2a;
  const double A = fma(px, x, py * y);
  const double B = fma(px, y, -(py * x));
  const double T = fma(r, A, a * B) * ira;
  const double Z = (z * pz) * ir;
  const double ell = (T + Z) - pt;
  const double rsig = (r2 * r) * isig;
  const double fl = ((2.0 * M) * rsig) * ell;
  const double Fi = fl * ira;
  const double Fr = Fi * r, Fa = Fi * a;
  const double flir = fl * ir;
  d[0] = fma(-Fr, x, fma(-Fa, y, px));
  d[1] = fma(-Fr, y, fma(Fa, x, py));
  d[2] = fma(-flir, z, pz);
  const double dldr = fma(fma(-2.0 * r, T, A), ira, -(Z * ir));
  const double inner = fma(ell * ir, fma(q + q, isig, -0.5), dldr);
  const double G = fl * inner;
  const double Gr = G * rsig;
  d[3] = fma(Gr, x, fma(Fr, px, -(Fa * py)));
  d[4] = fma(Gr, y, fma(Fr, py, Fa * px));
  d[5] = fma(z * isig, fma(G * r, r2a, -((a2 * ell) * fl)), flir * pz);
}

// Kerr, src/metal.jl:466-508 (implicit-quartic r, four derivative terms).
template <typename R>
__device__ __forceinline__ void rhs_kerr(const R* s, R pt, R M, R a, R* d) {
  if constexpr (std::is_same<R, float>::value) {
    rhs_kerr_f32(s, pt, M, a, d);
    return;
  }
  const R x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const R a2 = a * a, z2 = z * z;
  R r2 = ks_r2(x, y, z, a);
  r2 = max_(r2, R(1e-12));
  R r, inv_r;
  r_and_inv(r2, r, inv_r);
  const R r3 = r2 * r;
  const R inv_sig = rcp_(r2 * r2 + a2 * z2);
  const R r2a = r2 + a2;
  const R ira = rcp_(r2a);
  const R Lx = (r * x + a * y) * ira;
  const R Ly = (r * y - a * x) * ira;
  const R Lz = z * inv_r;
  const R ell = -pt + Lx * px + Ly * py + Lz * pz;
  const R f = R(2) * M * r3 * inv_sig;
  const R fl = f * ell;
  const R drx = x * r3 * inv_sig;
  const R dry = y * r3 * inv_sig;
  const R drz = z * r * r2a * inv_sig;
  const R dfdr = R(2) * M * r2 * (R(3) * a2 * z2 - r2 * r2) * inv_sig * inv_sig;
  const R dfz0 = R(-4) * M * r3 * a2 * z * inv_sig * inv_sig;
  const R dlx0 = (r * px - a * py) * ira;
  const R dly0 = (a * px + r * py) * ira;
  const R dlz0 = pz * inv_r;
  const R dldr = (px * (x * r2a - R(2) * r * (r * x + a * y)) + py * (y * r2a - R(2) * r * (r * y - a * x))) *
                     ira * ira -
                 z * pz * inv_r * inv_r;
  const R hl2 = R(0.5) * ell * ell;
  d[0] = px - fl * Lx;
  d[1] = py - fl * Ly;
  d[2] = pz - fl * Lz;
  d[3] = hl2 * (dfdr * drx) + fl * (dldr * drx + dlx0);
  d[4] = hl2 * (dfdr * dry) + fl * (dldr * dry + dly0);
  d[5] = hl2 * (dfdr * drz + dfz0) + fl * (dldr * drz + dlz0);
}

template <int KERR, typename R>
__device__ __forceinline__ void rhs(const R* s, R pt, R M, R a, R* d) {
  if constexpr (KERR) rhs_kerr(s, pt, M, a, d); else rhs_schw(s, pt, M, d);
}

// Packed FP32 pairs (Blackwell FFMA2 / FMUL2 / FADD2): one issued
// instruction does the float operation on both halves, each rounded as the
// scalar __fmaf_rn / __fmul_rn / __fadd_rn would.
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Classical RK4 increment (src/metal.jl:1382-1401); k1 is the slope at y.
// In float the six components run as three packed pairs.
template <int KERR, typename R>
__device__ __forceinline__ void rk4_inc(const R* y, R pt, R M, R a, R h, const R* k1, R* inc) {
  if constexpr (std::is_same<R, float>::value) {
    const float2 hh = pk(0.5f * h, 0.5f * h), hf = pk(h, h), two = pk(2.f, 2.f);
    float2 Y[3], S[3], T[3];
    float t[6], k[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Y[i] = pk(y[2 * i], y[2 * i + 1]);
      S[i] = pk(k1[2 * i], k1[2 * i + 1]);
      T[i] = fma2(hh, S[i], Y[i]);
      t[2 * i] = T[i].x; t[2 * i + 1] = T[i].y;
    }
    rhs<KERR>(t, pt, M, a, k);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 K = pk(k[2 * i], k[2 * i + 1]);
      S[i] = fma2(two, K, S[i]);
      T[i] = fma2(hh, K, Y[i]);
      t[2 * i] = T[i].x; t[2 * i + 1] = T[i].y;
    }
    rhs<KERR>(t, pt, M, a, k);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 K = pk(k[2 * i], k[2 * i + 1]);
      S[i] = fma2(two, K, S[i]);
      T[i] = fma2(hf, K, Y[i]);
      t[2 * i] = T[i].x; t[2 * i + 1] = T[i].y;
    }
    rhs<KERR>(t, pt, M, a, k);
    const float h6 = h / 6.f;
    const float2 h6p = pk(h6, h6);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 o = mul2(h6p, add2(S[i], pk(k[2 * i], k[2 * i + 1])));
      inc[2 * i] = o.x; inc[2 * i + 1] = o.y;
    }
    return;
  }
  R t[6], k[6], sum[6];
  const R hh = R(0.5) * h;
#pragma unroll
  for (int i = 0; i < 6; ++i) { t[i] = y[i] + hh * k1[i]; sum[i] = k1[i]; }
  rhs<KERR>(t, pt, M, a, k);
#pragma unroll
  for (int i = 0; i < 6; ++i) { sum[i] = sum[i] + R(2) * k[i]; t[i] = y[i] + hh * k[i]; }
  rhs<KERR>(t, pt, M, a, k);
#pragma unroll
  for (int i = 0; i < 6; ++i) { sum[i] = sum[i] + R(2) * k[i]; t[i] = y[i] + h * k[i]; }
  rhs<KERR>(t, pt, M, a, k);
  const R h6 = h / R(6);
#pragma unroll
  for (int i = 0; i < 6; ++i) inc[i] = h6 * (sum[i] + k[i]);
}

// (hi + lo) += d with Knuth's TwoSum; hi keeps the rounded sum.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float d) {
  const float s = __fadd_rn(hi, d);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
  const float l2 = __fadd_rn(lo, e);
  const float t = __fadd_rn(s, l2);
  lo = __fsub_rn(l2, __fsub_rn(t, s));
  hi = t;
}

// ---------------------------------------------------------------------------
// Emission models (see the oracle for the reference line numbers).
// ---------------------------------------------------------------------------

// Exact emitter shift 1+z = -p.u/E, src/metal.jl:396-428.
template <typename R>
__device__ __forceinline__ R emitter_opz(R sx, R sy, R psx, R psy, R E, R M, R a, R r_isco, R E_isco, R L_isco) {
  const R a2 = a * a;
  const R s2 = sx * sx + sy * sy;
  const R r = sqrt_(max_(s2 - a2, R(1e-6)));
  const R sqM = sqrt_(M), sqr = sqrt_(r), r32 = r * sqr;
  const R delta = r * r - R(2) * M * r + a2;
  R ut, uphi, ur = R(0);
  R ux, uy;
  if (r >= r_isco) {
    const R den = r32 - R(3) * M * sqr + R(2) * a * sqM;
    if constexpr (IsD<R>::v) {
      ut = (r32 + a * sqM) / (sqrt_(r32) * sqrt_(max_(den, R(1e-2))));
      uphi = sqM / (r32 + a * sqM) * ut;
    } else {
      // one reciprocal square root for 1 / (sqrt(r^3/2) sqrt(den)); uphi's
      // (r^3/2 + a sqrt M) cancels against ut's
      const R inv = rsqrtf(r32 * max_(den, R(1e-2)));
      ut = (r32 + a * sqM) * inv;
      uphi = sqM * inv;
    }
    // circular orbit: u^r = 0, so the radial basis vector drops out exactly
    // (0 * cos(phi) - y u^phi rounds as -y u^phi)
    ux = -(sy * uphi);
    uy = sx * uphi;
  } else {
    const R inv_d = R(1) / max_(delta, R(1e-3));
    ut = ((r * r + a2 + R(2) * M * a2 / r) * E_isco - R(2) * M * a * L_isco / r) * inv_d;
    uphi = (R(2) * M * a * E_isco / r + (R(1) - R(2) * M / r) * L_isco) * inv_d;
    const R t1 = E_isco * (r * r + a2) - a * L_isco;
    const R t2 = L_isco - a * E_isco;
    const R Rr = t1 * t1 - delta * (r * r + t2 * t2);
    ur = -sqrt_(max_(Rr, R(0))) / (r * r);
    ut += R(2) * M * r * inv_d * ur;
    uphi += a * inv_d * ur;
    const R inv_s2 = R(1) / max_(s2, R(1e-6));
    const R cphi = (r * sx + a * sy) * inv_s2;
    const R sphi = (r * sy - a * sx) * inv_s2;
    ux = ur * cphi - sy * uphi;
    uy = ur * sphi + sx * uphi;
  }
  const R Es = fabs_(E) > R(1e-6) ? E : R(1e-6);
  return clamp_(ut - (psx * ux + psy * uy) / Es, R(0.1), R(20));
}

// LUT colour; RENDER rounds half to even (Julia round), DRAFT truncates x+0.5.
// The blackbody table staged in the pixel kernel's dynamic shared memory
// (TraceParams::lut_stage; the kernel copies it there before its first ray).
extern __shared__ float4 st_lut_smem[];

template <typename R>
__device__ __forceinline__ float4 lut_color(const TraceParams& p, R T, bool render_rule) {
  const R tmin = PR(lut_tmin), tmax = PR(lut_tmax);
  int idx;
  if constexpr (IsD<R>::v) {
    const R fr = (clamp_(T, tmin, tmax) - tmin) / (tmax - tmin);
    if (render_rule) idx = (int)rint(fr * R(p.lut_size - 1));
    else idx = (int)(fr * (R(p.lut_size) - R(1)) + R(0.5));
  } else {  // the index scale comes from the host: no division per lookup
    const R x = (clamp_(T, tmin, tmax) - tmin) * p.f.lut_sc;
    idx = render_rule ? (int)rintf(x) : (int)(x + R(0.5));
  }
  idx = min(max(idx, 0), p.lut_size - 1);
  if (p.lut_stage) return st_lut_smem[idx];
  return __ldg(p.lut + idx);
}

// Trilinear gas density, src/metal.jl:569-610.
template <typename R>
__device__ __forceinline__ R sample_volume(const TraceParams& p, R sc, R phi, R z) {
  const int nr = p.nr, nphi = p.nphi, nz = p.nz;
  const float* v = p.vol;
  if constexpr (!IsD<R>::v) {
    // The gas march calls this with sc > 1e-6 and |z| < zmax already checked.
    // (ln s - ln s_in) (nr - 1) / (ln s_out - ln s_in) from log2 s, with the
    // scale and offset from the host; inside the grid iff 0 < fr < nr - 1, so
    // floor(fr) lies in [0, nr - 2] with no clamp.
    const float fr = fmaf(lg2_(sc), p.f.vol_sr2, p.f.vol_r0);
    if (!(fr > 0.f && fr < p.f.vol_rmax)) return 0.f;
    const float flr = floorf(fr);
    const int i0 = (int)flr;
    const float tr = fr - flr;
    // phi comes from atan2: |phi| <= pi, so mod(phi, 2 pi) is one conditional
    // add, fp lies in [0, nphi] and its floor wraps by one compare
    const float pm = phi < 0.f ? phi + 6.283185307179586f : phi;
    const float fp = pm * p.f.vol_sp;
    const float flp = floorf(fp);
    const int j0 = (int)flp;
    const float tp = fp - flp;
    const int ja = j0 >= nphi ? j0 - nphi : j0;
    const int jb = ja + 1 >= nphi ? 0 : ja + 1;
    // z + zmax > 0, so only the upper end needs the clamp
    const float fz = (z + PR(zmax)) * p.f.vol_sz;
    const int k0 = min((int)floorf(fz), nz - 2);
    const float tz = fz - (float)k0;
    // 32-bit offsets (the context limits the grid to 2^31 cells)
    const int sk = nr * nphi;
    const int base = i0 + sk * k0;
    const float* v00 = v + (base + nr * ja);
    const float* v10 = v + (base + nr * jb);
    const float* v01 = v00 + sk;
    const float* v11 = v10 + sk;
    const float d000 = __ldg(v00), d100 = __ldg(v00 + 1);
    const float d010 = __ldg(v10), d110 = __ldg(v10 + 1);
    const float d001 = __ldg(v01), d101 = __ldg(v01 + 1);
    const float d011 = __ldg(v11), d111 = __ldg(v11 + 1);
    const float c00 = d000 + tr * (d100 - d000);
    const float c10 = d010 + tr * (d110 - d010);
    const float c01 = d001 + tr * (d101 - d001);
    const float c11 = d011 + tr * (d111 - d011);
    const float c0 = c00 + tp * (c10 - c00);
    const float c1 = c01 + tp * (c11 - c01);
    return c0 + tz * (c1 - c0);
  } else {
    const R zmax = PR(zmax);
    if (sc <= R(0) || fabs_(z) >= zmax) return R(0);
    const R ls = log_(sc);
    const R lin = PR(ls_in), lout = PR(ls_out);
    if (ls <= lin || ls >= lout) return R(0);
    const R two_pi = R(6.283185307179586);
    R pm = phi;
    if (pm < R(0)) pm += two_pi;
    const R fr = (ls - lin) / (lout - lin) * R(nr - 1);
    const R fp = pm / two_pi * R(nphi);
    const R fz = (z + zmax) / (R(2) * zmax) * R(nz - 1);
    const int i0 = min(max((int)floor_(fr), 0), nr - 2);
    const R tr = fr - R(i0);
    const int j0 = (int)floor_(fp);
    const R tp = fp - R(j0);
    const int k0 = min(max((int)floor_(fz), 0), nz - 2);
    const R tz = fz - R(k0);
    // j0 is in [0, nphi] (fp < nphi up to rounding): wrap by compare, not by division
    const int ja = j0 >= nphi ? j0 - nphi : (j0 < 0 ? j0 + nphi : j0);
    const int jb = ja + 1 >= nphi ? ja + 1 - nphi : ja + 1;
    const size_t sj = (size_t)nr, sk = (size_t)nr * nphi;
    const size_t b00 = (size_t)i0 + sj * ja + sk * k0, b10 = (size_t)i0 + sj * jb + sk * k0;
    const size_t b01 = b00 + sk, b11 = b10 + sk;
    const R d000 = __ldg(v + b00), d100 = __ldg(v + b00 + 1);
    const R d010 = __ldg(v + b10), d110 = __ldg(v + b10 + 1);
    const R d001 = __ldg(v + b01), d101 = __ldg(v + b01 + 1);
    const R d011 = __ldg(v + b11), d111 = __ldg(v + b11 + 1);
    const R c00 = d000 + tr * (d100 - d000);
    const R c10 = d010 + tr * (d110 - d010);
    const R c01 = d001 + tr * (d101 - d001);
    const R c11 = d011 + tr * (d111 - d011);
    const R c0 = c00 + tp * (c10 - c00);
    const R c1 = c01 + tp * (c11 - c01);
    return c0 + tz * (c1 - c0);
  }
}

// Bilinear equirectangular sky, src/metal.jl:523-561 / src/raytrace.jl:154-177.
template <typename R>
__device__ __forceinline__ void sample_sky(const TraceParams& p, R theta, R phi, R* rgb) {
  const int W = p.sky_w, H = p.sky_h;
  const R pi = R(3.141592653589793), two_pi = R(6.283185307179586);
  const R v = clamp_(theta / pi, R(0), R(1));
  R pm = phi;  // from atan2: |phi| <= pi
  if (pm < R(0)) pm += two_pi;
  const R u = clamp_(pm / two_pi, R(0), R(1));
  const R xf = u * R(W - 1), yf = v * R(H - 1);
  const int x0 = min(max((int)floor_(xf), 0), W - 1);
  const int x1 = min(x0 + 1, W - 1);
  const int y0 = min(max((int)floor_(yf), 0), H - 1);
  const int y1 = min(y0 + 1, H - 1);
  const R fx = xf - R(x0), fy = yf - R(y0);
  const float4 c00 = __ldg(p.sky + (size_t)y0 * W + x0), c10 = __ldg(p.sky + (size_t)y0 * W + x1);
  const float4 c01 = __ldg(p.sky + (size_t)y1 * W + x0), c11 = __ldg(p.sky + (size_t)y1 * W + x1);
  const R w00 = (R(1) - fx) * (R(1) - fy), w10 = fx * (R(1) - fy), w01 = (R(1) - fx) * fy, w11 = fx * fy;
  rgb[0] = R(c00.x) * w00 + R(c10.x) * w10 + R(c01.x) * w01 + R(c11.x) * w11;
  rgb[1] = R(c00.y) * w00 + R(c10.y) * w10 + R(c01.y) * w01 + R(c11.y) * w11;
  rgb[2] = R(c00.z) * w00 + R(c10.z) * w10 + R(c01.z) * w01 + R(c11.z) * w11;
}

// ---------------------------------------------------------------------------
// Ray state machine.
// ---------------------------------------------------------------------------

template <int PREC>
struct RealOf { using T = float; };
template <>
struct RealOf<ST_PREC_FP64> { using T = double; };

template <typename R>
struct RayState {
  R y[6];        // (x, y, z, p_x, p_y, p_z); hi parts under FP32_GUARDED
  float lo[6];   // FP32_GUARDED low parts
  R pt;          // conserved p_t
  R scam;        // camera shift applied to shading (1 if not relativistic)
  R acc[3];
  R alpha;
  R r_prev;      // DRAFT Schwarzschild inward test
  R r_floor;
  R march_acc;   // arc length since the last gas sample
  R lambda;      // affine parameter (RENDER budget)
  int steps, fp64_steps, gas;
  int flags;     // ST_RAY_* bits in progress
  int pix;       // global ray index
  float r_cross, g_cross;
  R r_esc;       // escape radius of this ray's frame
  int nmax;      // step budget of this ray's frame
  bool inside0;  // RENDER: camera inside r = 2.00001
  bool guard_ray;
  // adaptive Tsitouras 5(4) state (order 45/46): carried step, previous
  // error for the PI controller, FSAL slope
  R h_carry, err_prev;
  R k1c[6];
  bool k1_valid;
  R r_layer_prev;  // layer pass: previous radius beyond the gate
  R ell;           // depth buckets: path length travelled
};

// Depth bucket of path length ell (1-based as in the reference): the first
// below 1.5 M, log-spaced to 120 M, the last (nb) kept for the sky.
template <typename R>
__device__ __forceinline__ int depth_bucket(R ell, int nb) {
  if (ell <= R(1.5)) return 1;
  const R bscale = nb > 2 ? R(nb - 2) * R(0.22820f) : R(1);
  const int b = (int)((log_(ell) - R(0.405465f)) * bscale) + 1;
  return min(max(b, 1), nb - 1);
}

// Depth-bucket mode keeps nothing in acc between steps: the emission of one
// step (disc crossing or gas samples) is moved into the bucket of the path
// length reached at that step, src/metal.jl:1489-1497, 1556-1563.
template <typename R>
__device__ __forceinline__ void flush_bucket(const TraceParams& p, int pix, R ell, R* acc) {
  if (acc[0] == R(0) && acc[1] == R(0) && acc[2] == R(0)) return;
  float* b = p.buckets + (size_t)pix * 3 * p.nb + 3 * (depth_bucket(ell, p.nb) - 1);
  b[0] += p.weight * (float)acc[0];
  b[1] += p.weight * (float)acc[1];
  b[2] += p.weight * (float)acc[2];
  acc[0] = R(0); acc[1] = R(0); acc[2] = R(0);
}

// A DRAFT ray the Bardeen launch test proves captured is black whatever its
// integration does (the classification of src/metal.jl:1633-1636); with neither
// disc nor gas in the scene there is nothing for it to collect on the way in,
// so its pixel is final at launch and the integration is skipped.
template <int SEM>
__device__ __forceinline__ bool final_at_launch(const TraceParams& p, int flags) {
  if constexpr (SEM != ST_SEM_DRAFT) return false;
  return (flags & ST_RAY_BCAPT) && !p.disc_on && !p.vol_on && !p.layer;
}

// Internal ray flag of the layer pass: the fan proves the ray misses the gate.
constexpr int ST_RAY_LAYER_CULLED = 1 << 20;
// Internal ray flag of the guarded schedule: the ray stopped before its first
// FP64 guard step, its state saved for the resume kernel.
constexpr int ST_RAY_DEFER = 1 << 21;
constexpr int ST_RAY_INTERNAL = ST_RAY_LAYER_CULLED | ST_RAY_DEFER;

// Camera tetrad for the current ray; per-frame data lives in TraceParams for
// single frames and in FrameCam for batched tracks (st_render_frames).
struct CamView {
  const double* pos;
  const double* Ef;
  const double* Er;
  const double* Eu;
  const double* U;
  double r_escape;
  int nmax;
};

template <int KERR, typename D>
__device__ __forceinline__ void lower_photon(const D* x, const D* q, D M, D a, D* s, D* pt) {
  D l[3], f;
  if constexpr (KERR) {
    const D a2 = a * a;
    const D rk2 = ks_r2(x[0], x[1], x[2], a);
    const D rk = sqrt_(max_(rk2, D(1e-12)));
    const D ira = D(1) / (rk2 + a2);
    l[0] = (rk * x[0] + a * x[1]) * ira;
    l[1] = (rk * x[1] - a * x[0]) * ira;
    l[2] = x[2] / rk;
    f = D(2) * M * rk2 * rk / (rk2 * rk2 + a2 * x[2] * x[2]);
  } else {
    const D r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    l[0] = x[0] / r; l[1] = x[1] / r; l[2] = x[2] / r;
    f = D(2) * M / r;
  }
  const D lq = q[0] + l[0] * q[1] + l[1] * q[2] + l[2] * q[3];
  *pt = -q[0] + f * lq;
#pragma unroll
  for (int k = 0; k < 3; ++k) { s[k] = x[k]; s[k + 3] = q[k + 1] + f * lq * l[k]; }
}

// Bardeen launch-time capture test (Kerr), src/metal.jl:1026-1094.
template <typename D>
__device__ void bardeen(const D* y, D pt, D M, D a, bool* captured0, bool* graze0) {
  *captured0 = false;
  *graze0 = false;
  const D E0 = -pt;
  if (!(fabs_(E0) > D(1e-6))) return;
  const D x = y[0], yy = y[1], z = y[2], px = y[3], py = y[4], pz = y[5];
  const D a2 = a * a;
  const D rk2 = ks_r2(x, yy, z, a);
  const D rk = sqrt_(max_(rk2, D(1e-12)));
  const D cth = z / rk;
  const D s2 = max_(D(1) - cth * cth, D(1e-8));
  const D sth = sqrt_(s2);
  const D Lz0 = x * py - yy * px;
  const D pth = (cth / sth) * (x * px + yy * py) - rk * sth * pz;
  const D Q0 = pth * pth + cth * cth * (Lz0 * Lz0 / s2 - a2 * E0 * E0);
  const D lam = Lz0 / E0, eta = Q0 / (E0 * E0);
  const D c2 = a2 - lam * lam - eta;
  const D c1 = D(2) * M * (eta + (lam - a) * (lam - a));
  const D c0 = -a2 * eta;
  const D rplus = M + sqrt_(max_(M * M - a2, D(0)));
  D v[6];
  rhs_kerr(y, pt, M, a, v);
  const D rdot = rk2 * (x * v[0] + yy * v[1]) + (rk2 + a2) * z * v[2];
  if (!(rdot < D(0))) return;
  const D pb = D(0.5) * c2, qb = D(0.25) * c1;
  const D Db = D(0.25) * qb * qb + pb * pb * pb / D(27);
  bool cap = true;
  if (Db >= D(0)) {
    const D sD = sqrt_(Db);
    const D u1 = D(-0.5) * qb + sD, u2 = D(-0.5) * qb - sD;
    const D s1 = u1 > D(0) ? D(1) : (u1 < D(0) ? D(-1) : D(0));
    const D s2b = u2 > D(0) ? D(1) : (u2 < D(0) ? D(-1) : D(0));
    const D rc = s1 * exp_(log_(max_(fabs_(u1), D(1e-30))) / D(3)) + s2b * exp_(log_(max_(fabs_(u2), D(1e-30))) / D(3));
    if (rc > rplus && rc < rk) {
      const D Rv = ((rc * rc + c2) * rc + c1) * rc + c0;
      cap = Rv > D(0);
      if (fabs_(Rv) < D(0.08) * max_(rc * rc * rc * rc, D(1))) *graze0 = true;
    }
  } else {
    const D mb = D(2) * sqrt_(-pb / D(3));
    const D ac = clamp_(D(3) * qb / (pb * mb), D(-1), D(1));
    const D tb = acos_(ac) / D(3);
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) {
      const D rc = mb * cos_(tb - D(2.0943951023931953) * D(kk));
      if (rc > rplus && rc < rk) {
        const D Rv = ((rc * rc + c2) * rc + c1) * rc + c0;
        if (Rv <= D(0)) cap = false;
        if (fabs_(Rv) < D(0.08) * max_(rc * rc * rc * rc, D(1))) *graze0 = true;
      }
    }
  }
  *captured0 = cap;
}

template <int PREC, int KERR, int SEM>
__device__ void init_ray_dir(const TraceParams& p, const CamView& cam, int i1, int j1,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cf,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cr,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cu,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type offr,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type offu,
                             RayState<typename RealOf<PREC>::T>& st);

// Build the ray of pixel (i0, j0) (0-based, frame-local).  Ray generation and
// index lowering run in D (double for FP64 and FP32_GUARDED, float for FP32).
template <int PREC, int KERR, int SEM>
__device__ void init_ray(const TraceParams& p, const CamView& cam, int i0, int j0, RayState<typename RealOf<PREC>::T>& st) {
  using R = typename RealOf<PREC>::T;
  using D = typename std::conditional<PREC == ST_PREC_FP32, float, double>::type;
  const int i1 = i0 + 1, j1 = j0 + 1;
  D ju = D(p.ju), jv = D(p.jv);
  if (p.jw > 0.0) {
    ju += D(sim_hash(i1, j1, p.jseed)) * D(p.jw);
    jv += D(sim_hash(i1, j1, p.jseed + 271)) * D(p.jw);
  }
  const D half_h = D(p.height) / D(2);
  const D u = (D(i1) - D(1) + ju - D(p.width) / D(2)) / half_h;
  const D v = (D(j1) - D(1) + jv - D(p.height) / D(2)) / half_h;
  D offr = D(0), offu = D(0);
  if (p.lens_w > 0.0 && p.ap_r > 0.0) {
    const D u01 = D(p.lens_u0) + D(sim_hash(i1, j1, p.lens_seed)) * D(p.lens_w);
    const D v01 = D(p.lens_v0) + D(sim_hash(i1, j1, p.lens_seed + 7919)) * D(p.lens_w);
    const D ox = D(2) * u01 - D(1), oy = D(2) * v01 - D(1);
    if (ox != D(0) || oy != D(0)) {
      D rr, th;
      const D qpi = D(0.7853981633974483);
      if (fabs_(ox) > fabs_(oy)) { rr = ox; th = qpi * (oy / ox); }
      else { rr = oy; th = D(2) * qpi - qpi * (ox / oy); }
      offr = D(p.ap_r) * rr * cos_(th);
      offu = D(p.ap_r) * rr * sin_(th);
    }
  }
  D cf, cr, cu;
  if (p.projection == ST_PROJ_FISHEYE) {
    const D rho = sqrt_(u * u + v * v);
    const D tp = rho * D(p.fisheye_rad);
    const D s = sin_(tp);
    const D ir = rho > D(1e-8) ? D(1) / rho : D(0);
    cr = s * u * ir; cu = s * v * ir; cf = cos_(tp);
  } else {
    D dxl = u * D(p.fov), dyl = v * D(p.fov);
    D nu = sqrt_(dxl * dxl + dyl * dyl + D(1));
    if (offr != D(0) || offu != D(0)) {
      const D k = nu / D(p.focus);
      dxl -= offr * k; dyl -= offu * k;
      nu = sqrt_(dxl * dxl + dyl * dyl + D(1));
    }
    cr = dxl / nu; cu = dyl / nu; cf = D(1) / nu;
  }
  init_ray_dir<PREC, KERR, SEM>(p, cam, i1, j1, cf, cr, cu, offr, offu, st);
}

// The ray along camera-frame direction (cf, cr, cu) from the lens point
// (offr, offu) of pixel (i1, j1) (1-based, for the shutter hash): pose,
// photon lowering, launch tests and the initial state.
template <int PREC, int KERR, int SEM>
__device__ void init_ray_dir(const TraceParams& p, const CamView& cam, int i1, int j1,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cf,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cr,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type cu,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type offr,
                             typename std::conditional<PREC == ST_PREC_FP32, float, double>::type offu,
                             RayState<typename RealOf<PREC>::T>& st) {
  using R = typename RealOf<PREC>::T;
  using D = typename std::conditional<PREC == ST_PREC_FP32, float, double>::type;
  // the pose; with the per-pixel shutter on, moved toward the stratum's end
  // pose by a hashed fraction (src/metal.jl:843-857)
  D cpos[3], cEf[4], cEr[4], cEu[4], cU[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) cpos[k] = D(cam.pos[k]);
#pragma unroll
  for (int k = 0; k < 4; ++k) { cEf[k] = D(cam.Ef[k]); cEr[k] = D(cam.Er[k]); cEu[k] = D(cam.Eu[k]); cU[k] = D(cam.U[k]); }
  if (p.shutter_seed > 0) {
    const D tau = D(sim_hash(i1, j1, p.shutter_seed));
#pragma unroll
    for (int k = 0; k < 3; ++k) cpos[k] += tau * (D(p.pos_end[k]) - cpos[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      cEf[k] += tau * (D(p.Ef_end[k]) - cEf[k]);
      cEr[k] += tau * (D(p.Er_end[k]) - cEr[k]);
      cEu[k] += tau * (D(p.Eu_end[k]) - cEu[k]);
      cU[k] += tau * (D(p.U_end[k]) - cU[k]);
    }
  }
  D x[3], q[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) x[k] = cpos[k] + offr * cEr[k + 1] + offu * cEu[k + 1];
#pragma unroll
  for (int k = 0; k < 4; ++k) q[k] = cf * cEf[k] + cr * cEr[k] + cu * cEu[k] - cU[k];
  D s[6], pt;
  lower_photon<KERR>(x, q, D(p.M), D(p.a), s, &pt);

  st.flags = 0;
  st.guard_ray = false;
  if constexpr (KERR && SEM == ST_SEM_DRAFT) {
    bool c0 = false, g0 = false;
    bardeen(s, pt, D(p.M), D(p.a), &c0, &g0);
    if (c0) st.flags |= ST_RAY_BCAPT;
    if (g0) st.flags |= ST_RAY_GRAZE;
    st.guard_ray = g0 && p.crit_band > 0.0;
  }
  if constexpr (!KERR && PREC == ST_PREC_FP32_GUARDED) {
    // critical impact-parameter band: b = |x cross p| / E, b_crit = 3 sqrt(3) M
    const D Lx = s[1] * s[5] - s[2] * s[4], Ly = s[2] * s[3] - s[0] * s[5], Lz = s[0] * s[4] - s[1] * s[3];
    const D b = sqrt_(Lx * Lx + Ly * Ly + Lz * Lz) / fabs_(pt);
    st.guard_ray = p.crit_band > 0.0 && fabs_(b - D(p.b_crit)) < D(p.crit_band);
  }
  if constexpr (PREC == ST_PREC_FP32_GUARDED) {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float h = (float)s[k];
      st.y[k] = h;
      st.lo[k] = (float)(s[k] - (D)h);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) { st.y[k] = R(s[k]); st.lo[k] = 0.f; }
  }
  st.pt = R(pt);
  const D g = D(1) / clamp_(fabs_(pt), D(0.05), D(20));
  st.scam = p.relativistic ? R(g) : R(1);
  st.acc[0] = st.acc[1] = st.acc[2] = R(0);
  st.alpha = R(1);
  st.r_prev = R(-1);
  const D r0 = sqrt_(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  st.r_floor = r0 > D(2.05) * D(p.M) ? R(2) * PR(M) : R(0.3) * PR(M);
  st.inside0 = r0 < D(2.00001);
  st.march_acc = R(0);
  st.lambda = R(0);
  st.r_esc = R(cam.r_escape);
  st.nmax = cam.nmax;
  st.h_carry = R(-1);
  st.err_prev = R(1e-4);
  st.k1_valid = false;
  st.steps = st.fp64_steps = st.gas = 0;
  st.r_cross = -1.f;
  st.g_cross = 0.f;
  st.r_layer_prev = R(-1);
  st.ell = R(0);
  if constexpr (!KERR && SEM == ST_SEM_DRAFT) {
    // Layer pass: a ray launched beyond the gate whose fan entry (by its
    // local angle to the radial axis) escapes with periapsis beyond the gate
    // never meets the disc or gas (src/metal.jl:1103-1133).  The ring pass
    // instead keeps only the rays whose periapsis is below ring_rmin.
    if (p.layer && (r0 > D(p.layer_gate) || p.ring_rmin > 0.0) && p.fan_n > 1) {
      const D cpsi = clamp_(pt * D(p.er[0]) + s[3] * D(p.er[1]) + s[4] * D(p.er[2]) + s[5] * D(p.er[3]), D(-1), D(1));
      const D N1 = D(p.fan_n - 1);
      const D tf = acos_(cpsi) * N1 / D(3.141592653589793);
      const int k0 = min(max((int)tf, 0), p.fan_n - 2);
      const D fr = tf - D(k0);
      const float4 fa = p.fan[k0], fb = p.fan[k0 + 1];
      const D esc = D(fa.x) + fr * (D(fb.x) - D(fa.x));
      const D rmin = D(fa.w) + fr * (D(fb.w) - D(fa.w));
      const bool cull = p.ring_rmin > 0.0 ? rmin >= D(p.ring_rmin) : (esc > D(0.999) && rmin > D(p.layer_gate));
      if (cull) st.flags |= ST_RAY_LAYER_CULLED;
    }
  }
}

// Land a step on the sphere |x| = target: the RK4 step of size hc from yp
// (slope k1) is a polynomial state y(hc); find hc in (0, h) with
// |y(hc)| = target by false position with the Illinois modification, the
// bracket [0, h] kept throughout (g(0) = r0 - target and g(h) = rn - target
// have opposite signs).  A step that crosses the sphere far from linearly in
// hc (a ray leaving the horizon's neighbourhood within one step) stays
// bracketed where plain secant iterations can wander off the sphere.
// Iterates until |g| < tol or the bracket stops shrinking; the first iterate
// is the linear guess h (target - r0) / (rn - r0).
template <int KERR, typename R>
__device__ __forceinline__ void land_on_sphere(const R* yp, R pt, R M, R a, R h, const R* k1, R r0, R rn, R target,
                                               R* yout) {
  const R tol = sizeof(R) == 8 ? R(1e-14) : R(1e-6) * target;
  const R eps = sizeof(R) == 8 ? R(1e-15) : R(1e-7);
  R ha = R(0), ga = r0 - target, hb = h, gb = rn - target;
  int side = 0;
  R inc[6];
#pragma unroll 1
  for (int it = 0; it < 60; ++it) {
    R hc = (ha * gb - hb * ga) / (gb - ga);
    if (!(hc > ha && hc < hb)) hc = R(0.5) * (ha + hb);
    rk4_inc<KERR>(yp, pt, M, a, hc, k1, inc);
#pragma unroll
    for (int k = 0; k < 6; ++k) yout[k] = yp[k] + inc[k];
    const R gc = sqrt_(yout[0] * yout[0] + yout[1] * yout[1] + yout[2] * yout[2]) - target;
    if (gc == R(0) || (hb - ha) < eps * h) break;
    if ((gc > R(0)) == (gb > R(0))) {
      hb = hc; gb = gc;
      if (side == -1) ga *= R(0.5);
      side = -1;
    } else {
      ha = hc; ga = gc;
      if (side == 1) gb *= R(0.5);
      side = 1;
    }
    if (fabs_(gc) < tol) break;
  }
}

// ---- shading pieces applied at interpolated points --------------------------

template <typename R>
__device__ __forceinline__ R disc_kepler(const TraceParams& p, R X0, R X1, const R* Pm, R pt, R gcam, R* acc, R* alpha) {
  const R M = PR(M);
  const R r = sqrt_(X0 * X0 + X1 * X1);
  if (!(PR(disc_inner) < r && r < PR(disc_outer))) return R(0);
  const R f = R(2) * M / r;
  const R kap = (X0 * Pm[0] + X1 * Pm[1]) / r;
  const R c1 = f * (-pt + kap) / r;
  const R pc0 = Pm[0] - c1 * X0, pc1 = Pm[1] - c1 * X1, pc2 = Pm[2];
  const R R_ = r / (R(2) * M);
  const R T_emit = exp_(R(10.034259) - R(0.375) * log_(R_ * R_));
  R vmag = R(0.70710678) / sqrt_(max_(R_ - R(1), R(0.1)));
  vmag = clamp_(vmag, R(0), R(0.999));
  const R n0 = X0 / r, n1 = X1 / r;
  const R dv0 = -vmag * n1, dv1 = vmag * n0;
  const R vsq = clamp_(dv0 * dv0 + dv1 * dv1, R(0), R(0.99));
  const R gam = R(1) / sqrt_(R(1) - vsq);
  const R pn = sqrt_(pc0 * pc0 + pc1 * pc1 + pc2 * pc2);
  const R opz_d = gam * (R(1) + (dv0 * pc0 + dv1 * pc1) / pn);
  const R opz_g = R(1) / sqrt_(max_(R(1) - R(1) / max_(R_, R(1)), R(0.01)));
  const R T_obs = T_emit * gcam / max_(opz_d * opz_g, R(0.1));
  const R inten = R(100) / (exp_(R(29622.4) / max_(T_obs, R(1))) - R(1));
  const float4 col = lut_color(p, T_obs, true);
  const R R_in = PR(disc_inner) / (R(2) * M), R_out = PR(disc_outer) / (R(2) * M);
  const R iscotaper = clamp_((R_ * R_ - R_in * R_in) * R(0.3), R(0), R(1));
  const R outertaper = clamp_(T_emit / R(1000), R(0), R(1));
  const R dens = clamp_((R_out - R_) / (R_out - R_in), R(0), R(1));
  const R fall = PR(disc_falloff);
  const R dpow = (fall == R(0)) ? R(1) : (dens <= R(0) ? R(0) : exp_(fall * log_(dens)));
  const R op = iscotaper * outertaper * dpow;
  const R w = inten * (*alpha * op);
  acc[0] += w * R(col.x); acc[1] += w * R(col.y); acc[2] += w * R(col.z);
  *alpha *= (R(1) - op);
  return T_obs / T_emit;
}

template <typename R>
__device__ __forceinline__ R disc_exact(const TraceParams& p, R xh, R yh, R pxh, R pyh, R pt, R scam, R* acc, R* alpha) {
  const R M = PR(M);
  const R sc = sqrt_(xh * xh + yh * yh);
  if (!(PR(disc_inner) < sc && sc < PR(disc_outer))) return R(0);
  const R r_isco = PR(r_isco);
  const R R_ = sc / (R(2) * M);
  const R RT = max_(sc, r_isco) / (R(2) * M);
  const R T_emit = exp_(R(10.034259) - R(0.375) * log_(RT * RT));
  const R t3 = sc / r_isco;
  const R plunge = sc < r_isco ? t3 * t3 * t3 : R(1);
  const R opz = emitter_opz(xh, yh, pxh, pyh, -pt, M, PR(a), r_isco, PR(E_isco), PR(L_isco));
  const R T_obs = T_emit * scam / opz;
  const R inten = R(100) / (exp_(R(29622.4) / max_(T_obs, R(1))) - R(1));
  const float4 col = lut_color(p, T_obs, false);
  const R R_in = PR(disc_inner) / (R(2) * M), R_out = PR(disc_outer) / (R(2) * M);
  const R iscotaper = clamp_((R_ * R_ - R_in * R_in) * R(0.3), R(0), R(1));
  const R outertaper = clamp_(T_emit / R(1000), R(0), R(1));
  const R dens = clamp_((R_out - R_) / (R_out - R_in), R(0), R(1));
  const R fall = PR(disc_falloff);
  const R dpow = dens <= R(1e-6) ? (fall > R(0) ? R(0) : R(1)) : exp_(fall * log_(dens));
  const R op = iscotaper * outertaper * dpow * plunge;
  const R w = *alpha * op * inten;
  acc[0] += w * R(col.x); acc[1] += w * R(col.y); acc[2] += w * R(col.z);
  *alpha *= (R(1) - op);
  return T_obs / T_emit;
}

// Gas march along one accepted step, src/metal.jl:1429-1513.  Returns true
// when the transmittance is exhausted.
template <typename R>
__device__ __forceinline__ bool march_gas(const TraceParams& p, const R* yp, const R* yn, R r2p, R h_used, R vlen,
                                          RayState<R>& st) {
  const R r2n = yn[0] * yn[0] + yn[1] * yn[1] + yn[2] * yn[2];
  if (!(st.alpha > R(0.003) && min_(r2p, r2n) < PR(vol_rb2))) return false;
  const R ds = PR(ds_gas);
  const R seg = h_used * vlen;
  // a step spans at most a few M of arc; anything else (overflow, NaN) is not marched
  if (!(seg < R(64))) return false;
  R t_s = ds - st.march_acc;
  if (t_s > seg) { st.march_acc += seg; return false; }
  const R zmax = PR(zmax);
  const R r_isco = PR(r_isco), M = PR(M);
  const R inv_seg = R(1) / seg;
  // bounded: seg < 64 and ds >= dt, so at most 64/dt + 1 samples (capped at 8192)
  for (int guard = 0; guard < 8192 && t_s <= seg && st.alpha > R(0.003); ++guard) {
    const R fs = IsD<R>::v ? t_s / seg : t_s * inv_seg;
    const R sx = yp[0] + fs * (yn[0] - yp[0]);
    const R sy = yp[1] + fs * (yn[1] - yp[1]);
    const R sz = yp[2] + fs * (yn[2] - yp[2]);
    if (fabs_(sz) < zmax) {
      const R scyl = sqrt_(sx * sx + sy * sy);
      if (scyl > R(1e-6)) {
        const R phi = atan2_(sy, sx);
        R rho = sample_volume(p, scyl, phi, sz);
        ++st.gas;
        if (rho > R(1e-4)) {
          R T_emit;
          if constexpr (IsD<R>::v) {
            const R Rr = max_(scyl, r_isco) / (R(2) * M);
            T_emit = exp_(R(10.034259) - R(0.375) * log_(max_(Rr * Rr, R(1e-6))));
          } else {
            // base 2: exp(c - 0.375 ln Rr^2) = 2^(c log2(e) - 0.75 log2 Rr)
            const float Rr = fmaxf(scyl, r_isco) * p.f.inv_2m;
            T_emit = ex2_(fmaf(-0.75f, lg2_(fmaxf(Rr, 1e-3f)), float(10.034259 * kLog2e)));
          }
          if (scyl < r_isco) { const R t3 = scyl / r_isco; rho *= t3 * t3 * t3; }
          const R psx = yp[3] + fs * (yn[3] - yp[3]);
          const R psy = yp[4] + fs * (yn[4] - yp[4]);
          const R opz = emitter_opz(sx, sy, psx, psy, -st.pt, M, PR(a), r_isco, PR(E_isco), PR(L_isco));
          const R T_obs = T_emit * st.scam / opz;
          const float4 col = lut_color(p, T_obs, false);
          R aa, w;
          if constexpr (IsD<R>::v) {
            const R inten = R(100) / (exp_(R(29622.4) / max_(T_obs, R(1))) - R(1));
            const R tau = PR(opac) * rho * ds;
            aa = R(1) - exp_(-tau);
            w = st.alpha * aa * inten * PR(emis);
          } else {
            // 100 emis / (exp(29622.4 / T) - 1) and 1 - exp(-opac rho ds) in base 2,
            // the products of constants from the host
            const float inte = p.f.emis100 * rcp_(ex2_(float(29622.4 * kLog2e) * rcp_(fmaxf(T_obs, 1.f))) - 1.f);
            aa = 1.f - ex2_(-(rho * p.f.opds_l2));
            w = st.alpha * aa * inte;
          }
          st.acc[0] += w * R(col.x); st.acc[1] += w * R(col.y); st.acc[2] += w * R(col.z);
          st.alpha *= (R(1) - aa);
        }
      }
    }
    t_s += ds;
  }
  st.march_acc = seg - (t_s - ds);
  return st.alpha < R(0.003);
}

// Null-constraint renormalisation in FP64: rescale the spatial momentum so
// that H = 1/2(-p_t^2 + |p|^2 - f l^2) = 0 at fixed p_t.
template <int KERR>
__device__ __forceinline__ void null_renorm(double* y, double pt, double M, double a) {
  double f, L[3];
  if constexpr (KERR) {
    const double a2 = a * a;
    const double r2 = fmax(ks_r2(y[0], y[1], y[2], a), 1e-12);
    const double r = sqrt(r2);
    const double ira = 1.0 / (r2 + a2);
    L[0] = (r * y[0] + a * y[1]) * ira;
    L[1] = (r * y[1] - a * y[0]) * ira;
    L[2] = y[2] / r;
    f = 2.0 * M * r2 * r / (r2 * r2 + a2 * y[2] * y[2]);
  } else {
    const double r = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    L[0] = y[0] / r; L[1] = y[1] / r; L[2] = y[2] / r;
    f = 2.0 * M / r;
  }
  const double kap = L[0] * y[3] + L[1] * y[4] + L[2] * y[5];
  const double pp = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
  const double A = pp - f * kap * kap;
  const double B = 2.0 * f * pt * kap;
  const double C = -(1.0 + f) * pt * pt;
  const double disc = B * B - 4.0 * A * C;
  if (!(A > 0.0) || !(disc >= 0.0)) return;
  const double lam = (-B + sqrt(disc)) / (2.0 * A);
  if (lam > 0.9 && lam < 1.1) { y[3] *= lam; y[4] *= lam; y[5] *= lam; }
}

// Tsitouras (2011) 5(4) pair, FSAL (published tableau).
struct Tsit5C {
  static constexpr double A21 = 0.161;
  static constexpr double A31 = -0.008480655492356989, A32 = 0.335480655492357;
  static constexpr double A41 = 2.897153057105493, A42 = -6.359448489975075, A43 = 4.3622954328695815;
  static constexpr double A51 = 5.325864828439257, A52 = -11.748883564062828, A53 = 7.4955393428898365,
                          A54 = -0.09249506636175525;
  static constexpr double A61 = 5.86145544294642, A62 = -12.92096931784711, A63 = 8.159367898576159,
                          A64 = -0.071584973281401, A65 = -0.028269050394068383;
  static constexpr double B1 = 0.09646076681806523, B2 = 0.01, B3 = 0.4798896504144996, B4 = 1.379008574103742,
                          B5 = -3.290069515436081, B6 = 2.324710524099774;
  static constexpr double E1 = -0.00178001105222577714, E2 = -0.0008164344596567469, E3 = 0.007880878010261995,
                          E4 = -0.1447110071732629, E5 = 0.5823571654525552, E6 = -0.45808210592918697,
                          E7 = 0.015151515151515152;
};

// The kernel's adaptive step (src/metal.jl:1278-1381): up to four attempts
// from s0 with first stage k1; mixed absolute/relative error
// max(h|e_x|, h|e_p|) / (tol (1 + max(r, |p|))), PI growth
// 0.9 err^-0.14 err_prev^0.08 in [0.2, 4], shrink 0.9 err^-0.2 >= 0.2.
// Writes the accepted (or last) state to sn, the FSAL slope to k7; returns
// the step taken.
template <int KERR, typename R>
__device__ __forceinline__ R tsit5_adaptive(const R* s0, R pt, R M, R a, R r, R hstart, R hmax, R tol, R dt,
                                           const R* k1, R* sn, R* k7, R& h_carry, R& err_prev) {
  using C = Tsit5C;
  R hh = min_(h_carry > R(0) ? h_carry : hstart, hmax);
  R h_used = hh;
  const R pn = sqrt_(s0[3] * s0[3] + s0[4] * s0[4] + s0[5] * s0[5]);
  const R sc = max_(tol * (R(1) + max_(r, pn)), R(1e-30));
#pragma unroll 1
  for (int att = 0; att < 4; ++att) {
    R k2[6], k3[6], k4[6], k5[6], k6[6], t[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = s0[i] + hh * (R(C::A21) * k1[i]);
    rhs<KERR>(t, pt, M, a, k2);
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = s0[i] + hh * (R(C::A31) * k1[i] + R(C::A32) * k2[i]);
    rhs<KERR>(t, pt, M, a, k3);
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = s0[i] + hh * (R(C::A41) * k1[i] + R(C::A42) * k2[i] + R(C::A43) * k3[i]);
    rhs<KERR>(t, pt, M, a, k4);
#pragma unroll
    for (int i = 0; i < 6; ++i)
      t[i] = s0[i] + hh * (R(C::A51) * k1[i] + R(C::A52) * k2[i] + R(C::A53) * k3[i] + R(C::A54) * k4[i]);
    rhs<KERR>(t, pt, M, a, k5);
#pragma unroll
    for (int i = 0; i < 6; ++i)
      t[i] = s0[i] + hh * (R(C::A61) * k1[i] + R(C::A62) * k2[i] + R(C::A63) * k3[i] + R(C::A64) * k4[i] +
                           R(C::A65) * k5[i]);
    rhs<KERR>(t, pt, M, a, k6);
#pragma unroll
    for (int i = 0; i < 6; ++i)
      sn[i] = s0[i] + hh * (R(C::B1) * k1[i] + R(C::B2) * k2[i] + R(C::B3) * k3[i] + R(C::B4) * k4[i] +
                            R(C::B5) * k5[i] + R(C::B6) * k6[i]);
    rhs<KERR>(sn, pt, M, a, k7);
    h_used = hh;
    R e[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
      e[i] = R(C::E1) * k1[i] + R(C::E2) * k2[i] + R(C::E3) * k3[i] + R(C::E4) * k4[i] + R(C::E5) * k5[i] +
             R(C::E6) * k6[i] + R(C::E7) * k7[i];
    const R ex = hh * sqrt_(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    const R ep = hh * sqrt_(e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
    const R err = max_(ex, ep) / sc;
    if (err <= R(1) || hh <= R(1e-4) * dt) {
      const R g = err > R(1e-12) ? R(0.9) * exp_(R(-0.14) * log_(err) + R(0.08) * log_(err_prev)) : R(4);
      h_carry = min_(hh * clamp_(g, R(0.2), R(4)), hmax);
      err_prev = max_(err, R(1e-4));
      break;
    }
    hh = max_(hh * max_(R(0.9) * exp_(R(-0.2) * log_(err)), R(0.2)), R(1e-4) * dt);
  }
  return h_used;
}

// RHS of the guard steps: the regrouped Kerr form in double, Schwarzschild as is.
template <int KERR>
__device__ __forceinline__ void rhs_guard(const double* s, double pt, double M, double a, double* d) {
  if constexpr (KERR) rhs_kerr_rg64(s, pt, M, a, d); else rhs_schw(s, pt, M, d);
}

// FP64 guard step on the float-float state (classical RK4 in double).
template <int KERR>
__device__ __forceinline__ void guard_step_fp64(float* y, float* lo, float pt, double M, double a, float h) {
  double yd[6], k1d[6], inc[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) yd[k] = (double)y[k] + (double)lo[k];
  const double ptd = (double)pt;
  rhs_guard<KERR>(yd, ptd, M, a, k1d);
  {
    double t[6], k[6], sum[6];
    const double hd = (double)h, hh = 0.5 * hd;
#pragma unroll
    for (int i = 0; i < 6; ++i) { t[i] = fma(hh, k1d[i], yd[i]); sum[i] = k1d[i]; }
    rhs_guard<KERR>(t, ptd, M, a, k);
#pragma unroll
    for (int i = 0; i < 6; ++i) { sum[i] = fma(2.0, k[i], sum[i]); t[i] = fma(hh, k[i], yd[i]); }
    rhs_guard<KERR>(t, ptd, M, a, k);
#pragma unroll
    for (int i = 0; i < 6; ++i) { sum[i] = fma(2.0, k[i], sum[i]); t[i] = fma(hd, k[i], yd[i]); }
    rhs_guard<KERR>(t, ptd, M, a, k);
    const double h6 = hd * (1.0 / 6.0);
#pragma unroll
    for (int i = 0; i < 6; ++i) inc[i] = h6 * (sum[i] + k[i]);
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double v = yd[k] + inc[k];
    const float hi = (float)v;
    y[k] = hi;
    lo[k] = (float)(v - (double)hi);
  }
}

// ---------------------------------------------------------------------------
// Double-float arithmetic on the FP32 pipe (ST_PREC_FP32_GUARDED_DF): a value
// is hi + lo, two floats with |lo| <= ulp(hi) / 2, about 48 significant bits.
// Sums by Knuth's TwoSum and Dekker's FastTwoSum, products by the exact FMA
// residual, reciprocal and (reciprocal) square roots by one Newton-Raphson
// step from the float value (which doubles its ~23 correct bits).  Every
// operation is a rounded intrinsic, so neither contraction nor fast-math
// flags of the translation unit change the error-free transformations.
// ---------------------------------------------------------------------------
struct df2 {
  float hi, lo;
};
__device__ __forceinline__ df2 dfq(float a) { return df2{a, 0.f}; }
__device__ __forceinline__ df2 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return df2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// |a| >= |b| (or a = 0)
__device__ __forceinline__ df2 df_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// x + y with one TwoSum on the high parts and the low parts added in float
// (Dekker's add): the error is about 2^-47 of max(|x|, |y|) -- an absolute
// bound at the operands' scale, which is what a guard step's state needs --
// for half the instructions of the form that also bounds it relative to the
// sum under cancellation
__device__ __forceinline__ df2 df_add(df2 x, df2 y) {
  const df2 s = df_two_sum(x.hi, y.hi);
  return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ df2 df_neg(df2 x) { return df2{-x.hi, -x.lo}; }
__device__ __forceinline__ df2 df_sub(df2 x, df2 y) { return df_add(x, df_neg(y)); }
__device__ __forceinline__ df2 df_mul(df2 x, df2 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast(p, e);
}
__device__ __forceinline__ df2 df_mulf(df2 x, float f) {
  const float p = __fmul_rn(x.hi, f);
  return df_fast(p, __fmaf_rn(x.lo, f, __fmaf_rn(x.hi, f, -p)));
}
// x y + z
__device__ __forceinline__ df2 df_fma(df2 x, df2 y, df2 z) { return df_add(df_mul(x, y), z); }
// 1 / x: r0 + r0 (1 - x r0)
__device__ __forceinline__ df2 df_rcp(df2 x) {
  const float r0 = __frcp_rn(x.hi);
  const df2 e = df_sub(dfq(1.f), df_mulf(x, r0));
  return df_fast(r0, __fmul_rn(r0, e.hi));
}
// sqrt(x), x > 0: s0 + (x - s0^2) / (2 s0)
__device__ __forceinline__ df2 df_sqrt(df2 x) {
  if (!(x.hi > 0.f)) return dfq(0.f);
  const float s0 = __fsqrt_rn(x.hi);
  const float p = __fmul_rn(s0, s0);
  const df2 d = df_sub(x, df2{p, __fmaf_rn(s0, s0, -p)});
  return df_fast(s0, __fmul_rn(d.hi, __frcp_rn(__fmul_rn(2.f, s0))));
}
// 1 / sqrt(x), x > 0: r0 + r0 (1 - x r0^2) / 2
__device__ __forceinline__ df2 df_rsqrt(df2 x) {
  const float r0 = __frsqrt_rn(x.hi);
  const float p = __fmul_rn(r0, r0);
  const df2 e = df_sub(dfq(1.f), df_mul(x, df2{p, __fmaf_rn(r0, r0, -p)}));
  return df_fast(r0, __fmul_rn(__fmul_rn(0.5f, r0), e.hi));
}

// The guard RHS in double-float: the regrouped Kerr form of rhs_kerr_f32 /
// rhs_kerr_rg64, and the Schwarzschild form of rhs_schw.
template <int KERR>
__device__ __forceinline__ void rhs_df(const df2* s, df2 pt, df2 M, df2 a, df2* d) {
  const df2 x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  if constexpr (KERR) {
    const df2 a2 = df_mul(a, a), z2 = df_mul(z, z);
    const df2 q = df_mul(a2, z2);
    const df2 wh = df_sub(df_mulf(df_add(df_add(df_mul(x, x), df_mul(y, y)), z2), 0.5f), df_mulf(a2, 0.5f));
    df2 r2 = df_add(wh, df_sqrt(df_add(df_mul(wh, wh), q)));
    if (!(r2.hi > 1e-12f)) r2 = dfq(1e-12f);
    const df2 ir = df_rsqrt(r2), r = df_mul(r2, ir);
    const df2 isig = df_rcp(df_add(df_mul(r2, r2), q));
    const df2 r2a = df_add(r2, a2);
    const df2 ira = df_rcp(r2a);
    const df2 A = df_add(df_mul(px, x), df_mul(py, y));
    const df2 B = df_sub(df_mul(px, y), df_mul(py, x));
    const df2 T = df_mul(df_add(df_mul(r, A), df_mul(a, B)), ira);
    const df2 Z = df_mul(df_mul(z, pz), ir);
    const df2 ell = df_sub(df_add(T, Z), pt);
    const df2 rsig = df_mul(df_mul(r2, r), isig);
    const df2 fl = df_mul(df_mul(df_mulf(M, 2.f), rsig), ell);
    const df2 Fi = df_mul(fl, ira);
    const df2 Fr = df_mul(Fi, r), Fa = df_mul(Fi, a);
    const df2 flir = df_mul(fl, ir);
    d[0] = df_sub(df_sub(px, df_mul(Fr, x)), df_mul(Fa, y));
    d[1] = df_add(df_sub(py, df_mul(Fr, y)), df_mul(Fa, x));
    d[2] = df_sub(pz, df_mul(flir, z));
    const df2 dldr = df_sub(df_mul(df_sub(A, df_mul(df_mulf(r, 2.f), T)), ira), df_mul(Z, ir));
    const df2 inner = df_add(df_mul(df_mul(ell, ir), df_sub(df_mul(df_mulf(q, 2.f), isig), dfq(0.5f))), dldr);
    const df2 G = df_mul(fl, inner);
    const df2 Gr = df_mul(G, rsig);
    d[3] = df_sub(df_add(df_mul(Gr, x), df_mul(Fr, px)), df_mul(Fa, py));
    d[4] = df_add(df_add(df_mul(Gr, y), df_mul(Fr, py)), df_mul(Fa, px));
    d[5] = df_add(df_mul(df_mul(z, isig), df_sub(df_mul(df_mul(G, r), r2a), df_mul(df_mul(a2, ell), fl))),
                  df_mul(flir, pz));
  } else {
    const df2 r2 = df_add(df_add(df_mul(x, x), df_mul(y, y)), df_mul(z, z));
    const df2 ir = df_rsqrt(r2);
    const df2 f = df_mul(df_mulf(M, 2.f), ir);
    const df2 kap = df_mul(df_add(df_add(df_mul(x, px), df_mul(y, py)), df_mul(z, pz)), ir);
    const df2 ell = df_sub(kap, pt);
    const df2 c1 = df_mul(df_mul(f, ell), ir);
    const df2 c2 = df_mul(df_mul(c1, df_add(df_mulf(ell, 0.5f), kap)), ir);
    d[0] = df_sub(px, df_mul(c1, x));
    d[1] = df_sub(py, df_mul(c1, y));
    d[2] = df_sub(pz, df_mul(c1, z));
    d[3] = df_sub(df_mul(c1, px), df_mul(c2, x));
    d[4] = df_sub(df_mul(c1, py), df_mul(c2, y));
    d[5] = df_sub(df_mul(c1, pz), df_mul(c2, z));
  }
}

// Guard step in double-float on the float-float state (classical RK4).
template <int KERR>
__device__ __forceinline__ void guard_step_df(float* y, float* lo, float pt, const TraceParams& p, float h) {
  df2 Y[6], k1[6], k[6], sum[6], t[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) Y[i] = df2{y[i], lo[i]};
  const df2 PT = dfq(pt), M = df2{p.f.M, p.f.M_lo}, A = df2{p.f.a, p.f.a_lo};
  const df2 hd = dfq(h), hh = dfq(0.5f * h);
  rhs_df<KERR>(Y, PT, M, A, k1);
#pragma unroll
  for (int i = 0; i < 6; ++i) { t[i] = df_fma(hh, k1[i], Y[i]); sum[i] = k1[i]; }
  rhs_df<KERR>(t, PT, M, A, k);
#pragma unroll
  for (int i = 0; i < 6; ++i) { sum[i] = df_add(sum[i], df_mulf(k[i], 2.f)); t[i] = df_fma(hh, k[i], Y[i]); }
  rhs_df<KERR>(t, PT, M, A, k);
#pragma unroll
  for (int i = 0; i < 6; ++i) { sum[i] = df_add(sum[i], df_mulf(k[i], 2.f)); t[i] = df_fma(hd, k[i], Y[i]); }
  rhs_df<KERR>(t, PT, M, A, k);
  const df2 h6 = df_mul(hd, df_rcp(dfq(6.f)));
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const df2 v = df_add(Y[i], df_mul(h6, df_add(sum[i], k[i])));
    y[i] = v.hi;
    lo[i] = v.lo;
  }
}

// The null renormalisation (null_renorm) in double-float, for the guarded
// path's double-float mode.
template <int KERR>
__device__ __forceinline__ void renorm_df(float* y, float* lo, float pt, const TraceParams& p) {
  df2 Y[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) Y[i] = df2{y[i], lo[i]};
  const df2 M = df2{p.f.M, p.f.M_lo}, PT = dfq(pt);
  df2 f, L[3];
  if constexpr (KERR) {
    const df2 a = df2{p.f.a, p.f.a_lo};
    const df2 a2 = df_mul(a, a), z2 = df_mul(Y[2], Y[2]), q = df_mul(a2, z2);
    const df2 wh = df_sub(df_mulf(df_add(df_add(df_mul(Y[0], Y[0]), df_mul(Y[1], Y[1])), z2), 0.5f), df_mulf(a2, 0.5f));
    df2 r2 = df_add(wh, df_sqrt(df_add(df_mul(wh, wh), q)));
    if (!(r2.hi > 1e-12f)) r2 = dfq(1e-12f);
    const df2 ir = df_rsqrt(r2), r = df_mul(r2, ir);
    const df2 ira = df_rcp(df_add(r2, a2));
    L[0] = df_mul(df_add(df_mul(r, Y[0]), df_mul(a, Y[1])), ira);
    L[1] = df_mul(df_sub(df_mul(r, Y[1]), df_mul(a, Y[0])), ira);
    L[2] = df_mul(Y[2], ir);
    f = df_mul(df_mul(df_mulf(M, 2.f), df_mul(r2, r)), df_rcp(df_add(df_mul(r2, r2), q)));
  } else {
    const df2 ir = df_rsqrt(df_add(df_add(df_mul(Y[0], Y[0]), df_mul(Y[1], Y[1])), df_mul(Y[2], Y[2])));
    L[0] = df_mul(Y[0], ir); L[1] = df_mul(Y[1], ir); L[2] = df_mul(Y[2], ir);
    f = df_mul(df_mulf(M, 2.f), ir);
  }
  const df2 kap = df_add(df_add(df_mul(L[0], Y[3]), df_mul(L[1], Y[4])), df_mul(L[2], Y[5]));
  const df2 pp = df_add(df_add(df_mul(Y[3], Y[3]), df_mul(Y[4], Y[4])), df_mul(Y[5], Y[5]));
  const df2 A = df_sub(pp, df_mul(f, df_mul(kap, kap)));
  const df2 B = df_mulf(df_mul(df_mul(f, PT), kap), 2.f);
  const df2 C = df_neg(df_mul(df_add(dfq(1.f), f), df_mul(PT, PT)));
  const df2 disc = df_sub(df_mul(B, B), df_mulf(df_mul(A, C), 4.f));
  if (!(A.hi > 0.f) || !(disc.hi >= 0.f)) return;
  const df2 lam = df_mul(df_sub(df_sqrt(disc), B), df_rcp(df_mulf(A, 2.f)));
  if (!(lam.hi > 0.9f && lam.hi < 1.1f)) return;
#pragma unroll
  for (int i = 3; i < 6; ++i) {
    const df2 v = df_mul(Y[i], lam);
    y[i] = v.hi;
    lo[i] = v.lo;
  }
}

template <int KERR>
__device__ __forceinline__ void renorm_fp64(float* y, float* lo, float pt, double M, double a) {
  double yd[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) yd[k] = (double)y[k] + (double)lo[k];
  null_renorm<KERR>(yd, (double)pt, M, a);
#pragma unroll
  for (int k = 3; k < 6; ++k) {
    const float hi = (float)yd[k];
    y[k] = hi;
    lo[k] = (float)(yd[k] - (double)hi);
  }
}

// One integration step for the variant; returns true when the ray is done.
// Mirrors the step loop of src/metal.jl:1201-1572 (DRAFT) and the callback
// structure of src/raytrace.jl:339-373 (RENDER).  DEFER (FP32_GUARDED): a
// step that would run in FP64 is not taken; the ray returns flagged
// ST_RAY_DEFER with its state as it entered the call (the only field the
// call has written, r_prev, is rewritten to the same value when the step is
// taken again), so the resume kernel can take it in a dense FP64 warp.
template <int PREC, int KERR, int VOL, int SEM, int ORD = 4, int DEPTH = 0, int DEFER = 0>
__device__ __forceinline__ bool step_ray(const TraceParams& p, RayState<typename RealOf<PREC>::T>& st) {
  using R = typename RealOf<PREC>::T;
  const R M = PR(M), a = PR(a);
  R* y = st.y;
  const R r2 = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
  const R r = sqrt_(r2);
  R rk2 = r2;
  if constexpr (!KERR && SEM == ST_SEM_DRAFT) {
    if (p.layer) {
      // culled by the fan, or outbound beyond the gate: a null geodesic has
      // at most one radial turning point, so it cannot come back, and the
      // sky is the composite's job (src/metal.jl:1204-1212)
      if (st.flags & ST_RAY_LAYER_CULLED) return true;
      if (r > PR(layer_gate) && st.r_layer_prev > R(0) && r > st.r_layer_prev) {
        st.flags |= ST_RAY_ESCAPED;
        return true;
      }
      st.r_layer_prev = r;
    }
  }
  if (st.steps >= st.nmax) { st.flags |= ST_RAY_BUDGET; return true; }
  if constexpr (SEM == ST_SEM_DRAFT) {
    if constexpr (KERR) {
      rk2 = ks_r2(y[0], y[1], y[2], a);
      if (rk2 < PR(rkill2)) { st.flags |= ST_RAY_CAPTURED; return true; }
    } else {
      if (r < R(3.2) * M) {
        if (r < st.r_floor || (r < R(2.95) * M && st.r_prev > R(0) && r < st.r_prev - R(1e-4) * M)) {
          st.flags |= ST_RAY_CAPTURED;
          return true;
        }
        st.r_prev = r;
      }
    }
    if (r > st.r_esc) { st.flags |= ST_RAY_ESCAPED; return true; }
  } else {
    if (r >= st.r_esc) { st.flags |= ST_RAY_ESCAPED; return true; }
    if (st.lambda >= PR(tspan)) { st.flags |= ST_RAY_BUDGET; return true; }
    // A ray moving inward below 2.95M never escapes (escaping rays have
    // periapsis > 3M).  In ingoing KS coordinates the backward ray reaches the
    // past horizon only asymptotically, which a fixed step cannot follow, so
    // it ends here as horizon-bound (the reference's adaptive integrator
    // follows it down to its r = 2.00001 callback; the colour is the same).
    if (r < R(2.95) * M && st.r_prev > R(0) && r < st.r_prev - R(1e-4) * M) {
      st.flags |= ST_RAY_CAPTURED;
      return true;
    }
    st.r_prev = r;
  }
  // radius-adaptive step, src/metal.jl:1250-1260
  const R cap = (VOL && r2 < PR(vol_rb2)) ? R(2) : PR(hcap);
  R h;
  if constexpr (IsD<R>::v) {
    h = PR(dt) * min_(max_(PR(hcoef) * r / M, R(1)), cap);
    if constexpr (KERR) {
      const R rk = PR(rkill2);
      const R fr = clamp_((rk2 - rk) / max_(rk, R(1e-6)), R(0), R(1));
      h *= R(0.12) + R(0.88) * fr;
    }
  } else {
    const float hb = fminf(fmaxf(p.f.hcoef_m * r, 1.f), cap);
    if constexpr (KERR) {
      // dt (0.12 + 0.88 clamp((rk2 - rkill2) / rkill2, 0, 1)): one saturated
      // multiply-add, dt folded into the host's 0.12 dt and 0.88 dt
      const float fr = __saturatef(fmaf(rk2, p.f.inv_rkill2, -p.f.rkill_n));
      h = hb * fmaf(p.f.dt_span, fr, p.f.dt_lo);
    } else {
      h = PR(dt) * hb;
    }
  }
  if constexpr (SEM == ST_SEM_RENDER) h = min_(h, PR(tspan) - st.lambda);

  R yp[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) yp[k] = y[k];
  R k1[6];
  if constexpr (ORD == 45 || ORD == 46) {
    if (st.k1_valid) {
#pragma unroll
      for (int k = 0; k < 6; ++k) k1[k] = st.k1c[k];
    } else {
      rhs<KERR>(y, st.pt, M, a, k1);
    }
  } else if constexpr (KERR && SEM == ST_SEM_DRAFT && std::is_same<R, float>::value) {
    rhs_kerr_f32(y, st.pt, M, a, k1, rk2);  // the kill test's r^2 of this state
  } else {
    rhs<KERR>(y, st.pt, M, a, k1);
  }

  bool fp64_step = false;
  if constexpr (PREC == ST_PREC_FP32_GUARDED) {
    fp64_step = (st.guard_ray && (PR(crit_r2) <= R(0) || rk2 < PR(crit_r2))) ||
                (!(st.flags & ST_RAY_BCAPT) && rk2 < PR(r_guard2));
    if constexpr (DEFER) {
      if (fp64_step) {
        st.flags |= ST_RAY_DEFER;
        return true;
      }
    }
  }
  if constexpr (ORD == 45 || ORD == 46) {
    // adaptive Tsit5 (src/metal.jl:1278-1381); 45 caps the step at the
    // radius-adaptive h, 46 runs free up to 50 dt with the thin-disc approach guard
    R hmax = h;
    if constexpr (ORD == 46) {
      hmax = R(50) * PR(dt);
      if (!VOL && p.disc_on) hmax = min_(hmax, max_(h, R(0.5) * (r - PR(disc_outer))));
    }
    R sn[6], k7[6];
    h = tsit5_adaptive<KERR>(yp, st.pt, M, a, r, h, hmax, PR(tol), PR(dt), k1, sn, k7, st.h_carry, st.err_prev);
#pragma unroll
    for (int k = 0; k < 6; ++k) { y[k] = sn[k]; st.k1c[k] = k7[k]; }
    st.k1_valid = true;
  } else if (fp64_step) {
    if constexpr (PREC == ST_PREC_FP32_GUARDED) {
      // the guard step: FP64, or double-float on the FP32 pipe (counted alike)
      if (p.guard_df) guard_step_df<KERR>(y, st.lo, st.pt, p, h);
      else guard_step_fp64<KERR>(y, st.lo, st.pt, p.M, p.a, h);
      ++st.fp64_steps;
    }
  } else {
    R inc[6];
    rk4_inc<KERR>(y, st.pt, M, a, h, k1, inc);
    if constexpr (PREC == ST_PREC_FP32_GUARDED) {
#pragma unroll
      for (int k = 0; k < 6; ++k) ff_add(y[k], st.lo[k], inc[k]);
    } else if constexpr (std::is_same<R, float>::value) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float2 o = add2(pk(y[2 * k], y[2 * k + 1]), pk(inc[2 * k], inc[2 * k + 1]));
        y[2 * k] = o.x; y[2 * k + 1] = o.y;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) y[k] = y[k] + inc[k];
    }
  }
  ++st.steps;
  if constexpr (PREC == ST_PREC_FP32_GUARDED) {
    if (p.renorm_every > 0 && (st.steps % p.renorm_every) == 0) {
      if (p.guard_df) renorm_df<KERR>(y, st.lo, st.pt, p);
      else renorm_fp64<KERR>(y, st.lo, st.pt, p.M, p.a);
    }
  }
  if (!(y[0] == y[0]) || !(y[2] == y[2]) || !(y[3] == y[3])) { st.flags |= ST_RAY_CAPTURED; return true; }

  if constexpr (SEM == ST_SEM_DRAFT) {
    const R vlen = max_(sqrt_(k1[0] * k1[0] + k1[1] * k1[1] + k1[2] * k1[2]), R(1e-20));
    if constexpr (DEPTH) st.ell += h * vlen;
    if constexpr (VOL) {
      const bool opaque = march_gas(p, yp, y, r2, h, vlen, st);
      if constexpr (DEPTH) flush_bucket(p, st.pix, st.ell, st.acc);
      if (opaque) return true;
    } else {
      if (p.disc_on && st.alpha > R(0.001) && yp[2] * y[2] < R(0)) {
        const R cfz = yp[2] / (yp[2] - y[2]);
        const R xh = yp[0] + cfz * (y[0] - yp[0]);
        const R yh = yp[1] + cfz * (y[1] - yp[1]);
        const R pxh = yp[3] + cfz * (y[3] - yp[3]);
        const R pyh = yp[4] + cfz * (y[4] - yp[4]);
        R g;
        if (p.emitter == ST_EMIT_KEPLER) {
          const R pzh = yp[5] + cfz * (y[5] - yp[5]);
          const R Pm[3] = {pxh, pyh, pzh};
          g = disc_kepler(p, xh, yh, Pm, st.pt, st.scam, st.acc, &st.alpha);
        } else {
          g = disc_exact(p, xh, yh, pxh, pyh, st.pt, st.scam, st.acc, &st.alpha);
        }
        if (g > R(0) && st.r_cross < 0.f) {
          st.r_cross = (float)sqrt_(xh * xh + yh * yh);
          st.g_cross = (float)g;
          st.flags |= ST_RAY_CROSSED;
        }
        if constexpr (DEPTH) flush_bucket(p, st.pix, st.ell, st.acc);
      }
    }
    if (p.exit_landing) {
      const R rn2 = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
      if (rn2 > st.r_esc * st.r_esc) {  // beyond the escape sphere (squared: no root per step)
        const R rn = sqrt_(rn2);
        R yt[6];
        land_on_sphere<KERR>(yp, st.pt, M, a, h, k1, r, rn, st.r_esc, yt);
#pragma unroll
        for (int k = 0; k < 6; ++k) { y[k] = yt[k]; st.lo[k] = 0.f; }
        st.flags |= ST_RAY_ESCAPED;
        return true;
      }
    }
  } else {
    // RENDER: z = 0 disc events (shading only), then the terminating boundary
    if (p.disc_on && yp[2] * y[2] < R(0)) {
      const R cfz = yp[2] / (yp[2] - y[2]);
      const R xh = yp[0] + cfz * (y[0] - yp[0]);
      const R yh = yp[1] + cfz * (y[1] - yp[1]);
      const R Pm[3] = {yp[3] + cfz * (y[3] - yp[3]), yp[4] + cfz * (y[4] - yp[4]), yp[5] + cfz * (y[5] - yp[5])};
      R g;
      if (p.emitter == ST_EMIT_KEPLER) g = disc_kepler(p, xh, yh, Pm, st.pt, st.scam, st.acc, &st.alpha);
      else g = disc_exact(p, xh, yh, Pm[0], Pm[1], st.pt, st.scam, st.acc, &st.alpha);
      if (g > R(0) && st.r_cross < 0.f) {
        st.r_cross = (float)sqrt_(xh * xh + yh * yh);
        st.g_cross = (float)g;
        st.flags |= ST_RAY_CROSSED;
      }
    }
    st.lambda += h;
    const R rn = sqrt_(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    R rb = R(-1);
    if (st.inside0) { if (rn >= R(2.00001)) rb = R(2.00001); }
    else if (rn <= R(2.00001)) rb = R(2.00001);
    else if (rn >= st.r_esc) rb = st.r_esc;
    if (rb > R(0)) {
      R yt[6];
      land_on_sphere<KERR>(yp, st.pt, M, a, h, k1, r, rn, rb, yt);
#pragma unroll
      for (int k = 0; k < 6; ++k) { y[k] = yt[k]; st.lo[k] = 0.f; }
      st.flags |= (rb == st.r_esc) ? ST_RAY_ESCAPED : ST_RAY_CAPTURED;
      return true;
    }
  }
  return false;
}

// Procedural stars along unit direction d (starfield_mtl, src/metal.jl:652-724;
// the CPU renderer's starfield_color, src/starfield.jl:83-150): the ray's own
// lattice cell and its eight neighbours, each holding at most one star placed
// by the hash; Gaussian PSF of width sigma, cut at 5 sigma; occupancy thinned
// away from the galactic plane; flux xi^(-2/3); colour from the stars' table,
// indexed as the disc's (DRAFT rounds half up, RENDER to nearest even).
template <int SEM, typename R>
__device__ __forceinline__ void star_light(const TraceParams& p, R dx, R dy, R dz, R* rgb) {
  const R N = R(p.star_N);
  const int Ni = (int)p.star_N;
  const R two_pi = R(6.283185307179586);
  const R u = atan2_(dy, dx) / two_pi + R(0.5);
  const R v = (dz + R(1)) * R(0.5);
  const int i0 = (int)floor_(u * N), j0 = (int)floor_(v * N);
  const R sig = R(p.star_sigma);
  const R inv2s2 = R(1) / (R(2) * sig * sig);
  const R cut = R(25) * sig * sig;
  const R fill = R(p.star_fill), conc = R(p.star_conc), flux0 = R(p.star_flux);
  const R gx = R(p.star_g[0]), gy = R(p.star_g[1]), gz = R(p.star_g[2]);
  const R tmin = R(p.star_tmin), tspan = R(p.star_tspan);
  const R lt0 = R(p.star_lut_tmin), lt1 = R(p.star_lut_tmax);
  const int n = p.star_lut_size;
  const int seed = p.star_seed;
  R ar = R(0), ag = R(0), ab = R(0);
#pragma unroll 1
  for (int dj = -1; dj <= 1; ++dj) {
    const int jj = j0 + dj;
    if (jj < 0 || jj >= Ni) continue;
#pragma unroll 1
    for (int di = -1; di <= 1; ++di) {
      int ii = (i0 + di) % Ni;
      if (ii < 0) ii += Ni;
      const R su = R(sim_hash(ii, jj, seed + 1)), sv = R(sim_hash(ii, jj, seed + 2));
      const R phs = ((R(ii) + su) / N - R(0.5)) * two_pi;
      const R sz = R(2) * (R(jj) + sv) / N - R(1);
      const R sr = sqrt_(max_(R(1) - sz * sz, R(0)));
      const R sx = sr * cos_(phs), sy = sr * sin_(phs);
      const R ex = dx - sx, ey = dy - sy, ez = dz - sz;
      const R d2 = ex * ex + ey * ey + ez * ez;
      if (d2 > cut) continue;
      R occ = fill;
      if (conc > R(0)) occ *= exp_(-fabs_(sx * gx + sy * gy + sz * gz) * conc);
      if (!(R(sim_hash(ii, jj, seed)) < occ)) continue;
      const R xi = max_(R(sim_hash(ii, jj, seed + 3)), R(1e-4f));
      const R w = flux0 * exp_(R(-0.6666667f) * log_(xi)) * exp_(-d2 * inv2s2);
      const R T = tmin + tspan * R(sim_hash(ii, jj, seed + 4));
      const R frac = (clamp_(T, lt0, lt1) - lt0) / max_(lt1 - lt0, R(1e-6));
      int li;
      if constexpr (SEM == ST_SEM_DRAFT) li = (int)(frac * R(n - 1) + R(0.5));
      else li = (int)rint(frac * R(n - 1));
      li = min(max(li, 0), n - 1);
      const float4 c = p.star_lut[li];
      ar += w * R(c.x); ag += w * R(c.y); ab += w * R(c.z);
    }
  }
  rgb[0] = ar; rgb[1] = ag; rgb[2] = ab;
}

// Classification, sky and output (src/metal.jl:1629-1704, src/raytrace.jl:267-298).
template <int PREC, int KERR, int SEM, int DEPTH = 0>
__device__ __forceinline__ void finish_ray(const TraceParams& p, RayState<typename RealOf<PREC>::T>& st, int out_index,
                                           int diag_index) {
  using R = typename RealOf<PREC>::T;
  if constexpr (!KERR && SEM == ST_SEM_DRAFT) {
    if (p.layer) {
      // layer output: premultiplied emission and transmittance, by
      // assignment; capture blackness is the composite's (src/metal.jl:1616-1626)
      p.out[out_index] = make_float4((float)st.acc[0], (float)st.acc[1], (float)st.acc[2], (float)st.alpha);
      return;
    }
  }
  const R M = PR(M), a = PR(a);
  R yv[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) yv[k] = st.y[k];
  const R rf = max_(sqrt_(yv[0] * yv[0] + yv[1] * yv[1] + yv[2] * yv[2]), R(1e-6));
  R vel[6];
  rhs<KERR>(yv, st.pt, M, a, vel);
  const R vl = max_(sqrt_(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]), R(1e-20));
  const R d0 = vel[0] / vl, d1 = vel[1] / vl, d2 = vel[2] / vl;
  bool black;
  if constexpr (SEM == ST_SEM_DRAFT) black = (st.flags & (ST_RAY_CAPTURED | ST_RAY_BCAPT)) || rf < R(4) * M;
  else black = (st.flags & ST_RAY_CAPTURED) || rf < R(2.1) * M;
  R rgb[3] = {st.acc[0], st.acc[1], st.acc[2]};
  if (!black) {
    const R th = acos_(clamp_(d2, R(-1), R(1)));
    const R ph = atan2_(d1, d0);
    R sky[3];
    sample_sky(p, th, ph, sky);
    if (p.star_strength > 0.0) {
      // the image under the stars, then the stars (src/metal.jl:1668-1677;
      // src/starfield.jl:157-164), both before the relativistic tint
      R sl[3];
      star_light<SEM>(p, d0, d1, d2, sl);
      const R tw = R(p.star_tw), ss = R(p.star_strength);
      sky[0] = sky[0] * tw + ss * sl[0];
      sky[1] = sky[1] * tw + ss * sl[1];
      sky[2] = sky[2] * tw + ss * sl[2];
    }
    const R g = st.scam;
    if (g != R(1)) {
      sky[0] *= R(57.4) / (exp_(R(4.067) / g) - R(1));
      sky[1] *= R(90.2) / (exp_(R(4.513) / g) - R(1));
      sky[2] *= R(206.5) / (exp_(R(5.335) / g) - R(1));
    }
    rgb[0] += st.alpha * sky[0];
    rgb[1] += st.alpha * sky[1];
    rgb[2] += st.alpha * sky[2];
    if constexpr (DEPTH) {  // the background lives in the last (infinity) bucket
      float* b = p.buckets + (size_t)out_index * 3 * p.nb + 3 * (p.nb - 1);
      b[0] += p.weight * (float)(st.alpha * sky[0]);
      b[1] += p.weight * (float)(st.alpha * sky[1]);
      b[2] += p.weight * (float)(st.alpha * sky[2]);
    }
  } else {
    st.flags |= ST_RAY_BLACK;
  }
  const float w = p.weight;
  if (p.stat) {
    // per-ray luminance moments and the graze fraction for adaptive
    // refinement (src/metal.jl:1640-1700); weights sum to 1 over the base passes
    const float L = 0.2126f * (float)rgb[0] + 0.7152f * (float)rgb[1] + 0.0722f * (float)rgb[2];
    float4 s4 = p.stat[out_index];
    s4.x += w * L;
    s4.y += w * L * L;
    if (st.flags & ST_RAY_GRAZE) s4.z += w;
    p.stat[out_index] = s4;
  }
  if constexpr (!DEPTH) {  // bucketed emission was written during the march
    float4 o = make_float4(w * (float)rgb[0], w * (float)rgb[1], w * (float)rgb[2], (float)st.alpha);
    if (!p.first_pass) {
      const float4 prev = p.out[out_index];
      o.x += prev.x; o.y += prev.y; o.z += prev.z;
    }
    p.out[out_index] = o;
  }
  if (p.diag) {
    st_ray_diag d;
    d.dir[0] = (double)d0; d.dir[1] = (double)d1; d.dir[2] = (double)d2;
    d.flags = (st.flags & ~ST_RAY_INTERNAL) | (st.guard_ray ? ST_RAY_GUARDED : 0);
    d.r_final = (float)rf;
    d.alpha = (float)st.alpha;
    d.r_cross = st.r_cross;
    d.g_cross = st.g_cross;
    d.steps = st.steps;
    d.fp64_steps = st.fp64_steps;
    d.lambda = (float)st.lambda;
    d.pad[0] = d.pad[1] = 0;
    p.diag[diag_index] = d;
  }
}

}  // namespace st
