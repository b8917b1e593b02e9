// st_api.cu -- host side of libspacetime_gb300.so: the C ABI declared in
// include/spacetime_gb300.h.  FP64 host work (camera tetrad, blackbody LUT,
// reference step/escape rules) plus device-memory management and launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "st_internal.h"

namespace st {
cudaError_t launch_trace_fp64(const Variant&, const TraceParams&, int, int, int, cudaStream_t);
cudaError_t launch_trace_fp32(const Variant&, const TraceParams&, int, int, int, cudaStream_t);
cudaError_t launch_trace_fp32_guarded(const Variant&, const TraceParams&, int, int, int, cudaStream_t);
int variant_registers_fp64(const Variant&);
int variant_registers_fp32(const Variant&);
int variant_registers_fp32_guarded(const Variant&);

cudaError_t launch_trace(const Variant& v, const TraceParams& p, int bx, int by, int num_sms, cudaStream_t s) {
  switch (v.prec) {
    case ST_PREC_FP64: return launch_trace_fp64(v, p, bx, by, num_sms, s);
    case ST_PREC_FP32: return launch_trace_fp32(v, p, bx, by, num_sms, s);
    default: return launch_trace_fp32_guarded(v, p, bx, by, num_sms, s);
  }
}

int variant_registers(const Variant& v) {
  switch (v.prec) {
    case ST_PREC_FP64: return variant_registers_fp64(v);
    case ST_PREC_FP32: return variant_registers_fp32(v);
    default: return variant_registers_fp32_guarded(v);
  }
}

__global__ void pack_rgb_kernel(const float4* __restrict__ fb, float* __restrict__ rgb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float4 c = fb[i];
    rgb[3 * i + 0] = c.x;
    rgb[3 * i + 1] = c.y;
    rgb[3 * i + 2] = c.z;
  }
}

cudaError_t launch_pack_rgb(const float4* fb, float* rgb, int n, cudaStream_t s) {
  pack_rgb_kernel<<<(n + 255) / 256, 256, 0, s>>>(fb, rgb, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 host physics (the reference computes these on the CPU in Float64).
// ---------------------------------------------------------------------------

struct V4 { double c[4]; };

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// ks_camera_tetrad (src/preview.jl:93-198): static / 2.5M free-faller
// observer (a = 0) or static->ZAMO blend (a != 0), Gram-Schmidt under the KS
// metric with forward first, then the Lorentz boost by beta.
static void host_tetrad(const double* pos, const double* fwd, const double* right, const double* up, double M,
                        double a, const double* beta, double* U, double* Ef, double* Er, double* Eu) {
  double l[3], f, u[4];
  if (a == 0.0) {
    const double r = std::sqrt(dot3(pos, pos));
    for (int k = 0; k < 3; ++k) l[k] = pos[k] / r;
    f = 2.0 * M / r;
    const double E = std::sqrt(std::max(1.0 - 2.0 / 2.5, 1.0 - f));
    const double v = -std::sqrt(std::max(E * E - (1.0 - f), 0.0));
    const double w = (1.0 - E * (E - v)) / (E - v);
    const double lu = E + w;
    u[0] = E + f * lu;
    for (int k = 0; k < 3; ++k) u[k + 1] = (w - f * lu) * l[k];
  } else {
    const double x = pos[0], y = pos[1], z = pos[2], a2 = a * a;
    const double wq = x * x + y * y + z * z - a2;
    const double rk2 = 0.5 * (wq + std::sqrt(wq * wq + 4.0 * a2 * z * z));
    const double rk = std::sqrt(std::max(rk2, 1e-12));
    const double ira = 1.0 / (rk2 + a2);
    l[0] = (rk * x + a * y) * ira;
    l[1] = (rk * y - a * x) * ira;
    l[2] = z / rk;
    const double sig = rk2 * rk2 + a2 * z * z;
    f = 2.0 * M * rk2 * rk / sig;
    const double delta = std::max(rk2 - 2.0 * M * rk + a2, 1e-6);
    const double kA = 2.0 * M * rk / delta;
    const double gr[3] = {x * rk2 * rk / sig, y * rk2 * rk / sig, z * rk * (rk2 + a2) / sig};
    const double luc = 1.0 + kA * dot3(l, gr);
    double uz[4] = {1.0 + f * luc, 0, 0, 0};
    for (int c = 0; c < 3; ++c) uz[c + 1] = kA * gr[c] - (f * luc) * l[c];
    const double luz = uz[0] + l[0] * uz[1] + l[1] * uz[2] + l[2] * uz[3];
    const double n2 = -uz[0] * uz[0] + uz[1] * uz[1] + uz[2] * uz[2] + uz[3] * uz[3] + f * luz * luz;
    double zamo[4];
    for (int c = 0; c < 4; ++c) zamo[c] = uz[c] / std::sqrt(-n2);
    if (f >= 0.88) {
      std::memcpy(u, zamo, sizeof u);
    } else {
      double wb = std::min(std::max((f - 0.72) / 0.16, 0.0), 1.0);
      wb = wb * wb * (3.0 - 2.0 * wb);
      const double us[4] = {1.0 / std::sqrt(1.0 - f), 0, 0, 0};
      if (wb == 0.0) {
        std::memcpy(u, us, sizeof u);
      } else {
        double um[4];
        for (int c = 0; c < 4; ++c) um[c] = (1.0 - wb) * us[c] + wb * zamo[c];
        const double lu = um[0] + l[0] * um[1] + l[1] * um[2] + l[2] * um[3];
        const double nn = -um[0] * um[0] + um[1] * um[1] + um[2] * um[2] + um[3] * um[3] + f * lu * lu;
        for (int c = 0; c < 4; ++c) u[c] = um[c] / std::sqrt(-nn);
      }
    }
  }
  auto ld = [&](const double* A) { return A[0] + l[0] * A[1] + l[1] * A[2] + l[2] * A[3]; };
  auto g = [&](const double* A, const double* B) {
    return -A[0] * B[0] + A[1] * B[1] + A[2] * B[2] + A[3] * B[3] + f * ld(A) * ld(B);
  };
  double ef[4] = {0, fwd[0], fwd[1], fwd[2]}, er[4] = {0, right[0], right[1], right[2]},
         eu[4] = {0, up[0], up[1], up[2]};
  auto axpy = [](double* y, double s, const double* x) { for (int k = 0; k < 4; ++k) y[k] += s * x[k]; };
  auto scale = [](double* y, double s) { for (int k = 0; k < 4; ++k) y[k] /= s; };
  axpy(ef, g(ef, u), u);
  scale(ef, std::sqrt(g(ef, ef)));
  axpy(er, g(er, u), u);
  axpy(er, -g(er, ef), ef);
  scale(er, std::sqrt(g(er, er)));
  axpy(eu, g(eu, u), u);
  {
    const double c1 = g(eu, ef), c2 = g(eu, er);
    for (int k = 0; k < 4; ++k) eu[k] -= c1 * ef[k] + c2 * er[k];
  }
  scale(eu, std::sqrt(g(eu, eu)));
  const double b2raw = dot3(beta, beta);
  if (b2raw > 1e-12) {
    const double b2 = std::min(b2raw, 0.9801);
    const double s = std::sqrt(b2 / b2raw);
    const double b[3] = {beta[0] * s, beta[1] * s, beta[2] * s};
    const double gam = 1.0 / std::sqrt(1.0 - b2);
    double bE[4];
    for (int k = 0; k < 4; ++k) bE[k] = b[0] * ef[k] + b[1] * er[k] + b[2] * eu[k];
    const double kk = (gam - 1.0) / b2;
    for (int k = 0; k < 4; ++k) {
      const double common = kk * bE[k] + gam * u[k];
      U[k] = gam * (u[k] + bE[k]);
      Ef[k] = ef[k] + b[0] * common;
      Er[k] = er[k] + b[1] * common;
      Eu[k] = eu[k] + b[2] * common;
    }
    return;
  }
  std::memcpy(U, u, sizeof u);
  std::memcpy(Ef, ef, sizeof ef);
  std::memcpy(Er, er, sizeof er);
  std::memcpy(Eu, eu, sizeof eu);
}

// CIE piecewise-Gaussian blackbody colour, src/blackbody.jl:5-35.
static double cie_g(double lam, double mu, double s1, double s2) {
  const double s = lam < mu ? s1 : s2;
  const double t = (lam - mu) / s;
  return std::exp(-0.5 * t * t);
}
void host_blackbody(double T, double* rgb) {
  double X = 0, Y = 0, Z = 0;
  for (int i = 0; i <= 80; ++i) {
    const double lam = 380.0 + 5.0 * i, lm = lam * 1e-9;
    const double B = 1.0 / (std::pow(lm, 5) * (std::exp(0.014388 / (lm * T)) - 1.0));
    X += B * (1.056 * cie_g(lam, 599.8, 37.9, 31.0) + 0.362 * cie_g(lam, 442.0, 16.0, 26.7) -
              0.065 * cie_g(lam, 501.1, 20.4, 26.2));
    Y += B * (0.821 * cie_g(lam, 568.8, 46.9, 40.5) + 0.286 * cie_g(lam, 530.9, 16.3, 31.1));
    Z += B * (1.217 * cie_g(lam, 437.0, 11.8, 36.0) + 0.681 * cie_g(lam, 459.0, 26.0, 13.8));
  }
  const double r = std::max(3.2406 * X - 1.5372 * Y - 0.4986 * Z, 0.0);
  const double gg = std::max(-0.9689 * X + 1.8758 * Y + 0.0415 * Z, 0.0);
  const double b = std::max(0.0557 * X - 0.2040 * Y + 1.0570 * Z, 0.0);
  const double m = std::max(std::max(r, gg), std::max(b, 1e-10));
  rgb[0] = r / m; rgb[1] = gg / m; rgb[2] = b / m;
}

// ISCO (BPT 1972), as the kernel's isco_mtl (src/metal.jl:371-380) in double.
static void host_isco(double M, double a, double* r_isco, double* E, double* L) {
  auto cb = [](double x) { return std::exp(std::log(std::max(x, 1e-12)) / 3.0); };
  const double q = a / M;
  const double z1 = 1.0 + cb(1.0 - q * q) * (cb(1.0 + q) + cb(1.0 - q));
  const double z2 = std::sqrt(3.0 * q * q + z1 * z1);
  const double r = M * (3.0 + z2 - std::sqrt(std::max((3.0 - z1) * (3.0 + z1 + 2.0 * z2), 0.0)));
  *r_isco = r;
  *E = std::sqrt(1.0 - 2.0 * M / (3.0 * r));
  *L = (2.0 * M / (3.0 * std::sqrt(3.0))) * (1.0 + 2.0 * std::sqrt(3.0 * r / M - 2.0));
}

// Prograde photon orbit, src/gr.jl:58-60.
static double host_photon_orbit_min(double M, double a) {
  if (a == 0.0) return 3.0 * M;
  return 2.0 * M * (1.0 + std::cos((2.0 / 3.0) * std::acos(-a / M)));
}

// The static observer's orthonormal frame at pos with radial / polar /
// azimuthal axes (Gram-Schmidt under the KS metric), lowered to covectors, and
// the camera's KS radius, polar angle and azimuth: the surrogate's frame.
static void host_static_frame(const double* pos, double M, double a, SurFrame* f) {
  const double rr = std::sqrt(dot3(pos, pos));
  const double ct = pos[2] / rr, stt = std::sqrt(std::max(1.0 - ct * ct, 0.0));
  const double ph = std::atan2(pos[1], pos[0]), cp = std::cos(ph), sp = std::sin(ph);
  const double e[3][3] = {{pos[0] / rr, pos[1] / rr, ct}, {ct * cp, ct * sp, -stt}, {-sp, cp, 0.0}};
  double l[3], fk, rk;
  if (a != 0.0) {
    const double w = dot3(pos, pos) - a * a;
    const double rk2 = 0.5 * (w + std::sqrt(w * w + 4.0 * a * a * pos[2] * pos[2]));
    rk = std::sqrt(std::max(rk2, 1e-12));
    const double ira = 1.0 / (rk2 + a * a);
    l[0] = (rk * pos[0] + a * pos[1]) * ira;
    l[1] = (rk * pos[1] - a * pos[0]) * ira;
    l[2] = pos[2] / rk;
    fk = 2.0 * M * rk2 * rk / (rk2 * rk2 + a * a * pos[2] * pos[2]);
  } else {
    rk = rr;
    for (int k = 0; k < 3; ++k) l[k] = pos[k] / rr;
    fk = 2.0 * M / rr;
  }
  auto g = [&](const double* A, const double* B) {
    const double la = A[0] + l[0] * A[1] + l[1] * A[2] + l[2] * A[3];
    const double lb = B[0] + l[0] * B[1] + l[1] * B[2] + l[2] * B[3];
    return -A[0] * B[0] + A[1] * B[1] + A[2] * B[2] + A[3] * B[3] + fk * la * lb;
  };
  double U[4] = {1.0 / std::sqrt(1.0 - fk), 0, 0, 0}, E[3][4];
  for (int m = 0; m < 3; ++m) {
    double v[4] = {0.0, e[m][0], e[m][1], e[m][2]};
    double c = g(v, U);
    for (int k = 0; k < 4; ++k) v[k] += c * U[k];
    for (int q = 0; q < m; ++q) {
      c = g(v, E[q]);
      for (int k = 0; k < 4; ++k) v[k] -= c * E[q][k];
    }
    c = std::sqrt(g(v, v));
    for (int k = 0; k < 4; ++k) E[m][k] = v[k] / c;
  }
  auto lower = [&](const double* V, double* out) {
    const double lv = V[0] + l[0] * V[1] + l[1] * V[2] + l[2] * V[3];
    out[0] = -V[0] + fk * lv;
    for (int k = 0; k < 3; ++k) out[k + 1] = V[k + 1] + fk * lv * l[k];
  };
  lower(U, f->Ul);
  lower(E[0], f->E1l);
  lower(E[1], f->E2l);
  lower(E[2], f->E3l);
  f->r = rk;
  f->th = std::acos(std::min(std::max(pos[2] / rk, -1.0), 1.0));
  for (int k = 0; k < 3; ++k) f->xh[k] = pos[k] / rr;
}

// splitmix64 for the host-side pass shuffles
struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  int below(int n) { return (int)(next() % (uint64_t)n); }
};
static void shuffle(std::vector<int>& v, Rng& r) {
  for (int i = (int)v.size() - 1; i > 0; --i) std::swap(v[i], v[r.below(i + 1)]);
}

}  // namespace st

// ---------------------------------------------------------------------------
// Context.
// ---------------------------------------------------------------------------

struct st_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  float4* d_sky = nullptr;
  int sky_w = 0, sky_h = 0;
  float4* d_lut = nullptr;
  int lut_size = 0;
  double lut_tmin = 500.0, lut_tmax = 30000.0;
  st_disc disc{};
  bool disc_on = false;
  float* d_vol = nullptr;
  size_t vol_bytes = 0;
  st_volume vol{};
  bool vol_on = false;
  float4* d_fb = nullptr;
  size_t fb_cap = 0;
  float* d_rgb = nullptr;
  size_t rgb_cap = 0;
  st_ray_diag* d_diag = nullptr;
  size_t diag_cap = 0;
  st::FrameCam* d_frames = nullptr;
  size_t frames_cap = 0;
  unsigned long long* d_counters = nullptr;
  unsigned int* d_queue = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // camera-track path: pinned staging and the captured graph
  st::FrameCam* h_frames = nullptr;
  size_t h_frames_cap = 0;
  unsigned long long* h_cnt = nullptr;
  cudaGraphExec_t gexec = nullptr;
  st::TraceParams gkey{};
  st::Variant gvar{};
  size_t gbytes = 0;
  // procedural stars: host parameters and the stars' own colour table
  st_starfield star{};
  bool star_on = false;
  float4* d_star_lut = nullptr;
  int star_lut_size = 0;
  double star_lut_tmin = 500.0, star_lut_tmax = 30000.0;
  // layered engine: deflection fans, their critical band, the disc / gas layer
  float4* d_fan = nullptr;
  float4* d_fine = nullptr;
  float* d_band = nullptr;
  float4* d_layer = nullptr;
  size_t layer_cap = 0;
  float4* d_ring = nullptr;  // the ring pass's layer
  size_t ring_cap = 0;
  // the fans depend only on the camera radius and the integration rules:
  // the parameters of the last build, and whether the buffers hold them
  st::lay::FanParams fan_key;
  int fan_prec = -1;
  bool fan_valid = false;
  cudaStream_t side = nullptr;  // the fine fan runs here, beside the layer pass
  cudaEvent_t ev_coarse = nullptr, ev_fine = nullptr;
  // adaptive refinement: per-pixel luminance moments, the flagged box
  float4* d_stat = nullptr;
  size_t stat_cap = 0;
  float* d_buckets = nullptr;  // depth buckets, 3 nb floats per pixel
  size_t buckets_cap = 0;
  unsigned* d_box = nullptr;
  st_surrogate* sur = nullptr;  // attached surrogate (not owned)
  int* d_list = nullptr;        // surrogate fallback pixels
  size_t list_cap = 0;
  int* d_count = nullptr;
  // FP32_GUARDED deferral: saved ray states and their count
  unsigned char* d_defer = nullptr;
  size_t defer_cap = 0;  // bytes
  unsigned* d_defer_count = nullptr;
  // centre-first tile order of full-frame pixel launches, cached per grid and
  // centre tile
  int* d_order = nullptr;
  size_t order_cap = 0;
  int order_key[4] = {-1, -1, -1, -1};
  std::vector<int> h_order;
  size_t h2d_extra = 0;  // bytes uploaded by the current call beyond its parameters
};

namespace {

using st::TraceParams;

#define ST_CUDA(call)                         \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return ST_ECUDA;   \
  } while (0)

template <class T>
int ensure(T** ptr, size_t* cap, size_t n) {
  if (*cap >= n && *ptr) return ST_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  if (cudaMalloc((void**)ptr, n * sizeof(T)) != cudaSuccess) return ST_ENOMEM;
  *cap = n;
  return ST_OK;
}

double norm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// FP32_GUARDED on the pixel schedule (RK4, no depth buckets), with the
// environment variable SPACETIME_GB300_GUARD_DEFER=1: space for every ray of
// one launch to be saved before its first FP64 guard step, so the guard steps
// run in full warps of a resume kernel.  Off by default: on the 1080p config-1
// frame the split measured slower than the guard steps inline (103.2 vs
// 94.5 ms), because the resumed rays' FP64 work no longer overlaps the
// other warps' FP32 work and their FP64 segments end at different steps.
int setup_defer(st_context* ctx, TraceParams* p, const st::Variant& v, size_t nrays) {
  p->defer_state = nullptr;
  p->defer_count = nullptr;
  p->defer_cap = 0;
  if (v.prec != ST_PREC_FP32_GUARDED || v.sched != ST_SCHED_PIXEL || p->order != 4 || p->nb > 0) return ST_OK;
  const char* e = std::getenv("SPACETIME_GB300_GUARD_DEFER");
  if (!e || std::strcmp(e, "1") != 0) return ST_OK;
  if (nrays > (size_t)INT_MAX) return ST_EINVAL;
  int rc = ensure(&ctx->d_defer, &ctx->defer_cap, nrays * st::guarded_ray_state_bytes());
  if (rc != ST_OK) return rc;
  if (!ctx->d_defer_count && cudaMalloc(&ctx->d_defer_count, sizeof(unsigned)) != cudaSuccess) return ST_ENOMEM;
  p->defer_state = ctx->d_defer;
  p->defer_count = ctx->d_defer_count;
  p->defer_cap = (int)nrays;
  return ST_OK;
}

// Rays a persistent warp takes from the queue at a time: one 8x4 tile (the
// measured best of 32, 128 and 512 on the 1080p config-1 frame: 39.3, 41.3,
// 56.5 ms; larger windows leave long rays in a few warps' windows at the end);
// SPACETIME_GB300_REFILL_WINDOW=<n> (a multiple of 32) for A/B.
int refill_window() {
  const char* e = std::getenv("SPACETIME_GB300_REFILL_WINDOW");
  const int n = e ? std::atoi(e) : 0;
  return n >= 32 ? n & ~31 : 32;
}

// Fill the frame-independent part of TraceParams and the camera of `cam`.
int fill_params(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
                TraceParams* p, st::Variant* v) {
  if (!ctx || !cam || !stp || !rp) return ST_EINVAL;
  const double M = stp->M, a = stp->a;
  if (!(M > 0.0) || !(std::fabs(a) <= M)) return ST_EINVAL;
  if (rp->width <= 0 || rp->height <= 0 || rp->samples <= 0 || !(rp->dt > 0.0)) return ST_EINVAL;
  if ((long long)rp->width * rp->height > (1ll << 30)) return ST_EINVAL;
  if (rp->precision < ST_PREC_FP64 || rp->precision > ST_PREC_FP32_GUARDED_DF) return ST_EINVAL;
  if (rp->semantics != ST_SEM_RENDER && rp->semantics != ST_SEM_DRAFT) return ST_EINVAL;
  const double rpos = norm3(cam->pos);
  if (!(rpos > 0.0) || !std::isfinite(rpos)) return ST_EINVAL;
  if (rp->semantics == ST_SEM_RENDER) {
    // the reference's CPU renderer has Schwarzschild methods only
    if (a != 0.0) return ST_EUNSUPPORTED;
    if (ctx->vol_on) return ST_EUNSUPPORTED;
  }
  const int order = rp->order == 0 ? 4 : rp->order;
  if (order != 4 && order != 45 && order != 46) return ST_EINVAL;
  if (order != 4 && (rp->semantics != ST_SEM_DRAFT || rp->precision == ST_PREC_FP32_GUARDED ||
                     rp->precision == ST_PREC_FP32_GUARDED_DF ||
                     rp->schedule == ST_SCHED_PERSISTENT))
    return ST_EUNSUPPORTED;
  if (rp->surrogate) {
    if (!ctx->sur) return ST_ESTATE;
    if (rp->semantics != ST_SEM_DRAFT || rp->samples != 1 || ctx->vol_on) return ST_EUNSUPPORTED;
  }
  std::memset(p, 0, sizeof(*p));
  const double beta[3] = {st::dot3(cam->velocity, cam->fwd), st::dot3(cam->velocity, cam->right),
                          st::dot3(cam->velocity, cam->up)};
  st::host_tetrad(cam->pos, cam->fwd, cam->right, cam->up, M, a, beta, p->U, p->Ef, p->Er, p->Eu);
  for (int k = 0; k < 3; ++k) p->pos[k] = cam->pos[k];
  p->fov = cam->fov_factor;
  p->projection = cam->projection;
  p->fisheye_rad = std::max(cam->fisheye_deg, 0.0) * 3.141592653589793 / 180.0;
  p->focus = cam->focus_dist > 0.0 ? cam->focus_dist : 1.0;
  p->width = rp->width;
  p->height = rp->height;
  p->frame_stride = rp->width * rp->height;
  p->M = M;
  p->a = a;
  const double rph = st::host_photon_orbit_min(M, a);
  {
    // the kernel holds the kill radius in Float32 (src/metal.jl:355-356)
    const float rk = (float)(0.995 * rph);
    p->rkill2 = (double)(rk * rk);
  }
  st::host_isco(M, a, &p->r_isco, &p->E_isco, &p->L_isco);
  p->dt = rp->dt;
  p->hcoef = 0.16;
  p->hcap = 8.0;
  p->order = order;
  p->tol = rp->tol > 0.0 ? rp->tol : 1e-4;
  p->relativistic = rp->relativistic ? 1 : 0;
  if (rp->semantics == ST_SEM_DRAFT) {
    // src/metal.jl:2058-2062: r_escape = 2 max(|pos|, 15M) (Float32);
    // nmax = min(max(1000, ceil((75 + 6.5 ln(r_esc/M)) M/dt)), 40000)
    const double re = rp->r_escape > 0.0 ? rp->r_escape : (double)(float)(2.0 * std::max(rpos, 15.0 * M));
    p->r_escape = re;
    if (rp->nmax > 0) {
      p->nmax = rp->nmax;
    } else {
      const double Mf = (double)(float)M, dtf = (double)(float)rp->dt;
      const double lg = (double)std::log((float)((float)re / (float)M));
      const double n = std::ceil((75.0 + 6.5 * lg) * Mf / dtf);
      p->nmax = (int)std::min(std::max(1000.0, n), 40000.0);
    }
    p->tspan = 0.0;
    p->exit_landing = rp->exit_landing ? 1 : 0;
  } else {
    // src/raytrace.jl:352-354, 373: r_max = max(5|pos|, 100); tspan = max(10|pos|, 500);
    // the step budget stands in for maxiters = 50_000
    p->r_escape = rp->r_escape > 0.0 ? rp->r_escape : std::max(5.0 * rpos, 100.0);
    p->tspan = rp->tspan > 0.0 ? rp->tspan : std::max(10.0 * rpos, 500.0);
    p->nmax = rp->nmax > 0 ? rp->nmax : 50000;
    p->exit_landing = 1;
  }
  // FP32_GUARDED policy
  const double rg = rp->r_guard > 0.0 ? rp->r_guard : 0.0;
  p->r_guard2 = rg * rg;
  p->crit_band = rp->crit_band;
  p->crit_r2 = rp->crit_r > 0.0 ? rp->crit_r * rp->crit_r : 0.0;
  p->b_crit = 3.0 * std::sqrt(3.0) * M;
  p->renorm_every = rp->renorm_every;
  // disc
  p->disc_on = (ctx->disc_on && ctx->disc.inner > 0.0 && ctx->disc.outer > ctx->disc.inner) ? 1 : 0;
  p->emitter = ctx->disc.emitter;
  p->disc_inner = ctx->disc.inner;
  p->disc_outer = ctx->disc.outer;
  p->disc_falloff = ctx->disc.falloff;
  p->lut = ctx->d_lut;
  p->lut_size = ctx->lut_size;
  p->lut_tmin = ctx->lut_tmin;
  p->lut_tmax = ctx->lut_tmax;
  if (!ctx->d_lut || ctx->lut_size < 1) return ST_ESTATE;
  // volume (DRAFT only), src/metal.jl:1147-1159
  p->vol_on = (rp->semantics == ST_SEM_DRAFT && ctx->vol_on) ? 1 : 0;
  if (p->vol_on) {
    const st_volume& vv = ctx->vol;
    p->vol = ctx->d_vol;
    p->nr = vv.nr; p->nphi = vv.nphi; p->nz = vv.nz;
    p->ls_in = vv.log_s_in; p->ls_out = vv.log_s_out; p->zmax = vv.z_max;
    p->emis = vv.emission_scale; p->opac = vv.opacity_scale;
    const int stride = std::min(std::max(vv.march_stride, 1), 16);
    p->ds_gas = stride * rp->dt;
    const double so = std::exp((double)vv.log_s_out);
    p->vol_rb2 = so * so + (double)vv.z_max * vv.z_max;
  } else {
    p->vol_rb2 = -1.0;
  }
  p->sky = ctx->d_sky;
  p->sky_w = ctx->sky_w;
  p->sky_h = ctx->sky_h;
  if (ctx->star_on) {
    // set_starfield! packing (src/metal.jl:268-290): sigma from the PSF in
    // pixels and the vertical field, unit galactic normal, temperature span
    const st_starfield& sf = ctx->star;
    const double gn = std::sqrt(sf.galactic[0] * sf.galactic[0] + sf.galactic[1] * sf.galactic[1] +
                                sf.galactic[2] * sf.galactic[2]);
    p->star_strength = sf.strength;
    p->star_tw = sf.texture_weight;
    p->star_N = sf.density;
    p->star_fill = sf.fill;
    p->star_sigma = sf.psf_pixels * 2.0 * sf.fov_factor / sf.height;
    p->star_flux = sf.flux;
    for (int k = 0; k < 3; ++k) p->star_g[k] = sf.galactic[k] / gn;
    p->star_conc = sf.concentration;
    p->star_tmin = sf.temp_min;
    p->star_tspan = sf.temp_max - sf.temp_min;
    p->star_lut = ctx->d_star_lut;
    p->star_lut_size = ctx->star_lut_size;
    p->star_lut_tmin = ctx->star_lut_tmin;
    p->star_lut_tmax = ctx->star_lut_tmax;
    p->star_seed = sf.seed;
  } else {
    p->star_strength = 0.0;
  }
  p->counters = ctx->d_counters;
  p->queue = ctx->d_queue;
  p->chunk_steps = rp->chunk_steps > 0 ? rp->chunk_steps : 32;
  p->refill_window = refill_window();
  // double-float guards run in the FP32_GUARDED kernels
  v->prec = rp->precision == ST_PREC_FP32_GUARDED_DF ? ST_PREC_FP32_GUARDED : rp->precision;
  p->guard_df = rp->precision == ST_PREC_FP32_GUARDED_DF ? 1 : 0;
  v->kerr = (a != 0.0) ? 1 : 0;
  v->vol = p->vol_on;
  v->sem = rp->semantics;
  v->sched = rp->schedule == ST_SCHED_PERSISTENT ? ST_SCHED_PERSISTENT : ST_SCHED_PIXEL;
  st::fill_float_copies(p);
  return ST_OK;
}

struct PassPlan {
  double ju, jv, jw;
  int jseed;
  double lens_u0, lens_v0, lens_w;
  int lens_seed;
  int time_m;        // shutter stratum of this pass (motion blur)
  int shutter_seed;  // per-pixel shutter hash seed of this pass
};

// Motion blur of one render (st_render_motion): the caller's camera_at
// evaluated at the fractions the passes use.
struct Motion {
  const st_camera* poses;
  int nposes;
  int per_pixel;
};

// Depth-bucket output of render_depth_mtl (src/metal.jl:1935-1990).
struct Depth {
  int nb;
  float* host;  // (3 nb, width, height)
};

// The samples^2 passes of render_draft_mtl (src/metal.jl:2091-2168) or of
// render's stratified offsets (src/raytrace.jl:375-419).  Host draws use
// splitmix64 seeded by p->seed.
std::vector<PassPlan> plan_passes(const st_render_params* rp, const st_camera* cam, int block = 0) {
  const int S = rp->samples;
  const int n = S * S;
  // block b > 0: a refinement block, with fresh strata and pass numbers
  // continuing after the base passes (src/metal.jl:2116-2120, 2218-2227)
  st::Rng rng{(rp->seed ^ 0x5eed5eedull) + 0x9e3779b97f4a7c15ull * (unsigned long long)block};
  std::vector<int> order(n), lens(n), tperm(n);
  for (int k = 0; k < n; ++k) { order[k] = k; lens[k] = k; tperm[k] = k; }
  if (rp->pixel_jitter) st::shuffle(order, rng);
  st::shuffle(lens, rng);
  st::shuffle(tperm, rng);  // time strata pair randomly with the others (src/metal.jl:2124-2130)
  const bool dof = cam->aperture_world > 0.0 && cam->projection == ST_PROJ_PINHOLE;
  std::vector<PassPlan> out(n);
  for (int k = 0; k < n; ++k) {
    const int m = order[k];
    const int a = m / S, b = m % S;
    PassPlan pp{};
    const double shift = rp->semantics == ST_SEM_RENDER ? 0.5 : 0.0;  // CPU pixel-centre convention
    if (rp->pixel_jitter) {
      pp.ju = (double)a / S + shift;
      pp.jv = (double)b / S + shift;
      pp.jw = 1.0 / S;
    } else {
      pp.ju = (a + 0.5) / S + shift;
      pp.jv = (b + 0.5) / S + shift;
      pp.jw = 0.0;
    }
    const int pass = block * n + k + 1;
    pp.jseed = 15485863 + pass;
    if (dof) {
      const int lm = lens[k];
      pp.lens_u0 = (double)(lm / S) / S;
      pp.lens_v0 = (double)(lm % S) / S;
      pp.lens_w = 1.0 / S;
      pp.lens_seed = pass;
    }
    pp.time_m = tperm[k];
    pp.shutter_seed = 104729 + pass;  // clear of the lens seeds (src/metal.jl:2148-2150)
    out[k] = pp;
  }
  return out;
}

// The tetrad of a motion pose: the pose's position, axes, field and velocity
// with the render's own projection and lens settings (_ks_cam_params of
// camera_at(s) with the call's fisheye_deg / focus_dist, src/metal.jl:2141-2158).
int pose_params(st_context* ctx, const st_camera* cam, const st_camera* pose, const st_spacetime* stp,
                const st_render_params* rp, TraceParams* out) {
  st_camera pc = *cam;
  for (int k = 0; k < 3; ++k) {
    pc.pos[k] = pose->pos[k]; pc.fwd[k] = pose->fwd[k]; pc.right[k] = pose->right[k];
    pc.up[k] = pose->up[k]; pc.velocity[k] = pose->velocity[k];
  }
  pc.fov_factor = pose->fov_factor;
  st::Variant w;
  return fill_params(ctx, &pc, stp, rp, out, &w);
}

// Adaptive refinement (src/metal.jl:2189-2213): a pixel is flagged when its
// per-ray luminance std-dev exceeds var (mean + 0.01) or its graze fraction
// exceeds graze; box = {min col, min row} (init all ones) and {max col + 1,
// max row + 1} (init 0) of the flagged pixels.
__global__ void refine_box_kernel(const float4* __restrict__ stat, int W, int H, float var, float graze,
                                  unsigned* box) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= W || j >= H) return;
  const float4 s4 = stat[j * W + i];
  const float s2 = s4.y - s4.x * s4.x;
  if ((s2 > 0.f && sqrtf(s2) > var * (s4.x + 0.01f)) || s4.z > graze) {
    atomicMin(box + 0, (unsigned)i);
    atomicMin(box + 1, (unsigned)j);
    atomicMax(box + 2, (unsigned)(i + 1));
    atomicMax(box + 3, (unsigned)(j + 1));
  }
}

// The refined box holds refine x the weight of the rest: renormalise.
__global__ void scale_box_kernel(float4* fb, int W, int c0, int r0, int cols, int rows, float s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= cols || j >= rows) return;
  float4& o = fb[(r0 + j) * W + (c0 + i)];
  o.x *= s; o.y *= s; o.z *= s;
}

// Iteration budget of the persistent kernel's outer loop: enough for every
// ray of the launch to take its whole step budget in chunk-sized slices.  The
// environment variable SPACETIME_GB300_QUEUE_BUDGET=<n> lowers it to n, so a
// test can make the queue run out (the kernel then reports ST_EBUDGET and
// returns; rays it had not finished are left unwritten).
long long queue_budget(long long computed) {
  const char* e = std::getenv("SPACETIME_GB300_QUEUE_BUDGET");
  if (e) {
    const long long n = std::atoll(e);
    if (n > 0 && n < computed) return n;
  }
  return computed;
}

// Centre-first dispatch order of a full-frame pixel launch.  A block's cost is
// its slowest ray, and the slowest rays sit near the hole: on the 1080p
// config-1 frame with FP64 guard steps the longest blocks run 70-84 ms, and in
// raster order they start 20-27 ms into a frame whose blocks average 1.6 ms,
// so the frame ends on them.  Tiles are sorted by Chebyshev distance, in
// tiles, from the tile the hole projects into (pinhole projection of the
// direction to the origin on the camera's axes; the frame centre when the hole
// is behind the camera or the lens is a fisheye), nearest first: a counting
// sort, O(tiles).  The order only moves when the grid or that tile changes.
int ensure_tile_order(st_context* ctx, const st_camera* cam, int width, int height, int bx, int by,
                      cudaStream_t s, const int** out) {
  const int gx = (width + bx - 1) / bx, gy = (height + by - 1) / by, n = gx * gy;
  double hi = 0.5 * width, hj = 0.5 * height;
  const double d[3] = {-cam->pos[0], -cam->pos[1], -cam->pos[2]};
  const double xf = st::dot3(d, cam->fwd), xr = st::dot3(d, cam->right), xu = st::dot3(d, cam->up);
  if (cam->projection != ST_PROJ_FISHEYE && xf > 0.0 && cam->fov_factor > 0.0) {
    hi = 0.5 * width + (xr / (xf * cam->fov_factor)) * 0.5 * height;
    hj = 0.5 * height + (xu / (xf * cam->fov_factor)) * 0.5 * height;
  }
  // clamp in double first: a hole almost square to the view axis projects far
  // off the frame, beyond what an int holds
  if (!std::isfinite(hi) || !std::isfinite(hj)) { hi = 0.5 * width; hj = 0.5 * height; }
  hi = std::min(std::max(hi, 0.0), (double)width - 1.0);
  hj = std::min(std::max(hj, 0.0), (double)height - 1.0);
  const int cx = std::min(std::max((int)std::floor(hi / bx), 0), gx - 1);
  const int cy = std::min(std::max((int)std::floor(hj / by), 0), gy - 1);
  if (ctx->order_key[0] != gx || ctx->order_key[1] != gy || ctx->order_key[2] != cx || ctx->order_key[3] != cy) {
    int rc = ensure(&ctx->d_order, &ctx->order_cap, (size_t)n);
    if (rc != ST_OK) return rc;
    const int maxd = std::max(std::max(cx, gx - 1 - cx), std::max(cy, gy - 1 - cy));
    std::vector<int> start(maxd + 2, 0);
    for (int ty = 0; ty < gy; ++ty)
      for (int tx = 0; tx < gx; ++tx) ++start[std::max(std::abs(tx - cx), std::abs(ty - cy)) + 1];
    for (int k = 1; k <= maxd + 1; ++k) start[k] += start[k - 1];
    ctx->h_order.assign(n, 0);
    for (int ty = 0; ty < gy; ++ty)
      for (int tx = 0; tx < gx; ++tx) ctx->h_order[start[std::max(std::abs(tx - cx), std::abs(ty - cy))]++] = ty * gx + tx;
    if (cudaMemcpyAsync(ctx->d_order, ctx->h_order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s) !=
        cudaSuccess)
      return ST_ECUDA;
    ctx->order_key[0] = gx; ctx->order_key[1] = gy; ctx->order_key[2] = cx; ctx->order_key[3] = cy;
    ctx->h2d_extra += (size_t)n * sizeof(int);
  }
  *out = ctx->d_order;
  return ST_OK;
}

// The learned surrogate's domain: camera KS radius in [4, 50] M, above the
// equatorial plane, 0 <= a <= 0.99 M, M = 1 (the training ranges).  Fills
// the camera's static frame.
bool surrogate_domain(const st_camera* cam, const st_spacetime* stp, st::SurFrame* sf) {
  st::host_static_frame(cam->pos, stp->M, stp->a, sf);
  return sf->r >= 4.0 * stp->M && sf->r <= 50.0 * stp->M && sf->th <= 1.5707963267948966 && stp->a >= 0.0 &&
         stp->a <= 0.99 * stp->M && stp->M == 1.0;
}

int do_render(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
              float* host_rgb, st_ray_diag* host_diag, const float** dev_rgba, st_stats* stats,
              const Motion* mo = nullptr, const Depth* depth = nullptr) {
  const auto t0 = std::chrono::steady_clock::now();
  TraceParams p;
  st::Variant v;
  int rc = fill_params(ctx, cam, stp, rp, &p, &v);
  if (rc != ST_OK) return rc;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  ctx->h2d_extra = 0;
  const size_t npix = (size_t)rp->width * rp->height;
  if ((rc = ensure(&ctx->d_fb, &ctx->fb_cap, npix)) != ST_OK) return rc;
  if (host_rgb && (rc = ensure(&ctx->d_rgb, &ctx->rgb_cap, 3 * npix)) != ST_OK) return rc;
  if (host_diag && (rc = ensure(&ctx->d_diag, &ctx->diag_cap, npix)) != ST_OK) return rc;
  p.out = ctx->d_fb;
  p.diag = host_diag ? ctx->d_diag : nullptr;
  p.ap_r = cam->aperture_world > 0.0 ? cam->aperture_world / 2.0 : 0.0;
  cudaStream_t s = ctx->stream;
  st::SurFrame sf{};
  if (rp->surrogate) {
    if (!surrogate_domain(cam, stp, &sf)) return ST_EUNSUPPORTED;
    sf.sigma_max = rp->surrogate_sigma > 0.0 ? rp->surrogate_sigma : 1e-4;
    if ((rc = ensure(&ctx->d_list, &ctx->list_cap, npix)) != ST_OK) return rc;
    if (!ctx->d_count && cudaMalloc(&ctx->d_count, sizeof(int)) != cudaSuccess) return ST_ENOMEM;
    v.sched = ST_SCHED_PIXEL;
  }
  const int refine = rp->refine > 1 ? rp->refine : 1;
  if (depth) {
    // emission binned by path length replaces the plain frame
    if (rp->semantics != ST_SEM_DRAFT || rp->surrogate || refine > 1) return ST_EUNSUPPORTED;
    if (p.order != 4) return ST_EUNSUPPORTED;  // render_depth_mtl integrates with RK4
    v.sched = ST_SCHED_PIXEL;                  // the bucket kernels are pixel-scheduled
    if ((rc = ensure(&ctx->d_buckets, &ctx->buckets_cap, 3 * (size_t)depth->nb * npix)) != ST_OK) return rc;
    ST_CUDA(cudaMemsetAsync(ctx->d_buckets, 0, 3 * (size_t)depth->nb * npix * sizeof(float), s));
    p.nb = depth->nb;
    p.buckets = ctx->d_buckets;
  }
  if (refine > 1) {
    if (rp->semantics != ST_SEM_DRAFT || rp->surrogate) return ST_EUNSUPPORTED;
    if ((rc = ensure(&ctx->d_stat, &ctx->stat_cap, npix)) != ST_OK) return rc;
    if (!ctx->d_box && cudaMalloc(&ctx->d_box, 4 * sizeof(unsigned)) != cudaSuccess) return ST_ENOMEM;
    v.sched = ST_SCHED_PIXEL;  // refinement passes dispatch a box of the pixel grid
  }
  if ((rc = setup_defer(ctx, &p, v, npix)) != ST_OK) return rc;
  ST_CUDA(cudaMemsetAsync(ctx->d_counters, 0, st::CNT_N * sizeof(unsigned long long), s));
  const std::vector<PassPlan> passes = plan_passes(rp, cam);
  p.weight = (float)(1.0 / passes.size());
  ST_CUDA(cudaEventRecord(ctx->ev0, s));
  if (refine > 1) {
    ST_CUDA(cudaMemsetAsync(ctx->d_stat, 0, npix * sizeof(float4), s));
    p.stat = ctx->d_stat;
  }
  int launches = 0;
  auto run_pass = [&](const PassPlan& pp, bool first) -> int {
    p.ju = pp.ju; p.jv = pp.jv; p.jw = pp.jw; p.jseed = pp.jseed;
    p.lens_u0 = pp.lens_u0; p.lens_v0 = pp.lens_v0; p.lens_w = pp.lens_w; p.lens_seed = pp.lens_seed;
    p.first_pass = first ? 1 : 0;
    if (mo) {
      // this pass's pose: the stratum midpoint, or its start with the end
      // pose for the per-pixel shutter
      TraceParams q;
      if ((rc = pose_params(ctx, cam, &mo->poses[pp.time_m], stp, rp, &q)) != ST_OK) return rc;
      std::memcpy(p.pos, q.pos, sizeof p.pos);
      std::memcpy(p.Ef, q.Ef, sizeof p.Ef);
      std::memcpy(p.Er, q.Er, sizeof p.Er);
      std::memcpy(p.Eu, q.Eu, sizeof p.Eu);
      std::memcpy(p.U, q.U, sizeof p.U);
      p.fov = q.fov;
      p.shutter_seed = 0;
      if (mo->per_pixel) {
        if ((rc = pose_params(ctx, cam, &mo->poses[pp.time_m + 1], stp, rp, &q)) != ST_OK) return rc;
        std::memcpy(p.pos_end, q.pos, sizeof p.pos_end);
        std::memcpy(p.Ef_end, q.Ef, sizeof p.Ef_end);
        std::memcpy(p.Er_end, q.Er, sizeof p.Er_end);
        std::memcpy(p.Eu_end, q.Eu, sizeof p.Eu_end);
        std::memcpy(p.U_end, q.U, sizeof p.U_end);
        p.shutter_seed = pp.shutter_seed;
      }
    }
    if (rp->surrogate) {
      const PassPlan& pp0 = passes[0];
      (void)pp0;
      if ((rc = st::surrogate_frame(ctx->sur, p, v, sf, ctx->d_list, ctx->d_count, s)) != ST_OK) return rc;
      p.pix_list = ctx->d_list;
      p.n_list = ctx->d_count;
    }
    if (v.sched == ST_SCHED_PERSISTENT) {
      ST_CUDA(cudaMemsetAsync(ctx->d_queue, 0, sizeof(unsigned int), s));
      const long long tiles = (long long)((rp->width + 7) / 8) * ((rp->height + 3) / 4);
      p.n_rays = (int)(tiles * 32);
      p.budget_iters = queue_budget(((long long)p.n_rays + 32) * ((long long)p.nmax / std::max(p.chunk_steps, 1) + 2));
    }
    p.tile_order = nullptr;
    if (v.sched == ST_SCHED_PIXEL && !p.pix_list && p.box_cols == 0) {
      // the launch's grid (launch_variant's rule for the tile shape)
      int bx = rp->block_x, by = rp->block_y;
      if (bx <= 0 || by <= 0 || bx * by != 128) { bx = 16; by = 8; }
      if ((rc = ensure_tile_order(ctx, cam, rp->width, rp->height, bx, by, s, &p.tile_order)) != ST_OK) return rc;
    }
    ST_CUDA(st::launch_trace(v, p, rp->block_x, rp->block_y, ctx->num_sms, s));
    ++launches;
    return ST_OK;
  };
  for (size_t k = 0; k < passes.size(); ++k)
    if ((rc = run_pass(passes[k], k == 0)) != ST_OK) return rc;
  if (refine > 1) {
    // the flagged box (+ margin), re-rendered refine - 1 more times with fresh
    // strata, then renormalised (src/metal.jl:2189-2240)
    p.stat = nullptr;
    ST_CUDA(cudaMemsetAsync(ctx->d_box, 0xFF, 2 * sizeof(unsigned), s));
    ST_CUDA(cudaMemsetAsync(ctx->d_box + 2, 0, 2 * sizeof(unsigned), s));
    const dim3 blk(16, 8), grd((rp->width + 15) / 16, (rp->height + 7) / 8);
    refine_box_kernel<<<grd, blk, 0, s>>>(ctx->d_stat, rp->width, rp->height, (float)rp->refine_var,
                                          (float)rp->refine_graze, ctx->d_box);
    ST_CUDA(cudaGetLastError());
    unsigned box[4];
    ST_CUDA(cudaMemcpyAsync(box, ctx->d_box, sizeof box, cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaStreamSynchronize(s));
    if (box[2] > 0) {
      const int m = std::max(rp->refine_margin, 0);
      const int c0 = std::max((int)box[0] - m, 0), r0 = std::max((int)box[1] - m, 0);
      const int c1 = std::min((int)box[2] + m, rp->width), r1 = std::min((int)box[3] + m, rp->height);
      p.box_col0 = c0; p.box_row0 = r0; p.box_cols = c1 - c0; p.box_rows = r1 - r0;
      for (int b = 1; b < refine; ++b) {
        const std::vector<PassPlan> more = plan_passes(rp, cam, b);
        for (const PassPlan& pp : more)
          if ((rc = run_pass(pp, false)) != ST_OK) return rc;
      }
      const dim3 gb((p.box_cols + 15) / 16, (p.box_rows + 7) / 8);
      scale_box_kernel<<<gb, blk, 0, s>>>(ctx->d_fb, rp->width, c0, r0, p.box_cols, p.box_rows,
                                          1.0f / (float)refine);
      ST_CUDA(cudaGetLastError());
      p.box_cols = 0;
    }
  }
  ST_CUDA(cudaEventRecord(ctx->ev1, s));
  unsigned long long cnt[st::CNT_N];
  ST_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, s));
  int n_fallback = 0;
  if (rp->surrogate) ST_CUDA(cudaMemcpyAsync(&n_fallback, ctx->d_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  unsigned long long d2h = 0;
  if (host_rgb) {
    ST_CUDA(st::launch_pack_rgb(ctx->d_fb, ctx->d_rgb, (int)npix, s));
    ST_CUDA(cudaMemcpyAsync(host_rgb, ctx->d_rgb, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost, s));
    d2h += 3 * npix * sizeof(float);
  }
  if (host_diag) {
    ST_CUDA(cudaMemcpyAsync(host_diag, ctx->d_diag, npix * sizeof(st_ray_diag), cudaMemcpyDeviceToHost, s));
    d2h += npix * sizeof(st_ray_diag);
  }
  if (depth) {
    const size_t nbytes = 3 * (size_t)depth->nb * npix * sizeof(float);
    ST_CUDA(cudaMemcpyAsync(depth->host, ctx->d_buckets, nbytes, cudaMemcpyDeviceToHost, s));
    d2h += nbytes;
  }
  ST_CUDA(cudaStreamSynchronize(s));
  if (dev_rgba) *dev_rgba = reinterpret_cast<const float*>(ctx->d_fb);
  const int status = cnt[st::CNT_STATUS] ? (int)cnt[st::CNT_STATUS] : ST_OK;
  if (stats) {
    float ms = 0.f;
    // a failed query must not leave an error pending for the next launch check
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) { (void)cudaGetLastError(); ms = 0.f; }
    std::memset(stats, 0, sizeof(*stats));
    stats->kernel_ms = ms;
    stats->rays = cnt[st::CNT_RAYS];
    stats->steps = cnt[st::CNT_STEPS];
    stats->fp64_steps = cnt[st::CNT_FP64];
    stats->gas_samples = cnt[st::CNT_GAS];
    stats->surrogate_rays = rp->surrogate ? (unsigned long long)(npix - (size_t)n_fallback) : 0ull;
    if (rp->surrogate) stats->rays += stats->surrogate_rays;
    stats->launches = launches;
    stats->status = status;
    stats->h2d_bytes = sizeof(TraceParams) * launches + ctx->h2d_extra;
    stats->d2h_bytes = d2h + sizeof cnt;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return status;
}

constexpr int FAN_N = 4096, FAN_FINE = 1024, FAN_PAD = 3;

// Deflection fans for the camera's radius (update_sky_fan!, src/metal.jl:2978-3036):
// the coarse fan over psi in [0, pi], its escape/capture band, the fine fan
// across the band; and the static frame's radial axis at the camera (er).
int build_fans(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
               const TraceParams& p, double er[4], cudaStream_t s) {
  const double r = std::sqrt(st::dot3(cam->pos, cam->pos));
  // the fan camera: at (r, 0, 0), forward +x, right +y, up +z, at rest
  st_camera fc{};
  fc.pos[0] = r;
  fc.fwd[0] = 1.0; fc.right[1] = 1.0; fc.up[2] = 1.0;
  fc.fov_factor = 1.0;
  fc.projection = ST_PROJ_PINHOLE;
  fc.focus_dist = 1.0;
  st::lay::FanParams fp;
  std::memset(&fp, 0, sizeof fp);
  st::Variant w;
  int rc = fill_params(ctx, &fc, stp, rp, &fp.p, &w);
  if (rc != ST_OK) return rc;
  fp.p.disc_on = 0;
  fp.p.vol_on = 0;
  fp.p.vol_rb2 = -1.0;
  fp.p.layer = 0;
  fp.p.star_strength = 0.0;
  fp.p.shutter_seed = 0;
  fp.p.r_escape = p.r_escape;
  fp.p.nmax = p.nmax;
  st::fill_float_copies(&fp.p);
  if (!ctx->d_fan && cudaMalloc(&ctx->d_fan, FAN_N * sizeof(float4)) != cudaSuccess) return ST_ENOMEM;
  if (!ctx->d_fine && cudaMalloc(&ctx->d_fine, FAN_FINE * sizeof(float4)) != cudaSuccess) return ST_ENOMEM;
  if (!ctx->d_band && cudaMalloc(&ctx->d_band, 2 * sizeof(float)) != cudaSuccess) return ST_ENOMEM;
  if (!ctx->side && cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess) return ST_ECUDA;
  if (!ctx->ev_coarse && cudaEventCreateWithFlags(&ctx->ev_coarse, cudaEventDisableTiming) != cudaSuccess)
    return ST_ECUDA;
  if (!ctx->ev_fine && cudaEventCreateWithFlags(&ctx->ev_fine, cudaEventDisableTiming) != cudaSuccess)
    return ST_ECUDA;
  fp.out = ctx->d_fan;
  fp.n = FAN_N;
  fp.band = 0;
  fp.band_lohi = ctx->d_band;
  const bool cached = ctx->fan_valid && ctx->fan_prec == rp->precision &&
                      std::memcmp(&ctx->fan_key, &fp, sizeof fp) == 0;
  if (!cached) {
    ctx->fan_valid = false;
    // coarse fan and its band on the main stream; the fine fan (which only
    // the composite reads) on the side stream, overlapping the layer pass
    ST_CUDA(cudaMemsetAsync(ctx->d_band, 0, 2 * sizeof(float), s));
    ST_CUDA(st::launch_skyfan(rp->precision, fp, s));
    ST_CUDA(st::launch_fanband(ctx->d_fan, FAN_N, FAN_PAD, ctx->d_band, s));
    ST_CUDA(cudaEventRecord(ctx->ev_coarse, s));
    ST_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_coarse, 0));
    st::lay::FanParams ff = fp;
    ff.out = ctx->d_fine;
    ff.n = FAN_FINE;
    ff.band = 1;
    ST_CUDA(st::launch_skyfan(rp->precision, ff, ctx->side));
    ST_CUDA(cudaEventRecord(ctx->ev_fine, ctx->side));
    ctx->fan_key = fp;
    ctx->fan_prec = rp->precision;
    ctx->fan_valid = true;
  }
  // the radial axis of the static frame at the camera: the forward vector of
  // a camera at rest looking straight out (any completion of the basis)
  double xh[3];
  for (int k = 0; k < 3; ++k) xh[k] = cam->pos[k] / r;
  const double ax[3] = {std::fabs(xh[2]) < 0.9 ? 0.0 : 1.0, 0.0, std::fabs(xh[2]) < 0.9 ? 1.0 : 0.0};
  double b1[3] = {ax[1] * xh[2] - ax[2] * xh[1], ax[2] * xh[0] - ax[0] * xh[2], ax[0] * xh[1] - ax[1] * xh[0]};
  const double nb = std::sqrt(st::dot3(b1, b1));
  for (int k = 0; k < 3; ++k) b1[k] /= nb;
  const double b2[3] = {xh[1] * b1[2] - xh[2] * b1[1], xh[2] * b1[0] - xh[0] * b1[2], xh[0] * b1[1] - xh[1] * b1[0]};
  const double beta[3] = {0.0, 0.0, 0.0};
  double U[4], Er[4], Eu[4];
  st::host_tetrad(cam->pos, xh, b1, b2, stp->M, 0.0, beta, U, er, Er, Eu);
  return ST_OK;
}

int layered_check(const st_camera* cam, const st_spacetime* stp, const st_render_params* rp) {
  if (!cam || !stp || !rp) return ST_EINVAL;
  if (stp->a != 0.0 || rp->semantics != ST_SEM_DRAFT || rp->surrogate ||
      (rp->precision != ST_PREC_FP64 && rp->precision != ST_PREC_FP32))
    return ST_EUNSUPPORTED;
  // the fan is indexed in the static frame: an unboosted camera at rest, r >= 2.5 M
  if (st::dot3(cam->velocity, cam->velocity) != 0.0 || std::sqrt(st::dot3(cam->pos, cam->pos)) < 2.5 * stp->M)
    return ST_EUNSUPPORTED;
  return ST_OK;
}

}  // namespace

// Blackbody(wb_temperature, table_min, table_max, table_size), src/blackbody.jl:51-60,
// uploaded as float4 entries.
static int upload_lut(st_context* ctx, double wb, double tmin, double tmax, int n) {
  if (!(tmax > tmin) || n < 2 || n > (1 << 20)) return ST_EINVAL;
  double ref[3];
  st::host_blackbody(wb > 0.0 ? wb : 6500.0, ref);
  std::vector<float4> lut(n);
  for (int i = 0; i < n; ++i) {
    const double T = tmin + (tmax - tmin) * i / (n - 1);
    double c[3];
    st::host_blackbody(std::max(T, 1.0), c);
    lut[i] = make_float4((float)(c[0] / ref[0]), (float)(c[1] / ref[1]), (float)(c[2] / ref[2]), 0.f);
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  if (ctx->d_lut && ctx->lut_size != n) { cudaFree(ctx->d_lut); ctx->d_lut = nullptr; ctx->lut_size = 0; }
  if (!ctx->d_lut && cudaMalloc(&ctx->d_lut, n * sizeof(float4)) != cudaSuccess) return ST_ENOMEM;
  if (cudaMemcpy(ctx->d_lut, lut.data(), n * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess)
    return ST_ECUDA;
  ctx->lut_size = n;
  ctx->lut_tmin = tmin;
  ctx->lut_tmax = tmax;
  return ST_OK;
}


namespace st {
int context_volume(st_context* ctx, CtxVolume* out) {
  if (!ctx || !out) return ST_EINVAL;
  out->device = ctx->device;
  out->stream = ctx->stream;
  out->d_vol = ctx->d_vol;
  out->meta = ctx->vol;
  out->on = ctx->vol_on && ctx->d_vol != nullptr;
  return ST_OK;
}

}  // namespace st

namespace {

// Foveated ring pass options (render_layered_gpu!, src/metal.jl:3040-3118).
struct Ring {
  int width, height;  // ring layer size (<= 0: the display)
  double rmin;        // periapsis bound in M; <= 0 = no ring pass
  int box;            // dispatch only the screen box that can hold wound rays
};
struct RingBox {
  int c0, cols, r0, rows;
};

// Screen box of the rays the ring pass keeps (_ring_screen_box,
// src/metal.jl:2522-2666).  In Schwarzschild a ray's periapsis is below R > 3M
// exactly when its impact parameter b = |x x p| / |p_t| is below
// b(R) = R / sqrt(1 - 2M/R) (captured rays included), and b is conserved, so
// a probe grid of camera rays built as the kernel builds them (tetrad,
// projection, index lowering; pixel centres) decides it without
// integration.  The box of the probes under 1.06 b(R), padded by two probe
// spacings + 3 pixels, contains the wound set; a set smaller than the probe
// spacing is seeded at the nearest-approach probe.  Leaves *box as the whole
// layer when no bound applies or the box covers more than 55 % of it.
void ring_screen_box(const TraceParams& p, const st_render_params* rp, double ring_rmin, int rw, int rh,
                     RingBox* box) {
  *box = RingBox{0, rw, 0, rh};
  const double M = p.M;
  if (!(ring_rmin > 2.0 * M)) return;
  const double bR = ring_rmin / std::sqrt(1.0 - 2.0 * M / ring_rmin) * 1.06;
  const double x = p.pos[0], y = p.pos[1], z = p.pos[2];
  const double r = std::sqrt(x * x + y * y + z * z);
  if (!(r > 2.0 * M)) return;
  const double f = 2.0 * M / r;
  const bool fish = p.projection == ST_PROJ_FISHEYE;
  const int probes = 81, margin = 3;
  const int nv = std::max(9, probes);
  const int nu = std::max(9, (int)std::nearbyint((double)probes * rw / rh));
  const double half_h = rh / 2.0;
  int imin = INT_MAX, imax = INT_MIN, jmin = INT_MAX, jmax = INT_MIN;
  double bbest = INFINITY;
  int ibest = 1, jbest = 1;
  for (int pj = 1; pj <= nv; ++pj)
    for (int pi = 1; pi <= nu; ++pi) {
      const double ipx = 1.0 + (pi - 1) * (double)(rw - 1) / (nu - 1);
      const double jpx = 1.0 + (pj - 1) * (double)(rh - 1) / (nv - 1);
      const double u = (ipx - 1.0 + 0.5 - rw / 2.0) / half_h;
      const double v = (jpx - 1.0 + 0.5 - rh / 2.0) / half_h;
      double cr, cu, cf;
      if (fish) {
        const double rho = std::sqrt(u * u + v * v);
        const double th = rho * p.fisheye_rad;
        const double sth = std::sin(th);
        const double inv = rho > 1e-8 ? 1.0 / rho : 0.0;
        cr = sth * u * inv; cu = sth * v * inv; cf = std::cos(th);
      } else {
        const double dxl = u * p.fov, dyl = v * p.fov;
        const double nu_ = std::sqrt(dxl * dxl + dyl * dyl + 1.0);
        cr = dxl / nu_; cu = dyl / nu_; cf = 1.0 / nu_;
      }
      double q[4];
      for (int c = 0; c < 4; ++c) q[c] = cf * p.Ef[c] + cr * p.Er[c] + cu * p.Eu[c] - p.U[c];
      const double lq = q[0] + (x * q[1] + y * q[2] + z * q[3]) / r;
      const double pt = -q[0] + f * lq;
      const double flr = f * lq / r;
      const double px = q[1] + flr * x, py = q[2] + flr * y, pz = q[3] + flr * z;
      const double E = std::fabs(pt);
      if (!(E > 1e-12)) continue;
      const double Lx = y * pz - z * py, Ly = z * px - x * pz, Lz = x * py - y * px;
      const double b = std::sqrt(Lx * Lx + Ly * Ly + Lz * Lz) / E;
      const int ip = (int)std::nearbyint(ipx), jp = (int)std::nearbyint(jpx);
      if (b < bbest) { bbest = b; ibest = ip; jbest = jp; }
      if (b < bR) {
        imin = std::min(imin, ip); imax = std::max(imax, ip);
        jmin = std::min(jmin, jp); jmax = std::max(jmax, jp);
      }
    }
  if (imin > imax) { imin = imax = ibest; jmin = jmax = jbest; }
  const int du = 2 * (int)std::ceil((double)(rw - 1) / (nu - 1)) + margin;
  const int dv = 2 * (int)std::ceil((double)(rh - 1) / (nv - 1)) + margin;
  const int c0 = std::min(std::max(imin - du, 1), rw) - 1;
  const int c1 = std::min(std::max(imax + du, 1), rw);
  const int r0 = std::min(std::max(jmin - dv, 1), rh) - 1;
  const int r1 = std::min(std::max(jmax + dv, 1), rh);
  const int cols = c1 - c0, rows = r1 - r0;
  if ((double)cols * rows > 0.55 * rw * rh) return;
  *box = RingBox{c0, cols, r0, rows};
  (void)rp;
}

int layered_render(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
                   int layer_width, int layer_height, const Ring& ring, float* out_rgb, st_ray_diag* host_diag,
                   st_stats* stats) {
  if (!ctx || !out_rgb) return ST_EINVAL;
  int rc = layered_check(cam, stp, rp);
  if (rc != ST_OK) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  TraceParams p;
  st::Variant v;
  if ((rc = fill_params(ctx, cam, stp, rp, &p, &v)) != ST_OK) return rc;
  const int lw = layer_width > 0 ? layer_width : rp->width, lh = layer_height > 0 ? layer_height : rp->height;
  if (lw < 2 || lh < 2 || (long long)lw * lh > (1ll << 30)) return ST_EINVAL;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  cudaStream_t s = ctx->stream;
  const size_t npix = (size_t)rp->width * rp->height;
  if ((rc = ensure(&ctx->d_fb, &ctx->fb_cap, npix)) != ST_OK) return rc;
  if ((rc = ensure(&ctx->d_rgb, &ctx->rgb_cap, 3 * npix)) != ST_OK) return rc;
  if (host_diag && (rc = ensure(&ctx->d_diag, &ctx->diag_cap, npix)) != ST_OK) return rc;
  const bool matter = ctx->disc_on || ctx->vol_on;
  if (matter && (rc = ensure(&ctx->d_layer, &ctx->layer_cap, (size_t)lw * lh)) != ST_OK) return rc;
  // the ring pass (render_layered_gpu!'s ring_out / ring_rmin, src/metal.jl:3102-3118)
  const bool use_ring = matter && ring.rmin > 0.0;
  const int rw = ring.width > 0 ? ring.width : rp->width, rh = ring.height > 0 ? ring.height : rp->height;
  if (use_ring && (rw < 2 || rh < 2 || (long long)rw * rh > (1ll << 30))) return ST_EINVAL;
  if (use_ring && (rc = ensure(&ctx->d_ring, &ctx->ring_cap, (size_t)rw * rh)) != ST_OK) return rc;
  ST_CUDA(cudaMemsetAsync(ctx->d_counters, 0, st::CNT_N * sizeof(unsigned long long), s));
  ST_CUDA(cudaEventRecord(ctx->ev0, s));
  double er[4];
  if ((rc = build_fans(ctx, cam, stp, rp, p, er, s)) != ST_OK) return rc;
  for (int k = 0; k < 4; ++k) p.er[k] = er[k];
  // the gate: no ray whose periapsis stays beyond it meets the disc or the gas
  double gate = 0.0;
  if (ctx->disc_on) gate = std::max(gate, ctx->disc.outer);
  if (ctx->vol_on && p.vol_rb2 > 0.0) gate = std::max(gate, std::sqrt(p.vol_rb2));
  const std::vector<PassPlan> passes = plan_passes(rp, cam);
  int launches = 0;
  RingBox box{0, rw, 0, rh};
  if (use_ring && ring.box) ring_screen_box(p, rp, ring.rmin, rw, rh, &box);
  for (size_t k = 0; k < passes.size(); ++k) {
    const PassPlan& pp = passes[k];
    p.ju = pp.ju; p.jv = pp.jv; p.jw = pp.jw; p.jseed = pp.jseed;
    p.lens_u0 = pp.lens_u0; p.lens_v0 = pp.lens_v0; p.lens_w = pp.lens_w; p.lens_seed = pp.lens_seed;
    st::lay::CompParams cp{ctx->d_fan, FAN_N, ctx->d_fine, FAN_FINE, ctx->d_band, nullptr, lw, lh,
                           nullptr, 0, 0, 0.f};
    if (matter) {
      // the disc / gas layer of this pass at the layer resolution
      TraceParams lp = p;
      lp.width = lw;
      lp.height = lh;
      lp.layer = 1;
      lp.layer_gate = gate;
      lp.fan = ctx->d_fan;
      lp.fan_n = FAN_N;
      lp.out = ctx->d_layer;
      lp.diag = nullptr;
      lp.first_pass = 1;
      lp.weight = 1.0f;
      st::fill_float_copies(&lp);
      st::Variant lv = v;
      lv.sched = ST_SCHED_PIXEL;
      ST_CUDA(st::launch_trace(lv, lp, rp->block_x, rp->block_y, ctx->num_sms, s));
      ++launches;
      cp.layer = ctx->d_layer;
      if (use_ring) {
        // a finer layer of the wound rays only, over the box that can hold them
        ST_CUDA(st::launch_fill_transparent(ctx->d_ring, (size_t)rw * rh, s));
        TraceParams rq = lp;
        rq.width = rw;
        rq.height = rh;
        rq.ring_rmin = ring.rmin;
        rq.out = ctx->d_ring;
        rq.box_col0 = box.c0; rq.box_cols = box.cols;
        rq.box_row0 = box.r0; rq.box_rows = box.rows;
        ST_CUDA(st::launch_trace(lv, rq, rp->block_x, rp->block_y, ctx->num_sms, s));
        launches += 2;
        cp.ring = ctx->d_ring;
        cp.rw = rw;
        cp.rh = rh;
        cp.ring_rmin = (float)ring.rmin;
      }
    }
    p.out = ctx->d_fb;
    p.diag = host_diag ? ctx->d_diag : nullptr;
    p.first_pass = (k == 0) ? 1 : 0;
    p.weight = (float)(1.0 / passes.size());
    if (k == 0) ST_CUDA(cudaStreamWaitEvent(s, ctx->ev_fine, 0));
    ST_CUDA(st::launch_composite(rp->precision, p, cp, s));
    ++launches;
  }
  ST_CUDA(cudaEventRecord(ctx->ev1, s));
  unsigned long long cnt[st::CNT_N];
  ST_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, s));
  ST_CUDA(st::launch_pack_rgb(ctx->d_fb, ctx->d_rgb, (int)npix, s));
  ST_CUDA(cudaMemcpyAsync(out_rgb, ctx->d_rgb, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (host_diag)
    ST_CUDA(cudaMemcpyAsync(host_diag, ctx->d_diag, npix * sizeof(st_ray_diag), cudaMemcpyDeviceToHost, s));
  ST_CUDA(cudaStreamSynchronize(s));
  const int status = cnt[st::CNT_STATUS] ? (int)cnt[st::CNT_STATUS] : ST_OK;
  if (stats) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) { (void)cudaGetLastError(); ms = 0.f; }
    std::memset(stats, 0, sizeof(*stats));
    stats->kernel_ms = ms;
    stats->rays = npix * passes.size();
    stats->steps = cnt[st::CNT_STEPS];
    stats->gas_samples = cnt[st::CNT_GAS];
    stats->launches = launches + 3;
    stats->status = status;
    stats->h2d_bytes = sizeof(TraceParams) * (launches + 3);
    stats->d2h_bytes = 3 * npix * sizeof(float) + sizeof cnt;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return status;
}

}  // namespace

extern "C" {

int st_abi_version(void) { return ST_ABI_VERSION; }

const char* st_strerror(int code) {
  switch (code) {
    case ST_OK: return "ok";
    case ST_EINVAL: return "invalid argument";
    case ST_ECUDA: return "CUDA runtime error";
    case ST_EBUDGET: return "persistent queue iteration budget exhausted";
    case ST_ENOMEM: return "out of memory";
    case ST_EUNSUPPORTED: return "unsupported combination";
    case ST_ESTATE: return "context not ready for this request";
    case ST_ELIMIT: return "request exceeds the fixed scratch capacity of the allocation-free entry point";
    default: return "unknown status";
  }
}

void st_render_params_default(st_render_params* p, int semantics) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->samples = 1;
  p->dt = 0.02;
  p->semantics = semantics;
  p->schedule = ST_SCHED_PIXEL;
  p->seed = 0;
  p->r_guard = 3.0;
  p->crit_band = 0.05;
  p->crit_r = 0.0;
  p->renorm_every = 64;
  p->surrogate_sigma = 1e-4;
  p->chunk_steps = 32;
  p->order = 4;
  p->tol = 1e-4;
  p->refine = 1;
  p->refine_var = 0.35;
  p->refine_graze = 0.05;
  p->refine_margin = 8;
  if (semantics == ST_SEM_RENDER) {
    // render(...; width=400, height=200, samples=1): FP64 like the CPU path
    p->width = 400; p->height = 200;
    p->precision = ST_PREC_FP64;
    p->exit_landing = 1;
    p->pixel_jitter = 0;
  } else {
    // render_draft_mtl(...; width=1920, height=1080, samples=2, dt=0.02): Float32
    p->width = 1920; p->height = 1080; p->samples = 2;
    p->precision = ST_PREC_FP32;
    p->exit_landing = 0;
    p->pixel_jitter = 1;
  }
}

int st_context_create(st_context** out, const float* sky_rgb, int sky_w, int sky_h, int device) {
  if (!out || !sky_rgb || sky_w < 2 || sky_h < 2) return ST_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ST_ECUDA;
  if (device < 0 || device >= ndev) return ST_EINVAL;
  st_context* c = new (std::nothrow) st_context();
  if (!c) return ST_ENOMEM;
  c->device = device;
  auto fail = [&](int code) { st_context_destroy(c); return code; };
  if (cudaSetDevice(device) != cudaSuccess) return fail(ST_ECUDA);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(ST_ECUDA);
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) return fail(ST_ECUDA);
  // sky: (3, W, H) column-major RGB -> float4 [H][W]
  const size_t n = (size_t)sky_w * sky_h;
  std::vector<float4> host(n);
  for (size_t i = 0; i < n; ++i) host[i] = make_float4(sky_rgb[3 * i], sky_rgb[3 * i + 1], sky_rgb[3 * i + 2], 0.f);
  if (cudaMalloc(&c->d_sky, n * sizeof(float4)) != cudaSuccess) return fail(ST_ENOMEM);
  if (cudaMemcpy(c->d_sky, host.data(), n * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(ST_ECUDA);
  c->sky_w = sky_w;
  c->sky_h = sky_h;
  {
    const int rc = upload_lut(c, 6500.0, 500.0, 30000.0, 1024);  // Blackbody() defaults
    if (rc != ST_OK) return fail(rc);
  }
  if (cudaMalloc(&c->d_counters, st::CNT_N * sizeof(unsigned long long)) != cudaSuccess) return fail(ST_ENOMEM);
  if (cudaMalloc(&c->d_queue, sizeof(unsigned int)) != cudaSuccess) return fail(ST_ENOMEM);
  *out = c;
  return ST_OK;
}

int st_context_set_disc(st_context* ctx, const st_disc* d) {
  if (!ctx) return ST_EINVAL;
  if (!d) { ctx->disc_on = false; return ST_OK; }
  const int n = d->table_size > 0 ? d->table_size : 1024;
  const double tmin = d->table_size > 0 ? d->table_min : 500.0;
  const double tmax = d->table_size > 0 ? d->table_max : 30000.0;
  if (d->emitter != ST_EMIT_KEPLER && d->emitter != ST_EMIT_KS_EXACT) return ST_EINVAL;
  const int rc = upload_lut(ctx, d->wb_temperature, tmin, tmax, n);
  if (rc != ST_OK) return rc;
  ctx->disc = *d;
  ctx->disc.table_min = tmin;
  ctx->disc.table_max = tmax;
  ctx->disc.table_size = n;
  ctx->disc_on = true;
  return ST_OK;
}

int st_context_set_volume(st_context* ctx, const st_volume* v) {
  if (!ctx) return ST_EINVAL;
  if (!v) { ctx->vol_on = false; return ST_OK; }
  if (!v->density || v->nr < 2 || v->nphi < 1 || v->nz < 2) return ST_EINVAL;
  if (!(v->log_s_out > v->log_s_in) || !(v->z_max > 0.0f)) return ST_EINVAL;
  const size_t n = (size_t)v->nr * v->nphi * v->nz;
  if (n >= ((size_t)1 << 31)) return ST_EINVAL;  // the float sampler indexes the grid in 32 bits
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  if (ctx->d_vol && ctx->vol_bytes != n * sizeof(float)) { cudaFree(ctx->d_vol); ctx->d_vol = nullptr; }
  if (!ctx->d_vol && cudaMalloc(&ctx->d_vol, n * sizeof(float)) != cudaSuccess) return ST_ENOMEM;
  if (cudaMemcpy(ctx->d_vol, v->density, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return ST_ECUDA;
  ctx->vol_bytes = n * sizeof(float);
  ctx->vol = *v;
  ctx->vol.density = nullptr;
  ctx->vol_on = true;
  return ST_OK;
}

void st_starfield_default(st_starfield* sf) {
  if (!sf) return;
  std::memset(sf, 0, sizeof(*sf));
  sf->strength = 1.0;
  sf->texture_weight = 0.0;
  sf->height = 1080;
  sf->fov_factor = 0.55;
  sf->density = 384.0;
  sf->fill = 0.5;
  sf->flux = 0.011;
  sf->psf_pixels = 0.5;
  sf->galactic[2] = 1.0;
  sf->concentration = 3.0;
  sf->temp_min = 3000.0;
  sf->temp_max = 16000.0;
  sf->seed = 12345;
  sf->wb_temperature = 10000.0;  // STAR_WB_TEMPERATURE, src/metal.jl:75
  sf->saturation = 1.0;
  sf->table_size = 1024;
}

// Star colour table (_star_lut_cpu, src/metal.jl:86-104): Blackbody(wb) entries
// over [500, 30000] K in single precision, chroma scaled by `saturation`
// about Rec.709 luminance.
int st_context_set_starfield(st_context* ctx, const st_starfield* sf) {
  if (!ctx) return ST_EINVAL;
  if (!sf || !(sf->strength > 0.0)) { ctx->star_on = false; return ST_OK; }
  const double gn = std::sqrt(sf->galactic[0] * sf->galactic[0] + sf->galactic[1] * sf->galactic[1] +
                              sf->galactic[2] * sf->galactic[2]);
  if (!(gn > 0.0) || sf->height < 1 || !(sf->density >= 1.0) || !(sf->psf_pixels > 0.0) ||
      sf->table_size < 2 || sf->table_size > (1 << 20) || !(sf->wb_temperature > 0.0))
    return ST_EINVAL;
  const int n = sf->table_size;
  const double tmin = 500.0, tmax = 30000.0;
  double ref[3];
  st::host_blackbody(sf->wb_temperature, ref);
  std::vector<float4> lut(n);
  const float sat = (float)sf->saturation;
  for (int i = 0; i < n; ++i) {
    const double T = tmin + (tmax - tmin) * i / (n - 1);
    double c[3];
    st::host_blackbody(std::max(T, 1.0), c);
    float r = (float)(c[0] / ref[0]), g = (float)(c[1] / ref[1]), b = (float)(c[2] / ref[2]);
    if (sf->saturation != 1.0) {
      const float L = 0.2126f * r + 0.7152f * g + 0.0722f * b;
      r = L + sat * (r - L); g = L + sat * (g - L); b = L + sat * (b - L);
    }
    lut[i] = make_float4(r, g, b, 0.f);
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  if (ctx->d_star_lut && ctx->star_lut_size != n) {
    cudaFree(ctx->d_star_lut);
    ctx->d_star_lut = nullptr;
    ctx->star_lut_size = 0;
  }
  if (!ctx->d_star_lut && cudaMalloc(&ctx->d_star_lut, n * sizeof(float4)) != cudaSuccess) return ST_ENOMEM;
  if (cudaMemcpy(ctx->d_star_lut, lut.data(), n * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess)
    return ST_ECUDA;
  ctx->star_lut_size = n;
  ctx->star_lut_tmin = tmin;
  ctx->star_lut_tmax = tmax;
  ctx->star = *sf;
  ctx->star_on = true;
  return ST_OK;
}

void st_context_destroy(st_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_sky);
  cudaFree(ctx->d_lut);
  cudaFree(ctx->d_star_lut);
  cudaFree(ctx->d_stat);
  cudaFree(ctx->d_defer);
  cudaFree(ctx->d_defer_count);
  cudaFree(ctx->d_buckets);
  cudaFree(ctx->d_box);
  cudaFree(ctx->d_fan);
  cudaFree(ctx->d_fine);
  cudaFree(ctx->d_band);
  cudaFree(ctx->d_layer);
  cudaFree(ctx->d_ring);
  if (ctx->ev_coarse) cudaEventDestroy(ctx->ev_coarse);
  if (ctx->ev_fine) cudaEventDestroy(ctx->ev_fine);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  cudaFree(ctx->d_vol);
  cudaFree(ctx->d_fb);
  cudaFree(ctx->d_rgb);
  cudaFree(ctx->d_diag);
  cudaFree(ctx->d_frames);
  cudaFree(ctx->d_counters);
  cudaFree(ctx->d_queue);
  cudaFree(ctx->d_list);
  cudaFree(ctx->d_count);
  cudaFree(ctx->d_order);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  cudaFreeHost(ctx->h_frames);
  cudaFreeHost(ctx->h_cnt);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int st_render(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
              float* out_rgb, st_stats* stats) {
  if (!out_rgb) return ST_EINVAL;
  return do_render(ctx, cam, st, p, out_rgb, nullptr, nullptr, stats);
}

int st_render_diag(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                   float* out_rgb, st_ray_diag* diag, st_stats* stats) {
  if (!out_rgb || !diag) return ST_EINVAL;
  return do_render(ctx, cam, st, p, out_rgb, diag, nullptr, stats);
}

int st_render_motion(st_context* ctx, const st_camera* cam, const st_camera* poses, int nposes,
                     int per_pixel_shutter, const st_spacetime* st, const st_render_params* p, float* out_rgb,
                     st_ray_diag* diag, st_stats* stats) {
  if (!out_rgb || !cam || !poses || !p || p->samples <= 0) return ST_EINVAL;
  const int n = p->samples * p->samples;
  if (nposes != (per_pixel_shutter ? n + 1 : n)) return ST_EINVAL;
  if (p->surrogate) return ST_EUNSUPPORTED;
  const Motion mo{poses, nposes, per_pixel_shutter ? 1 : 0};
  return do_render(ctx, cam, st, p, out_rgb, diag, nullptr, stats, &mo);
}

int st_render_depth(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                    int nbuckets, float* out_buckets, st_stats* stats) {
  if (!out_buckets) return ST_EINVAL;
  if (nbuckets < 3 || nbuckets > 64) return ST_EINVAL;
  const Depth d{nbuckets, out_buckets};
  return do_render(ctx, cam, st, p, nullptr, nullptr, nullptr, stats, nullptr, &d);
}

int st_sky_fan(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
               float* fan, float* fine, float* band) {
  if (!ctx || !fan || !fine || !band) return ST_EINVAL;
  int rc = layered_check(cam, stp, rp);
  if (rc != ST_OK) return rc;
  TraceParams p;
  st::Variant v;
  if ((rc = fill_params(ctx, cam, stp, rp, &p, &v)) != ST_OK) return rc;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  cudaStream_t s = ctx->stream;
  double er[4];
  if ((rc = build_fans(ctx, cam, stp, rp, p, er, s)) != ST_OK) return rc;
  ST_CUDA(cudaStreamWaitEvent(s, ctx->ev_fine, 0));
  ST_CUDA(cudaMemcpyAsync(fan, ctx->d_fan, FAN_N * sizeof(float4), cudaMemcpyDeviceToHost, s));
  ST_CUDA(cudaMemcpyAsync(fine, ctx->d_fine, FAN_FINE * sizeof(float4), cudaMemcpyDeviceToHost, s));
  ST_CUDA(cudaMemcpyAsync(band, ctx->d_band, 2 * sizeof(float), cudaMemcpyDeviceToHost, s));
  ST_CUDA(cudaStreamSynchronize(s));
  return ST_OK;
}

int st_render_layered(st_context* ctx, const st_camera* cam, const st_spacetime* stp, const st_render_params* rp,
                      int layer_width, int layer_height, float* out_rgb, st_ray_diag* host_diag, st_stats* stats) {
  return layered_render(ctx, cam, stp, rp, layer_width, layer_height, Ring{0, 0, 0.0, 0}, out_rgb, host_diag, stats);
}

int st_render_layered_ring(st_context* ctx, const st_camera* cam, const st_spacetime* stp,
                           const st_render_params* rp, int layer_width, int layer_height, int ring_width,
                           int ring_height, double ring_rmin, int ring_box, float* out_rgb, st_ray_diag* host_diag,
                           st_stats* stats) {
  if (!(ring_rmin >= 0.0) || !std::isfinite(ring_rmin)) return ST_EINVAL;
  return layered_render(ctx, cam, stp, rp, layer_width, layer_height,
                        Ring{ring_width, ring_height, ring_rmin, ring_box ? 1 : 0}, out_rgb, host_diag, stats);
}

int st_render_device(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                     const float** dev_rgba, st_stats* stats) {
  if (!dev_rgba) return ST_EINVAL;
  return do_render(ctx, cam, st, p, nullptr, nullptr, dev_rgba, stats);
}

// A camera track with the learned surrogate: each frame's network inputs are
// taken in that frame's own static frame, so the frames run one after
// another through the single-frame path (a surrogate pass, then one trace
// launch over the pixels the gate left), into consecutive slots of out_rgb.
// Every camera is checked first, so a track with a camera outside the
// network's domain is refused whole and nothing is written.  The first frame
// that returns a status other than ST_OK ends the call with that status.
int render_frames_surrogate(st_context* ctx, int nframes, const st_camera* cams, const st_spacetime* stp,
                            const st_render_params* rp, float* out_rgb, st_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  const size_t npix = (size_t)rp->width * rp->height;
  if (rp->width <= 0 || rp->height <= 0 || npix * (size_t)nframes > (size_t)1 << 31) return ST_EINVAL;
  for (int f = 0; f < nframes; ++f) {
    TraceParams q;
    st::Variant w;
    const int rc = fill_params(ctx, &cams[f], stp, rp, &q, &w);
    if (rc != ST_OK) return rc;
    st::SurFrame sf{};
    if (!surrogate_domain(&cams[f], stp, &sf)) return ST_EUNSUPPORTED;
  }
  st_stats tot;
  std::memset(&tot, 0, sizeof tot);
  for (int f = 0; f < nframes; ++f) {
    st_stats one;
    std::memset(&one, 0, sizeof one);
    one.status = -1;  // stays -1 if the call fails before its stats are written
    const int rc = do_render(ctx, &cams[f], stp, rp, out_rgb + 3 * npix * (size_t)f, nullptr, nullptr, &one);
    if (rc != ST_OK && one.status == -1) return rc;
    tot.kernel_ms += one.kernel_ms;
    tot.rays += one.rays;
    tot.steps += one.steps;
    tot.fp64_steps += one.fp64_steps;
    tot.gas_samples += one.gas_samples;
    tot.surrogate_rays += one.surrogate_rays;
    tot.launches += one.launches;
    tot.h2d_bytes += one.h2d_bytes;
    tot.d2h_bytes += one.d2h_bytes;
    tot.status = one.status;
    if (rc != ST_OK) break;
  }
  tot.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = tot;
  return tot.status;
}

int st_render_frames(st_context* ctx, int nframes, const st_camera* cams, const st_spacetime* stp,
                     const st_render_params* rp, float* out_rgb, st_stats* stats) {
  if (!ctx || nframes <= 0 || !cams || !stp || !rp || !out_rgb) return ST_EINVAL;
  if (rp->semantics != ST_SEM_DRAFT || rp->samples != 1) return ST_EUNSUPPORTED;
  if (rp->surrogate) return render_frames_surrogate(ctx, nframes, cams, stp, rp, out_rgb, stats);
  if (rp->order != 0 && rp->order != 4 && rp->schedule == ST_SCHED_PERSISTENT) return ST_EUNSUPPORTED;
  const auto t0 = std::chrono::steady_clock::now();
  TraceParams p;
  st::Variant v;
  int rc = fill_params(ctx, &cams[0], stp, rp, &p, &v);
  if (rc != ST_OK) return rc;
  const size_t npix = (size_t)rp->width * rp->height;
  if (npix * (size_t)nframes > (size_t)1 << 31) return ST_EINVAL;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return ST_ECUDA;
  if (ctx->h_frames_cap < (size_t)nframes) {
    cudaFreeHost(ctx->h_frames);
    ctx->h_frames = nullptr;
    ctx->h_frames_cap = 0;
    if (cudaMallocHost(&ctx->h_frames, nframes * sizeof(st::FrameCam)) != cudaSuccess) return ST_ENOMEM;
    ctx->h_frames_cap = nframes;
  }
  if (!ctx->h_cnt && cudaMallocHost(&ctx->h_cnt, st::CNT_N * sizeof(unsigned long long)) != cudaSuccess)
    return ST_ENOMEM;
  st::FrameCam* fc = ctx->h_frames;
  int nmax_max = 0;
  for (int f = 0; f < nframes; ++f) {
    TraceParams q;
    st::Variant w;
    rc = fill_params(ctx, &cams[f], stp, rp, &q, &w);
    if (rc != ST_OK) return rc;
    std::memcpy(fc[f].pos, q.pos, sizeof q.pos);
    std::memcpy(fc[f].Ef, q.Ef, sizeof q.Ef);
    std::memcpy(fc[f].Er, q.Er, sizeof q.Er);
    std::memcpy(fc[f].Eu, q.Eu, sizeof q.Eu);
    std::memcpy(fc[f].U, q.U, sizeof q.U);
    fc[f].r_escape = q.r_escape;
    fc[f].nmax = q.nmax;
    fc[f].pad = 0;
    nmax_max = std::max(nmax_max, q.nmax);
  }
  if ((rc = ensure(&ctx->d_frames, &ctx->frames_cap, (size_t)nframes)) != ST_OK) return rc;
  if ((rc = ensure(&ctx->d_fb, &ctx->fb_cap, npix * nframes)) != ST_OK) return rc;
  if ((rc = ensure(&ctx->d_rgb, &ctx->rgb_cap, 3 * npix * nframes)) != ST_OK) return rc;
  cudaStream_t s = ctx->stream;
  const std::vector<PassPlan> passes = plan_passes(rp, &cams[0]);
  const PassPlan& pp = passes[0];
  p.ju = pp.ju; p.jv = pp.jv; p.jw = pp.jw; p.jseed = pp.jseed;
  p.weight = 1.0f;
  p.first_pass = 1;
  p.out = ctx->d_fb;
  p.frames = ctx->d_frames;
  p.n_frames = nframes;
  p.frame_stride = (int)npix;
  // the frame-independent camera fields are unused with a frame table: zero
  // them so the graph key depends only on sizes and rules
  std::memset(p.pos, 0, sizeof p.pos);
  std::memset(p.Ef, 0, sizeof p.Ef);
  std::memset(p.Er, 0, sizeof p.Er);
  std::memset(p.Eu, 0, sizeof p.Eu);
  std::memset(p.U, 0, sizeof p.U);
  p.r_escape = 0.0;
  const long long tiles = (long long)((rp->width + 7) / 8) * ((rp->height + 3) / 4);
  // the queue counts rays of whole 8x4 tiles in a 32-bit int
  if (tiles * 32 * nframes > (long long)INT_MAX) return ST_EINVAL;
  p.n_rays = (int)(tiles * 32 * nframes);
  p.chunk_steps = rp->chunk_steps > 0 ? rp->chunk_steps : 32;
  p.budget_iters = queue_budget(((long long)p.n_rays + 32) * ((long long)nmax_max / p.chunk_steps + 2));
  p.nmax = nmax_max;
  v.sched = rp->schedule == ST_SCHED_PIXEL ? ST_SCHED_PIXEL : ST_SCHED_PERSISTENT;
  if ((rc = setup_defer(ctx, &p, v, npix * nframes)) != ST_OK) return rc;
  ctx->h2d_extra = 0;
  if (v.sched == ST_SCHED_PIXEL) {
    // every frame's slice of the grid dispatched centre first (the first
    // camera's projection of the hole)
    int bx = rp->block_x, by = rp->block_y;
    if (bx <= 0 || by <= 0 || bx * by != 128) { bx = 16; by = 8; }
    if ((rc = ensure_tile_order(ctx, &cams[0], rp->width, rp->height, bx, by, s, &p.tile_order)) != ST_OK) return rc;
  }
  // the device work of one call: stage cameras, clear queue and counters,
  // trace all frames in one launch, pack, read the counters
  // Under stream capture a plain event record only orders streams; the
  // external flag makes it an event-record node, so replays are timed too.
  auto enqueue = [&](bool capturing) -> int {
    const unsigned ev_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    ST_CUDA(cudaMemcpyAsync(ctx->d_frames, ctx->h_frames, nframes * sizeof(st::FrameCam), cudaMemcpyHostToDevice, s));
    ST_CUDA(cudaMemsetAsync(ctx->d_counters, 0, st::CNT_N * sizeof(unsigned long long), s));
    ST_CUDA(cudaMemsetAsync(ctx->d_queue, 0, sizeof(unsigned int), s));
    ST_CUDA(cudaEventRecordWithFlags(ctx->ev0, s, ev_flags));
    ST_CUDA(st::launch_trace(v, p, rp->block_x, rp->block_y, ctx->num_sms, s));
    ST_CUDA(cudaEventRecordWithFlags(ctx->ev1, s, ev_flags));
    ST_CUDA(st::launch_pack_rgb(ctx->d_fb, ctx->d_rgb, (int)(npix * nframes), s));
    ST_CUDA(cudaMemcpyAsync(ctx->h_cnt, ctx->d_counters, st::CNT_N * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
    return ST_OK;
  };
  if (rp->graph) {
    const size_t key_bytes = (size_t)nframes;
    const bool same = ctx->gexec && ctx->gbytes == key_bytes && std::memcmp(&ctx->gkey, &p, sizeof p) == 0 &&
                      std::memcmp(&ctx->gvar, &v, sizeof v) == 0;
    if (!same) {
      if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
      cudaGraph_t g = nullptr;
      ST_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int erc = enqueue(true);
      const cudaError_t ec = cudaStreamEndCapture(s, &g);
      if (erc != ST_OK || ec != cudaSuccess) { if (g) cudaGraphDestroy(g); return ST_ECUDA; }
      const cudaError_t ei = cudaGraphInstantiate(&ctx->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) { ctx->gexec = nullptr; return ST_ECUDA; }
      ctx->gkey = p;
      ctx->gvar = v;
      ctx->gbytes = key_bytes;
    }
    ST_CUDA(cudaGraphLaunch(ctx->gexec, s));
  } else {
    if ((rc = enqueue(false)) != ST_OK) return rc;
  }
  ST_CUDA(cudaMemcpyAsync(out_rgb, ctx->d_rgb, 3 * npix * nframes * sizeof(float), cudaMemcpyDeviceToHost, s));
  ST_CUDA(cudaStreamSynchronize(s));
  const unsigned long long* cnt = ctx->h_cnt;
  const int status = cnt[st::CNT_STATUS] ? (int)cnt[st::CNT_STATUS] : ST_OK;
  if (stats) {
    float ms = 0.f;
    // a failed query must not leave an error pending for the next launch check
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) { (void)cudaGetLastError(); ms = 0.f; }
    std::memset(stats, 0, sizeof(*stats));
    stats->kernel_ms = ms;
    stats->rays = cnt[st::CNT_RAYS];
    stats->steps = cnt[st::CNT_STEPS];
    stats->fp64_steps = cnt[st::CNT_FP64];
    stats->gas_samples = cnt[st::CNT_GAS];
    stats->launches = 1;
    stats->status = status;
    stats->h2d_bytes = nframes * sizeof(st::FrameCam) + (rp->graph ? 0 : sizeof(TraceParams)) + ctx->h2d_extra;
    stats->d2h_bytes = 3 * npix * nframes * sizeof(float) + st::CNT_N * sizeof(unsigned long long);
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return status;
}

int st_context_set_surrogate(st_context* ctx, st_surrogate* s) {
  if (!ctx) return ST_EINVAL;
  ctx->sur = s;
  return ST_OK;
}

int st_camera_tetrad(const st_camera* cam, const st_spacetime* stp, double out16[16]) {
  if (!cam || !stp || !out16) return ST_EINVAL;
  if (!(stp->M > 0.0) || !(std::fabs(stp->a) <= stp->M)) return ST_EINVAL;
  const double beta[3] = {st::dot3(cam->velocity, cam->fwd), st::dot3(cam->velocity, cam->right),
                          st::dot3(cam->velocity, cam->up)};
  st::host_tetrad(cam->pos, cam->fwd, cam->right, cam->up, stp->M, stp->a, beta, out16, out16 + 4, out16 + 8,
                  out16 + 12);
  return ST_OK;
}

}  // extern "C"

// Camera- and rule-dependent part of a trace launch for one camera, without a
// context (used by the allocation-free entry point in st_noalloc.cu).
namespace st {
int fill_frame_params(const st_camera* cam, const st_spacetime* stp, const st_render_params* rp, TraceParams* p) {
  if (!cam || !stp || !rp || !p) return ST_EINVAL;
  const double M = stp->M, a = stp->a;
  if (!(M > 0.0) || !(std::fabs(a) <= M)) return ST_EINVAL;
  if (rp->width <= 0 || rp->height <= 0 || !(rp->dt > 0.0)) return ST_EINVAL;
  if (rp->precision < ST_PREC_FP64 || rp->precision > ST_PREC_FP32_GUARDED_DF) return ST_EINVAL;
  const double rpos = norm3(cam->pos);
  if (!(rpos > 0.0) || !std::isfinite(rpos)) return ST_EINVAL;
  std::memset(p, 0, sizeof(*p));
  const double beta[3] = {dot3(cam->velocity, cam->fwd), dot3(cam->velocity, cam->right),
                          dot3(cam->velocity, cam->up)};
  host_tetrad(cam->pos, cam->fwd, cam->right, cam->up, M, a, beta, p->U, p->Ef, p->Er, p->Eu);
  for (int k = 0; k < 3; ++k) p->pos[k] = cam->pos[k];
  p->fov = cam->fov_factor;
  p->projection = cam->projection;
  p->fisheye_rad = std::max(cam->fisheye_deg, 0.0) * 3.141592653589793 / 180.0;
  p->focus = cam->focus_dist > 0.0 ? cam->focus_dist : 1.0;
  p->width = rp->width;
  p->height = rp->height;
  p->frame_stride = rp->width * rp->height;
  p->M = M;
  p->a = a;
  const float rk = (float)(0.995 * host_photon_orbit_min(M, a));
  p->rkill2 = (double)(rk * rk);
  host_isco(M, a, &p->r_isco, &p->E_isco, &p->L_isco);
  p->dt = rp->dt;
  p->hcoef = 0.16;
  p->hcap = 8.0;
  p->order = 4;
  p->tol = 1e-4;
  p->relativistic = rp->relativistic ? 1 : 0;
  const double re = rp->r_escape > 0.0 ? rp->r_escape : (double)(float)(2.0 * std::max(rpos, 15.0 * M));
  p->r_escape = re;
  if (rp->nmax > 0) {
    p->nmax = rp->nmax;
  } else {
    const double lg = (double)std::log((float)((float)re / (float)M));
    const double n = std::ceil((75.0 + 6.5 * lg) * (double)(float)M / (double)(float)rp->dt);
    p->nmax = (int)std::min(std::max(1000.0, n), 40000.0);
  }
  p->exit_landing = rp->exit_landing ? 1 : 0;
  const double rg = rp->r_guard > 0.0 ? rp->r_guard : 0.0;
  p->r_guard2 = rg * rg;
  p->crit_band = rp->crit_band;
  p->crit_r2 = rp->crit_r > 0.0 ? rp->crit_r * rp->crit_r : 0.0;
  p->b_crit = 3.0 * std::sqrt(3.0) * M;
  p->renorm_every = rp->renorm_every;
  p->guard_df = rp->precision == ST_PREC_FP32_GUARDED_DF ? 1 : 0;
  p->refill_window = 32;
  p->chunk_steps = rp->chunk_steps > 0 ? rp->chunk_steps : 32;
  return ST_OK;
}
}  // namespace st
