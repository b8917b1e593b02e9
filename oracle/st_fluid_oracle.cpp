// st_fluid_oracle.cpp -- CPU restatement of the live fluid disc
// (DiscFluidSim / step_sim!, src/disc_sim.jl), TEST INFRASTRUCTURE ONLY: the
// checker the CUDA solver is compared against, never part of the product.
//
// Follows the reference kernel by kernel, unfused, each over the whole grid
// with its own output buffer, in float with every operation rounded as
// written (the build uses -ffp-contract=off):
//   construction      src/disc_sim.jl:45-91 (and _disc_radial_profile,
//                     src/disc_volume.jl:274-283)
//   _sim_hash / _sim_noise / _sim_sample   :80-134
//   k_advect_vel!, k_force!, k_div!, k_jacobi!, k_subgrad!   :136-203
//   k_adv_scalar!, k_maccormack!, k_extrude!                 :205-266
//   step_sim!         :287-320
// Parity unpinned: the reference has no tests, fixtures or golden outputs
// for this solver and cannot run here, so the restatement is checked by
// properties its equations fix (construction, zero-velocity shear transport,
// divergence reduction, extrusion) in the CPU tests.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "st_oracle.h"

namespace {

float fhash(int32_t x, int32_t y, int32_t z) {
  uint32_t h = (uint32_t)x * 0x8da6b343u ^ (uint32_t)y * 0xd8163841u ^ (uint32_t)z * 0xcb1ab31fu;
  h ^= h >> 13;
  h *= 0x9e3779b9u;
  h ^= h >> 16;
  return (float)(h & 0x00ffffffu) * 5.9604645e-8f;
}

float fnoise(float x, float y, float z) {
  const int32_t ix = (int32_t)std::floor(x), iy = (int32_t)std::floor(y), iz = (int32_t)std::floor(z);
  float fx = x - std::floor(x), fy = y - std::floor(y), fz = z - std::floor(z);
  fx = fx * fx * (3.0f - 2.0f * fx);
  fy = fy * fy * (3.0f - 2.0f * fy);
  fz = fz * fz * (3.0f - 2.0f * fz);
  const int32_t i1 = ix + 1, j1 = iy + 1, k1 = iz + 1;
  const float c00 = fhash(ix, iy, iz) + fx * (fhash(i1, iy, iz) - fhash(ix, iy, iz));
  const float c10 = fhash(ix, j1, iz) + fx * (fhash(i1, j1, iz) - fhash(ix, j1, iz));
  const float c01 = fhash(ix, iy, k1) + fx * (fhash(i1, iy, k1) - fhash(ix, iy, k1));
  const float c11 = fhash(ix, j1, k1) + fx * (fhash(i1, j1, k1) - fhash(ix, j1, k1));
  const float c0 = c00 + fy * (c10 - c00);
  const float c1 = c01 + fy * (c11 - c01);
  return c0 + fz * (c1 - c0);
}

// Julia's mod: the result has the sign of the divisor
int jl_mod(int a, int n) { return ((a % n) + n) % n; }
float jl_clamp(float x, float lo, float hi) { return x > hi ? hi : (x < lo ? lo : x); }

struct Grid {
  int nr, nphi;
  float& at(std::vector<float>& f, int i, int j) const { return f[(size_t)(i - 1) + (size_t)nr * (j - 1)]; }
  float at(const std::vector<float>& f, int i, int j) const { return f[(size_t)(i - 1) + (size_t)nr * (j - 1)]; }
};

float sample(const Grid& g, const std::vector<float>& f, float x, float y) {
  const int nr = g.nr, nphi = g.nphi;
  x = jl_clamp(x, 1.0f, (float)nr);
  const int i0 = std::min(std::max((int)std::floor(x), 1), nr - 1);
  const float tx = x - (float)i0;
  const float yw = y - (float)nphi * std::floor((y - 1.0f) / (float)nphi);
  const int j0 = (int)std::floor(yw);
  const float ty = yw - (float)j0;
  const int j0a = jl_mod(j0 - 1, nphi) + 1;
  const int j1a = jl_mod(j0, nphi) + 1;
  const float a = g.at(f, i0, j0a) + tx * (g.at(f, i0 + 1, j0a) - g.at(f, i0, j0a));
  const float b = g.at(f, i0, j1a) + tx * (g.at(f, i0 + 1, j1a) - g.at(f, i0, j1a));
  return a + ty * (b - a);
}

void adv_scalar(const Grid& g, std::vector<float>& dst, const std::vector<float>& src, const std::vector<float>& vu,
                const std::vector<float>& vv, const std::vector<float>& shear, float dt) {
  for (int j = 1; j <= g.nphi; ++j)
    for (int i = 1; i <= g.nr; ++i) {
      const float x = (float)i - dt * g.at(vu, i, j);
      const float y = (float)j - dt * (g.at(vv, i, j) + shear[i - 1]);
      g.at(dst, i, j) = sample(g, src, x, y);
    }
}

}  // namespace

extern "C" {

int orc_fluid_init(orc_fluid* f, const float* vol_density, float log_s_in, float log_s_out, float z_max,
                   double scale_height, double M, double inner, double outer, double falloff) {
  if (!f || !vol_density || f->nr < 2 || f->nphi < 1 || f->nz < 2) return 1;
  if (!f->vu || !f->vv || !f->dens || !f->base || !f->env || !f->shear) return 1;
  const int nr = f->nr, nphi = f->nphi, nz = f->nz;
  const size_t n = (size_t)nr * nphi;
  const int kmid = (nz + 1) / 2;  // 1-based
  const float* slice = vol_density + (size_t)(kmid - 1) * n;
  float peak = slice[0];
  for (size_t c = 0; c < n; ++c) peak = std::max(peak, slice[c]);
  for (size_t c = 0; c < n; ++c) f->dens[c] = peak > 0.0f ? slice[c] / peak : slice[c];
  const float dlog = log_s_out - log_s_in;
  const float hsc = (float)scale_height;
  for (int i = 1; i <= nr; ++i) {
    const double s = std::exp((double)log_s_in + (double)(i - 1) / (double)(nr - 1) * (double)dlog);
    const double R = s / (2.0 * M), R_in = inner / (2.0 * M), R_out = outer / (2.0 * M);
    const double iscotaper = std::min(std::max((R * R - R_in * R_in) * 0.3, 0.0), 1.0);
    const double T_emit = std::exp(10.034259 - 0.375 * std::log(R * R));
    const double outertaper = std::min(std::max(T_emit / 1000.0, 0.0), 1.0);
    const double density = std::min(std::max((R_out - R) / (R_out - R_in), 0.0), 1.0);
    const float b = (float)(iscotaper * outertaper * std::pow(density, falloff));
    for (int j = 1; j <= nphi; ++j) f->base[(size_t)(i - 1) + (size_t)nr * (j - 1)] = b;
    const double H = (double)hsc * s;
    for (int k = 1; k <= nz; ++k) {
      const double z = -(double)z_max + (double)(k - 1) / (double)(nz - 1) * 2.0 * (double)z_max;
      f->env[(size_t)(i - 1) + (size_t)nr * (k - 1)] = (float)std::exp(-(z * z) / (2.0 * H * H));
    }
    f->shear[i - 1] = (float)(std::sqrt(M / (s * s * s)) * nphi / (2.0 * M_PI));
  }
  std::fill(f->vu, f->vu + n, 0.0f);
  std::fill(f->vv, f->vv + n, 0.0f);
  f->t = 0.0f;
  return 0;
}

int orc_fluid_step(orc_fluid* f, float* vol_out, double dt_in, int jacobi, int nsteps) {
  if (!f || jacobi < 0 || nsteps < 0) return 1;
  const Grid g{f->nr, f->nphi};
  const int nr = f->nr, nphi = f->nphi, nz = f->nz;
  const size_t n = (size_t)nr * nphi;
  const float dt = (float)dt_in;
  std::vector<float> vu(f->vu, f->vu + n), vv(f->vv, f->vv + n), dens(f->dens, f->dens + n);
  const std::vector<float> base(f->base, f->base + n), shear(f->shear, f->shear + nr);
  std::vector<float> vu2(n), vv2(n), dv(n), prs(n), prs2(n), dens2(n), dens3(n);
  const float amp = (float)f->forcing, drag = (float)f->drag, relax = (float)f->relax;
  for (int step = 0; step < nsteps; ++step) {
    const float t = f->t;
    // k_advect_vel!
    for (int j = 1; j <= nphi; ++j)
      for (int i = 1; i <= nr; ++i) {
        const float x = (float)i - dt * g.at(vu, i, j);
        const float y = (float)j - dt * (g.at(vv, i, j) + shear[i - 1]);
        g.at(vu2, i, j) = sample(g, vu, x, y);
        g.at(vv2, i, j) = sample(g, vv, x, y);
      }
    std::swap(vu, vu2);
    std::swap(vv, vv2);
    // k_force!
    for (int j = 1; j <= nphi; ++j)
      for (int i = 1; i <= nr; ++i) {
        const float sc = 0.085f;
        const float x = (float)i * sc, y = (float)j * sc, z = t * 0.35f;
        const float e = 0.35f;
        const float dpy = fnoise(x, y + e, z) - fnoise(x, y - e, z);
        const float dpx = fnoise(x + e, y, z) - fnoise(x - e, y, z);
        const float fu = dpy / (2.0f * e);
        const float fv = -dpx / (2.0f * e);
        float edge = std::min((float)i - 1.0f, (float)(nr - i)) * 0.125f;
        edge = jl_clamp(edge, 0.0f, 1.0f);
        const float damp = std::exp(-drag * dt);
        g.at(vu, i, j) = (g.at(vu, i, j) + dt * amp * fu * edge) * damp * edge;
        g.at(vv, i, j) = (g.at(vv, i, j) + dt * amp * fv * edge) * damp;
      }
    // k_div!
    for (int j = 1; j <= nphi; ++j)
      for (int i = 1; i <= nr; ++i) {
        const int ip = std::min(i + 1, nr), im = std::max(i - 1, 1);
        const int jp = jl_mod(j, nphi) + 1, jm = jl_mod(j - 2, nphi) + 1;
        g.at(dv, i, j) = 0.5f * (g.at(vu, ip, j) - g.at(vu, im, j) + g.at(vv, i, jp) - g.at(vv, i, jm));
      }
    // pressure: 2 ceil(jacobi / 2) sweeps from 0
    std::fill(prs.begin(), prs.end(), 0.0f);
    const int sweeps = 2 * ((jacobi + 1) / 2);
    for (int k = 0; k < sweeps; ++k) {
      for (int j = 1; j <= nphi; ++j)
        for (int i = 1; i <= nr; ++i) {
          const int ip = std::min(i + 1, nr), im = std::max(i - 1, 1);
          const int jp = jl_mod(j, nphi) + 1, jm = jl_mod(j - 2, nphi) + 1;
          g.at(prs2, i, j) =
              0.25f * (g.at(prs, ip, j) + g.at(prs, im, j) + g.at(prs, i, jp) + g.at(prs, i, jm) - g.at(dv, i, j));
        }
      std::swap(prs, prs2);
    }
    // k_subgrad!
    for (int j = 1; j <= nphi; ++j)
      for (int i = 1; i <= nr; ++i) {
        const int ip = std::min(i + 1, nr), im = std::max(i - 1, 1);
        const int jp = jl_mod(j, nphi) + 1, jm = jl_mod(j - 2, nphi) + 1;
        g.at(vu, i, j) -= 0.5f * (g.at(prs, ip, j) - g.at(prs, im, j));
        g.at(vv, i, j) -= 0.5f * (g.at(prs, i, jp) - g.at(prs, i, jm));
      }
    // MacCormack: forward, backward, corrected combine
    adv_scalar(g, dens2, dens, vu, vv, shear, dt);
    adv_scalar(g, dens3, dens2, vu, vv, shear, -dt);
    std::vector<float> dnew(n);
    for (int j = 1; j <= nphi; ++j)
      for (int i = 1; i <= nr; ++i) {
        const float x = (float)i - dt * g.at(vu, i, j);
        const float y = (float)j - dt * (g.at(vv, i, j) + shear[i - 1]);
        const float xc = jl_clamp(x, 1.0f, (float)nr);
        const int i0 = std::min(std::max((int)std::floor(xc), 1), nr - 1);
        const float yw = y - (float)nphi * std::floor((y - 1.0f) / (float)nphi);
        const int j0 = (int)std::floor(yw);
        const int j0a = jl_mod(j0 - 1, nphi) + 1, j1a = jl_mod(j0, nphi) + 1;
        const int i1 = i0 + 1;
        const float lo = std::min(std::min(g.at(dens, i0, j0a), g.at(dens, i1, j0a)),
                                  std::min(g.at(dens, i0, j1a), g.at(dens, i1, j1a)));
        const float hi = std::max(std::max(g.at(dens, i0, j0a), g.at(dens, i1, j0a)),
                                  std::max(g.at(dens, i0, j1a), g.at(dens, i1, j1a)));
        const float a = jl_clamp(g.at(dens2, i, j) + 0.5f * (g.at(dens, i, j) - g.at(dens3, i, j)), lo, hi);
        const float nz_ = fnoise((float)i * 0.11f, (float)j * 0.11f, t * 0.25f);
        const float tgt = g.at(base, i, j) * std::exp(1.2f * (2.0f * nz_ - 1.0f));
        g.at(dnew, i, j) = std::max(a + relax * dt * (tgt - a), 0.0f);
      }
    dens.swap(dnew);
    f->t = t + dt;
  }
  std::copy(vu.begin(), vu.end(), f->vu);
  std::copy(vv.begin(), vv.end(), f->vv);
  std::copy(dens.begin(), dens.end(), f->dens);
  // k_extrude!
  if (vol_out)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nphi; ++j)
        for (int i = 1; i <= nr; ++i)
          vol_out[(size_t)(i - 1) + (size_t)nr * ((j - 1) + (size_t)nphi * (k - 1))] =
              g.at(dens, i, j) * f->env[(size_t)(i - 1) + (size_t)nr * (k - 1)];
  return 0;
}

}  // extern "C"
