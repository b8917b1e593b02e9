// st_oracle.cpp -- CPU FP64 oracle for the null-geodesic render path.
//
// TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
// CPU baseline leg of bench.py as the checker; never by the product library.
// Every routine below is a double-precision restatement of the SpaceTime.jl
// routine named in its comment (paths relative to the SpaceTime.jl project).
#include "st_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 2.0 * kPi;

inline double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }
inline double sq(double x) { return x * x; }

// ---------------------------------------------------------------------------
// Geodesic right-hand sides in Cartesian Kerr-Schild coordinates.
// ---------------------------------------------------------------------------

// Schwarzschild: src/gr.jl:85-109, src/metal.jl:324-340, src/preview.jl:44-55.
// H = 1/2(-p_t^2 + |p|^2 - f l^2), f = 2M/r, l = -p_t + x.p/r.
inline void rhs_schw(const double* s, double pt, double M, double* d) {
  const double x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const double inv_r = 1.0 / std::sqrt(x * x + y * y + z * z);
  const double f = 2.0 * M * inv_r;
  const double kap = (x * px + y * py + z * pz) * inv_r;
  const double ell = -pt + kap;
  const double c1 = f * ell * inv_r;
  const double c2 = f * ell * (0.5 * ell + kap) * inv_r * inv_r;
  d[0] = px - c1 * x;
  d[1] = py - c1 * y;
  d[2] = pz - c1 * z;
  d[3] = c1 * px - c2 * x;
  d[4] = c1 * py - c2 * y;
  d[5] = c1 * pz - c2 * z;
}

// Kerr-Schild radius from the implicit quartic r^4 - (rho^2 - a^2) r^2 - a^2 z^2 = 0.
inline double ks_r2(double x, double y, double z, double a) {
  const double a2 = a * a;
  const double w = x * x + y * y + z * z - a2;
  return 0.5 * (w + std::sqrt(w * w + 4.0 * a2 * z * z));
}

// Kerr: src/metal.jl:466-508 (the Float32 kernel RHS restated in double).
inline void rhs_kerr(const double* s, double pt, double M, double a, double* d) {
  const double x = s[0], y = s[1], z = s[2], px = s[3], py = s[4], pz = s[5];
  const double a2 = a * a, z2 = z * z;
  double r2 = ks_r2(x, y, z, a);
  r2 = std::max(r2, 1e-12);
  const double r = std::sqrt(r2);
  const double r3 = r2 * r;
  const double inv_sig = 1.0 / (r2 * r2 + a2 * z2);
  const double r2a = r2 + a2;
  const double ira = 1.0 / r2a;
  const double inv_r = 1.0 / r;
  const double Lx = (r * x + a * y) * ira;
  const double Ly = (r * y - a * x) * ira;
  const double Lz = z * inv_r;
  const double ell = -pt + Lx * px + Ly * py + Lz * pz;
  const double f = 2.0 * M * r3 * inv_sig;
  const double fl = f * ell;
  const double drx = x * r3 * inv_sig;
  const double dry = y * r3 * inv_sig;
  const double drz = z * r * r2a * inv_sig;
  const double dfdr = 2.0 * M * r2 * (3.0 * a2 * z2 - r2 * r2) * inv_sig * inv_sig;
  const double dfz0 = -4.0 * M * r3 * a2 * z * inv_sig * inv_sig;
  const double dlx0 = (r * px - a * py) * ira;
  const double dly0 = (a * px + r * py) * ira;
  const double dlz0 = pz * inv_r;
  const double dldr = (px * (x * r2a - 2.0 * r * (r * x + a * y)) +
                       py * (y * r2a - 2.0 * r * (r * y - a * x))) * ira * ira -
                      z * pz * inv_r * inv_r;
  const double hl2 = 0.5 * ell * ell;
  d[0] = px - fl * Lx;
  d[1] = py - fl * Ly;
  d[2] = pz - fl * Lz;
  d[3] = hl2 * (dfdr * drx) + fl * (dldr * drx + dlx0);
  d[4] = hl2 * (dfdr * dry) + fl * (dldr * dry + dly0);
  d[5] = hl2 * (dfdr * drz + dfz0) + fl * (dldr * drz + dlz0);
}

struct Phys {
  double M, a;
  bool kerr;  // the kernel's KERR switch is `a != 0` (src/metal.jl:1847-1848)
  void rhs(const double* s, double pt, double* d) const {
    if (kerr) rhs_kerr(s, pt, M, a, d); else rhs_schw(s, pt, M, d);
  }
};

// ---------------------------------------------------------------------------
// Camera tetrad and photon initialisation: src/preview.jl:93-227.
// ---------------------------------------------------------------------------

struct Tetrad { double u[4], Ef[4], Er[4], Eu[4]; };

void camera_tetrad(const double* pos, const double* fwd, const double* right, const double* up,
                   double M, double a, const double* beta, Tetrad* T) {
  double l[3], f, u[4];
  if (a == 0.0) {
    // static for r >= 2.5M, radial faller dropped from 2.5M inside
    const double r = std::sqrt(sq(pos[0]) + sq(pos[1]) + sq(pos[2]));
    for (int k = 0; k < 3; ++k) l[k] = pos[k] / r;
    f = 2.0 * M / r;
    const double freeze_e2 = 1.0 - 2.0 / 2.5;
    const double E = std::sqrt(std::max(freeze_e2, 1.0 - f));
    const double v = -std::sqrt(std::max(E * E - (1.0 - f), 0.0));
    const double w = (1.0 - E * (E - v)) / (E - v);
    const double lu = E + w;
    u[0] = E + f * lu;
    for (int k = 0; k < 3; ++k) u[k + 1] = (w - f * lu) * l[k];
  } else {
    // static where f <= 0.72, blended to the ZAMO by f = 0.88
    const double x = pos[0], y = pos[1], z = pos[2];
    const double a2 = a * a;
    const double rk2 = ks_r2(x, y, z, a);
    const double rk = std::sqrt(std::max(rk2, 1e-12));
    const double ira = 1.0 / (rk2 + a2);
    l[0] = (rk * x + a * y) * ira;
    l[1] = (rk * y - a * x) * ira;
    l[2] = z / rk;
    const double sig = rk2 * rk2 + a2 * z * z;
    f = 2.0 * M * rk2 * rk / sig;
    const double delta = std::max(rk2 - 2.0 * M * rk + a2, 1e-6);
    const double k = 2.0 * M * rk / delta;
    const double gr[3] = {x * rk2 * rk / sig, y * rk2 * rk / sig, z * rk * (rk2 + a2) / sig};
    const double luc = 1.0 + k * (l[0] * gr[0] + l[1] * gr[1] + l[2] * gr[2]);
    double uz[4];
    uz[0] = 1.0 + f * luc;
    for (int c = 0; c < 3; ++c) uz[c + 1] = k * gr[c] - (f * luc) * l[c];
    const double lu_z = uz[0] + l[0] * uz[1] + l[1] * uz[2] + l[2] * uz[3];
    const double nrm2 = -uz[0] * uz[0] + uz[1] * uz[1] + uz[2] * uz[2] + uz[3] * uz[3] + f * lu_z * lu_z;
    double uzamo[4];
    for (int c = 0; c < 4; ++c) uzamo[c] = uz[c] / std::sqrt(-nrm2);
    if (f >= 0.88) {
      for (int c = 0; c < 4; ++c) u[c] = uzamo[c];
    } else {
      const double ust[4] = {1.0 / std::sqrt(1.0 - f), 0.0, 0.0, 0.0};
      double wb = clampd((f - 0.72) / 0.16, 0.0, 1.0);
      wb = wb * wb * (3.0 - 2.0 * wb);
      if (wb == 0.0) {
        for (int c = 0; c < 4; ++c) u[c] = ust[c];
      } else {
        double um[4];
        for (int c = 0; c < 4; ++c) um[c] = (1.0 - wb) * ust[c] + wb * uzamo[c];
        const double lu = um[0] + l[0] * um[1] + l[1] * um[2] + l[2] * um[3];
        const double nn = -um[0] * um[0] + um[1] * um[1] + um[2] * um[2] + um[3] * um[3] + f * lu * lu;
        for (int c = 0; c < 4; ++c) u[c] = um[c] / std::sqrt(-nn);
      }
    }
  }
  auto ldot = [&](const double* A) { return A[0] + l[0] * A[1] + l[1] * A[2] + l[2] * A[3]; };
  auto gdot = [&](const double* A, const double* B) {
    return -A[0] * B[0] + A[1] * B[1] + A[2] * B[2] + A[3] * B[3] + f * ldot(A) * ldot(B);
  };
  double Ef[4] = {0.0, fwd[0], fwd[1], fwd[2]};
  double Er[4] = {0.0, right[0], right[1], right[2]};
  double Eu[4] = {0.0, up[0], up[1], up[2]};
  double c;
  c = gdot(Ef, u); for (int k = 0; k < 4; ++k) Ef[k] += c * u[k];
  c = std::sqrt(gdot(Ef, Ef)); for (int k = 0; k < 4; ++k) Ef[k] /= c;
  c = gdot(Er, u); for (int k = 0; k < 4; ++k) Er[k] += c * u[k];
  c = gdot(Er, Ef); for (int k = 0; k < 4; ++k) Er[k] -= c * Ef[k];
  c = std::sqrt(gdot(Er, Er)); for (int k = 0; k < 4; ++k) Er[k] /= c;
  c = gdot(Eu, u); for (int k = 0; k < 4; ++k) Eu[k] += c * u[k];
  {
    const double cf = gdot(Eu, Ef), cr = gdot(Eu, Er);
    for (int k = 0; k < 4; ++k) Eu[k] -= cf * Ef[k] + cr * Er[k];
  }
  c = std::sqrt(gdot(Eu, Eu)); for (int k = 0; k < 4; ++k) Eu[k] /= c;

  const double b2raw = beta ? beta[0] * beta[0] + beta[1] * beta[1] + beta[2] * beta[2] : 0.0;
  if (b2raw > 1e-12) {
    const double b2 = std::min(b2raw, 0.9801);
    const double sc = std::sqrt(b2 / b2raw);
    const double b[3] = {beta[0] * sc, beta[1] * sc, beta[2] * sc};
    const double g = 1.0 / std::sqrt(1.0 - b2);
    double bE[4];
    for (int k = 0; k < 4; ++k) bE[k] = b[0] * Ef[k] + b[1] * Er[k] + b[2] * Eu[k];
    const double kk = (g - 1.0) / b2;
    for (int k = 0; k < 4; ++k) {
      const double common = kk * bE[k] + g * u[k];
      T->u[k] = g * (u[k] + bE[k]);
      T->Ef[k] = Ef[k] + b[0] * common;
      T->Er[k] = Er[k] + b[1] * common;
      T->Eu[k] = Eu[k] + b[2] * common;
    }
    return;
  }
  for (int k = 0; k < 4; ++k) { T->u[k] = u[k]; T->Ef[k] = Ef[k]; T->Er[k] = Er[k]; T->Eu[k] = Eu[k]; }
}

// Index lowering p_mu = eta q + f l (l.q): src/metal.jl:971-995, src/preview.jl:221-226.
void lower_photon(const double* x, const double* q, const Phys& P, double* s, double* pt) {
  double l[3], f;
  if (P.kerr) {
    const double a = P.a, a2 = a * a;
    const double rk2 = ks_r2(x[0], x[1], x[2], a);
    const double rk = std::sqrt(std::max(rk2, 1e-12));
    const double ira = 1.0 / (rk2 + a2);
    l[0] = (rk * x[0] + a * x[1]) * ira;
    l[1] = (rk * x[1] - a * x[0]) * ira;
    l[2] = x[2] / rk;
    f = 2.0 * P.M * rk2 * rk / (rk2 * rk2 + a2 * x[2] * x[2]);
  } else {
    const double r = std::sqrt(sq(x[0]) + sq(x[1]) + sq(x[2]));
    for (int k = 0; k < 3; ++k) l[k] = x[k] / r;
    f = 2.0 * P.M / r;
  }
  const double lq = q[0] + l[0] * q[1] + l[1] * q[2] + l[2] * q[3];
  *pt = -q[0] + f * lq;
  for (int k = 0; k < 3; ++k) { s[k] = x[k]; s[k + 3] = q[k + 1] + f * lq * l[k]; }
}

// Integer hash -> [0,1): src/disc_sim.jl:83-91.
inline float sim_hash(int32_t x, int32_t y, int32_t z) {
  uint32_t h = (uint32_t)x * 0x8da6b343u ^ (uint32_t)y * 0xd8163841u ^ (uint32_t)z * 0xcb1ab31fu;
  h ^= h >> 13;
  h *= 0x9e3779b9u;
  h ^= h >> 16;
  return (float)(h & 0x00ffffffu) * 5.9604645e-8f;
}

// ---------------------------------------------------------------------------
// Emission models.
// ---------------------------------------------------------------------------

// ISCO of the prograde equatorial orbit (BPT 1972): src/metal.jl:371-380.
inline double cbrt_clamped(double x) { return std::exp(std::log(std::max(x, 1e-12)) / 3.0); }
void isco(double M, double a, double* r_isco, double* E_isco, double* L_isco) {
  const double q = a / M;
  const double z1 = 1.0 + cbrt_clamped(1.0 - q * q) * (cbrt_clamped(1.0 + q) + cbrt_clamped(1.0 - q));
  const double z2 = std::sqrt(3.0 * q * q + z1 * z1);
  const double r = M * (3.0 + z2 - std::sqrt(std::max((3.0 - z1) * (3.0 + z1 + 2.0 * z2), 0.0)));
  *r_isco = r;
  *E_isco = std::sqrt(1.0 - 2.0 * M / (3.0 * r));
  *L_isco = (2.0 * M / (3.0 * std::sqrt(3.0))) * (1.0 + 2.0 * std::sqrt(3.0 * r / M - 2.0));
}

// Exact emitter shift 1+z = -p.u/E: src/metal.jl:396-428.
double emitter_opz(double sx, double sy, double psx, double psy, double E, double M, double a,
                   double r_isco, double E_isco, double L_isco) {
  const double a2 = a * a;
  const double s2 = sx * sx + sy * sy;
  const double r = std::sqrt(std::max(s2 - a2, 1e-6));
  const double sqM = std::sqrt(M), sqr = std::sqrt(r), r32 = r * sqr;
  const double delta = r * r - 2.0 * M * r + a2;
  double ut, uphi, ur = 0.0;
  if (r >= r_isco) {
    const double den = r32 - 3.0 * M * sqr + 2.0 * a * sqM;
    ut = (r32 + a * sqM) / (std::sqrt(r32) * std::sqrt(std::max(den, 1e-2)));
    uphi = sqM / (r32 + a * sqM) * ut;
  } else {
    const double inv_d = 1.0 / std::max(delta, 1e-3);
    ut = ((r * r + a2 + 2.0 * M * a2 / r) * E_isco - 2.0 * M * a * L_isco / r) * inv_d;
    uphi = (2.0 * M * a * E_isco / r + (1.0 - 2.0 * M / r) * L_isco) * inv_d;
    const double Rr = sq(E_isco * (r * r + a2) - a * L_isco) - delta * (r * r + sq(L_isco - a * E_isco));
    ur = -std::sqrt(std::max(Rr, 0.0)) / (r * r);
    ut += 2.0 * M * r * inv_d * ur;
    uphi += a * inv_d * ur;
  }
  const double inv_s2 = 1.0 / std::max(s2, 1e-6);
  const double cphi = (r * sx + a * sy) * inv_s2;
  const double sphi = (r * sy - a * sx) * inv_s2;
  const double ux = ur * cphi - sy * uphi;
  const double uy = ur * sphi + sx * uphi;
  const double Es = std::fabs(E) > 1e-6 ? E : 1e-6;
  return clampd(ut - (psx * ux + psy * uy) / Es, 0.1, 20.0);
}

// CIE-fit blackbody colour: src/blackbody.jl:5-35.
inline double cie_gauss(double lam, double mu, double s1, double s2) {
  const double s = lam < mu ? s1 : s2;
  return std::exp(-0.5 * sq((lam - mu) / s));
}
void blackbody_rgb(double T, double* rgb) {
  double X = 0, Y = 0, Z = 0;
  for (int i = 0; i <= 80; ++i) {
    const double lam = 380.0 + 5.0 * i;
    const double lm = lam * 1e-9;
    const double B = 1.0 / (std::pow(lm, 5) * (std::exp(0.014388 / (lm * T)) - 1.0));
    const double xb = 1.056 * cie_gauss(lam, 599.8, 37.9, 31.0) + 0.362 * cie_gauss(lam, 442.0, 16.0, 26.7) -
                      0.065 * cie_gauss(lam, 501.1, 20.4, 26.2);
    const double yb = 0.821 * cie_gauss(lam, 568.8, 46.9, 40.5) + 0.286 * cie_gauss(lam, 530.9, 16.3, 31.1);
    const double zb = 1.217 * cie_gauss(lam, 437.0, 11.8, 36.0) + 0.681 * cie_gauss(lam, 459.0, 26.0, 13.8);
    X += B * xb; Y += B * yb; Z += B * zb;
  }
  const double r = std::max(3.2406 * X - 1.5372 * Y - 0.4986 * Z, 0.0);
  const double g = std::max(-0.9689 * X + 1.8758 * Y + 0.0415 * Z, 0.0);
  const double b = std::max(0.0557 * X - 0.2040 * Y + 1.0570 * Z, 0.0);
  const double m = std::max(std::max(r, g), std::max(b, 1e-10));
  rgb[0] = r / m; rgb[1] = g / m; rgb[2] = b / m;
}

struct Scene {
  const orc_scene* s;
  Phys P;
  Tetrad T;
  double rkill2;       // (0.995 r_ph)^2, src/metal.jl:347-357
  double r_isco, E_isco, L_isco;
  double hcoef, hcap;
  bool draft, tsit5, disc_on, vol_on, kepler;
  int ksteps;  // 0, or 45 / 46: the kernel's adaptive twin
  double ds_gas, vol_rb2;
  int nmax;
  const double* dirs = nullptr;  // orc_trace_dirs: (cf, cr, cu) per ray instead of pixels
};

// LUT colour. RENDER rounds half to even (Julia `round`, src/blackbody.jl:78);
// DRAFT truncates frac*(N-1)+0.5 (src/metal.jl:1539).
inline void lut_color(const Scene& S, double T, bool render_rule, double* col) {
  const orc_scene* s = S.s;
  const double fr = (clampd(T, s->lut_tmin, s->lut_tmax) - s->lut_tmin) / (s->lut_tmax - s->lut_tmin);
  int idx;
  if (render_rule) idx = (int)std::nearbyint(fr * (s->lut_size - 1));
  else idx = (int)(fr * (s->lut_size - 1.0) + 0.5);
  idx = std::min(std::max(idx, 0), s->lut_size - 1);
  for (int c = 0; c < 3; ++c) col[c] = s->bb_lut[3 * idx + c];
}

// Thin-disc Keplerian Planck-Doppler shading of the CPU renderer:
// src/accretion_disc.jl:19-49 and the opacity model of src/callbacks.jl:49-90.
// X: crossing position (z = 0), P: covariant momentum there.
double disc_kepler(const Scene& S, const double* X, const double* Pm, double pt, double gcam,
                   double* acc, double* alpha) {
  const double M = S.P.M;
  const double r = std::sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
  const orc_scene* s = S.s;
  if (!(s->disc_inner < r && r < s->disc_outer)) return 0.0;
  const double f = 2.0 * M / r;
  const double kap = (X[0] * Pm[0] + X[1] * Pm[1] + X[2] * Pm[2]) / r;
  const double c1 = f * (-pt + kap) / r;
  double pc[3];
  for (int k = 0; k < 3; ++k) pc[k] = Pm[k] - c1 * X[k];
  const double R = r / (2.0 * M);
  const double T_emit = std::exp(10.034259 - 0.375 * std::log(R * R));
  double vmag = 0.70710678 * std::pow(std::max(R - 1.0, 0.1), -0.5);
  vmag = clampd(vmag, 0.0, 0.999);
  const double npos[3] = {X[0] / r, X[1] / r, X[2] / r};
  const double dv[3] = {-vmag * npos[1], vmag * npos[0], 0.0};
  const double vsq = clampd(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2], 0.0, 0.99);
  const double gam = 1.0 / std::sqrt(1.0 - vsq);
  const double pn = std::sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
  const double opz_d = gam * (1.0 + (dv[0] * pc[0] + dv[1] * pc[1] + dv[2] * pc[2]) / pn);
  const double opz_g = 1.0 / std::sqrt(std::max(1.0 - 1.0 / std::max(R, 1.0), 0.01));
  const double T_obs = T_emit * gcam / std::max(opz_d * opz_g, 0.1);
  const double inten = 100.0 / (std::exp(29622.4 / std::max(T_obs, 1.0)) - 1.0);
  double col[3];
  lut_color(S, T_obs, true, col);
  const double R_in = s->disc_inner / (2.0 * M), R_out = s->disc_outer / (2.0 * M);
  const double iscotaper = clampd((R * R - R_in * R_in) * 0.3, 0.0, 1.0);
  const double outertaper = clampd(T_emit / 1000.0, 0.0, 1.0);
  const double dens = clampd((R_out - R) / (R_out - R_in), 0.0, 1.0);
  const double dpow = (s->disc_falloff == 0.0) ? 1.0 : std::pow(dens, s->disc_falloff);
  const double op = iscotaper * outertaper * dpow;
  for (int c = 0; c < 3; ++c) acc[c] += inten * col[c] * (*alpha * op);
  *alpha *= (1.0 - op);
  return T_obs / T_emit;
}

// Thin-disc exact-emitter shading of the kernel: src/metal.jl:1522-1570.
double disc_exact(const Scene& S, double xh, double yh, double pxh, double pyh, double pt, double scam,
                  double* acc, double* alpha) {
  const orc_scene* s = S.s;
  const double M = S.P.M;
  const double sc = std::sqrt(xh * xh + yh * yh);
  if (!(s->disc_inner < sc && sc < s->disc_outer)) return 0.0;
  const double R = sc / (2.0 * M);
  const double RT = std::max(sc, S.r_isco) / (2.0 * M);
  const double T_emit = std::exp(10.034259 - 0.375 * std::log(RT * RT));
  const double plunge = sc < S.r_isco ? std::pow(sc / S.r_isco, 3) : 1.0;
  const double opz = emitter_opz(xh, yh, pxh, pyh, -pt, M, S.P.a, S.r_isco, S.E_isco, S.L_isco);
  const double T_obs = T_emit * scam / opz;
  const double inten = 100.0 / (std::exp(29622.4 / std::max(T_obs, 1.0)) - 1.0);
  double col[3];
  lut_color(S, T_obs, false, col);
  const double R_in = s->disc_inner / (2.0 * M), R_out = s->disc_outer / (2.0 * M);
  const double iscotaper = clampd((R * R - R_in * R_in) * 0.3, 0.0, 1.0);
  const double outertaper = clampd(T_emit / 1000.0, 0.0, 1.0);
  const double dens = clampd((R_out - R) / (R_out - R_in), 0.0, 1.0);
  const double dpow = dens <= 1e-6 ? (s->disc_falloff > 0.0 ? 0.0 : 1.0)
                                   : std::exp(s->disc_falloff * std::log(dens));
  const double op = iscotaper * outertaper * dpow * plunge;
  const double w = *alpha * op * inten;
  for (int c = 0; c < 3; ++c) acc[c] += w * col[c];
  *alpha *= (1.0 - op);
  return T_obs / T_emit;
}

// Trilinear gas density: src/metal.jl:569-610 / src/disc_volume.jl:486-509.
double sample_volume(const orc_scene* s, double sc, double phi, double z) {
  const double zmax = s->vol_zmax;
  if (sc <= 0.0 || std::fabs(z) >= zmax) return 0.0;
  const double ls = std::log(sc);
  if (ls <= s->vol_ls_in || ls >= s->vol_ls_out) return 0.0;
  const int nr = s->nr, nphi = s->nphi, nz = s->nz;
  const double fr = (ls - s->vol_ls_in) / (s->vol_ls_out - s->vol_ls_in) * (nr - 1);
  double pm = std::fmod(phi, kTwoPi);
  if (pm < 0) pm += kTwoPi;
  const double fp = pm / kTwoPi * nphi;
  const double fz = (z + zmax) / (2.0 * zmax) * (nz - 1);
  const int i0 = std::min(std::max((int)std::floor(fr), 0), nr - 2);
  const double tr = fr - i0;
  const int j0 = (int)std::floor(fp);
  const double tp = fp - j0;
  const int k0 = std::min(std::max((int)std::floor(fz), 0), nz - 2);
  const double tz = fz - k0;
  const int ja = ((j0 % nphi) + nphi) % nphi, jb = (((j0 + 1) % nphi) + nphi) % nphi;
  auto D = [&](int i, int j, int k) { return (double)s->vol[i + (size_t)nr * (j + (size_t)nphi * k)]; };
  const double c00 = D(i0, ja, k0) + tr * (D(i0 + 1, ja, k0) - D(i0, ja, k0));
  const double c10 = D(i0, jb, k0) + tr * (D(i0 + 1, jb, k0) - D(i0, jb, k0));
  const double c01 = D(i0, ja, k0 + 1) + tr * (D(i0 + 1, ja, k0 + 1) - D(i0, ja, k0 + 1));
  const double c11 = D(i0, jb, k0 + 1) + tr * (D(i0 + 1, jb, k0 + 1) - D(i0, jb, k0 + 1));
  const double c0 = c00 + tp * (c10 - c00);
  const double c1 = c01 + tp * (c11 - c01);
  return c0 + tz * (c1 - c0);
}

// Bilinear equirectangular sky, first index phi: src/raytrace.jl:154-177,
// src/metal.jl:523-561 (the same arithmetic in 0-based form).
void sample_sky(const orc_scene* s, double theta, double phi, double* rgb) {
  const int W = s->sky_w, H = s->sky_h;
  const double v = clampd(theta / kPi, 0.0, 1.0);
  double pm = std::fmod(phi, kTwoPi);
  if (pm < 0) pm += kTwoPi;
  const double u = clampd(pm / kTwoPi, 0.0, 1.0);
  const double xf = u * (W - 1), yf = v * (H - 1);
  const int x0 = std::min(std::max((int)std::floor(xf), 0), W - 1);
  const int x1 = std::min(x0 + 1, W - 1);
  const int y0 = std::min(std::max((int)std::floor(yf), 0), H - 1);
  const int y1 = std::min(y0 + 1, H - 1);
  const double fx = xf - x0, fy = yf - y0;
  const double w00 = (1 - fx) * (1 - fy), w10 = fx * (1 - fy), w01 = (1 - fx) * fy, w11 = fx * fy;
  for (int c = 0; c < 3; ++c) {
    auto T = [&](int x, int y) { return (double)s->sky[c + 3 * (x + (size_t)W * y)]; };
    rgb[c] = T(x0, y0) * w00 + T(x1, y0) * w10 + T(x0, y1) * w01 + T(x1, y1) * w11;
  }
}

// Relativistic sky tint: src/raytrace.jl:53-58, src/metal.jl:1679-1686.
void sky_tint(double g, double* rgb) {
  if (g == 1.0) return;
  rgb[0] *= 57.4 / (std::exp(4.067 / g) - 1.0);
  rgb[1] *= 90.2 / (std::exp(4.513 / g) - 1.0);
  rgb[2] *= 206.5 / (std::exp(5.335 / g) - 1.0);
}

// ---------------------------------------------------------------------------
// Integrator steps.
// ---------------------------------------------------------------------------

void rk4_step(const Phys& P, const double* y, double pt, double h, const double* k1, double* out) {
  double k2[6], k3[6], k4[6], t[6];
  for (int i = 0; i < 6; ++i) t[i] = y[i] + 0.5 * h * k1[i];
  P.rhs(t, pt, k2);
  for (int i = 0; i < 6; ++i) t[i] = y[i] + 0.5 * h * k2[i];
  P.rhs(t, pt, k3);
  for (int i = 0; i < 6; ++i) t[i] = y[i] + h * k3[i];
  P.rhs(t, pt, k4);
  for (int i = 0; i < 6; ++i) out[i] = y[i] + (h / 6.0) * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
}

// Tsitouras (2011) 5(4) pair, FSAL; coefficients from the published tableau.
constexpr double TA21 = 0.161;
constexpr double TA31 = -0.008480655492356989, TA32 = 0.335480655492357;
constexpr double TA41 = 2.897153057105493, TA42 = -6.359448489975075, TA43 = 4.3622954328695815;
constexpr double TA51 = 5.325864828439257, TA52 = -11.748883564062828, TA53 = 7.4955393428898365,
                 TA54 = -0.09249506636175525;
constexpr double TA61 = 5.86145544294642, TA62 = -12.92096931784711, TA63 = 8.159367898576159,
                 TA64 = -0.071584973281401, TA65 = -0.028269050394068383;
constexpr double TB1 = 0.09646076681806523, TB2 = 0.01, TB3 = 0.4798896504144996, TB4 = 1.379008574103742,
                 TB5 = -3.290069515436081, TB6 = 2.324710524099774;
constexpr double TE1 = -0.00178001105222577714, TE2 = -0.0008164344596567469, TE3 = 0.007880878010261995,
                 TE4 = -0.1447110071732629, TE5 = 0.5823571654525552, TE6 = -0.45808210592918697,
                 TE7 = 0.015151515151515152;

// One Tsit5 step of size h from y with first stage k1; writes the 5th-order
// solution, its slope (FSAL) and the embedded error vector.
void tsit5_step(const Phys& P, const double* y, double pt, double h, const double* k1, double* yn,
                double* k7, double* err) {
  double k2[6], k3[6], k4[6], k5[6], k6[6], t[6];
  for (int i = 0; i < 6; ++i) t[i] = y[i] + h * (TA21 * k1[i]);
  P.rhs(t, pt, k2);
  for (int i = 0; i < 6; ++i) t[i] = y[i] + h * (TA31 * k1[i] + TA32 * k2[i]);
  P.rhs(t, pt, k3);
  for (int i = 0; i < 6; ++i) t[i] = y[i] + h * (TA41 * k1[i] + TA42 * k2[i] + TA43 * k3[i]);
  P.rhs(t, pt, k4);
  for (int i = 0; i < 6; ++i) t[i] = y[i] + h * (TA51 * k1[i] + TA52 * k2[i] + TA53 * k3[i] + TA54 * k4[i]);
  P.rhs(t, pt, k5);
  for (int i = 0; i < 6; ++i)
    t[i] = y[i] + h * (TA61 * k1[i] + TA62 * k2[i] + TA63 * k3[i] + TA64 * k4[i] + TA65 * k5[i]);
  P.rhs(t, pt, k6);
  for (int i = 0; i < 6; ++i)
    yn[i] = y[i] + h * (TB1 * k1[i] + TB2 * k2[i] + TB3 * k3[i] + TB4 * k4[i] + TB5 * k5[i] + TB6 * k6[i]);
  P.rhs(yn, pt, k7);
  for (int i = 0; i < 6; ++i)
    err[i] = h * (TE1 * k1[i] + TE2 * k2[i] + TE3 * k3[i] + TE4 * k4[i] + TE5 * k5[i] + TE6 * k6[i] + TE7 * k7[i]);
}

inline double rnorm(const double* s) { return std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]); }

// ---------------------------------------------------------------------------
// Per-ray trace.
// ---------------------------------------------------------------------------

struct RayOut {
  double rgb[3];
  orc_ray rec;
};

// Radius-adaptive step: src/metal.jl:1250-1260.
inline double step_rule(const Scene& S, const double* y, double r2, double rk2) {
  const double r = std::sqrt(r2);
  const double cap = (S.vol_on && r2 < S.vol_rb2) ? 2.0 : S.hcap;
  double h = S.s->dt * std::min(std::max(S.hcoef * r / S.P.M, 1.0), cap);
  if (S.P.kerr) {
    const double fr = clampd((rk2 - S.rkill2) / std::max(S.rkill2, 1e-6), 0.0, 1.0);
    h *= 0.12 + 0.88 * fr;
  }
  (void)y;
  return h;
}

// Gas march over one accepted step (DRAFT): src/metal.jl:1429-1513.
// Returns true when the transmittance is exhausted.
bool march_gas(const Scene& S, const double* yp, const double* yn, double pt, double h_used, double vlen,
               double r2p, double scam, double* march_acc, double* acc, double* alpha) {
  const orc_scene* s = S.s;
  const double r2n = yn[0] * yn[0] + yn[1] * yn[1] + yn[2] * yn[2];
  if (!(*alpha > 0.003 && std::min(r2p, r2n) < S.vol_rb2)) return false;
  const double seg = h_used * vlen;
  if (!(seg < 64.0)) return false;
  double t_s = S.ds_gas - *march_acc;
  if (t_s > seg) { *march_acc += seg; return false; }
  for (int guard = 0; guard < 8192 && t_s <= seg && *alpha > 0.003; ++guard) {
    const double fs = t_s / seg;
    const double sx = yp[0] + fs * (yn[0] - yp[0]);
    const double sy = yp[1] + fs * (yn[1] - yp[1]);
    const double sz = yp[2] + fs * (yn[2] - yp[2]);
    if (std::fabs(sz) < s->vol_zmax) {
      const double scyl = std::sqrt(sx * sx + sy * sy);
      if (scyl > 1e-6) {
        const double phi = std::atan2(sy, sx);
        double rho = sample_volume(s, scyl, phi, sz);
        if (rho > 1e-4) {
          const double R = std::max(scyl, S.r_isco) / (2.0 * S.P.M);
          const double T_emit = std::exp(10.034259 - 0.375 * std::log(std::max(R * R, 1e-6)));
          if (scyl < S.r_isco) rho *= std::pow(scyl / S.r_isco, 3);
          const double psx = yp[3] + fs * (yn[3] - yp[3]);
          const double psy = yp[4] + fs * (yn[4] - yp[4]);
          const double opz = emitter_opz(sx, sy, psx, psy, -pt, S.P.M, S.P.a, S.r_isco, S.E_isco, S.L_isco);
          const double T_obs = T_emit * scam / opz;
          const double inten = 100.0 / (std::exp(29622.4 / std::max(T_obs, 1.0)) - 1.0);
          double col[3];
          lut_color(S, T_obs, false, col);
          const double tau = s->vol_opac * rho * S.ds_gas;
          const double aa = 1.0 - std::exp(-tau);
          const double w = *alpha * aa * inten * s->vol_emis;
          for (int c = 0; c < 3; ++c) acc[c] += w * col[c];
          *alpha *= (1.0 - aa);
        }
      }
    }
    t_s += S.ds_gas;
  }
  *march_acc = seg - (t_s - S.ds_gas);
  return *alpha < 0.003;
}

// Bardeen launch-time capture test (Kerr): src/metal.jl:1026-1094.
void bardeen(const Scene& S, const double* y, double pt, bool* captured0, bool* graze0) {
  *captured0 = false; *graze0 = false;
  const double a = S.P.a, M = S.P.M;
  if (!(S.P.kerr && a != 0.0)) return;
  const double E0 = -pt;
  if (!(std::fabs(E0) > 1e-6)) return;
  const double x = y[0], yy = y[1], z = y[2], px = y[3], py = y[4], pz = y[5];
  const double a2 = a * a;
  const double rk2 = ks_r2(x, yy, z, a);
  const double rk = std::sqrt(std::max(rk2, 1e-12));
  const double cth = z / rk;
  const double s2 = std::max(1.0 - cth * cth, 1e-8);
  const double sth = std::sqrt(s2);
  const double Lz0 = x * py - yy * px;
  const double pth = (cth / sth) * (x * px + yy * py) - rk * sth * pz;
  const double Q0 = pth * pth + cth * cth * (Lz0 * Lz0 / s2 - a2 * E0 * E0);
  const double lam = Lz0 / E0, eta = Q0 / (E0 * E0);
  const double c2 = a2 - lam * lam - eta;
  const double c1 = 2.0 * M * (eta + (lam - a) * (lam - a));
  const double c0 = -a2 * eta;
  const double rplus = M + std::sqrt(std::max(M * M - a2, 0.0));
  double v[6];
  rhs_kerr(y, pt, M, a, v);
  const double rdot = rk2 * (x * v[0] + yy * v[1]) + (rk2 + a2) * z * v[2];
  if (!(rdot < 0.0)) return;
  const double pb = 0.5 * c2, qb = 0.25 * c1;
  const double Db = 0.25 * qb * qb + pb * pb * pb / 27.0;
  bool cap = true;
  auto sgn = [](double t) { return t > 0 ? 1.0 : (t < 0 ? -1.0 : 0.0); };
  if (Db >= 0.0) {
    const double sD = std::sqrt(Db);
    const double u1 = -0.5 * qb + sD, u2 = -0.5 * qb - sD;
    const double rc = sgn(u1) * std::exp(std::log(std::max(std::fabs(u1), 1e-30)) / 3.0) +
                      sgn(u2) * std::exp(std::log(std::max(std::fabs(u2), 1e-30)) / 3.0);
    if (rc > rplus && rc < rk) {
      const double Rv = ((rc * rc + c2) * rc + c1) * rc + c0;
      cap = Rv > 0.0;
      if (std::fabs(Rv) < 0.08 * std::max(rc * rc * rc * rc, 1.0)) *graze0 = true;
    }
  } else {
    const double mb = 2.0 * std::sqrt(-pb / 3.0);
    const double ac = clampd(3.0 * qb / (pb * mb), -1.0, 1.0);
    const double tb = std::acos(ac) / 3.0;
    for (int kk = 0; kk < 3; ++kk) {
      const double rc = mb * std::cos(tb - 2.0943951023931953 * kk);
      if (rc > rplus && rc < rk) {
        const double Rv = ((rc * rc + c2) * rc + c1) * rc + c0;
        if (Rv <= 0.0) cap = false;
        if (std::fabs(Rv) < 0.08 * std::max(rc * rc * rc * rc, 1.0)) *graze0 = true;
      }
    }
  }
  *captured0 = cap;
}

// Secant (Illinois) on the step size h in (0, h1] for g(step(y0, h)) = 0,
// each trial a fresh step from y0 of the integrator in use.
template <class StepFn, class G>
void locate(StepFn step, G g, double g0, double g1, double h1, double* yout) {
  double ha = 0.0, ga = g0, hb = h1, gb = g1;
  int side = 0;
  double hc = h1;
  for (int it = 0; it < 60; ++it) {
    hc = (ha * gb - hb * ga) / (gb - ga);
    if (!(hc > ha && hc < hb)) hc = 0.5 * (ha + hb);
    step(hc, yout);
    const double gc = g(yout);
    if (gc == 0.0 || (hb - ha) < 1e-15 * h1) break;
    if ((gc > 0) == (gb > 0)) {
      hb = hc; gb = gc;
      if (side == -1) ga *= 0.5;
      side = -1;
    } else {
      ha = hc; ga = gc;
      if (side == 1) gb *= 0.5;
      side = 1;
    }
    if (std::fabs(gc) < 1e-14) break;
  }
}

// Procedural stars along unit direction d (starfield_mtl, src/metal.jl:652-724;
// starfield_color, src/starfield.jl:83-150): the direction's lattice cell on a
// star_N x star_N grid of (u = atan2(y,x)/2pi + 1/2, v = (z+1)/2) and its eight
// neighbours; a star per cell at a hashed point, kept with probability
// fill exp(-|n.s| concentration), flux xi^(-2/3), Gaussian PSF, colour from the
// star table (DRAFT index rounds half up, RENDER to nearest even).
void star_light(const orc_scene* s, bool draft, double dx, double dy, double dz, double* rgb) {
  const double N = s->star_N;
  const int Ni = (int)s->star_N;
  const double two_pi = 2.0 * kPi;
  const double u = std::atan2(dy, dx) / two_pi + 0.5;
  const double v = (dz + 1.0) * 0.5;
  const int i0 = (int)std::floor(u * N), j0 = (int)std::floor(v * N);
  const double sig = s->star_sigma;
  const double inv2s2 = 1.0 / (2.0 * sig * sig), cut = 25.0 * sig * sig;
  const int n = s->star_lut_size, seed = s->star_seed;
  double ar = 0.0, ag = 0.0, ab = 0.0;
  for (int dj = -1; dj <= 1; ++dj) {
    const int jj = j0 + dj;
    if (jj < 0 || jj >= Ni) continue;
    for (int di = -1; di <= 1; ++di) {
      int ii = (i0 + di) % Ni;
      if (ii < 0) ii += Ni;
      const double su = sim_hash(ii, jj, seed + 1), sv = sim_hash(ii, jj, seed + 2);
      const double phs = ((ii + su) / N - 0.5) * two_pi;
      const double sz = 2.0 * (jj + sv) / N - 1.0;
      const double sr = std::sqrt(std::max(1.0 - sz * sz, 0.0));
      const double sx = sr * std::cos(phs), sy = sr * std::sin(phs);
      const double ex = dx - sx, ey = dy - sy, ez = dz - sz;
      const double d2 = ex * ex + ey * ey + ez * ez;
      if (d2 > cut) continue;
      double occ = s->star_fill;
      if (s->star_conc > 0.0)
        occ *= std::exp(-std::fabs(sx * s->star_g[0] + sy * s->star_g[1] + sz * s->star_g[2]) * s->star_conc);
      if (!((double)sim_hash(ii, jj, seed) < occ)) continue;
      const double xi = std::max((double)sim_hash(ii, jj, seed + 3), (double)1e-4f);
      const double w = s->star_flux * std::exp((double)-0.6666667f * std::log(xi)) * std::exp(-d2 * inv2s2);
      const double T = s->star_tmin + s->star_tspan * (double)sim_hash(ii, jj, seed + 4);
      const double lt0 = s->star_lut_tmin, lt1 = s->star_lut_tmax;
      const double frac = (clampd(T, lt0, lt1) - lt0) / std::max(lt1 - lt0, 1e-6);
      int li = draft ? (int)(frac * (n - 1) + 0.5) : (int)std::nearbyint(frac * (n - 1));
      li = std::min(std::max(li, 0), n - 1);
      ar += w * s->star_lut[3 * li];
      ag += w * s->star_lut[3 * li + 1];
      ab += w * s->star_lut[3 * li + 2];
    }
  }
  rgb[0] = ar; rgb[1] = ag; rgb[2] = ab;
}

// Depth bucket of path length ell, 1-based (src/metal.jl:1489-1492): bucket 1
// below 1.5 M, then trunc((ln ell - ln 1.5) (nb - 2) 0.22820) + 1 clamped to
// [1, nb - 1]; bucket nb is the sky's.
int depth_bucket(double ell, int nb) {
  if (ell <= 1.5) return 1;
  const double bscale = nb > 2 ? (nb - 2) * 0.22820 : 1.0;
  const int b = (int)((std::log(ell) - 0.405465) * bscale) + 1;
  return std::min(std::max(b, 1), nb - 1);
}

// bk (3 nb doubles, may be null): depth-bucket mode; emission is moved into
// bk as it happens and the sky (times the transmittance) into the last bucket
// (src/metal.jl:1170-1175, 1425-1426, 1489-1497, 1556-1563, 1687-1690).
void trace_ray(const Scene& S, int i0, int j0, RayOut* ro, double* bk = nullptr, int nb = 0) {
  const orc_scene* s = S.s;
  const Phys& P = S.P;
  const double M = P.M;
  orc_ray& rec = ro->rec;
  std::memset(&rec, 0, sizeof(rec));
  rec.r_cross = -1.0;
  const int i1 = i0 + 1, j1 = j0 + 1;  // 1-based pixel indices, as hashed by the reference

  // Sensor coordinate (GPU convention, src/metal.jl:863-872).
  double ju = s->ju, jv = s->jv;
  if (s->jitter_w > 0.0) {
    ju += (double)sim_hash(i1, j1, s->jitter_seed) * s->jitter_w;
    jv += (double)sim_hash(i1, j1, s->jitter_seed + 271) * s->jitter_w;
  }
  const double half_h = s->height / 2.0;
  const double u = (i1 - 1.0 + ju - s->width / 2.0) / half_h;
  const double v = (j1 - 1.0 + jv - s->height / 2.0) / half_h;

  // Thin-lens stratum point, concentric map (src/metal.jl:881-903).
  double offr = 0.0, offu = 0.0;
  if (s->lens_w > 0.0 && s->aperture_radius > 0.0) {
    const double u01 = s->lens_u0 + (double)sim_hash(i1, j1, s->lens_seed) * s->lens_w;
    const double v01 = s->lens_v0 + (double)sim_hash(i1, j1, s->lens_seed + 7919) * s->lens_w;
    const double ox = 2.0 * u01 - 1.0, oy = 2.0 * v01 - 1.0;
    if (ox != 0.0 || oy != 0.0) {
      double rr, th;
      if (std::fabs(ox) > std::fabs(oy)) { rr = ox; th = (kPi / 4) * (oy / ox); }
      else { rr = oy; th = kPi / 2 - (kPi / 4) * (ox / oy); }
      offr = s->aperture_radius * rr * std::cos(th);
      offu = s->aperture_radius * rr * std::sin(th);
    }
  }
  // Projection (src/metal.jl:907-949).
  double cf, cr, cu;
  if (s->projection == 1) {
    const double rho = std::sqrt(u * u + v * v);
    const double tp = rho * s->fisheye_rad;
    const double st = std::sin(tp);
    const double ir = rho > 1e-8 ? 1.0 / rho : 0.0;
    cr = st * u * ir; cu = st * v * ir; cf = std::cos(tp);
  } else {
    double dxl = u * s->fov, dyl = v * s->fov;
    double nu = std::sqrt(dxl * dxl + dyl * dyl + 1.0);
    if (offr != 0.0 || offu != 0.0) {
      const double k = nu / s->focus_dist;
      dxl -= offr * k; dyl -= offu * k;
      nu = std::sqrt(dxl * dxl + dyl * dyl + 1.0);
    }
    cr = dxl / nu; cu = dyl / nu; cf = 1.0 / nu;
  }
  if (S.dirs) {  // a given camera-frame direction (orc_trace_dirs), no lens offset
    cf = S.dirs[3 * (size_t)i0]; cr = S.dirs[3 * (size_t)i0 + 1]; cu = S.dirs[3 * (size_t)i0 + 2];
    offr = offu = 0.0;
  }
  // Per-pixel shutter: the pose moves toward the stratum's end pose by a
  // hashed fraction of the way (src/metal.jl:843-857).
  Tetrad T = S.T;
  double cpos[3] = {s->pos[0], s->pos[1], s->pos[2]};
  if (s->shutter_seed > 0) {
    const double tau = (double)sim_hash(i1, j1, s->shutter_seed);
    for (int k = 0; k < 3; ++k) cpos[k] += tau * (s->pos_end[k] - cpos[k]);
    for (int k = 0; k < 4; ++k) {
      T.Ef[k] += tau * (s->Ef_end[k] - T.Ef[k]);
      T.Er[k] += tau * (s->Er_end[k] - T.Er[k]);
      T.Eu[k] += tau * (s->Eu_end[k] - T.Eu[k]);
      T.u[k] += tau * (s->u_end[k] - T.u[k]);
    }
  }
  double origin[3], q[4];
  for (int k = 0; k < 3; ++k) origin[k] = cpos[k] + offr * T.Er[k + 1] + offu * T.Eu[k + 1];
  for (int k = 0; k < 4; ++k) q[k] = cf * T.Ef[k] + cr * T.Er[k] + cu * T.Eu[k] - T.u[k];
  double y[6], pt;
  lower_photon(origin, q, P, y, &pt);
  const double gshift = 1.0 / clampd(std::fabs(pt), 0.05, 20.0);
  const double scam = s->relativistic ? gshift : 1.0;

  bool captured0 = false, graze0 = false;
  if (S.draft) bardeen(S, y, pt, &captured0, &graze0);
  if (captured0) rec.flags |= ORC_RAY_BCAPT;
  if (graze0) rec.flags |= ORC_RAY_GRAZE;

  double acc[3] = {0, 0, 0}, alpha = 1.0;
  const double r_start = rnorm(y);
  const double r_floor = r_start > 2.05 * M ? 2.0 * M : 0.3 * M;
  double r_prev = -1.0;
  double march_acc = 0.0;
  bool hit = false, escaped = false, budget = true;
  double lambda = 0.0;
  double ell = 0.0;  // depth buckets: path length
  auto flush_bucket = [&]() {
    if (!bk) return;
    double* b = bk + 3 * (depth_bucket(ell, nb) - 1);
    for (int c = 0; c < 3; ++c) { b[c] += acc[c]; acc[c] = 0.0; }
  };
  double k1[6];
  P.rhs(y, pt, k1);
  int rhs_evals = 1;
  int steps = 0;
  double h_carry = -1.0;
  double kerr_prev = 1e-4;   // kernel twin: previous accepted error (PI)
  // RENDER boundary function (r - 2.00001)(r_max - r) and its sign at launch
  auto gb = [&](const double* st) { const double r = rnorm(st); return (r - 2.00001) * (s->r_escape - r); };
  const double gb0 = gb(y);
  const int max_steps = S.tsit5 ? 8 * S.nmax : S.nmax;

  auto disc_event = [&](const double* ye, double pm_t) {
    // shading at a crossing state ye (z ~ 0); records the first annulus hit
    double g;
    if (S.kepler) {
      const double X[3] = {ye[0], ye[1], 0.0};
      g = disc_kepler(S, X, ye + 3, pm_t, scam, acc, &alpha);
    } else {
      g = disc_exact(S, ye[0], ye[1], ye[3], ye[4], pm_t, scam, acc, &alpha);
    }
    if (g > 0.0 && rec.r_cross < 0.0) {
      rec.r_cross = std::sqrt(ye[0] * ye[0] + ye[1] * ye[1]);
      rec.g_cross = g;
      rec.flags |= ORC_RAY_CROSSED;
    }
  };

  for (int step = 0; step < max_steps; ++step) {
    const double r2 = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
    const double r = std::sqrt(r2);
    double rk2 = r2;
    if (S.draft) {
      if (P.kerr) {
        rk2 = ks_r2(y[0], y[1], y[2], P.a);
        if (rk2 < S.rkill2) { hit = true; budget = false; break; }
      } else if (r < 3.2 * M) {
        if (r < r_floor || (r < 2.95 * M && r_prev > 0.0 && r < r_prev - 1e-4 * M)) {
          hit = true; budget = false; break;
        }
        r_prev = r;
      }
      if (r > s->r_escape) { escaped = true; budget = false; break; }
    } else {
      if (r >= s->r_escape) { escaped = true; budget = false; break; }
      if (lambda >= s->tspan) break;
      // Fixed-step twin only: a ray moving inward below 2.95M never escapes
      // (escaping rays have periapsis > 3M); in ingoing KS coordinates the
      // backward ray approaches the past horizon only asymptotically, which a
      // fixed step cannot follow, so it is ended here as horizon-bound.
      if (!S.tsit5 && r < 2.95 * M && r_prev > 0.0 && r < r_prev - 1e-4 * M) {
        hit = true; budget = false; break;
      }
      r_prev = r;
    }
    double h = step_rule(S, y, r2, rk2);
    if (!S.draft) h = std::min(h, s->tspan - lambda);

    double yn[6], kn[6];
    double h_used = h;
    if (S.ksteps) {
      // src/metal.jl:1278-1381 restated in double
      double hmax = h;
      if (S.ksteps == 46) {
        hmax = 50.0 * s->dt;
        if (S.disc_on && !S.vol_on) hmax = std::min(hmax, std::max(h, 0.5 * (r - s->disc_outer)));
      }
      double hh = std::min(h_carry > 0.0 ? h_carry : h, hmax);
      const double pn = std::sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
      const double sc = std::max(s->tol * (1.0 + std::max(r, pn)), 1e-30);
      for (int att = 0; att < 4; ++att) {
        double e[6];
        tsit5_step(P, y, pt, hh, k1, yn, kn, e);
        rhs_evals += 6;
        h_used = hh;
        const double ex = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        const double ep = std::sqrt(e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
        const double err = std::max(ex, ep) / sc;  // e carries the factor h already
        if (err <= 1.0 || hh <= 1e-4 * s->dt) {
          const double g = err > 1e-12 ? 0.9 * std::exp(-0.14 * std::log(err) + 0.08 * std::log(kerr_prev)) : 4.0;
          h_carry = std::min(hh * clampd(g, 0.2, 4.0), hmax);
          kerr_prev = std::max(err, 1e-4);
          break;
        }
        hh = std::max(hh * std::max(0.9 * std::exp(-0.2 * std::log(err)), 0.2), 1e-4 * s->dt);
      }
    } else if (!S.tsit5) {
      rk4_step(P, y, pt, h, k1, yn);
      rhs_evals += 3;
    } else {
      // adaptive: error-controlled step, capped by the kernel's rule in DRAFT
      double hh = (h_carry > 0.0) ? std::min(h_carry, S.draft ? h : 1e30) : h;
      if (!S.draft) hh = std::min(hh, s->tspan - lambda);
      for (int att = 0; att < 60; ++att) {
        double e[6];
        tsit5_step(P, y, pt, hh, k1, yn, kn, e);
        rhs_evals += 6;
        double en = 0.0;
        for (int c = 0; c < 6; ++c) {
          const double sc = s->atol + s->rtol * std::max(std::fabs(y[c]), std::fabs(yn[c]));
          en += sq(e[c] / sc);
        }
        en = std::sqrt(en / 6.0);
        if (en <= 1.0 || hh < 1e-12) {
          const double fac = en > 1e-30 ? 0.9 * std::pow(en, -0.2) : 5.0;
          h_carry = hh * clampd(fac, 0.2, 5.0);
          break;
        }
        hh *= std::max(0.9 * std::pow(en, -0.2), 0.1);
      }
      h_used = hh;
    }
    if (!(yn[0] == yn[0]) || !(yn[2] == yn[2]) || !(yn[3] == yn[3])) { hit = true; budget = false; break; }

    auto step_from = [&](double hx, double* out) {
      if (S.tsit5) { double kx[6], ex[6]; tsit5_step(P, y, pt, hx, k1, out, kx, ex); }
      else rk4_step(P, y, pt, hx, k1, out);  // the kernel lands with RK4 in every mode
    };

    if (!S.draft) {
      // RENDER: z = 0 events (located, state unchanged) then the boundary.
      if (s->disc_on && y[2] * yn[2] < 0.0) {
        double ye[6];
        if (S.tsit5) {
          locate(step_from, [](const double* st) { return st[2]; }, y[2], yn[2], h_used, ye);
        } else {
          const double cfz = y[2] / (y[2] - yn[2]);
          for (int c = 0; c < 6; ++c) ye[c] = y[c] + cfz * (yn[c] - y[c]);
          ye[2] = 0.0;
        }
        disc_event(ye, pt);
      }
      const double rn = rnorm(yn);
      const bool inside0 = gb0 < 0.0 && r_start < 2.00001;
      double rb = -1.0;
      if (inside0) { if (rn >= 2.00001) rb = 2.00001; }
      else if (rn <= 2.00001) rb = 2.00001;
      else if (rn >= s->r_escape) rb = s->r_escape;
      if (rb > 0.0) {
        // boundary inside this step: land on it, as the reference's terminating callback does
        double ye[6];
        auto gr = [&](const double* st) { return rnorm(st) - rb; };
        locate(step_from, gr, r - rb, rn - rb, h_used, ye);
        for (int c = 0; c < 6; ++c) y[c] = ye[c];
        if (rb == s->r_escape) escaped = true; else hit = true;
        budget = false;
        lambda += h_used;
        ++steps;
        break;
      }
      lambda += h_used;
    } else {
      lambda += h_used;
      const double vlen = std::max(std::sqrt(k1[0] * k1[0] + k1[1] * k1[1] + k1[2] * k1[2]), 1e-20);
      bool stop = false;
      if (bk) ell += h_used * vlen;
      if (S.vol_on) stop = march_gas(S, y, yn, pt, h_used, vlen, r2, scam, &march_acc, acc, &alpha);
      flush_bucket();
      if (stop) {
        for (int c = 0; c < 6; ++c) y[c] = yn[c];
        ++steps;
        budget = false;
        break;
      }
      if (S.disc_on && !S.vol_on && alpha > 0.001 && y[2] * yn[2] < 0.0) {
        double ye[6];
        if (S.tsit5) {
          locate(step_from, [](const double* st) { return st[2]; }, y[2], yn[2], h_used, ye);
        } else {
          const double cfz = y[2] / (y[2] - yn[2]);
          for (int c = 0; c < 6; ++c) ye[c] = y[c] + cfz * (yn[c] - y[c]);
        }
        disc_event(ye, pt);
        flush_bucket();
      }
      // exit landing: the first state beyond r_escape is replaced by the state on it
      if (s->exit_landing) {
        const double rn = rnorm(yn);
        if (rn > s->r_escape) {
          double ye[6];
          auto gr = [&](const double* st) { return rnorm(st) - s->r_escape; };
          locate(step_from, gr, r - s->r_escape, rn - s->r_escape, h_used, ye);
          for (int c = 0; c < 6; ++c) y[c] = ye[c];
          escaped = true; budget = false;
          ++steps;
          break;
        }
      }
    }
    for (int c = 0; c < 6; ++c) y[c] = yn[c];
    if (S.tsit5 || S.ksteps) { for (int c = 0; c < 6; ++c) k1[c] = kn[c]; }
    else { P.rhs(y, pt, k1); rhs_evals += 1; }
    ++steps;
  }

  // Classification and sky (src/metal.jl:1629-1704; src/raytrace.jl:267-298).
  const double rf = std::max(rnorm(y), 1e-6);
  double vel[6];
  P.rhs(y, pt, vel);
  const double vl = std::max(std::sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]), 1e-20);
  for (int c = 0; c < 3; ++c) rec.dir[c] = vel[c] / vl;
  bool black;
  if (S.draft) black = hit || captured0 || rf < 4.0 * M;
  else black = hit || rf < 2.1 * M;
  double rgb[3] = {acc[0], acc[1], acc[2]};
  if (!black) {
    const double th = std::acos(clampd(rec.dir[2], -1.0, 1.0));
    const double ph = std::atan2(rec.dir[1], rec.dir[0]);
    double sky[3];
    sample_sky(s, th, ph, sky);
    if (s->star_strength > 0.0) {
      double sl[3];
      star_light(s, S.draft, rec.dir[0], rec.dir[1], rec.dir[2], sl);
      for (int c = 0; c < 3; ++c) sky[c] = sky[c] * s->star_tw + s->star_strength * sl[c];
    }
    sky_tint(scam, sky);
    for (int c = 0; c < 3; ++c) rgb[c] += alpha * sky[c];
    if (bk)
      for (int c = 0; c < 3; ++c) bk[3 * (nb - 1) + c] += alpha * sky[c];
  }
  rec.flags |= (escaped ? ORC_RAY_ESCAPED : 0) | (hit ? ORC_RAY_CAPTURED : 0) | (budget ? ORC_RAY_BUDGET : 0) |
               (black ? ORC_RAY_BLACK : 0);
  rec.r_final = rf;
  rec.alpha = alpha;
  rec.lambda = lambda;
  rec.steps = steps;
  rec.rhs_evals = rhs_evals;
  for (int c = 0; c < 3; ++c) { rec.rgb[c] = rgb[c]; ro->rgb[c] = rgb[c]; }
}

}  // namespace

extern "C" {

static void setup_scene(const orc_scene* s, Scene& S) {
  S.s = s;
  S.P.M = s->M; S.P.a = s->a; S.P.kerr = (s->a != 0.0);
  double beta[3];
  orc_camera_beta(s->velocity, s->fwd, s->right, s->up, beta);
  camera_tetrad(s->pos, s->fwd, s->right, s->up, s->M, s->a, beta, &S.T);
  const double rph = orc_photon_orbit_min(s->M, s->a);
  S.rkill2 = sq(0.995 * rph);
  isco(s->M, s->a, &S.r_isco, &S.E_isco, &S.L_isco);
  S.hcoef = s->hstep_coef; S.hcap = s->hstep_cap;
  S.draft = s->semantics == ORC_SEM_DRAFT;
  S.tsit5 = s->integrator == ORC_INT_TSIT5;
  S.ksteps = s->integrator == ORC_INT_TSIT5_K45 ? 45 : (s->integrator == ORC_INT_TSIT5_K46 ? 46 : 0);
  S.vol_on = S.draft && s->vol_on && s->vol != nullptr;
  S.disc_on = s->disc_on && s->disc_inner > 0.0 && s->disc_outer > s->disc_inner && s->bb_lut;
  S.kepler = s->emitter == ORC_EMIT_KEPLER;
  const int stride = std::min(std::max(s->vol_stride, 1), 16);
  S.ds_gas = stride * s->dt;
  if (S.vol_on) {
    const double so = std::exp(s->vol_ls_out);
    S.vol_rb2 = so * so + s->vol_zmax * s->vol_zmax;
  } else {
    S.vol_rb2 = -1.0;
  }
  S.nmax = s->nmax;
}

int orc_render(const orc_scene* s, float* out_rgb, orc_ray* rays, int nthreads) {
  if (!s || s->width <= 0 || s->height <= 0 || s->cols <= 0 || s->rows <= 0) return 1;
  if (std::fabs(s->a) > s->M) return 1;
  Scene S;
  setup_scene(s, S);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const int cols = s->cols, rows = s->rows;
#pragma omp parallel for schedule(dynamic, 1)
  for (int jj = 0; jj < rows; ++jj) {
    for (int ii = 0; ii < cols; ++ii) {
      RayOut ro;
      trace_ray(S, s->col0 + ii, s->row0 + jj, &ro);
      const size_t o = (size_t)ii + (size_t)cols * jj;
      if (out_rgb)
        for (int c = 0; c < 3; ++c) out_rgb[3 * o + c] = (float)ro.rgb[c];
      if (rays) rays[o] = ro.rec;
    }
  }
  return 0;
}

int orc_render_depth(const orc_scene* s, int nb, float* out, int nthreads) {
  if (!s || !out || nb < 3 || s->width <= 0 || s->height <= 0 || s->cols <= 0 || s->rows <= 0) return 1;
  if (std::fabs(s->a) > s->M || s->semantics != ORC_SEM_DRAFT) return 1;
  Scene S;
  setup_scene(s, S);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const int cols = s->cols, rows = s->rows;
#pragma omp parallel for schedule(dynamic, 1)
  for (int jj = 0; jj < rows; ++jj) {
    std::vector<double> bk(3 * (size_t)nb);
    for (int ii = 0; ii < cols; ++ii) {
      std::fill(bk.begin(), bk.end(), 0.0);
      RayOut ro;
      trace_ray(S, s->col0 + ii, s->row0 + jj, &ro, bk.data(), nb);
      float* o = out + 3 * (size_t)nb * ((size_t)ii + (size_t)cols * jj);
      for (int k = 0; k < 3 * nb; ++k) o[k] = (float)bk[k];
    }
  }
  return 0;
}

int orc_trace_dirs(const orc_scene* s, int n, const double* dirs, orc_ray* rays, int nthreads) {
  if (!s || n <= 0 || !dirs || !rays || std::fabs(s->a) > s->M) return 1;
  Scene S;
  setup_scene(s, S);
  S.dirs = dirs;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (int k = 0; k < n; ++k) {
    RayOut ro;
    trace_ray(S, k, 0, &ro);
    rays[k] = ro.rec;
  }
  return 0;
}

void orc_rhs(int kerr, const double s[6], double pt, double M, double a, double d[6]) {
  if (kerr) rhs_kerr(s, pt, M, a, d); else rhs_schw(s, pt, M, d);
}

void orc_camera_tetrad(const double pos[3], const double fwd[3], const double right[3], const double up[3],
                       double M, double a, const double beta[3], double u[4], double Ef[4], double Er[4],
                       double Eu[4]) {
  Tetrad T;
  camera_tetrad(pos, fwd, right, up, M, a, beta, &T);
  for (int k = 0; k < 4; ++k) { u[k] = T.u[k]; Ef[k] = T.Ef[k]; Er[k] = T.Er[k]; Eu[k] = T.Eu[k]; }
}

// src/camera.jl:19-22
void orc_camera_beta(const double vel[3], const double fwd[3], const double right[3], const double up[3],
                     double beta[3]) {
  beta[0] = vel[0] * fwd[0] + vel[1] * fwd[1] + vel[2] * fwd[2];
  beta[1] = vel[0] * right[0] + vel[1] * right[1] + vel[2] * right[2];
  beta[2] = vel[0] * up[0] + vel[1] * up[1] + vel[2] * up[2];
}

void orc_init_photon(const double origin[3], const double q[4], double M, double a, double state[6],
                     double* pt) {
  Phys P{M, a, a != 0.0};
  lower_photon(origin, q, P, state, pt);
}

// Kerr-Schild metric g = eta + f l l (covariant l = (1, l)), src/gr.jl:164-190,
// and its inverse eta - f l l with l^t = -1, src/gr.jl:119-153.
static void ks_fl(double M, double a, const double x[3], double* f, double l[3]) {
  if (a == 0.0) {
    const double r = std::sqrt(sq(x[0]) + sq(x[1]) + sq(x[2]));
    *f = 2.0 * M / r;
    for (int k = 0; k < 3; ++k) l[k] = x[k] / r;
  } else {
    const double r2 = ks_r2(x[0], x[1], x[2], a);
    const double r = std::sqrt(std::max(r2, 2.220446049250313e-16));
    *f = 2.0 * M * r * r * r / (r2 * r2 + a * a * x[2] * x[2]);
    const double ra = r2 + a * a;
    l[0] = (r * x[0] + a * x[1]) / ra;
    l[1] = (r * x[1] - a * x[0]) / ra;
    l[2] = x[2] / r;
  }
}
void orc_metric(double M, double a, const double x[3], double g[16]) {
  double f, l[3];
  ks_fl(M, a, x, &f, l);
  const double lD[4] = {1.0, l[0], l[1], l[2]};
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) g[4 * m + n] = (m == n ? (m == 0 ? -1.0 : 1.0) : 0.0) + f * lD[m] * lD[n];
}
void orc_metric_inverse(double M, double a, const double x[3], double gi[16]) {
  double f, l[3];
  ks_fl(M, a, x, &f, l);
  const double lU[4] = {-1.0, l[0], l[1], l[2]};
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) gi[4 * m + n] = (m == n ? (m == 0 ? -1.0 : 1.0) : 0.0) - f * lU[m] * lU[n];
}

// src/gr.jl:42-43, 58-60
double orc_horizon_radius(double M, double a) { return M + std::sqrt(std::max(M * M - a * a, 0.0)); }
double orc_photon_orbit_min(double M, double a) {
  if (a == 0.0) return 3.0 * M;
  return 2.0 * M * (1.0 + std::cos((2.0 / 3.0) * std::acos(-a / M)));
}
void orc_isco(double M, double a, double out[3]) { isco(M, a, &out[0], &out[1], &out[2]); }
void orc_blackbody_rgb(double T, double rgb[3]) { blackbody_rgb(T, rgb); }

// Blackbody LUT with white-balance gains: src/blackbody.jl:51-60.
void orc_blackbody_lut(double wb_temperature, double tmin, double tmax, int n, float* lut) {
  double ref[3];
  blackbody_rgb(wb_temperature, ref);
  const double gains[3] = {1.0 / ref[0], 1.0 / ref[1], 1.0 / ref[2]};
  for (int i = 0; i < n; ++i) {
    const double T = (n == 1) ? tmin : tmin + (tmax - tmin) * i / (n - 1);
    double c[3];
    blackbody_rgb(std::max(T, 1.0), c);
    for (int k = 0; k < 3; ++k) lut[3 * i + k] = (float)(c[k] * gains[k]);
  }
}
float orc_sim_hash(int x, int y, int z) { return sim_hash(x, y, z); }

// src/utils.jl:31-37
double orc_shadow_radius(double r_cam, double M, double fov) {
  const double sa = 3.0 * std::sqrt(3.0) * M / r_cam;
  if (sa >= 1.0) return INFINITY;
  return std::tan(std::asin(sa)) / fov;
}

// test/runtests.jl:612-636 restated: L_z drift along fixed-step Kerr RK4.
double orc_lz_drift(double a, double h, int nmax) {
  double y[6] = {12.0, 0.7, 0.9, -1.0, 0.15, 0.05};
  const double Lz0 = y[0] * y[4] - y[1] * y[3];
  const double rp = orc_horizon_radius(1.0, a);
  double worst = 0.0;
  Phys P{1.0, a, true};
  for (int n = 0; n < nmax; ++n) {
    const double r = rnorm(y);
    if (r < 1.15 * rp + 0.35 || r > 80.0) break;
    double k1[6], yn[6];
    P.rhs(y, -1.0, k1);
    rk4_step(P, y, -1.0, h, k1, yn);
    for (int c = 0; c < 6; ++c) y[c] = yn[c];
    worst = std::max(worst, std::fabs((y[0] * y[4] - y[1] * y[3]) - Lz0) / std::fabs(Lz0));
  }
  return worst;
}

}  // extern "C"
