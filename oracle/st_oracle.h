/*
 * st_oracle.h -- CPU FP64 oracle for the per-pixel null-geodesic render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a double-precision C++ restatement of
 * SpaceTime.jl's render semantics, used by tests/, the smoke check and the
 * CPU baseline leg of bench.py as the checker.  The product library
 * (spacetime_gb300/csrc) never includes, links or calls it.
 *
 * Two semantics are restated (they differ on purpose in the reference):
 *   ORC_SEM_RENDER  the CPU renderer `render` (src/raytrace.jl:339-428,
 *                   src/callbacks.jl:7-105, src/accretion_disc.jl:19-49):
 *                   horizon at r = 2.00001, escape at r_max, affine budget
 *                   tspan, Keplerian Planck-Doppler disc, black iff r < 2.1M.
 *   ORC_SEM_DRAFT   the GPU kernel `trace_kernel_mtl!` (src/metal.jl:750-1707):
 *                   radius-adaptive step, photon-orbit / 2.95M kill tests,
 *                   Bardeen launch capture test, exact Kerr-Schild emitter,
 *                   volumetric gas march, black iff r < 4M.
 * and two integrators:
 *   ORC_INT_RK4     fixed-step RK4 on the kernel's step rule ("kernel twin",
 *                   src/metal.jl:1382-1401, src/preview.jl:62-69)
 *   ORC_INT_TSIT5   adaptive Tsitouras 5(4) (Tsitouras 2011) with step-size
 *                   secant event location for z = 0 and r = r_escape; stands
 *                   in for DifferentialEquations' Tsit5 + ContinuousCallback
 *                   (src/raytrace.jl:369-373).
 * Parity status: unit pieces are pinned to the reference's own known-answer
 * tests (test/runtests.jl); image-level output is unpinned by the reference
 * (no reference test compares pixel values) and is pinned here by
 * convergence of the two integrators against each other.
 */
#ifndef ST_ORACLE_H
#define ST_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_SEM_RENDER = 0, ORC_SEM_DRAFT = 1 };
enum { ORC_INT_RK4 = 0, ORC_INT_TSIT5 = 1,
       /* twins of the kernel's own adaptive modes (render_draft_mtl order 45 / 46,
        * src/metal.jl:1278-1381): same controller, same step caps */
       ORC_INT_TSIT5_K45 = 2, ORC_INT_TSIT5_K46 = 3 };
enum { ORC_EMIT_KEPLER = 0, ORC_EMIT_KS_EXACT = 1 };

/* per-ray outcome flags */
enum {
  ORC_RAY_ESCAPED = 1,   /* reached the escape radius */
  ORC_RAY_CAPTURED = 2,  /* killed / horizon / Bardeen / NaN */
  ORC_RAY_BUDGET = 4,    /* ran out of steps or affine budget */
  ORC_RAY_BLACK = 8,     /* background not added (captured or r < r_black) */
  ORC_RAY_CROSSED = 16,  /* crossed z = 0 inside the disc annulus at least once */
  ORC_RAY_GRAZE = 32,    /* Bardeen graze0 flag (Kerr) */
  ORC_RAY_BCAPT = 64     /* Bardeen captured0 flag (Kerr) */
};

typedef struct {
  /* camera: world-frame axes (orthonormal), fov factor, world velocity (c) */
  double pos[3], fwd[3], right[3], up[3];
  double fov;
  double velocity[3];
  int projection;          /* 0 pinhole, 1 fisheye */
  double fisheye_rad;      /* half-angle at the top edge */
  double aperture_radius;  /* world units; 0 = pinhole */
  double focus_dist;
  int lens_seed;           /* per-pass hash seed of the lens stratum */
  double lens_u0, lens_v0, lens_w;  /* lens stratum origin and width */
  /* spacetime */
  double M, a;
  /* thin disc */
  int disc_on;
  double disc_inner, disc_outer, disc_falloff;
  int emitter;
  const float* bb_lut;     /* (3, lut_size) */
  int lut_size;
  double lut_tmin, lut_tmax;
  /* volumetric gas (DRAFT only) */
  int vol_on;
  const float* vol;        /* (nr, nphi, nz) column-major */
  int nr, nphi, nz;
  double vol_ls_in, vol_ls_out, vol_zmax, vol_emis, vol_opac;
  int vol_stride;
  /* sky */
  const float* sky;        /* (3, sky_w, sky_h) column-major */
  int sky_w, sky_h;
  /* frame */
  int width, height;
  int col0, cols, row0, rows;   /* sub-rectangle to render */
  double ju, jv;           /* sub-pixel offset, GPU convention (0.5 = centre) */
  double jitter_w;         /* > 0: per-pixel hashed jitter inside the stratum */
  int jitter_seed;
  /* integration */
  int semantics, integrator;
  double dt;
  int nmax;
  double r_escape;         /* DRAFT escape radius / RENDER r_max */
  double tspan;            /* RENDER affine budget */
  double hstep_coef, hstep_cap;
  double rtol, atol;
  int relativistic;
  int exit_landing;        /* land exactly on r_escape (DRAFT) */
  double tol;              /* kernel-twin adaptive tolerance */
  /* per-pixel shutter (src/metal.jl:829-857): seed 0 = off; the pose at the
   * far end of the stratum, interpolated per pixel at tau = hash(i, j, seed) */
  int shutter_seed;
  double pos_end[3], u_end[4], Ef_end[4], Er_end[4], Eu_end[4];
  /* procedural stars (src/metal.jl:652-724, src/starfield.jl:83-150); strength 0 = off */
  double star_strength, star_tw;
  double star_N, star_fill, star_sigma, star_flux;
  double star_g[3], star_conc, star_tmin, star_tspan;
  const float* star_lut;   /* (3, star_lut_size) */
  int star_lut_size, star_seed;
  double star_lut_tmin, star_lut_tmax;
} orc_scene;

typedef struct {
  double dir[3];      /* unit escape direction (coordinate velocity) */
  double r_final;
  double alpha;       /* remaining transmittance */
  double r_cross;     /* first disc-annulus crossing radius, -1 if none */
  double g_cross;     /* 1/(1+z) at that crossing */
  double rgb[3];      /* this ray's colour (not weighted) */
  double lambda;      /* affine parameter travelled */
  int flags;
  int steps;          /* accepted steps */
  int rhs_evals;
  int pad;
} orc_ray;

/* Render the sub-rectangle into out_rgb ((3, cols, rows) column-major,
 * i.e. [rows][cols][3]) and optionally the per-ray records ([rows][cols]). */
int orc_render(const orc_scene* sc, float* out_rgb, orc_ray* rays, int nthreads);

/* DRAFT render of the sub-rectangle with emission split into nb >= 3 depth
 * buckets (render_depth_mtl, src/metal.jl:1935-1990): out[rows][cols][nb][3],
 * one unweighted pass; bucket nb - 1 (0-based) holds the sky. */
int orc_render_depth(const orc_scene* sc, int nb, float* out, int nthreads);

/* Trace n rays from the scene's camera along camera-frame directions
 * dirs[n][3] = (cf, cr, cu) (forward, right, up coefficients of the tetrad,
 * as a pixel's projection produces them), no lens, jitter or shutter: the
 * twin of the layered engine's deflection fan.  Pixel fields are unused. */
int orc_trace_dirs(const orc_scene* sc, int n, const double* dirs, orc_ray* rays, int nthreads);

/* --- live fluid disc (DiscFluidSim / step_sim!, src/disc_sim.jl) ---------
 * All arrays are caller-owned, (nr, nphi) column-major unless noted. */
typedef struct {
  int nr, nphi, nz;
  float* vu; float* vv;      /* velocity, grid cells per M-time */
  float* dens;               /* surface density */
  float* base;               /* relaxation target (radial profile) */
  float* env;                /* (nr, nz) vertical envelope */
  float* shear;              /* [nr] Keplerian shear, phi cells per M-time */
  float t;                   /* simulation clock */
  double forcing, drag, relax;
} orc_fluid;
/* DiscFluidSim construction from a (nr, nphi, nz) density texture. */
int orc_fluid_init(orc_fluid* f, const float* vol_density, float log_s_in, float log_s_out, float z_max,
                   double scale_height, double M, double inner, double outer, double falloff);
/* nsteps step_sim! steps; vol_out (may be NULL) receives the extruded
 * (nr, nphi, nz) texture of the final state. */
int orc_fluid_step(orc_fluid* f, float* vol_out, double dt, int jacobi, int nsteps);

/* --- unit pieces, for known-answer tests --- */
void orc_rhs(int kerr, const double s[6], double pt, double M, double a, double d[6]);
void orc_camera_tetrad(const double pos[3], const double fwd[3], const double right[3],
                       const double up[3], double M, double a, const double beta[3],
                       double u[4], double Ef[4], double Er[4], double Eu[4]);
void orc_camera_beta(const double vel[3], const double fwd[3], const double right[3],
                     const double up[3], double beta[3]);
void orc_init_photon(const double origin[3], const double q[4], double M, double a,
                     double state[6], double* pt);
void orc_metric(double M, double a, const double x[3], double g[16]);
void orc_metric_inverse(double M, double a, const double x[3], double gi[16]);
double orc_horizon_radius(double M, double a);
double orc_photon_orbit_min(double M, double a);
void orc_isco(double M, double a, double out[3]);
void orc_blackbody_rgb(double T, double rgb[3]);
void orc_blackbody_lut(double wb_temperature, double tmin, double tmax, int n, float* lut);
float orc_sim_hash(int x, int y, int z);
double orc_shadow_radius(double r_cam, double M, double fov);
/* Fixed-step RK4 of the Kerr RHS (as in the reference's L_z test) -> worst
 * relative L_z drift. */
double orc_lz_drift(double a, double h, int nmax);

#ifdef __cplusplus
}
#endif
#endif
