/*
 * spacetime_gb300.h -- C ABI of libspacetime_gb300.so, the GB300 (sm_103a)
 * implementation of SpaceTime.jl's per-pixel null-geodesic render path.
 *
 * Plain C: POD structs, pointers and sizes, integer status codes, no C++
 * exceptions across the boundary.  A Julia `ccall`, Python `ctypes` or any
 * C caller binds it directly.
 *
 * Reference interfaces replaced (paths within SpaceTime.jl):
 *   st_context_create      MetalPreviewContext(bg, w, h; dt, nmax, disc, volume)
 *                          src/metal.jl:129-182 (sky uploaded once, :111-121, :134)
 *   st_context_set_disc    the disc block of MetalPreviewContext, src/metal.jl:140-154,
 *                          and set_disc_enabled!, src/metal.jl:206-214
 *   st_context_set_volume  the volume block of MetalPreviewContext, src/metal.jl:155-166,
 *                          set_volume_enabled! / set_march_stride!, src/metal.jl:192-308
 *   st_render              render(cam, bh, sky; disc, width, height, samples, relativistic)
 *                          src/raytrace.jl:339-428 (semantics ST_SEM_RENDER), and
 *                          render_draft_mtl(ctx, cam, st; width, height, samples, dt,
 *                          fisheye_deg, aperture_world, focus_dist, relativistic, order)
 *                          src/metal.jl:2040-2242 (semantics ST_SEM_DRAFT)
 *   st_render_frames       the per-frame loop of the examples/videos scripts over
 *                          render_draft_mtl, batched into one persistent launch
 *   st_render_device       _trace_preview_gpu!, src/metal.jl:1825-1881 (result left
 *                          on the device, no download)
 *   st_camera_tetrad       ks_camera_tetrad + camera_beta, src/preview.jl:93-198,
 *                          src/camera.jl:19-22
 *   st_context_set_starfield  set_starfield!(ctx; ...), src/metal.jl:257-295, and the
 *                          CPU renderer's Starfield(...), src/starfield.jl:60-81
 *   st_render_motion       render_draft_mtl(...; camera_at, per_pixel_shutter),
 *                          src/metal.jl:2017-2030, 2130-2169, 829-857
 *   st_save_raw / st_load_raw  save_raw / load_raw, src/rawio.jl:18-42 (host only)
 *   st_sky_fan             update_sky_fan!, src/metal.jl:2978-3036 (sky_fan_kernel!,
 *                          fan_band_kernel!, src/metal.jl:2416-2517, 2888-2898)
 *   st_render_layered      render_layered_gpu!, src/metal.jl:3040-3147 (layer pass of
 *                          trace_kernel_mtl!, sky_composite_kernel!, :2707-2880)
 *   st_render_layered_ring the same with its foveated ring pass (ring_out, ring_rmin,
 *                          ring_box; _ring_screen_box :2522-2666)
 *   st_render_depth        render_depth_mtl, src/metal.jl:1935-1990 (trace_kernel_mtl!
 *                          with NB > 0: :1170-1175, 1425-1426, 1489-1497, 1556-1563,
 *                          1687-1690)
 *   st_fluid_create / st_fluid_step  DiscFluidSim(vol, disc; M, forcing, drag, relax) and
 *                          step_sim!(sim, ctx; dt, jacobi), src/disc_sim.jl:38-91, 280-320
 *
 * Output layout: linear HDR RGB float32 in the reference's column-major
 * (3, width, height) order, i.e. out[3*(i + width*j) + c] for 0-based pixel
 * (i, j); row j = 0 is the bottom of the frame (v < 0), as in
 * src/metal.jl:870-872 and src/camera.jl:391-396.
 *
 * Threading: one context is single-threaded (one CUDA stream).  Independent
 * contexts may be driven from different host threads.  st_render is
 * synchronous: it returns after the device-to-host copy.
 */
#ifndef SPACETIME_GB300_H
#define SPACETIME_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ST_ABI_VERSION 1

typedef struct st_context st_context;

/* status codes; ST_EINVAL mirrors the reference's ArgumentError (src/gr.jl:31) */
enum {
  ST_OK = 0,
  ST_EINVAL = 1,        /* bad argument: |a| > M, sizes <= 0, NULL pointer, ... */
  ST_ECUDA = 2,         /* a CUDA runtime call failed */
  ST_EBUDGET = 3,       /* the persistent queue hit its iteration budget */
  ST_ENOMEM = 4,        /* device or host allocation failed */
  ST_EUNSUPPORTED = 5,  /* combination not provided (e.g. Kerr with ST_SEM_RENDER) */
  ST_ESTATE = 6,        /* context not ready (e.g. surrogate requested, none loaded) */
  ST_ELIMIT = 7         /* request exceeds the fixed scratch capacity of
                           st_render_frames_noalloc */
};

enum { ST_PROJ_PINHOLE = 0, ST_PROJ_FISHEYE = 1 };
/* disc emitter model: the CPU renderer's Keplerian Planck-Doppler shading
 * (src/accretion_disc.jl:19-49) or the kernel's exact Kerr-Schild emitter
 * (src/metal.jl:396-428) */
enum { ST_EMIT_KEPLER = 0, ST_EMIT_KS_EXACT = 1 };
/* which reference path's rules are reproduced (they differ on purpose):
 * RENDER = src/raytrace.jl render (horizon 2.00001, r_max, affine budget,
 * black iff r < 2.1M); DRAFT = src/metal.jl trace_kernel_mtl! (photon-orbit
 * and 2.95M kill tests, Bardeen launch test, black iff r < 4M). */
enum { ST_SEM_RENDER = 0, ST_SEM_DRAFT = 1 };
/* arithmetic of the geodesic integration */
enum {
  ST_PREC_FP64 = 0,          /* everything in double */
  ST_PREC_FP32_GUARDED = 1,  /* FP32 RK4 with a compensated (float-float) state;
                                FP64 for steps inside r_guard, for rays in the
                                critical band, and for the null-constraint
                                renormalisation */
  ST_PREC_FP32 = 2,          /* plain FP32, as the reference's Metal kernel */
  ST_PREC_FP32_GUARDED_DF = 3  /* ST_PREC_FP32_GUARDED with the guard steps and
                                the null renormalisation in double-float
                                arithmetic (pairs of floats, about 47-bit
                                significands) on the FP32 pipe instead of
                                FP64, whose rate on GB300 is a small fraction
                                of FP32's */
};
/* launch schedule */
enum {
  ST_SCHED_PIXEL = 0,       /* one thread per pixel, 2-D tiles */
  ST_SCHED_PERSISTENT = 1   /* persistent CTAs, device ray queue, per-lane refill */
};

typedef struct {
  double pos[3];
  double fwd[3], right[3], up[3];  /* orthonormal camera axes (world frame) */
  double fov_factor;               /* tan(half vertical fov); Lens(f) -> 18/f */
  double velocity[3];              /* world-frame 3-velocity in units of c */
  int projection;                  /* ST_PROJ_* */
  double fisheye_deg;              /* fisheye half-angle at the top edge */
  double aperture_world;           /* thin-lens aperture diameter; 0 = pinhole */
  double focus_dist;               /* thin-lens focus distance (world units) */
} st_camera;

typedef struct {
  double M; /* mass */
  double a; /* spin, |a| <= M; 0 = Schwarzschild */
} st_spacetime;

typedef struct {
  double inner, outer;       /* annulus radii; inner <= 0 disables the disc */
  double falloff;            /* density_falloff */
  double wb_temperature;     /* Blackbody(wb_temperature=...) */
  double table_min, table_max;
  int table_size;
  int emitter;               /* ST_EMIT_* */
} st_disc;

typedef struct {
  const float* density;      /* (nr, nphi, nz) column-major, peak-normalised */
  int nr, nphi, nz;
  float log_s_in, log_s_out, z_max;
  float emission_scale, opacity_scale;
  int march_stride;          /* gas sampled every march_stride*dt of arc, 1..16 */
} st_volume;

/* Procedural point stars, evaluated per escaping ray in the source sky
 * (starfield_mtl, src/metal.jl:652-724; starfield_color, src/starfield.jl:83-150).
 * Stars sit on a density x density lattice of directions (u = atan2(y,x)/2pi +
 * 1/2, v = (z+1)/2), at most one per cell, placed, thinned and coloured by
 * the reference's hash; each is a Gaussian of width
 * psf_pixels * 2 fov_factor / height radians.  The sky image is scaled by
 * texture_weight under them.  Star colour comes from the stars' own
 * blackbody table (white point wb_temperature, chroma scaled by saturation
 * about Rec.709 luminance), never the disc's. */
typedef struct {
  double strength;           /* 0 disables */
  double texture_weight;     /* sky image weight under the stars */
  int height;                /* render height the PSF is sized for */
  double fov_factor;         /* the vertical field is 2 fov_factor across height rows */
  double density, fill, flux, psf_pixels;
  double galactic[3];        /* galactic-plane normal (need not be unit) */
  double concentration;      /* occupancy thinning exp(-|n.s| concentration) */
  double temp_min, temp_max; /* star temperatures, uniform */
  int seed;
  double wb_temperature;     /* star white point */
  double saturation;         /* chroma scale of the star table */
  int table_size;            /* star table entries */
} st_starfield;

typedef struct {
  int width, height;
  int samples;               /* samples^2 stratified passes per pixel */
  double dt;                 /* base affine step */
  int nmax;                  /* step budget; 0 = the reference's rule */
  int semantics;             /* ST_SEM_* */
  int precision;             /* ST_PREC_* */
  int schedule;              /* ST_SCHED_* */
  double r_escape;           /* DRAFT escape radius / RENDER r_max; 0 = rule */
  double tspan;              /* RENDER affine budget; 0 = rule */
  int relativistic;          /* per-ray camera/infinity shift on shading */
  int exit_landing;          /* land exactly on r_escape before reading the sky */
  int pixel_jitter;          /* per-pixel hashed jitter inside each stratum */
  unsigned long long seed;   /* pass shuffles and hash seeds */
  double r_guard;            /* FP32_GUARDED: FP64 steps inside this KS radius
                                (rays not already proven captured); 0 = off */
  double crit_band;          /* FP32_GUARDED: critical-band rays get FP64 steps:
                                |b - b_crit| < crit_band (Schwarzschild) or the
                                Bardeen graze flag (Kerr); <= 0 = off */
  double crit_r;             /* ...but only inside this KS radius; 0 = whole ray */
  int renorm_every;          /* FP32_GUARDED: FP64 null renormalisation period; 0 = off */
  int surrogate;             /* 1 = gate + learned surrogate (st_surrogate_*) */
  double surrogate_sigma;    /* gate: max predicted std-dev (rad) served */
  int block_x, block_y;      /* ST_SCHED_PIXEL tile; 0 = tuned default */
  int chunk_steps;           /* ST_SCHED_PERSISTENT steps per refill check */
  int graph;                 /* st_render_frames: capture the device work in a
                                CUDA graph and replay it while the frame count,
                                sizes and rules are unchanged */
  int order;                 /* integrator, render_draft_mtl's `order`: 4 = RK4,
                                45 / 46 = adaptive Tsitouras 5(4) capped at the
                                radius-adaptive step / free up to 50 dt
                                (DRAFT, FP32 or FP64, pixel schedule) */
  double tol;                /* adaptive tolerance (`tol`, default 1e-4) */
  /* adaptive refinement (render_draft_mtl `refine`, src/metal.jl:2104-2240):
   * refine > 1 flags pixels whose per-ray luminance std-dev over the base
   * passes exceeds refine_var * (mean + 0.01) or whose Bardeen graze fraction
   * exceeds refine_graze, and re-renders their bounding box (+ refine_margin
   * pixels) refine - 1 more times with fresh strata; DRAFT, no surrogate */
  int refine;                /* default 1 (off) */
  double refine_var;         /* default 0.35 */
  double refine_graze;       /* default 0.05 */
  int refine_margin;         /* default 8 */
} st_render_params;

typedef struct {
  double total_ms;           /* wall time of the call */
  double kernel_ms;          /* device time of the trace kernels (CUDA events) */
  unsigned long long rays;
  unsigned long long steps;        /* accepted integration steps */
  unsigned long long fp64_steps;   /* of which ran in FP64 */
  unsigned long long gas_samples;
  unsigned long long surrogate_rays;
  int launches;              /* trace-kernel launches issued */
  int status;                /* ST_OK or the persistent queue's status */
  unsigned long long h2d_bytes, d2h_bytes;
} st_stats;

/* per-ray record (st_render_diag) */
typedef struct {
  double dir[3];             /* unit escape direction (coordinate velocity) */
  float r_final, alpha, r_cross, g_cross;
  float lambda;              /* affine parameter travelled (RENDER) */
  int flags;                 /* ST_RAY_* */
  int steps, fp64_steps;
  int pad[2];
} st_ray_diag;

enum {
  ST_RAY_ESCAPED = 1, ST_RAY_CAPTURED = 2, ST_RAY_BUDGET = 4, ST_RAY_BLACK = 8,
  ST_RAY_CROSSED = 16, ST_RAY_GRAZE = 32, ST_RAY_BCAPT = 64, ST_RAY_SURROGATE = 128,
  ST_RAY_GUARDED = 256
};

int st_abi_version(void);
const char* st_strerror(int code);

/* Fill *p with the defaults of the given semantics (the reference's keyword
 * defaults: dt 0.02, samples 1, rule-based nmax / r_escape / tspan). */
void st_render_params_default(st_render_params* p, int semantics);

/* Create a context on `device`; copies the (3, sky_w, sky_h) float sky to HBM. */
int st_context_create(st_context** out, const float* sky_rgb, int sky_w, int sky_h, int device);
/* NULL disables the thin disc (the gas keeps the last blackbody table; a new
 * context starts with Blackbody() defaults: 6500 K white point, 500-30000 K,
 * 1024 entries). */
int st_context_set_disc(st_context* ctx, const st_disc* disc);
/* NULL disables the volume; the density grid is copied to HBM.  ST_EINVAL for
 * nr < 2, nphi < 1, nz < 2, log_s_out <= log_s_in, z_max <= 0 or a grid of
 * 2^31 cells or more. */
int st_context_set_volume(st_context* ctx, const st_volume* vol);
/* set_starfield! defaults: strength 1, texture_weight 0, height 1080,
 * fov_factor 0.55, density 384, fill 0.5, flux 0.011, psf_pixels 0.5,
 * galactic (0,0,1), concentration 3, temperatures 3000-16000 K, seed 12345,
 * white point 10000 K, saturation 1, 1024 entries. */
void st_starfield_default(st_starfield* sf);
/* NULL or strength <= 0 disables the stars (the context default).  Rejects a
 * zero galactic normal (ArgumentError in the reference), height < 1,
 * density < 1, psf_pixels <= 0 or table_size < 2 with ST_EINVAL. */
int st_context_set_starfield(st_context* ctx, const st_starfield* sf);
void st_context_destroy(st_context* ctx);

/* Render one frame into caller-owned host memory out_rgb[3*width*height]. */
int st_render(st_context* ctx, const st_camera* cam, const st_spacetime* st,
              const st_render_params* p, float* out_rgb, st_stats* stats);

/* As st_render, also writing one st_ray_diag per pixel of the last pass. */
int st_render_diag(st_context* ctx, const st_camera* cam, const st_spacetime* st,
                   const st_render_params* p, float* out_rgb, st_ray_diag* diag,
                   st_stats* stats);

/* Render and leave the frame on the device: *dev_rgba receives a pointer to
 * the context's float4 [height][width] framebuffer (valid until the next call). */
int st_render_device(st_context* ctx, const st_camera* cam, const st_spacetime* st,
                     const st_render_params* p, const float** dev_rgba, st_stats* stats);

/* Motion blur, render_draft_mtl(...; camera_at, per_pixel_shutter)
 * (src/metal.jl:2130-2169).  Each of the samples^2 passes owns one shutter
 * stratum m (shuffled, like the pixel and lens strata).  The caller evaluates
 * its camera_at(s) at the fractions the passes need and passes the poses:
 *   per_pixel_shutter = 0: poses[m] = camera_at((m + 0.5) / samples^2),
 *                          m < samples^2: each pass renders from the
 *                          midpoint of its stratum (nposes = samples^2);
 *   per_pixel_shutter = 1: poses[m] = camera_at(m / samples^2), m <= samples^2:
 *                          each pixel moves the pose from poses[m] toward
 *                          poses[m + 1] by a hashed fraction
 *                          (src/metal.jl:843-857; nposes = samples^2 + 1).
 * A pose supplies position, axes, fov_factor and velocity; projection and lens
 * come from cam, which also sets the escape radius and the step budget, as
 * the reference's render call does.  diag (may be NULL) receives the last
 * pass's per-ray records.  No surrogate (ST_EUNSUPPORTED). */
int st_render_motion(st_context* ctx, const st_camera* cam, const st_camera* poses, int nposes,
                     int per_pixel_shutter, const st_spacetime* st, const st_render_params* p,
                     float* out_rgb, st_ray_diag* diag, st_stats* stats);

/* Depth-bucketed draft frame (render_depth_mtl): the DRAFT trace with each
 * disc / gas emission written into one of nbuckets path-length buckets instead
 * of the pixel sum.  Path length ell is the integral of |dx/dlambda| over the
 * accepted steps; bucket 1 takes ell <= 1.5 M, buckets 1..nbuckets-1 are
 * log-spaced to 120 M (index trunc((ln ell - ln 1.5) (nbuckets - 2) / ln 80) + 1,
 * clamped), and bucket nbuckets holds the escaped sky times the remaining
 * transmittance.  out_buckets is the reference's (3 nbuckets, width, height)
 * column-major array: out[3 nbuckets (i + width j) + 3 b + c] for 0-based
 * bucket b and channel c; the samples^2 passes are averaged as in st_render.
 * nbuckets in [3, 64] (ST_EINVAL otherwise; the reference requires >= 3).
 * DRAFT only, no surrogate, no refinement (ST_EUNSUPPORTED). */
int st_render_depth(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                    int nbuckets, float* out_buckets, st_stats* stats);

/* ---- live fluid disc (DiscFluidSim, src/disc_sim.jl) -------------------------
 * A 2-D stable-fluids solver (semi-Lagrangian advection on the Keplerian
 * shear, curl-noise forcing, Jacobi pressure projection, MacCormack density
 * advection relaxed toward the disc profile) on the context volume's own
 * (log s, phi) grid; every step extrudes the surface density through the
 * vertical envelope exp(-z^2 / 2 H^2), H = scale_height s, into the
 * context's density texture, so the next render traces the new gas.  The
 * solver starts from the texture's midplane slice (k = (nz + 1) / 2,
 * 1-based) normalised to a peak of 1.  Units: M-time; velocities in grid
 * cells per M-time.  The context must hold a volume (ST_ESTATE otherwise) and
 * must outlive the solver; replacing its volume with another grid makes
 * st_fluid_step return ST_ESTATE. */
typedef struct st_fluid st_fluid;
typedef struct {
  double M;                  /* default 1 */
  double forcing;            /* eddy forcing amplitude, default 6 */
  double drag;               /* velocity damping per M-time, default 0.15 */
  double relax;              /* density relaxation toward the profile per M-time, default 0.05 */
  double scale_height;       /* the volume's H(s) = scale_height s, default 0.08 */
} st_fluid_params;
void st_fluid_params_default(st_fluid_params* p);
/* disc: the AccretionDisc whose radial profile (inner, outer, falloff) the
 * density relaxes toward. */
int st_fluid_create(st_fluid** out, st_context* ctx, const st_disc* disc, const st_fluid_params* p);
/* nsteps steps of dt (step_sim! defaults: dt 0.05, jacobi 8, i.e.
 * 2 ceil(jacobi / 2) Jacobi sweeps), queued on the context's stream.
 * use_graph = 1 replays a CUDA graph of the step's launches; ms (may be
 * NULL) receives the device time of the steps (the call then waits for them). */
int st_fluid_step(st_fluid* f, double dt, int jacobi, int nsteps, int use_graph, float* ms);
/* Host copies of the solver state ((nr, nphi) column-major; any may be NULL):
 * the velocity, the surface density, the context's density texture
 * ((nr, nphi, nz)) and the simulation clock. */
int st_fluid_state(st_fluid* f, float* vu, float* vv, float* dens, float* volume, double* t);
void st_fluid_destroy(st_fluid* f);

/* Raw HDR frame files, save_raw / load_raw (src/rawio.jl:18-42): a linear,
 * unclamped 32-bit float RGB TIFF in display orientation (the reference's
 * rotr90 of the frame: TIFF pixel (row r, column c) = frame pixel
 * (width - 1 - c, r)) and a TOML sidecar <path>.toml holding metadata_toml
 * (may be NULL) followed by the keys `format` and `saved_at`.  rgb is the
 * frame in this ABI's output layout.  Host only (no GPU). */
int st_save_raw(const char* path, const float* rgb, int width, int height, const char* metadata_toml);
/* Frame size of a raw file (float32 RGB chunky TIFF, uncompressed). */
int st_load_raw_size(const char* path, int* width, int* height);
/* The frame back in the output layout; width and height must match. */
int st_load_raw(const char* path, float* rgb, int width, int height);

/* ---- layered engine (Schwarzschild) ----------------------------------------
 * By spherical symmetry the sky a static observer at radius r sees depends on
 * one angle, psi, between the ray and the outward radial axis.  A fan of 4096
 * geodesics over psi in [0, pi] (plus 1024 across the escape/capture
 * transition, padded by 3 coarse spacings) replaces per-pixel sky
 * integration; only the disc and gas are traced per pixel (at the layer
 * resolution; rays the fan proves miss them are skipped) and composited over
 * the fan-driven sky.  Schwarzschild, DRAFT rules, FP64 or FP32, an
 * unboosted camera at rest with r >= 2.5 M (ST_EUNSUPPORTED otherwise). */
#define ST_FAN_N 4096
#define ST_FAN_FINE 1024
/* The fans for this camera: fan[ST_FAN_N][4] and fine[ST_FAN_FINE][4] =
 * (escaped 0/1, cos theta_f, sin theta_f, periapsis) with theta_f the exit
 * direction's angle from the radial axis in the ray's plane; band[2] = the
 * fine fan's psi range ((0, 0) when the coarse fan has no transition). */
int st_sky_fan(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
               float* fan, float* fine, float* band);
/* The layered frame into out_rgb[3*width*height]; layer_width / height <= 0
 * mean the display size; diag (may be NULL) holds the fan-derived exit
 * direction per pixel (last pass). */
int st_render_layered(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                      int layer_width, int layer_height, float* out_rgb, st_ray_diag* diag, st_stats* stats);
/* The layered frame with the foveated ring pass (render_layered_gpu!'s
 * ring_out / ring_rmin / ring_box, src/metal.jl:3102-3118, 2846-2863): a second
 * layer of ring_width x ring_height (<= 0: the display) traced only for the
 * rays whose fan periapsis is below ring_rmin (the wound rays of the photon
 * ring; the others are transparent), blended over the bulk layer with weight
 * 1 - smoothstep((r_p - 0.8 ring_rmin) / (0.2 ring_rmin)).  ring_box = 1
 * dispatches only the screen box that can hold wound rays (a probe grid of
 * camera rays against the impact-parameter bound 1.06 R / sqrt(1 - 2M/R),
 * R = ring_rmin); outside it the ring layer is transparent either way.
 * ring_rmin = 0 is st_render_layered. */
int st_render_layered_ring(st_context* ctx, const st_camera* cam, const st_spacetime* st, const st_render_params* p,
                           int layer_width, int layer_height, int ring_width, int ring_height, double ring_rmin,
                           int ring_box, float* out_rgb, st_ray_diag* diag, st_stats* stats);

/* Render `nframes` camera poses (a camera track) in one persistent launch;
 * out_rgb holds nframes frames back to back.  With p->surrogate the frames
 * run one after another (a surrogate pass and a trace launch each, the
 * network's inputs in each frame's own static frame); every camera must lie
 * in the network's domain (KS radius 4-50 M above the equatorial plane,
 * 0 <= a <= 0.99, M = 1), else ST_EUNSUPPORTED and nothing is written. */
int st_render_frames(st_context* ctx, int nframes, const st_camera* cams,
                     const st_spacetime* st, const st_render_params* p,
                     float* out_rgb, st_stats* stats);

/* ---- learned exit-direction surrogate -------------------------------------
 * No counterpart in the reference.  A 6 -> 256x4 -> 6 SiLU MLP (200,710
 * parameters) mapping (camera r in [4,50] M, inclination in [0,90] deg, spin
 * a in [0,0.99], unit ray direction in the static observer's radial / polar /
 * azimuthal frame) to the exit direction as two angles in the ray's own
 * plane (in-plane deflection from the launch direction, out-of-plane tilt; the
 * third direction output is unused), the first equatorial-crossing radius,
 * the redshift there and the log-variance of the angles.  Hidden layers run on the tensor
 * cores in BF16 with FP32 accumulation; training runs on the GPU.
 * With st_context_set_surrogate and p.surrogate = 1, st_render serves camera
 * rays the gate accepts (predicted std-dev < p.surrogate_sigma, not near the
 * critical curve, predicted not to cross the disc annulus, no gas) from the
 * network and integrates the rest (DRAFT rules, samples = 1). */
typedef struct st_surrogate st_surrogate;
int st_surrogate_create(st_surrogate** out, int device, unsigned long long seed);
void st_surrogate_destroy(st_surrogate* s);
int st_surrogate_num_params(void);
int st_surrogate_get_params(st_surrogate* s, float* host_params);
int st_surrogate_set_params(st_surrogate* s, const float* host_params);
/* normalised inputs x[n][6] -> outputs out[n][6] */
int st_surrogate_forward(st_surrogate* s, const float* x, int n, float* out);
/* the same, computed by the frame pass's tcgen05 / TMEM kernel (the one
 * st_render runs); ST_ECUDA if one of its bounded waits ran out */
int st_surrogate_forward_tc(st_surrogate* s, const float* x, int n, float* out);
/* loss (total, direction MSE, radius MSE, g MSE) and parameter gradient of
 * targets t[n][8] = (in-plane deflection, out-of-plane tilt, 0, radius, g-1,
 * direction mask, crossing mask, 0) */
int st_surrogate_loss_grad(st_surrogate* s, const float* x, const float* t, int n, float* loss4, float* grad);
/* n FP64-labelled Sobol samples kept on the device as the training set;
 * host copies are optional (raw[n][15] = r, theta, a, n0, n1, n2, flags,
 * steps, exit direction (3), first crossing radius or -1, launch coordinate
 * direction (3)) */
int st_surrogate_generate(st_surrogate* s, long long n, long long sobol_offset, double dt, float* host_x,
                          float* host_t, float* host_raw);
/* AdamW steps over the generated set; loss_hist[steps] optional */
int st_surrogate_train(st_surrogate* s, int steps, int batch, float lr, float weight_decay, float* loss_hist);
/* Attach (or detach, NULL) a surrogate to a context for p.surrogate = 1. */
int st_context_set_surrogate(st_context* ctx, st_surrogate* s);

/* Allocation-free camera-track render.  No counterpart in the reference.
 * For callers that cannot allocate device memory: a renderer embedded in an
 * engine whose device memory belongs to its own pool, or a real-time loop
 * that budgets memory up front and cannot afford the device-wide
 * synchronisation a cudaMalloc brings.  The caller passes its own device buffers: the sky as
 * float4 texels [sky_h][sky_w] (RGB + unused), the gas density (may be NULL
 * with vol NULL) and the output frames, float4 [nframes][height][width]; the
 * kernel's working memory (ray-queue head, counters, per-frame cameras and the
 * blackbody table) lives in a fixed 80 KiB device array of the library, held on
 * every device that loads it until exit.  Limits: nframes <= 64, blackbody
 * table <= 4096 entries (ST_ELIMIT beyond); DRAFT semantics, samples = 1,
 * RK4, no surrogate (ST_EUNSUPPORTED otherwise); the disc and volume are
 * checked as st_context_set_disc / st_context_set_volume check them.
 * The first call on a device resolves the array's address with that device
 * current: make that first call before any stream capture.  All calls share
 * the array (queue head and counters are cleared per call): calls whose GPU
 * work overlaps race and must be serialised by the caller.  `stream` is a
 * cudaStream_t (NULL = legacy default stream); the call returns after it
 * completes.  It calls no cudaMalloc, cudaFree or allocating library routine. */
int st_render_frames_noalloc(const float* dev_sky_rgba, int sky_w, int sky_h, const st_disc* disc,
                             const float* dev_density, const st_volume* vol, int nframes,
                             const st_camera* cams, const st_spacetime* st, const st_render_params* p,
                             float* dev_out_rgba, void* stream, st_stats* stats);

/* Measured FP32 fused-multiply-add ceiling of `device` (TFLOP/s, 2 flops per
 * FMA; the best of three timed launches of an FMA-chain kernel holding every
 * SM at full occupancy, `iters` x 128 FMAs per thread; ms_out may be NULL).
 * No counterpart in the reference: the denominator of the trace kernel's
 * roofline fraction, whose bound is FP32 issue. */
int st_measure_fp32_peak(int device, int iters, double* tflops, double* ms_out);

/* The camera's orthonormal Kerr-Schild tetrad (u, Ef, Er, Eu), each a
 * contravariant (t, x, y, z) 4-vector, boosted by the camera velocity. */
int st_camera_tetrad(const st_camera* cam, const st_spacetime* st, double out16[16]);

#ifdef __cplusplus
}
#endif
#endif /* SPACETIME_GB300_H */
