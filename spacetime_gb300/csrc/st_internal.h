// st_internal.h -- device-side parameter block and launch entry points shared
// by the host API (st_api.cu) and the trace kernels (st_trace.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/spacetime_gb300.h"

namespace st {

// The context's gas volume as another unit sees it (st_api.cu owns the
// context; the fluid solver writes the density texture in place).
struct CtxVolume {
  int device;
  cudaStream_t stream;
  float* d_vol;              // (nr, nphi, nz) column-major
  st_volume meta;            // grid and bounds; meta.density is null
  bool on;
};
int context_volume(st_context* ctx, CtxVolume* out);

// Counters written by the trace kernels (one slot each, 64-bit).
enum { CNT_STEPS = 0, CNT_FP64 = 1, CNT_GAS = 2, CNT_RAYS = 3, CNT_SURR = 4, CNT_QUEUE = 5,
       CNT_STATUS = 6, CNT_N = 8 };

// Per-frame camera of a batched track (st_render_frames).
struct FrameCam {
  double pos[3];
  double Ef[4], Er[4], Eu[4], U[4];
  double r_escape;
  int nmax;
  int pad;
};

// Everything a trace launch needs, passed by value as a __grid_constant__
// kernel parameter (about 1.2 KB, under the 4 KB limit).
struct TraceParams {
  // camera tetrad (FP64 host computation, src/preview.jl:93-198)
  double pos[3];
  double Ef[4], Er[4], Eu[4], U[4];
  double fov;
  int projection;
  double fisheye_rad;
  double ap_r, focus;
  int lens_seed;
  double lens_u0, lens_v0, lens_w;
  // frame / pass
  int width, height;
  int frame_stride;          // pixels per frame in the output (batched frames)
  double ju, jv, jw;
  int jseed;
  float weight;
  int first_pass;            // 1: assign instead of accumulate
  // spacetime and integration
  double M, a, rkill2;
  double r_escape, tspan;
  double hcoef, hcap, dt;
  int nmax;
  int order;                 // 4 (RK4) or 45 / 46 (adaptive Tsit5)
  double tol;                // adaptive tolerance
  double r_isco, E_isco, L_isco;
  int relativistic, exit_landing;
  // FP32_GUARDED policy
  double r_guard2, crit_band, b_crit, crit_r2;
  int renorm_every;
  int guard_df;              // guard steps in double-float on the FP32 pipe (ST_PREC_FP32_GUARDED_DF)
  // thin disc
  int disc_on, emitter;
  double disc_inner, disc_outer, disc_falloff;
  const float4* lut;         // [lut_size] RGB_
  int lut_size;
  int lut_stage;             // pixel kernel: copy the table to shared memory first
  double lut_tmin, lut_tmax;
  // volume
  int vol_on;
  const float* vol;
  int nr, nphi, nz;
  double ls_in, ls_out, zmax, emis, opac, ds_gas, vol_rb2;
  // sky
  const float4* sky;         // [sky_h][sky_w] RGB_
  int sky_w, sky_h;
  // procedural stars (starfield_mtl, src/metal.jl:652-724); strength 0 = off
  double star_strength, star_tw;  // star weight, sky-image weight under them
  double star_N, star_fill, star_sigma, star_flux;
  double star_g[3], star_conc, star_tmin, star_tspan;
  const float4* star_lut;    // [star_lut_size] RGB_, the stars' own white point
  int star_lut_size, star_seed;
  double star_lut_tmin, star_lut_tmax;
  // depth buckets (render_depth_mtl, src/metal.jl:1170-1175, 1425-1426,
  // 1489-1497, 1556-1563, 1687-1690): nb > 0 routes emission into
  // buckets[pixel][3 nb] by path length, log-spaced over [1.5, 120] M, and the
  // escaped sky into the last bucket
  int nb;
  float* buckets;
  // adaptive refinement (src/metal.jl:1640-1700, 2104-2240): per-pixel
  // (sum w L, sum w L^2, sum w graze, -) over the base passes, or null; and
  // the dispatch box of a refinement pass (box_cols = 0: the whole frame)
  float4* stat;
  int box_col0, box_row0, box_cols, box_rows;
  // layered engine's disc / gas layer (src/metal.jl:1096-1135, 1204-1212,
  // 1616-1626; Schwarzschild, DRAFT): layer = 1 traces only emission and
  // transmittance, culling rays the deflection fan proves stay outside
  // layer_gate; er = the static frame's radial axis at the camera
  int layer;
  double layer_gate;
  // ring pass of the layer (src/metal.jl:1105-1127): ring_rmin > 0 keeps only
  // the rays whose fan periapsis falls below it (the strongly wound rays of
  // the photon ring) and writes transparency for the rest
  double ring_rmin;
  double er[4];
  const float4* fan;         // [fan_n] (escaped, cos, sin, periapsis)
  int fan_n;
  // per-pixel shutter (src/metal.jl:829-857): seed 0 = off; the camera pose
  // at the far end of this pass's shutter stratum
  int shutter_seed;
  double pos_end[3], Ef_end[4], Er_end[4], Eu_end[4], U_end[4];
  // outputs
  float4* out;               // [height][width] (x frames)
  st_ray_diag* diag;         // optional
  unsigned long long* counters;  // CNT_N slots
  // pixel schedule over a compacted list (surrogate fallback rays)
  const int* pix_list;       // optional pixel indices (device)
  const int* n_list;         // their count (device)
  // FP32_GUARDED pixel schedule: rays stop before their first FP64 guard step
  // and are saved here (defer_cap states of the trace unit's ray-state size,
  // in the order their warps reached it); a resume kernel over the saved
  // rays runs the FP64 steps in full warps.  Null: guard steps inline.
  void* defer_state;
  unsigned int* defer_count;
  int defer_cap;
  // pixel schedule of one full frame: block b traces tile tile_order[b]
  // (row-major over the grid); null = raster order
  const int* tile_order;
  // persistent schedule
  const FrameCam* frames;    // optional per-frame cameras (device)
  int n_frames;              // frames in the table (pixel schedule: grid z)
  int n_rays;                // rays in the queue (frames x pixels)
  int chunk_steps;
  int refill_window;         // rays a warp takes from the queue at a time (multiple of 32)
  unsigned int* queue;       // queue head (device)
  long long budget_iters;    // per-warp loop bound of the persistent kernel
  // single-precision copies of the parameters the per-step code reads, so a
  // float variant never converts from double inside its loop (on GB300 every
  // double -> float conversion issues on the FP64 pipe)
  struct Flt {
    // M and a as double-float pairs (hi + lo = the double) for the
    // double-float guard steps
    float M_lo, a_lo;
    float M, a, rkill2, vol_rb2, hcap, dt, hcoef, tspan, ds_gas, zmax, r_isco, E_isco, L_isco, opac, emis, disc_inner, disc_outer, disc_falloff, lut_tmin, lut_tmax, ls_in, ls_out, crit_r2, r_guard2, tol, layer_gate;
    // float step rule without per-step divisions: hcoef / M and 1 / max(rkill2, 1e-6)
    float hcoef_m, inv_rkill2;
    // float gas-grid index scales: (nr - 1) / (ls_out - ls_in), nphi / 2 pi,
    // (nz - 1) / (2 zmax)
    float vol_sr, vol_sp, vol_sz;
    // blackbody table index scale (lut_size - 1) / (lut_tmax - lut_tmin)
    float lut_sc;
    // Kerr step shrink: rkill2 / max(rkill2, 1e-6), 0.12 dt, 0.88 dt
    float rkill_n, dt_lo, dt_span;
    // gas grid radial coordinate from log2 s: vol_sr ln 2, -ls_in vol_sr, nr - 1
    float vol_sr2, vol_r0, vol_rmax;
    // gas emission: 1 / (2M), 100 emis, opac ds_gas log2(e)
    float inv_2m, emis100, opds_l2;
  } f;
};

// Fill TraceParams::f from the double fields (host, after they are set).
inline void fill_float_copies(TraceParams* p) {
  p->f.M = (float)p->M;
  p->f.a = (float)p->a;
  p->f.M_lo = (float)(p->M - (double)p->f.M);
  p->f.a_lo = (float)(p->a - (double)p->f.a);
  p->f.rkill2 = (float)p->rkill2;
  p->f.vol_rb2 = (float)p->vol_rb2;
  p->f.hcap = (float)p->hcap;
  p->f.dt = (float)p->dt;
  p->f.hcoef = (float)p->hcoef;
  p->f.tspan = (float)p->tspan;
  p->f.ds_gas = (float)p->ds_gas;
  p->f.zmax = (float)p->zmax;
  p->f.r_isco = (float)p->r_isco;
  p->f.E_isco = (float)p->E_isco;
  p->f.L_isco = (float)p->L_isco;
  p->f.opac = (float)p->opac;
  p->f.emis = (float)p->emis;
  p->f.disc_inner = (float)p->disc_inner;
  p->f.disc_outer = (float)p->disc_outer;
  p->f.disc_falloff = (float)p->disc_falloff;
  p->f.lut_tmin = (float)p->lut_tmin;
  p->f.lut_tmax = (float)p->lut_tmax;
  p->f.ls_in = (float)p->ls_in;
  p->f.ls_out = (float)p->ls_out;
  p->f.crit_r2 = (float)p->crit_r2;
  p->f.r_guard2 = (float)p->r_guard2;
  p->f.tol = (float)p->tol;
  p->f.layer_gate = (float)p->layer_gate;
  p->f.hcoef_m = (float)(p->hcoef / p->M);
  p->f.inv_rkill2 = (float)(1.0 / (p->rkill2 > 1e-6 ? p->rkill2 : 1e-6));
  p->f.vol_sr = p->ls_out > p->ls_in ? (float)((p->nr - 1) / (p->ls_out - p->ls_in)) : 0.f;
  p->f.vol_sp = (float)(p->nphi / 6.283185307179586);
  p->f.vol_sz = p->zmax > 0.0 ? (float)((p->nz - 1) / (2.0 * p->zmax)) : 0.f;
  p->f.lut_sc = p->lut_tmax > p->lut_tmin ? (float)((p->lut_size - 1) / (p->lut_tmax - p->lut_tmin)) : 0.f;
  const double rkd = p->rkill2 > 1e-6 ? p->rkill2 : 1e-6;
  p->f.rkill_n = (float)(p->rkill2 / rkd);
  p->f.dt_lo = (float)(0.12 * p->dt);
  p->f.dt_span = (float)(0.88 * p->dt);
  const double sr = p->ls_out > p->ls_in ? (p->nr - 1) / (p->ls_out - p->ls_in) : 0.0;
  p->f.vol_sr2 = (float)(sr * 0.6931471805599453);
  p->f.vol_r0 = (float)(-p->ls_in * sr);
  p->f.vol_rmax = (float)(p->nr - 1);
  p->f.inv_2m = (float)(1.0 / (2.0 * p->M));
  p->f.emis100 = (float)(100.0 * p->emis);
  p->f.opds_l2 = (float)(p->opac * p->ds_gas * 1.4426950408889634);
}

// Variant key of the compiled kernels (the reference's Val{...} switches,
// src/metal.jl:759-763, plus precision and schedule).
struct Variant {
  int prec;       // ST_PREC_*
  int kerr;       // a != 0
  int vol;        // volume on (DRAFT only)
  int sem;        // ST_SEM_*
  int sched;      // ST_SCHED_*
};

// Surrogate frame constants: the static observer's frame at the camera,
// lowered (covariant) so g(q, E) is a plain dot product, and the camera's
// unit position, which with each ray's launch direction spans the ray plane
// the network's angles live in.
struct SurFrame {
  double Ul[4], E1l[4], E2l[4], E3l[4];
  double r, th;
  double xh[3];  // unit Cartesian position of the camera (the ray plane's first axis)
  double sigma_max;
};

// Surrogate pass over the frame (st_surrogate.cu): network inputs, batched
// inference, and the gate, which writes served pixels to p.out and compacts
// the rest into list / *count (device).  Returns an ST_* status.
int surrogate_frame(struct ::st_surrogate* s, const TraceParams& p, const Variant& v, const SurFrame& f,
                    int* list, int* count, cudaStream_t stream);

// Layered engine (st_layered.cu).
namespace lay {
// One deflection fan: a TraceParams with the fan camera's tetrad (at (r,0,0)
// looking along +x, right +y) and no disc, gas or layer, so each entry is
// what the trace kernel computes for that ray.
struct FanParams {
  TraceParams p;
  float4* out;       // [n] (escaped, cos theta_f, sin theta_f, periapsis)
  int n;
  int band;          // 0: psi = pi k / (n - 1); 1: across band_lohi
  const float* band_lohi;
};
// The composite's fan and layer.
struct CompParams {
  const float4* fan;
  int n;
  const float4* fine;
  int nf;
  const float* band;
  const float4* layer;  // [lh][lw] premultiplied RGB + transmittance, or null (transparent)
  int lw, lh;
  const float4* ring;   // [rh][rw] the ring pass's layer, or null
  int rw, rh;
  float ring_rmin;      // blend toward the ring layer below this fan periapsis
};
}  // namespace lay
cudaError_t launch_skyfan(int prec, const lay::FanParams& fp, cudaStream_t stream);
cudaError_t launch_fanband(const float4* fan, int n, int pad, float* band, cudaStream_t stream);
cudaError_t launch_composite(int prec, const TraceParams& p, const lay::CompParams& cp, cudaStream_t stream);
// Fill a layer with transparency (0, 0, 0, 1).
cudaError_t launch_fill_transparent(float4* layer, size_t n, cudaStream_t stream);

// The white-balance-free CIE blackbody colour of temperature T, normalised to
// its largest channel (src/blackbody.jl:15-35); host, double precision.
void host_blackbody(double T, double* rgb);

// Launch one trace pass; returns a cudaError_t.
cudaError_t launch_trace(const Variant& v, const TraceParams& p, int block_x, int block_y,
                         int num_sms, cudaStream_t stream);

// Pack the float4 framebuffer into RGB float32 (3, W, H) for download.
cudaError_t launch_pack_rgb(const float4* fb, float* rgb, int n, cudaStream_t stream);

// Number of registers the pixel kernel of a variant uses (for reporting).
int variant_registers(const Variant& v);

// Bytes of one saved ray state of the FP32_GUARDED deferral (defer_state).
size_t guarded_ray_state_bytes();

}  // namespace st
