// st_noalloc.cu -- st_render_frames_noalloc: the batched camera-track render
// (persistent trace kernel with its device ray queue) for callers that must
// not allocate device memory.
//
// Who needs it: code that runs inside another runtime's memory discipline --
// a renderer embedded in a game engine or compositor whose device memory is
// all owned by its own pool allocator, or a real-time loop that has budgeted
// its memory up front and treats any allocation (cudaMalloc synchronises the
// device) as a stall.  Such a caller already owns the sky texels and the
// output frames; what it cannot provide is the persistent kernel's own
// working memory, so that lives here, in a fixed file-scope device array.
//
// The scratch array (NOALLOC_SCRATCH_BYTES, 80 KiB, held on every device that
// loads the library until the process exits) holds the ray-queue head, the
// launch counters, up to NOALLOC_MAX_FRAMES per-frame cameras and a blackbody
// table of up to NOALLOC_MAX_LUT entries.  All calls share it, and it keeps
// the previous call's contents: the queue head and counters are cleared on
// every call.  Calls whose GPU work overlaps (two streams, or two host threads)
// race on it and must be serialised by the caller.  The call is synchronous:
// it waits for the caller's stream before it returns.
#include <cuda_runtime.h>

#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "st_internal.h"

namespace st {
cudaError_t launch_trace(const Variant& v, const TraceParams& p, int bx, int by, int num_sms, cudaStream_t s);
}

namespace {

constexpr int NOALLOC_MAX_FRAMES = 64;
constexpr int NOALLOC_MAX_LUT = 4096;
constexpr size_t OFF_COUNTERS = 0;                                   // CNT_N x u64
constexpr size_t OFF_QUEUE = 256;                                    // u32 queue head
constexpr size_t OFF_FRAMES = 512;                                   // FrameCam[MAX_FRAMES]
constexpr size_t OFF_LUT = OFF_FRAMES + ((NOALLOC_MAX_FRAMES * sizeof(st::FrameCam) + 255) / 256) * 256;
constexpr size_t NOALLOC_SCRATCH_BYTES = OFF_LUT + NOALLOC_MAX_LUT * sizeof(float4);
static_assert(NOALLOC_SCRATCH_BYTES <= 80 * 1024, "scratch budget");

static __device__ __align__(256) unsigned char g_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_scratch per device, resolved once with that device
// current.  In host code the name g_scratch is only a host-side stand-in.
constexpr int MAX_DEVICES = 64;
void* g_scratch_addr[MAX_DEVICES] = {nullptr};

}  // namespace

// Tetrad and rule helpers of the regular path (st_api.cu), reused through a
// render-independent entry: fill a TraceParams for one camera.
namespace st {
int fill_frame_params(const st_camera* cam, const st_spacetime* stp, const st_render_params* rp, TraceParams* p);
}

extern "C" int st_render_frames_noalloc(const float* dev_sky_rgba, int sky_w, int sky_h, const st_disc* disc,
                                        const float* dev_density, const st_volume* vol, int nframes,
                                        const st_camera* cams, const st_spacetime* stp,
                                        const st_render_params* rp, float* dev_out_rgba, void* stream,
                                        st_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!dev_sky_rgba || sky_w < 2 || sky_h < 2 || !cams || !stp || !rp || !dev_out_rgba || nframes <= 0)
    return ST_EINVAL;
  if (nframes > NOALLOC_MAX_FRAMES) return ST_ELIMIT;
  // the same rule checks as st_render_frames and the context setters
  if (rp->semantics != ST_SEM_DRAFT || rp->samples != 1 || rp->surrogate) return ST_EUNSUPPORTED;
  if (rp->order != 0 && rp->order != 4) return ST_EUNSUPPORTED;  // the persistent kernel integrates with RK4
  if (disc && disc->emitter != ST_EMIT_KEPLER && disc->emitter != ST_EMIT_KS_EXACT) return ST_EINVAL;
  const int lut_n = (disc && disc->table_size > 0) ? disc->table_size : 1024;
  if (lut_n > NOALLOC_MAX_LUT || lut_n < 2) return ST_ELIMIT;
  if (vol && (!dev_density || vol->nr < 2 || vol->nphi < 1 || vol->nz < 2)) return ST_EINVAL;
  if (vol && (!(vol->log_s_out > vol->log_s_in) || !(vol->z_max > 0.0f))) return ST_EINVAL;
  if (vol && (size_t)vol->nr * vol->nphi * vol->nz >= ((size_t)1 << 31)) return ST_EINVAL;  // 32-bit grid offsets
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return ST_ECUDA;
  // one-time set-up per device (the first call on a device: keep it outside
  // any stream capture)
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) return ST_ECUDA;
    g_scratch_addr[dev] = ptr;
  }
  unsigned char* base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t npix = (size_t)rp->width * rp->height;
  if (rp->width <= 0 || rp->height <= 0 || npix * (size_t)nframes > ((size_t)1 << 31)) return ST_EINVAL;

  // per-frame cameras and the frame-independent parameters
  st::TraceParams p;
  int rc = st::fill_frame_params(&cams[0], stp, rp, &p);
  if (rc != ST_OK) return rc;
  // host staging (host memory is outside the no-device-allocation contract;
  // kept off the stack, whose size an embedding thread may limit)
  std::vector<st::FrameCam> fc(nframes);
  int nmax_max = 0;
  for (int f = 0; f < nframes; ++f) {
    st::TraceParams q;
    rc = st::fill_frame_params(&cams[f], stp, rp, &q);
    if (rc != ST_OK) return rc;
    std::memcpy(fc[f].pos, q.pos, sizeof q.pos);
    std::memcpy(fc[f].Ef, q.Ef, sizeof q.Ef);
    std::memcpy(fc[f].Er, q.Er, sizeof q.Er);
    std::memcpy(fc[f].Eu, q.Eu, sizeof q.Eu);
    std::memcpy(fc[f].U, q.U, sizeof q.U);
    fc[f].r_escape = q.r_escape;
    fc[f].nmax = q.nmax;
    fc[f].pad = 0;
    nmax_max = q.nmax > nmax_max ? q.nmax : nmax_max;
  }
  // blackbody table into scratch
  std::vector<float4> lut(lut_n);
  const double tmin = (disc && disc->table_size > 0) ? disc->table_min : 500.0;
  const double tmax = (disc && disc->table_size > 0) ? disc->table_max : 30000.0;
  if (!(tmax > tmin)) return ST_EINVAL;
  {
    double ref[3];
    st::host_blackbody(disc && disc->wb_temperature > 0.0 ? disc->wb_temperature : 6500.0, ref);
    for (int i = 0; i < lut_n; ++i) {
      double c[3];
      st::host_blackbody(std::fmax(tmin + (tmax - tmin) * i / (lut_n - 1), 1.0), c);
      lut[i] = make_float4((float)(c[0] / ref[0]), (float)(c[1] / ref[1]), (float)(c[2] / ref[2]), 0.f);
    }
  }
  unsigned long long* counters = reinterpret_cast<unsigned long long*>(base + OFF_COUNTERS);
  unsigned int* queue = reinterpret_cast<unsigned int*>(base + OFF_QUEUE);
  st::FrameCam* frames = reinterpret_cast<st::FrameCam*>(base + OFF_FRAMES);
  float4* dlut = reinterpret_cast<float4*>(base + OFF_LUT);
  if (cudaMemsetAsync(counters, 0, st::CNT_N * sizeof(unsigned long long), s) != cudaSuccess) return ST_ECUDA;
  if (cudaMemsetAsync(queue, 0, sizeof(unsigned int), s) != cudaSuccess) return ST_ECUDA;
  if (cudaMemcpyAsync(frames, fc.data(), nframes * sizeof(st::FrameCam), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return ST_ECUDA;
  if (cudaMemcpyAsync(dlut, lut.data(), lut_n * sizeof(float4), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return ST_ECUDA;

  // disc, gas, sky and outputs
  p.disc_on = (disc && disc->inner > 0.0 && disc->outer > disc->inner) ? 1 : 0;
  p.emitter = disc ? disc->emitter : ST_EMIT_KS_EXACT;
  p.disc_inner = disc ? disc->inner : 0.0;
  p.disc_outer = disc ? disc->outer : 0.0;
  p.disc_falloff = disc ? disc->falloff : 0.0;
  p.lut = dlut;
  p.lut_size = lut_n;
  p.lut_tmin = tmin;
  p.lut_tmax = tmax;
  p.vol_on = vol ? 1 : 0;
  if (vol) {
    p.vol = dev_density;
    p.nr = vol->nr; p.nphi = vol->nphi; p.nz = vol->nz;
    p.ls_in = vol->log_s_in; p.ls_out = vol->log_s_out; p.zmax = vol->z_max;
    p.emis = vol->emission_scale; p.opac = vol->opacity_scale;
    const int stride = vol->march_stride < 1 ? 1 : (vol->march_stride > 16 ? 16 : vol->march_stride);
    p.ds_gas = stride * rp->dt;
    const double so = std::exp((double)vol->log_s_out);
    p.vol_rb2 = so * so + (double)vol->z_max * vol->z_max;
  } else {
    p.vol_rb2 = -1.0;
  }
  p.sky = reinterpret_cast<const float4*>(dev_sky_rgba);
  p.sky_w = sky_w;
  p.sky_h = sky_h;
  p.out = reinterpret_cast<float4*>(dev_out_rgba);
  p.diag = nullptr;
  p.counters = counters;
  p.queue = queue;
  p.frames = frames;
  p.frame_stride = (int)npix;
  p.ju = 0.5; p.jv = 0.5; p.jw = 0.0; p.jseed = 0;
  p.weight = 1.0f;
  p.first_pass = 1;
  const long long tiles = (long long)((rp->width + 7) / 8) * ((rp->height + 3) / 4);
  // the queue counts rays of whole 8x4 tiles in a 32-bit int
  if (tiles * 32 * nframes > (long long)INT_MAX) return ST_EINVAL;
  p.n_rays = (int)(tiles * 32 * nframes);
  p.chunk_steps = rp->chunk_steps > 0 ? rp->chunk_steps : 32;
  p.budget_iters = ((long long)p.n_rays + 32) * ((long long)nmax_max / p.chunk_steps + 2);
  p.nmax = nmax_max;
  st::Variant v;
  v.prec = rp->precision == ST_PREC_FP32_GUARDED_DF ? ST_PREC_FP32_GUARDED : rp->precision;
  v.kerr = stp->a != 0.0 ? 1 : 0;
  v.vol = p.vol_on;
  v.sem = ST_SEM_DRAFT;
  v.sched = ST_SCHED_PERSISTENT;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ST_ECUDA;
  st::fill_float_copies(&p);
  if (st::launch_trace(v, p, 0, 0, nsm, s) != cudaSuccess) return ST_ECUDA;
  unsigned long long cnt[st::CNT_N];
  if (cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, s) != cudaSuccess) return ST_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return ST_ECUDA;
  const int status = cnt[st::CNT_STATUS] ? (int)cnt[st::CNT_STATUS] : ST_OK;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->rays = cnt[st::CNT_RAYS];
    stats->steps = cnt[st::CNT_STEPS];
    stats->fp64_steps = cnt[st::CNT_FP64];
    stats->gas_samples = cnt[st::CNT_GAS];
    stats->launches = 1;
    stats->status = status;
    stats->h2d_bytes = sizeof(st::TraceParams) + nframes * sizeof(st::FrameCam) + lut_n * sizeof(float4);
    stats->d2h_bytes = sizeof cnt;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return status;
}
