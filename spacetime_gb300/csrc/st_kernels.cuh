// st_kernels.cuh -- the trace kernels (per-pixel and persistent schedules)
// and their launchers, instantiated per precision in st_trace_*.cu.
#pragma once

#include <cstdlib>

#include "st_trace.cuh"

// Minimum resident blocks per SM requested from ptxas (register budget);
// set per translation unit by the build.
#ifndef ST_MINB
#define ST_MINB 1
#endif
// The adaptive Tsit5 modes (order 45 / 46) hold more state per ray; they keep
// the budget of at most 5 blocks.
#ifndef ST_MINB_ADAPTIVE
#define ST_MINB_ADAPTIVE (ST_MINB < 5 ? ST_MINB : 5)
#endif

namespace st {

__device__ __forceinline__ void flush_counters(const TraceParams& p, unsigned long long steps,
                                               unsigned long long f64, unsigned long long gas,
                                               unsigned long long rays) {
  // warp-aggregated atomics on the launch counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    steps += __shfl_down_sync(0xffffffffu, steps, o);
    f64 += __shfl_down_sync(0xffffffffu, f64, o);
    gas += __shfl_down_sync(0xffffffffu, gas, o);
    rays += __shfl_down_sync(0xffffffffu, rays, o);
  }
  const unsigned lin = threadIdx.y * blockDim.x + threadIdx.x;  // lane = linear index mod 32
  if ((lin & 31) == 0 && p.counters) {
    if (steps) atomicAdd(p.counters + CNT_STEPS, steps);
    if (f64) atomicAdd(p.counters + CNT_FP64, f64);
    if (gas) atomicAdd(p.counters + CNT_GAS, gas);
    if (rays) atomicAdd(p.counters + CNT_RAYS, rays);
  }
}

// One thread per pixel over a 2-D grid of tiles (blockDim.x * blockDim.y a
// multiple of 32; threads are linearised so a warp covers a compact tile).
template <int PREC, int KERR, int VOL, int SEM, int ORD = 4, int DEPTH = 0, int DEFER = 0>
__global__ void __launch_bounds__(128, ORD == 4 ? ST_MINB : ST_MINB_ADAPTIVE) trace_pixel_kernel(const __grid_constant__ TraceParams p) {
  using R = typename RealOf<PREC>::T;
  if (p.lut_stage) {
    // the blackbody table into shared memory, once per block (16 KiB for the
    // default 1024 entries), before any thread takes a ray
    const int lin = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    for (int k = lin; k < p.lut_size; k += nthr) st_lut_smem[k] = __ldg(p.lut + k);
    __syncthreads();
  }
  int tbx = blockIdx.x, tby = blockIdx.y;
  if (p.tile_order) {  // a full frame dispatched centre first
    const int t = __ldg(p.tile_order + blockIdx.y * gridDim.x + blockIdx.x);
    tby = t / (int)gridDim.x;
    tbx = t - tby * (int)gridDim.x;
  }
  int i = tbx * blockDim.x + threadIdx.x;
  int j = tby * blockDim.y + threadIdx.y;
  if (p.box_cols > 0) {  // a refinement pass over its box only
    if (i >= p.box_cols || j >= p.box_rows) i = p.width;  // idle
    i += p.box_col0;
    j += p.box_row0;
  }
  if (p.pix_list) {  // 1-D over a compacted pixel list
    const int t = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    if (t < *p.n_list) {
      const int pix = p.pix_list[t];
      i = pix % p.width;
      j = pix / p.width;
    } else {
      i = p.width;  // idle
      j = 0;
    }
  }
  unsigned long long steps = 0, f64 = 0, gas = 0, rays = 0;
  if (i < p.width && j < p.height) {
    RayState<R> st;
    CamView cam{p.pos, p.Ef, p.Er, p.Eu, p.U, p.r_escape, p.nmax};
    int base = 0;
    if (p.frames) {  // batched track: one frame per grid z-slice
      const FrameCam& fc = p.frames[blockIdx.z];
      cam = CamView{fc.pos, fc.Ef, fc.Er, fc.Eu, fc.U, fc.r_escape, fc.nmax};
      base = blockIdx.z * p.frame_stride;
    }
    init_ray<PREC, KERR, SEM>(p, cam, i, j, st);
    st.pix = base + j * p.width + i;
    if (final_at_launch<SEM>(p, st.flags)) st.flags |= ST_RAY_CAPTURED;
    else
      while (!step_ray<PREC, KERR, VOL, SEM, ORD, DEPTH, DEFER>(p, st)) {
      }
    bool deferred = false;
    if constexpr (DEFER) deferred = (st.flags & ST_RAY_DEFER) != 0;
    if (!deferred) {
      finish_ray<PREC, KERR, SEM, DEPTH>(p, st, st.pix, p.frames ? st.pix : j * p.width + i);
      steps = st.steps; f64 = st.fp64_steps; gas = st.gas; rays = 1;
    }
    if constexpr (DEFER) {
      // save the suspended ray (its counters travel with it); one atomic per
      // warp, consecutive slots for the warp's deferring lanes
      const unsigned act = __activemask();
      const unsigned want = __ballot_sync(act, deferred);
      if (deferred) {
        const int leader = __ffs(want) - 1;
        const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
        unsigned slot0 = 0;
        if (lane == leader) slot0 = atomicAdd(p.defer_count, (unsigned)__popc(want));
        slot0 = __shfl_sync(want, slot0, leader);
        const unsigned slot = slot0 + __popc(want & ((1u << lane) - 1u));
        if (slot < (unsigned)p.defer_cap) {
          st.flags &= ~ST_RAY_DEFER;
          static_cast<RayState<R>*>(p.defer_state)[slot] = st;
        } else if (p.counters) {
          atomicMax(p.counters + CNT_STATUS, (unsigned long long)ST_ECUDA);  // cannot happen: cap >= rays
        }
      }
    }
  }
  flush_counters(p, steps, f64, gas, rays);
}

// FP32_GUARDED: the rays the pixel kernel saved before their first FP64 step,
// one thread each, so the FP64 steps they start with run in full warps; each
// continues to its end with the guard steps inline.
template <int KERR, int VOL, int SEM>
__global__ void __launch_bounds__(128, ST_MINB) trace_resume_kernel(const __grid_constant__ TraceParams p) {
  using R = float;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long steps = 0, f64 = 0, gas = 0, rays = 0;
  if (t < min(*p.defer_count, (unsigned)p.defer_cap)) {
    RayState<R> st = static_cast<const RayState<R>*>(p.defer_state)[t];
    while (!step_ray<ST_PREC_FP32_GUARDED, KERR, VOL, SEM, 4, 0, 0>(p, st)) {
    }
    finish_ray<ST_PREC_FP32_GUARDED, KERR, SEM, 0>(p, st, st.pix, st.pix);
    steps = st.steps; f64 = st.fp64_steps; gas = st.gas; rays = 1;
  }
  flush_counters(p, steps, f64, gas, rays);
}

// Persistent schedule: each warp pulls rays from a device queue; a lane whose
// ray retires is refilled at the next chunk boundary (warp-ballot refill), so
// short escaping rays do not idle lanes while photon-ring rays run on.  Queue
// indices are ordered in 8x4 pixel tiles.  A warp takes the queue in windows of
// refill_window consecutive indices (whole tiles: a strip of neighbouring
// tiles) and refills its lanes from its own window before it takes the next,
// so a refilled lane traces a neighbour of the rays still running beside it
// (refill_window = 32: every refill from the global queue, as one tile).
// The outer loop is bounded by budget_iters; on exhaustion the kernel records
// ST_EBUDGET in the status counter and returns.
template <int PREC, int KERR, int VOL, int SEM>
__global__ void __launch_bounds__(128, ST_MINB) trace_persistent_kernel(const __grid_constant__ TraceParams p) {
  using R = typename RealOf<PREC>::T;
  const unsigned FULL = 0xffffffffu;
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
  const int tiles_x = (p.width + 7) >> 3;
  const int tiles_y = (p.height + 3) >> 2;
  const int per_frame = tiles_x * tiles_y * 32;
  RayState<R> st;
  bool active = false, exhausted = false, done = false;
  int out_idx = 0;
  unsigned long long steps = 0, f64 = 0, gas = 0, rays = 0;
  const unsigned nr = (unsigned)p.n_rays;
  const unsigned win = p.refill_window >= 32 ? (unsigned)(p.refill_window & ~31) : 32u;
  unsigned w_next = 0, w_end = 0;  // this warp's window of the queue (warp-uniform)
  for (long long it = 0; it < p.budget_iters; ++it) {
    const unsigned idle = __ballot_sync(FULL, !active);
    if (idle && !exhausted) {
      const unsigned need = (unsigned)__popc(idle);
      const unsigned rank = __popc(idle & ((1u << lane) - 1u));
      unsigned idx = 0xffffffffu;
      // first from the window, then from a fresh one
      const unsigned take = min(need, w_end - w_next);
      if (!active && rank < take) idx = w_next + rank;
      w_next += take;
      if (take < need) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(p.queue, win);
        base = __shfl_sync(FULL, base, 0);
        if (base >= nr) {
          exhausted = true;
        } else {
          w_next = base;
          w_end = min(base + win, nr);
          const unsigned t2 = min(need - take, w_end - w_next);
          if (!active && rank >= take && rank - take < t2) idx = w_next + (rank - take);
          w_next += t2;
        }
      }
      if (!active) {
        if (idx < nr) {
          const int frame = (int)idx / per_frame;
          const int w = (int)idx - frame * per_frame;
          const int tile = w >> 5, within = w & 31;
          const int ti = tile % tiles_x, tj = tile / tiles_x;
          const int i = ti * 8 + (within & 7), j = tj * 4 + (within >> 3);
          if (i < p.width && j < p.height) {
            CamView cam{p.pos, p.Ef, p.Er, p.Eu, p.U, p.r_escape, p.nmax};
            if (p.frames) {
              const FrameCam& fc = p.frames[frame];
              cam = CamView{fc.pos, fc.Ef, fc.Er, fc.Eu, fc.U, fc.r_escape, fc.nmax};
            }
            init_ray<PREC, KERR, SEM>(p, cam, i, j, st);
            out_idx = frame * p.frame_stride + j * p.width + i;
            st.pix = out_idx;
            active = true;
          }
        }
      }
    }
    // leave only when the queue is drained and no lane holds a ray (a refill
    // that drew only off-frame slots loops back for more)
    if (!__any_sync(FULL, active)) {
      if (exhausted) { done = true; break; }
      continue;
    }
    if (active) {
      bool fin = final_at_launch<SEM>(p, st.flags);
      if (fin) st.flags |= ST_RAY_CAPTURED;
      for (int s = 0; s < p.chunk_steps && !fin; ++s) fin = step_ray<PREC, KERR, VOL, SEM>(p, st);
      if (fin) {
        finish_ray<PREC, KERR, SEM>(p, st, out_idx, out_idx);
        steps += st.steps; f64 += st.fp64_steps; gas += st.gas; rays += 1;
        active = false;
      }
    }
  }
  flush_counters(p, steps, f64, gas, rays);
  if (!done && lane == 0 && p.counters) atomicMax(p.counters + CNT_STATUS, (unsigned long long)ST_EBUDGET);
}

// SPACETIME_GB300_LUT_SMEM=1: the plain pixel kernels stage the blackbody
// table in shared memory instead of reading it through L1.
inline bool lut_staging() {
  const char* e = std::getenv("SPACETIME_GB300_LUT_SMEM");
  return e && e[0] == '1';
}

template <int PREC, int KERR, int VOL, int SEM>
cudaError_t launch_variant(const TraceParams& p, int sched, int bx, int by, int num_sms, cudaStream_t s) {
  if (sched == ST_SCHED_PERSISTENT) {
    auto k = trace_persistent_kernel<PREC, KERR, VOL, SEM>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    k<<<num_sms * per_sm, 128, 0, s>>>(p);
  } else {
    if (bx <= 0 || by <= 0 || bx * by != 128) { bx = 16; by = 8; }
    dim3 block(bx, by);
    dim3 grid((p.width + bx - 1) / bx, (p.height + by - 1) / by);
    if (p.box_cols > 0) grid = dim3((p.box_cols + bx - 1) / bx, (p.box_rows + by - 1) / by);
    if (p.pix_list) grid = dim3((unsigned)(((long long)p.width * p.height + 127) / 128), 1);
    else if (p.frames) grid.z = (unsigned)(p.n_frames > 0 ? p.n_frames : 1);
    if constexpr (SEM == ST_SEM_DRAFT) {
      // depth buckets: their own instantiation, so the plain kernels carry none of it
      if (p.nb > 0) { trace_pixel_kernel<PREC, KERR, VOL, SEM, 4, 1><<<grid, block, 0, s>>>(p); return cudaGetLastError(); }
    }
    if constexpr (SEM == ST_SEM_DRAFT && PREC != ST_PREC_FP32_GUARDED) {
      if (p.order == 45) { trace_pixel_kernel<PREC, KERR, VOL, SEM, 45><<<grid, block, 0, s>>>(p); return cudaGetLastError(); }
      if (p.order == 46) { trace_pixel_kernel<PREC, KERR, VOL, SEM, 46><<<grid, block, 0, s>>>(p); return cudaGetLastError(); }
    }
    if constexpr (PREC == ST_PREC_FP32_GUARDED) {
      if (p.defer_state && p.defer_count && p.defer_cap > 0) {
        // guard steps gathered into full warps: stop each ray before its first
        // FP64 step, then resume the saved rays one per thread
        cudaError_t e = cudaMemsetAsync(p.defer_count, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) return e;
        trace_pixel_kernel<PREC, KERR, VOL, SEM, 4, 0, 1><<<grid, block, 0, s>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        trace_resume_kernel<KERR, VOL, SEM><<<(unsigned)((p.defer_cap + 127) / 128), 128, 0, s>>>(p);
        return cudaGetLastError();
      }
    }
    if (lut_staging() && p.lut && p.lut_size > 0 && p.lut_size <= 3072 && (p.vol_on || p.disc_on)) {
      // the blackbody table read from shared memory (at most 48 KiB)
      TraceParams q = p;
      q.lut_stage = 1;
      trace_pixel_kernel<PREC, KERR, VOL, SEM><<<grid, block, (size_t)p.lut_size * sizeof(float4), s>>>(q);
      return cudaGetLastError();
    }
    trace_pixel_kernel<PREC, KERR, VOL, SEM><<<grid, block, 0, s>>>(p);
  }
  return cudaGetLastError();
}

template <int PREC>
int variant_regs_impl(int kerr, int vol, int sem) {
  cudaFuncAttributes a{};
  cudaError_t e;
  if (sem == ST_SEM_RENDER) e = cudaFuncGetAttributes(&a, trace_pixel_kernel<PREC, 0, 0, ST_SEM_RENDER>);
  else if (kerr && vol) e = cudaFuncGetAttributes(&a, trace_pixel_kernel<PREC, 1, 1, ST_SEM_DRAFT>);
  else if (kerr) e = cudaFuncGetAttributes(&a, trace_pixel_kernel<PREC, 1, 0, ST_SEM_DRAFT>);
  else if (vol) e = cudaFuncGetAttributes(&a, trace_pixel_kernel<PREC, 0, 1, ST_SEM_DRAFT>);
  else e = cudaFuncGetAttributes(&a, trace_pixel_kernel<PREC, 0, 0, ST_SEM_DRAFT>);
  return e == cudaSuccess ? a.numRegs : -1;
}

// Per-precision dispatch over the remaining switches.  RENDER semantics is
// Schwarzschild-only and has no volume (as the reference's CPU renderer).
template <int PREC>
cudaError_t launch_prec(const Variant& v, const TraceParams& p, int bx, int by, int num_sms, cudaStream_t s) {
  if (v.sem == ST_SEM_RENDER) return launch_variant<PREC, 0, 0, ST_SEM_RENDER>(p, v.sched, bx, by, num_sms, s);
  if (v.kerr) {
    if (v.vol) return launch_variant<PREC, 1, 1, ST_SEM_DRAFT>(p, v.sched, bx, by, num_sms, s);
    return launch_variant<PREC, 1, 0, ST_SEM_DRAFT>(p, v.sched, bx, by, num_sms, s);
  }
  if (v.vol) return launch_variant<PREC, 0, 1, ST_SEM_DRAFT>(p, v.sched, bx, by, num_sms, s);
  return launch_variant<PREC, 0, 0, ST_SEM_DRAFT>(p, v.sched, bx, by, num_sms, s);
}

}  // namespace st
