// st_trace_fp32_guarded.cu -- trace kernels instantiated for ST_PREC_FP32_GUARDED
// (one translation unit per precision so the build compiles them in parallel).
#include "st_kernels.cuh"

namespace st {

cudaError_t launch_trace_fp32_guarded(const Variant& v, const TraceParams& p, int bx, int by, int num_sms,
                               cudaStream_t s) {
  return launch_prec<ST_PREC_FP32_GUARDED>(v, p, bx, by, num_sms, s);
}

int variant_registers_fp32_guarded(const Variant& v) { return variant_regs_impl<ST_PREC_FP32_GUARDED>(v.kerr, v.vol, v.sem); }

size_t guarded_ray_state_bytes() { return sizeof(RayState<float>); }

}  // namespace st
