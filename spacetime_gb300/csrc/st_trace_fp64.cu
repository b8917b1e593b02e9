// st_trace_fp64.cu -- trace kernels instantiated for ST_PREC_FP64
// (one translation unit per precision so the build compiles them in parallel).
#include "st_kernels.cuh"

namespace st {

cudaError_t launch_trace_fp64(const Variant& v, const TraceParams& p, int bx, int by, int num_sms,
                               cudaStream_t s) {
  return launch_prec<ST_PREC_FP64>(v, p, bx, by, num_sms, s);
}

int variant_registers_fp64(const Variant& v) { return variant_regs_impl<ST_PREC_FP64>(v.kerr, v.vol, v.sem); }

}  // namespace st
