// xdem_fused_fp64.cu -- plain FP64 instantiation of the fused contact kernel.
// Compiled with -fmad=false: contact classification and forces follow the
// reference's FP64 arithmetic operation by operation.
#include "xdem_fused.cuh"

namespace xdem {
cudaError_t launch_fused_contact_fp64(const ContactLaunch& c, cudaStream_t st)
{
    return launch_fused_contact_t<double>(c, st);
}
}  // namespace xdem
