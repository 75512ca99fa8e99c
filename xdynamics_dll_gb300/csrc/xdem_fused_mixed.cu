// xdem_fused_mixed.cu -- mixed-precision instantiation of the fused contact
// kernel: contact geometry and forces in FP32 (FMA contraction on); positions,
// velocities, tangential history and force/torque accumulation in FP64.
#include "xdem_fused.cuh"

namespace xdem {
cudaError_t launch_fused_contact_mixed(const ContactLaunch& c, cudaStream_t st)
{
    return launch_fused_contact_t<float>(c, st);
}
}  // namespace xdem
