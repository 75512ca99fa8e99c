// xdem_fused_mixed.cu -- the mixed form's sphere kernels without meshes (the
// candidate-list and stencil-walk pair kernels, the sphere body kernel) and
// the launch of the whole contact stage.  Compiled without implicit FMA
// contraction; the kernels are in xdem_fused_mixed.cuh.
#include "xdem_fused_mixed.cuh"

namespace xdem {
namespace {

template <unsigned int NT, unsigned int STAGE, unsigned int OCC>
cudaError_t launch_pairs(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs<false, NT, STAGE, OCC><<<(c.nentry + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT, unsigned int STAGE>
cudaError_t launch_pairs_occ(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.occ_pairs == 1024 ? launch_pairs<NT, STAGE, 1024>(c, st) : launch_pairs<NT, STAGE, 768>(c, st);
}
template <unsigned int NT>
cudaError_t launch_pairs_stage(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.stage == 8 ? launch_pairs_occ<NT, 8>(c, st) : launch_pairs_occ<NT, 16>(c, st);
}
cudaError_t launch_pairs_nt(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.nt_pairs) {
    case 64: return launch_pairs_stage<64>(c, st);
    case 256: return launch_pairs_stage<256>(c, st);
    default: return launch_pairs_stage<128>(c, st);
    }
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_list(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs_list<false, NT, OCC><<<(c.np + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
cudaError_t launch_list_nt(const ContactLaunch& c, cudaStream_t st)
{
    const bool hi = c.tune.occ_pairs == 1024;
    switch (c.tune.nt_pairs) {
    case 64: return hi ? launch_list<64, 1024>(c, st) : launch_list<64, 768>(c, st);
    case 256: return hi ? launch_list<256, 1024>(c, st) : launch_list<256, 768>(c, st);
    default: return hi ? launch_list<128, 1024>(c, st) : launch_list<128, 768>(c, st);
    }
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_bodies(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_bodies<NT, OCC><<<(c.nentry + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT>
cudaError_t launch_bodies_occ(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.occ_bodies) {
    case 768: return launch_bodies<NT, 768>(c, st);
    case 1024: return launch_bodies<NT, 1024>(c, st);
    default: return launch_bodies<NT, 512>(c, st);
    }
}

}  // namespace

// The block shapes come from c.tune (the autotuner's choice; by default 128
// threads, stage 16 and 768 threads per SM for the pairs, 128 threads and 512
// per SM for the bodies).  Body wrench partials are written by the kernel
// that owns the body (meshes: pairs, one row per block; planes and
// cylinders: the sphere body kernel, one row per warp; clusters: the cluster
// body kernel, one row per block) into rows of c.nblocks entries.  Scenes
// with meshes and cluster bodies run the kernels of xdem_fused_mixed_mesh.cu.
cudaError_t launch_fused_contact_mixed(const ContactLaunch& c, cudaStream_t st)
{
    if (c.nentry == 0) return cudaSuccess;
    cudaError_t e = c.nmesh ? launch_mixed_mesh_pairs(c, st) : c.use_list ? launch_list_nt(c, st) : launch_pairs_nt(c, st);
    if (e != cudaSuccess) return e;
    if (c.cl.ns) {
        e = launch_mixed_cluster_bodies(c, st);
    } else {
        switch (c.tune.nt_bodies) {
        case 64: e = launch_bodies_occ<64>(c, st); break;
        case 256: e = launch_bodies_occ<256>(c, st); break;
        default: e = launch_bodies_occ<128>(c, st); break;
        }
    }
    if (e != cudaSuccess || !c.use_list) return e;
    k_vl_roll<<<1, 1, 0, st>>>(c.vl_flag);
    return cudaGetLastError();
}

}  // namespace xdem
