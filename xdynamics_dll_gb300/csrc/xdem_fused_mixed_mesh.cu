// xdem_fused_mixed_mesh.cu -- the mixed form's kernels for scenes with
// triangle meshes (the pair kernels' mesh forms: candidate list and stencil
// walk) and the cluster body kernel.  Compiled with FMA contraction: their
// FP64 closest-point geometry and cluster rotations run on GB300's slow FP64
// pipe, where a fused multiply-add is one operation instead of two.  The
// list kernel's walk is inlined here, as it is in the walk kernel, so the two
// forms still compute the same bits.  The kernels are in
// xdem_fused_mixed.cuh.
#include "xdem_fused_mixed.cuh"

namespace xdem {
namespace {

template <unsigned int NT, unsigned int STAGE, unsigned int OCC>
cudaError_t launch_pairs_mesh(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs<true, NT, STAGE, OCC><<<(c.nentry + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT, unsigned int STAGE>
cudaError_t launch_pairs_mesh_occ(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.occ_pairs == 1024 ? launch_pairs_mesh<NT, STAGE, 1024>(c, st)
                                    : launch_pairs_mesh<NT, STAGE, 768>(c, st);
}
template <unsigned int NT>
cudaError_t launch_pairs_mesh_stage(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.stage == 8 ? launch_pairs_mesh_occ<NT, 8>(c, st) : launch_pairs_mesh_occ<NT, 16>(c, st);
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_list_mesh(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs_list<true, NT, OCC><<<(c.np + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT>
cudaError_t launch_mesh_nt(const ContactLaunch& c, cudaStream_t st)
{
    if (!c.use_list) return launch_pairs_mesh_stage<NT>(c, st);
    return c.tune.occ_pairs == 1024 ? launch_list_mesh<NT, 1024>(c, st) : launch_list_mesh<NT, 768>(c, st);
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_cluster_bodies(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_cluster_bodies<NT, OCC><<<(c.cl.ns + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT>
cudaError_t launch_cluster_bodies_occ(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.occ_bodies) {
    case 768: return launch_cluster_bodies<NT, 768>(c, st);
    case 1024: return launch_cluster_bodies<NT, 1024>(c, st);
    default: return launch_cluster_bodies<NT, 512>(c, st);
    }
}

}  // namespace

cudaError_t launch_mixed_mesh_pairs(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.nt_pairs) {
    case 64: return launch_mesh_nt<64>(c, st);
    case 256: return launch_mesh_nt<256>(c, st);
    default: return launch_mesh_nt<128>(c, st);
    }
}

cudaError_t launch_mixed_cluster_bodies(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.nt_bodies) {
    case 64: return launch_cluster_bodies_occ<64>(c, st);
    case 256: return launch_cluster_bodies_occ<256>(c, st);
    default: return launch_cluster_bodies_occ<128>(c, st);
    }
}

}  // namespace xdem
