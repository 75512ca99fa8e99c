// xdem_io.cu -- part files of a scene handle: the state and the pair lists
// with their tangential history, in the layout xResultManager::
// export_step_data_to_file writes (source/xdynamics_manager/
// xResultManager.cpp:828-903, version 2):
//
//   double   time
//   uint32   np, ns                         (spheres, clusters; ns == np: free spheres)
//   double   mass[ns]
//   double   pos[np*4], vel[ns*3], acc[ns*3], ep[ns*4], ev[ns*4], ea[ns*4]
//   double   cpos[ns*4]                     (clusters only)
//   uint32   p2p count[np], id[np*12]; double p2p tsd[np*24]    (particle pairs)
//   uint32   p2pl count[np], id[np*3]; double p2pl tsd[np*6]    (planes)
//   uint32   p2cyl count[np], id[np*3]; double p2cyl tsd[np*6]  (cylinders)
//   uint32   p2tri count[np], id[np*5]; double p2tri tsd[np*10] (meshes)
//
// little-endian, no padding.  The reference writes the pair blocks of the
// contact kinds the model has, and a multibody block between the state and
// the pairs when the model has one; a handle has no multibody system (its
// bodies are posed by the caller), so it writes and reads none.  Loading a
// part file restores the pair lists and their history, which the
// reference's resume leaves empty (xContactManager.cpp:316-322).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "xdem_sim_impl.h"

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

template <class T>
bool put(FILE* f, const std::vector<T>& v)
{
    return v.empty() || std::fwrite(v.data(), sizeof(T), v.size(), f) == v.size();
}
template <class T>
bool get(FILE* f, std::vector<T>& v)
{
    return v.empty() || std::fread(v.data(), sizeof(T), v.size(), f) == v.size();
}

// The pair blocks a handle's part file holds, in file order, as pair kinds
// of xdem_sim_get_pairs (0 particles, 1 planes, 3 cylinders, 2 meshes).
constexpr int kBlocks = 4;
const int kBlockKind[kBlocks] = {0, 1, 3, 2};
const unsigned int kBlockCap[kBlocks] = {MAX_P2P_COUNT, MAX_P2PL_COUNT, MAX_P2CY_COUNT, MAX_P2MS_COUNT};
void blocks(const xdem_sim* s, bool want[kBlocks])
{
    want[0] = s->has_pp;
    want[1] = !s->planes.empty();
    want[2] = !s->cylinders.empty();
    want[3] = !s->meshes.empty();
}

}  // namespace

XDEM_API int xdem_sim_save_part(xdem_sim* s, const char* path, double time)
{
    if (!s || !path) return XDEM_ERR_ARG;
    if (int r = xdem_sim_step(s, 0)) return r;  // tables exist (a fresh handle saves empty lists)
    const size_t np = s->np, ns = s->ns;
    std::vector<double> pos(np * 4), vel(ns * 3), acc(ns * 3), ep(ns * 4), ev(ns * 4), ea(ns * 4), mass(ns),
        cpos(s->clusters ? ns * 4 : 0);
    if (int r = xdem_sim_get_state(s, pos.data(), vel.data(), acc.data(), ep.data(), ev.data(), ea.data(),
                                   s->clusters ? cpos.data() : nullptr))
        return r;
    if (cudaMemcpy(mass.data(), s->mass, ns * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return XDEM_ERR_CUDA;
    bool want[kBlocks];
    blocks(s, want);
    File out(path, "wb");
    if (!out.f) return XDEM_ERR_ARG;
    const unsigned int n32[2] = {(unsigned int)np, (unsigned int)ns};
    bool ok = std::fwrite(&time, sizeof(double), 1, out.f) == 1 && std::fwrite(n32, sizeof(n32), 1, out.f) == 1;
    ok = ok && put(out.f, mass) && put(out.f, pos) && put(out.f, vel) && put(out.f, acc) && put(out.f, ep) &&
         put(out.f, ev) && put(out.f, ea) && put(out.f, cpos);
    for (int b = 0; b < kBlocks && ok; ++b) {
        if (!want[b]) continue;
        std::vector<unsigned int> cnt(np), ids(np * kBlockCap[b]);
        std::vector<double> tsd(np * kBlockCap[b] * 2);
        if (int r = xdem_sim_get_pairs(s, kBlockKind[b], cnt.data(), ids.data(), tsd.data())) return r;
        ok = put(out.f, cnt) && put(out.f, ids) && put(out.f, tsd);
    }
    return ok ? XDEM_OK : XDEM_ERR_ARG;
}

XDEM_API int xdem_sim_load_part(xdem_sim* s, const char* path, double* time)
{
    if (!s || !path) return XDEM_ERR_ARG;
    File in(path, "rb");
    if (!in.f) return XDEM_ERR_ARG;
    double t = 0.0;
    unsigned int n32[2] = {0, 0};
    if (std::fread(&t, sizeof(double), 1, in.f) != 1 || std::fread(n32, sizeof(n32), 1, in.f) != 1)
        return XDEM_ERR_ARG;
    const size_t np = s->np, ns = s->ns;
    if (n32[0] != np || n32[1] != ns) return XDEM_ERR_ARG;  // another model
    std::vector<double> pos(np * 4), vel(ns * 3), acc(ns * 3), ep(ns * 4), ev(ns * 4), ea(ns * 4), mass(ns),
        cpos(s->clusters ? ns * 4 : 0);
    bool ok = get(in.f, mass) && get(in.f, pos) && get(in.f, vel) && get(in.f, acc) && get(in.f, ep) &&
              get(in.f, ev) && get(in.f, ea) && get(in.f, cpos);
    if (!ok) return XDEM_ERR_ARG;
    bool want[kBlocks];
    blocks(s, want);
    std::vector<unsigned int> cnt[kBlocks], ids[kBlocks];
    std::vector<double> tsd[kBlocks];
    for (int b = 0; b < kBlocks; ++b) {
        if (!want[b]) continue;
        cnt[b].resize(np);
        ids[b].resize(np * kBlockCap[b]);
        tsd[b].resize(np * kBlockCap[b] * 2);
        if (!(get(in.f, cnt[b]) && get(in.f, ids[b]) && get(in.f, tsd[b]))) return XDEM_ERR_ARG;
    }
    char extra;
    if (std::fread(&extra, 1, 1, in.f) != 0) return XDEM_ERR_ARG;  // blocks this handle has no contacts for
    // every list is checked before anything of the file reaches the handle,
    // so a corrupt file leaves the handle as it was
    for (int b = 0; b < kBlocks; ++b)
        if (want[b])
            if (int r = sim_check_pairs(s, kBlockKind[b], cnt[b].data(), ids[b].data())) return r;
    // the inertia is not in the file: the handle keeps its own
    std::vector<double> iner(ns * 3);
    if (cudaMemcpy(iner.data(), s->inertia, ns * 3 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return XDEM_ERR_CUDA;
    if (int r = xdem_sim_set_state(s, pos.data(), vel.data(), acc.data(), ep.data(), ev.data(), ea.data(),
                                   mass.data(), iner.data()))
        return r;
    if (s->clusters) {
        if (cudaMemcpy(s->cpos, cpos.data(), cpos.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
            return XDEM_ERR_CUDA;
    }
    if (int r = xdem_sim_step(s, 0)) return r;  // pair tables exist before they are filled
    for (int b = 0; b < kBlocks; ++b) {
        if (!want[b]) continue;
        if (int r = xdem_sim_set_pairs(s, kBlockKind[b], cnt[b].data(), ids[b].data(), tsd[b].data())) return r;
    }
    if (time) *time = t;
    return XDEM_OK;
}
