// xdem_tune.cu -- block-shape autotuner of the mixed contact stage.
//
// xdem_sim_autotune times every candidate shape of the two mixed contact
// kernels (threads per block of the pair and body kernels, depth of the pair
// kernel's candidate stage) on the handle's own scene, with CUDA events
// around the contact stage, and keeps the fastest.  Each candidate starts
// from the same saved state, and the state is put back at the end, so
// tuning does not advance the simulation.  The shapes do not change results:
// every sphere's arithmetic is the same whatever block it runs in.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "xdem_sim_impl.h"

namespace {

// A device copy of everything a step reads and writes.
struct Snapshot {
    std::vector<std::pair<void*, size_t>> bufs;  // (copy, bytes)
    std::vector<void**> live;                     // the handle fields copied, in order
    cudaError_t take(xdem_sim* s)
    {
        // the FP64 acc and ea arrays are what is copied: bring them up to
        // date from a mixed sphere handle's FP32 copies first
        if (fused_sync_fp64(s->fs, s->acc, s->ea, s->st) != XDEM_OK) return cudaErrorInvalidValue;
        const size_t n = s->np, ns = s->ns;
        const size_t bytes[] = {n * 32, ns * 24, ns * 24, ns * 32, ns * 32, ns * 32,
                                n * 4, n * MAX_P2P_COUNT * 4, n * MAX_P2P_COUNT * 16,
                                n * 4, n * MAX_P2PL_COUNT * 4, n * MAX_P2PL_COUNT * 16,
                                n * 4, n * MAX_P2MS_COUNT * 4, n * MAX_P2MS_COUNT * 16, ns * 32};
        void** fields[] = {reinterpret_cast<void**>(&s->pos), reinterpret_cast<void**>(&s->vel),
                           reinterpret_cast<void**>(&s->acc), reinterpret_cast<void**>(&s->ep),
                           reinterpret_cast<void**>(&s->ev), reinterpret_cast<void**>(&s->ea),
                           reinterpret_cast<void**>(&s->pp_count), reinterpret_cast<void**>(&s->pp_id),
                           reinterpret_cast<void**>(&s->pp_tsd), reinterpret_cast<void**>(&s->pl_count),
                           reinterpret_cast<void**>(&s->pl_id), reinterpret_cast<void**>(&s->pl_tsd),
                           reinterpret_cast<void**>(&s->ms_count), reinterpret_cast<void**>(&s->ms_id),
                           reinterpret_cast<void**>(&s->ms_tsd), reinterpret_cast<void**>(&s->cpos)};
        for (size_t i = 0; i < sizeof(bytes) / sizeof(bytes[0]); ++i) {
            if (!*fields[i]) continue;
            void* c = nullptr;
            cudaError_t e = cudaMalloc(&c, bytes[i]);
            if (e == cudaSuccess) e = cudaMemcpyAsync(c, *fields[i], bytes[i], cudaMemcpyDeviceToDevice, s->st);
            if (e != cudaSuccess) {
                if (c) cudaFree(c);
                return e;
            }
            bufs.push_back({c, bytes[i]});
            live.push_back(fields[i]);
        }
        return cudaStreamSynchronize(s->st);
    }
    // copies back into whatever buffers the handle's fields point to now
    cudaError_t put(xdem_sim* s) const
    {
        cudaError_t e = cudaSuccess;
        for (size_t i = 0; i < bufs.size() && e == cudaSuccess; ++i)
            e = cudaMemcpyAsync(*live[i], bufs[i].first, bufs[i].second, cudaMemcpyDeviceToDevice, s->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        fused_state_written(s->fs);
        return e;
    }
    ~Snapshot()
    {
        for (auto& b : bufs) cudaFree(b.first);
    }
};

bool shape_ok(unsigned int nt) { return nt == 64 || nt == 128 || nt == 256; }

// Body wrench partials need one block size for both kernels.
bool keeps_wrenches(const xdem_sim* s) { return s->nscene == 1 && !s->bodies.empty(); }

MixedTune from_abi(const xdem_tune& t)
{
    return MixedTune{t.nt_pairs, t.stage, t.nt_bodies, t.occ_pairs, t.occ_bodies, t.skin_div};
}
xdem_tune to_abi(const MixedTune& m, double ms)
{
    return xdem_tune{m.nt_pairs, m.stage, m.nt_bodies, m.occ_pairs, m.occ_bodies, m.skin_div, ms};
}

}  // namespace

XDEM_API int xdem_sim_set_tune(xdem_sim* s, const xdem_tune* t)
{
    if (!s || !t) return XDEM_ERR_ARG;
    if (!shape_ok(t->nt_pairs) || !shape_ok(t->nt_bodies) || (t->stage != 8 && t->stage != 16)) return XDEM_ERR_ARG;
    if (t->occ_pairs != 768 && t->occ_pairs != 1024) return XDEM_ERR_ARG;
    if (t->occ_bodies != 512 && t->occ_bodies != 768 && t->occ_bodies != 1024) return XDEM_ERR_ARG;
    if (t->skin_div != 0 && t->skin_div != 8 && t->skin_div != 16 && t->skin_div != 32) return XDEM_ERR_ARG;
    if (keeps_wrenches(s) && t->nt_pairs != t->nt_bodies) return XDEM_ERR_ARG;
    s->fs.tune = from_abi(*t);
    fused_invalidate(s->fs);  // the captured step graphs bake in the shapes
    return XDEM_OK;
}

XDEM_API int xdem_sim_get_tune(xdem_sim* s, xdem_tune* t)
{
    if (!s || !t) return XDEM_ERR_ARG;
    *t = to_abi(s->fs.tune, 0.0);
    return XDEM_OK;
}

XDEM_API int xdem_sim_autotune(xdem_sim* s, unsigned int trial_steps, xdem_tune* best, xdem_tune* all,
                               unsigned int* nall)
{
    if (!s || !best || trial_steps == 0) return XDEM_ERR_ARG;
    // only the mixed fused step has shapes to choose
    if (!s->precision_mixed() || s->cfg.launcher_path) {
        xdem_sim_get_tune(s, best);
        if (nall) *nall = 0;
        return XDEM_OK;
    }
    if (int r = xdem_sim_step(s, 0)) return r;  // tables exist before the snapshot
    // status bits raised by the caller's own steps survive the trials
    const int pending = xdem_sim_status(s);
    if (pending & XDEM_ERR_CUDA) return XDEM_ERR_CUDA;
    Snapshot snap;
    if (cudaError_t e = snap.take(s)) {
        fprintf(stderr, "xdem_sim_autotune: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
        return XDEM_ERR_ALLOC;
    }
    const MixedTune keep = s->fs.tune;
    const bool prof = s->profiling;
    std::vector<xdem_tune> tried;
    // one trial: from the snapshot, 2 warm-up steps, trial_steps timed
    auto trial = [&](const MixedTune& t, double& ms) -> int {
        if (snap.put(s) != cudaSuccess) return XDEM_ERR_CUDA;
        s->fs.tune = t;
        s->profiling = false;
        if (int r = xdem_sim_step(s, 2)) return r;
        s->profiling = true;
        if (int r = xdem_sim_step(s, trial_steps)) return r;
        const unsigned int nrec = s->prof_contact_launches;
        ms = nrec ? s->prof_ms / nrec : 1e300;
        tried.push_back(to_abi(t, ms));
        return XDEM_OK;
    };
    const unsigned int nts[3] = {64, 128, 256}, stages[2] = {8, 16}, occp[2] = {768, 1024};
    const unsigned int occb[3] = {512, 768, 1024};
    int r = XDEM_OK;
    MixedTune win = keep;
    double win_ms = 1e300;
    auto consider = [&](const MixedTune& t) {
        if (r != XDEM_OK) return;
        double ms = 0.0;
        r = trial(t, ms);
        if (r == XDEM_OK && ms < win_ms) {
            win_ms = ms;
            win = t;
        }
    };
    if (keeps_wrenches(s)) {
        for (unsigned int nt : nts)
            for (unsigned int st : stages)
                for (unsigned int op : occp)
                    for (unsigned int ob : occb) consider(MixedTune{nt, st, nt, op, ob, keep.skin_div});
    } else {
        for (unsigned int nt : nts)
            for (unsigned int st : stages)
                for (unsigned int op : occp)
                    consider(MixedTune{nt, st, keep.nt_bodies, op, keep.occ_bodies, keep.skin_div});
        const MixedTune pw = win;
        for (unsigned int nt : nts)
            for (unsigned int ob : occb) consider(MixedTune{pw.nt_pairs, pw.stage, nt, pw.occ_pairs, ob, pw.skin_div});
    }
    // pair search: stencil walk every step, or candidate lists of three skins
    const MixedTune bw = win;
    const unsigned int skins[4] = {0, 8, 16, 32};
    for (unsigned int sk : skins) {
        if (sk == bw.skin_div) continue;
        MixedTune t = bw;
        t.skin_div = sk;
        consider(t);
    }
    s->profiling = prof;
    if (snap.put(s) != cudaSuccess && r == XDEM_OK) r = XDEM_ERR_CUDA;
    xdem_sim_status(s);  // the trials' bits belong to no user step
    if (pending) {
        const unsigned int h = (unsigned int)pending;
        if (cudaMemcpy(s->d_status, &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess && r == XDEM_OK)
            r = XDEM_ERR_CUDA;
    }
    if (r != XDEM_OK) {
        s->fs.tune = keep;
        return r;
    }
    s->fs.tune = win;
    *best = to_abi(win, win_ms);
    if (all && nall) {
        const unsigned int n = std::min<unsigned int>(*nall, (unsigned int)tried.size());
        for (unsigned int i = 0; i < n; ++i) all[i] = tried[i];
    }
    if (nall) *nall = (unsigned int)tried.size();
    return XDEM_OK;
}

XDEM_API int xdem_sim_list_rebuilds(xdem_sim* s, unsigned int* rebuilds)
{
    if (!s || !rebuilds) return XDEM_ERR_ARG;
    *rebuilds = 0;
    if (!s->fs.vl_flag) return XDEM_OK;
    cudaError_t e = cudaMemcpyAsync(rebuilds, s->fs.vl_flag + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    return e == cudaSuccess ? XDEM_OK : XDEM_ERR_CUDA;
}
