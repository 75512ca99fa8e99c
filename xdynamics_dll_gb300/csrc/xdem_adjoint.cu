// xdem_adjoint.cu -- reverse-mode adjoint of the FP64 DEM trajectory of a
// scene handle, with checkpoints.
//
// The forward is the handle's own FP64 step (xdem_sim_step); the adjoint
// stores its state every K steps.  The reverse sweep takes the segments last
// to first: it restores the segment's checkpoint into the handle, re-runs the
// K steps keeping every state, then walks them backwards with three kernels
// per step:
//   k_adj_velocity  reverse of the velocity half (impl:192-222): the force and
//                   moment adjoints of every sphere, and the uceom / rotation
//                   terms of its Euler parameters;
//   k_adj_contacts  reverse of the particle-particle (impl:613-733) and plane
//                   (impl:950-1080) contacts of each sphere, in the order the
//                   step visited them; the partner's share of each pair is
//                   written to the pair's slot, the history adjoints are
//                   mapped back to the slots they came from, the material
//                   gradients are block-summed;
//   k_adj_gather    each sphere collects its partners' shares, then the
//                   angular-velocity and position halves are reversed
//                   (impl:32-41, 135-147).
// The math and its VJPs are in xdem_adjoint.cuh.  Everything is FP64 and
// deterministic: block sums have a fixed order and no atomics are used.
//
// xdem_adj_tangent is the forward mode of the same linearisation, as an
// independent check of the adjoint: it re-runs the stored trajectory from
// its first checkpoint and carries the derivative of the state along it in
// up to kTanDirs parameter directions at once, with three kernels per step
// (position half, contacts, velocity half) that evaluate the header's
// forward pieces on dual numbers.  Its material derivatives come from
// central differences of getConstant (make_mat_pair) on the host, not from
// the chain rule the adjoint's gradients go through.
// The unit is compiled with -fmad=false so the recomputed overlaps round
// exactly as the forward step's did.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <new>
#include <vector>

#include "xdem_adjoint.cuh"
#include "xdem_sim_impl.h"

namespace {

constexpr unsigned int kAdjThreads = 128;
constexpr unsigned int kMaxAdjPlanes = 16;
constexpr int kGradFields = 5;  // Eeq, Seq8, beta, vs1, fric

int cerr(cudaError_t e)
{
    if (e == cudaSuccess) return XDEM_OK;
    fprintf(stderr, "xdem_adj: CUDA error %s\n", cudaGetErrorString(e));
    return XDEM_ERR_CUDA;
}

// Device arrays of one stored state (reference layouts).
struct Slab {
    double *pos, *vel, *acc, *ep, *ev, *ea;
    unsigned int *ppc, *ppi;
    double* ppt;
    unsigned int *plc, *pli;
    double* plt;
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t slab_bytes(size_t np, bool pp, bool pl)
{
    size_t b = align256(np * 4 * 8) * 4 + align256(np * 3 * 8) * 2;  // pos ep ev ea, vel acc
    if (pp) b += align256(np * 4) + align256(np * MAX_P2P_COUNT * 4) + align256(np * MAX_P2P_COUNT * 16);
    if (pl) b += align256(np * 4) + align256(np * MAX_P2PL_COUNT * 4) + align256(np * MAX_P2PL_COUNT * 16);
    return b;
}

Slab carve(char* base, size_t np, bool pp, bool pl)
{
    Slab s{};
    char* p = base;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += align256(bytes);
        return r;
    };
    s.pos = reinterpret_cast<double*>(take(np * 32));
    s.ep = reinterpret_cast<double*>(take(np * 32));
    s.ev = reinterpret_cast<double*>(take(np * 32));
    s.ea = reinterpret_cast<double*>(take(np * 32));
    s.vel = reinterpret_cast<double*>(take(np * 24));
    s.acc = reinterpret_cast<double*>(take(np * 24));
    if (pp) {
        s.ppc = reinterpret_cast<unsigned int*>(take(np * 4));
        s.ppi = reinterpret_cast<unsigned int*>(take(np * MAX_P2P_COUNT * 4));
        s.ppt = reinterpret_cast<double*>(take(np * MAX_P2P_COUNT * 16));
    }
    if (pl) {
        s.plc = reinterpret_cast<unsigned int*>(take(np * 4));
        s.pli = reinterpret_cast<unsigned int*>(take(np * MAX_P2PL_COUNT * 4));
        s.plt = reinterpret_cast<double*>(take(np * MAX_P2PL_COUNT * 16));
    }
    return s;
}

// Everything the adjoint kernels read besides the two states.
struct AdjArgs {
    unsigned int np, nplane, nprop;
    int model, vel_compat;
    double dt, h2;  // dt, dt^2 / 2
    const double *mass, *inertia;
    const adj::Mat* mat;                   // [nprop]: 0 particle pairs, 1 + k plane k
    const adj::PlaneContact* planes;       // [nplane]
    const unsigned int* plane_pid;         // [nplane] device_plane_info::id of plane k
    // state adjoints, in place: at the start of a reverse step those of
    // state n+1, at its end those of state n
    double *lx, *lv, *la, *le, *led, *lea;
    double *lF, *lM, *lw;                  // per sphere, this step
    const double *lpp_new, *lpl_new;       // history adjoints of the stored lists n+1
    double *lpp_old, *lpl_old;             // ... mapped onto lists n
    double* other;                         // [np * 12 * 9] the partner's share of each pair
    double* gpart;                         // [nblocks * nprop * 5] material gradients
};

__device__ __forceinline__ adj::V lv3(const double* a, size_t i) { return adj::mkv(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
__device__ __forceinline__ adj::V lv4(const double* a, size_t i) { return adj::mkv(a[4 * i], a[4 * i + 1], a[4 * i + 2]); }
__device__ __forceinline__ adj::Q lq4(const double* a, size_t i)
{
    return adj::mkq(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]);
}
__device__ __forceinline__ void sv3(double* a, size_t i, adj::V v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
__device__ __forceinline__ void sq4(double* a, size_t i, adj::Q q)
{
    a[4 * i] = q.x; a[4 * i + 1] = q.y; a[4 * i + 2] = q.z; a[4 * i + 3] = q.w;
}

// Reverse of the velocity half of step n -> n+1 for sphere i.
__global__ void k_adj_velocity(AdjArgs A, Slab S0, Slab S1)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.np) return;
    using namespace adj;
    const double hdt = 0.5 * A.dt;
    const V lv1 = lv3(A.lv, i), la1 = lv3(A.la, i);
    const Q led1 = lq4(A.led, i), lea1 = lq4(A.lea, i);
    const Q e1 = lq4(S1.ep, i), d0 = lq4(S0.ev, i), q = lq4(S1.ea, i);
    const V J = lv3(A.inertia, i);
    const double inv = 1.0 / A.mass[i];
    // e_dot1 = e_dot0 + hdt (e_ddot0 + q), e_ddot1 = q
    const Q lq = lea1 + hdt * led1;
    Q led0 = led1;
    const Q lea0 = hdt * led1;
    // v1 = v0 + hdt (a0 + a1) (or v1 = v0), a1 = inv (F + m g)
    V la1t = la1, la0 = mkv(0, 0, 0);
    if (!A.vel_compat) {
        la1t = la1 + hdt * lv1;
        la0 = hdt * lv1;
    }
    const V lF = inv * la1t;
    // q = uceom(J, e1, e_dot0, A(e1)^T M)
    const V n = uceom_torque(J, e1, d0, q);
    Q le1 = lq4(A.le, i);
    V ln = mkv(0, 0, 0);
    uceom_vjp(J, e1, d0, n, lq, le1, led0, ln);
    const V M = to_global(n, e1);
    V lM = mkv(0, 0, 0);
    to_local_vjp(M, e1, ln, lM, le1);
    sv3(A.lF, i, lF);
    sv3(A.lM, i, lM);
    sq4(A.le, i, le1);
    sq4(A.led, i, led0);
    sq4(A.lea, i, lea0);
    sv3(A.lv, i, lv1);
    sv3(A.la, i, la0);
}

// Fixed-order block sum of kGradFields values per thread, added to out.
__device__ void block_add(const double* vals, double* sm, double* out)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int c = 0; c < kGradFields; ++c) {
        double v = vals[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[warp * kGradFields + c] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < kGradFields) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += sm[w * kGradFields + threadIdx.x];
        out[threadIdx.x] += s;
    }
    __syncthreads();
}

// Reverse of the contacts of step n -> n+1 for sphere i (one thread each).
__global__ void __launch_bounds__(kAdjThreads) k_adj_contacts(AdjArgs A, Slab S0, Slab S1)
{
    using namespace adj;
    __shared__ double sm[(kAdjThreads / 32) * kGradFields];
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < A.np;
    MatGrad gpp{0, 0, 0, 0, 0};
    MatGrad gpl[MAX_P2PL_COUNT];
    int kpl[MAX_P2PL_COUNT];
    for (int s = 0; s < (int)MAX_P2PL_COUNT; ++s) {
        gpl[s] = MatGrad{0, 0, 0, 0, 0};
        kpl[s] = -1;
    }
    if (live) {
        Body bi;
        bi.x = lv4(S1.pos, i);
        bi.r = S1.pos[4 * (size_t)i + 3];
        bi.v = lv3(S0.vel, i);
        bi.w = ang_vel(lq4(S1.ep, i), lq4(S0.ev, i));
        bi.m = A.mass[i];
        const V lF = lv3(A.lF, i), lM = lv3(A.lM, i);
        V lxi = mkv(0, 0, 0), lvi = mkv(0, 0, 0), lwi = mkv(0, 0, 0);
        const size_t sid = (size_t)i * MAX_P2P_COUNT;
        // ------------------------------------------------ particle pairs
        if (S1.ppc) {
            const int n = (int)min(S1.ppc[i], (unsigned int)MAX_P2P_COUNT);
            const int n_old = (int)min(S0.ppc[i], (unsigned int)MAX_P2P_COUNT);
            Body nb[kMaxPairs];
            double ds0[kMaxPairs], dots0[kMaxPairs], lds1[kMaxPairs], ldots1[kMaxPairs];
            double lds0[kMaxPairs], ldots0[kMaxPairs];
            int src[kMaxPairs];
            V lxj[kMaxPairs], lvj[kMaxPairs], lwj[kMaxPairs];
            for (int s = 0; s < n; ++s) {
                const unsigned int j = S1.ppi[sid + s];
                nb[s].x = lv4(S1.pos, j);
                nb[s].r = S1.pos[4 * (size_t)j + 3];
                nb[s].v = lv3(S0.vel, j);
                nb[s].w = ang_vel(lq4(S1.ep, j), lq4(S0.ev, j));
                nb[s].m = A.mass[j];
                src[s] = -1;
                ds0[s] = 0.0;
                dots0[s] = 0.0;
                for (int q = 0; q < n_old; ++q)
                    if (S0.ppi[sid + q] == j) {
                        src[s] = q;
                        ds0[s] = S0.ppt[2 * (sid + q)];
                        dots0[s] = S0.ppt[2 * (sid + q) + 1];
                        break;
                    }
                lds1[s] = A.lpp_new[2 * (sid + s)];
                ldots1[s] = A.lpp_new[2 * (sid + s) + 1];
                lds0[s] = ldots0[s] = 0.0;
                lxj[s] = lvj[s] = lwj[s] = mkv(0, 0, 0);
            }
            pp_sphere_vjp(A.model, A.dt, A.mat[0], bi, nb, ds0, dots0, n, lF, lM, lds1, ldots1, lxi, lvi, lwi, lxj,
                          lvj, lwj, lds0, ldots0, gpp);
            for (int q = 0; q < (int)MAX_P2P_COUNT; ++q) {
                A.lpp_old[2 * (sid + q)] = 0.0;
                A.lpp_old[2 * (sid + q) + 1] = 0.0;
            }
            for (int s = 0; s < n; ++s) {
                if (src[s] >= 0) {
                    A.lpp_old[2 * (sid + src[s])] = lds0[s];
                    A.lpp_old[2 * (sid + src[s]) + 1] = ldots0[s];
                }
                double* o = A.other + 9 * (sid + s);
                o[0] = lxj[s].x; o[1] = lxj[s].y; o[2] = lxj[s].z;
                o[3] = lvj[s].x; o[4] = lvj[s].y; o[5] = lvj[s].z;
                o[6] = lwj[s].x; o[7] = lwj[s].y; o[8] = lwj[s].z;
            }
        }
        // ------------------------------------------------ planes
        // The plane list is updated in place: plane k's history lookup scans
        // all slots, including those the planes before it rewrote in this
        // step and stale ones (impl:962-1014); untouched slots carry over.
        if (S1.plc) {
            const size_t pid0 = (size_t)i * MAX_P2PL_COUNT;
            const int cnt = (int)min(S1.plc[i], (unsigned int)MAX_P2PL_COUNT);
            unsigned int cur_id[MAX_P2PL_COUNT];
            int cur_src[MAX_P2PL_COUNT], src[MAX_P2PL_COUNT];
            for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q) {
                cur_id[q] = S0.pli[pid0 + q];
                cur_src[q] = q;  // < 3: slot q of list n; >= 3: slot (src - 3) of this step
                src[q] = -1;
            }
            for (int s = 0; s < cnt; ++s) {
                const unsigned int pid = S1.pli[pid0 + s];
                for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q)
                    if (cur_id[q] == pid) { src[s] = cur_src[q]; break; }
                cur_id[s] = pid;
                cur_src[s] = (int)MAX_P2PL_COUNT + s;
            }
            double acc_ds[MAX_P2PL_COUNT] = {0, 0, 0}, acc_dots[MAX_P2PL_COUNT] = {0, 0, 0};
            double lold_ds[MAX_P2PL_COUNT] = {0, 0, 0}, lold_dots[MAX_P2PL_COUNT] = {0, 0, 0};
            for (int s = cnt - 1; s >= 0; --s) {
                const unsigned int pid = S1.pli[pid0 + s];
                int k = -1;
                for (unsigned int p = 0; p < A.nplane; ++p)
                    if (A.plane_pid[p] == pid) { k = (int)p; break; }
                if (k < 0) continue;  // not a plane of this handle (the step writes only its own ids)
                double ds0 = 0.0, dots0 = 0.0;
                if (src[s] >= 0 && src[s] < (int)MAX_P2PL_COUNT) {
                    ds0 = S0.plt[2 * (pid0 + src[s])];
                    dots0 = S0.plt[2 * (pid0 + src[s]) + 1];
                } else if (src[s] >= (int)MAX_P2PL_COUNT) {
                    const int t = src[s] - (int)MAX_P2PL_COUNT;
                    ds0 = S1.plt[2 * (pid0 + t)];
                    dots0 = S1.plt[2 * (pid0 + t) + 1];
                }
                const double lds1 = A.lpl_new[2 * (pid0 + s)] + acc_ds[s];
                const double ldots1 = A.lpl_new[2 * (pid0 + s) + 1] + acc_dots[s];
                double lds0 = 0.0, ldots0 = 0.0;
                plane_contact_vjp(A.model, A.dt, A.planes[k], bi, ds0, dots0, lF, lM, lds1, ldots1, lxi, lvi, lwi,
                                  lds0, ldots0, gpl[s]);
                kpl[s] = k;
                if (src[s] >= 0 && src[s] < (int)MAX_P2PL_COUNT) {
                    lold_ds[src[s]] += lds0;
                    lold_dots[src[s]] += ldots0;
                } else if (src[s] >= (int)MAX_P2PL_COUNT) {
                    acc_ds[src[s] - MAX_P2PL_COUNT] += lds0;
                    acc_dots[src[s] - MAX_P2PL_COUNT] += ldots0;
                }
            }
            for (int s = cnt; s < (int)MAX_P2PL_COUNT; ++s) {
                lold_ds[s] += A.lpl_new[2 * (pid0 + s)];
                lold_dots[s] += A.lpl_new[2 * (pid0 + s) + 1];
            }
            for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q) {
                A.lpl_old[2 * (pid0 + q)] = lold_ds[q];
                A.lpl_old[2 * (pid0 + q) + 1] = lold_dots[q];
            }
        }
        sv3(A.lx, i, lv3(A.lx, i) + lxi);
        sv3(A.lv, i, lv3(A.lv, i) + lvi);
        sv3(A.lw, i, lwi);
    }
    // material gradients: one fixed-order block sum per contact property
    for (unsigned int p = 0; p < A.nprop; ++p) {
        double v[kGradFields] = {0, 0, 0, 0, 0};
        if (p == 0) {
            v[0] = gpp.Eeq; v[1] = gpp.Seq8; v[2] = gpp.beta; v[3] = gpp.vs1; v[4] = gpp.fric;
        } else {
            for (int s = 0; s < (int)MAX_P2PL_COUNT; ++s)
                if (kpl[s] == (int)p - 1) {
                    v[0] += gpl[s].Eeq; v[1] += gpl[s].Seq8; v[2] += gpl[s].beta; v[3] += gpl[s].vs1;
                    v[4] += gpl[s].fric;
                }
        }
        block_add(v, sm, A.gpart + ((size_t)blockIdx.x * A.nprop + p) * kGradFields);
    }
}

// Each sphere collects its partners' shares, then the angular-velocity and
// position halves of step n -> n+1 are reversed.
__global__ void k_adj_gather(AdjArgs A, Slab S0, Slab S1)
{
    using namespace adj;
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= A.np) return;
    V lx = lv3(A.lx, j), lv = lv3(A.lv, j), lw = lv3(A.lw, j);
    if (S1.ppc) {
        const int n = (int)min(S1.ppc[j], (unsigned int)MAX_P2P_COUNT);
        for (int s = 0; s < n; ++s) {
            const unsigned int i = S1.ppi[(size_t)j * MAX_P2P_COUNT + s];
            const int ni = (int)min(S1.ppc[i], (unsigned int)MAX_P2P_COUNT);
            for (int t = 0; t < ni; ++t)
                if (S1.ppi[(size_t)i * MAX_P2P_COUNT + t] == j) {
                    const double* o = A.other + 9 * ((size_t)i * MAX_P2P_COUNT + t);
                    lx = lx + mkv(o[0], o[1], o[2]);
                    lv = lv + mkv(o[3], o[4], o[5]);
                    lw = lw + mkv(o[6], o[7], o[8]);
                    break;
                }
        }
    }
    // omega = ang_vel(e1, e_dot0)
    Q le1 = lq4(A.le, j), led0 = lq4(A.led, j);
    ang_vel_vjp(lq4(S1.ep, j), lq4(S0.ev, j), lw, le1, led0);
    // x1 = x0 + dt v0 + h a0
    lv = lv + A.dt * lx;
    const V la0 = lv3(A.la, j) + A.h2 * lx;
    // e1 = normalize((e0 + dt e_dot0) + h e_ddot0)
    const Q ep = (lq4(S0.ep, j) + A.dt * lq4(S0.ev, j)) + A.h2 * lq4(S0.ea, j);
    Q lep = mkq(0, 0, 0, 0);
    normalize_vjp(ep, le1, lep);
    led0 = led0 + A.dt * lep;
    const Q lea0 = lq4(A.lea, j) + A.h2 * lep;
    sv3(A.lx, j, lx);
    sv3(A.lv, j, lv);
    sv3(A.la, j, la0);
    sq4(A.le, j, lep);
    sq4(A.led, j, led0);
    sq4(A.lea, j, lea0);
}

// ---------------------------------------------------------------- forward mode
constexpr int kTanDirs = 3;
using DT = adj::Dual<kTanDirs>;

// Tangent arrays hold kTanDirs values per component: component c of sphere
// i, direction k at [(i * ncomp + c) * kTanDirs + k].
struct TanArgs {
    unsigned int np, nplane;
    int model, vel_compat;
    double dt, h2;
    const double *mass, *inertia;
    const adj::Mat* mat;            // [nprop] values
    const double* tmat;             // [nprop][5: Eeq, Seq8, beta, vs1, fric][kTanDirs]
    const adj::PlaneContact* planes;
    const unsigned int* plane_pid;
    double *tx, *tv, *ta, *te, *ted, *tea;  // state tangents, n -> n+1 in place
    double *tF, *tM, *Mv;                   // this step's force and moment tangents, moment values
    const double* tpp_old;                  // [np * 12 * 2][kTanDirs] history tangents of lists n
    double* tpp_new;                        // ... of lists n+1
    const double* tpl_old;
    double* tpl_new;
};

__device__ __forceinline__ DT dual_of(double v, const double* t)
{
    DT r(v);
    for (int k = 0; k < kTanDirs; ++k) r.d[k] = t[k];
    return r;
}
__device__ __forceinline__ void put_tan(double* t, const DT& x)
{
    for (int k = 0; k < kTanDirs; ++k) t[k] = x.d[k];
}
__device__ __forceinline__ adj::VT<DT> dv3(const double* val, size_t vi, const double* tan, size_t ti)
{
    return adj::VT<DT>{dual_of(val[vi], tan + ti * kTanDirs), dual_of(val[vi + 1], tan + (ti + 1) * kTanDirs),
                       dual_of(val[vi + 2], tan + (ti + 2) * kTanDirs)};
}
__device__ __forceinline__ adj::QT<DT> dq4(const double* val, size_t vi, const double* tan, size_t ti)
{
    return adj::QT<DT>{dual_of(val[vi], tan + ti * kTanDirs), dual_of(val[vi + 1], tan + (ti + 1) * kTanDirs),
                       dual_of(val[vi + 2], tan + (ti + 2) * kTanDirs),
                       dual_of(val[vi + 3], tan + (ti + 3) * kTanDirs)};
}
__device__ __forceinline__ void put3(double* tan, size_t ti, const adj::VT<DT>& v)
{
    put_tan(tan + ti * kTanDirs, v.x);
    put_tan(tan + (ti + 1) * kTanDirs, v.y);
    put_tan(tan + (ti + 2) * kTanDirs, v.z);
}
__device__ __forceinline__ void put4(double* tan, size_t ti, const adj::QT<DT>& q)
{
    put_tan(tan + ti * kTanDirs, q.x);
    put_tan(tan + (ti + 1) * kTanDirs, q.y);
    put_tan(tan + (ti + 2) * kTanDirs, q.z);
    put_tan(tan + (ti + 3) * kTanDirs, q.w);
}
__device__ __forceinline__ adj::MatT<DT> dual_mat(const TanArgs& T, unsigned int p)
{
    const adj::Mat& m = T.mat[p];
    const double* t = T.tmat + (size_t)p * 5 * kTanDirs;
    adj::MatT<DT> r;
    r.Eeq = dual_of(m.Eeq, t);
    r.Seq8 = dual_of(m.Seq8, t + kTanDirs);
    r.beta = dual_of(m.beta, t + 2 * kTanDirs);
    r.vs1 = dual_of(m.vs1, t + 3 * kTanDirs);
    r.sratio = DT(m.sratio);
    r.fric = dual_of(m.fric, t + 4 * kTanDirs);
    return r;
}

// Position half of step n -> n+1: x1 = x0 + dt v0 + h a0, e1 = normalize(e0
// + dt e_dot0 + h e_ddot0); tx and te become those of state n+1.
__global__ void k_tan_position(TanArgs T, Slab S0)
{
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= T.np) return;
    using namespace adj;
    const VT<DT> x0 = dv3(S0.pos, 4 * (size_t)j, T.tx, 3 * (size_t)j);
    const VT<DT> v0 = dv3(S0.vel, 3 * (size_t)j, T.tv, 3 * (size_t)j);
    const VT<DT> a0 = dv3(S0.acc, 3 * (size_t)j, T.ta, 3 * (size_t)j);
    put3(T.tx, 3 * (size_t)j, (x0 + T.dt * v0) + T.h2 * a0);
    const QT<DT> e0 = dq4(S0.ep, 4 * (size_t)j, T.te, 4 * (size_t)j);
    const QT<DT> d0 = dq4(S0.ev, 4 * (size_t)j, T.ted, 4 * (size_t)j);
    const QT<DT> q0 = dq4(S0.ea, 4 * (size_t)j, T.tea, 4 * (size_t)j);
    put4(T.te, 4 * (size_t)j, normalize((e0 + T.dt * d0) + T.h2 * q0));
}

// Sphere i as the contacts of step n -> n+1 see it: centre and Euler
// parameters of state n+1, velocities of state n.
__device__ __forceinline__ adj::BodyT<DT> tan_body(const TanArgs& T, const Slab& S0, const Slab& S1, unsigned int i)
{
    adj::BodyT<DT> b;
    b.x = dv3(S1.pos, 4 * (size_t)i, T.tx, 3 * (size_t)i);
    b.r = S1.pos[4 * (size_t)i + 3];
    b.v = dv3(S0.vel, 3 * (size_t)i, T.tv, 3 * (size_t)i);
    b.w = adj::ang_vel(dq4(S1.ep, 4 * (size_t)i, T.te, 4 * (size_t)i),
                       dq4(S0.ev, 4 * (size_t)i, T.ted, 4 * (size_t)i));
    b.m = T.mass[i];
    return b;
}

// Contacts of step n -> n+1 for sphere i on dual numbers: the particle pairs
// of list n+1 in list order with the history each carried from list n, then
// the planes with the in-place slot rule of the forward step.
__global__ void __launch_bounds__(kAdjThreads) k_tan_contacts(TanArgs T, Slab S0, Slab S1)
{
    using namespace adj;
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.np) return;
    const BodyT<DT> bi = tan_body(T, S0, S1, i);
    VT<DT> F = vzero<DT>(), M = vzero<DT>();
    if (S1.ppc) {
        const size_t sid = (size_t)i * MAX_P2P_COUNT;
        const int n = (int)min(S1.ppc[i], (unsigned int)MAX_P2P_COUNT);
        const int n_old = (int)min(S0.ppc[i], (unsigned int)MAX_P2P_COUNT);
        BodyT<DT> nb[kMaxPairs];
        DT ds0[kMaxPairs], dots0[kMaxPairs], ds1[kMaxPairs], dots1[kMaxPairs];
        for (int s = 0; s < n; ++s) {
            const unsigned int j = S1.ppi[sid + s];
            nb[s] = tan_body(T, S0, S1, j);
            ds0[s] = DT(0.0);
            dots0[s] = DT(0.0);
            for (int q = 0; q < n_old; ++q)
                if (S0.ppi[sid + q] == j) {
                    ds0[s] = dual_of(S0.ppt[2 * (sid + q)], T.tpp_old + 2 * (sid + q) * kTanDirs);
                    dots0[s] = dual_of(S0.ppt[2 * (sid + q) + 1], T.tpp_old + (2 * (sid + q) + 1) * kTanDirs);
                    break;
                }
        }
        pp_sphere_fwd(T.model, T.dt, dual_mat(T, 0), bi, nb, ds0, dots0, n, F, M, ds1, dots1);
        for (int s = 0; s < (int)MAX_P2P_COUNT; ++s) {
            const DT a = s < n ? ds1[s] : DT(0.0), b = s < n ? dots1[s] : DT(0.0);
            put_tan(T.tpp_new + 2 * (sid + s) * kTanDirs, a);
            put_tan(T.tpp_new + (2 * (sid + s) + 1) * kTanDirs, b);
        }
    }
    if (S1.plc) {
        const size_t pid0 = (size_t)i * MAX_P2PL_COUNT;
        const int cnt = (int)min(S1.plc[i], (unsigned int)MAX_P2PL_COUNT);
        // slot contents as the step walks the planes: ids and histories of
        // list n, overwritten slot by slot by this step's contacts
        unsigned int cur_id[MAX_P2PL_COUNT];
        DT cur_ds[MAX_P2PL_COUNT], cur_dots[MAX_P2PL_COUNT];
        for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q) {
            cur_id[q] = S0.pli[pid0 + q];
            cur_ds[q] = dual_of(S0.plt[2 * (pid0 + q)], T.tpl_old + 2 * (pid0 + q) * kTanDirs);
            cur_dots[q] = dual_of(S0.plt[2 * (pid0 + q) + 1], T.tpl_old + (2 * (pid0 + q) + 1) * kTanDirs);
        }
        for (int s = 0; s < cnt; ++s) {
            const unsigned int pid = S1.pli[pid0 + s];
            int k = -1;
            for (unsigned int p = 0; p < T.nplane; ++p)
                if (T.plane_pid[p] == pid) { k = (int)p; break; }
            DT ds0(0.0), dots0(0.0);
            for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q)
                if (cur_id[q] == pid) { ds0 = cur_ds[q]; dots0 = cur_dots[q]; break; }
            DT ds1 = ds0, dots1 = dots0;
            if (k >= 0)
                plane_contact_fwd_t(T.model, T.dt, T.planes[k], dual_mat(T, 1 + k), bi, ds0, dots0, F, M, ds1, dots1);
            cur_id[s] = pid;
            cur_ds[s] = ds1;
            cur_dots[s] = dots1;
        }
        for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q) {
            put_tan(T.tpl_new + 2 * (pid0 + q) * kTanDirs, cur_ds[q]);
            put_tan(T.tpl_new + (2 * (pid0 + q) + 1) * kTanDirs, cur_dots[q]);
        }
    }
    put3(T.tF, 3 * (size_t)i, F);
    put3(T.tM, 3 * (size_t)i, M);
    T.Mv[3 * (size_t)i] = M.x.v;
    T.Mv[3 * (size_t)i + 1] = M.y.v;
    T.Mv[3 * (size_t)i + 2] = M.z.v;
}

// Velocity half of step n -> n+1: a1 = F / m + g, v1 = v0 + dt/2 (a0 + a1)
// (v1 = v0 in the velocity-compat mode), q = uceom(J, e1, e_dot0, A(e1)^T M),
// e_dot1 = e_dot0 + dt/2 (e_ddot0 + q), e_ddot1 = q.
__global__ void k_tan_velocity(TanArgs T, Slab S0, Slab S1)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.np) return;
    using namespace adj;
    const double hdt = 0.5 * T.dt, inv = 1.0 / T.mass[i];
    const VT<DT> F = dv3(S1.acc, 3 * (size_t)i, T.tF, 3 * (size_t)i);  // value unused: only tangents flow
    const VT<DT> a1 = inv * F;
    const VT<DT> v0 = dv3(S0.vel, 3 * (size_t)i, T.tv, 3 * (size_t)i);
    const VT<DT> a0 = dv3(S0.acc, 3 * (size_t)i, T.ta, 3 * (size_t)i);
    put3(T.tv, 3 * (size_t)i, T.vel_compat ? v0 : v0 + hdt * (a0 + a1));
    put3(T.ta, 3 * (size_t)i, a1);
    const V J = mkv(T.inertia[3 * (size_t)i], T.inertia[3 * (size_t)i + 1], T.inertia[3 * (size_t)i + 2]);
    const QT<DT> e1 = dq4(S1.ep, 4 * (size_t)i, T.te, 4 * (size_t)i);
    const QT<DT> d0 = dq4(S0.ev, 4 * (size_t)i, T.ted, 4 * (size_t)i);
    const QT<DT> q0 = dq4(S0.ea, 4 * (size_t)i, T.tea, 4 * (size_t)i);
    const VT<DT> M = dv3(T.Mv, 3 * (size_t)i, T.tM, 3 * (size_t)i);
    const QT<DT> q = uceom(J, e1, d0, to_local(M, e1));
    put4(T.ted, 4 * (size_t)i, d0 + hdt * (q0 + q));
    put4(T.tea, 4 * (size_t)i, q);
}

}  // namespace

struct xdem_adj {
    xdem_sim* s = nullptr;
    unsigned int K = 0, np = 0, nplane = 0, nprop = 0, nblocks = 0, nsteps = 0;
    bool pp = false, pl = false;
    size_t sbytes = 0;
    char* ckpt_mem = nullptr;
    size_t ckpt_n = 0;  // checkpoints allocated
    std::vector<Slab> ckpt;
    char* seg_mem = nullptr;
    std::vector<Slab> seg;  // K + 1 states of the segment being reversed
    double *lx = nullptr, *lv = nullptr, *la = nullptr, *le = nullptr, *led = nullptr, *lea = nullptr;
    double *lF = nullptr, *lM = nullptr, *lw = nullptr, *other = nullptr, *gpart = nullptr;
    double *lpp[2] = {nullptr, nullptr}, *lpl[2] = {nullptr, nullptr};
    adj::Mat* d_mat = nullptr;
    adj::PlaneContact* d_planes = nullptr;
    unsigned int* d_pid = nullptr;
    std::vector<device_contact_property> cps;  // [nprop] properties the forward ran with
    // forward mode (xdem_adj_tangent)
    double *tx = nullptr, *tv = nullptr, *ta = nullptr, *te = nullptr, *ted = nullptr, *tea = nullptr;
    double *tF = nullptr, *tM = nullptr, *Mv = nullptr, *tmat = nullptr;
    double *tpp[2] = {nullptr, nullptr}, *tpl[2] = {nullptr, nullptr};
};

namespace {

cudaError_t copy_state(const Slab& d, const double* pos, const double* vel, const double* acc, const double* ep,
                       const double* ev, const double* ea, const unsigned int* ppc, const unsigned int* ppi,
                       const double* ppt, const unsigned int* plc, const unsigned int* pli, const double* plt,
                       size_t np, cudaStream_t st)
{
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpyAsync(d.pos, pos, np * 32, k, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.vel, vel, np * 24, k, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.acc, acc, np * 24, k, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.ep, ep, np * 32, k, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.ev, ev, np * 32, k, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.ea, ea, np * 32, k, st);
    if (d.ppc && e == cudaSuccess) e = cudaMemcpyAsync(d.ppc, ppc, np * 4, k, st);
    if (d.ppi && e == cudaSuccess) e = cudaMemcpyAsync(d.ppi, ppi, np * MAX_P2P_COUNT * 4, k, st);
    if (d.ppt && e == cudaSuccess) e = cudaMemcpyAsync(d.ppt, ppt, np * MAX_P2P_COUNT * 16, k, st);
    if (d.plc && e == cudaSuccess) e = cudaMemcpyAsync(d.plc, plc, np * 4, k, st);
    if (d.pli && e == cudaSuccess) e = cudaMemcpyAsync(d.pli, pli, np * MAX_P2PL_COUNT * 4, k, st);
    if (d.plt && e == cudaSuccess) e = cudaMemcpyAsync(d.plt, plt, np * MAX_P2PL_COUNT * 16, k, st);
    return e;
}

// handle -> slab
cudaError_t save_state(xdem_adj* a, const Slab& d)
{
    xdem_sim* s = a->s;
    return copy_state(d, s->pos, s->vel, s->acc, s->ep, s->ev, s->ea, s->pp_count, s->pp_id, s->pp_tsd,
                      s->pl_count, s->pl_id, s->pl_tsd, a->np, s->st);
}

// slab -> handle; the next step starts over from the restored state
cudaError_t restore_state(xdem_adj* a, const Slab& src)
{
    xdem_sim* s = a->s;
    Slab d{};
    d.pos = s->pos; d.vel = s->vel; d.acc = s->acc; d.ep = s->ep; d.ev = s->ev; d.ea = s->ea;
    if (a->pp) { d.ppc = s->pp_count; d.ppi = s->pp_id; d.ppt = s->pp_tsd; }
    if (a->pl) { d.plc = s->pl_count; d.pli = s->pl_id; d.plt = s->pl_tsd; }
    cudaError_t e = copy_state(d, src.pos, src.vel, src.acc, src.ep, src.ev, src.ea, src.ppc, src.ppi, src.ppt,
                               src.plc, src.pli, src.plt, a->np, s->st);
    fused_invalidate(s->fs);
    return e;
}

cudaError_t copy_slab(xdem_adj* a, const Slab& d, const Slab& src)
{
    return copy_state(d, src.pos, src.vel, src.acc, src.ep, src.ev, src.ea, src.ppc, src.ppi, src.ppt, src.plc,
                      src.pli, src.plt, a->np, a->s->st);
}

template <class T>
cudaError_t dalloc(T*& p, size_t n)
{
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T));
}

// Tables of the contact properties and planes the forward runs with.
int build_tables(xdem_adj* a)
{
    xdem_sim* s = a->s;
    const int model = s->cfg.contact_model;
    std::vector<adj::Mat> mats(a->nprop);
    a->cps.assign(a->nprop, device_contact_property{});
    for (unsigned int p = 0; p < a->nprop; ++p) {
        const device_contact_property cp = p == 0 ? s->pp_cp : s->body_cp[p - 1];
        a->cps[p] = cp;
        const mat_pair m = make_mat_pair(cp, model, false);
        mats[p] = adj::Mat{m.Eeq, m.Seq8, m.beta, m.vs1, m.sratio, m.fric};
    }
    std::vector<adj::PlaneContact> pcs(a->nplane);
    std::vector<unsigned int> pid(a->nplane);
    for (unsigned int k = 0; k < a->nplane; ++k) {
        const device_plane_info& pl = s->planes[k];
        adj::PlaneContact& c = pcs[k];
        auto v = [](const xdem_double3& d) { return adj::mkv(d.x, d.y, d.z); };
        c.rect.xw = v(pl.xw); c.rect.u1 = v(pl.u1); c.rect.u2 = v(pl.u2); c.rect.uw = v(pl.uw);
        c.rect.w2 = v(pl.w2); c.rect.w3 = v(pl.w3); c.rect.w4 = v(pl.w4);
        c.rect.l1 = pl.l1; c.rect.l2 = pl.l2;
        const double* r = s->bodies[k].rec;
        c.bp = adj::mkv(r[XDEM_PX], r[XDEM_PY], r[XDEM_PZ]);
        c.bv = adj::mkv(r[XDEM_VX], r[XDEM_VY], r[XDEM_VZ]);
        c.bw = adj::ang_vel(adj::mkq(r[XDEM_E0], r[XDEM_E1], r[XDEM_E2], r[XDEM_E3]),
                            adj::mkq(r[XDEM_ED0], r[XDEM_ED1], r[XDEM_ED2], r[XDEM_ED3]));
        c.mat = mats[1 + k];
        pid[k] = pl.id;
        for (unsigned int q = 0; q < k; ++q)
            if (pid[q] == pid[k]) return XDEM_ERR_ARG;  // plane ids must tell the planes apart
    }
    cudaStream_t st = s->st;
    cudaError_t e = cudaMemcpyAsync(a->d_mat, mats.data(), a->nprop * sizeof(adj::Mat), cudaMemcpyHostToDevice, st);
    if (a->nplane && e == cudaSuccess)
        e = cudaMemcpyAsync(a->d_planes, pcs.data(), a->nplane * sizeof(adj::PlaneContact), cudaMemcpyHostToDevice,
                            st);
    if (a->nplane && e == cudaSuccess)
        e = cudaMemcpyAsync(a->d_pid, pid.data(), a->nplane * sizeof(unsigned int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cerr(e);
}

// d(Eeq, Seq8, beta, vs1, fric) / d(fric, rest, Ei, Ej) applied to one
// property's accumulated gradient (getConstant, impl:362-386).
void chain_property(const device_contact_property& cp, int model, const double g[kGradFields], double out[4])
{
    const double Ei = cp.Ei, Ej = cp.Ej, pi = cp.pri, pj = cp.prj;
    const double D = Ei * (1 - pj * pj) + Ej * (1 - pi * pi);
    const double dEeq_dEi = Ej * Ej * (1 - pi * pi) / (D * D);
    const double dEeq_dEj = Ei * Ei * (1 - pj * pj) / (D * D);
    const double ci = 2.0 * (2.0 - pi) * (1.0 + pi), cj = 2.0 * (2.0 - pj) * (1.0 + pj);
    const double S = ci / Ei + cj / Ej;
    const double dSeq8_dEi = 8.0 * ci / (Ei * Ei) / (S * S);
    const double dSeq8_dEj = 8.0 * cj / (Ej * Ej) / (S * S);
    const double L = std::log(cp.rest), pi2 = XDEM_PI * XDEM_PI;
    const double dbeta_drest = -pi2 / (cp.rest * std::pow(L * L + pi2, 1.5));
    const double dvs1_dbeta = model == 1 ? 2.0 * std::sqrt(5.0 / 6.0) : cp.sratio;
    out[0] = g[4];
    out[1] = (g[2] + g[3] * dvs1_dbeta) * dbeta_drest;
    out[2] = g[0] * dEeq_dEi + g[1] * dSeq8_dEi;
    out[3] = g[0] * dEeq_dEj + g[1] * dSeq8_dEj;
}

int reverse_step(xdem_adj* a, const Slab& S0, const Slab& S1, int cur)
{
    xdem_sim* s = a->s;
    AdjArgs A{};
    A.np = a->np;
    A.nplane = a->nplane;
    A.nprop = a->nprop;
    A.model = s->cfg.contact_model;
    A.vel_compat = s->cfg.velocity_compat;
    A.dt = s->prm.dt;
    A.h2 = s->prm.half2dt;
    A.mass = s->mass;
    A.inertia = s->inertia;
    A.mat = a->d_mat;
    A.planes = a->d_planes;
    A.plane_pid = a->d_pid;
    A.lx = a->lx; A.lv = a->lv; A.la = a->la; A.le = a->le; A.led = a->led; A.lea = a->lea;
    A.lF = a->lF; A.lM = a->lM; A.lw = a->lw;
    A.lpp_new = a->lpp[cur]; A.lpp_old = a->lpp[cur ^ 1];
    A.lpl_new = a->lpl[cur]; A.lpl_old = a->lpl[cur ^ 1];
    A.other = a->other;
    A.gpart = a->gpart;
    Slab s0 = S0, s1 = S1;
    if (!a->pp) { s0.ppc = s1.ppc = nullptr; }
    if (!a->pl) { s0.plc = s1.plc = nullptr; }
    const unsigned int nb = a->nblocks;
    k_adj_velocity<<<nb, kAdjThreads, 0, s->st>>>(A, s0, s1);
    k_adj_contacts<<<nb, kAdjThreads, 0, s->st>>>(A, s0, s1);
    k_adj_gather<<<nb, kAdjThreads, 0, s->st>>>(A, s0, s1);
    return cerr(cudaGetLastError());
}

}  // namespace

XDEM_API int xdem_adj_create(xdem_sim* s, unsigned int checkpoint_every, xdem_adj** out)
{
    if (!s || !out || checkpoint_every == 0) return XDEM_ERR_ARG;
    *out = nullptr;
    // the adjoint covers free spheres, planes and the FP64 step without
    // cohesion or rolling resistance, one scene per handle
    if (s->cfg.precision != XDEM_FP64 || s->clusters || !s->meshes.empty() || s->nscene != 1) return XDEM_ERR_ARG;
    if (s->cfg.contact_model != 0 && s->cfg.contact_model != 1) return XDEM_ERR_ARG;
    if (s->planes.size() > kMaxAdjPlanes) return XDEM_ERR_ARG;
    if (s->has_pp && (s->pp_cp.coh != 0.0 || s->pp_cp.rfric != 0.0)) return XDEM_ERR_ARG;
    for (const device_contact_property& cp : s->body_cp)
        if (cp.coh != 0.0 || cp.rfric != 0.0) return XDEM_ERR_ARG;
    xdem_adj* a = new (std::nothrow) xdem_adj();
    if (!a) return XDEM_ERR_ALLOC;
    a->s = s;
    a->K = checkpoint_every;
    a->np = s->np;
    a->nplane = (unsigned int)s->planes.size();
    a->nprop = 1 + a->nplane;
    a->nblocks = (a->np + kAdjThreads - 1) / kAdjThreads;
    a->pp = s->has_pp;
    a->pl = a->nplane > 0;
    a->sbytes = slab_bytes(a->np, a->pp, a->pl);
    const size_t np = a->np;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&a->seg_mem), a->sbytes * (a->K + 1));
    if (e == cudaSuccess) {
        for (unsigned int t = 0; t <= a->K; ++t) a->seg.push_back(carve(a->seg_mem + t * a->sbytes, np, a->pp, a->pl));
    }
    if (e == cudaSuccess) e = dalloc(a->lx, np * 3);
    if (e == cudaSuccess) e = dalloc(a->lv, np * 3);
    if (e == cudaSuccess) e = dalloc(a->la, np * 3);
    if (e == cudaSuccess) e = dalloc(a->le, np * 4);
    if (e == cudaSuccess) e = dalloc(a->led, np * 4);
    if (e == cudaSuccess) e = dalloc(a->lea, np * 4);
    if (e == cudaSuccess) e = dalloc(a->lF, np * 3);
    if (e == cudaSuccess) e = dalloc(a->lM, np * 3);
    if (e == cudaSuccess) e = dalloc(a->lw, np * 3);
    if (e == cudaSuccess) e = dalloc(a->other, np * MAX_P2P_COUNT * 9);
    if (e == cudaSuccess) e = dalloc(a->lpp[0], np * MAX_P2P_COUNT * 2);
    if (e == cudaSuccess) e = dalloc(a->lpp[1], np * MAX_P2P_COUNT * 2);
    if (e == cudaSuccess) e = dalloc(a->lpl[0], np * MAX_P2PL_COUNT * 2);
    if (e == cudaSuccess) e = dalloc(a->lpl[1], np * MAX_P2PL_COUNT * 2);
    if (e == cudaSuccess) e = dalloc(a->gpart, (size_t)a->nblocks * a->nprop * kGradFields);
    if (e == cudaSuccess) e = dalloc(a->d_mat, a->nprop);
    if (e == cudaSuccess) e = dalloc(a->d_planes, std::max(1u, a->nplane));
    if (e == cudaSuccess) e = dalloc(a->d_pid, std::max(1u, a->nplane));
    if (e != cudaSuccess) {
        xdem_adj_destroy(a);
        cudaGetLastError();
        return XDEM_ERR_ALLOC;
    }
    *out = a;
    return XDEM_OK;
}

XDEM_API int xdem_adj_destroy(xdem_adj* a)
{
    if (!a) return XDEM_ERR_ARG;
    void* ps[] = {a->ckpt_mem, a->seg_mem, a->lx, a->lv, a->la, a->le, a->led, a->lea, a->lF, a->lM, a->lw,
                  a->other, a->gpart, a->lpp[0], a->lpp[1], a->lpl[0], a->lpl[1], a->d_mat, a->d_planes, a->d_pid,
                  a->tx, a->tv, a->ta, a->te, a->ted, a->tea, a->tF, a->tM, a->Mv, a->tmat, a->tpp[0], a->tpp[1],
                  a->tpl[0], a->tpl[1]};
    for (void* p : ps)
        if (p) cudaFree(p);
    delete a;
    return XDEM_OK;
}

XDEM_API int xdem_adj_forward(xdem_adj* a, unsigned int nsteps)
{
    if (!a || nsteps == 0) return XDEM_ERR_ARG;
    xdem_sim* s = a->s;
    if (s->planes.size() != a->nplane || s->has_pp != a->pp || !s->meshes.empty()) return XDEM_ERR_ARG;
    const size_t ncp = (nsteps + a->K - 1) / a->K;
    if (ncp > a->ckpt_n) {
        if (a->ckpt_mem) cudaFree(a->ckpt_mem);
        a->ckpt_mem = nullptr;
        a->ckpt.clear();
        a->ckpt_n = 0;
        if (cudaMalloc(reinterpret_cast<void**>(&a->ckpt_mem), a->sbytes * ncp) != cudaSuccess) {
            cudaGetLastError();
            return XDEM_ERR_ALLOC;
        }
        for (size_t c = 0; c < ncp; ++c) a->ckpt.push_back(carve(a->ckpt_mem + c * a->sbytes, a->np, a->pp, a->pl));
        a->ckpt_n = ncp;
    }
    // a zero-step call sets up the pair tables before the first checkpoint;
    // the status word starts clean so that the forward's own bits are seen
    if (int r = xdem_sim_step(s, 0)) return r;
    if (xdem_sim_status(s) & XDEM_ERR_CUDA) return XDEM_ERR_CUDA;
    a->nsteps = 0;
    for (size_t c = 0; c < ncp; ++c) {
        const unsigned int t0 = (unsigned int)(c * a->K);
        const unsigned int n = std::min(a->K, nsteps - t0);
        if (cudaError_t e = save_state(a, a->ckpt[c])) return cerr(e);
        // every segment starts the step over from its stored state, as the
        // reverse sweep's re-run will
        fused_invalidate(s->fs);
        if (int r = xdem_sim_step(s, n)) return r;
        a->nsteps = t0 + n;
    }
    if (int r = build_tables(a)) return r;
    const int st = xdem_sim_status(s);
    if (st != XDEM_OK) {
        a->nsteps = 0;  // overflowed pair lists or non-finite positions: no adjoint
        return st;
    }
    return XDEM_OK;
}

XDEM_API int xdem_adj_backward(xdem_adj* a, const double* dl_dpos, const double* dl_dvel, double* grad,
                               double* dl_dpos0, double* dl_dvel0)
{
    if (!a || a->nsteps == 0) return XDEM_ERR_ARG;
    xdem_sim* s = a->s;
    cudaStream_t st = s->st;
    const size_t np = a->np;
    cudaError_t e = cudaSuccess;
    auto seed = [&](double* d, const double* src, size_t n) {
        if (e != cudaSuccess) return;
        e = src ? cudaMemcpyAsync(d, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st)
                : cudaMemsetAsync(d, 0, n * sizeof(double), st);
    };
    seed(a->lx, dl_dpos, np * 3);
    seed(a->lv, dl_dvel, np * 3);
    seed(a->la, nullptr, np * 3);
    seed(a->le, nullptr, np * 4);
    seed(a->led, nullptr, np * 4);
    seed(a->lea, nullptr, np * 4);
    seed(a->lpp[0], nullptr, np * MAX_P2P_COUNT * 2);
    seed(a->lpl[0], nullptr, np * MAX_P2PL_COUNT * 2);
    seed(a->gpart, nullptr, (size_t)a->nblocks * a->nprop * kGradFields);
    if (e != cudaSuccess) return cerr(e);
    int cur = 0;
    const unsigned int ncp = (a->nsteps + a->K - 1) / a->K;
    for (int c = (int)ncp - 1; c >= 0; --c) {
        const unsigned int t0 = (unsigned int)c * a->K;
        const unsigned int n = std::min(a->K, a->nsteps - t0);
        // re-run the segment from its checkpoint, keeping every state
        if ((e = restore_state(a, a->ckpt[c])) != cudaSuccess) return cerr(e);
        if ((e = copy_slab(a, a->seg[0], a->ckpt[c])) != cudaSuccess) return cerr(e);
        for (unsigned int t = 0; t < n; ++t) {
            if (int r = xdem_sim_step(s, 1)) return r;
            if ((e = save_state(a, a->seg[t + 1])) != cudaSuccess) return cerr(e);
        }
        for (int t = (int)n - 1; t >= 0; --t) {
            if (int r = reverse_step(a, a->seg[t], a->seg[t + 1], cur)) return r;
            cur ^= 1;
        }
    }
    if (dl_dpos0) e = cudaMemcpyAsync(dl_dpos0, a->lx, np * 3 * sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (dl_dvel0 && e == cudaSuccess)
        e = cudaMemcpyAsync(dl_dvel0, a->lv, np * 3 * sizeof(double), cudaMemcpyDeviceToDevice, st);
    std::vector<double> part((size_t)a->nblocks * a->nprop * kGradFields);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(part.data(), a->gpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cerr(e);
    if (grad) {
        for (unsigned int p = 0; p < a->nprop; ++p) {
            double g[kGradFields] = {0, 0, 0, 0, 0};
            for (unsigned int b = 0; b < a->nblocks; ++b)
                for (int f = 0; f < kGradFields; ++f) g[f] += part[((size_t)b * a->nprop + p) * kGradFields + f];
            chain_property(a->cps[p], s->cfg.contact_model, g, grad + 4 * p);
        }
    }
    return XDEM_OK;
}

namespace {

// getConstant's terms (Eeq, Seq8, beta, vs1, fric) of property cp moved by
// h * d, d = (fric, rest, Ei, Ej).
void mat_terms(const device_contact_property& cp, int model, const double* d, double h, double out[5])
{
    device_contact_property c = cp;
    c.fric += h * d[0];
    c.rest += h * d[1];
    c.Ei += h * d[2];
    c.Ej += h * d[3];
    const mat_pair m = make_mat_pair(c, model, false);
    out[0] = m.Eeq; out[1] = m.Seq8; out[2] = m.beta; out[3] = m.vs1; out[4] = m.fric;
}

}  // namespace

XDEM_API int xdem_adj_tangent(xdem_adj* a, unsigned int ndir, const double* dparam, double* tpos, double* tvel)
{
    if (!a || a->nsteps == 0 || ndir == 0 || ndir > (unsigned int)kTanDirs || !dparam) return XDEM_ERR_ARG;
    xdem_sim* s = a->s;
    cudaStream_t st = s->st;
    const size_t np = a->np;
    const int model = s->cfg.contact_model;
    cudaError_t e = cudaSuccess;
    auto need = [&](double*& p, size_t n) {
        if (e == cudaSuccess && !p) e = cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * 8);
    };
    const size_t D = kTanDirs;
    need(a->tx, np * 3 * D); need(a->tv, np * 3 * D); need(a->ta, np * 3 * D);
    need(a->te, np * 4 * D); need(a->ted, np * 4 * D); need(a->tea, np * 4 * D);
    need(a->tF, np * 3 * D); need(a->tM, np * 3 * D); need(a->Mv, np * 3);
    need(a->tmat, (size_t)a->nprop * 5 * D);
    need(a->tpp[0], np * MAX_P2P_COUNT * 2 * D); need(a->tpp[1], np * MAX_P2P_COUNT * 2 * D);
    need(a->tpl[0], np * MAX_P2PL_COUNT * 2 * D); need(a->tpl[1], np * MAX_P2PL_COUNT * 2 * D);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return XDEM_ERR_ALLOC;
    }
    // material tangents by central differences of getConstant (smooth in
    // the parameters): a relative step of 1e-6 in the largest component
    std::vector<double> tm((size_t)a->nprop * 5 * D, 0.0);
    for (unsigned int k = 0; k < ndir; ++k)
        for (unsigned int p = 0; p < a->nprop; ++p) {
            const double* d = dparam + ((size_t)k * a->nprop + p) * 4;
            const device_contact_property& cp = a->cps[p];
            const double base[4] = {cp.fric, cp.rest, cp.Ei, cp.Ej};
            double rel = 0.0;
            for (int c = 0; c < 4; ++c)
                if (d[c] != 0.0) rel = std::max(rel, std::fabs(d[c]) / std::max(std::fabs(base[c]), 1e-300));
            if (rel == 0.0) continue;
            const double h = 1e-6 / rel;
            double fp[5], fm[5];
            mat_terms(cp, model, d, h, fp);
            mat_terms(cp, model, d, -h, fm);
            for (int f = 0; f < 5; ++f) tm[((size_t)p * 5 + f) * D + k] = (fp[f] - fm[f]) / (2.0 * h);
        }
    e = cudaMemcpyAsync(a->tmat, tm.data(), tm.size() * 8, cudaMemcpyHostToDevice, st);
    for (double* p : {a->tx, a->tv, a->ta, a->tF, a->tM})
        if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, np * 3 * D * 8, st);
    for (double* p : {a->te, a->ted, a->tea})
        if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, np * 4 * D * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->tpp[0], 0, np * MAX_P2P_COUNT * 2 * D * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->tpl[0], 0, np * MAX_P2PL_COUNT * 2 * D * 8, st);
    if (e != cudaSuccess) return cerr(e);
    // the stored trajectory again, from its first checkpoint
    if ((e = restore_state(a, a->ckpt[0])) != cudaSuccess) return cerr(e);
    if ((e = copy_slab(a, a->seg[0], a->ckpt[0])) != cudaSuccess) return cerr(e);
    TanArgs T{};
    T.np = a->np;
    T.nplane = a->nplane;
    T.model = model;
    T.vel_compat = s->cfg.velocity_compat;
    T.dt = s->prm.dt;
    T.h2 = s->prm.half2dt;
    T.mass = s->mass;
    T.inertia = s->inertia;
    T.mat = a->d_mat;
    T.tmat = a->tmat;
    T.planes = a->d_planes;
    T.plane_pid = a->d_pid;
    T.tx = a->tx; T.tv = a->tv; T.ta = a->ta; T.te = a->te; T.ted = a->ted; T.tea = a->tea;
    T.tF = a->tF; T.tM = a->tM; T.Mv = a->Mv;
    const unsigned int nb = a->nblocks;
    int cur = 0;
    for (unsigned int t = 0; t < a->nsteps; ++t) {
        if (int r = xdem_sim_step(s, 1)) return r;
        Slab s0 = a->seg[t & 1], s1 = a->seg[(t + 1) & 1];
        if ((e = save_state(a, s1)) != cudaSuccess) return cerr(e);
        if (!a->pp) { s0.ppc = s1.ppc = nullptr; }
        if (!a->pl) { s0.plc = s1.plc = nullptr; }
        T.tpp_old = a->tpp[cur]; T.tpp_new = a->tpp[cur ^ 1];
        T.tpl_old = a->tpl[cur]; T.tpl_new = a->tpl[cur ^ 1];
        k_tan_position<<<nb, kAdjThreads, 0, st>>>(T, s0);
        k_tan_contacts<<<nb, kAdjThreads, 0, st>>>(T, s0, s1);
        k_tan_velocity<<<nb, kAdjThreads, 0, st>>>(T, s0, s1);
        if ((e = cudaGetLastError()) != cudaSuccess) return cerr(e);
        cur ^= 1;
    }
    // direction-major outputs: out[k * np * 3 + 3 i + c]
    std::vector<double> h(np * 3 * D);
    auto out = [&](const double* src, double* dst) {
        if (!dst || e != cudaSuccess) return;
        e = cudaMemcpyAsync(h.data(), src, h.size() * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return;
        std::vector<double> o(np * 3 * ndir);
        for (unsigned int k = 0; k < ndir; ++k)
            for (size_t c = 0; c < np * 3; ++c) o[k * np * 3 + c] = h[c * D + k];
        e = cudaMemcpyAsync(dst, o.data(), o.size() * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    };
    out(a->tx, tpos);
    out(a->tv, tvel);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cerr(e);
    return xdem_sim_status(s);  // the re-run's own overflow or non-finite bits, if any
}

XDEM_API int xdem_adj_info(xdem_adj* a, unsigned int* nprop, unsigned int* nsteps, unsigned long long* bytes)
{
    if (!a) return XDEM_ERR_ARG;
    if (nprop) *nprop = a->nprop;
    if (nsteps) *nsteps = a->nsteps;
    if (bytes) *bytes = (unsigned long long)a->sbytes * (a->K + 1 + a->ckpt_n);
    return XDEM_OK;
}
