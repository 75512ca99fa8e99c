// xdem_kernels.cu -- FP64 DEM kernels of the launcher surface.
//
// One thread per particle (or cluster / triangle) in the caller's order, the
// reference's layouts and pair-list slot rules.  Compiled with -fmad=false:
// every product and sum rounds on its own, so cell ids, sort order and pair
// lists agree bit for bit with the CPU oracle and forces agree to rounding.
//
// Deviations from the literal reference, shared with the oracle:
//  * a pair beyond a particle's slot capacity is not stored (the reference
//    writes it into the next particle's slots) and raises a status bit; its
//    force is still applied;
//  * pow(x, 1.5) is evaluated as x * sqrt(x) and pow(x, 2.0) as x * x;
//  * the Euler-parameter acceleration uses the closed-form inverse of the
//    reference's 4x4 system (see uceom in xdem_device.cuh).
#include "xdem_device.cuh"
#include "xdem_kernels.h"

namespace xdem {

// ---------------------------------------------------------------- block sums
// Reduces six per-thread doubles over the block; thread 0 gets the totals.
__device__ __forceinline__ void block_sum6(double v[6], double* smem /* [6 * 32] */)
{
#pragma unroll
    for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int c = 0; c < 6; ++c) smem[c * 32 + warp] = v[c];
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (warp == 0) {
        for (int c = 0; c < 6; ++c) {
            double x = lane < nw ? smem[c * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[c] = x;
        }
    }
}

__device__ __forceinline__ void emit_body_partials(const BodyPartials& bp, unsigned int id, bool valid,
                                                   double f[6])
{
    if (valid && bp.fx) {
        bp.fx[id] = f[0]; bp.fy[id] = f[1]; bp.fz[id] = f[2];
        bp.mx[id] = f[3]; bp.my[id] = f[4]; bp.mz[id] = f[5];
    }
    if (bp.block_sums) {
        __shared__ double sm[6 * 32];
        double v[6];
        for (int c = 0; c < 6; ++c) v[c] = valid ? f[c] : 0.0;
        block_sum6(v, sm);
        if (threadIdx.x == 0)
            for (int c = 0; c < 6; ++c) bp.block_sums[blockIdx.x * 6 + c] = v[c];
    }
}

// ---------------------------------------------------------------- VV (impl:135-222)
__global__ void k_vv_position(device_dem_parameters p, double* pos, double* ep, const double* vel, const double* ev,
                              const double* acc, const double* ea, unsigned int n)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = p.dt, h = p.half2dt;
    const d4 e = (ld4(ep, i) + dt * ld4(ev, i)) + h * ld4(ea, i);
    const double l = sqrt(dot(e, e));
    st4(ep, i, mk4(e.x / l, e.y / l, e.z / l, e.w / l));
    const d3 d = dt * ld3(vel, i) + h * ld3(acc, i);
    double4_32a* p4 = reinterpret_cast<double4_32a*>(pos) + i;
    double4_32a q = *p4;
    q.x += d.x; q.y += d.y; q.z += d.z;
    *p4 = q;
}

__global__ void k_vv_velocity(device_dem_parameters p, double* vel, double* acc, const double* ep, double* ev,
                              double* ea, double* force, double* moment, const double* mass, const double* iner,
                              unsigned int n, int compat)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hdt = 0.5 * p.dt;
    const double m = mass[i];
    const double inv = 1.0 / m;
    const d3 a = inv * (ld3(force, i) + m * dv3(p.gravity));
    const d4 e = ld4(ep, i);
    d4 av = ld4(ev, i);
    const d3 nb = to_local(ld3(moment, i), e);
    const d4 q = uceom(ld3(iner, i), e, av, nb);
    av = av + hdt * (ld4(ea, i) + q);
    st3(force, i, mk3(0, 0, 0));
    st3(moment, i, mk3(0, 0, 0));
    if (!compat) st3(vel, i, ld3(vel, i) + hdt * (ld3(acc, i) + a));
    st4(ev, i, av);
    st3(acc, i, a);
    st4(ea, i, q);
}

// ---------------------------------------------------------------- grid (impl:290-360)
__global__ void k_hash(device_dem_parameters p, unsigned int* hash, unsigned int* index, const double* pos,
                       unsigned int sid, unsigned int n, unsigned int* status)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const d3 q = ld4xyz(pos, i);
    if (!(isfinite(q.x) && isfinite(q.y) && isfinite(q.z))) atomicOr(status, (unsigned int)XDEM_ERR_NONFINITE);
    const int3v g = grid_pos(p, q);
    hash[sid + i] = grid_hash(p, g.x, g.y, g.z);
    index[sid + i] = sid + i;
}

__global__ void k_cell_bounds(const unsigned int* key, const unsigned int* val, unsigned int* cstart,
                              unsigned int* cend, unsigned int* sorted_index, unsigned int n)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int h = key[i];
    if (i == 0 || h != key[i - 1]) {
        cstart[h] = i;
        if (i > 0) cend[key[i - 1]] = i;
    }
    if (i == n - 1) cend[h] = i + 1;
    sorted_index[i] = val[i];
}

__global__ void k_clear_cells(const unsigned int* key, unsigned int n, unsigned int* cstart, unsigned int* cend,
                              const unsigned int* gate)
{
    if (gate && !*gate) return;
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int h = key[i];
    cstart[h] = 0xffffffffu;
    cend[h] = 0u;
}

__global__ void k_fill_u32(unsigned int* a, unsigned int v, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] = v;
}

// ---------------------------------------------------------------- particle-particle (impl:613-733)
template <int CAP>
struct OldPairs {
    unsigned int id[CAP];
    double sd0[CAP], sd1[CAP];
    unsigned int count;
    __device__ __forceinline__ void load(const unsigned int* pair_id, const double* tsd, unsigned int sid,
                                         unsigned int cnt)
    {
        count = cnt;
#pragma unroll
        for (int i = 0; i < CAP; ++i) {
            id[i] = pair_id[sid + i];
            const double2 t = reinterpret_cast<const double2*>(tsd)[sid + i];
            sd0[i] = t.x; sd1[i] = t.y;
        }
    }
    // first slot below `lim` holding k
    __device__ __forceinline__ bool find(unsigned int k, unsigned int lim, double& a, double& b) const
    {
        bool hit = false;
#pragma unroll
        for (int i = 0; i < CAP; ++i) {
            if (!hit && (unsigned int)i < lim && id[i] == k) { a = sd0[i]; b = sd1[i]; hit = true; }
        }
        return hit;
    }
};

__device__ __forceinline__ void store_pair(unsigned int* pair_id, double* tsd, unsigned int sid, unsigned int& cnt,
                                           unsigned int cap, unsigned int k, double a, double b, unsigned int& bits,
                                           unsigned int err)
{
    if (cnt < cap) {
        pair_id[sid + cnt] = k;
        reinterpret_cast<double2*>(tsd)[sid + cnt] = make_double2(a, b);
        cnt++;
    } else {
        bits |= err;
    }
}

__global__ void __launch_bounds__(kThreads)
k_p2p(device_dem_parameters p, const double* pos, const double* ep, const double* vel, const double* ev,
      double* force, double* moment, const double* mass, double* tmax, double* rres, unsigned int* pair_count,
      unsigned int* pair_id, double* tsd, const unsigned int* sorted_index, const unsigned int* cstart,
      const unsigned int* cend, const mat_pair* mpp, unsigned int n, unsigned int* status)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const mat_pair mp = *mpp;
    const int model = p.contact_model;
    const double dt = p.dt;
    const unsigned int sid = id * MAX_P2P_COUNT;
    OldPairs<MAX_P2P_COUNT> old;
    {
        unsigned int c = pair_count[id];
        old.load(pair_id, tsd, sid, c > MAX_P2P_COUNT ? MAX_P2P_COUNT : c);
    }
    const d4 ip4 = ld4(pos, id);
    const d3 ipos = mk3(ip4.x, ip4.y, ip4.z);
    const d3 ivel = ld3(vel, id);
    const d3 iom = ang_vel(ld4(ep, id), ld4(ev, id));
    const int3v g = grid_pos(p, ipos);
    const double ir = ip4.w, im = mass[id];
    d3 Ft = mk3(0, 0, 0), Fn = mk3(0, 0, 0), sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
    double res = 0.0;
    unsigned int cnt = 0, bits = 0;
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                const unsigned int h = grid_hash(p, g.x + x, g.y + y, g.z + z);
                const unsigned int start = cstart[h];
                if (start == 0xffffffffu) continue;
                const unsigned int end = cend[h];
                for (unsigned int j = start; j < end; ++j) {
                    const unsigned int k = sorted_index[j];
                    if (id == k || k >= n) continue;
                    const d4 jp4 = ld4(pos, k);
                    const double jr = jp4.w;
                    const d3 rp = mk3(jp4.x - ip4.x, jp4.y - ip4.y, jp4.z - ip4.z);
                    const double dist = length(rp);
                    const double cdist = (ir + jr) - dist;
                    double cs = 0.0;
                    if (mp.coh) cs = limit_cohesion_depth(mp, ir, jr);
                    if (cdist > 0) {
                        double sd0 = 0.0, sd1 = 0.0;
                        old.find(k, old.count, sd0, sd1);
                        const d3 unit = rp / dist;
                        const d3 cpt = ipos + ir * unit;
                        const d3 jvel = ld3(vel, k);
                        const d3 jom = ang_vel(ld4(ep, k), ld4(ev, k));
                        const double jm = mass[k];
                        const d3 dcpr = cpt - ipos;
                        const d3 dcpr_j = cpt - mk3(jp4.x, jp4.y, jp4.z);
                        const d3 rv = (jvel + cross(jom, dcpr_j)) - (ivel + cross(iom, dcpr));
                        const fconst c = get_constant(mp, model, ir, jr, im, jm);
                        contact_model(model, c, mp, ir, jr, dt, cdist, sd0, sd1, rv, unit, Ft, Fn);
                        rolling_accumulate(mp.rfric, ir, jr, dcpr, Fn, Ft, res, tma);
                        sumF = sumF + (Fn + Ft);
                        sumM = sumM + cross(dcpr, Fn + Ft);
                        store_pair(pair_id, tsd, sid, cnt, MAX_P2P_COUNT, k, sd0, sd1, bits, XDEM_ERR_P2P_OVERFLOW);
                    } else if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
                        const d3 unit = rp / dist;
                        const double f = jkr_separation_force(mp, ir, jr);
                        const double cf = cohesion_force(mp, ir, jr, f);
                        sumF = sumF - cf * unit;
                        store_pair(pair_id, tsd, sid, cnt, MAX_P2P_COUNT, k, 0.0, 0.0, bits, XDEM_ERR_P2P_OVERFLOW);
                    }
                }
            }
    add3to(force, id, sumF);
    add3to(moment, id, sumM);
    pair_count[id] = cnt;
    add3to(tmax, id, tma);
    rres[id] += res;
    if (bits) atomicOr(status, bits);
}

// ---------------------------------------------------------------- planes (impl:817-1080)
template <bool CLUSTER>
__global__ void __launch_bounds__(kThreads)
k_plane(device_dem_parameters p, const device_plane_info* planep, const double* dbi, const mat_pair* mpp,
        BodyPartials bp,
        const double* pos, const double* cpos, const double* ep, const double* vel, const double* ev,
        double* force, double* moment, const double* mass, double* tmax, double* rres, unsigned int* pair_count,
        unsigned int* pair_id, double* tsd, const xClusterInformation* xci, unsigned int n, unsigned int* status)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = id < n;
    double f6[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const mat_pair mp = *mpp;
        const device_plane_info& plane = *planep;
        const int model = p.contact_model;
        const double dt = p.dt;
        const body_state b = load_body(dbi);
        const unsigned int sid = id * MAX_P2PL_COUNT;
        OldPairs<MAX_P2PL_COUNT> old;
        const unsigned int old_count = pair_count[id];
        old.load(pair_id, tsd, sid, old_count);
        unsigned int ci = id;
        if (CLUSTER) {
            const unsigned int ne = cluster_neach(xci, p.nClusterObject, id);
            ci = ne ? id / ne : 0;
        }
        const double m = mass[ci];
        const d4 ip4 = ld4(pos, id);
        const d3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        const double r = ip4.w;
        const unsigned int k = plane.id;
        const d3 ivel = ld3(vel, ci);
        const d3 iom = ang_vel(ld4(ep, ci), ld4(ev, ci));
        d3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0), sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = k ? old_count : 0, bits = 0;
        const d3 dp = ipos - dv3(plane.xw);
        d3 unit = mk3(0, 0, 0);
        const d3 wp = mk3(dot(dp, dv3(plane.u1)), dot(dp, dv3(plane.u2)), dot(dp, dv3(plane.uw)));
        // cluster kernel: body lever arm from the particle centre (impl:881-882)
        const d3 dcpr_j_cl = ipos - b.p;
        const double cdist = plane_detection(plane, ipos, wp, unit, r);
        double cs = 0.0;
        if (mp.coh) cs = limit_cohesion_depth(mp, r, 0.0);
        const d3 cpt = ipos + r * unit;
        const d3 dcpr_j = CLUSTER ? dcpr_j_cl : cpt - b.p;
        bool store = false;
        double sd0 = 0.0, sd1 = 0.0;
        d3 mf = mk3(0, 0, 0);
        if (cdist > 0) {
            old.find(k, MAX_P2PL_COUNT, sd0, sd1);
            const d3 dcpr = CLUSTER ? cpt - ld4xyz(cpos, ci) : cpt - ipos;
            const d3 dv = (b.v + cross(b.om, dcpr_j)) - (ivel + cross(iom, dcpr));
            const fconst c = get_constant(mp, model, r, 0.0, m, CLUSTER ? b.m : 0.0);
            contact_model(model, c, mp, r, 0.0, dt, cdist, sd0, sd1, dv, unit, Ft, Fn);
            rolling_accumulate(mp.rfric, r, 0.0, dcpr, Fn, Ft, res, tma);
            mf = Fn + Ft;
            sumF = sumF + mf;
            sumM = sumM + cross(dcpr, mf);
            store = true;
        } else if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
            const double f = jkr_separation_force(mp, r, 0.0);
            const double cf = cohesion_force(mp, r, 0.0, f);
            mf = (-cf) * unit;
            sumF = sumF + mf;
            store = true;
        }
        if (store) {
            f6[0] = -mf.x; f6[1] = -mf.y; f6[2] = -mf.z;
            const d3 bm = -cross(dcpr_j, mf);
            f6[3] = bm.x; f6[4] = bm.y; f6[5] = bm.z;
            store_pair(pair_id, tsd, sid, cnt, MAX_P2PL_COUNT, k, sd0, sd1, bits, XDEM_ERR_P2PL_OVERFLOW);
        }
        add3to(force, id, sumF);
        add3to(moment, id, sumM);
        pair_count[id] = cnt;
        add3to(tmax, id, tma);
        rres[id] += res;
        if (bits) atomicOr(status, bits);
    }
    emit_body_partials(bp, id, valid, f6);
}

// ---------------------------------------------------------------- cylinders (impl:1083-1601)
// impl:1324-1601: one cylinder against every particle.  The side/annulus/
// rim contact carries pair id k = cyl->id, the inner cap of a sphere inside
// k + 1000; slots follow the plane rule (k == 0 restarts the list), bounded
// by MAX_P2CY_COUNT here (the reference writes on without a bound).
// CLUSTER: members with their cluster's mass, velocity and spin, lever arms
// from the cluster centre.  The body's mass does not enter the effective
// mass (getConstant(r, 0, m, 0, ...)).
template <bool CLUSTER>
__global__ void __launch_bounds__(kThreads)
k_cylinder(device_dem_parameters p, const device_cylinder_info* cylp, const double* bi, const mat_pair* mpp,
           BodyPartials bp, const double* pos, const double* cpos, const double* ep, const double* vel,
           const double* ev, double* force, double* moment, const double* mass, double* tmax, double* rres,
           unsigned int* pair_count, unsigned int* pair_id, double* tsd, const xClusterInformation* xci,
           unsigned int n, unsigned int* status)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = id < n;
    double f6[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const mat_pair mp = *mpp;
        const device_cylinder_info cy = *cylp;
        const int model = p.contact_model;
        const double dt = p.dt;
        const body_state b = load_body(bi);
        const unsigned int sid = id * MAX_P2CY_COUNT;
        OldPairs<MAX_P2CY_COUNT> old;
        const unsigned int old_count = pair_count[id];
        old.load(pair_id, tsd, sid, old_count);
        unsigned int ci = id;
        if (CLUSTER) {
            const unsigned int ne = cluster_neach(xci, p.nClusterObject, id);
            ci = ne ? id / ne : 0;
        }
        const double m = mass[ci];
        const d4 ip4 = ld4(pos, id);
        const d3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        const double r = ip4.w;
        const unsigned int k = cy.id;
        const d3 ivel = ld3(vel, ci);
        const d3 iom = ang_vel(ld4(ep, ci), ld4(ev, ci));
        const d3 arm0 = CLUSTER ? ld4xyz(cpos, ci) : ipos;
        d3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = k ? old_count : 0, bits = 0;
        bool inner = false;
        d3 unit = mk3(0, 0, 0);
        double cdist = cylinder_detection(cy, bi, ipos, unit, r, inner);
        double cs = 0.0;
        if (mp.coh) cs = limit_cohesion_depth(mp, r, 0.0);
        d3 cpt = ipos + r * unit;
        for (int pass = 0; pass < 2; ++pass) {
            const unsigned int pid = pass ? k + 1000 : k;
            if (pass) {
                if (!inner) break;
                cdist = cylinder_inner_cap(cy, bi, ipos, unit, cpt, cy.empty_part, r);
            }
            d3 mf = mk3(0, 0, 0);
            double sd0 = 0.0, sd1 = 0.0;
            if (cdist > 0) {
                old.find(pid, MAX_P2CY_COUNT, sd0, sd1);
                const d3 po2cp = cpt - b.p;
                const d3 rc = cpt - arm0;
                const d3 dv = (b.v + cross(b.om, po2cp)) - (ivel + cross(iom, rc));
                const fconst c = get_constant(mp, model, r, 0.0, m, 0.0);
                d3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
                contact_model(model, c, mp, r, 0.0, dt, cdist, sd0, sd1, dv, unit, Ft, Fn);
                rolling_accumulate(mp.rfric, r, 0.0, rc, Fn, Ft, res, tma);
                mf = Fn + Ft;
                sumF = sumF + mf;
                sumM = sumM + cross(rc, mf);
            } else if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
                const double f = jkr_separation_force(mp, r, 0.0);
                const double cf = cohesion_force(mp, r, 0.0, f);
                mf = (-cf) * unit;
                sumF = sumF + mf;
            } else {
                continue;
            }
            f6[0] += -mf.x; f6[1] += -mf.y; f6[2] += -mf.z;
            const d3 bm = -cross(cpt - b.p, mf);
            f6[3] += bm.x; f6[4] += bm.y; f6[5] += bm.z;
            store_pair(pair_id, tsd, sid, cnt, MAX_P2CY_COUNT, pid, sd0, sd1, bits, XDEM_ERR_P2CY_OVERFLOW);
        }
        add3to(force, id, sumF);
        add3to(moment, id, sumM);
        pair_count[id] = cnt;
        add3to(tmax, id, tma);
        rres[id] += res;
        if (bits) atomicOr(status, bits);
    }
    emit_body_partials(bp, id, valid, f6);
}

// ---------------------------------------------------------------- meshes (impl:1748-2268)
struct TriHit { unsigned int id; d3 cpt; };

template <bool CLUSTER>
__global__ void __launch_bounds__(kThreads)
k_mesh(device_dem_parameters p, const device_triangle_info* dti, unsigned int lo_base, int lo_field,
       const double* dbi,
       const mat_pair* mpp,
       BodyPartials bp, const double* pos, const double* cpos, const double* ep, const double* vel, const double* ev,
       double* force, double* moment, const double* mass, double* tmax, double* rres, unsigned int* pair_count,
       unsigned int* pair_id, double* tsd, const unsigned int* sorted_index, const unsigned int* cstart,
       const unsigned int* cend, const xClusterInformation* xci, unsigned int n, unsigned int ntri,
       unsigned int* status)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = id < n;
    double f6[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const mat_pair mp = *mpp;
        const unsigned int lo = lo_base + (lo_field == 1 ? dti[0].tid : lo_field == 2 ? (unsigned int)dti[0].id : 0u);
        const int model = p.contact_model;
        const double dt = p.dt;
        const unsigned int sid = id * MAX_P2MS_COUNT;
        OldPairs<MAX_P2MS_COUNT> old;
        old.load(pair_id, tsd, sid, pair_count[id]);
        unsigned int ci = id;
        if (CLUSTER) {
            const unsigned int ne = cluster_neach(xci, p.nClusterObject, id);
            ci = ne ? id / ne : 0;
        }
        const double im = mass[ci];
        const d4 ip4 = ld4(pos, id);
        const d3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        const d3 icp = CLUSTER ? ld4xyz(cpos, ci) : mk3(0, 0, 0);
        const d3 ivel = ld3(vel, ci);
        const d3 iom = ang_vel(ld4(ep, ci), ld4(ev, ci));
        const double ir = ip4.w;
        const int3v g = grid_pos(p, ipos);
        unsigned int bits = 0;
        // candidate lists: faces, edges, vertices (impl:1975-1977)
        TriHit hf[XDEM_MAX_TRI_CANDIDATES], hl[XDEM_MAX_TRI_CANDIDATES], hp[XDEM_MAX_TRI_CANDIDATES];
        unsigned int nf = 0, nl = 0, np_ = 0;
        d3 prev_line = mk3(0, 0, 0), prev_point = mk3(0, 0, 0);
        double cs = 0.0;
        if (mp.coh) cs = limit_cohesion_depth(mp, ir, 0.0);
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    const unsigned int h = grid_hash(p, g.x + x, g.y + y, g.z + z);
                    const unsigned int start = cstart[h];
                    if (start == 0xffffffffu) continue;
                    const unsigned int end = cend[h];
                    for (unsigned int j = start; j < end; ++j) {
                        unsigned int tk = sorted_index[j];
                        if (!(tk >= lo && tk < lo + ntri)) continue;
                        tk -= lo;
                        int t = -1;
                        const d3 cpt = closest_pt_triangle(dti[tk], ipos, t);
                        const double cdist = ir - length(ipos - cpt);
                        bool take = false;
                        if (cdist > 0) {
                            if (t == 1) {
                                if (check_overlap(prev_line, cpt)) continue;
                                prev_line = cpt;
                            } else if (t == 0) {
                                if (check_overlap(prev_point, cpt)) continue;
                                prev_point = cpt;
                            }
                            take = true;
                        } else if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
                            take = true;
                        }
                        if (!take) continue;
                        const TriHit hit{tk, cpt};
                        if (t == 2) { if (nf < XDEM_MAX_TRI_CANDIDATES) hf[nf++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                        else if (t == 1) { if (nl < XDEM_MAX_TRI_CANDIDATES) hl[nl++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                        else if (t == 0) { if (np_ < XDEM_MAX_TRI_CANDIDATES) hp[np_++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                    }
                }
        const TriHit* list = nf ? hf : (nl ? hl : hp);
        const unsigned int nlist = nf ? nf : (nl ? nl : np_);
        const body_state b = load_body(dbi);
        d3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = 0;
        for (unsigned int q = 0; q < nlist; ++q) {
            const TriHit hit = list[q];
            double sd0 = 0.0, sd1 = 0.0;
            const d3 po2cp = hit.cpt - b.p;
            d3 unit;
            double cdist;
            if (!CLUSTER) {
                const d3 rp = hit.cpt - ipos;
                const double dist = length(rp);
                unit = rp / dist;
                cdist = ir - dist;
            } else {
                unit = hit.cpt - ipos;
                cdist = ir - length(ipos - hit.cpt);
            }
            if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
                const double f = jkr_separation_force(mp, ir, 0.0);
                const double cf = cohesion_force(mp, ir, 0.0, f);
                sumF = sumF - cf * unit;
            } else {
                d3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
                d3 rc;
                if (!CLUSTER) {
                    rc = hit.cpt - ipos;
                } else {
                    rc = hit.cpt - icp;
                    unit = unit / length(unit);
                }
                old.find(hit.id, MAX_P2MS_COUNT, sd0, sd1);
                const d3 dv = (b.v + cross(b.om, po2cp)) - (ivel + cross(iom, rc));
                const fconst c = get_constant(mp, model, ir, 0.0, im, b.m);
                contact_model(model, c, mp, ir, 0.0, dt, cdist, sd0, sd1, dv, unit, Ft, Fn);
                rolling_accumulate(mp.rfric, ir, 0.0, rc, Fn, Ft, res, tma);
                const d3 mf = Fn + Ft;
                sumF = sumF + mf;
                sumM = sumM + cross(rc, mf);
                f6[0] += -mf.x; f6[1] += -mf.y; f6[2] += -mf.z;
                const d3 mm = -cross(po2cp, mf);
                f6[3] += mm.x; f6[4] += mm.y; f6[5] += mm.z;
            }
            store_pair(pair_id, tsd, sid, cnt, MAX_P2MS_COUNT, hit.id, sd0, sd1, bits, XDEM_ERR_P2MS_OVERFLOW);
        }
        add3to(force, id, sumF);
        add3to(moment, id, sumM);
        pair_count[id] = cnt;
        add3to(tmax, id, tma);
        rres[id] += res;
        if (bits) atomicOr(status, bits);
    }
    emit_body_partials(bp, id, valid, f6);
}

// ---------------------------------------------------------------- rolling (impl:2420-2500)
// per_sphere: J = inertia[3 i], the sphere's own entry, instead of the flat
// entry i the reference reads (impl:2434)
__global__ void k_rolling(device_dem_parameters p, double* tmax, double* rres, const double* inertia,
                          const double* ep, const double* ev, double* moment, unsigned int n, int per_sphere)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double Tr = rres[i];
    if (!Tr) return;
    const d3 Tm = ld3(tmax, i);
    const double J = per_sphere ? inertia[3 * (size_t)i] : inertia[i];
    const d3 om = ang_vel(ld4(ep, i), ld4(ev, i));
    const d3 T = (J * p.dt) * om - Tm;
    const double lT = length(T);
    if (lT && Tr) {
        d3 Tr3 = Tr * (T / lT);
        if (length(Tr3) >= lT) Tr3 = T;
        add3to(moment, i, Tr3);
    }
    st3(tmax, i, mk3(0, 0, 0));
    rres[i] = 0.0;
}

__global__ void k_cluster_rolling(device_dem_parameters p, double* tmax, double* rres, const double* inertia,
                                  const double* ep, const double* ev, double* moment, const xClusterInformation* xci,
                                  unsigned int n)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double Tr = rres[i];
    if (!Tr) return;
    const unsigned int ne = cluster_neach(xci, p.nClusterObject, i);
    const unsigned int cid = ne ? i / ne : 0;
    const d3 Tm = ld3(tmax, i);
    const d3 J = ld3(inertia, cid);
    const d3 om = ang_vel(ld4(ep, cid), ld4(ev, cid));
    const d3 Jw = mk3(J.x * om.x, J.y * om.y, J.z * om.z);
    const d3 T = p.dt * Jw - Tm;
    const double lT = length(T);
    if (lT && Tr) {
        d3 Tr3 = Tr * (T / lT);
        if (length(Tr3) >= lT) Tr3 = T;
        st3(moment, i, ld3(moment, i) - Tr3);
    }
    st3(tmax, i, mk3(0, 0, 0));
    rres[i] = 0.0;
}

// ---------------------------------------------------------------- mesh pose (impl:2544-2601)
__global__ void k_update_mesh(const double* dbi, const double* vlist, double* sphere, const double* dlocal,
                              device_triangle_info* dpi, unsigned int ntri)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntri) return;
    const d3 bp = mk3(dbi[XDEM_PX], dbi[XDEM_PY], dbi[XDEM_PZ]);
    const d4 e = mk4(dbi[XDEM_E0], dbi[XDEM_E1], dbi[XDEM_E2], dbi[XDEM_E3]);
    const double* v = vlist + 9 * (size_t)i;
    const d3 P = bp + to_global(mk3(v[0], v[1], v[2]), e);
    const d3 Q = bp + to_global(mk3(v[3], v[4], v[5]), e);
    const d3 R = bp + to_global(mk3(v[6], v[7], v[8]), e);
    const d3 c = bp + to_global(ld3(dlocal, i), e);
    sphere[4 * (size_t)i] = c.x; sphere[4 * (size_t)i + 1] = c.y; sphere[4 * (size_t)i + 2] = c.z;
    dpi[i].P = xdem_double3{P.x, P.y, P.z};
    dpi[i].Q = xdem_double3{Q.x, Q.y, Q.z};
    dpi[i].R = xdem_double3{R.x, R.y, R.z};
}

// ---------------------------------------------------------------- clusters (impl:149-287, 485-611)
__global__ void __launch_bounds__(kThreads)
k_clusters_p2p(device_dem_parameters p, const double* pos, const double* cpos, const double* ep, const double* vel,
               const double* ev, double* force, double* moment, const double* mass, double* tmax, double* rres,
               unsigned int* pair_count, unsigned int* pair_id, double* tsd, const unsigned int* sorted_index,
               const unsigned int* cstart, const unsigned int* cend, const mat_pair* mpp,
               const xClusterInformation* xci, unsigned int n, unsigned int* status)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const mat_pair mp = *mpp;
    const int model = p.contact_model;
    const double dt = p.dt;
    const unsigned int sid = id * MAX_P2P_COUNT;
    OldPairs<MAX_P2P_COUNT> old;
    {
        unsigned int c = pair_count[id];
        old.load(pair_id, tsd, sid, c > MAX_P2P_COUNT ? MAX_P2P_COUNT : c);
    }
    const unsigned int neach = cluster_neach(xci, p.nClusterObject, id);
    const unsigned int cid = neach ? id / neach : 0;
    const d3 icpos = ld4xyz(cpos, cid);
    const d4 ip4 = ld4(pos, id);
    const d3 ipos = mk3(ip4.x, ip4.y, ip4.z);
    const d3 ivel = ld3(vel, cid);
    const d3 iom = ang_vel(ld4(ep, cid), ld4(ev, cid));
    const int3v g = grid_pos(p, ipos);
    const double ir = ip4.w, im = mass[cid];
    d3 Ft = mk3(0, 0, 0), Fn = mk3(0, 0, 0), sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
    double res = 0.0;
    unsigned int cnt = 0, bits = 0;
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                const unsigned int h = grid_hash(p, g.x + x, g.y + y, g.z + z);
                const unsigned int start = cstart[h];
                if (start == 0xffffffffu) continue;
                const unsigned int end = cend[h];
                for (unsigned int j = start; j < end; ++j) {
                    const unsigned int k = sorted_index[j];
                    const unsigned int di = id >= k ? id - k : k - id;
                    if (id == k || k >= n || di <= neach) continue;
                    const d4 jp4 = ld4(pos, k);
                    const double jr = jp4.w;
                    const d3 rp = mk3(jp4.x - ip4.x, jp4.y - ip4.y, jp4.z - ip4.z);
                    const double dist = length(rp);
                    const double cdist = (ir + jr) - dist;
                    if (cdist > 0) {
                        const unsigned int ck = neach ? k / neach : 0;
                        double sd0 = 0.0, sd1 = 0.0;
                        old.find(k, old.count, sd0, sd1);
                        const d3 jvel = ld3(vel, ck);
                        const d3 jom = ang_vel(ld4(ep, ck), ld4(ev, ck));
                        const double jm = mass[ck];
                        const d3 jcpos = ld4xyz(cpos, ck);
                        const d3 unit = rp / dist;
                        const d3 cpt = ipos + ir * unit;
                        const d3 dcpr = cpt - icpos;
                        const d3 dcpr_j = cpt - jcpos;
                        const d3 rv = (jvel + cross(jom, dcpr_j)) - (ivel + cross(iom, dcpr));
                        const fconst c = get_constant(mp, model, ir, jr, im, jm);
                        contact_model(model, c, mp, ir, jr, dt, cdist, sd0, sd1, rv, unit, Ft, Fn);
                        rolling_accumulate(mp.rfric, ir, jr, dcpr, Fn, Ft, res, tma);
                        sumF = sumF + (Fn + Ft);
                        sumM = sumM + cross(dcpr, Fn + Ft);
                        store_pair(pair_id, tsd, sid, cnt, MAX_P2P_COUNT, k, sd0, sd1, bits, XDEM_ERR_P2P_OVERFLOW);
                    }
                }
            }
    add3to(force, id, sumF);
    add3to(moment, id, sumM);
    pair_count[id] = cnt;
    add3to(tmax, id, tma);
    rres[id] += res;
    if (bits) atomicOr(status, bits);
}

__device__ __forceinline__ void cluster_slot(const xClusterInformation* xci, unsigned int nco, unsigned int i,
                                             unsigned int& neach, unsigned int& seach, unsigned int& sbegin,
                                             unsigned int& scl)
{
    neach = 0; seach = 0; sbegin = 0; scl = 0;
    for (unsigned int k = 0; k < nco; ++k) {
        const xClusterInformation c = xci[k];
        if (i >= c.scid && i < c.scid + c.count) { scl = c.scid; neach = c.neach; return; }
        seach += c.neach;
        sbegin += c.count * c.neach;
    }
}

__global__ void k_vv_cluster_position(device_dem_parameters p, double* pos, double* cpos, double* ep,
                                      const double* rloc, const double* vel, const double* acc, const double* ev,
                                      const double* ea, const xClusterInformation* xci, unsigned int ns)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ns) return;
    unsigned int neach, seach, sbegin, scl;
    cluster_slot(xci, p.nClusterObject, id, neach, seach, sbegin, scl);
    const double dt = p.dt, h = p.half2dt;
    const d4 cp = ld4(cpos, id);
    const d3 npos = (mk3(cp.x, cp.y, cp.z) + dt * ld3(vel, id)) + h * ld3(acc, id);
    st4(cpos, id, mk4(npos.x, npos.y, npos.z, cp.w));
    d4 e = (ld4(ep, id) + dt * ld4(ev, id)) + h * ld4(ea, id);
    const double l = sqrt(dot(e, e));
    e = mk4(e.x / l, e.y / l, e.z / l, e.w / l);
    st4(ep, id, e);
    const unsigned int sid = sbegin + (id - scl) * neach;
    for (unsigned int j = 0; j < neach; ++j) {
        const d3 m = npos + to_global(ld3(rloc, seach + j), e);
        double* q = pos + 4 * (size_t)(sid + j);
        q[0] = m.x; q[1] = m.y; q[2] = m.z;
    }
}

__global__ void k_vv_cluster_velocity(device_dem_parameters p, double* vel, double* acc, const double* ep,
                                      double* ev, double* ea, double* force, double* moment, const double* mass,
                                      const double* iner, const xClusterInformation* xci, unsigned int ns)
{
    const unsigned int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ns) return;
    unsigned int neach, seach, sbegin, scl;
    cluster_slot(xci, p.nClusterObject, id, neach, seach, sbegin, scl);
    const double hdt = 0.5 * p.dt;
    const double m = mass[id];
    d3 v = ld3(vel, id), a = ld3(acc, id);
    d4 av = ld4(ev, id);
    const d4 aa0 = ld4(ea, id), e = ld4(ep, id);
    const double inv_m = 1.0 / m;
    d3 F = mk3(0, 0, 0), T = mk3(0, 0, 0);
    const unsigned int sid = sbegin + (id - scl) * neach;
    for (unsigned int j = 0; j < neach; ++j) {
        F = F + ld3(force, sid + j);
        T = T + ld3(moment, sid + j);
        st3(force, sid + j, mk3(0, 0, 0));
        st3(moment, sid + j, mk3(0, 0, 0));
    }
    F = F + m * dv3(p.gravity);
    const d4 q = uceom(ld3(iner, id), e, av, to_local(T, e));
    v = v + hdt * a;
    av = av + hdt * aa0;
    a = inv_m * F;
    st3(vel, id, v + hdt * a);
    st4(ev, id, av + hdt * q);
    st3(acc, id, a);
    st4(ea, id, q);
}

// ---------------------------------------------------------------- material constants
__global__ void k_make_mat_pair(const device_contact_property* cp, int model, int swap, mat_pair* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *out = make_mat_pair(*cp, model, swap != 0);
}

// ---------------------------------------------------------------- reductions
__global__ void k_reduce_partial(const double* in, unsigned int n, double* out)
{
    __shared__ double sm[32];
    double s = 0.0;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += in[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) out[blockIdx.x] = s;
    }
}

__global__ void k_sum_block_partials(const double* part, unsigned int nb, double* out6)
{
    __shared__ double sm[6][32];
    const int c = threadIdx.y;  // 6 rows of 32 threads
    double s = 0.0;
    for (unsigned int b = threadIdx.x; b < nb; b += 32) s += part[b * 6 + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) sm[c][0] = s;
    __syncthreads();
    if (threadIdx.x == 0) out6[c] = sm[c][0];
}

// ================================================================ launch wrappers
#define XDEM_LAUNCH(kernel, n, ...)                                                   \
    do {                                                                              \
        if ((n) == 0) return cudaSuccess;                                             \
        kernel<<<blocks_for(n), kThreads, 0, st>>>(__VA_ARGS__);                      \
        return cudaGetLastError();                                                    \
    } while (0)

cudaError_t launch_vv_position(const device_dem_parameters& p, double* pos, double* ep, const double* vel,
                               const double* ev, const double* acc, const double* ea, unsigned int n,
                               cudaStream_t st)
{
    XDEM_LAUNCH(k_vv_position, n, p, pos, ep, vel, ev, acc, ea, n);
}

cudaError_t launch_vv_velocity(const device_dem_parameters& p, double* vel, double* acc, const double* ep,
                               double* ev, double* ea, double* force, double* moment, const double* mass,
                               const double* iner, unsigned int n, int compat, cudaStream_t st)
{
    XDEM_LAUNCH(k_vv_velocity, n, p, vel, acc, ep, ev, ea, force, moment, mass, iner, n, compat);
}

cudaError_t launch_hash(const device_dem_parameters& p, unsigned int* hash, unsigned int* index, const double* pos,
                        unsigned int sid, unsigned int n, unsigned int* status, cudaStream_t st)
{
    XDEM_LAUNCH(k_hash, n, p, hash, index, pos, sid, n, status);
}

cudaError_t launch_cell_bounds(const unsigned int* skey, const unsigned int* sval, unsigned int* cstart,
                               unsigned int* cend, unsigned int* sorted_index, unsigned int n, cudaStream_t st)
{
    XDEM_LAUNCH(k_cell_bounds, n, skey, sval, cstart, cend, sorted_index, n);
}

cudaError_t launch_clear_cells(const unsigned int* keys, unsigned int n, unsigned int* cstart, unsigned int* cend,
                               cudaStream_t st, const unsigned int* gate)
{
    XDEM_LAUNCH(k_clear_cells, n, keys, n, cstart, cend, gate);
}

cudaError_t launch_fill_u32(unsigned int* a, unsigned int v, size_t n, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const unsigned int nb = (unsigned int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
    k_fill_u32<<<nb, 256, 0, st>>>(a, v, n);
    return cudaGetLastError();
}

cudaError_t launch_p2p(const device_dem_parameters& p, const double* pos, const double* ep, const double* vel,
                       const double* ev, double* force, double* moment, const double* mass, double* tmax,
                       double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                       const unsigned int* sorted_index, const unsigned int* cstart, const unsigned int* cend,
                       const mat_pair* mp, unsigned int n, unsigned int* status, cudaStream_t st)
{
    XDEM_LAUNCH(k_p2p, n, p, pos, ep, vel, ev, force, moment, mass, tmax, rres, pair_count, pair_id, tsd,
                sorted_index, cstart, cend, mp, n, status);
}

cudaError_t launch_plane(const device_dem_parameters& p, const device_plane_info* plane, const double* dbi,
                         const mat_pair* mp, const BodyPartials& bp, const double* pos,
                         const double* ep, const double* vel, const double* ev, double* force, double* moment,
                         const double* mass, double* tmax, double* rres, unsigned int* pair_count,
                         unsigned int* pair_id, double* tsd, unsigned int n, unsigned int* status, cudaStream_t st)
{
    XDEM_LAUNCH(k_plane<false>, n, p, plane, dbi, mp, bp, pos, nullptr, ep, vel, ev, force, moment, mass, tmax,
                rres, pair_count, pair_id, tsd, nullptr, n, status);
}

cudaError_t launch_cluster_plane(const device_dem_parameters& p, const device_plane_info* plane, const double* dbi,
                                 const mat_pair* mp, const BodyPartials& bp, const double* pos,
                                 const double* cpos, const double* ep, const double* vel, const double* ev,
                                 double* force, double* moment, const double* mass, double* tmax, double* rres,
                                 unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                 const xClusterInformation* xci, unsigned int n, unsigned int* status,
                                 cudaStream_t st)
{
    XDEM_LAUNCH(k_plane<true>, n, p, plane, dbi, mp, bp, pos, cpos, ep, vel, ev, force, moment, mass, tmax, rres,
                pair_count, pair_id, tsd, xci, n, status);
}

cudaError_t launch_cylinder(const device_dem_parameters& p, const device_cylinder_info* cyl, const double* bi,
                            const mat_pair* mp, const BodyPartials& bp, const double* pos, const double* cpos,
                            const double* ep, const double* vel, const double* ev, double* force, double* moment,
                            const double* mass, double* tmax, double* rres, unsigned int* pair_count,
                            unsigned int* pair_id, double* tsd, const xClusterInformation* xci, unsigned int n,
                            unsigned int* status, cudaStream_t st)
{
    if (cpos)
        XDEM_LAUNCH(k_cylinder<true>, n, p, cyl, bi, mp, bp, pos, cpos, ep, vel, ev, force, moment, mass, tmax,
                    rres, pair_count, pair_id, tsd, xci, n, status);
    XDEM_LAUNCH(k_cylinder<false>, n, p, cyl, bi, mp, bp, pos, nullptr, ep, vel, ev, force, moment, mass, tmax,
                rres, pair_count, pair_id, tsd, nullptr, n, status);
}

cudaError_t launch_mesh(const device_dem_parameters& p, const device_triangle_info* dti, unsigned int lo_base,
                        int lo_field, const double* dbi, const mat_pair* mp, const BodyPartials& bp,
                        const double* pos, const double* cpos, const double* ep, const double* vel,
                        const double* ev, double* force, double* moment, const double* mass, double* tmax,
                        double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                        const unsigned int* sorted_index, const unsigned int* cstart, const unsigned int* cend,
                        const xClusterInformation* xci, unsigned int n, unsigned int ntri, unsigned int* status,
                        cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (cpos)
        k_mesh<true><<<blocks_for(n), kThreads, 0, st>>>(p, dti, lo_base, lo_field, dbi, mp, bp, pos, cpos, ep, vel, ev, force,
                                                         moment, mass, tmax, rres, pair_count, pair_id, tsd,
                                                         sorted_index, cstart, cend, xci, n, ntri, status);
    else
        k_mesh<false><<<blocks_for(n), kThreads, 0, st>>>(p, dti, lo_base, lo_field, dbi, mp, bp, pos, nullptr, ep, vel, ev, force,
                                                          moment, mass, tmax, rres, pair_count, pair_id, tsd,
                                                          sorted_index, cstart, cend, nullptr, n, ntri, status);
    return cudaGetLastError();
}

cudaError_t launch_rolling(const device_dem_parameters& p, double* tmax, double* rres, const double* inertia,
                           const double* ep, const double* ev, double* moment, unsigned int n, cudaStream_t st,
                           int per_sphere)
{
    XDEM_LAUNCH(k_rolling, n, p, tmax, rres, inertia, ep, ev, moment, n, per_sphere);
}

cudaError_t launch_cluster_rolling(const device_dem_parameters& p, double* tmax, double* rres, const double* inertia,
                                   const double* ep, const double* ev, double* moment,
                                   const xClusterInformation* xci, unsigned int n, cudaStream_t st)
{
    XDEM_LAUNCH(k_cluster_rolling, n, p, tmax, rres, inertia, ep, ev, moment, xci, n);
}

cudaError_t launch_update_mesh(const double* dbi, const double* vlist, double* sphere, const double* dlocal,
                               device_triangle_info* dpi, unsigned int ntri, cudaStream_t st)
{
    XDEM_LAUNCH(k_update_mesh, ntri, dbi, vlist, sphere, dlocal, dpi, ntri);
}

cudaError_t launch_clusters_p2p(const device_dem_parameters& p, const double* pos, const double* cpos,
                                const double* ep, const double* vel, const double* ev, double* force,
                                double* moment, const double* mass, double* tmax, double* rres,
                                unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                const unsigned int* sorted_index, const unsigned int* cstart,
                                const unsigned int* cend, const mat_pair* mp,
                                const xClusterInformation* xci, unsigned int n, unsigned int* status,
                                cudaStream_t st)
{
    XDEM_LAUNCH(k_clusters_p2p, n, p, pos, cpos, ep, vel, ev, force, moment, mass, tmax, rres, pair_count, pair_id,
                tsd, sorted_index, cstart, cend, mp, xci, n, status);
}

cudaError_t launch_vv_cluster_position(const device_dem_parameters& p, double* pos, double* cpos, double* ep,
                                       const double* rloc, const double* vel, const double* acc, const double* ev,
                                       const double* ea, const xClusterInformation* xci, unsigned int ns,
                                       cudaStream_t st)
{
    XDEM_LAUNCH(k_vv_cluster_position, ns, p, pos, cpos, ep, rloc, vel, acc, ev, ea, xci, ns);
}

cudaError_t launch_vv_cluster_velocity(const device_dem_parameters& p, double* vel, double* acc, const double* ep,
                                       double* ev, double* ea, double* force, double* moment, const double* mass,
                                       const double* iner, const xClusterInformation* xci, unsigned int ns,
                                       cudaStream_t st)
{
    XDEM_LAUNCH(k_vv_cluster_velocity, ns, p, vel, acc, ep, ev, ea, force, moment, mass, iner, xci, ns);
}

cudaError_t launch_make_mat_pair(const device_contact_property* cp, int model, int swap_fric, mat_pair* out,
                                 cudaStream_t st)
{
    k_make_mat_pair<<<1, 32, 0, st>>>(cp, model, swap_fric, out);
    return cudaGetLastError();
}

size_t reduce_tmp_size(unsigned int n)
{
    (void)n;
    return 1024;
}

cudaError_t launch_reduce_sum(const double* in, unsigned int n, double* tmp, double* out, cudaStream_t st)
{
    unsigned int nb = (n + 255) / 256;
    if (nb > 1024) nb = 1024;
    if (nb == 0) nb = 1;
    k_reduce_partial<<<nb, 256, 0, st>>>(in, n, tmp);
    k_reduce_partial<<<1, 1024, 0, st>>>(tmp, nb, out);
    return cudaGetLastError();
}

cudaError_t launch_sum_block_partials(const double* partials, unsigned int nblocks, double* out6, cudaStream_t st)
{
    k_sum_block_partials<<<1, dim3(32, 6), 0, st>>>(partials, nblocks, out6);
    return cudaGetLastError();
}

}  // namespace xdem

namespace xdem {
size_t mat_pair_size() { return sizeof(mat_pair); }
}  // namespace xdem
