// xdem_fused.cuh -- the fused contact + integration kernel of the plain FP64
// form, and the contact-model helpers it shares with the mixed form
// (xdem_fused_mixed.cu), which are generic in the arithmetic type R of the
// contact geometry and forces.
//
// One thread per cell-sorted entry.  Neighbours are read from the sorted
// snapshot (coalesced along a cell, cached across the 27-cell stencil); an
// FP32 prefilter on the snapshot's centre-relative float4 positions rejects
// far candidates before the FP64 distance test, which follows the reference's
// arithmetic (impl:676-679) exactly.  Contact physics restates impl:362-483
// (constants, Hertz-Mindlin / DHS, rolling), impl:735-1080 (planes) and
// impl:1655-2109 (triangle meshes); the per-particle tail restates
// impl:2420-2454 (rolling), impl:192-222 (velocity) and impl:135-147 +
// 290-302 (next position and its cell hash).
#pragma once

#include "xdem_device.cuh"
#include "xdem_fused.h"

namespace xdem {

template <class R>
struct V3 { R x, y, z; };
template <class R> __device__ __forceinline__ V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return v3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return v3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a) { return v3<R>(-a.x, -a.y, -a.z); }
template <class R> __device__ __forceinline__ V3<R> operator*(R s, V3<R> a) { return v3<R>(s * a.x, s * a.y, s * a.z); }
template <class R> __device__ __forceinline__ V3<R> operator/(V3<R> a, R s) { return v3<R>(a.x / s, a.y / s, a.z / s); }
template <class R> __device__ __forceinline__ R tdot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> __device__ __forceinline__ R tlen(V3<R> a) { return sqrt(tdot(a, a)); }
template <class R> __device__ __forceinline__ V3<R> tcross(V3<R> a, V3<R> b)
{
    return v3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> __device__ __forceinline__ V3<R> cvt(d3 a) { return v3<R>((R)a.x, (R)a.y, (R)a.z); }
template <class R> __device__ __forceinline__ d3 cvt_back(V3<R> a) { return mk3((double)a.x, (double)a.y, (double)a.z); }

// Material constants in the contact arithmetic type.
template <class R>
struct MatR {
    R Eeq, Seq8, beta, vs1, sratio, fric, rfric;
    bool coh;
};
template <class R>
__device__ __forceinline__ MatR<R> mat_r(const mat_pair& m)
{
    return MatR<R>{(R)m.Eeq, (R)m.Seq8, (R)m.beta, (R)m.vs1, (R)m.sratio, (R)m.fric, (R)m.rfric, m.coh != 0.0};
}

template <class R>
struct FC { R kn, vn, ks, vs, mu, eq_r, eq_m; };

template <class R>
__device__ __forceinline__ FC<R> fconst_r(const MatR<R>& m, int model, R ir, R jr, R im, R jm)
{
    FC<R> c;
    c.eq_m = jm != R(0) ? (im * jm) / (im + jm) : im;
    c.eq_r = jr != R(0) ? (ir * jr) / (ir + jr) : ir;
    c.kn = (R(4.0) / R(3.0)) * m.Eeq * sqrt(c.eq_r);
    c.vn = m.beta;
    c.ks = model == 1 ? m.Seq8 : c.kn * m.sratio;
    c.vs = m.vs1;
    c.mu = m.fric;
    return c;
}

// impl:432-474 in type R; the tangential history (ds, previous s_dot) stays
// FP64.  Cohesion is handled by the caller (FP64 path only).
template <class R>
__device__ __forceinline__ void model_r(int model, const FC<R>& c, double dt, R cdist, double& ds_io,
                                        double& dots_io, V3<R> dv, V3<R> unit, V3<R>& Ft, V3<R>& Fn, R fca)
{
    const R fsn = -c.kn * (cdist * sqrt(cdist));
    const R fdn = c.vn * tdot(dv, unit);
    Fn = (fsn + fca + fdn) * unit;
    const V3<R> e = dv - tdot(dv, unit) * unit;
    const R mag_e = tlen(e);
    if (mag_e != R(0)) {
        const V3<R> s_hat = e / mag_e;
        const R s_dot = tdot(dv, s_hat);
        const double ds = ds_io + dt * ((double)s_dot + dots_io);
        ds_io = ds;
        dots_io = (double)s_dot;
        R a;
        if (model == 1) {
            const R S_t = c.ks * sqrt(c.eq_r * cdist);
            a = S_t * (R)ds + c.vs * sqrt(S_t * c.eq_m);
        } else {
            a = c.ks * (R)ds + c.vs * tdot(dv, s_hat);
        }
        const R b = c.mu * tlen(Fn);
        Ft = (a < b ? a : b) * s_hat;
    }
}

__device__ __forceinline__ void block_sum6_f(double v[6], double* sm)
{
#pragma unroll
    for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int c = 0; c < 6; ++c) sm[c * 32 + warp] = v[c];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        for (int c = 0; c < 6; ++c) {
            double x = lane < nw ? sm[c * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[c] = x;
        }
    }
    __syncthreads();
}

// Block-sums six per-thread values into out[0..5]; skips the reduction when
// no thread of the block contributed.
__device__ __forceinline__ void emit_body(double f6[6], bool any, double* out, double* sm)
{
    if (!__syncthreads_or(any ? 1 : 0)) {
        if (threadIdx.x == 0)
            for (int c = 0; c < 6; ++c) out[c] = 0.0;
        return;
    }
    block_sum6_f(f6, sm);
    if (threadIdx.x == 0)
        for (int c = 0; c < 6; ++c) out[c] = f6[c];
}

template <class R, bool MESH>
__global__ void __launch_bounds__(kFusedThreads, 1)
k_fused_contact(const ContactLaunch c)
{
    __shared__ double sm[6 * 32];
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int oid = 0xffffffffu;
    if (s < c.nentry) oid = c.sorted_index[s];
    const bool live = oid < c.np;
    const device_dem_parameters& p = c.prm;
    const int model = p.contact_model;
    const double dt = p.dt;

    d4 ip = mk4(0, 0, 0, 0), iv = mk4(0, 0, 0, 0), io = mk4(0, 0, 0, 0);
    float4 ipf = make_float4(0.f, 0.f, 0.f, -1.f);
    unsigned int gx = 0, gy = 0, gz = 0;
    if (live) {
        ip = ld4(c.snap_pos, s);
        iv = ld4(c.snap_vel, s);
        io = ld4(c.snap_om, s);
        ipf = reinterpret_cast<const float4*>(c.snap_f)[s];
        // own cell from the sorted key: (z * gy + y) * gx + x with power-of-two
        // extents; neighbour hashes only need the wrapped coordinates
        const unsigned int key = c.skey[s];
        const unsigned int shx = __ffs(p.grid_size.x) - 1, shxy = shx + __ffs(p.grid_size.y) - 1;
        gx = key & (p.grid_size.x - 1);
        gy = (key >> shx) & (p.grid_size.y - 1);
        gz = key >> shxy;
    }
    const d3 ipos = mk3(ip.x, ip.y, ip.z);
    const double ir = ip.w, im = iv.w;
    const V3<R> ivel = cvt<R>(mk3(iv.x, iv.y, iv.z));
    const V3<R> iom = cvt<R>(mk3(io.x, io.y, io.z));
    d3 F = mk3(0, 0, 0), M = mk3(0, 0, 0), tma = mk3(0, 0, 0);
    double res = 0.0;
    unsigned int bits = 0;
    const unsigned int scene = live ? scene_index(c, oid) : 0u;

    // ------------------------------------------------ particle-particle (impl:613-733)
    if (live && c.has_pp) {
        const mat_pair mp = c.mp[scene];
        const MatR<R> mr = mat_r<R>(mp);
        const unsigned int sid = oid * MAX_P2P_COUNT;
        unsigned int old_count = c.pp_count_old[oid];
        if (old_count > MAX_P2P_COUNT) old_count = MAX_P2P_COUNT;
        V3<R> Ft = v3<R>(0, 0, 0), Fn = v3<R>(0, 0, 0);
        d3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0);
        unsigned int cnt = 0;
        const float rr_i = ipf.w;
        const bool filt = !mp.coh;
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    const unsigned int h = grid_hash(p, (int)gx + x, (int)gy + y, (int)gz + z);
                    const unsigned int start = c.cstart[h];
                    if (start == 0xffffffffu) continue;
                    const unsigned int end = c.cend[h];
                    for (unsigned int j = start; j < end; ++j) {
                        const unsigned int k = c.sorted_index[j];
                        if (k == oid || k >= c.np) continue;
                        if (c.scene_of && c.scene_of[k] != scene) continue;  // another scene of the batch
                        if (filt) {
                            const float4 jf = reinterpret_cast<const float4*>(c.snap_f)[j];
                            if (rr_i >= 0.f && jf.w >= 0.f) {
                                const float dx = jf.x - ipf.x, dy = jf.y - ipf.y, dz = jf.z - ipf.z;
                                const float lim = rr_i + jf.w + c.margin;
                                if (dx * dx + dy * dy + dz * dz > lim * lim) continue;
                            }
                        }
                        const d4 jp = ld4(c.snap_pos, j);
                        const double jr = jp.w;
                        const d3 rpd = mk3(jp.x - ip.x, jp.y - ip.y, jp.z - ip.z);
                        double cdist;
                        V3<R> rp;
                        R dist;
                        if (sizeof(R) == sizeof(double)) {
                            const double dd = length(rpd);
                            cdist = (ir + jr) - dd;
                            rp = cvt<R>(rpd);
                            dist = (R)dd;
                        } else {
                            rp = cvt<R>(rpd);
                            dist = tlen(rp);
                            cdist = (double)(((R)ir + (R)jr) - dist);
                        }
                        double cs = 0.0;
                        if (mp.coh) cs = limit_cohesion_depth(mp, ir, jr);
                        if (cdist > 0) {
                            double sd0 = 0.0, sd1 = 0.0;
                            for (unsigned int q = 0; q < old_count; ++q)
                                if (c.pp_id_old[sid + q] == k) {
                                    const double2 t = reinterpret_cast<const double2*>(c.pp_tsd_old)[sid + q];
                                    sd0 = t.x; sd1 = t.y;
                                    break;
                                }
                            const d4 jv = ld4(c.snap_vel, j);
                            const d4 jo = ld4(c.snap_om, j);
                            const V3<R> unit = rp / dist;
                            const R rir = (R)ir;
                            const V3<R> cpt = cvt<R>(ipos) + rir * unit;
                            const V3<R> dcpr = sizeof(R) == sizeof(double) ? cpt - cvt<R>(ipos) : rir * unit;
                            const V3<R> dcpr_j = sizeof(R) == sizeof(double) ? cpt - cvt<R>(mk3(jp.x, jp.y, jp.z))
                                                                             : rir * unit - rp;
                            const V3<R> jvel = cvt<R>(mk3(jv.x, jv.y, jv.z));
                            const V3<R> jom = cvt<R>(mk3(jo.x, jo.y, jo.z));
                            const V3<R> rv = (jvel + tcross(jom, dcpr_j)) - (ivel + tcross(iom, dcpr));
                            const FC<R> fc = fconst_r<R>(mr, model, rir, (R)jr, (R)im, (R)jv.w);
                            R fca = R(0);
                            if (mp.coh) {
                                const double fsn = -(double)fc.kn * (cdist * sqrt(cdist));
                                const double fdn = (double)fc.vn * (double)tdot(rv, unit);
                                fca = (R)(-cohesion_force(mp, ir, jr, fsn + fdn));
                            }
                            model_r<R>(model, fc, dt, (R)cdist, sd0, sd1, rv, unit, Ft, Fn, fca);
                            const V3<R> fsum = Fn + Ft;
                            if (c.rolling) {
                                tma = tma + cvt_back<R>(tcross(dcpr, fsum));
                                const R Rij = jr ? rir * (R)jr / (rir + (R)jr) : rir;
                                res += (double)(Rij * mr.rfric * tlen(Fn));
                            }
                            sumF = sumF + cvt_back<R>(fsum);
                            sumM = sumM + cvt_back<R>(tcross(dcpr, fsum));
                            if (cnt < MAX_P2P_COUNT) {
                                c.pp_id_new[sid + cnt] = k;
                                reinterpret_cast<double2*>(c.pp_tsd_new)[sid + cnt] = make_double2(sd0, sd1);
                                cnt++;
                            } else {
                                bits |= XDEM_ERR_P2P_OVERFLOW;
                            }
                        } else if (cdist <= 0 && fabs(cdist) < fabs(cs)) {
                            const d3 unit = rpd / length(rpd);
                            const double f = jkr_separation_force(mp, ir, jr);
                            const double cf = cohesion_force(mp, ir, jr, f);
                            sumF = sumF - cf * unit;
                            if (cnt < MAX_P2P_COUNT) {
                                c.pp_id_new[sid + cnt] = k;
                                reinterpret_cast<double2*>(c.pp_tsd_new)[sid + cnt] = make_double2(0.0, 0.0);
                                cnt++;
                            } else {
                                bits |= XDEM_ERR_P2P_OVERFLOW;
                            }
                        }
                    }
                }
        c.pp_count_new[oid] = cnt;
        F = F + sumF;
        M = M + sumM;
    }

    // ------------------------------------------------ planes in id order (impl:950-1080)
    if (c.nplane) {
        unsigned int sl_id[MAX_P2PL_COUNT];
        double sl_a[MAX_P2PL_COUNT], sl_b[MAX_P2PL_COUNT];
        unsigned int cnt = 0;
        const unsigned int sid = live ? oid * MAX_P2PL_COUNT : 0;
        if (live) {
#pragma unroll
            for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q) {
                sl_id[q] = c.pl_id[sid + q];
                const double2 t = reinterpret_cast<const double2*>(c.pl_tsd)[sid + q];
                sl_a[q] = t.x; sl_b[q] = t.y;
            }
        }
        // a batched scene sees only its own planes and keeps no wrenches (no
        // block reduction, so threads may walk different plane ranges)
        const bool batched = c.scene_plane_first != nullptr;
        const unsigned int kbeg = batched ? c.scene_plane_first[scene] : 0u;
        const unsigned int kend = batched ? (live ? c.scene_plane_first[scene + 1] : kbeg) : c.nplane;
        for (unsigned int k = kbeg; k < kend; ++k) {
            double f6[6] = {0, 0, 0, 0, 0, 0};
            bool touched = false;
            // Conservative FP32 test: every region of the plane test (corner,
            // edge, face; impl:735-815) needs the centre within r of the
            // plane and of the rectangle's extent, up to the cohesion range.
            bool near = true;
            if (live && ipf.w >= 0.f && c.mp[c.nscene + k].coh == 0.0) {
                const PlaneF pf = c.planef[k];
                const float dx = ipf.x - pf.v[0], dy = ipf.y - pf.v[1], dz = ipf.z - pf.v[2];
                const float wx = dx * pf.v[3] + dy * pf.v[4] + dz * pf.v[5];
                const float wy = dx * pf.v[6] + dy * pf.v[7] + dz * pf.v[8];
                const float wz = dx * pf.v[9] + dy * pf.v[10] + dz * pf.v[11];
                const float lim = ipf.w + c.margin;
                near = fabsf(wz) <= lim && wx >= -lim && wx <= pf.v[12] + lim && wy >= -lim && wy <= pf.v[13] + lim;
            }
            if (live && near) {
                const device_plane_info& pl = c.planes[k];
                const unsigned int pid = pl.id;
                const mat_pair mp = c.mp[c.nscene + k];
                const MatR<R> mr = mat_r<R>(mp);
                const body_state b = load_body(c.body + 15 * k);
                if (k == kbeg) cnt = 0;  // the scene's first plane restarts the list (impl:989)
                const d3 dp = ipos - dv3(pl.xw);
                d3 unit = mk3(0, 0, 0);
                const d3 wp = mk3(dot(dp, dv3(pl.u1)), dot(dp, dv3(pl.u2)), dot(dp, dv3(pl.uw)));
                const double cdist = plane_detection(pl, ipos, wp, unit, ir);
                double cs = 0.0;
                if (mp.coh) cs = limit_cohesion_depth(mp, ir, 0.0);
                if (cdist > 0 || (cdist <= 0 && fabs(cdist) < fabs(cs))) {
                    double sd0 = 0.0, sd1 = 0.0;
                    const d3 cpt = ipos + ir * unit;
                    const d3 dcpr_j = cpt - b.p;
                    d3 mf;
                    if (cdist > 0) {
                        for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q)
                            if (sl_id[q] == pid) { sd0 = sl_a[q]; sd1 = sl_b[q]; break; }
                        const V3<R> dcpr = cvt<R>(cpt - ipos);
                        const V3<R> dv = cvt<R>(b.v + cross(b.om, dcpr_j)) - (ivel + tcross(iom, dcpr));
                        const FC<R> fc = fconst_r<R>(mr, model, (R)ir, R(0), (R)im, R(0));
                        R fca = R(0);
                        const V3<R> un = cvt<R>(unit);
                        if (mp.coh) {
                            const double fsn = -(double)fc.kn * (cdist * sqrt(cdist));
                            const double fdn = (double)fc.vn * (double)tdot(dv, un);
                            fca = (R)(-cohesion_force(mp, ir, 0.0, fsn + fdn));
                        }
                        V3<R> Ft = v3<R>(0, 0, 0), Fn = v3<R>(0, 0, 0);
                        model_r<R>(model, fc, dt, (R)cdist, sd0, sd1, dv, un, Ft, Fn, fca);
                        const V3<R> fsum = Fn + Ft;
                        if (c.rolling) {
                            tma = tma + cvt_back<R>(tcross(dcpr, fsum));
                            res += (double)((R)ir * mr.rfric * tlen(Fn));
                        }
                        mf = cvt_back<R>(fsum);
                        F = F + (mk3(0, 0, 0) + mf);
                        M = M + (mk3(0, 0, 0) + cvt_back<R>(tcross(dcpr, fsum)));
                    } else {
                        const double f = jkr_separation_force(mp, ir, 0.0);
                        const double cf = cohesion_force(mp, ir, 0.0, f);
                        mf = (-cf) * unit;
                        F = F + mf;
                    }
                    f6[0] = -mf.x; f6[1] = -mf.y; f6[2] = -mf.z;
                    const d3 bm = -cross(dcpr_j, mf);
                    f6[3] = bm.x; f6[4] = bm.y; f6[5] = bm.z;
                    touched = true;
                    if (cnt < MAX_P2PL_COUNT) {
                        c.pl_id[sid + cnt] = pid;
                        reinterpret_cast<double2*>(c.pl_tsd)[sid + cnt] = make_double2(sd0, sd1);
                        // the next plane launch of the reference re-reads these slots
#pragma unroll
                        for (int q = 0; q < (int)MAX_P2PL_COUNT; ++q)
                            if ((unsigned int)q == cnt) { sl_id[q] = pid; sl_a[q] = sd0; sl_b[q] = sd1; }
                        cnt++;
                    } else {
                        bits |= XDEM_ERR_P2PL_OVERFLOW;
                    }
                }
            }
            if (!batched) emit_body(f6, touched, c.bsums + ((size_t)k * c.nblocks + blockIdx.x) * 6, sm);
        }
        if (live) c.pl_count[oid] = cnt;
    }

    // ------------------------------------------------ triangle meshes (impl:1930-2109)
    if (MESH) {
        for (unsigned int m = 0; m < c.nmesh; ++m) {
            double f6[6] = {0, 0, 0, 0, 0, 0};
            bool touched = false;
            if (live) {
                const unsigned int lo = c.np + c.mesh_first[m], ntri = c.mesh_ntri[m];
                const int bidx = c.mesh_body[m];
                const mat_pair mp = c.mp[c.nscene + bidx];
                const MatR<R> mr = mat_r<R>(mp);
                const unsigned int sid = oid * MAX_P2MS_COUNT;
                unsigned int o_id[MAX_P2MS_COUNT];
                double o_a[MAX_P2MS_COUNT], o_b[MAX_P2MS_COUNT];
#pragma unroll
                for (int q = 0; q < (int)MAX_P2MS_COUNT; ++q) {
                    o_id[q] = c.ms_id[sid + q];
                    const double2 t = reinterpret_cast<const double2*>(c.ms_tsd)[sid + q];
                    o_a[q] = t.x; o_b[q] = t.y;
                }
                struct Hit { unsigned int id; d3 cpt; };
                Hit hf[XDEM_MAX_TRI_CANDIDATES], hl[XDEM_MAX_TRI_CANDIDATES], hp[XDEM_MAX_TRI_CANDIDATES];
                unsigned int nf = 0, nl = 0, npt = 0;
                d3 prev_line = mk3(0, 0, 0), prev_point = mk3(0, 0, 0);
                double cs = 0.0;
                if (mp.coh) cs = limit_cohesion_depth(mp, ir, 0.0);
                for (int z = -1; z <= 1; ++z)
                    for (int y = -1; y <= 1; ++y)
                        for (int x = -1; x <= 1; ++x) {
                            const unsigned int h = grid_hash(p, (int)gx + x, (int)gy + y, (int)gz + z);
                            const unsigned int start = c.cstart[h];
                            if (start == 0xffffffffu) continue;
                            const unsigned int end = c.cend[h];
                            for (unsigned int j = start; j < end; ++j) {
                                unsigned int tk = c.sorted_index[j];
                                if (!(tk >= lo && tk < lo + ntri)) continue;
                                tk -= lo;
                                int t = -1;
                                const d3 cpt = closest_pt_triangle(c.tri[c.mesh_first[m] + tk], ipos, t);
                                const double cd = ir - length(ipos - cpt);
                                bool take = false;
                                if (cd > 0) {
                                    if (t == 1) {
                                        if (check_overlap(prev_line, cpt)) continue;
                                        prev_line = cpt;
                                    } else if (t == 0) {
                                        if (check_overlap(prev_point, cpt)) continue;
                                        prev_point = cpt;
                                    }
                                    take = true;
                                } else if (cd <= 0 && fabs(cd) < fabs(cs)) {
                                    take = true;
                                }
                                if (!take) continue;
                                const Hit hit{tk, cpt};
                                if (t == 2) { if (nf < XDEM_MAX_TRI_CANDIDATES) hf[nf++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                                else if (t == 1) { if (nl < XDEM_MAX_TRI_CANDIDATES) hl[nl++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                                else if (t == 0) { if (npt < XDEM_MAX_TRI_CANDIDATES) hp[npt++] = hit; else bits |= XDEM_ERR_TRI_CANDIDATES; }
                            }
                        }
                const Hit* list = nf ? hf : (nl ? hl : hp);
                const unsigned int nlist = nf ? nf : (nl ? nl : npt);
                const body_state b = load_body(c.body + 15 * bidx);
                d3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0);
                unsigned int cnt = 0;
                for (unsigned int q = 0; q < nlist; ++q) {
                    const Hit hit = list[q];
                    double sd0 = 0.0, sd1 = 0.0;
                    const d3 po2cp = hit.cpt - b.p;
                    const d3 rpd = hit.cpt - ipos;
                    const double dist = length(rpd);
                    const d3 unit = rpd / dist;
                    const double cd = ir - dist;
                    if (cd <= 0 && fabs(cd) < fabs(cs)) {
                        const double f = jkr_separation_force(mp, ir, 0.0);
                        const double cf = cohesion_force(mp, ir, 0.0, f);
                        sumF = sumF - cf * unit;
                    } else {
                        for (int r = 0; r < (int)MAX_P2MS_COUNT; ++r)
                            if (o_id[r] == hit.id) { sd0 = o_a[r]; sd1 = o_b[r]; break; }
                        const V3<R> rc = cvt<R>(rpd);
                        const V3<R> dv = cvt<R>(b.v + cross(b.om, po2cp)) - (ivel + tcross(iom, rc));
                        const FC<R> fc = fconst_r<R>(mr, model, (R)ir, R(0), (R)im, (R)b.m);
                        const V3<R> un = cvt<R>(unit);
                        R fca = R(0);
                        if (mp.coh) {
                            const double fsn = -(double)fc.kn * (cd * sqrt(cd));
                            const double fdn = (double)fc.vn * (double)tdot(dv, un);
                            fca = (R)(-cohesion_force(mp, ir, 0.0, fsn + fdn));
                        }
                        V3<R> Ft = v3<R>(0, 0, 0), Fn = v3<R>(0, 0, 0);
                        model_r<R>(model, fc, dt, (R)cd, sd0, sd1, dv, un, Ft, Fn, fca);
                        const V3<R> fsum = Fn + Ft;
                        tma = tma + cvt_back<R>(tcross(rc, fsum));
                        res += (double)((R)ir * mr.rfric * tlen(Fn));
                        const d3 mf = cvt_back<R>(fsum);
                        sumF = sumF + mf;
                        sumM = sumM + cvt_back<R>(tcross(rc, fsum));
                        f6[0] += -mf.x; f6[1] += -mf.y; f6[2] += -mf.z;
                        const d3 mm = -cross(po2cp, mf);
                        f6[3] += mm.x; f6[4] += mm.y; f6[5] += mm.z;
                        touched = true;
                    }
                    if (cnt < MAX_P2MS_COUNT) {
                        c.ms_id[sid + cnt] = hit.id;
                        reinterpret_cast<double2*>(c.ms_tsd)[sid + cnt] = make_double2(sd0, sd1);
                        cnt++;
                    } else {
                        bits |= XDEM_ERR_P2MS_OVERFLOW;
                    }
                }
                c.ms_count[oid] = cnt;
                F = F + sumF;
                M = M + sumM;
            }
            emit_body(f6, touched, c.bsums + ((size_t)(c.mesh_body[m]) * c.nblocks + blockIdx.x) * 6, sm);
        }
    }

    if (!live) return;

    // ------------------------------------------------ rolling resistance (impl:2420-2454)
    const double Tr = res;
    if (Tr) {
        // the flat entry oid of the double3 array as impl:2434 reads it, or
        // the sphere's own (rolling_per_sphere)
        const double J = c.rolling_per_sphere ? c.inertia[3 * (size_t)oid] : c.inertia[oid];
        const d3 om = mk3(io.x, io.y, io.z);
        const d3 T = (J * p.dt) * om - tma;
        const double lT = length(T);
        if (lT && Tr) {
            d3 Tr3 = Tr * (T / lT);
            if (length(Tr3) >= lT) Tr3 = T;
            M = M + Tr3;
        }
    }

    // ------------------------------------------------ velocity update (impl:192-222)
    const double hdt = 0.5 * p.dt;
    const double inv = 1.0 / im;
    const d3 a_new = inv * (F + im * dv3(p.gravity));
    const d4 e = ld4(c.ep_cur, oid);
    d4 av = ld4(c.ev, oid);
    const d3 nb = to_local(M, e);
    const d4 q = uceom(ld3(c.inertia, oid), e, av, nb);
    av = av + hdt * (ld4(c.ea, oid) + q);
    d3 v = mk3(iv.x, iv.y, iv.z);
    if (!c.vel_compat) v = v + hdt * (ld3(c.acc, oid) + a_new);
    st3(c.vel, oid, v);
    st4(c.ev, oid, av);
    st3(c.acc, oid, a_new);
    st4(c.ea, oid, q);

    // ------------------------------------------------ next position + hash (impl:135-147, 290-302)
    const d4 e2 = (e + dt * av) + p.half2dt * q;
    const double l = sqrt(dot(e2, e2));
    st4(c.ep_next, oid, mk4(e2.x / l, e2.y / l, e2.z / l, e2.w / l));
    const d3 dpos = dt * v + p.half2dt * a_new;
    const d3 xn = mk3(ip.x + dpos.x, ip.y + dpos.y, ip.z + dpos.z);
    st4(c.pos_next, oid, mk4(xn.x, xn.y, xn.z, ip.w));
    if (!(isfinite(xn.x) && isfinite(xn.y) && isfinite(xn.z))) bits |= XDEM_ERR_NONFINITE;
    const int3v g = grid_pos(p, xn);
    c.k_out[oid] = grid_hash(p, g.x, g.y, g.z);
    c.v_out[oid] = oid;
    if (bits) atomicOr(c.status, bits);
}

template <class R>
cudaError_t launch_fused_contact_t(const ContactLaunch& c, cudaStream_t st)
{
    if (c.nentry == 0) return cudaSuccess;
    const unsigned int nb = (c.nentry + kFusedThreads - 1) / kFusedThreads;
    if (c.nmesh)
        k_fused_contact<R, true><<<nb, kFusedThreads, 0, st>>>(c);
    else
        k_fused_contact<R, false><<<nb, kFusedThreads, 0, st>>>(c);
    return cudaGetLastError();
}

}  // namespace xdem
