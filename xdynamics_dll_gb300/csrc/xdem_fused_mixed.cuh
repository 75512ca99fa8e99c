// xdem_fused_mixed.cuh -- the contact and integration kernels of the mixed
// form: contact geometry and forces in FP32, positions, velocities, Euler
// parameters and their rates kept in FP64.
//
// GB300 runs FP64 arithmetic and FP64<->FP32 conversions at about 1/64 of the
// FP32 rate, so the per-sphere FP64 work is held to the one operation that
// needs it: adding an FP32 increment to an FP64 state value (14 additions per
// sphere: velocity 3, Euler-parameter rates 4, Euler parameters 4, position
// 3).  Conversions run on the integer pipes (xdem_df.cuh); quantities that
// need more than FP32 (plane distances, the cell of the new centre, the norm
// of the Euler parameters) are formed in float pairs.  Force and torque sums
// are compensated FP32 sums (about 48 bits).  The tangential history keeps
// of particle pairs is FP32 (float2 slots in the reference's double2
// buffers); plane, mesh and cylinder histories keep FP64 storage.
//
// Physics and slot rules are those of the FP64 kernel (xdem_fused.cuh):
// impl:613-733 (particle-particle), impl:735-1080 (planes), impl:1930-2109
// (meshes; FP64 geometry here too), impl:2420-2454 (rolling), impl:192-222
// and 135-147 (velocity and position update), impl:290-302 (next hash).
//
// Two translation units instantiate these kernels with different compile
// flags: xdem_fused_mixed.cu (sphere scenes without meshes: the candidate
// list and walk kernels, the sphere body kernel; no implicit FMA
// contraction, so the list kernel's walk behind a call computes the bits of
// the walk inlined elsewhere) and xdem_fused_mixed_mesh.cu (the mesh forms of
// the pair kernels and the cluster body kernel, with contraction: their FP64
// closest-point geometry runs on GB300's slow FP64 pipe, where a fused
// multiply-add is one operation instead of two; their walks are inlined).
#pragma once
#include "xdem_df.cuh"
#include "xdem_fused.cuh"

namespace xdem {
namespace {

__device__ __forceinline__ MatR<float> matr(const MatF& m)
{
    return MatR<float>{m.Eeq, m.Seq8, m.beta, m.vs1, m.sratio, m.fric, m.rfric, m.coh != 0};
}
__device__ __forceinline__ float3 d2f3(d3 a) { return make_float3(d2f_rn(a.x), d2f_rn(a.y), d2f_rn(a.z)); }

// IEEE quotient a / b, skipping the division when a is zero (common: axis-
// aligned contacts, no moment about an axis).  Bit-identical to a / b for
// normal b; a reciprocal-multiply would not be: the unit vector of an
// axis-aligned contact must come out exactly (0, 1, 0), or the tangential
// model sees a spurious tangential velocity along the normal.
__device__ __forceinline__ float qdiv(float a, float b) { return a == 0.f ? a : a / b; }
__device__ __forceinline__ V3<float> qdiv(V3<float> a, float b)
{
    return v3<float>(qdiv(a.x, b), qdiv(a.y, b), qdiv(a.z, b));
}
// Square root and quotient at the hardware approximation (sqrt.approx.f32,
// __fdividef: relative error of a few 2^-23): for the contact constants,
// the magnitudes of the contact model and the seed of the float-pair square
// root, where an error of 1e-7 of the value is below the FP32 rounding the
// contact force carries anyway; each saves the IEEE sequence's Newton steps
// and special-case check in the per-contact loop.  The unit normal keeps
// the IEEE quotient (qdiv above).
__device__ __forceinline__ float sqrt_fast(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float div_fast(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float len_fast(V3<float> a) { return sqrt_fast(tdot(a, a)); }

// Contact constants of a pair (fconst_r of the FP64 form) with the fast
// quotient and square root.
__device__ __forceinline__ FC<float> fconst_f(const MatR<float>& m, int model, float ir, float jr, float im, float jm)
{
    FC<float> c;
    c.eq_m = jm != 0.f ? div_fast(im * jm, im + jm) : im;
    c.eq_r = jr != 0.f ? div_fast(ir * jr, ir + jr) : ir;
    c.kn = (4.f / 3.f) * m.Eeq * sqrt_fast(c.eq_r);
    c.vn = m.beta;
    c.ks = model == 1 ? m.Seq8 : c.kn * m.sratio;
    c.vs = m.vs1;
    c.mu = m.fric;
    return c;
}

__device__ __forceinline__ unsigned int umax(unsigned int a, unsigned int b) { return a > b ? a : b; }
__device__ __forceinline__ unsigned int umin(unsigned int a, unsigned int b) { return a < b ? a : b; }

// Asynchronous global -> shared copies (cp.async, sm_80+): the thread's old
// pair list is fetched while it walks its stencil.  Each thread copies and
// later reads only its own shared slots, so a per-thread wait suffices.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned int s = (unsigned int)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Float-pair square of a float pair, and the float-pair square root.
__device__ __forceinline__ df df_sqr(df a)
{
    const df p = two_prod(a.hi, a.hi);
    return fast_two_sum(p.hi, p.lo + 2.f * a.hi * a.lo);
}
// The seed s may be a few ulp off: the remainder a - s^2 is exact (two_prod,
// Sterbenz) and the correction step r / 2s brings the pair to the float-pair
// square root all the same.
__device__ __forceinline__ df df_sqrt(df a)
{
    const float s = sqrt_fast(a.hi);
    if (!(s > 0.f)) return df{s, 0.f};
    const df p = two_prod(s, s);
    const float r = ((a.hi - p.hi) - p.lo) + a.lo;
    return fast_two_sum(s, r * div_fast(0.5f, s));
}
// One component of the relative position of neighbour j from sphere i as a
// float pair: (A_j + L_j) - (A_i + L_i) + step, with step = +-cell size or 0
// (float pair step_hi + step_lo).
__device__ __forceinline__ df rel_df(float aj, float lj, float ai, float li, float step_hi, float step_lo)
{
    df s = two_sum(aj, -ai);
    s = df_add_f(s, step_hi);
    return df_add_f(s, (lj - li) + step_lo);
}
__device__ __forceinline__ float4 d2f4(d4 a) { return make_float4(d2f_rn(a.x), d2f_rn(a.y), d2f_rn(a.z), d2f_rn(a.w)); }
__device__ __forceinline__ V3<float> vf(float3 a) { return v3<float>(a.x, a.y, a.z); }

// Euler-parameter acceleration (closed form of calculate_uceom, impl:74-133)
// and the frame rotations in FP32.
__device__ __forceinline__ float4 uceom_f(float3 J, float4 e, float4 ev, float3 n)
{
    const float T0 = J.x * (-e.y * ev.x + e.x * ev.y + e.w * ev.z - e.z * ev.w);
    const float T1 = J.y * (-e.z * ev.x - e.w * ev.y + e.x * ev.z + e.y * ev.w);
    const float T2 = J.z * (-e.w * ev.x + e.z * ev.y - e.y * ev.z + e.x * ev.w);
    const float4 h = make_float4(4.f * (-ev.y * T0 - ev.z * T1 - ev.w * T2), 4.f * (ev.x * T0 - ev.w * T1 + ev.z * T2),
                                 4.f * (ev.w * T0 + ev.x * T1 - ev.y * T2), 4.f * (-ev.z * T0 + ev.y * T1 + ev.x * T2));
    const float r0 = n.x - (-e.y * h.x + e.x * h.y + e.w * h.z - e.z * h.w);
    const float r1 = n.y - (-e.z * h.x - e.w * h.y + e.x * h.z + e.y * h.w);
    const float r2 = n.z - (-e.w * h.x + e.z * h.y - e.y * h.z + e.x * h.w);
    const float r3 = -(ev.x * ev.x + ev.y * ev.y + ev.z * ev.z + ev.w * ev.w);
    const float ie2 = 1.f / (e.x * e.x + e.y * e.y + e.z * e.z + e.w * e.w);
    const float a0 = qdiv(r0 * ie2, 2.f * J.x), a1 = qdiv(r1 * ie2, 2.f * J.y), a2 = qdiv(r2 * ie2, 2.f * J.z);
    const float a3 = r3 * ie2;
    return make_float4(-e.y * a0 - e.z * a1 - e.w * a2 + e.x * a3, e.x * a0 - e.w * a1 + e.z * a2 + e.y * a3,
                       e.w * a0 + e.x * a1 - e.y * a2 + e.z * a3, -e.z * a0 + e.y * a1 + e.x * a2 + e.w * a3);
}
__device__ __forceinline__ float3 to_local_f(float3 v, float4 e)
{
    const float3 r0 = make_float3(2.f * (e.x * e.x + e.y * e.y - 0.5f), 2.f * (e.y * e.z - e.x * e.w),
                                  2.f * (e.y * e.w + e.x * e.z));
    const float3 r1 = make_float3(2.f * (e.y * e.z + e.x * e.w), 2.f * (e.x * e.x + e.z * e.z - 0.5f),
                                  2.f * (e.z * e.w - e.x * e.y));
    const float3 r2 = make_float3(2.f * (e.y * e.w - e.x * e.z), 2.f * (e.z * e.w + e.x * e.y),
                                  2.f * (e.x * e.x + e.w * e.w - 0.5f));
    return make_float3(r0.x * v.x + r1.x * v.y + r2.x * v.z, r0.y * v.x + r1.y * v.y + r2.y * v.z,
                       r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
// A(e) v: body frame to global frame.
__device__ __forceinline__ float3 to_global_f(float3 v, float4 e)
{
    return make_float3(2.f * ((e.x * e.x + e.y * e.y - 0.5f) * v.x + (e.y * e.z - e.x * e.w) * v.y +
                              (e.y * e.w + e.x * e.z) * v.z),
                       2.f * ((e.y * e.z + e.x * e.w) * v.x + (e.x * e.x + e.z * e.z - 0.5f) * v.y +
                              (e.z * e.w - e.x * e.y) * v.z),
                       2.f * ((e.y * e.w - e.x * e.z) * v.x + (e.z * e.w + e.x * e.y) * v.y +
                              (e.x * e.x + e.w * e.w - 0.5f) * v.z));
}
__device__ __forceinline__ float3 ang_vel_f(float4 e, float4 d)
{
    return make_float3(2.f * (-e.y * d.x + e.x * d.y - e.w * d.z + e.z * d.w),
                       2.f * (-e.z * d.x + e.w * d.y + e.x * d.z - e.y * d.w),
                       2.f * (-e.w * d.x - e.z * d.y + e.y * d.z + e.x * d.w));
}

// Hertz-Mindlin / DHS (impl:432-474) in FP32 with the tangential history
// (ds, previous s_dot) in FP32 registers.
__device__ __forceinline__ void model_f(int model, const FC<float>& c, float dt, float cdist, float& ds_io,
                                        float& dots_io, V3<float> dv, V3<float> unit, V3<float>& Ft, V3<float>& Fn,
                                        float fca)
{
    const float fsn = -c.kn * (cdist * sqrt_fast(cdist));
    const float dvn = tdot(dv, unit);
    Fn = (fsn + fca + c.vn * dvn) * unit;
    const V3<float> e = dv - dvn * unit;
    // an exactly zero tangential velocity is common (stacked spheres); skip
    // the square root's special-case path for it
    const float me2 = tdot(e, e);
    const float mag_e = me2 == 0.f ? 0.f : sqrt_fast(me2);
    if (mag_e != 0.f) {
        const float inv_e = div_fast(1.f, mag_e);
        const V3<float> s_hat = v3<float>(e.x * inv_e, e.y * inv_e, e.z * inv_e);
        const float s_dot = tdot(dv, s_hat);
        const float ds = ds_io + dt * (s_dot + dots_io);
        ds_io = ds;
        dots_io = s_dot;
        float a;
        if (model == 1) {
            const float S_t = c.ks * sqrt_fast(c.eq_r * cdist);
            a = S_t * ds + c.vs * sqrt_fast(S_t * c.eq_m);
        } else {
            a = c.ks * ds + c.vs * s_dot;
        }
        const float b = c.mu * len_fast(Fn);
        Ft = (a < b ? a : b) * s_hat;
    }
}

// Block sum of six per-thread FP32 values into out[0..5] (FP64): compensated
// warp butterflies, then one compensated combine of the warps.  Skips the
// reduction when no thread of the block contributed.  Two barriers; the
// shared array is reused by the next call only after its first barrier.
__device__ __forceinline__ void emit_body_f(const float f6[6], bool any, double* out, float* sm)
{
    if (!__syncthreads_or(any ? 1 : 0)) {
        if (threadIdx.x == 0)
            for (int c = 0; c < 6; ++c) out[c] = 0.0;
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        float hi = f6[c], lo = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
            const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
            const df s = two_sum(hi, oh);
            hi = s.hi;
            lo = (lo + ol) + s.lo;
        }
        if (lane == 0) {
            sm[(warp * 6 + c) * 2] = hi;
            sm[(warp * 6 + c) * 2 + 1] = lo;
        }
    }
    __syncthreads();
    if (warp == 0 && lane < 6) {
        const int nw = blockDim.x >> 5;
        CSum s;
        for (int w = 0; w < nw; ++w) {
            s.add(sm[(w * 6 + lane) * 2]);
            s.lo += sm[(w * 6 + lane) * 2 + 1];
        }
        out[lane] = f2d(s.hi) + f2d(s.lo);
    }
}

// Warp sum of six per-thread FP32 values into out[0..5] (FP64), written by
// lane 0: the compensated butterflies of emit_body_f without its combine
// across warps, so no block barrier.  Every lane of the warp calls it.
__device__ __forceinline__ void emit_warp_f(const float f6[6], bool any, double* out)
{
    const int lane = threadIdx.x & 31;
    if (!__any_sync(0xffffffffu, any)) {
        if (lane < 6) out[lane] = 0.0;
        return;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        float hi = f6[c], lo = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
            const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
            const df t = two_sum(hi, oh);
            hi = t.hi;
            lo = (lo + ol) + t.lo;
        }
        if (lane == 0) out[c] = f2d(hi) + f2d(lo);
    }
}

// Per-sphere accumulators of the mixed kernel.
struct Acc {
    CSum f[3], m[3];
    V3<float> tm;   // rolling: sum of contact moments (impl:476-483)
    float rs;       // rolling: resistance
};

// Particle-particle contact (impl:613-733) over the FP32 snapshot, in two
// passes so that the neighbour walk and the contact arithmetic do not hold
// their registers at the same time:
//  1. walk the 27-cell stencil (9 rows of 3 cells; the six cell-range loads
//     of a row are issued together) and stage, in walk order, the sorted
//     positions of the candidates whose FP32 squared distance is within
//     1 + 2^-11 of the squared contact distance (its FP32 rounding is below
//     2^-21).  The relative position of a neighbour is (stencil step) * cell
//     size + (offset difference), both small, so FP32 resolves it to ~1e-9 m
//     wherever the spheres are;
//  2. measure each staged candidate again in float pairs (offsets and radii
//     carry their low parts), so the overlap -- which can be 1e-6 of the
//     radius -- keeps ~1e-16 m resolution and the contact test classifies as
//     the FP64 form does; then the contact force.
// The stage holds STAGE entries per thread in shared memory (a tuning
// parameter, as is the block size NT: shared arrays are laid out
// [slot][thread] with stride NT); when more pass the screen, the walk is
// repeated for the rest, in the same order.  Entries
// whose packed unwrapped cell is not one of the stencil's are aliases of the
// wrapping hash and are skipped.
// Pass 2 for one candidate: sphere k with packed cell Tk and records Aj, Lj,
// Bj, Cj.
template <unsigned int NT>
__device__ __forceinline__ void p2p_pair_rec(const ContactLaunch& c, unsigned int k, unsigned int Tk, float4 Aj,
                                             float4 Lj, float4 Bj, float4 Cj, unsigned int ux, unsigned int uy,
                                             unsigned int uz, float4 Ai, float4 Li, float4 Bi, float4 Ci,
                                             unsigned int sid, unsigned int old_count, const unsigned int* old_id,
                                             unsigned int scene, const MatR<float>& mr, bool coh, V3<float>& Ft,
                                             V3<float>& Fn, unsigned int& cnt, Acc& acc, unsigned int& bits)
{
    const float cs = c.cs_f, cs_lo = c.cs_lo;
    const uint2 it = make_uint2(k, Tk);
    // stencil steps (+1) from the packed cells, and the shifts as float pairs
    const unsigned int xs = (it.y - ux + 1u) & 2047u;
    const unsigned int ys = ((it.y >> 11) - uy + 1u) & 2047u;
    const unsigned int zs = ((it.y >> 22) - uz + 1u) & 1023u;
    const float shx = xs == 0u ? -cs : (xs == 2u ? cs : 0.f), shx_lo = xs == 0u ? -cs_lo : (xs == 2u ? cs_lo : 0.f);
    const float shy = ys == 0u ? -cs : (ys == 2u ? cs : 0.f), shy_lo = ys == 0u ? -cs_lo : (ys == 2u ? cs_lo : 0.f);
    const float shz = zs == 0u ? -cs : (zs == 2u ? cs : 0.f), shz_lo = zs == 0u ? -cs_lo : (zs == 2u ? cs_lo : 0.f);
    const df rx = rel_df(Aj.x, Lj.x, Ai.x, Li.x, shx, shx_lo);
    const df ry = rel_df(Aj.y, Lj.y, Ai.y, Li.y, shy, shy_lo);
    const df rz = rel_df(Aj.z, Lj.z, Ai.z, Li.z, shz, shz_lo);
    const df dd = df_sqrt(df_add(df_add(df_sqr(rx), df_sqr(ry)), df_sqr(rz)));
    const float cdist = df_f(df_sub(df_add(df{Ai.w, Li.w}, df{Aj.w, Lj.w}), dd));
    const float dist = df_f(dd);
    const V3<float> rp = v3<float>(df_f(rx), df_f(ry), df_f(rz));
    const float ir = Ai.w;
    const unsigned int slot = sid + cnt;
    if (!(cdist > 0.f)) {
        if (!coh) return;
        const mat_pair& mp = c.mp[scene];
        const double csd = limit_cohesion_depth(mp, ir, Aj.w);
        if (!(fabs((double)cdist) < fabs(csd))) return;
        const V3<float> unit = qdiv(rp, dist);
        const double f = jkr_separation_force(mp, ir, Aj.w);
        const float cf = (float)cohesion_force(mp, ir, Aj.w, f);
        acc.f[0].add(-cf * unit.x); acc.f[1].add(-cf * unit.y); acc.f[2].add(-cf * unit.z);
        if (cnt < MAX_P2P_COUNT) {
            c.pp_id_new[slot] = k;
            reinterpret_cast<float2*>(c.pp_tsd_new)[slot] = make_float2(0.f, 0.f);
            cnt++;
        } else {
            bits |= XDEM_ERR_P2P_OVERFLOW;
        }
        return;
    }
    // history (impl:683-690): partner ids from the shared-memory copy of the
    // old list, the matching history from global memory.  A partner id occurs
    // once in a list, so the slot found does not depend on where the search
    // starts; it starts at this contact's new slot, where the partner sits
    // whenever the contacts before it are those of the last step
    float sd0 = 0.f, sd1 = 0.f;
    unsigned int hit = old_count;
    if (cnt < old_count && old_id[cnt * NT] == k) {
        hit = cnt;
    } else {
        for (unsigned int q = 0; q < old_count; ++q)
            if (old_id[q * NT] == k) {
                hit = q;
                break;
            }
    }
    if (hit < old_count) {
        // FP32 history (float2 slots in the double2 buffer)
        const float2 t = reinterpret_cast<const float2*>(c.pp_tsd_old)[sid + hit];
        sd0 = t.x; sd1 = t.y;
    }
    const V3<float> unit = qdiv(rp, dist);
    const V3<float> dcpr = ir * unit;
    const V3<float> dcpr_j = dcpr - rp;
    const V3<float> rv = (v3<float>(Bj.x, Bj.y, Bj.z) + tcross(v3<float>(Cj.x, Cj.y, Cj.z), dcpr_j)) -
                         (v3<float>(Bi.x, Bi.y, Bi.z) + tcross(v3<float>(Ci.x, Ci.y, Ci.z), dcpr));
    const FC<float> fc = fconst_f(mr, c.prm.contact_model, ir, Aj.w, Bi.w, Bj.w);
    float fca = 0.f;
    if (coh) {
        const double fsn = -(double)fc.kn * ((double)cdist * sqrt((double)cdist));
        const double fdn = (double)fc.vn * (double)tdot(rv, unit);
        fca = (float)(-cohesion_force(c.mp[scene], ir, Aj.w, fsn + fdn));
    }
    model_f(c.prm.contact_model, fc, c.dt_f, cdist, sd0, sd1, rv, unit, Ft, Fn, fca);
    const V3<float> fsum = Fn + Ft;
    // moment dcpr x (Fn + Ft) with dcpr = r n and Fn parallel to n: only the
    // tangential force turns the sphere.  Forming r (n x Ft) leaves out the
    // FP32 residue of crossing two parallel vectors (~1e-7 of r |Fn|), which
    // would otherwise be the whole moment of a contact without friction
    const V3<float> mm = ir * tcross(unit, Ft);
    acc.f[0].add(fsum.x); acc.f[1].add(fsum.y); acc.f[2].add(fsum.z);
    acc.m[0].add(mm.x); acc.m[1].add(mm.y); acc.m[2].add(mm.z);
    if (c.rolling) {
        acc.tm = acc.tm + mm;
        const float Rij = ir * Aj.w / (ir + Aj.w);
        acc.rs += Rij * mr.rfric * tlen(Fn);
    }
    if (cnt < MAX_P2P_COUNT) {
        c.pp_id_new[slot] = k;
        reinterpret_cast<float2*>(c.pp_tsd_new)[slot] = make_float2(sd0, sd1);
        cnt++;
    } else {
        bits |= XDEM_ERR_P2P_OVERFLOW;
    }
}

// Pass 2 for one staged candidate at sorted position j (every record of the
// candidate in one round trip: the screen is tight, so velocity and spin are
// nearly always needed).
template <unsigned int NT>
__device__ __forceinline__ void p2p_pair(const ContactLaunch& c, unsigned int oid, unsigned int j, unsigned int ux,
                                         unsigned int uy, unsigned int uz, float4 Ai, float4 Li, float4 Bi, float4 Ci,
                                         unsigned int sid, unsigned int old_count, const unsigned int* old_id,
                                         unsigned int scene, const MatR<float>& mr, bool coh, V3<float>& Ft,
                                         V3<float>& Fn, unsigned int& cnt, Acc& acc, unsigned int& bits)
{
    const uint2 it = reinterpret_cast<const uint2*>(c.mIT)[j];
    if (c.scene_of && c.scene_of[it.x] != scene) return;  // another scene of the batch
    const float4 Aj = reinterpret_cast<const float4*>(c.mA)[j];
    const float4 Lj = reinterpret_cast<const float4*>(c.mL)[j];
    const float4 Bj = reinterpret_cast<const float4*>(c.mB)[j];
    const float4 Cj = reinterpret_cast<const float4*>(c.mC)[j];
    p2p_pair_rec<NT>(c, it.x, it.y, Aj, Lj, Bj, Cj, ux, uy, uz, Ai, Li, Bi, Ci, sid, old_count, old_id, scene, mr, coh,
                     Ft, Fn, cnt, acc, bits);
}

// Pass 1 + 2 over the 27-cell stencil.  With `build` the screen widens by
// the skin and every candidate it passes (at most kListCap; the count keeps
// going past it to flag an overflow) goes to the sphere's candidate list.
template <unsigned int NT, unsigned int STAGE>
__device__ __forceinline__ void p2p_mixed(const ContactLaunch& c, unsigned int oid, unsigned int gx,
                                          unsigned int gy, unsigned int gz, float4 Ai, float4 Li, unsigned int Ti,
                                          float4 Bi, float4 Ci, unsigned int* stage, unsigned int* old_id,
                                          Acc& acc, unsigned int& bits, bool build = false)
{
    const device_dem_parameters& p = c.prm;
    unsigned int nlist = 0;
    unsigned int* vl = build ? c.vl_ids + (size_t)oid * kListCap : nullptr;
    const unsigned int scene = scene_index(c, oid);
    const MatR<float> mr = matr(c.mpf[scene]);  // the pair material, once per sphere
    const bool coh = c.mpf[scene].coh != 0;
    const float cs = c.cs_f;
    const float screen = 1.0f + 0x1p-11f;
    const unsigned int ux = Ti & 2047u, uy = (Ti >> 11) & 2047u, uz = Ti >> 22;
    const unsigned int sid = oid * MAX_P2P_COUNT;
    // partners k with |oid - k| <= excl are skipped: the sphere itself, and
    // for clusters every sphere up to neach ids away (impl:556-558)
    const unsigned int excl = c.cl.neach;
    unsigned int old_count = c.pp_count_old[oid];
    if (old_count > MAX_P2P_COUNT) old_count = MAX_P2P_COUNT;
    // the old partner ids travel to shared memory while the stencil is walked
    for (unsigned int q = 0; q < old_count; ++q) cp_async4(old_id + q * NT, c.pp_id_old + sid + q);
    cp_async_commit();
    V3<float> Ft = v3<float>(0, 0, 0), Fn = v3<float>(0, 0, 0);
    unsigned int cnt = 0, done = 0;
    bool more = true;
    while (more) {
        // ---- pass 1: screened candidates done, done + 1, ... of the walk
        more = false;
        unsigned int seen = 0, nc = 0;
        // rows in walk order (z outer, y inner); software-pipelined: the next
        // row's six cell-range loads and the first entry of each of this
        // row's three cells are in flight together
        unsigned int rs[3], re[3];
#pragma unroll
        for (int x = -1; x <= 1; ++x) {
            const unsigned int h = grid_hash(p, (int)gx + x, (int)gy - 1, (int)gz - 1);
            rs[x + 1] = c.cstart[h];
            re[x + 1] = c.cend[h];
        }
        for (int row = 0; row < 9 && !more; ++row) {
            const int z = row / 3 - 1, y = row % 3 - 1;
            uint2 it0[3];
            float4 A0[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                it0[r] = make_uint2(0u, 0u);
                A0[r] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (rs[r] != 0xffffffffu) {
                    it0[r] = reinterpret_cast<const uint2*>(c.mIT)[rs[r]];
                    A0[r] = reinterpret_cast<const float4*>(c.mA)[rs[r]];
                }
            }
            unsigned int nrs[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, nre[3] = {0u, 0u, 0u};
            if (row < 8) {
                const int nz = (row + 1) / 3 - 1, ny = (row + 1) % 3 - 1;
#pragma unroll
                for (int x = -1; x <= 1; ++x) {
                    const unsigned int h = grid_hash(p, (int)gx + x, (int)gy + ny, (int)gz + nz);
                    nrs[x + 1] = c.cstart[h];
                    nre[x + 1] = c.cend[h];
                }
            }
            {
                const unsigned int want_yz = pack_cell(0, (int)uy + y, (int)uz + z);
                const float sy = (y < 0 ? -cs : (y > 0 ? cs : 0.f)) - Ai.y;
                const float sz = (z < 0 ? -cs : (z > 0 ? cs : 0.f)) - Ai.z;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    if (rs[r] == 0xffffffffu || more) continue;
                    const unsigned int end = re[r];
                    for (unsigned int j = rs[r]; j < end; ++j) {
                        const uint2 it = j == rs[r] ? it0[r] : reinterpret_cast<const uint2*>(c.mIT)[j];
                        const float4 Aj = j == rs[r] ? A0[r] : reinterpret_cast<const float4*>(c.mA)[j];
                        const unsigned int xs = (it.y - ux + 1u) & 2047u;  // x step + 1 unless an alias
                        if ((it.y & ~2047u) != want_yz || xs > 2u || umax(it.x, oid) - umin(it.x, oid) <= excl ||
                            it.x >= c.np)
                            continue;
                        if (!coh) {
                            const float dx = Aj.x + ((xs == 0u ? -cs : (xs == 2u ? cs : 0.f)) - Ai.x);
                            const float dy = Aj.y + sy, dz = Aj.z + sz;
                            const float rr = Ai.w + Aj.w;
                            const float lim = build ? (rr + c.skin_f) * (rr + c.skin_f) : rr * rr * screen;
                            if (!(dx * dx + dy * dy + dz * dz < lim)) continue;
                        }
                        if (seen++ < done) continue;
                        if (nc == STAGE) {
                            more = true;
                            break;
                        }
                        stage[nc++ * NT] = j;
                        if (build) {
                            if (nlist < kListCap) vl[nlist] = it.x;
                            nlist++;
                        }
                    }
                }
            }
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                rs[x] = nrs[x];
                re[x] = nre[x];
            }
        }
        done += nc;
        cp_async_wait_all();
        // ---- pass 2: float-pair overlap and contact force, in walk order
        for (unsigned int q = 0; q < nc; ++q)
            p2p_pair<NT>(c, oid, stage[q * NT], ux, uy, uz, Ai, Li, Bi, Ci, sid, old_count, old_id, scene, mr,
                     coh, Ft, Fn, cnt, acc, bits);
    }
    c.pp_count_new[oid] = cnt;
    if (build) {
        if (nlist > kListCap) {
            atomicOr(c.vl_flag + kVlOverflow, 1u);
        } else {
            // the row ascends by id, so that a list step's (stencil cell,
            // slot) keys order the contacts by (cell, id) as the walk does
            for (unsigned int a = 1; a < nlist; ++a) {
                const unsigned int v = vl[a];
                unsigned int b = a;
                for (; b > 0 && vl[b - 1] > v; --b) vl[b] = vl[b - 1];
                vl[b] = v;
            }
        }
        c.vl_cnt[oid] = nlist;
        reinterpret_cast<float4*>(c.vl_xb)[oid] =
            make_float4((float)ux * cs + Ai.x, (float)uy * cs + Ai.y, (float)uz * cs + Ai.z, 0.f);
    }
}

// The same contacts from sphere oid's candidate list instead of the stencil
// walk.  The walk meets neighbours cell by cell (z, then y, then x offset of
// the neighbour's cell from oid's, each -1..1) and, within a cell, in sorted
// order, which is ascending id (the sort is stable and its input is in id
// order).  Sorting the candidates by (cell offset, id) from this step's
// cells therefore visits the contacts in the walk's order: pair lists, the
// Ft a zero-slip contact keeps and every sum come out the same.  The list
// holds every sphere within r_i + r_j + skin at its build, so while no
// sphere has moved half the skin it holds every contact.
static_assert(kListCap <= 32, "a list sort key keeps the slot in 5 bits");

template <unsigned int NT>
__device__ __forceinline__ void p2p_list(const ContactLaunch& c, unsigned int oid, float4 Ai, float4 Li,
                                         unsigned int Ti, float4 Bi, float4 Ci, unsigned int* old_id,
                                         unsigned int* keys, Acc& acc, unsigned int& bits)
{
    const unsigned int scene = scene_index(c, oid);
    const MatR<float> mr = matr(c.mpf[scene]);  // the pair material, once per sphere
    const bool coh = false;  // lists are only kept without cohesion
    const float cs = c.cs_f;
    const float screen = 1.0f + 0x1p-11f;
    const unsigned int ux = Ti & 2047u, uy = (Ti >> 11) & 2047u, uz = Ti >> 22;
    const unsigned int sid = oid * MAX_P2P_COUNT;
    unsigned int old_count = c.pp_count_old[oid];
    if (old_count > MAX_P2P_COUNT) old_count = MAX_P2P_COUNT;
    for (unsigned int q = 0; q < old_count; ++q) cp_async4(old_id + q * NT, c.pp_id_old + sid + q);
    cp_async_commit();
    const unsigned int n = c.vl_cnt[oid];
    const unsigned int* ids = c.vl_ids + (size_t)oid * kListCap;
    // the first four candidates come with the count (a row is 96 bytes, so
    // 16-byte aligned), not after it: their records' loads start a round
    // trip earlier
    const uint4 head = reinterpret_cast<const uint4*>(ids)[0];
    // Key phase: each candidate's position (A) and cell (C) records; those
    // inside this step's stencil that pass the walk's FP32 screen (squared
    // distance within 1 + 2^-11 of the squared contact distance, so no
    // contact is ever dropped: the float-pair test below decides) get a key
    // (stencil cell << 5 | slot).  The row is sorted by id when it is built,
    // so ascending keys visit the contacts in the walk's (cell, id) order.
    // Keys are sorted in shared memory, [slot][thread] with stride NT.
    unsigned int nk = 0;
#pragma unroll 2
    for (unsigned int q = 0; q < n; ++q) {
        const unsigned int k = q == 0 ? head.x : q == 1 ? head.y : q == 2 ? head.z : q == 3 ? head.w : ids[q];
        if (c.scene_of && c.scene_of[k] != scene) continue;  // another scene of the batch
        const float4* r = c.rec + 4 * (size_t)k;
        const float4 Aj = r[kRecA];
        const unsigned int Tk = rec_cell(r[kRecC]);
        const unsigned int xs = (Tk - ux + 1u) & 2047u;
        const unsigned int ys = ((Tk >> 11) - uy + 1u) & 2047u;
        const unsigned int zs = ((Tk >> 22) - uz + 1u) & 1023u;
        if (xs > 2u || ys > 2u || zs > 2u) continue;
        const float dx = Aj.x + ((xs == 0u ? -cs : (xs == 2u ? cs : 0.f)) - Ai.x);
        const float dy = Aj.y + ((ys == 0u ? -cs : (ys == 2u ? cs : 0.f)) - Ai.y);
        const float dz = Aj.z + ((zs == 0u ? -cs : (zs == 2u ? cs : 0.f)) - Ai.z);
        const float rr = Ai.w + Aj.w;
        if (!(dx * dx + dy * dy + dz * dz < rr * rr * screen)) continue;
        const unsigned int key = (((zs * 3u + ys) * 3u + xs) << 5) | q;
        unsigned int p = nk++;
        while (p > 0 && keys[(p - 1) * NT] > key) {
            keys[p * NT] = keys[(p - 1) * NT];
            --p;
        }
        keys[p * NT] = key;
    }
    cp_async_wait_all();
    V3<float> Ft = v3<float>(0, 0, 0), Fn = v3<float>(0, 0, 0);
    unsigned int cnt = 0;
    for (unsigned int q = 0; q < nk; ++q) {
        const unsigned int k = ids[keys[q * NT] & 31u];
        const float4* r = c.rec + 4 * (size_t)k;
        const float4 Aj = r[kRecA], Lj = r[kRecL], Bj = r[kRecB], Cj = r[kRecC];
        p2p_pair_rec<NT>(c, k, rec_cell(Cj), Aj, Lj, Bj, Cj, ux, uy, uz, Ai, Li, Bi, Ci, sid, old_count, old_id, scene,
                         mr, coh, Ft, Fn, cnt, acc, bits);
    }
    c.pp_count_new[oid] = cnt;
}

// Plane contact region and depth (impl:735-815, plane_detection) for a plane
// that is an orthonormal rectangle, in its local frame: the centre's local
// coordinates are float-pair dot products of (x - xw) with u1, u2 and the
// unit normal, so the depth keeps ~1e-15 m resolution however far the plane
// reaches.  Returns the depth (0 when no region applies) and the unit vector
// with the reference's orientation per region (corners: corner -> centre;
// edges: centre -> edge; face: minus the normal).
__device__ __forceinline__ float plane_rect(const PlaneDF& pd, const df xd[3], df rd, V3<float>& u)
{
    df dp[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) dp[i] = df_sub(xd[i], df{pd.xw_hi[i], pd.xw_lo[i]});
    df w[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        w[a] =df_add(df_add(df_mul(dp[0], df{pd.u_hi[3 * a], pd.u_lo[3 * a]}),
                             df_mul(dp[1], df{pd.u_hi[3 * a + 1], pd.u_lo[3 * a + 1]})),
                      df_mul(dp[2], df{pd.u_hi[3 * a + 2], pd.u_lo[3 * a + 2]}));
    }
    const float wx = df_f(w[0]), wy = df_f(w[1]), wz = df_f(w[2]);
    const float r = df_f(rd);
    const df l1 = df{pd.l1_hi, pd.l1_lo}, l2 = df{pd.l2_hi, pd.l2_lo};
    const float l1f = df_f(l1), l2f = df_f(l2);
    const float dx1 = df_f(df_sub(w[0], l1)), dy2 = df_f(df_sub(w[1], l2));
    const float sqa = wx * wx, sqb = wy * wy, sqc = wz * wz, sqr = r * r, a_l1 = dx1 * dx1, b_l2 = dy2 * dy2;
    float lx = 0.f, ly = 0.f, lz = wz;
    int kind = 0;  // 1 corner, 2 edge, 3 face
    if (wx < 0 && wy < 0 && (sqa + sqb + sqc) < sqr) { lx = wx; ly = wy; kind = 1; }
    else if (wx > l1f && wy < 0 && (a_l1 + sqb + sqc) < sqr) { lx = dx1; ly = wy; kind = 1; }
    else if (wx > l1f && wy > l2f && (a_l1 + b_l2 + sqc) < sqr) { lx = dx1; ly = dy2; kind = 1; }
    else if (wx < 0 && wy > l2f && (sqa + b_l2 + sqc) < sqr) { lx = wx; ly = dy2; kind = 1; }
    else if ((wx > 0 && wx < l1f) && wy < 0 && (sqb + sqc) < sqr) { ly = wy; kind = 2; }
    else if ((wx > 0 && wx < l1f) && wy > l2f && (b_l2 + sqc) < sqr) { ly = dy2; kind = 2; }
    else if ((wx > 0 && wy < l2f) && wx > l1f && (a_l1 + sqc) < sqr) { lx = dx1; kind = 2; }
    else if ((wx > 0 && wx < l1f) && (wy > 0 && wy < l2f)) kind = 3;
    const V3<float> u1 = v3<float>(pd.u_hi[0], pd.u_hi[1], pd.u_hi[2]);
    const V3<float> u2 = v3<float>(pd.u_hi[3], pd.u_hi[4], pd.u_hi[5]);
    const V3<float> un = v3<float>(pd.u_hi[6], pd.u_hi[7], pd.u_hi[8]);
    if (kind == 0) return 0.f;
    if (kind == 3) {
        u = -un;
        const df awz = w[2].hi < 0.f ? df_neg(w[2]) : w[2];
        return df_f(df_sub(rd, awz));
    }
    const float h = sqrtf(lx * lx + ly * ly + lz * lz);
    const V3<float> X = (lx * u1 + ly * u2) + lz * un;
    u = kind == 1 ? qdiv(X, h) : -qdiv(X, h);
    return r - h;
}

// Rigid-body record (decl:20) in FP32: velocity and angular velocity; the
// reference point as float pairs.
struct BodyF {
    df p[3];
    V3<float> v, om;
    float m;
};
__device__ __forceinline__ BodyF load_body_f(const double* dbi)
{
    BodyF b;
    b.m = d2f_rn(dbi[XDEM_MM]);
    b.p[0] = split_d(dbi[XDEM_PX]); b.p[1] = split_d(dbi[XDEM_PY]); b.p[2] = split_d(dbi[XDEM_PZ]);
    b.v = v3<float>(d2f_rn(dbi[XDEM_VX]), d2f_rn(dbi[XDEM_VY]), d2f_rn(dbi[XDEM_VZ]));
    const float4 e = make_float4(d2f_rn(dbi[XDEM_E0]), d2f_rn(dbi[XDEM_E1]), d2f_rn(dbi[XDEM_E2]), d2f_rn(dbi[XDEM_E3]));
    const float4 d = make_float4(d2f_rn(dbi[XDEM_ED0]), d2f_rn(dbi[XDEM_ED1]), d2f_rn(dbi[XDEM_ED2]),
                                 d2f_rn(dbi[XDEM_ED3]));
    b.om = vf(ang_vel_f(e, d));
    return b;
}

// Plane slots of one sphere (impl:950-1080 slot rule), loaded on first use.

// One sphere against plane k: contact force into `acc`, the body's share
// into f6.  Returns true when the sphere touched the plane.
// The plane slots (impl:950-1080 slot rule) are read from memory when a
// plane needs them: the thread owns its slots and writes them as it goes, so
// memory holds exactly what the reference's next plane launch re-reads.
// Cluster members (impl:817-948) differ in two places: the body's lever arm
// is taken from the member's centre (dcpr_j before the contact normal is
// known, impl:881-882), and the body's mass enters the effective mass.
__device__ __forceinline__ bool plane_mixed(const ContactLaunch& c, unsigned int k, unsigned int kbeg,
                                            unsigned int oid, d4 ip, V3<float> ivel, V3<float> iom, float im,
                                            unsigned int& pl_cnt, Acc& acc, float f6[6], unsigned int& bits)
{
    const bool member = c.cl.neach != 0;
    const device_dem_parameters& p = c.prm;
    const device_plane_info& pl = c.planes[k];
    const PlaneDF& pd = c.planedf[k];
    const unsigned int pid = pl.id;
    const mat_pair& mp = c.mp[c.nscene + k];  // FP64 constants: cohesion only
    const MatR<float> mr = matr(c.mpf[c.nscene + k]);
    const unsigned int sid = oid * MAX_P2PL_COUNT;
    if (k == kbeg) pl_cnt = 0;  // the scene's first plane restarts the list (impl:989)
    const df xd[3] = {split_d(ip.x), split_d(ip.y), split_d(ip.z)};
    const df rd = split_d(ip.w);
    const BodyF b = load_body_f(c.body + 15 * k);
    float cd;
    V3<float> un, rel;
    bool hit;
    double cdd = 0.0;
    if (pd.rect && !mr.coh) {
        cd = plane_rect(pd, xd, rd, un);
        hit = cd > 0.f;
        cdd = cd;
        rel = v3<float>(df_f(df_sub(xd[0], b.p[0])), df_f(df_sub(xd[1], b.p[1])), df_f(df_sub(xd[2], b.p[2])));
    } else {
        // general parallelogram or cohesion: FP64 region test (rare)
        const d3 ipos = mk3(ip.x, ip.y, ip.z);
        const d3 dp = ipos - dv3(pl.xw);
        d3 unit = mk3(0, 0, 0);
        const d3 wp = mk3(dot(dp, dv3(pl.u1)), dot(dp, dv3(pl.u2)), dot(dp, dv3(pl.uw)));
        cdd = plane_detection(pl, ipos, wp, unit, ip.w);
        double csd = 0.0;
        if (mr.coh) csd = limit_cohesion_depth(mp, ip.w, 0.0);
        hit = cdd > 0 || (cdd <= 0 && fabs(cdd) < fabs(csd));
        cd = (float)cdd;
        un = cvt<float>(unit);
        const double* bp = c.body + 15 * k;
        rel = v3<float>(d2f_rn(ip.x - bp[XDEM_PX]), d2f_rn(ip.y - bp[XDEM_PY]), d2f_rn(ip.z - bp[XDEM_PZ]));
    }
    if (!hit) return false;
    const float r = df_f(rd);
    const V3<float> dcpr = r * un;
    const V3<float> dcpr_j = member ? rel : rel + dcpr;
    float sd0 = 0.f, sd1 = 0.f;
    V3<float> mf;
    if (cdd > 0) {
        for (unsigned int q = 0; q < MAX_P2PL_COUNT; ++q)
            if (c.pl_id[sid + q] == pid) {
                const double2 t = reinterpret_cast<const double2*>(c.pl_tsd)[sid + q];
                sd0 = d2f_rn(t.x); sd1 = d2f_rn(t.y);
                break;
            }
        const V3<float> dv = (b.v + tcross(b.om, dcpr_j)) - (ivel + tcross(iom, dcpr));
        const FC<float> fc = fconst_f(mr, p.contact_model, r, 0.f, im, member ? b.m : 0.f);
        float fca = 0.f;
        if (mr.coh) {
            const double fsn = -(double)fc.kn * (cdd * sqrt(cdd));
            const double fdn = (double)fc.vn * (double)tdot(dv, un);
            fca = (float)(-cohesion_force(mp, ip.w, 0.0, fsn + fdn));
        }
        V3<float> Ft = v3<float>(0, 0, 0), Fn = v3<float>(0, 0, 0);
        model_f(p.contact_model, fc, c.dt_f, cd, sd0, sd1, dv, un, Ft, Fn, fca);
        mf = Fn + Ft;
        // dcpr = r un is parallel to Fn: only Ft turns the sphere (no FP32
        // residue of crossing parallel vectors)
        const V3<float> mm = r * tcross(un, Ft);
        acc.m[0].add(mm.x); acc.m[1].add(mm.y); acc.m[2].add(mm.z);
        if (c.rolling) {
            acc.tm = acc.tm + mm;
            acc.rs += r * mr.rfric * tlen(Fn);
        }
    } else {
        const double f = jkr_separation_force(mp, ip.w, 0.0);
        const float cf = (float)cohesion_force(mp, ip.w, 0.0, f);
        mf = (-cf) * un;
    }
    acc.f[0].add(mf.x); acc.f[1].add(mf.y); acc.f[2].add(mf.z);
    const V3<float> bm = tcross(dcpr_j, mf);
    f6[0] = -mf.x; f6[1] = -mf.y; f6[2] = -mf.z;
    f6[3] = -bm.x; f6[4] = -bm.y; f6[5] = -bm.z;
    if (pl_cnt < MAX_P2PL_COUNT) {
        c.pl_id[sid + pl_cnt] = pid;
        reinterpret_cast<double2*>(c.pl_tsd)[sid + pl_cnt] = make_double2(f2d(sd0), f2d(sd1));
        pl_cnt++;
    } else {
        bits |= XDEM_ERR_P2PL_OVERFLOW;
    }
    return true;
}

// One sphere against mesh m (impl:1930-2109): triangle candidates from the
// grid, FP64 closest-point geometry (the candidate classification and the
// 1e-9 de-duplication need it), FP32 forces.  Returns true when touched.
__device__ __forceinline__ bool mesh_mixed(const ContactLaunch& c, unsigned int m, unsigned int oid, unsigned int gx,
                                           unsigned int gy, unsigned int gz, d4 ip, V3<float> ivel, V3<float> iom,
                                           float im, Acc& acc, float f6[6], unsigned int& bits)
{
    const device_dem_parameters& p = c.prm;
    const d3 ipos = mk3(ip.x, ip.y, ip.z);
    const double ir = ip.w;
    const unsigned int lo = c.np + c.mesh_first[m], ntri = c.mesh_ntri[m];
    const int bidx = c.mesh_body[m];
    const mat_pair& mp = c.mp[c.nscene + bidx];  // FP64 constants: cohesion only
    const MatR<float> mr = matr(c.mpf[c.nscene + bidx]);
    const unsigned int sid = oid * MAX_P2MS_COUNT;
    unsigned int o_id[MAX_P2MS_COUNT];
    float o_a[MAX_P2MS_COUNT], o_b[MAX_P2MS_COUNT];
#pragma unroll
    for (int q = 0; q < (int)MAX_P2MS_COUNT; ++q) {
        o_id[q] = c.ms_id[sid + q];
        const double2 t = reinterpret_cast<const double2*>(c.ms_tsd)[sid + q];
        o_a[q] = d2f_rn(t.x); o_b[q] = d2f_rn(t.y);
    }
    struct Hit { unsigned int id; d3 cpt; };
    Hit hf[XDEM_MAX_TRI_CANDIDATES], hl[XDEM_MAX_TRI_CANDIDATES], hp[XDEM_MAX_TRI_CANDIDATES];
    unsigned int nf = 0, nl = 0, npt = 0;
    d3 prev_line = mk3(0, 0, 0), prev_point = mk3(0, 0, 0);
    double cs = 0.0;
    if (mr.coh) cs = limit_cohesion_depth(mp, ir, 0.0);
    // FP32 screen of a triangle by its fitted sphere, which contains it: a
    // sphere of the particle farther than r_tri + r from the centre cannot
    // touch the triangle (off with cohesion, which reaches beyond contact)
    const float xf = d2f_rn(ipos.x), yf = d2f_rn(ipos.y), zf = d2f_rn(ipos.z), rf = d2f_rn(ir);
    const double* sph = c.tri_sphere + 4 * (size_t)c.mesh_first[m];
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                const unsigned int h = grid_hash(p, (int)gx + x, (int)gy + y, (int)gz + z);
                const unsigned int start = c.cstart[h];
                if (start == 0xffffffffu) continue;
                const unsigned int end = c.cend[h];
                // a cell's entries are in ascending id (stable sort of an
                // id-ordered input): this mesh's spheres, ids lo .. lo + ntri
                // - 1, follow every particle; later meshes follow them
                // both scans take four entries a step, their loads issued
                // together, so a sphere's walk is a quarter as many
                // dependent loads long
                unsigned int jm = end;
                while (jm > start) {
                    const unsigned int n4 = umin(4u, jm - start);
                    unsigned int sk[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) sk[q] = (unsigned int)q < n4 ? c.sorted_index[jm - 1 - q] : 0u;
                    unsigned int k = 0;
                    while (k < n4 && sk[k] >= lo) ++k;
                    jm -= k;
                    if (k < n4) break;
                }
                for (unsigned int j0 = jm; j0 < end; j0 += 4) {
                    unsigned int tks[4];
                    unsigned int take4 = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        tks[q] = j0 + q < end ? c.sorted_index[j0 + q] - lo : 0xffffffffu;
                        if (tks[q] < ntri) take4 |= 1u << q;
                    }
                    // ids ascend within the cell: a later mesh's entry ends this one's
                    const bool last = take4 != 0xfu;
                    if (!mr.coh) {
                        float4 fs[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            fs[q] = make_float4(0.f, 0.f, 0.f, -1.f);
                            if (take4 >> q & 1u) {
                                const double2 q0 = reinterpret_cast<const double2*>(sph)[2 * tks[q]];
                                const double2 q1 = reinterpret_cast<const double2*>(sph)[2 * tks[q] + 1];
                                fs[q] = make_float4(d2f_rn(q0.x), d2f_rn(q0.y), d2f_rn(q1.x), d2f_rn(q1.y));
                            }
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float dx = fs[q].x - xf, dy = fs[q].y - yf, dz = fs[q].z - zf;
                            const float lim = fs[q].w + rf + 1e-5f;
                            if (dx * dx + dy * dy + dz * dz > lim * lim) take4 &= ~(1u << q);
                        }
                    }
                    for (int q = 0; q < 4; ++q) {
                    if (!(take4 >> q & 1u)) continue;
                    const unsigned int tk = tks[q];
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
                    if (last) break;
                }
            }
    const Hit* list = nf ? hf : (nl ? hl : hp);
    const unsigned int nlist = nf ? nf : (nl ? nl : npt);
    const BodyF b = load_body_f(c.body + 15 * bidx);
    const d3 bpos = mk3(c.body[15 * bidx + XDEM_PX], c.body[15 * bidx + XDEM_PY], c.body[15 * bidx + XDEM_PZ]);
    bool touched = false;
    unsigned int cnt = 0;
    for (unsigned int q = 0; q < nlist; ++q) {
        const Hit hit = list[q];
        float sd0 = 0.f, sd1 = 0.f;
        const V3<float> po2cp = cvt<float>(hit.cpt - bpos);
        const d3 rpd = hit.cpt - ipos;
        const double dist = length(rpd);
        const V3<float> un = cvt<float>(rpd / dist);
        const double cd = ir - dist;
        if (cd <= 0 && fabs(cd) < fabs(cs)) {
            const double f = jkr_separation_force(mp, ir, 0.0);
            const float cf = (float)cohesion_force(mp, ir, 0.0, f);
            acc.f[0].add(-cf * un.x); acc.f[1].add(-cf * un.y); acc.f[2].add(-cf * un.z);
        } else {
            for (int r = 0; r < (int)MAX_P2MS_COUNT; ++r)
                if (o_id[r] == hit.id) { sd0 = o_a[r]; sd1 = o_b[r]; break; }
            const V3<float> rc = cvt<float>(rpd);
            const V3<float> dv = (b.v + tcross(b.om, po2cp)) - (ivel + tcross(iom, rc));
            const FC<float> fc = fconst_f(mr, p.contact_model, (float)ir, 0.f, im, b.m);
            float fca = 0.f;
            if (mr.coh) {
                const double fsn = -(double)fc.kn * (cd * sqrt(cd));
                const double fdn = (double)fc.vn * (double)tdot(dv, un);
                fca = (float)(-cohesion_force(mp, ir, 0.0, fsn + fdn));
            }
            V3<float> Ft = v3<float>(0, 0, 0), Fn = v3<float>(0, 0, 0);
            model_f(p.contact_model, fc, c.dt_f, (float)cd, sd0, sd1, dv, un, Ft, Fn, fca);
            const V3<float> fsum = Fn + Ft;
            const V3<float> mm = tcross(rc, fsum);
            acc.tm = acc.tm + mm;
            acc.rs += (float)ir * mr.rfric * tlen(Fn);
            acc.f[0].add(fsum.x); acc.f[1].add(fsum.y); acc.f[2].add(fsum.z);
            acc.m[0].add(mm.x); acc.m[1].add(mm.y); acc.m[2].add(mm.z);
            const V3<float> bm = tcross(po2cp, fsum);
            f6[0] -= fsum.x; f6[1] -= fsum.y; f6[2] -= fsum.z;
            f6[3] -= bm.x; f6[4] -= bm.y; f6[5] -= bm.z;
            touched = true;
        }
        if (cnt < MAX_P2MS_COUNT) {
            c.ms_id[sid + cnt] = hit.id;
            reinterpret_cast<double2*>(c.ms_tsd)[sid + cnt] = make_double2(f2d(sd0), f2d(sd1));
            cnt++;
        } else {
            bits |= XDEM_ERR_P2MS_OVERFLOW;
        }
    }
    c.ms_count[oid] = cnt;
    return touched;
}

// Velocity update, next Euler parameters and centre of body i -- a sphere,
// or a cluster's centre -- (impl:192-222 and 224-287, 135-147 and 149-190)
// from its force Ff and moment Mf (global frame).  FP64 work: the 14
// additions of FP32 increments to the FP64 state.  The Euler parameters are
// renormalised to second order, 1/sqrt(1 + eps) ~ 1 - eps/2 + 3/8 eps^2,
// with eps = |e + de|^2 - 1 formed in float pairs from the FP64 e.
// Writes vel, ev and ep_next of body i, and its new acceleration and Euler-
// parameter acceleration: to the FP32 copies (F32: spheres) or to the FP64
// arrays (clusters); returns the next centre, the next Euler parameters
// (FP64, as stored, and FP32), their new rates and the new velocity in FP32.
struct NextBody {
    d3 x;
    d4 e;
    float4 ef, ev;
    V3<float> v;
};
// The state integrate_f reads for body i: velocity, Euler parameters and
// their rates in FP64; acceleration, Euler-parameter acceleration and
// principal inertia in FP32 (the step computes the accelerations in FP32, so
// they are exact in either storage).
struct BodyIn {
    d3 v;
    d4 e, ev;
    float3 a, J;
    float4 ea;
};
// From the FP64 arrays of the reference layout (clusters).
__device__ __forceinline__ BodyIn body_in(const ContactLaunch& c, unsigned int i)
{
    BodyIn b;
    b.v = ld3(c.vel, i); b.a = d2f3(ld3(c.acc, i)); b.J = d2f3(ld3(c.inertia, i));
    b.e = ld4(c.ep_cur, i); b.ev = ld4(c.ev, i); b.ea = d2f4(ld4(c.ea, i));
    return b;
}
// From the FP32 copies of a sphere handle (acc, ea, and inertia + mass);
// m receives the mass.
__device__ __forceinline__ BodyIn body_in_f32(const ContactLaunch& c, unsigned int i, float& m)
{
    BodyIn b;
    b.v = ld3(c.vel, i);
    b.e = ld4(c.ep_cur, i); b.ev = ld4(c.ev, i);
    const float4 a = c.accf[i], jm = c.jm[i];
    b.a = make_float3(a.x, a.y, a.z);
    b.J = make_float3(jm.x, jm.y, jm.z);
    b.ea = c.eaf[i];
    m = jm.w;
    return b;
}
template <bool F32>
__device__ __forceinline__ NextBody integrate_f(const ContactLaunch& c, unsigned int i, d3 xi, float m,
                                                V3<float> Ff, V3<float> Mf, bool apply_vel, const BodyIn& in)
{
    const float dt = c.dt_f, hdt = c.hdt_f, h2 = c.h2_f;
    const float inv_m = 1.f / m;
    const V3<float> a_new = v3<float>(Ff.x * inv_m + c.g_f[0], Ff.y * inv_m + c.g_f[1], Ff.z * inv_m + c.g_f[2]);
    NextBody o;
    // translation
    const d3 v = in.v;
    V3<float> vn = vf(d2f3(v));
    if (apply_vel) {
        const V3<float> dv = hdt * (vf(in.a) + a_new);
        st3(c.vel, i, mk3(v.x + f2d(dv.x), v.y + f2d(dv.y), v.z + f2d(dv.z)));
        vn = vn + dv;
    }
    if (F32)
        c.accf[i] = make_float4(a_new.x, a_new.y, a_new.z, 0.f);
    else
        st3(c.acc, i, mk3(f2d(a_new.x), f2d(a_new.y), f2d(a_new.z)));
    // rotation
    const d4 e = in.e;
    const df e0 = split_d(e.x), e1 = split_d(e.y), e2 = split_d(e.z), e3 = split_d(e.w);
    const float4 ef = make_float4(df_f(e0), df_f(e1), df_f(e2), df_f(e3));
    const d4 ev = in.ev;
    const float4 evf = d2f4(ev);
    const float4 eaf = in.ea;
    const float3 J = in.J;
    const float4 q = uceom_f(J, ef, evf, to_local_f(make_float3(Mf.x, Mf.y, Mf.z), ef));
    const float4 dev = make_float4(hdt * (eaf.x + q.x), hdt * (eaf.y + q.y), hdt * (eaf.z + q.z), hdt * (eaf.w + q.w));
    st4(c.ev, i, mk4(ev.x + f2d(dev.x), ev.y + f2d(dev.y), ev.z + f2d(dev.z), ev.w + f2d(dev.w)));
    if (F32)
        c.eaf[i] = q;
    else
        st4(c.ea, i, mk4(f2d(q.x), f2d(q.y), f2d(q.z), f2d(q.w)));
    const float4 evn = make_float4(evf.x + dev.x, evf.y + dev.y, evf.z + dev.z, evf.w + dev.w);
    const float4 de = make_float4(dt * evn.x + h2 * q.x, dt * evn.y + h2 * q.y, dt * evn.z + h2 * q.z,
                                  dt * evn.w + h2 * q.w);
    // |e|^2 - 1 and e.de in float pairs (e is FP64; the terms cancel to ~1e-16)
    df n2 = two_prod(e0.hi, e0.hi);
    n2 = df_add(n2, two_prod(e1.hi, e1.hi));
    n2 = df_add(n2, two_prod(e2.hi, e2.hi));
    n2 = df_add(n2, two_prod(e3.hi, e3.hi));
    n2 = df_add_f(n2, 2.f * (e0.hi * e0.lo + e1.hi * e1.lo + e2.hi * e2.lo + e3.hi * e3.lo));
    n2 = df_add_f(n2, -1.f);
    df ed = two_prod(e0.hi, de.x);
    ed = df_add(ed, two_prod(e1.hi, de.y));
    ed = df_add(ed, two_prod(e2.hi, de.z));
    ed = df_add(ed, two_prod(e3.hi, de.w));
    ed = df_add_f(ed, e0.lo * de.x + e1.lo * de.y + e2.lo * de.z + e3.lo * de.w);
    const float eps = df_f(n2) + 2.f * df_f(ed) + (de.x * de.x + de.y * de.y + de.z * de.z + de.w * de.w);
    const float kk = eps * (-0.5f + 0.375f * eps);
    const float4 dn = make_float4(de.x + kk * (ef.x + de.x), de.y + kk * (ef.y + de.y), de.z + kk * (ef.z + de.z),
                                  de.w + kk * (ef.w + de.w));
    o.e = mk4(e.x + f2d(dn.x), e.y + f2d(dn.y), e.z + f2d(dn.z), e.w + f2d(dn.w));
    st4(c.ep_next, i, o.e);
    o.ef = make_float4(ef.x + dn.x, ef.y + dn.y, ef.z + dn.z, ef.w + dn.w);
    o.ev = evn;
    o.v = vn;
    // centre
    const V3<float> inc = dt * vn + h2 * a_new;
    o.x = mk3(xi.x + f2d(inc.x), xi.y + f2d(inc.y), xi.z + f2d(inc.z));
    return o;
}

// The next step's FP32 record of sphere oid centred at X (offset from the
// grid origin, float pairs): the cell of the centre and the offset from its
// corner -- exact to ~1e-15 m and in [0, cell size), so the binning agrees
// with the offsets the neighbour loop uses -- radius (rh + rl), velocity,
// mass and spin; the key and value of the next cell sort (impl:290-302);
// and the candidate lists' displacement check.
__device__ __forceinline__ void emit_rec(const ContactLaunch& c, unsigned int oid, const df X[3], float rh, float rl,
                                         V3<float> vn, float m, float3 w, unsigned int& bits)
{
    const df csd = df{c.cs_f, c.cs_lo};
    int cell[3];
    df A[3];
    bool fin = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const df rx = X[i];
        if (!isfinite(rx.hi)) {
            fin = false;
            cell[i] = 0;
            A[i] = df{rx.hi, 0.f};
            continue;
        }
        int ci = __float2int_rd(rx.hi * c.inv_cs_f);
        df off = df_sub(rx, df_mul_f(csd, (float)ci));
        if (off.hi < 0.f) {
            ci -= 1;
            off = df_add(off, csd);
        } else {
            const df t = df_sub(off, csd);
            if (t.hi >= 0.f) {
                ci += 1;
                off = t;
            }
        }
        cell[i] = ci;
        A[i] = off;
    }
    if (!fin) bits |= XDEM_ERR_NONFINITE;
    c.k_out[oid] = grid_hash(c.prm, cell[0], cell[1], cell[2]);
    c.v_out[oid] = oid;
    float4* r = c.rec + 4 * (size_t)oid;
    r[kRecA] = make_float4(A[0].hi, A[1].hi, A[2].hi, rh);
    r[kRecL] = make_float4(A[0].lo, A[1].lo, A[2].lo, rl);
    r[kRecB] = make_float4(vn.x, vn.y, vn.z, m);
    r[kRecC] = make_float4(w.x, w.y, w.z, __uint_as_float(pack_cell(cell[0], cell[1], cell[2])));
    if (c.use_list) {
        // distance from the centre at the last list build, in the lists'
        // frame (packed cell times cell size plus the offset)
        const float4 xb = reinterpret_cast<const float4*>(c.vl_xb)[oid];
        const float dx = (float)(cell[0] & 2047) * c.cs_f + A[0].hi - xb.x;
        const float dy = (float)(cell[1] & 2047) * c.cs_f + A[1].hi - xb.y;
        const float dz = (float)(cell[2] & 1023) * c.cs_f + A[2].hi - xb.z;
        if (!(dx * dx + dy * dy + dz * dz < c.half_skin2_f)) atomicOr(c.vl_flag + kVlMoved, 1u);
    }
}

// Sphere tail: integration, the next position and the next record.
// rh + rl: the radius as the record's float pair; m: the mass in FP32.
__device__ __forceinline__ void mixed_tail(const ContactLaunch& c, unsigned int oid, d4 ip, float rh, float rl,
                                           float m, V3<float> Ff, V3<float> Mf, unsigned int& bits,
                                           const BodyIn& in)
{
    const NextBody nx = integrate_f<true>(c, oid, mk3(ip.x, ip.y, ip.z), m, Ff, Mf, !c.vel_compat, in);
    st4(c.pos_next, oid, mk4(nx.x.x, nx.x.y, nx.x.z, ip.w));
    const df X[3] = {df_sub(split_d(nx.x.x), df{c.o_hi[0], c.o_lo[0]}),
                     df_sub(split_d(nx.x.y), df{c.o_hi[1], c.o_lo[1]}),
                     df_sub(split_d(nx.x.z), df{c.o_hi[2], c.o_lo[2]})};
    emit_rec(c, oid, X, rh, rl, nx.v, m, ang_vel_f(nx.ef, nx.ev), bits);
    if (bits) atomicOr(c.status, bits);
}

// One sphere against plane k behind a call boundary: few spheres are near a
// plane, and the float-pair plane geometry needs about 50 registers more than
// the rest of the kernel, so it gets its own allocation instead of setting
// the whole kernel's.  By value in and out; the force and moment come back
// as one contact's FP32 values for the caller's compensated sums.
struct PlaneOut {
    float f[3], m[3], w[6], tm[3], rs;
    unsigned int cnt, bits;
    int touched;
};
__device__ __noinline__ PlaneOut plane_call(const ContactLaunch* cp, unsigned int k, unsigned int kbeg,
                                            unsigned int oid, d4 ip, float4 Bi, float4 Ci, unsigned int cnt)
{
    Acc a;
    a.tm = v3<float>(0.f, 0.f, 0.f);
    a.rs = 0.f;
    float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    PlaneOut o;
    o.bits = 0;
    o.cnt = cnt;
    o.touched = plane_mixed(*cp, k, kbeg, oid, ip, v3<float>(Bi.x, Bi.y, Bi.z), v3<float>(Ci.x, Ci.y, Ci.z), Bi.w,
                            o.cnt, a, f6, o.bits);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o.f[i] = a.f[i].value();
        o.m[i] = a.m[i].value();
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) o.w[i] = f6[i];
    o.tm[0] = a.tm.x; o.tm[1] = a.tm.y; o.tm[2] = a.tm.z;
    o.rs = a.rs;
    return o;
}

// One sphere against cylinder k (impl:1083-1601, as the launcher kernel
// k_cylinder runs it): the FP64 regions of cylinder_detection (side, wall
// annulus, rim) and, for a sphere inside, the cap it faces (pair id + 1000);
// FP32 forces with the body's mass left out of the effective mass.  Both
// passes look their history up in the slots as they were before this
// cylinder wrote (the launcher kernel's per-launch copy); cylinder 0
// restarts the list, later ones append (impl:1172-1174), bounded by
// MAX_P2CY_COUNT.  Returns true when the sphere touched the cylinder.
__device__ __forceinline__ bool cylinder_mixed(const ContactLaunch& c, unsigned int k, unsigned int oid, d4 ip,
                                               V3<float> ivel, V3<float> iom, float im, unsigned int& cy_cnt,
                                               Acc& acc, float f6[6], unsigned int& bits)
{
    const device_dem_parameters& p = c.prm;
    const device_cylinder_info& cy = c.cyl[k];
    const unsigned int bidx = c.nplane + k;
    const double* bi = c.body + 15 * bidx;
    const MatR<float> mr = matr(c.mpf[c.nscene + bidx]);
    const unsigned int sid = oid * MAX_P2CY_COUNT;
    unsigned int old_id[MAX_P2CY_COUNT];
    double2 old_t[MAX_P2CY_COUNT];
    for (unsigned int q = 0; q < MAX_P2CY_COUNT; ++q) {
        old_id[q] = c.cy_id[sid + q];
        old_t[q] = reinterpret_cast<const double2*>(c.cy_tsd)[sid + q];
    }
    const unsigned int old_cnt = cy_cnt;
    if (cy.id == 0) cy_cnt = 0;
    const d3 ipos = mk3(ip.x, ip.y, ip.z);
    const double r = ip.w;
    bool inner = false;
    d3 unit = mk3(0, 0, 0);
    double cdist = cylinder_detection(cy, bi, ipos, unit, r, inner);
    d3 cpt = ipos + r * unit;
    const BodyF b = load_body_f(bi);
    const float rf = d2f_rn(r);
    bool touched = false;
    for (int pass = 0; pass < 2; ++pass) {
        const unsigned int pid = pass ? cy.id + 1000u : cy.id;
        if (pass) {
            if (!inner) break;
            cdist = cylinder_inner_cap(cy, bi, ipos, unit, cpt, cy.empty_part, r);
        }
        if (!(cdist > 0)) continue;
        float sd0 = 0.f, sd1 = 0.f;
        for (unsigned int q = 0; q < old_cnt && q < MAX_P2CY_COUNT; ++q)
            if (old_id[q] == pid) {
                sd0 = d2f_rn(old_t[q].x);
                sd1 = d2f_rn(old_t[q].y);
                break;
            }
        const V3<float> un = v3<float>(d2f_rn(unit.x), d2f_rn(unit.y), d2f_rn(unit.z));
        // lever arms: contact point from the body's reference point and from
        // the sphere's centre (r un for the side and for the inner cap)
        const V3<float> po2cp = v3<float>(d2f_rn(cpt.x - bi[XDEM_PX]), d2f_rn(cpt.y - bi[XDEM_PY]),
                                          d2f_rn(cpt.z - bi[XDEM_PZ]));
        const V3<float> rc = rf * un;
        const V3<float> dv = (b.v + tcross(b.om, po2cp)) - (ivel + tcross(iom, rc));
        const FC<float> fc = fconst_f(mr, p.contact_model, rf, 0.f, im, 0.f);
        V3<float> Ft = v3<float>(0, 0, 0), Fn = v3<float>(0, 0, 0);
        model_f(p.contact_model, fc, c.dt_f, d2f_rn(cdist), sd0, sd1, dv, un, Ft, Fn, 0.f);
        const V3<float> mf = Fn + Ft;
        const V3<float> mm = rf * tcross(un, Ft);  // rc parallel to Fn: only Ft turns the sphere
        acc.f[0].add(mf.x); acc.f[1].add(mf.y); acc.f[2].add(mf.z);
        acc.m[0].add(mm.x); acc.m[1].add(mm.y); acc.m[2].add(mm.z);
        if (c.rolling) {
            acc.tm = acc.tm + mm;
            acc.rs += rf * mr.rfric * tlen(Fn);
        }
        const V3<float> bm = tcross(po2cp, mf);
        f6[0] -= mf.x; f6[1] -= mf.y; f6[2] -= mf.z;
        f6[3] -= bm.x; f6[4] -= bm.y; f6[5] -= bm.z;
        if (cy_cnt < MAX_P2CY_COUNT) {
            c.cy_id[sid + cy_cnt] = pid;
            reinterpret_cast<double2*>(c.cy_tsd)[sid + cy_cnt] = make_double2(f2d(sd0), f2d(sd1));
            cy_cnt++;
        } else {
            bits |= XDEM_ERR_P2CY_OVERFLOW;
        }
        touched = true;
    }
    return touched;
}
// ... behind a call boundary, by value in and out like plane_call (the FP64
// region geometry and its transcendentals run for the few spheres near a
// cylinder).
__device__ __noinline__ PlaneOut cyl_call(const ContactLaunch* cp, unsigned int k, unsigned int oid, d4 ip, float4 Bi,
                                          float4 Ci, unsigned int cnt)
{
    Acc a;
    a.tm = v3<float>(0.f, 0.f, 0.f);
    a.rs = 0.f;
    float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    PlaneOut o;
    o.bits = 0;
    o.cnt = cnt;
    o.touched = cylinder_mixed(*cp, k, oid, ip, v3<float>(Bi.x, Bi.y, Bi.z), v3<float>(Ci.x, Ci.y, Ci.z), Bi.w, o.cnt,
                               a, f6, o.bits);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o.f[i] = a.f[i].value();
        o.m[i] = a.m[i].value();
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) o.w[i] = f6[i];
    o.tm[0] = a.tm.x; o.tm[1] = a.tm.y; o.tm[2] = a.tm.z;
    o.rs = a.rs;
    return o;
}

// One sphere against mesh m behind a call boundary (few spheres are near a
// mesh, and the triangle search holds three candidate arrays): the same
// value-in, value-out form as plane_call.  Both pair kernels go through it,
// so the walk and the candidate-list forms sum mesh contacts alike.
struct MeshOut {
    float f[3], m[3], w[6], tm[3], rs;
    unsigned int bits;
    int touched;
};
__device__ __noinline__ MeshOut mesh_call(const ContactLaunch* cp, unsigned int m, unsigned int oid, unsigned int gx,
                                          unsigned int gy, unsigned int gz, d4 ip, float4 Bi, float4 Ci)
{
    Acc a;
    a.tm = v3<float>(0.f, 0.f, 0.f);
    a.rs = 0.f;
    float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    MeshOut o;
    o.bits = 0;
    o.touched = mesh_mixed(*cp, m, oid, gx, gy, gz, ip, v3<float>(Bi.x, Bi.y, Bi.z), v3<float>(Ci.x, Ci.y, Ci.z),
                           Bi.w, a, f6, o.bits);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o.f[i] = a.f[i].value();
        o.m[i] = a.m[i].value();
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) o.w[i] = f6[i];
    o.tm[0] = a.tm.x; o.tm[1] = a.tm.y; o.tm[2] = a.tm.z;
    o.rs = a.rs;
    return o;
}

// Sphere (centre ip, radius ip.w) against the meshes, in mesh order: a mesh
// whose bounding sphere the sphere cannot reach (c.mesh_bs: centre relative
// to the grid origin, radius with the FP32 slack) holds no contact of it, so
// only its pair count is written (0, as the search would leave it); the rest
// search the grid for triangles.  Every thread of the block takes part (the
// body wrench partials are block sums).
__device__ __forceinline__ void meshes_mixed(const ContactLaunch& c, bool live, unsigned int oid, unsigned int gx,
                                             unsigned int gy, unsigned int gz, d4 ip, float4 Bi, float4 Ci,
                                             Acc& acc, unsigned int& bits, float* smf)
{
    const float xf = d2f_rn(ip.x) - c.o_hi[0], yf = d2f_rn(ip.y) - c.o_hi[1], zf = d2f_rn(ip.z) - c.o_hi[2];
    const float rf = d2f_rn(ip.w);
    for (unsigned int m = 0; m < c.nmesh; ++m) {
        float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool touched = false;
        if (live) {
            const float4 b = c.mesh_bs[m];
            const float dx = xf - b.x, dy = yf - b.y, dz = zf - b.z, lim = b.w + rf;
            if (dx * dx + dy * dy + dz * dz <= lim * lim) {
                const MeshOut o = mesh_call(&c, m, oid, gx, gy, gz, ip, Bi, Ci);
                bits |= o.bits;
                if (o.touched) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        acc.f[i].add(o.f[i]);
                        acc.m[i].add(o.m[i]);
                    }
#pragma unroll
                    for (int i = 0; i < 6; ++i) f6[i] = o.w[i];
                    acc.tm = acc.tm + v3<float>(o.tm[0], o.tm[1], o.tm[2]);
                    acc.rs += o.rs;
                    touched = true;
                }
            } else {
                c.ms_count[oid] = 0u;
            }
        }
        emit_body_f(f6, touched, c.bsums + ((size_t)(c.mesh_body[m]) * c.nblocks + blockIdx.x) * 6, smf);
    }
}

// Kernel 1 of the mixed step: one thread per cell-sorted entry, particle-
// particle contact (and triangle meshes, which need the grid too).  Writes
// the sphere's force, moment and rolling sums (original order) for kernel 2.
// It holds no plane or integration state, so it runs at twice the occupancy
// of a kernel doing all of it -- the stencil walk is latency-bound.
// NT threads per block, OCC / NT blocks per SM (OCC 768: 80 registers a
// thread, 1024: 64).
template <bool MESH, unsigned int NT, unsigned int STAGE, unsigned int OCC>
__global__ void __launch_bounds__(NT, OCC / NT) k_mixed_pairs(const __grid_constant__ ContactLaunch c)
{
    __shared__ float smf[(NT / 32) * 6 * 2];
    __shared__ unsigned int stage[STAGE * NT];                // p2p candidates, [slot][thread]
    __shared__ unsigned int old_id[MAX_P2P_COUNT * NT];       // old pair list, [slot][thread]
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int oid = 0xffffffffu;
    if (s < c.nentry) oid = c.sorted_index[s];
    const bool live = oid < c.np;
    const device_dem_parameters& p = c.prm;

    float4 Ai = make_float4(0.f, 0.f, 0.f, 0.f), Li = Ai, Bi = Ai, Ci = Ai;
    unsigned int Ti = 0, gx = 0, gy = 0, gz = 0;
    if (live) {
        Ai = reinterpret_cast<const float4*>(c.mA)[s];
        Li = reinterpret_cast<const float4*>(c.mL)[s];
        Ti = reinterpret_cast<const uint2*>(c.mIT)[s].y;
        Bi = reinterpret_cast<const float4*>(c.mB)[s];
        Ci = reinterpret_cast<const float4*>(c.mC)[s];
        const unsigned int key = c.skey[s];
        // (z * gy + y) * gx + x with power-of-two extents
        const unsigned int shx = __ffs(p.grid_size.x) - 1, shxy = shx + __ffs(p.grid_size.y) - 1;
        gx = key & (p.grid_size.x - 1);
        gy = (key >> shx) & (p.grid_size.y - 1);
        gz = key >> shxy;
    }
    Acc acc;
    acc.tm = v3<float>(0.f, 0.f, 0.f);
    acc.rs = 0.f;
    unsigned int bits = 0;
    const V3<float> ivel = v3<float>(Bi.x, Bi.y, Bi.z);
    const V3<float> iom = v3<float>(Ci.x, Ci.y, Ci.z);

    // ------------------------------------------------ particle-particle (impl:613-733)
    if (live && c.has_pp)
        p2p_mixed<NT, STAGE>(c, oid, gx, gy, gz, Ai, Li, Ti, Bi, Ci, stage + threadIdx.x, old_id + threadIdx.x, acc,
                             bits);

    // ------------------------------------------------ triangle meshes (impl:1930-2109)
    if (MESH) {
        d4 ip = mk4(0, 0, 0, 0);
        if (live) ip = ld4(c.pos_cur, oid);
        meshes_mixed(c, live, oid, gx, gy, gz, ip, Bi, Ci, acc, bits, smf);
    }
    if (!live) return;
    reinterpret_cast<float4*>(c.fA)[oid] = make_float4(acc.f[0].value(), acc.f[1].value(), acc.f[2].value(), acc.rs);
    reinterpret_cast<float4*>(c.fB)[oid] = make_float4(acc.m[0].value(), acc.m[1].value(), acc.m[2].value(), 0.f);
    if (c.rolling) reinterpret_cast<float4*>(c.fC)[oid] = make_float4(acc.tm.x, acc.tm.y, acc.tm.z, 0.f);
    if (bits) atomicOr(c.status, bits);
}

// Kernel 1 with candidate lists: one thread per sphere in original order.
// On a rebuild step every sphere walks the stencil and records its list;
// otherwise its contacts come from the list (a sphere whose list overflowed
// walks; the cell sort is kept up to date for it).  Writes the same sums as
// k_mixed_pairs for kernel 2.
// The stencil walk of the sphere list kernel (rebuild steps, and spheres
// whose list overflowed) behind a call boundary: inlined, its staged-row loads set the
// register allocation of the whole kernel and the list path spilled inside
// its per-contact loop.  Apart, the list path keeps its own allocation and
// the walk pays the call on the steps that need it.  Starts from empty sums
// and returns them by value, like plane_call.  Its unit
// (xdem_fused_mixed.cu) is compiled without implicit FMA contraction, so the
// call computes the same bits as the walk inlined in k_mixed_pairs.
struct WalkOut {
    Acc acc;
    unsigned int bits;
};
template <unsigned int NT>
__device__ __noinline__ WalkOut walk_call(const ContactLaunch* cp, unsigned int oid, unsigned int gx, unsigned int gy,
                                          unsigned int gz, float4 Ai, float4 Li, unsigned int Ti, float4 Bi, float4 Ci,
                                          unsigned int* stage, unsigned int* old_id, bool rebuild)
{
    WalkOut o;
    o.acc.tm = v3<float>(0.f, 0.f, 0.f);
    o.acc.rs = 0.f;
    o.bits = 0;
    p2p_mixed<NT, 16>(*cp, oid, gx, gy, gz, Ai, Li, Ti, Bi, Ci, stage, old_id, o.acc, o.bits, rebuild);
    return o;
}

// Block bx of the list pair kernel (spheres bx * NT ...).  stage: walk
// fallback candidates or the list's sort keys, old_id: the old pair list,
// both [slot][thread] with stride NT (kListCap and MAX_P2P_COUNT slots);
// smf: the mesh wrench partials.  Meshes write their rows at blockIdx.x, so
// with meshes bx must be blockIdx.x.
template <bool MESH, unsigned int NT>
__device__ __forceinline__ void pairs_list_block(const ContactLaunch& c, unsigned int bx, unsigned int* stage,
                                                 unsigned int* old_id, float* smf)
{
    const bool rebuild = c.vl_flag[kVlRebuild] != 0u;
    const unsigned int oid = bx * NT + threadIdx.x;
    const bool live = oid < c.np;
    if (!MESH && !live) return;
    float4 Ai = make_float4(0.f, 0.f, 0.f, 0.f), Li = Ai, Bi = Ai, Ci = Ai;
    if (live) {
        const float4* r = c.rec + 4 * (size_t)oid;
        Ai = r[kRecA]; Li = r[kRecL]; Bi = r[kRecB]; Ci = r[kRecC];
    }
    const unsigned int Ti = rec_cell(Ci);
    const device_dem_parameters& p = c.prm;
    const unsigned int gx = (Ti & 2047u) & (p.grid_size.x - 1), gy = ((Ti >> 11) & 2047u) & (p.grid_size.y - 1);
    const unsigned int gz = (Ti >> 22) & (p.grid_size.z - 1);
    Acc acc;
    acc.tm = v3<float>(0.f, 0.f, 0.f);
    acc.rs = 0.f;
    unsigned int bits = 0;
    if (live) {
        if (!rebuild && c.vl_cnt[oid] <= kListCap) {
            p2p_list<NT>(c, oid, Ai, Li, Ti, Bi, Ci, old_id + threadIdx.x, stage + threadIdx.x, acc, bits);
        } else if constexpr (MESH) {
            // the mesh form's unit contracts multiply-adds: the walk stays
            // inline, in the same context as in k_mixed_pairs
            p2p_mixed<NT, 16>(c, oid, gx, gy, gz, Ai, Li, Ti, Bi, Ci, stage + threadIdx.x, old_id + threadIdx.x, acc,
                              bits, rebuild);
        } else {
            // acc is still empty here: the walk's sums are the sphere's
            const WalkOut w = walk_call<NT>(&c, oid, gx, gy, gz, Ai, Li, Ti, Bi, Ci, stage + threadIdx.x,
                                            old_id + threadIdx.x, rebuild);
            acc = w.acc;
            bits |= w.bits;
        }
    }
    // triangle meshes (impl:1930-2109): the cell table holds the mesh
    // spheres as of the last sort, and a moved mesh forces a sort
    if (MESH) {
        d4 ip = mk4(0, 0, 0, 0);
        if (live) ip = ld4(c.pos_cur, oid);
        meshes_mixed(c, live, oid, gx, gy, gz, ip, Bi, Ci, acc, bits, smf);
    }
    if (!live) return;
    reinterpret_cast<float4*>(c.fA)[oid] = make_float4(acc.f[0].value(), acc.f[1].value(), acc.f[2].value(), acc.rs);
    reinterpret_cast<float4*>(c.fB)[oid] = make_float4(acc.m[0].value(), acc.m[1].value(), acc.m[2].value(), 0.f);
    if (c.rolling) reinterpret_cast<float4*>(c.fC)[oid] = make_float4(acc.tm.x, acc.tm.y, acc.tm.z, 0.f);
    if (bits) atomicOr(c.status, bits);
}

template <bool MESH, unsigned int NT, unsigned int OCC>
__global__ void __launch_bounds__(NT, OCC / NT) k_mixed_pairs_list(const __grid_constant__ ContactLaunch c)
{
    __shared__ float smf[MESH ? (NT / 32) * 6 * 2 : 1];
    __shared__ unsigned int stage[kListCap * NT];
    __shared__ unsigned int old_id[MAX_P2P_COUNT * NT];
    pairs_list_block<MESH, NT>(c, blockIdx.x, stage, old_id, smf);
}

// After kernel 2: this step's "moved too far" flag becomes the next step's
// rebuild flag (a rebuild also clears the overflow mark its build will
// set again if needed), and the next step's sort is needed on a rebuild or
// while a list overflowed.
__device__ __forceinline__ void vl_roll(unsigned int* flag)
{
    const unsigned int moved = flag[kVlMoved];
    flag[kVlRebuild] = moved;
    if (moved) {
        flag[kVlCount] += 1u;
        flag[kVlOverflow] = 0u;
    }
    flag[kVlSort] = moved | flag[kVlOverflow];
    flag[kVlMoved] = 0u;
}
__global__ void k_vl_roll(unsigned int* flag) { vl_roll(flag); }

// Kernel 2 of the mixed step: one thread per sphere in original order, so
// every state array is read and written coalesced.  Plane contact (planes in
// id order), rolling resistance, the velocity and position update and the
// next step's records, on top of kernel 1's particle-particle sums.
// OCC / NT blocks per SM (OCC 512: 128 registers a thread, 768: 80, 1024: 64).
// The sphere body kernel's cylinder loop behind a call boundary: its vote,
// FP64 region calls and wrench rows would otherwise raise the register
// allocation of the whole kernel, also for scenes without cylinders.  The
// caller's running sums come in and go out by value, so every addition
// happens in the same order as inline.  Every lane of the warp calls it.
struct CylsOut {
    Acc acc;
    unsigned int bits;
    float4 Bi, Ci;
    int have_bc;
};
template <unsigned int NT>
__device__ __noinline__ CylsOut cylinders_call(const ContactLaunch* cp, unsigned int oid, bool live, d4 ip, float rh,
                                               float4 Bi, float4 Ci, bool have_bc, Acc acc, unsigned int bits)
{
    const ContactLaunch& c = *cp;
    auto need_bc = [&]() {
        if (have_bc) return;
        const float4* r = c.rec + 4 * (size_t)oid;
        Bi = r[kRecB];
        Ci = r[kRecC];
        have_bc = true;
    };
    unsigned int cy_cnt = live ? c.cy_count[oid] : 0u;
    const unsigned int wrow = oid >> 5;  // oid = block * NT + thread
    const bool has_row = wrow < (c.nentry + 31u) / 32u;
    float3 xf = make_float3(0.f, 0.f, 0.f);
    if (live) xf = make_float3(d2f_rn(ip.x) - c.o_hi[0], d2f_rn(ip.y) - c.o_hi[1], d2f_rn(ip.z) - c.o_hi[2]);
    for (unsigned int k = 0; k < c.ncyl; ++k) {
        float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool touched = false;
        bool near = false;
        if (live) {
            // conservative FP32 test: every region lies within the sphere
            // around the middle of the axis through the rims and the wall
            const device_cylinder_info& cy = c.cyl[k];
            const double* bi = c.body + 15 * (c.nplane + k);
            const float4 e = make_float4(d2f_rn(bi[XDEM_E0]), d2f_rn(bi[XDEM_E1]), d2f_rn(bi[XDEM_E2]),
                                         d2f_rn(bi[XDEM_E3]));
            const float hx = 0.5f * (float)(cy.pbase.x + cy.ptop.x), hy = 0.5f * (float)(cy.pbase.y + cy.ptop.y),
                        hz = 0.5f * (float)(cy.pbase.z + cy.ptop.z);
            const float ax = (float)(cy.ptop.x - cy.pbase.x), ay = (float)(cy.ptop.y - cy.pbase.y),
                        az = (float)(cy.ptop.z - cy.pbase.z);
            const float half = 0.5f * sqrtf(ax * ax + ay * ay + az * az) + (float)cy.thickness;
            const float rad = fmaxf((float)cy.len_rr.y, (float)cy.len_rr.z) + (float)cy.thickness;
            const float3 m = to_global_f(make_float3(hx, hy, hz), e);
            const float dx = xf.x - (d2f_rn(bi[XDEM_PX]) - c.o_hi[0] + m.x);
            const float dy = xf.y - (d2f_rn(bi[XDEM_PY]) - c.o_hi[1] + m.y);
            const float dz = xf.z - (d2f_rn(bi[XDEM_PZ]) - c.o_hi[2] + m.z);
            const float lim = sqrtf(half * half + rad * rad) * (1.f + 1e-5f) + rh + c.margin;
            near = dx * dx + dy * dy + dz * dz <= lim * lim;
        }
        if (near) {
            need_bc();
            const PlaneOut o = cyl_call(&c, k, oid, ip, Bi, Ci, cy_cnt);
            touched = o.touched != 0;
            cy_cnt = o.cnt;
            bits |= o.bits;
            if (touched) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    acc.f[i].add(o.f[i]);
                    acc.m[i].add(o.m[i]);
                }
#pragma unroll
                for (int i = 0; i < 6; ++i) f6[i] = o.w[i];
                acc.tm = acc.tm + v3<float>(o.tm[0], o.tm[1], o.tm[2]);
                acc.rs += o.rs;
            }
        } else if (live && c.cyl[k].id == 0) {
            cy_cnt = 0;  // cylinder 0 restarts the list whether or not it is touched
        }
        if (has_row) emit_warp_f(f6, touched, c.bsums + ((size_t)(c.nplane + k) * c.nblocks + wrow) * 6);
    }
    if (live) c.cy_count[oid] = cy_cnt;
    CylsOut o;
    o.acc = acc;
    o.bits = bits;
    o.Bi = Bi;
    o.Ci = Ci;
    o.have_bc = have_bc ? 1 : 0;
    return o;
}

// Block bx of the sphere body kernel (spheres bx * NT ...).
template <unsigned int NT>
__device__ __forceinline__ void bodies_block(const ContactLaunch& c, unsigned int bx)
{
    const unsigned int oid = bx * NT + threadIdx.x;
    const bool live = oid < c.np;
    // the record's velocity + mass (B) and spin (C) are read only by a sphere
    // that meets a plane or has rolling resistance (one 32-byte sector); the
    // radius and mass come from the FP64 state, rounded as the record holds them
    float4 Bi = make_float4(0.f, 0.f, 0.f, 0.f), Ci = Bi;
    bool have_bc = false;
    auto need_bc = [&]() {
        if (have_bc) return;
        const float4* r = c.rec + 4 * (size_t)oid;
        Bi = r[kRecB];
        Ci = r[kRecC];
        have_bc = true;
    };
    d4 ip = mk4(0, 0, 0, 0);
    float rh = 0.f;
    Acc acc;
    acc.tm = v3<float>(0.f, 0.f, 0.f);
    acc.rs = 0.f;
    if (live) {
        ip = ld4(c.pos_cur, oid);
        rh = d2f_rn(ip.w);
        const float4 fa = reinterpret_cast<const float4*>(c.fA)[oid];
        const float4 fb = reinterpret_cast<const float4*>(c.fB)[oid];
        acc.f[0].hi = fa.x; acc.f[1].hi = fa.y; acc.f[2].hi = fa.z;
        acc.m[0].hi = fb.x; acc.m[1].hi = fb.y; acc.m[2].hi = fb.z;
        acc.rs = fa.w;
        if (c.rolling) {
            const float4 fc = reinterpret_cast<const float4*>(c.fC)[oid];
            acc.tm = v3<float>(fc.x, fc.y, fc.z);
        }
    }
    unsigned int bits = 0;

    // ------------------------------------------------ planes in id order (impl:950-1080)
    if (c.nplane) {
        float4 ipf = make_float4(0.f, 0.f, 0.f, -1.f);
        if (live)
            ipf = make_float4(d2f_rn(ip.x) - c.o_hi[0], d2f_rn(ip.y) - c.o_hi[1], d2f_rn(ip.z) - c.o_hi[2], rh);
        unsigned int pl_cnt = 0;
        // a batched scene sees only its own planes and keeps no wrenches (no
        // block reduction, so threads may walk different plane ranges)
        const bool batched = c.scene_plane_first != nullptr;
        const unsigned int scene = live ? scene_index(c, oid) : 0u;
        const unsigned int kbeg = batched ? c.scene_plane_first[scene] : 0u;
        const unsigned int kend = batched ? (live ? c.scene_plane_first[scene + 1] : kbeg) : c.nplane;
        // conservative FP32 test: every region of the plane test needs the
        // centre within r of the plane and of the rectangle's extent
        auto near_plane = [&](unsigned int k) {
            if (c.planedf[k].coh) return true;
            const PlaneF& pf = c.planef[k];
            const float dx = ipf.x - pf.v[0], dy = ipf.y - pf.v[1], dz = ipf.z - pf.v[2];
            const float wx = dx * pf.v[3] + dy * pf.v[4] + dz * pf.v[5];
            const float wy = dx * pf.v[6] + dy * pf.v[7] + dz * pf.v[8];
            const float wz = dx * pf.v[9] + dy * pf.v[10] + dz * pf.v[11];
            const float lim = ipf.w + c.margin;
            return fabsf(wz) <= lim && wx >= -lim && wx <= pf.v[12] + lim && wy >= -lim && wy <= pf.v[13] + lim;
        };
        // wrench partials: one row per warp (no block barrier in the loop);
        // the rows cover ceil(nentry / 32) warps, so a warp made only of the
        // last block's padding threads has no row and writes none
        const unsigned int wrow = oid >> 5;
        const bool has_row = wrow < (c.nentry + 31u) / 32u;
        for (unsigned int k = kbeg; k < kend; ++k) {
            float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            bool touched = false;
            const bool near = !live || near_plane(k);
            if (live && near) {
                need_bc();
                const PlaneOut o = plane_call(&c, k, kbeg, oid, ip, Bi, Ci, pl_cnt);
                touched = o.touched != 0;
                pl_cnt = o.cnt;
                bits |= o.bits;
                if (touched) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        acc.f[i].add(o.f[i]);
                        acc.m[i].add(o.m[i]);
                    }
#pragma unroll
                    for (int i = 0; i < 6; ++i) f6[i] = o.w[i];
                    acc.tm = acc.tm + v3<float>(o.tm[0], o.tm[1], o.tm[2]);
                    acc.rs += o.rs;
                }
            }
            if (!batched && has_row) emit_warp_f(f6, touched, c.bsums + ((size_t)k * c.nblocks + wrow) * 6);
        }
        if (live) c.pl_count[oid] = pl_cnt;
    }

    // ------------------------------------------------ cylinders in id order (impl:1083-1601)
    if (c.ncyl) {
        const CylsOut co = cylinders_call<NT>(&c, oid, live, ip, rh, Bi, Ci, have_bc, acc, bits);
        acc = co.acc;
        bits = co.bits;
        Bi = co.Bi;
        Ci = co.Ci;
        have_bc = co.have_bc != 0;
    }

    if (!live) return;

    // ------------------------------------------------ rolling resistance (impl:2420-2454)
    V3<float> Mf = v3<float>(acc.m[0].value(), acc.m[1].value(), acc.m[2].value());
    if (acc.rs != 0.f) {
        need_bc();
        const V3<float> iom = v3<float>(Ci.x, Ci.y, Ci.z);
        // the flat entry oid as impl:2434 reads it, or the sphere's own
        const float J = d2f_rn(c.rolling_per_sphere ? c.inertia[3 * (size_t)oid] : c.inertia[oid]);
        const V3<float> T = (J * c.dt_f) * iom - acc.tm;
        const float lT2 = tdot(T, T);
        const float lT = lT2 == 0.f ? 0.f : sqrtf(lT2);
        if (lT != 0.f) {
            V3<float> Tr3 = acc.rs * (T / lT);
            if (tlen(Tr3) >= lT) Tr3 = T;
            Mf = Mf + Tr3;
        }
    }
    const V3<float> Ff = v3<float>(acc.f[0].value(), acc.f[1].value(), acc.f[2].value());
    float m;
    const BodyIn in = body_in_f32(c, oid, m);
    mixed_tail(c, oid, ip, rh, d2f_rn(ip.w - f2d(rh)), m, Ff, Mf, bits, in);
}

template <unsigned int NT, unsigned int OCC>
__global__ void __launch_bounds__(NT, OCC / NT) k_mixed_bodies(const __grid_constant__ ContactLaunch c)
{
    bodies_block<NT>(c, blockIdx.x);
}

// The cluster body kernel's cylinder loop behind a call boundary (its
// geometry would otherwise raise the allocation of the whole kernel, also
// for scenes without cylinders).  Each member against each cylinder with its
// cluster's mass, velocity and spin, as k_cylinder<true> (xdem_kernels.cu):
// the member's rigid velocity vc + om x d makes the contact-point velocity
// vc + om x (cpt - x_c), and m + d x f is the moment about the cluster
// centre.  A member's count carries over from cylinder to cylinder;
// cylinder 0 restarts it.  The cluster's running sums come in and go out by
// value, so every addition happens in the same order as inline.  Every
// thread of the block calls it (block wrench rows).
struct ClusterSums {
    CSum F[3], M[3];
    unsigned int bits;
};
__device__ __noinline__ ClusterSums cluster_cylinders_call(const ContactLaunch* cp, unsigned int cid, bool live, d4 xc,
                                                           V3<float> vc, V3<float> om, float m, ClusterSums acc,
                                                           float* smf)
{
    const ContactLaunch& c = *cp;
    const unsigned int ne = c.cl.neach;
    const df xcd[3] = {split_d(xc.x), split_d(xc.y), split_d(xc.z)};
    for (unsigned int k = 0; k < c.ncyl; ++k) {
        float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool touched = false;
        const device_cylinder_info& cy = c.cyl[k];
        const double* bi = c.body + 15 * (c.nplane + k);
        for (unsigned int j = 0; live && j < ne; ++j) {
            const unsigned int id = cid * ne + j;
            const d4 ip = ld4(c.pos_cur, id);
            unsigned int cnt = c.cy_count[id];
            // conservative FP32 test: every region lies within the sphere
            // around the middle of the axis through the rims and the wall
            const float4 e = make_float4(d2f_rn(bi[XDEM_E0]), d2f_rn(bi[XDEM_E1]), d2f_rn(bi[XDEM_E2]),
                                         d2f_rn(bi[XDEM_E3]));
            const float hx = 0.5f * (float)(cy.pbase.x + cy.ptop.x), hy = 0.5f * (float)(cy.pbase.y + cy.ptop.y),
                        hz = 0.5f * (float)(cy.pbase.z + cy.ptop.z);
            const float ax = (float)(cy.ptop.x - cy.pbase.x), ay = (float)(cy.ptop.y - cy.pbase.y),
                        az = (float)(cy.ptop.z - cy.pbase.z);
            const float half = 0.5f * sqrtf(ax * ax + ay * ay + az * az) + (float)cy.thickness;
            const float rad = fmaxf((float)cy.len_rr.y, (float)cy.len_rr.z) + (float)cy.thickness;
            const float3 mid = to_global_f(make_float3(hx, hy, hz), e);
            const float dx = (d2f_rn(ip.x) - c.o_hi[0]) - (d2f_rn(bi[XDEM_PX]) - c.o_hi[0] + mid.x);
            const float dy = (d2f_rn(ip.y) - c.o_hi[1]) - (d2f_rn(bi[XDEM_PY]) - c.o_hi[1] + mid.y);
            const float dz = (d2f_rn(ip.z) - c.o_hi[2]) - (d2f_rn(bi[XDEM_PZ]) - c.o_hi[2] + mid.z);
            const float lim = sqrtf(half * half + rad * rad) * (1.f + 1e-5f) + d2f_rn(ip.w) + c.margin;
            if (dx * dx + dy * dy + dz * dz <= lim * lim) {
                const V3<float> d = v3<float>(df_f(df_sub(split_d(ip.x), xcd[0])), df_f(df_sub(split_d(ip.y), xcd[1])),
                                              df_f(df_sub(split_d(ip.z), xcd[2])));
                const V3<float> vm = vc + tcross(om, d);
                const PlaneOut o = cyl_call(&c, k, id, ip, make_float4(vm.x, vm.y, vm.z, m),
                                            make_float4(om.x, om.y, om.z, 0.f), cnt);
                acc.bits |= o.bits;
                cnt = o.cnt;
                if (o.touched) {
                    const V3<float> f = v3<float>(o.f[0], o.f[1], o.f[2]);
                    const V3<float> t = v3<float>(o.m[0], o.m[1], o.m[2]) + tcross(d, f);
                    acc.F[0].add(f.x); acc.F[1].add(f.y); acc.F[2].add(f.z);
                    acc.M[0].add(t.x); acc.M[1].add(t.y); acc.M[2].add(t.z);
#pragma unroll
                    for (int q = 0; q < 6; ++q) f6[q] += o.w[q];
                    touched = true;
                }
            } else if (cy.id == 0) {
                cnt = 0;  // cylinder 0 restarts the list whether or not it is touched
            }
            c.cy_count[id] = cnt;
        }
        emit_body_f(f6, touched, c.bsums + ((size_t)(c.nplane + k) * c.nblocks + blockIdx.x) * 6, smf);
    }
    return acc;
}

// Kernel 2 for clusters (impl:817-948, 224-287, 149-190): one thread per
// cluster.  The cluster's force is the sum of its members' particle-pair and
// plane forces, its moment the sum of the members' moments about their
// centres plus (x_m - x_c) x F_m, so the moment is taken about the cluster
// centre as impl:485-611 and 817-948 take it.  Then the velocity update and
// the next centre and Euler parameters, and for each member its next centre
// x_c + A(e) rloc -- formed in float pairs, so a member sits on its cluster
// to ~1e-15 m -- and its next record.  Members' plane slots follow the
// sphere rule, the count kept in pl_count between planes.
template <unsigned int NT, unsigned int OCC>
__global__ void __launch_bounds__(NT, OCC / NT) k_mixed_cluster_bodies(const __grid_constant__ ContactLaunch c)
{
    __shared__ float smf[(NT / 32) * 6 * 2];
    const unsigned int cid = blockIdx.x * NT + threadIdx.x;
    const bool live = cid < c.cl.ns;
    const unsigned int ne = c.cl.neach;
    d4 xc = mk4(0, 0, 0, 0);
    V3<float> vc = v3<float>(0.f, 0.f, 0.f), om = vc;
    float m = 1.f;
    if (live) {
        xc = ld4(c.cpos_cur, cid);
        vc = vf(d2f3(ld3(c.vel, cid)));
        om = vf(ang_vel_f(d2f4(ld4(c.ep_cur, cid)), d2f4(ld4(c.ev, cid))));
        m = d2f_rn(c.mass[cid]);
    }
    const df xcd[3] = {split_d(xc.x), split_d(xc.y), split_d(xc.z)};
    CSum F[3], M[3];
    unsigned int bits = 0;
    // lever arm of member j about the cluster centre (FP32)
    auto arm = [&](d4 ip) {
        return v3<float>(df_f(df_sub(split_d(ip.x), xcd[0])), df_f(df_sub(split_d(ip.y), xcd[1])),
                         df_f(df_sub(split_d(ip.z), xcd[2])));
    };
    auto add_member = [&](V3<float> d, V3<float> f, V3<float> mm) {
        const V3<float> t = mm + tcross(d, f);
        F[0].add(f.x); F[1].add(f.y); F[2].add(f.z);
        M[0].add(t.x); M[1].add(t.y); M[2].add(t.z);
    };

    // ------------------------------------------------ planes in id order (impl:817-948)
    if (c.nplane) {
        for (unsigned int k = 0; k < c.nplane; ++k) {
            float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            bool touched = false;
            for (unsigned int j = 0; live && j < ne; ++j) {
                const unsigned int id = cid * ne + j;
                if (k == 0) c.pl_count[id] = 0u;  // the first plane restarts the list (impl:989)
                const d4 ip = ld4(c.pos_cur, id);
                bool near = true;
                if (!c.planedf[k].coh) {
                    const PlaneF& pf = c.planef[k];
                    const float dx = (d2f_rn(ip.x) - c.o_hi[0]) - pf.v[0];
                    const float dy = (d2f_rn(ip.y) - c.o_hi[1]) - pf.v[1];
                    const float dz = (d2f_rn(ip.z) - c.o_hi[2]) - pf.v[2];
                    const float wx = dx * pf.v[3] + dy * pf.v[4] + dz * pf.v[5];
                    const float wy = dx * pf.v[6] + dy * pf.v[7] + dz * pf.v[8];
                    const float wz = dx * pf.v[9] + dy * pf.v[10] + dz * pf.v[11];
                    const float lim = d2f_rn(ip.w) + c.margin;
                    near = fabsf(wz) <= lim && wx >= -lim && wx <= pf.v[12] + lim && wy >= -lim &&
                           wy <= pf.v[13] + lim;
                }
                if (!near) continue;
                const V3<float> d = arm(ip);
                const V3<float> vm = vc + tcross(om, d);
                const unsigned int cnt = k == 0 ? 0u : c.pl_count[id];
                const PlaneOut o = plane_call(&c, k, 0, id, ip, make_float4(vm.x, vm.y, vm.z, m),
                                              make_float4(om.x, om.y, om.z, 0.f), cnt);
                bits |= o.bits;
                if (o.cnt != cnt) c.pl_count[id] = o.cnt;
                if (o.touched) {
                    add_member(d, v3<float>(o.f[0], o.f[1], o.f[2]), v3<float>(o.m[0], o.m[1], o.m[2]));
#pragma unroll
                    for (int q = 0; q < 6; ++q) f6[q] += o.w[q];
                    touched = true;
                }
            }
            emit_body_f(f6, touched, c.bsums + ((size_t)k * c.nblocks + blockIdx.x) * 6, smf);
        }
    }

    // ------------------------------------------------ cylinders in id order (impl:1324-1601)
    if (c.ncyl) {
        ClusterSums cs;
        for (int i = 0; i < 3; ++i) {
            cs.F[i] = F[i];
            cs.M[i] = M[i];
        }
        cs.bits = bits;
        cs = cluster_cylinders_call(&c, cid, live, xc, vc, om, m, cs, smf);
        for (int i = 0; i < 3; ++i) {
            F[i] = cs.F[i];
            M[i] = cs.M[i];
        }
        bits = cs.bits;
    }
    if (!live) return;

    // ------------------------------------------------ members' particle-pair and mesh sums
    for (unsigned int j = 0; j < ne; ++j) {
        const unsigned int id = cid * ne + j;
        const float4 fa = reinterpret_cast<const float4*>(c.fA)[id];
        const float4 fb = reinterpret_cast<const float4*>(c.fB)[id];
        add_member(arm(ld4(c.pos_cur, id)), v3<float>(fa.x, fa.y, fa.z), v3<float>(fb.x, fb.y, fb.z));
    }

    // ------------------------------------------------ integration (impl:224-287, 149-190)
    const V3<float> Ff = v3<float>(F[0].value(), F[1].value(), F[2].value());
    const V3<float> Mf = v3<float>(M[0].value(), M[1].value(), M[2].value());
    const NextBody nx = integrate_f<false>(c, cid, mk3(xc.x, xc.y, xc.z), m, Ff, Mf, true, body_in(c, cid));
    st4(c.cpos_next, cid, mk4(nx.x.x, nx.x.y, nx.x.z, xc.w));
    // A(e) of the next Euler parameters in float pairs (rows as rot_rows)
    const df e0 = split_d(nx.e.x), e1 = split_d(nx.e.y), e2 = split_d(nx.e.z), e3 = split_d(nx.e.w);
    auto twice = [](df a) { return df{2.f * a.hi, 2.f * a.lo}; };
    const df p00 = df_mul(e0, e0), p11 = df_mul(e1, e1), p22 = df_mul(e2, e2), p33 = df_mul(e3, e3);
    const df p01 = df_mul(e0, e1), p02 = df_mul(e0, e2), p03 = df_mul(e0, e3);
    const df p12 = df_mul(e1, e2), p13 = df_mul(e1, e3), p23 = df_mul(e2, e3);
    const df R[9] = {twice(df_add_f(df_add(p00, p11), -0.5f)), twice(df_sub(p12, p03)), twice(df_add(p13, p02)),
                     twice(df_add(p12, p03)), twice(df_add_f(df_add(p00, p22), -0.5f)), twice(df_sub(p23, p01)),
                     twice(df_sub(p13, p02)), twice(df_add(p23, p01)), twice(df_add_f(df_add(p00, p33), -0.5f))};
    const df X0[3] = {df_sub(split_d(nx.x.x), df{c.o_hi[0], c.o_lo[0]}),
                      df_sub(split_d(nx.x.y), df{c.o_hi[1], c.o_lo[1]}),
                      df_sub(split_d(nx.x.z), df{c.o_hi[2], c.o_lo[2]})};
    const float3 w = ang_vel_f(nx.ef, nx.ev);
    const V3<float> wn = vf(w);
    const double* rl = c.rloc + (size_t)cluster_type(c.cl, cid) * ne * 3;
    for (unsigned int j = 0; j < ne; ++j) {
        const unsigned int id = cid * ne + j;
        const df r0 = split_d(rl[3 * j]), r1 = split_d(rl[3 * j + 1]), r2 = split_d(rl[3 * j + 2]);
        df d[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            d[a] = df_add(df_add(df_mul(R[3 * a], r0), df_mul(R[3 * a + 1], r1)), df_mul(R[3 * a + 2], r2));
        const double rad = c.pos_cur[4 * (size_t)id + 3];
        st4(c.pos_next, id, mk4(nx.x.x + (f2d(d[0].hi) + f2d(d[0].lo)), nx.x.y + (f2d(d[1].hi) + f2d(d[1].lo)),
                                nx.x.z + (f2d(d[2].hi) + f2d(d[2].lo)), rad));
        const df X[3] = {df_add(X0[0], d[0]), df_add(X0[1], d[1]), df_add(X0[2], d[2])};
        const V3<float> dm = v3<float>(d[0].hi, d[1].hi, d[2].hi);
        const float rh = d2f_rn(rad);
        emit_rec(c, id, X, rh, d2f_rn(rad - f2d(rh)), nx.v + tcross(wn, dm), m, w, bits);
    }
    if (bits) atomicOr(c.status, bits);
}


}  // namespace
}  // namespace xdem
