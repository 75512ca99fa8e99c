// xdem_adjoint.cuh -- the FP64 step's per-sphere and per-contact math and
// its hand-written vector-Jacobian products (reverse mode), for the adjoint
// of the DEM trajectory.
//
// Every function here is __host__ __device__: the adjoint kernels
// (xdem_adjoint.cu) call them on the GPU, and a host program checks each VJP
// against central differences of its forward function.
//
// The forward pieces restate the step of the FP64 fused kernel, which follows
// the reference:
//  * angular velocity omega = 2 G(e) e_dot (impl:32-41);
//  * the Euler-parameter acceleration of calculate_uceom (impl:74-133) in the
//    closed form q = [L(e)^T (r / 2J) - (e_dot . e_dot) e] / |e|^2 with
//    r = A(e)^T M - L(e) 4 L(e_dot)^T (J L(e) e_dot);
//  * getConstant + HMCModel / DHSModel (impl:362-474) for one contact, with
//    the material terms of the pair precomputed (Eeq, 8 Seq, beta, vs1);
//  * the particle-particle geometry of calculate_p2p_kernel (impl:676-700)
//    and the plane regions of particle_plane_contact_detection
//    (impl:735-815);
//  * velocity Verlet (impl:135-147, 192-222 with the CPU integrator's
//    linear-velocity update, xIntegratorVV.cpp:143-149).
//
// Notation of the VJPs: for y = f(x), `lx += J^T ly`; every VJP adds into
// its outputs, so contributions from several uses of a value accumulate.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define XA_HD __host__ __device__ __forceinline__
#else
#define XA_HD inline
#endif

namespace xdem {
namespace adj {

struct V { double x, y, z; };
struct Q { double x, y, z, w; };

XA_HD V mkv(double x, double y, double z) { return V{x, y, z}; }
XA_HD Q mkq(double x, double y, double z, double w) { return Q{x, y, z, w}; }
XA_HD V operator+(V a, V b) { return mkv(a.x + b.x, a.y + b.y, a.z + b.z); }
XA_HD V operator-(V a, V b) { return mkv(a.x - b.x, a.y - b.y, a.z - b.z); }
XA_HD V operator-(V a) { return mkv(-a.x, -a.y, -a.z); }
XA_HD V operator*(double s, V a) { return mkv(s * a.x, s * a.y, s * a.z); }
XA_HD V operator/(V a, double s) { return mkv(a.x / s, a.y / s, a.z / s); }
XA_HD Q operator+(Q a, Q b) { return mkq(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
XA_HD Q operator-(Q a, Q b) { return mkq(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
XA_HD Q operator*(double s, Q a) { return mkq(s * a.x, s * a.y, s * a.z, s * a.w); }
XA_HD double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
XA_HD double dot(Q a, Q b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
XA_HD double len(V a) { return sqrt(dot(a, a)); }
XA_HD V cross(V a, V b) { return mkv(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
XA_HD void addv(V& a, V b) { a = a + b; }
XA_HD void addq(Q& a, Q b) { a = a + b; }

// ---------------------------------------------------------------- Euler parameters
// L(e) (3x4): rows (-e1, e0, e3, -e2), (-e2, -e3, e0, e1), (-e3, e2, -e1, e0)
// with e = (e0, e1, e2, e3) held as (x, y, z, w).  L(e) x = -L(x) e.
XA_HD V Lmul(Q e, Q x)
{
    return mkv(-e.y * x.x + e.x * x.y + e.w * x.z - e.z * x.w, -e.z * x.x - e.w * x.y + e.x * x.z + e.y * x.w,
               -e.w * x.x + e.z * x.y - e.y * x.z + e.x * x.w);
}
// L(e)^T r (4-vector).  L(e)^T r = M(r) e with M(r) skew:
// rows (0,-r0,-r1,-r2), (r0,0,r2,-r1), (r1,-r2,0,r0), (r2,r1,-r0,0).
XA_HD Q LTmul(Q e, V r)
{
    return mkq(-e.y * r.x - e.z * r.y - e.w * r.z, e.x * r.x - e.w * r.y + e.z * r.z,
               e.w * r.x + e.x * r.y - e.y * r.z, -e.z * r.x + e.y * r.y + e.x * r.z);
}
XA_HD Q MTmul(V r, Q l)  // M(r)^T l = -M(r) l
{
    return mkq(r.x * l.y + r.y * l.z + r.z * l.w, -r.x * l.x - r.z * l.z + r.y * l.w,
               -r.y * l.x + r.z * l.y - r.x * l.w, -r.z * l.x - r.y * l.y + r.x * l.z);
}
// G(e) (3x4) of the angular velocity: rows (-e1, e0, -e3, e2),
// (-e2, e3, e0, -e1), (-e3, -e2, e1, e0).  G(e) d = -G(d) e.
XA_HD V Gmul(Q e, Q d)
{
    return mkv(-e.y * d.x + e.x * d.y - e.w * d.z + e.z * d.w, -e.z * d.x + e.w * d.y + e.x * d.z - e.y * d.w,
               -e.w * d.x - e.z * d.y + e.y * d.z + e.x * d.w);
}
XA_HD Q GTmul(Q e, V w)
{
    return mkq(-e.y * w.x - e.z * w.y - e.w * w.z, e.x * w.x + e.w * w.y - e.z * w.z,
               -e.w * w.x + e.x * w.y + e.y * w.z, e.z * w.x - e.y * w.y + e.x * w.z);
}

// omega = 2 G(e) d (impl:32-41)
XA_HD V ang_vel(Q e, Q d) { return 2.0 * Gmul(e, d); }
XA_HD void ang_vel_vjp(Q e, Q d, V lw, Q& le, Q& ld)
{
    addq(ld, 2.0 * GTmul(e, lw));
    addq(le, -2.0 * GTmul(d, lw));
}

// Rotation A(e) (impl:8-30): A v (to_global) and A^T v (to_local).
XA_HD void rot_rows(Q e, V& r0, V& r1, V& r2)
{
    r0 = mkv(2.0 * (e.x * e.x + e.y * e.y - 0.5), 2.0 * (e.y * e.z - e.x * e.w), 2.0 * (e.y * e.w + e.x * e.z));
    r1 = mkv(2.0 * (e.y * e.z + e.x * e.w), 2.0 * (e.x * e.x + e.z * e.z - 0.5), 2.0 * (e.z * e.w - e.x * e.y));
    r2 = mkv(2.0 * (e.y * e.w - e.x * e.z), 2.0 * (e.z * e.w + e.x * e.y), 2.0 * (e.x * e.x + e.w * e.w - 0.5));
}
XA_HD V to_global(V v, Q e)
{
    V r0, r1, r2;
    rot_rows(e, r0, r1, r2);
    return mkv(dot(r0, v), dot(r1, v), dot(r2, v));
}
XA_HD V to_local(V v, Q e)
{
    V r0, r1, r2;
    rot_rows(e, r0, r1, r2);
    return mkv(r0.x * v.x + r1.x * v.y + r2.x * v.z, r0.y * v.x + r1.y * v.y + r2.y * v.z,
               r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
// n = A(e)^T m: lm += A(e) ln, le += grad_e (m^T A(e) ln).
XA_HD void to_local_vjp(V m, Q e, V ln, V& lm, Q& le)
{
    addv(lm, to_global(ln, e));
    const double u0 = m.x, u1 = m.y, u2 = m.z, w0 = ln.x, w1 = ln.y, w2 = ln.z;
    const double e0 = e.x, e1 = e.y, e2 = e.z, e3 = e.w;
    const double g0 = 2.0 * (u0 * w0 * (2.0 * e0) - u0 * w1 * e3 + u0 * w2 * e2 + u1 * w0 * e3 +
                             u1 * w1 * (2.0 * e0) - u1 * w2 * e1 - u2 * w0 * e2 + u2 * w1 * e1 + u2 * w2 * (2.0 * e0));
    const double g1 = 2.0 * (u0 * w0 * (2.0 * e1) + u0 * w1 * e2 + u0 * w2 * e3 + u1 * w0 * e2 - u1 * w2 * e0 +
                             u2 * w0 * e3 + u2 * w1 * e0);
    const double g2 = 2.0 * (u0 * w1 * e1 + u0 * w2 * e0 + u1 * w0 * e1 + u1 * w1 * (2.0 * e2) + u1 * w2 * e3 -
                             u2 * w0 * e0 + u2 * w1 * e3);
    const double g3 = 2.0 * (-u0 * w1 * e0 + u0 * w2 * e1 + u1 * w0 * e0 + u1 * w2 * e2 + u2 * w0 * e1 +
                             u2 * w1 * e2 + u2 * w2 * (2.0 * e3));
    addq(le, mkq(g0, g1, g2, g3));
}

// Euler-parameter acceleration (impl:74-133), closed form.
XA_HD Q uceom(V J, Q e, Q d, V n)
{
    const V w = Lmul(e, d);
    const V T = mkv(J.x * w.x, J.y * w.y, J.z * w.z);
    const Q h = 4.0 * LTmul(d, T);
    const V lh = Lmul(e, h);
    const V r = mkv((n.x - lh.x) / (2.0 * J.x), (n.y - lh.y) / (2.0 * J.y), (n.z - lh.z) / (2.0 * J.z));
    const double s2 = dot(e, e), c = dot(d, d);
    return (1.0 / s2) * (LTmul(e, r) - c * e);
}
// The moment in body axes that gave q (q = uceom(J, e, d, n)): L(e) q = r.
XA_HD V uceom_torque(V J, Q e, Q d, Q q)
{
    const V rq = Lmul(e, q);
    const V w = Lmul(e, d);
    const V T = mkv(J.x * w.x, J.y * w.y, J.z * w.z);
    const V lh = Lmul(e, 4.0 * LTmul(d, T));
    return mkv(2.0 * J.x * rq.x + lh.x, 2.0 * J.y * rq.y + lh.y, 2.0 * J.z * rq.z + lh.z);
}
XA_HD void uceom_vjp(V J, Q e, Q d, V n, Q lq, Q& le, Q& ld, V& ln)
{
    // forward intermediates
    const V w = Lmul(e, d);
    const V T = mkv(J.x * w.x, J.y * w.y, J.z * w.z);
    const Q h = 4.0 * LTmul(d, T);
    const V lh = Lmul(e, h);
    const V r = mkv((n.x - lh.x) / (2.0 * J.x), (n.y - lh.y) / (2.0 * J.y), (n.z - lh.z) / (2.0 * J.z));
    const double s2 = dot(e, e), c = dot(d, d);
    const Q p = LTmul(e, r);
    const Q q = (1.0 / s2) * (p - c * e);
    // q = (p - c e) / s2
    const Q lp = (1.0 / s2) * lq;
    const double lc = -dot(e, lq) / s2;
    const double ls2 = -dot(q, lq) / s2;
    addq(le, (-c / s2) * lq + (2.0 * ls2) * e);
    // c = d.d
    addq(ld, (2.0 * lc) * d);
    // p = L(e)^T r = M(r) e
    const V lr = Lmul(e, lp);
    addq(le, MTmul(r, lp));
    // r = (n - lh) / 2J
    const V lrs = mkv(lr.x / (2.0 * J.x), lr.y / (2.0 * J.y), lr.z / (2.0 * J.z));
    addv(ln, lrs);
    const V llh = -lrs;
    // lh = L(e) h = -L(h) e
    const Q lhq = LTmul(e, llh);
    addq(le, -1.0 * LTmul(h, llh));
    // h = 4 L(d)^T T = 4 M(T) d
    const V lT = 4.0 * Lmul(d, lhq);
    addq(ld, 4.0 * MTmul(T, lhq));
    // T = J w, w = L(e) d = -L(d) e
    const V lw = mkv(J.x * lT.x, J.y * lT.y, J.z * lT.z);
    addq(ld, LTmul(e, lw));
    addq(le, -1.0 * LTmul(d, lw));
}

// e1 = e' / |e'|
XA_HD Q normalize(Q e)
{
    const double l = sqrt(dot(e, e));
    return mkq(e.x / l, e.y / l, e.z / l, e.w / l);
}
XA_HD void normalize_vjp(Q e, Q l1, Q& le)
{
    const double l = sqrt(dot(e, e));
    const Q u = (1.0 / l) * e;
    addq(le, (1.0 / l) * (l1 - dot(u, l1) * u));
}

// ---------------------------------------------------------------- contact model
// Material terms of a contact pair (the precomputed fields of getConstant
// that the model reads; impl:362-386).
struct Mat {
    double Eeq, Seq8, beta, vs1, sratio, fric;
};
// Loss gradient with respect to those fields.
struct MatGrad {
    double Eeq, Seq8, beta, vs1, fric;
};
XA_HD void add_grad(MatGrad& a, const MatGrad& b)
{
    a.Eeq += b.Eeq; a.Seq8 += b.Seq8; a.beta += b.beta; a.vs1 += b.vs1; a.fric += b.fric;
}

// One contact of the model (HMCModel model 1, DHSModel model 0; impl:432-474)
// with its intermediates.  Inputs: the constants, the overlap delta, the unit
// normal u (from sphere i towards the partner), the relative velocity rv of
// the partner's contact point, the history (ds0, dots0) carried from the last
// step.  `tang` is false when the tangential velocity is exactly zero: the
// model then leaves Ft and the history untouched.
struct Core {
    double kn, vn, ks, vs, mu, Req, Meq;
    double delta, ds0, dots0;
    V u, rv;
    // outputs
    V Fn, Ft;
    double ds1, dots1;
    bool tang;
    // intermediates
    double fsn, cn, fn, me, sdot, St, a, b, nFn;
    V s;
};

XA_HD void core_consts(const Mat& m, int model, double ri, double rj, double mi, double mj, Core& c)
{
    c.Meq = mj != 0.0 ? (mi * mj) / (mi + mj) : mi;
    c.Req = rj != 0.0 ? (ri * rj) / (ri + rj) : ri;
    c.kn = (4.0 / 3.0) * m.Eeq * sqrt(c.Req);
    c.vn = m.beta;
    c.ks = model == 1 ? m.Seq8 : c.kn * m.sratio;
    c.vs = m.vs1;
    c.mu = m.fric;
}

XA_HD void core_fwd(int model, double dt, Core& c)
{
    c.fsn = -c.kn * (c.delta * sqrt(c.delta));
    c.cn = dot(c.rv, c.u);
    const double fdn = c.vn * c.cn;
    c.fn = c.fsn + fdn;
    c.Fn = c.fn * c.u;
    const V et = c.rv - dot(c.rv, c.u) * c.u;
    c.me = len(et);
    c.tang = c.me != 0.0;
    c.ds1 = c.ds0;
    c.dots1 = c.dots0;
    c.Ft = mkv(0, 0, 0);
    c.nFn = len(c.Fn);
    if (c.tang) {
        c.s = et / c.me;
        c.sdot = dot(c.rv, c.s);
        c.ds1 = c.ds0 + dt * (c.sdot + c.dots0);
        c.dots1 = c.sdot;
        if (model == 1) {
            c.St = c.ks * sqrt(c.Req * c.delta);
            c.a = c.St * c.ds1 + c.vs * sqrt(c.St * c.Meq);
        } else {
            c.St = 0.0;
            c.a = c.ks * c.ds1 + c.vs * dot(c.rv, c.s);
        }
        c.b = c.mu * c.nFn;
        c.Ft = (c.a < c.b ? c.a : c.b) * c.s;
    }
}

// Reverse of core_fwd.  lFn and lFt are the adjoints of the contact's normal
// and tangential force (lFt is ignored when !tang), lds1 / ldots1 those of
// the history the step stored.  Adds into ldelta, lu, lrv, lds0, ldots0 and
// the material gradient g.
XA_HD void core_vjp(int model, double dt, const Core& c, const Mat& m, V lFn, V lFt, double lds1, double ldots1,
                    double& ldelta, V& lu, V& lrv, double& lds0, double& ldots0, MatGrad& g)
{
    double lkn = 0.0, lks = 0.0;
    if (c.tang) {
        // Ft = min(a, b) s
        const double ft = c.a < c.b ? c.a : c.b;
        const double lft = dot(lFt, c.s);
        V ls = ft * lFt;
        const double la = c.a < c.b ? lft : 0.0;
        const double lb = c.a < c.b ? 0.0 : lft;
        // b = mu |Fn|
        g.fric += c.nFn * lb;
        if (c.nFn > 0.0) lFn = lFn + (c.mu * lb / c.nFn) * c.Fn;
        // a
        double lds1t = lds1, lsdot = ldots1;
        if (model == 1) {
            const double sm = sqrt(c.St * c.Meq);
            const double lSt = la * c.ds1 + (sm > 0.0 ? la * c.vs * c.Meq / (2.0 * sm) : 0.0);
            lds1t += c.St * la;
            g.vs1 += sm * la;
            const double sr = sqrt(c.Req * c.delta);
            lks += sr * lSt;
            if (sr > 0.0) ldelta += c.ks * c.Req / (2.0 * sr) * lSt;
        } else {
            lks += c.ds1 * la;
            lds1t += c.ks * la;
            g.vs1 += c.sdot * la;
            lsdot += c.vs * la;
        }
        // ds1 = ds0 + dt (sdot + dots0), dots1 = sdot
        lds0 += lds1t;
        lsdot += dt * lds1t;
        ldots0 += dt * lds1t;
        // sdot = rv . s
        lrv = lrv + lsdot * c.s;
        ls = ls + lsdot * c.rv;
        // s = et / me
        const V let = (1.0 / c.me) * (ls - dot(c.s, ls) * c.s);
        // et = rv - (rv . u) u
        lrv = lrv + let;
        const double lc = -dot(c.u, let);
        lu = lu - c.cn * let;
        lrv = lrv + lc * c.u;
        lu = lu + lc * c.rv;
    } else {
        lds0 += lds1;
        ldots0 += ldots1;
    }
    // Fn = fn u
    const double lfn = dot(lFn, c.u);
    lu = lu + c.fn * lFn;
    // fn = fsn + vn cn
    g.beta += c.cn * lfn;
    const double lcn = c.vn * lfn;
    lrv = lrv + lcn * c.u;
    lu = lu + lcn * c.rv;
    // fsn = -kn delta^1.5
    lkn += -(c.delta * sqrt(c.delta)) * lfn;
    ldelta += -1.5 * c.kn * sqrt(c.delta) * lfn;
    // constants
    if (model == 1) {
        g.Seq8 += lks;
    } else {
        lkn += m.sratio * lks;
    }
    g.Eeq += (4.0 / 3.0) * sqrt(c.Req) * lkn;
}

// ---------------------------------------------------------------- geometry
// Relative velocity of the partner's contact point seen from sphere i:
// rv = (vj + wj x dj) - (vi + wi x di) with di, dj the contact point relative
// to the two centres (impl:684-688).
XA_HD V rel_vel(V vi, V wi, V di, V vj, V wj, V dj) { return (vj + cross(wj, dj)) - (vi + cross(wi, di)); }
XA_HD void rel_vel_vjp(V wi, V di, V wj, V dj, V lrv, V& lvi, V& lwi, V& ldi, V& lvj, V& lwj, V& ldj)
{
    lvj = lvj + lrv;
    lvi = lvi - lrv;
    lwj = lwj + cross(dj, lrv);
    ldj = ldj + cross(lrv, wj);
    lwi = lwi - cross(di, lrv);
    ldi = ldi - cross(lrv, wi);
}

// Particle pair (impl:676-688): rp = xj - xi, delta = (ri + rj) - |rp|,
// u = rp / |rp|, contact point c = xi + ri u, di = c - xi, dj = c - xj.
struct PairGeom {
    V rp, u, di, dj;
    double dist, delta;
};
XA_HD void pair_geom(V xi, V xj, double ri, double rj, PairGeom& g)
{
    g.rp = mkv(xj.x - xi.x, xj.y - xi.y, xj.z - xi.z);
    g.dist = len(g.rp);
    g.delta = (ri + rj) - g.dist;
    g.u = g.rp / g.dist;
    const V cpt = xi + ri * g.u;
    g.di = cpt - xi;
    g.dj = cpt - xj;
}
XA_HD void pair_geom_vjp(const PairGeom& g, double ri, double ldelta, V lu, V ldi, V ldj, V& lxi, V& lxj)
{
    // di = ri u, dj = xi + ri u - xj
    lxi = lxi + ldj;
    lxj = lxj - ldj;
    lu = lu + ri * (ldi + ldj);
    // u = rp / dist, delta = ri + rj - dist
    const V lrp = (1.0 / g.dist) * (lu - dot(g.u, lu) * g.u) - ldelta * g.u;
    lxj = lxj + lrp;
    lxi = lxi - lrp;
}

// Plane regions of particle_plane_contact_detection (impl:735-815) for a
// rectangle with corner xw, edge vectors u1 (length l1) and u2 (length l2),
// normal uw and the other corners w2, w3, w4.  region: 0 none, 1 corner
// (u = (x - w) / |x - w|), 2 edge (u = -hs / |hs| with hs the part of x - w
// normal to the edge direction es), 3 face (u = -uw / |uw|,
// delta = r - |(x - xw) . u|).
struct PlaneGeom {
    int region;
    double delta, h, side;
    V u, X, es, hs;
};
struct PlaneRect {
    V xw, u1, u2, uw, w2, w3, w4;
    double l1, l2;
};
XA_HD double plane_geom(const PlaneRect& pe, V xp, double r, PlaneGeom& g)
{
    g.region = 0;
    g.delta = 0.0;
    const V dp = xp - pe.xw;
    const V wp = mkv(dot(dp, pe.u1), dot(dp, pe.u2), dot(dp, pe.uw));
    const double a_l1 = (wp.x - pe.l1) * (wp.x - pe.l1);
    const double b_l2 = (wp.y - pe.l2) * (wp.y - pe.l2);
    const double sqa = wp.x * wp.x, sqb = wp.y * wp.y, sqc = wp.z * wp.z, sqr = r * r;
    V w = pe.xw;
    bool corner = false;
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        w = pe.xw; corner = true;
    } else if (wp.x > pe.l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        w = pe.w2; corner = true;
    } else if (wp.x > pe.l1 && wp.y > pe.l2 && (a_l1 + b_l2 + sqc) < sqr) {
        w = pe.w3; corner = true;
    } else if (wp.x < 0 && wp.y > pe.l2 && (sqa + b_l2 + sqc) < sqr) {
        w = pe.w4; corner = true;
    }
    if (corner) {
        g.region = 1;
        g.X = xp - w;
        g.h = len(g.X);
        g.u = g.X / g.h;
        g.delta = r - g.h;
        return g.delta;
    }
    V e0 = pe.xw, e1 = pe.w2;
    bool edge = false;
    if ((wp.x > 0 && wp.x < pe.l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        e0 = pe.xw; e1 = pe.w2; edge = true;
    } else if ((wp.x > 0 && wp.x < pe.l1) && wp.y > pe.l2 && (b_l2 + sqc) < sqr) {
        e0 = pe.w4; e1 = pe.w3; edge = true;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x > pe.l1 && (a_l1 + sqc) < sqr) {
        e0 = pe.w2; e1 = pe.w3; edge = true;
    }
    if (edge) {
        g.region = 2;
        g.X = xp - e0;
        const V ev = e1 - e0;
        g.es = ev / len(ev);
        g.hs = g.X - dot(g.X, g.es) * g.es;
        g.h = len(g.hs);
        g.u = (-g.hs) / g.h;
        g.delta = r - g.h;
        return g.delta;
    }
    if ((wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2)) {
        g.region = 3;
        const V uu = pe.uw / len(pe.uw);
        g.u = -uu;
        const double sd = dot(dp, g.u);
        g.side = sd < 0.0 ? -1.0 : 1.0;
        g.delta = r - fabs(sd);
        return g.delta;
    }
    return 0.0;
}
XA_HD void plane_geom_vjp(const PlaneGeom& g, double ldelta, V lu, V& lx)
{
    if (g.region == 1) {
        lx = lx + (1.0 / g.h) * (lu - dot(g.u, lu) * g.u) - ldelta * g.u;
    } else if (g.region == 2) {
        // u = -n, n = hs / h, delta = r - h, hs = P X with P = I - es es^T
        const V n = g.hs / g.h;
        const V ln = -lu;
        const V lhs = (1.0 / g.h) * (ln - dot(n, ln) * n) - ldelta * n;
        lx = lx + (lhs - dot(g.es, lhs) * g.es);
    } else if (g.region == 3) {
        // delta = r - side * ((x - xw) . u), u constant
        lx = lx - (ldelta * g.side) * g.u;
    }
}

// ---------------------------------------------------------------- one sphere's contacts
// Sphere i and the state of one contact partner.
struct Body {
    V x, v, w;
    double r, m;
};

// Particle-particle contacts of sphere i in the order the step visited them
// (the order of its pair list), impl:613-733 as the FP64 fused kernel runs
// it: each contact adds Fn + Ft to F and di x (Fn + Ft) to M.  A contact
// whose tangential velocity is exactly zero keeps the Ft of the contact
// before it (the model leaves Ft untouched; impl:441-452).
XA_HD void pp_sphere_fwd(int model, double dt, const Mat& mat, const Body& bi, const Body* nb, const double* ds0,
                         const double* dots0, int n, V& F, V& M, double* ds1, double* dots1)
{
    V Ft = mkv(0, 0, 0);
    for (int s = 0; s < n; ++s) {
        PairGeom pg;
        pair_geom(bi.x, nb[s].x, bi.r, nb[s].r, pg);
        Core c;
        core_consts(mat, model, bi.r, nb[s].r, bi.m, nb[s].m, c);
        c.delta = pg.delta;
        c.u = pg.u;
        c.rv = rel_vel(bi.v, bi.w, pg.di, nb[s].v, nb[s].w, pg.dj);
        c.ds0 = ds0[s];
        c.dots0 = dots0[s];
        core_fwd(model, dt, c);
        if (c.tang) Ft = c.Ft;
        const V G = c.Fn + Ft;
        F = F + G;
        M = M + cross(pg.di, G);
        ds1[s] = c.ds1;
        dots1[s] = c.dots1;
    }
}

// Reverse of pp_sphere_fwd for n <= kMaxPairs contacts.  lF and lM are the
// adjoints of the sphere's force and moment sums, lds1 / ldots1 of the
// history it stored.  Adds into the sphere's lxi, lvi, lwi, into each
// partner's lxj[s], lvj[s], lwj[s], into the carried history lds0[s],
// ldots0[s] and into g.
constexpr int kMaxPairs = 12;
XA_HD void pp_sphere_vjp(int model, double dt, const Mat& mat, const Body& bi, const Body* nb, const double* ds0,
                         const double* dots0, int n, V lF, V lM, const double* lds1, const double* ldots1, V& lxi,
                         V& lvi, V& lwi, V* lxj, V* lvj, V* lwj, double* lds0, double* ldots0, MatGrad& g)
{
    V ftu[kMaxPairs];
    {
        V Ft = mkv(0, 0, 0);
        for (int s = 0; s < n; ++s) {
            PairGeom pg;
            pair_geom(bi.x, nb[s].x, bi.r, nb[s].r, pg);
            Core c;
            core_consts(mat, model, bi.r, nb[s].r, bi.m, nb[s].m, c);
            c.delta = pg.delta;
            c.u = pg.u;
            c.rv = rel_vel(bi.v, bi.w, pg.di, nb[s].v, nb[s].w, pg.dj);
            c.ds0 = ds0[s];
            c.dots0 = dots0[s];
            core_fwd(model, dt, c);
            if (c.tang) Ft = c.Ft;
            ftu[s] = Ft;
        }
    }
    V lcarry = mkv(0, 0, 0);  // adjoint of the Ft that later contacts kept
    for (int s = n - 1; s >= 0; --s) {
        PairGeom pg;
        pair_geom(bi.x, nb[s].x, bi.r, nb[s].r, pg);
        Core c;
        core_consts(mat, model, bi.r, nb[s].r, bi.m, nb[s].m, c);
        c.delta = pg.delta;
        c.u = pg.u;
        c.rv = rel_vel(bi.v, bi.w, pg.di, nb[s].v, nb[s].w, pg.dj);
        c.ds0 = ds0[s];
        c.dots0 = dots0[s];
        core_fwd(model, dt, c);
        const V G = c.Fn + ftu[s];
        const V lG = lF + cross(lM, pg.di);
        V ldi = cross(G, lM), ldj = mkv(0, 0, 0);
        V lFt = mkv(0, 0, 0);
        if (c.tang) {
            lFt = lG + lcarry;
            lcarry = mkv(0, 0, 0);
        } else {
            lcarry = lcarry + lG;
        }
        double ldelta = 0.0;
        V lu = mkv(0, 0, 0), lrv = mkv(0, 0, 0);
        core_vjp(model, dt, c, mat, lG, lFt, lds1[s], ldots1[s], ldelta, lu, lrv, lds0[s], ldots0[s], g);
        rel_vel_vjp(bi.w, pg.di, nb[s].w, pg.dj, lrv, lvi, lwi, ldi, lvj[s], lwj[s], ldj);
        pair_geom_vjp(pg, bi.r, ldelta, lu, ldi, ldj, lxi, lxj[s]);
    }
}

// One plane contact of sphere i (impl:950-1080): plane body at bp moving
// with (bv, bw); the model's partner mass and radius are 0 (impl:997-999).
struct PlaneContact {
    PlaneRect rect;
    V bp, bv, bw;
    Mat mat;
};
XA_HD void plane_contact_fwd(int model, double dt, const PlaneContact& pc, const Body& bi, double ds0, double dots0,
                             V& F, V& M, double& ds1, double& dots1)
{
    PlaneGeom pg;
    plane_geom(pc.rect, bi.x, bi.r, pg);
    const V cpt = bi.x + bi.r * pg.u;
    const V di = cpt - bi.x, dj = cpt - pc.bp;
    Core c;
    core_consts(pc.mat, model, bi.r, 0.0, bi.m, 0.0, c);
    c.delta = pg.delta;
    c.u = pg.u;
    c.rv = rel_vel(bi.v, bi.w, di, pc.bv, pc.bw, dj);
    c.ds0 = ds0;
    c.dots0 = dots0;
    core_fwd(model, dt, c);
    const V G = c.Fn + c.Ft;
    F = F + G;
    M = M + cross(di, G);
    ds1 = c.ds1;
    dots1 = c.dots1;
}
XA_HD void plane_contact_vjp(int model, double dt, const PlaneContact& pc, const Body& bi, double ds0, double dots0,
                             V lF, V lM, double lds1, double ldots1, V& lx, V& lv, V& lw, double& lds0,
                             double& ldots0, MatGrad& g)
{
    PlaneGeom pg;
    plane_geom(pc.rect, bi.x, bi.r, pg);
    const V cpt = bi.x + bi.r * pg.u;
    const V di = cpt - bi.x, dj = cpt - pc.bp;
    Core c;
    core_consts(pc.mat, model, bi.r, 0.0, bi.m, 0.0, c);
    c.delta = pg.delta;
    c.u = pg.u;
    c.rv = rel_vel(bi.v, bi.w, di, pc.bv, pc.bw, dj);
    c.ds0 = ds0;
    c.dots0 = dots0;
    core_fwd(model, dt, c);
    const V G = c.Fn + c.Ft;
    const V lG = lF + cross(lM, di);
    V ldi = cross(G, lM), ldj = mkv(0, 0, 0);
    double ldelta = 0.0;
    V lu = mkv(0, 0, 0), lrv = mkv(0, 0, 0);
    core_vjp(model, dt, c, pc.mat, lG, lG, lds1, ldots1, ldelta, lu, lrv, lds0, ldots0, g);
    V lbv = mkv(0, 0, 0), lbw = mkv(0, 0, 0);
    rel_vel_vjp(bi.w, di, pc.bw, dj, lrv, lv, lw, ldi, lbv, lbw, ldj);
    // di = r u, dj = x + r u - bp
    lx = lx + ldj;
    lu = lu + bi.r * (ldi + ldj);
    plane_geom_vjp(pg, ldelta, lu, lx);
}

// ---------------------------------------------------------------- velocity Verlet
// Position half (impl:135-147): x1 = x0 + dt v0 + h a0, e1 = normalize(e0 +
// dt e_dot0 + h e_ddot0) with h = dt^2 / 2.  Velocity half (impl:192-222):
// a1 = (F + m g) / m, v1 = v0 + dt/2 (a0 + a1) (kept at v0 in the
// velocity-compat mode), q = uceom(J, e1, e_dot0, A(e1)^T M),
// e_dot1 = e_dot0 + dt/2 (e_ddot0 + q), e_ddot1 = q.

}  // namespace adj
}  // namespace xdem
