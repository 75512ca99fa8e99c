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

// The forward pieces are templates on the scalar type: double for the
// forward restatement the VJPs differentiate, Dual (below) for the tangent
// (forward mode) of the same arithmetic.  The VJPs take V = VT<double>.
XA_HD double sqrt(double x) { return ::sqrt(x); }
XA_HD double fabs(double x) { return ::fabs(x); }

// Forward-mode dual number with N tangent directions: value v and
// derivatives d[k].  Arithmetic follows the product, quotient and chain
// rules; comparisons look at the value only, so a branch follows the
// forward computation.
template <int N>
struct Dual {
    double v;
    double d[N];
    XA_HD Dual() : v(0.0)
    {
        for (int k = 0; k < N; ++k) d[k] = 0.0;
    }
    XA_HD Dual(double x) : v(x)  // a constant
    {
        for (int k = 0; k < N; ++k) d[k] = 0.0;
    }
    friend XA_HD Dual operator+(const Dual& a, const Dual& b)
    {
        Dual r(a.v + b.v);
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
        return r;
    }
    friend XA_HD Dual operator-(const Dual& a, const Dual& b)
    {
        Dual r(a.v - b.v);
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
        return r;
    }
    friend XA_HD Dual operator-(const Dual& a)
    {
        Dual r(-a.v);
        for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
        return r;
    }
    friend XA_HD Dual operator*(const Dual& a, const Dual& b)
    {
        Dual r(a.v * b.v);
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
        return r;
    }
    friend XA_HD Dual operator/(const Dual& a, const Dual& b)
    {
        Dual r(a.v / b.v);
        for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
        return r;
    }
    friend XA_HD Dual sqrt(const Dual& a)
    {
        Dual r(::sqrt(a.v));
        for (int k = 0; k < N; ++k) r.d[k] = r.v > 0.0 ? a.d[k] / (2.0 * r.v) : 0.0;
        return r;
    }
    friend XA_HD Dual fabs(const Dual& a) { return a.v < 0.0 ? -a : a; }
    friend XA_HD bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend XA_HD bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend XA_HD bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend XA_HD bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend XA_HD bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend XA_HD bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
};

template <class T> struct VT { T x, y, z; };
template <class T> struct QT { T x, y, z, w; };
using V = VT<double>;
using Q = QT<double>;

XA_HD V mkv(double x, double y, double z) { return V{x, y, z}; }
XA_HD Q mkq(double x, double y, double z, double w) { return Q{x, y, z, w}; }
template <class T> XA_HD VT<T> vzero() { return VT<T>{T(0.0), T(0.0), T(0.0)}; }
// a constant vector (plane geometry, inertia) in the scalar type T
template <class T> XA_HD VT<T> vc(V a) { return VT<T>{T(a.x), T(a.y), T(a.z)}; }
template <class T> XA_HD VT<T> operator+(VT<T> a, VT<T> b) { return VT<T>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> XA_HD VT<T> operator-(VT<T> a, VT<T> b) { return VT<T>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> XA_HD VT<T> operator-(VT<T> a) { return VT<T>{-a.x, -a.y, -a.z}; }
template <class S, class T> XA_HD VT<T> operator*(S s, VT<T> a) { return VT<T>{s * a.x, s * a.y, s * a.z}; }
template <class T, class S> XA_HD VT<T> operator/(VT<T> a, S s) { return VT<T>{a.x / s, a.y / s, a.z / s}; }
template <class T> XA_HD QT<T> operator+(QT<T> a, QT<T> b) { return QT<T>{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> XA_HD QT<T> operator-(QT<T> a, QT<T> b) { return QT<T>{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class S, class T> XA_HD QT<T> operator*(S s, QT<T> a) { return QT<T>{s * a.x, s * a.y, s * a.z, s * a.w}; }
template <class T> XA_HD T dot(VT<T> a, VT<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> XA_HD T dot(QT<T> a, QT<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <class T> XA_HD T len(VT<T> a) { return sqrt(dot(a, a)); }
template <class T> XA_HD VT<T> cross(VT<T> a, VT<T> b)
{
    return VT<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
XA_HD void addv(V& a, V b) { a = a + b; }
XA_HD void addq(Q& a, Q b) { a = a + b; }

// ---------------------------------------------------------------- Euler parameters
// L(e) (3x4): rows (-e1, e0, e3, -e2), (-e2, -e3, e0, e1), (-e3, e2, -e1, e0)
// with e = (e0, e1, e2, e3) held as (x, y, z, w).  L(e) x = -L(x) e.
template <class T>
XA_HD VT<T> Lmul(QT<T> e, QT<T> x)
{
    return VT<T>{-e.y * x.x + e.x * x.y + e.w * x.z - e.z * x.w, -e.z * x.x - e.w * x.y + e.x * x.z + e.y * x.w,
               -e.w * x.x + e.z * x.y - e.y * x.z + e.x * x.w};
}
// L(e)^T r (4-vector).  L(e)^T r = M(r) e with M(r) skew:
// rows (0,-r0,-r1,-r2), (r0,0,r2,-r1), (r1,-r2,0,r0), (r2,r1,-r0,0).
template <class T>
XA_HD QT<T> LTmul(QT<T> e, VT<T> r)
{
    return QT<T>{-e.y * r.x - e.z * r.y - e.w * r.z, e.x * r.x - e.w * r.y + e.z * r.z,
               e.w * r.x + e.x * r.y - e.y * r.z, -e.z * r.x + e.y * r.y + e.x * r.z};
}
XA_HD Q MTmul(V r, Q l)  // M(r)^T l = -M(r) l
{
    return mkq(r.x * l.y + r.y * l.z + r.z * l.w, -r.x * l.x - r.z * l.z + r.y * l.w,
               -r.y * l.x + r.z * l.y - r.x * l.w, -r.z * l.x - r.y * l.y + r.x * l.z);
}
// G(e) (3x4) of the angular velocity: rows (-e1, e0, -e3, e2),
// (-e2, e3, e0, -e1), (-e3, -e2, e1, e0).  G(e) d = -G(d) e.
template <class T>
XA_HD VT<T> Gmul(QT<T> e, QT<T> d)
{
    return VT<T>{-e.y * d.x + e.x * d.y - e.w * d.z + e.z * d.w, -e.z * d.x + e.w * d.y + e.x * d.z - e.y * d.w,
               -e.w * d.x - e.z * d.y + e.y * d.z + e.x * d.w};
}
XA_HD Q GTmul(Q e, V w)
{
    return mkq(-e.y * w.x - e.z * w.y - e.w * w.z, e.x * w.x + e.w * w.y - e.z * w.z,
               -e.w * w.x + e.x * w.y + e.y * w.z, e.z * w.x - e.y * w.y + e.x * w.z);
}

// omega = 2 G(e) d (impl:32-41)
template <class T> XA_HD VT<T> ang_vel(QT<T> e, QT<T> d) { return 2.0 * Gmul(e, d); }
XA_HD void ang_vel_vjp(Q e, Q d, V lw, Q& le, Q& ld)
{
    addq(ld, 2.0 * GTmul(e, lw));
    addq(le, -2.0 * GTmul(d, lw));
}

// Rotation A(e) (impl:8-30): A v (to_global) and A^T v (to_local).
template <class T>
XA_HD void rot_rows(QT<T> e, VT<T>& r0, VT<T>& r1, VT<T>& r2)
{
    r0 = VT<T>{2.0 * (e.x * e.x + e.y * e.y - 0.5), 2.0 * (e.y * e.z - e.x * e.w), 2.0 * (e.y * e.w + e.x * e.z)};
    r1 = VT<T>{2.0 * (e.y * e.z + e.x * e.w), 2.0 * (e.x * e.x + e.z * e.z - 0.5), 2.0 * (e.z * e.w - e.x * e.y)};
    r2 = VT<T>{2.0 * (e.y * e.w - e.x * e.z), 2.0 * (e.z * e.w + e.x * e.y), 2.0 * (e.x * e.x + e.w * e.w - 0.5)};
}
template <class T>
XA_HD VT<T> to_global(VT<T> v, QT<T> e)
{
    VT<T> r0, r1, r2;
    rot_rows(e, r0, r1, r2);
    return VT<T>{dot(r0, v), dot(r1, v), dot(r2, v)};
}
template <class T>
XA_HD VT<T> to_local(VT<T> v, QT<T> e)
{
    VT<T> r0, r1, r2;
    rot_rows(e, r0, r1, r2);
    return VT<T>{r0.x * v.x + r1.x * v.y + r2.x * v.z, r0.y * v.x + r1.y * v.y + r2.y * v.z,
                 r0.z * v.x + r1.z * v.y + r2.z * v.z};
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
template <class T>
XA_HD QT<T> uceom(V J, QT<T> e, QT<T> d, VT<T> n)
{
    const VT<T> w = Lmul(e, d);
    const VT<T> Tj = VT<T>{J.x * w.x, J.y * w.y, J.z * w.z};
    const QT<T> h = 4.0 * LTmul(d, Tj);
    const VT<T> lh = Lmul(e, h);
    const VT<T> r = VT<T>{(n.x - lh.x) / (2.0 * J.x), (n.y - lh.y) / (2.0 * J.y), (n.z - lh.z) / (2.0 * J.z)};
    const T s2 = dot(e, e), c = dot(d, d);
    return (T(1.0) / s2) * (LTmul(e, r) - c * e);
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
template <class T>
XA_HD QT<T> normalize(QT<T> e)
{
    const T l = sqrt(dot(e, e));
    return QT<T>{e.x / l, e.y / l, e.z / l, e.w / l};
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
template <class T>
struct MatT {
    T Eeq, Seq8, beta, vs1, sratio, fric;
};
using Mat = MatT<double>;
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
template <class T>
struct CoreT {
    T kn, vn, ks, vs, mu, Req, Meq;
    T delta, ds0, dots0;
    VT<T> u, rv;
    // outputs
    VT<T> Fn, Ft;
    T ds1, dots1;
    bool tang;
    // intermediates
    T fsn, cn, fn, me, sdot, St, a, b, nFn;
    VT<T> s;
};
using Core = CoreT<double>;

template <class T>
XA_HD void core_consts(const MatT<T>& m, int model, double ri, double rj, double mi, double mj, CoreT<T>& c)
{
    c.Meq = T(mj != 0.0 ? (mi * mj) / (mi + mj) : mi);
    c.Req = T(rj != 0.0 ? (ri * rj) / (ri + rj) : ri);
    c.kn = (4.0 / 3.0) * m.Eeq * sqrt(c.Req);
    c.vn = m.beta;
    c.ks = model == 1 ? m.Seq8 : c.kn * m.sratio;
    c.vs = m.vs1;
    c.mu = m.fric;
}

template <class T>
XA_HD void core_fwd(int model, double dt, CoreT<T>& c)
{
    c.fsn = -c.kn * (c.delta * sqrt(c.delta));
    c.cn = dot(c.rv, c.u);
    const T fdn = c.vn * c.cn;
    c.fn = c.fsn + fdn;
    c.Fn = c.fn * c.u;
    const VT<T> et = c.rv - dot(c.rv, c.u) * c.u;
    c.me = len(et);
    c.tang = c.me != T(0.0);
    c.ds1 = c.ds0;
    c.dots1 = c.dots0;
    c.Ft = vzero<T>();
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
            c.St = T(0.0);
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
template <class T>
XA_HD VT<T> rel_vel(VT<T> vi, VT<T> wi, VT<T> di, VT<T> vj, VT<T> wj, VT<T> dj)
{
    return (vj + cross(wj, dj)) - (vi + cross(wi, di));
}
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
template <class T>
struct PairGeomT {
    VT<T> rp, u, di, dj;
    T dist, delta;
};
using PairGeom = PairGeomT<double>;
template <class T>
XA_HD void pair_geom(VT<T> xi, VT<T> xj, double ri, double rj, PairGeomT<T>& g)
{
    g.rp = VT<T>{xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
    g.dist = len(g.rp);
    g.delta = T(ri + rj) - g.dist;
    g.u = g.rp / g.dist;
    const VT<T> cpt = xi + ri * g.u;
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
template <class T>
struct PlaneGeomT {
    int region;
    T delta, h, side;
    VT<T> u, X, es, hs;
};
using PlaneGeom = PlaneGeomT<double>;
struct PlaneRect {
    V xw, u1, u2, uw, w2, w3, w4;
    double l1, l2;
};
template <class T>
XA_HD T plane_geom(const PlaneRect& pe, VT<T> xp, double r, PlaneGeomT<T>& g)
{
    g.region = 0;
    g.delta = T(0.0);
    const VT<T> dp = xp - vc<T>(pe.xw);
    const VT<T> wp = VT<T>{dot(dp, vc<T>(pe.u1)), dot(dp, vc<T>(pe.u2)), dot(dp, vc<T>(pe.uw))};
    const T a_l1 = (wp.x - pe.l1) * (wp.x - pe.l1);
    const T b_l2 = (wp.y - pe.l2) * (wp.y - pe.l2);
    const T sqa = wp.x * wp.x, sqb = wp.y * wp.y, sqc = wp.z * wp.z;
    const double sqr = r * r;
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
        g.X = xp - vc<T>(w);
        g.h = len(g.X);
        g.u = g.X / g.h;
        g.delta = T(r) - g.h;
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
        g.X = xp - vc<T>(e0);
        const V ev = e1 - e0;
        g.es = vc<T>(ev / len(ev));
        g.hs = g.X - dot(g.X, g.es) * g.es;
        g.h = len(g.hs);
        g.u = (-g.hs) / g.h;
        g.delta = T(r) - g.h;
        return g.delta;
    }
    if ((wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2)) {
        g.region = 3;
        const V uu = pe.uw / len(pe.uw);
        g.u = vc<T>(-uu);
        const T sd = dot(dp, g.u);
        g.side = T(sd < T(0.0) ? -1.0 : 1.0);
        g.delta = T(r) - fabs(sd);
        return g.delta;
    }
    return T(0.0);
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
template <class T>
struct BodyT {
    VT<T> x, v, w;
    double r, m;
};
using Body = BodyT<double>;

// Particle-particle contacts of sphere i in the order the step visited them
// (the order of its pair list), impl:613-733 as the FP64 fused kernel runs
// it: each contact adds Fn + Ft to F and di x (Fn + Ft) to M.  A contact
// whose tangential velocity is exactly zero keeps the Ft of the contact
// before it (the model leaves Ft untouched; impl:441-452).
template <class T>
XA_HD void pp_sphere_fwd(int model, double dt, const MatT<T>& mat, const BodyT<T>& bi, const BodyT<T>* nb,
                         const T* ds0, const T* dots0, int n, VT<T>& F, VT<T>& M, T* ds1, T* dots1)
{
    VT<T> Ft = vzero<T>();
    for (int s = 0; s < n; ++s) {
        PairGeomT<T> pg;
        pair_geom(bi.x, nb[s].x, bi.r, nb[s].r, pg);
        CoreT<T> c;
        core_consts(mat, model, bi.r, nb[s].r, bi.m, nb[s].m, c);
        c.delta = pg.delta;
        c.u = pg.u;
        c.rv = rel_vel(bi.v, bi.w, pg.di, nb[s].v, nb[s].w, pg.dj);
        c.ds0 = ds0[s];
        c.dots0 = dots0[s];
        core_fwd(model, dt, c);
        if (c.tang) Ft = c.Ft;
        const VT<T> G = c.Fn + Ft;
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
// The plane's material terms come in `mat` (pc.mat, or its dual form).
template <class T>
XA_HD void plane_contact_fwd_t(int model, double dt, const PlaneContact& pc, const MatT<T>& mat, const BodyT<T>& bi,
                               T ds0, T dots0, VT<T>& F, VT<T>& M, T& ds1, T& dots1)
{
    PlaneGeomT<T> pg;
    plane_geom(pc.rect, bi.x, bi.r, pg);
    const VT<T> cpt = bi.x + bi.r * pg.u;
    const VT<T> di = cpt - bi.x, dj = cpt - vc<T>(pc.bp);
    CoreT<T> c;
    core_consts(mat, model, bi.r, 0.0, bi.m, 0.0, c);
    c.delta = pg.delta;
    c.u = pg.u;
    c.rv = rel_vel(bi.v, bi.w, di, vc<T>(pc.bv), vc<T>(pc.bw), dj);
    c.ds0 = ds0;
    c.dots0 = dots0;
    core_fwd(model, dt, c);
    const VT<T> G = c.Fn + c.Ft;
    F = F + G;
    M = M + cross(di, G);
    ds1 = c.ds1;
    dots1 = c.dots1;
}
XA_HD void plane_contact_fwd(int model, double dt, const PlaneContact& pc, const Body& bi, double ds0, double dots0,
                             V& F, V& M, double& ds1, double& dots1)
{
    plane_contact_fwd_t<double>(model, dt, pc, pc.mat, bi, ds0, dots0, F, M, ds1, dots1);
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
