// xdem_hht.cu -- host multibody side of the DEM coupling: rigid bodies in
// Euler-parameter coordinates, revolute / translational joints and a
// rotation driver, advanced by the HHT-alpha integrator with a Newton loop
// (source/xdynamics_simulation/xIntegratorHHT.cpp:51-183 of xdynamics), the
// DEM wrench entering the force vector as xMultiBodySimulation::
// ConstructForceVector adds xPointMass::ContactForce / ContactMoment
// (source/xdynamics_simulation/xMultiBodySimulation.cpp:341-360).
//
// Coordinates of body b (b >= 1; body 0 is the ground and holds no
// unknowns): q_b = (r, p), r the centre of mass, p = (e0, e1, e2, e3).
// With G(p) the body-frame map (omega' = 2 G p_dot, rows of GMatrix in
// xAlgebraMath.cpp:663-670) and E(p) the global one (omega = 2 E p_dot):
//   mass block       diag(m I3, 4 G^T J' G)
//   force vector     (m g + F, 2 E^T n + 8 G_dot^T J' G_dot p)
// for a force F and moment n in the global frame.  The reference forms the
// rotational entry as 2 G^T n with the global moment, which equals 2 E^T n
// only while the body frame is aligned with the global frame; here the
// global moment goes through E.  Constraints: each joint's equations, the
// driver, and one normalisation p.p - 1 = 0 per body (Jacobian row 2 p^T).
//
// One step (HHT-alpha, alpha in [-1/3, 0], beta = (1 - alpha)^2 / 4,
// gamma = 1/2 - alpha) solves for the accelerations and Lagrange
// multipliers x = (q_dd, lambda) of
//   M q_dd / (1 + alpha) + Phi_q^T lambda - F + pre = 0,
//   Phi(q, t) / (beta dt^2) = 0,
// with q = ipp + beta dt^2 q_dd, q_dot = ipv + gamma dt q_dd and
// pre = alpha / (1 + alpha) (F - Phi_q^T lambda) at the previous step
// (PredictionStep), by Newton iterations whose matrix is
// [M/(1+alpha) + beta dt^2/(1+alpha) d(M q_dd)/dq, Phi_q^T; Phi_q, 0]
// (CorrectionStep and MassJacobian, without the force and constraint
// second-derivative terms, as there) until the residual norm is below the
// tolerance, at most 100 iterations.  The dense system is solved by
// Gaussian elimination with partial pivoting.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "xdem_kernels.h"

namespace {

struct V3 { double x, y, z; };
inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

// 3 x 4 matrices of Euler parameters, row-major
struct M34 { double a[3][4]; };
// body-frame map G(p) (GMatrix): omega' = 2 G p_dot
M34 Gm(const double* p)
{
    return M34{{{-p[1], p[0], p[3], -p[2]}, {-p[2], -p[3], p[0], p[1]}, {-p[3], p[2], -p[1], p[0]}}};
}
// global map E(p) (LMatrix): omega = 2 E p_dot
M34 Em(const double* p)
{
    return M34{{{-p[1], p[0], -p[3], p[2]}, {-p[2], p[3], p[0], -p[1]}, {-p[3], -p[2], p[1], p[0]}}};
}
// A(p) = E G^T: body to global
void Am(const double* p, double A[3][3])
{
    const double e0 = p[0], e1 = p[1], e2 = p[2], e3 = p[3];
    A[0][0] = 2 * (e0 * e0 + e1 * e1 - 0.5); A[0][1] = 2 * (e1 * e2 - e0 * e3);       A[0][2] = 2 * (e1 * e3 + e0 * e2);
    A[1][0] = 2 * (e1 * e2 + e0 * e3);       A[1][1] = 2 * (e0 * e0 + e2 * e2 - 0.5); A[1][2] = 2 * (e2 * e3 - e0 * e1);
    A[2][0] = 2 * (e1 * e3 - e0 * e2);       A[2][1] = 2 * (e2 * e3 + e0 * e1);       A[2][2] = 2 * (e0 * e0 + e3 * e3 - 0.5);
}
V3 mulA(const double A[3][3], V3 s)
{
    return v3(A[0][0] * s.x + A[0][1] * s.y + A[0][2] * s.z, A[1][0] * s.x + A[1][1] * s.y + A[1][2] * s.z,
              A[2][0] * s.x + A[2][1] * s.y + A[2][2] * s.z);
}
V3 mulAT(const double A[3][3], V3 s)
{
    return v3(A[0][0] * s.x + A[1][0] * s.y + A[2][0] * s.z, A[0][1] * s.x + A[1][1] * s.y + A[2][1] * s.z,
              A[0][2] * s.x + A[1][2] * s.y + A[2][2] * s.z);
}
// B(p, s') = d(A(p) s') / dp (BMatrix): columns 4 e0 s + 2 e x s, and
// 2 ((e.s) I + e s^T - e0 [s]x)
void Bm(const double* p, V3 s, double B[3][4])
{
    const V3 e = v3(p[1], p[2], p[3]);
    const V3 c0 = 4.0 * p[0] * s + 2.0 * cross(e, s);
    const double es = dot(e, s);
    const double S[3][3] = {{0, -s.z, s.y}, {s.z, 0, -s.x}, {-s.y, s.x, 0}};
    const double ev[3] = {e.x, e.y, e.z}, sv[3] = {s.x, s.y, s.z};
    const double c0v[3] = {c0.x, c0.y, c0.z};
    for (int r = 0; r < 3; ++r) {
        B[r][0] = c0v[r];
        for (int k = 0; k < 3; ++k) B[r][1 + k] = 2.0 * ((r == k ? es : 0.0) + ev[r] * sv[k] - p[0] * S[r][k]);
    }
}
V3 vec(const double* a) { return v3(a[0], a[1], a[2]); }

struct Body {
    double m = 0.0;
    V3 J{0, 0, 0};  // principal inertia in the body frame
    double q[7] = {0, 0, 0, 1, 0, 0, 0}, qd[7] = {}, qdd[7] = {};
    V3 F{0, 0, 0}, N{0, 0, 0};  // contact force and moment (global), held until replaced
};

enum JointKind { kRevolute = 0, kTranslational = 1 };
struct Joint {
    int kind;
    int i, j;         // bodies (0 = ground)
    V3 si, sj;        // joint point in each body frame
    V3 hi, hj;        // axis in each body frame
    V3 fi, gi;        // body i: two unit vectors normal to the axis (g = h x f)
    V3 fj, gj;        // body j: the same two directions at definition
};
struct Driver {
    int joint;        // a revolute joint: rotation of body j relative to body i about the axis
    double omega, theta0;
};

}  // namespace

struct xdem_mbd {
    double dt = 1e-5, alpha = -0.3, beta = 0.0, gamma = 0.0, eps = 1e-5, t = 0.0;
    V3 g{0, -9.80665, 0};
    std::vector<Body> bodies;  // [0] is the ground
    std::vector<Joint> joints;
    std::vector<Driver> drivers;
    bool ready = false;
    int last_iterations = 0;
    // unknowns: q_dd of every moving body (7 each), then the multipliers
    std::vector<double> lambda, pre, ipp, ipv;
    int mdim() const { return 7 * ((int)bodies.size() - 1); }
    int ncon() const
    {
        return 5 * (int)joints.size() + (int)drivers.size() + ((int)bodies.size() - 1);
    }
};

namespace {

// Index of body b's first unknown, -1 for the ground.
int off(int b) { return b == 0 ? -1 : 7 * (b - 1); }

// Adds v (3 wide, coefficients of r) and w (4 wide, of p) of body b to the
// Jacobian row r of the dense matrix (ncol columns).
void add_jac(std::vector<double>& Jq, int ncol, int row, int b, V3 v, const double w[4])
{
    const int o = off(b);
    if (o < 0) return;
    double* R = Jq.data() + (size_t)row * ncol;
    R[o + 0] += v.x; R[o + 1] += v.y; R[o + 2] += v.z;
    for (int k = 0; k < 4; ++k) R[o + 3 + k] += w[k];
}

// a^T B (1 x 4)
void aTB(V3 a, const double B[3][4], double out[4])
{
    for (int k = 0; k < 4; ++k) out[k] = a.x * B[0][k] + a.y * B[1][k] + a.z * B[2][k];
}

struct Frame {
    double A[3][3];
    V3 r;
    const double* p;
};
Frame frame(const xdem_mbd* m, int b)
{
    Frame f;
    const Body& B = m->bodies[b];
    Am(B.q + 3, f.A);
    f.r = vec(B.q);
    f.p = B.q + 3;
    return f;
}

// dot-1 constraint a_i . a_j (a_i = A_i a'_i): value, and Jacobian rows
double dot1(const Frame& Fi, V3 ai_l, const Frame& Fj, V3 aj_l, int bi, int bj, std::vector<double>* Jq, int ncol,
            int row)
{
    const V3 ai = mulA(Fi.A, ai_l), aj = mulA(Fj.A, aj_l);
    if (Jq) {
        double Bi[3][4], Bj[3][4], wi[4], wj[4];
        Bm(Fi.p, ai_l, Bi);
        Bm(Fj.p, aj_l, Bj);
        aTB(aj, Bi, wi);
        aTB(ai, Bj, wj);
        add_jac(*Jq, ncol, row, bi, v3(0, 0, 0), wi);
        add_jac(*Jq, ncol, row, bj, v3(0, 0, 0), wj);
    }
    return dot(ai, aj);
}

// dot-2 constraint a_i . d, d = r_j + A_j s_j - r_i - A_i s_i
double dot2(const Frame& Fi, V3 ai_l, V3 si_l, const Frame& Fj, V3 sj_l, int bi, int bj, std::vector<double>* Jq,
            int ncol, int row)
{
    const V3 ai = mulA(Fi.A, ai_l);
    const V3 d = Fj.r + mulA(Fj.A, sj_l) - Fi.r - mulA(Fi.A, si_l);
    if (Jq) {
        double Ba[3][4], Bs[3][4], Bj[3][4], w1[4], w2[4], wi[4], wj[4];
        Bm(Fi.p, ai_l, Ba);
        Bm(Fi.p, si_l, Bs);
        Bm(Fj.p, sj_l, Bj);
        aTB(d, Ba, w1);
        aTB(ai, Bs, w2);
        for (int k = 0; k < 4; ++k) wi[k] = w1[k] - w2[k];
        aTB(ai, Bj, wj);
        add_jac(*Jq, ncol, row, bi, -1.0 * ai, wi);
        add_jac(*Jq, ncol, row, bj, ai, wj);
    }
    return dot(ai, d);
}

// Constraint values Phi (ncon) and, when Jq is given, the Jacobian
// Phi_q (ncon x mdim, row-major) at the bodies' current q and time t.
void constraints(const xdem_mbd* m, double t, std::vector<double>& Phi, std::vector<double>* Jq)
{
    const int nc = m->ncon(), nd = m->mdim();
    Phi.assign(nc, 0.0);
    if (Jq) Jq->assign((size_t)nc * nd, 0.0);
    int row = 0;
    for (const Joint& jt : m->joints) {
        const Frame Fi = frame(m, jt.i), Fj = frame(m, jt.j);
        if (jt.kind == kRevolute) {
            // spherical part: r_i + A_i s_i - r_j - A_j s_j
            const V3 c = Fi.r + mulA(Fi.A, jt.si) - Fj.r - mulA(Fj.A, jt.sj);
            const double cv[3] = {c.x, c.y, c.z};
            double Bi[3][4], Bj[3][4];
            Bm(Fi.p, jt.si, Bi);
            Bm(Fj.p, jt.sj, Bj);
            for (int k = 0; k < 3; ++k) {
                Phi[row] = cv[k];
                if (Jq) {
                    const V3 e = v3(k == 0, k == 1, k == 2);
                    double wi[4], wj[4];
                    for (int q = 0; q < 4; ++q) { wi[q] = Bi[k][q]; wj[q] = -Bj[k][q]; }
                    add_jac(*Jq, nd, row, jt.i, e, wi);
                    add_jac(*Jq, nd, row, jt.j, -1.0 * e, wj);
                }
                ++row;
            }
            Phi[row] = dot1(Fi, jt.fi, Fj, jt.hj, jt.i, jt.j, Jq, nd, row); ++row;
            Phi[row] = dot1(Fi, jt.gi, Fj, jt.hj, jt.i, jt.j, Jq, nd, row); ++row;
        } else {
            // axis parallel, no motion across it, no rotation about it
            Phi[row] = dot1(Fi, jt.fi, Fj, jt.hj, jt.i, jt.j, Jq, nd, row); ++row;
            Phi[row] = dot1(Fi, jt.gi, Fj, jt.hj, jt.i, jt.j, Jq, nd, row); ++row;
            Phi[row] = dot2(Fi, jt.fi, jt.si, Fj, jt.sj, jt.i, jt.j, Jq, nd, row); ++row;
            Phi[row] = dot2(Fi, jt.gi, jt.si, Fj, jt.sj, jt.i, jt.j, Jq, nd, row); ++row;
            Phi[row] = dot1(Fi, jt.fi, Fj, jt.gj, jt.i, jt.j, Jq, nd, row); ++row;
        }
    }
    for (const Driver& d : m->drivers) {
        // rotation theta of body j about the joint axis, relative to body i:
        // cos theta = f_i . f_j, sin theta = g_i . f_j;
        // Phi = sin(th) (f_i . f_j) - cos(th) (g_i . f_j) = sin(th - theta)
        const Joint& jt = m->joints[d.joint];
        const Frame Fi = frame(m, jt.i), Fj = frame(m, jt.j);
        const double th = d.theta0 + d.omega * t;
        std::vector<double> tmp;
        std::vector<double>* Jrow = nullptr;
        if (Jq) {
            tmp.assign((size_t)2 * nd, 0.0);
            Jrow = &tmp;
        }
        const double c = dot1(Fi, jt.fi, Fj, jt.fj, jt.i, jt.j, Jrow, nd, 0);
        const double s = dot1(Fi, jt.gi, Fj, jt.fj, jt.i, jt.j, Jrow, nd, 1);
        Phi[row] = std::sin(th) * c - std::cos(th) * s;
        if (Jq)
            for (int k = 0; k < nd; ++k)
                (*Jq)[(size_t)row * nd + k] = std::sin(th) * tmp[k] - std::cos(th) * tmp[(size_t)nd + k];
        ++row;
    }
    for (size_t b = 1; b < m->bodies.size(); ++b) {
        const double* p = m->bodies[b].q + 3;
        Phi[row] = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3] - 1.0;
        if (Jq) {
            const double w[4] = {2 * p[0], 2 * p[1], 2 * p[2], 2 * p[3]};
            add_jac(*Jq, nd, row, (int)b, v3(0, 0, 0), w);
        }
        ++row;
    }
}

// Force vector (mdim): m g + F, and 2 E^T n + 8 G_dot^T J' G_dot p.
void force_vector(const xdem_mbd* m, std::vector<double>& f)
{
    f.assign(m->mdim(), 0.0);
    for (size_t b = 1; b < m->bodies.size(); ++b) {
        const Body& B = m->bodies[b];
        double* o = f.data() + off((int)b);
        const V3 fr = B.m * m->g + B.F;
        o[0] = fr.x; o[1] = fr.y; o[2] = fr.z;
        const M34 E = Em(B.q + 3);
        const M34 Gd = Gm(B.qd + 3);
        // G_dot p and J' (G_dot p)
        double gp[3];
        for (int r = 0; r < 3; ++r) {
            gp[r] = 0.0;
            for (int k = 0; k < 4; ++k) gp[r] += Gd.a[r][k] * B.q[3 + k];
        }
        const double Jg[3] = {B.J.x * gp[0], B.J.y * gp[1], B.J.z * gp[2]};
        const double n[3] = {B.N.x, B.N.y, B.N.z};
        for (int k = 0; k < 4; ++k) {
            double s = 0.0, t = 0.0;
            for (int r = 0; r < 3; ++r) {
                s += E.a[r][k] * n[r];
                t += Gd.a[r][k] * Jg[r];
            }
            o[3 + k] = 2.0 * s + 8.0 * t;
        }
    }
}

// Mass matrix times mul into the top-left block of the dense matrix L
// (ld columns), plus, when a is given, mul_j times d(M a)/dq of the
// rotational blocks: 4 (-G^T J' G(a) + Mm(J' G a)) (MassJacobian).
void mass_block(const xdem_mbd* m, double mul, const double* a, double mul_j, std::vector<double>& L, int ld)
{
    for (size_t b = 1; b < m->bodies.size(); ++b) {
        const Body& B = m->bodies[b];
        const int o = off((int)b);
        for (int k = 0; k < 3; ++k) L[(size_t)(o + k) * ld + o + k] += mul * B.m;
        const M34 G = Gm(B.q + 3);
        const double J[3] = {B.J.x, B.J.y, B.J.z};
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += G.a[k][r] * J[k] * G.a[k][c];
                L[(size_t)(o + 3 + r) * ld + o + 3 + c] += 4.0 * mul * s;
            }
        if (a) {
            const double* ar = a + o + 3;
            const M34 Ga = Gm(ar);
            double v[3];  // J' G(p) a
            for (int k = 0; k < 3; ++k) {
                double s = 0.0;
                for (int c = 0; c < 4; ++c) s += G.a[k][c] * ar[c];
                v[k] = J[k] * s;
            }
            // Mm(v) = d(G(p)^T v)/dp
            const double Mm[4][4] = {{0, -v[0], -v[1], -v[2]},
                                     {v[0], 0, v[2], -v[1]},
                                     {v[1], -v[2], 0, v[0]},
                                     {v[2], v[1], -v[0], 0}};
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) {
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k) s += G.a[k][r] * J[k] * Ga.a[k][c];
                    L[(size_t)(o + 3 + r) * ld + o + 3 + c] += 4.0 * mul_j * (-s + Mm[r][c]);
                }
        }
    }
}

// In-place dense solve of L x = b (n x n, row-major) by Gaussian
// elimination with partial pivoting; b becomes x.  Returns false when
// singular.
bool solve(std::vector<double>& L, std::vector<double>& b, int n)
{
    for (int c = 0; c < n; ++c) {
        int piv = c;
        double best = std::fabs(L[(size_t)c * n + c]);
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(L[(size_t)r * n + c]) > best) {
                best = std::fabs(L[(size_t)r * n + c]);
                piv = r;
            }
        if (!(best > 0.0) || !std::isfinite(best)) return false;
        if (piv != c) {
            for (int k = 0; k < n; ++k) std::swap(L[(size_t)c * n + k], L[(size_t)piv * n + k]);
            std::swap(b[c], b[piv]);
        }
        const double d = L[(size_t)c * n + c];
        for (int r = c + 1; r < n; ++r) {
            const double f = L[(size_t)r * n + c] / d;
            if (f == 0.0) continue;
            for (int k = c; k < n; ++k) L[(size_t)r * n + k] -= f * L[(size_t)c * n + k];
            b[r] -= f * b[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = b[r];
        for (int k = r + 1; k < n; ++k) s -= L[(size_t)r * n + k] * b[k];
        b[r] = s / L[(size_t)r * n + r];
    }
    return true;
}

// Assembles [mul_m M + d(M a)/dq mul_j, Phi_q^T; Phi_q, 0].
void system_matrix(const xdem_mbd* m, double mul_m, const double* a, double mul_j, const std::vector<double>& Jq,
                   std::vector<double>& L)
{
    const int nd = m->mdim(), nc = m->ncon(), n = nd + nc;
    L.assign((size_t)n * n, 0.0);
    mass_block(m, mul_m, a, mul_j, L, n);
    for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nd; ++c) {
            const double v = Jq[(size_t)r * nd + c];
            L[(size_t)(nd + r) * n + c] = v;
            L[(size_t)c * n + nd + r] = v;
        }
}

void unit_normals(V3 h, V3& f, V3& g)
{
    // f: the coordinate axis least aligned with h, made normal to it
    const double ax = std::fabs(h.x), ay = std::fabs(h.y), az = std::fabs(h.z);
    V3 e = ax <= ay && ax <= az ? v3(1, 0, 0) : (ay <= az ? v3(0, 1, 0) : v3(0, 0, 1));
    f = e - dot(e, h) * h;
    f = (1.0 / norm(f)) * f;
    g = cross(h, f);
}

}  // namespace

extern "C" {

XDEM_API int xdem_mbd_create(double dt, double alpha, const double gravity[3], xdem_mbd** out)
{
    if (!out || !(dt > 0.0) || !(alpha >= -1.0 / 3.0 && alpha <= 0.0)) return XDEM_ERR_ARG;
    xdem_mbd* m = new (std::nothrow) xdem_mbd();
    if (!m) return XDEM_ERR_ALLOC;
    m->dt = dt;
    m->alpha = alpha;
    m->beta = (1.0 - alpha) * (1.0 - alpha) / 4.0;
    m->gamma = 0.5 - alpha;
    if (gravity) m->g = v3(gravity[0], gravity[1], gravity[2]);
    m->bodies.resize(1);  // the ground
    *out = m;
    return XDEM_OK;
}

XDEM_API int xdem_mbd_destroy(xdem_mbd* m)
{
    if (!m) return XDEM_ERR_ARG;
    delete m;
    return XDEM_OK;
}

XDEM_API int xdem_mbd_set_tolerance(xdem_mbd* m, double eps)
{
    if (!m || !(eps > 0.0)) return XDEM_ERR_ARG;
    m->eps = eps;
    return XDEM_OK;
}

XDEM_API int xdem_mbd_add_body(xdem_mbd* m, double mass, const double inertia[3], const double pos[3],
                               const double ep[4], const double vel[3], const double ed[4], int* body)
{
    if (!m || m->ready || !(mass > 0.0) || !inertia || !pos || !ep) return XDEM_ERR_ARG;
    if (!(inertia[0] > 0.0 && inertia[1] > 0.0 && inertia[2] > 0.0)) return XDEM_ERR_ARG;
    Body b;
    b.m = mass;
    b.J = v3(inertia[0], inertia[1], inertia[2]);
    const double n = std::sqrt(ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2] + ep[3] * ep[3]);
    if (!(n > 0.0)) return XDEM_ERR_ARG;
    for (int k = 0; k < 3; ++k) b.q[k] = pos[k];
    for (int k = 0; k < 4; ++k) b.q[3 + k] = ep[k] / n;
    if (vel)
        for (int k = 0; k < 3; ++k) b.qd[k] = vel[k];
    if (ed)
        for (int k = 0; k < 4; ++k) b.qd[3 + k] = ed[k];
    m->bodies.push_back(b);
    if (body) *body = (int)m->bodies.size() - 1;
    return XDEM_OK;
}

// Joint between bodies i and j (0 = ground) at the global point loc with
// global axis dir, at the bodies' present poses.
static int add_joint(xdem_mbd* m, int kind, int i, int j, const double loc[3], const double dir[3], int* joint)
{
    const int nb = (int)m->bodies.size();
    if (m->ready || i < 0 || j < 0 || i >= nb || j >= nb || i == j || !loc || !dir) return XDEM_ERR_ARG;
    V3 h = vec(dir);
    const double hn = norm(h);
    if (!(hn > 0.0)) return XDEM_ERR_ARG;
    h = (1.0 / hn) * h;
    V3 f, g;
    unit_normals(h, f, g);
    const Frame Fi = frame(m, i), Fj = frame(m, j);
    Joint jt;
    jt.kind = kind;
    jt.i = i;
    jt.j = j;
    const V3 P = vec(loc);
    jt.si = mulAT(Fi.A, P - Fi.r);
    jt.sj = mulAT(Fj.A, P - Fj.r);
    jt.hi = mulAT(Fi.A, h);
    jt.hj = mulAT(Fj.A, h);
    jt.fi = mulAT(Fi.A, f);
    jt.gi = mulAT(Fi.A, g);
    jt.fj = mulAT(Fj.A, f);
    jt.gj = mulAT(Fj.A, g);
    m->joints.push_back(jt);
    if (joint) *joint = (int)m->joints.size() - 1;
    return XDEM_OK;
}

XDEM_API int xdem_mbd_add_revolute(xdem_mbd* m, int body_i, int body_j, const double loc[3], const double axis[3],
                                   int* joint)
{
    if (!m) return XDEM_ERR_ARG;
    return add_joint(m, kRevolute, body_i, body_j, loc, axis, joint);
}

XDEM_API int xdem_mbd_add_translational(xdem_mbd* m, int body_i, int body_j, const double loc[3],
                                        const double axis[3], int* joint)
{
    if (!m) return XDEM_ERR_ARG;
    return add_joint(m, kTranslational, body_i, body_j, loc, axis, joint);
}

XDEM_API int xdem_mbd_add_rotation_driver(xdem_mbd* m, int revolute_joint, double omega)
{
    if (!m || m->ready || revolute_joint < 0 || revolute_joint >= (int)m->joints.size() ||
        m->joints[revolute_joint].kind != kRevolute)
        return XDEM_ERR_ARG;
    // the driver starts from the joint's present angle (zero at definition)
    m->drivers.push_back(Driver{revolute_joint, omega, 0.0});
    return XDEM_OK;
}

// Consistent initial accelerations and multipliers (xIntegratorHHT::
// Initialize): [M, Phi_q^T; Phi_q, 0] (q_dd, lambda) = (F, 0).
XDEM_API int xdem_mbd_initialize(xdem_mbd* m)
{
    if (!m || m->bodies.size() < 2) return XDEM_ERR_ARG;
    const int nd = m->mdim(), nc = m->ncon(), n = nd + nc;
    if (nc > nd) return XDEM_ERR_ARG;
    std::vector<double> Phi, Jq, L, f;
    constraints(m, m->t, Phi, &Jq);
    force_vector(m, f);
    system_matrix(m, 1.0, nullptr, 0.0, Jq, L);
    std::vector<double> x(n, 0.0);
    for (int k = 0; k < nd; ++k) x[k] = f[k];
    if (!solve(L, x, n)) return XDEM_ERR_ARG;
    for (size_t b = 1; b < m->bodies.size(); ++b)
        for (int k = 0; k < 7; ++k) m->bodies[b].qdd[k] = x[off((int)b) + k];
    m->lambda.assign(x.begin() + nd, x.end());
    m->ready = true;
    return XDEM_OK;
}

// The contact force and moment (global frame) acting on a body until they
// are replaced: the DEM wrench of xdem_sim_body_wrench(es).
XDEM_API int xdem_mbd_set_contact_wrench(xdem_mbd* m, int body, const double w6[6])
{
    if (!m || body < 1 || body >= (int)m->bodies.size() || !w6) return XDEM_ERR_ARG;
    m->bodies[body].F = v3(w6[0], w6[1], w6[2]);
    m->bodies[body].N = v3(w6[3], w6[4], w6[5]);
    return XDEM_OK;
}

XDEM_API int xdem_mbd_step(xdem_mbd* m, int* iterations)
{
    if (!m || !m->ready) return XDEM_ERR_ARG;
    const int nd = m->mdim(), nc = m->ncon(), n = nd + nc;
    const double dt = m->dt, a = m->alpha, b = m->beta, g = m->gamma;
    const double divalpha = 1.0 / (1.0 + a);
    std::vector<double> Phi, Jq, L, f, x(n), ee(n);
    // ---- prediction (xIntegratorHHT::PredictionStep)
    constraints(m, m->t, Phi, &Jq);
    force_vector(m, f);
    m->pre.assign(nd, 0.0);
    for (int k = 0; k < nd; ++k) {
        double s = f[k];
        for (int r = 0; r < nc; ++r) s -= Jq[(size_t)r * nd + k] * m->lambda[r];
        m->pre[k] = a / (1.0 + a) * s;
    }
    m->ipp.assign(nd, 0.0);
    m->ipv.assign(nd, 0.0);
    for (size_t bb = 1; bb < m->bodies.size(); ++bb) {
        Body& B = m->bodies[bb];
        const int o = off((int)bb);
        for (int k = 0; k < 7; ++k) {
            m->ipp[o + k] = B.q[k] + dt * B.qd[k] + dt * dt * (1.0 - 2.0 * b) * 0.5 * B.qdd[k];
            m->ipv[o + k] = B.qd[k] + dt * (1.0 - g) * B.qdd[k];
            x[o + k] = B.qdd[k];
        }
    }
    for (int r = 0; r < nc; ++r) x[nd + r] = m->lambda[r];
    const double tn = m->t + dt;
    // a step that fails leaves the system as it was before the call
    const std::vector<Body> saved = m->bodies;
    auto fail = [&](int its) {
        m->bodies = saved;
        if (iterations) *iterations = its;
        return (int)XDEM_ERR_ARG;
    };
    auto place = [&]() {
        for (size_t bb = 1; bb < m->bodies.size(); ++bb) {
            Body& B = m->bodies[bb];
            const int o = off((int)bb);
            for (int k = 0; k < 7; ++k) {
                B.qdd[k] = x[o + k];
                B.q[k] = m->ipp[o + k] + b * dt * dt * x[o + k];
                B.qd[k] = m->ipv[o + k] + g * dt * x[o + k];
            }
        }
    };
    place();
    // ---- correction (xIntegratorHHT::CorrectionStep)
    int it = 0;
    while (true) {
        if (++it > 100) return fail(it - 1);  // no convergence
        constraints(m, tn, Phi, &Jq);
        force_vector(m, f);
        // ee = F - Phi_q^T lambda - M q_dd / (1 + alpha) - pre; -Phi / (beta dt^2)
        std::vector<double> Mx;
        {
            std::vector<double> Mm((size_t)nd * nd, 0.0);
            mass_block(m, divalpha, nullptr, 0.0, Mm, nd);
            Mx.assign(nd, 0.0);
            for (int r = 0; r < nd; ++r)
                for (int c = 0; c < nd; ++c) Mx[r] += Mm[(size_t)r * nd + c] * x[c];
        }
        for (int k = 0; k < nd; ++k) {
            double s = f[k] - Mx[k] - m->pre[k];
            for (int r = 0; r < nc; ++r) s -= Jq[(size_t)r * nd + k] * x[nd + r];
            ee[k] = s;
        }
        for (int r = 0; r < nc; ++r) ee[nd + r] = -Phi[r] / (b * dt * dt);
        double e2 = 0.0;
        for (int k = 0; k < n; ++k) e2 += ee[k] * ee[k];
        const double enorm = std::sqrt(e2);
        system_matrix(m, divalpha, x.data(), divalpha * b * dt * dt, Jq, L);
        if (!solve(L, ee, n)) return fail(it);
        for (int k = 0; k < n; ++k) x[k] += ee[k];
        place();
        if (enorm <= m->eps) break;
    }
    m->lambda.assign(x.begin() + nd, x.end());
    m->t = tn;
    m->last_iterations = it;
    if (iterations) *iterations = it;
    return XDEM_OK;
}

// q (7: r, p), q_dot and q_dd of a body; NULL skips.
XDEM_API int xdem_mbd_get_body(xdem_mbd* m, int body, double q[7], double qd[7], double qdd[7])
{
    if (!m || body < 1 || body >= (int)m->bodies.size()) return XDEM_ERR_ARG;
    const Body& B = m->bodies[body];
    if (q) std::memcpy(q, B.q, sizeof(B.q));
    if (qd) std::memcpy(qd, B.qd, sizeof(B.qd));
    if (qdd) std::memcpy(qdd, B.qdd, sizeof(B.qdd));
    return XDEM_OK;
}

// The body's 15-double record (mass, position, velocity, Euler parameters
// and their rates, decl:20) for xdem_sim_set_body(ies).
XDEM_API int xdem_mbd_body_record(xdem_mbd* m, int body, double rec[15])
{
    if (!m || body < 1 || body >= (int)m->bodies.size() || !rec) return XDEM_ERR_ARG;
    const Body& B = m->bodies[body];
    rec[XDEM_MM] = B.m;
    for (int k = 0; k < 3; ++k) {
        rec[XDEM_PX + k] = B.q[k];
        rec[XDEM_VX + k] = B.qd[k];
    }
    for (int k = 0; k < 4; ++k) {
        rec[XDEM_E0 + k] = B.q[3 + k];
        rec[XDEM_ED0 + k] = B.qd[3 + k];
    }
    return XDEM_OK;
}

// Time, Newton iterations of the last step, and the constraint count.
XDEM_API int xdem_mbd_info(xdem_mbd* m, double* time, int* iterations, int* nconstraint)
{
    if (!m) return XDEM_ERR_ARG;
    if (time) *time = m->t;
    if (iterations) *iterations = m->last_iterations;
    if (nconstraint) *nconstraint = m->ncon();
    return XDEM_OK;
}

// Multipliers of the constraints (ncon, in the order joints (5 each),
// drivers, Euler normalisations): the driver's multiplier is the torque
// the drive applies, up to the constraint's scaling.
XDEM_API int xdem_mbd_multipliers(xdem_mbd* m, double* lambda, int cap)
{
    if (!m || !lambda || cap < (int)m->lambda.size()) return XDEM_ERR_ARG;
    for (size_t k = 0; k < m->lambda.size(); ++k) lambda[k] = m->lambda[k];
    return XDEM_OK;
}

}  // extern "C"
