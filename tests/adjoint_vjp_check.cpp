// Host check of the hand-written VJPs of xdem_adjoint.cuh: for each forward
// function f and a random cotangent ly, the directional derivative of
// ly . f(x) along random directions d by central differences against
// (VJP ly) . d.  Prints one line "name max_relative_error" per check.
// The same forward pieces evaluated on dual numbers (the forward mode that
// xdem_adj_tangent runs) give ly . (J d) directly: "name_jvp" lines compare
// it with (VJP ly) . d and with the central differences.
// Built and run by tests/test_adjoint_math.py (g++, no GPU).
#include <cmath>
#include <cstdio>
#include <functional>
#include <random>
#include <vector>

#include "../xdynamics_dll_gb300/csrc/xdem_adjoint.cuh"

using namespace xdem::adj;
using Vec = std::vector<double>;

static std::mt19937_64 rng(12345);
static double nrm() { return std::normal_distribution<double>(0.0, 1.0)(rng); }
static double uni(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

// f(x, y); vjp(x, ly, lx) with lx zeroed by the caller
using Fwd = std::function<void(const Vec&, Vec&)>;
using Vjp = std::function<void(const Vec&, const Vec&, Vec&)>;

static double check(const char* name, const Vec& x, const Vec& scale, int nout, Fwd f, Vjp vjp, int ndir = 12)
{
    Vec ly(nout);
    Vec y0(nout);
    f(x, y0);
    for (int i = 0; i < nout; ++i) ly[i] = nrm();
    Vec lx(x.size(), 0.0);
    vjp(x, ly, lx);
    double worst = 0.0;
    for (int k = 0; k < ndir; ++k) {
        Vec d(x.size());
        for (size_t i = 0; i < x.size(); ++i) d[i] = scale[i] * nrm();
        const double h = 1e-6;
        Vec xp = x, xm = x, yp(nout), ym(nout);
        for (size_t i = 0; i < x.size(); ++i) {
            xp[i] += h * d[i];
            xm[i] -= h * d[i];
        }
        f(xp, yp);
        f(xm, ym);
        double fd = 0.0, an = 0.0, mag = 0.0;
        for (int i = 0; i < nout; ++i) fd += ly[i] * (yp[i] - ym[i]) / (2.0 * h);
        for (size_t i = 0; i < x.size(); ++i) {
            an += lx[i] * d[i];
            mag += std::fabs(lx[i] * d[i]);
        }
        const double err = std::fabs(fd - an) / std::max(std::max(std::fabs(fd), std::fabs(an)), 1e-300);
        // a cancelling directional derivative is judged against its terms
        const double err2 = std::fabs(fd - an) / std::max(mag, 1e-300);
        worst = std::max(worst, std::min(err, err2 * 10.0));
    }
    std::printf("%s %.3e\n", name, worst);
    return worst;
}

// Dual-number counterpart of check: for each random direction d the
// tangent ly . (J d) of fd (the forward on Dual<1> inputs x + eps d) against
// (VJP ly) . d and against central differences of f.
using D1 = Dual<1>;
using DVec = std::vector<D1>;
using FwdD = std::function<void(const DVec&, DVec&)>;
static double jvp_check(const char* name, const Vec& x, const Vec& scale, int nout, Fwd f, FwdD fd, Vjp vjp,
                        int ndir = 12)
{
    Vec ly(nout);
    for (int i = 0; i < nout; ++i) ly[i] = nrm();
    Vec lx(x.size(), 0.0);
    vjp(x, ly, lx);
    double worst = 0.0;
    for (int k = 0; k < ndir; ++k) {
        Vec d(x.size());
        for (size_t i = 0; i < x.size(); ++i) d[i] = scale[i] * nrm();
        DVec xd(x.size()), yd(nout);
        for (size_t i = 0; i < x.size(); ++i) {
            xd[i] = D1(x[i]);
            xd[i].d[0] = d[i];
        }
        fd(xd, yd);
        double jv = 0.0, jmag = 0.0, vj = 0.0, vmag = 0.0;
        for (int i = 0; i < nout; ++i) {
            jv += ly[i] * yd[i].d[0];
            jmag += std::fabs(ly[i] * yd[i].d[0]);
        }
        for (size_t i = 0; i < x.size(); ++i) {
            vj += lx[i] * d[i];
            vmag += std::fabs(lx[i] * d[i]);
        }
        const double h = 1e-6;
        Vec xp = x, xm = x, yp(nout), ym(nout);
        for (size_t i = 0; i < x.size(); ++i) {
            xp[i] += h * d[i];
            xm[i] -= h * d[i];
        }
        f(xp, yp);
        f(xm, ym);
        double fdd = 0.0;
        for (int i = 0; i < nout; ++i) fdd += ly[i] * (yp[i] - ym[i]) / (2.0 * h);
        // a cancelling directional derivative is judged against its terms
        const double mag = std::max(std::max(jmag, vmag), 1e-300);
        const double e1 = std::fabs(jv - vj) / mag;
        const double e2 = std::min(std::fabs(jv - fdd) / std::max(std::fabs(jv), 1e-300),
                                   10.0 * std::fabs(jv - fdd) / mag);
        worst = std::max(worst, std::max(e1, e2));
    }
    std::printf("%s_jvp %.3e\n", name, worst);
    return worst;
}
template <class T> static VT<T> gv(const std::vector<T>& x, int o) { return VT<T>{x[o], x[o + 1], x[o + 2]}; }
template <class T> static QT<T> gq(const std::vector<T>& x, int o) { return QT<T>{x[o], x[o + 1], x[o + 2], x[o + 3]}; }
template <class T> static void pv(std::vector<T>& y, int o, VT<T> v) { y[o] = v.x; y[o + 1] = v.y; y[o + 2] = v.z; }
template <class T> static void pq(std::vector<T>& y, int o, QT<T> q)
{
    y[o] = q.x; y[o + 1] = q.y; y[o + 2] = q.z; y[o + 3] = q.w;
}

static Q getq(const Vec& x, int o) { return mkq(x[o], x[o + 1], x[o + 2], x[o + 3]); }
static V getv(const Vec& x, int o) { return mkv(x[o], x[o + 1], x[o + 2]); }
static void putq(Vec& y, int o, Q q) { y[o] = q.x; y[o + 1] = q.y; y[o + 2] = q.z; y[o + 3] = q.w; }
static void putv(Vec& y, int o, V v) { y[o] = v.x; y[o + 1] = v.y; y[o + 2] = v.z; }
static void addq_to(Vec& y, int o, Q q) { y[o] += q.x; y[o + 1] += q.y; y[o + 2] += q.z; y[o + 3] += q.w; }
static void addv_to(Vec& y, int o, V v) { y[o] += v.x; y[o + 1] += v.y; y[o + 2] += v.z; }

static Q rand_unit_q()
{
    Q e = mkq(nrm(), nrm(), nrm(), nrm());
    return normalize(e);
}

// ------------------------------------------------------------ Euler parameters
static void euler_checks()
{
    {
        Vec x(8);
        putq(x, 0, rand_unit_q());
        putq(x, 4, mkq(nrm(), nrm(), nrm(), nrm()));
        check("ang_vel", x, Vec(8, 1.0), 3,
              [](const Vec& x, Vec& y) { putv(y, 0, ang_vel(getq(x, 0), getq(x, 4))); },
              [](const Vec& x, const Vec& ly, Vec& lx) {
                  Q le = mkq(0, 0, 0, 0), ld = mkq(0, 0, 0, 0);
                  ang_vel_vjp(getq(x, 0), getq(x, 4), getv(ly, 0), le, ld);
                  addq_to(lx, 0, le);
                  addq_to(lx, 4, ld);
              });
        jvp_check("ang_vel", x, Vec(8, 1.0), 3,
                  [](const Vec& x, Vec& y) { putv(y, 0, ang_vel(getq(x, 0), getq(x, 4))); },
                  [](const DVec& x, DVec& y) { pv(y, 0, ang_vel(gq(x, 0), gq(x, 4))); },
                  [](const Vec& x, const Vec& ly, Vec& lx) {
                      Q le = mkq(0, 0, 0, 0), ld = mkq(0, 0, 0, 0);
                      ang_vel_vjp(getq(x, 0), getq(x, 4), getv(ly, 0), le, ld);
                      addq_to(lx, 0, le);
                      addq_to(lx, 4, ld);
                  });
    }
    {
        Vec x(7);
        putv(x, 0, mkv(nrm(), nrm(), nrm()));
        putq(x, 3, rand_unit_q());
        check("to_local", x, Vec(7, 1.0), 3,
              [](const Vec& x, Vec& y) { putv(y, 0, to_local(getv(x, 0), getq(x, 3))); },
              [](const Vec& x, const Vec& ly, Vec& lx) {
                  V lm = mkv(0, 0, 0);
                  Q le = mkq(0, 0, 0, 0);
                  to_local_vjp(getv(x, 0), getq(x, 3), getv(ly, 0), lm, le);
                  addv_to(lx, 0, lm);
                  addq_to(lx, 3, le);
              });
        jvp_check("to_local", x, Vec(7, 1.0), 3,
                  [](const Vec& x, Vec& y) { putv(y, 0, to_local(getv(x, 0), getq(x, 3))); },
                  [](const DVec& x, DVec& y) { pv(y, 0, to_local(gv(x, 0), gq(x, 3))); },
                  [](const Vec& x, const Vec& ly, Vec& lx) {
                      V lm = mkv(0, 0, 0);
                      Q le = mkq(0, 0, 0, 0);
                      to_local_vjp(getv(x, 0), getq(x, 3), getv(ly, 0), lm, le);
                      addv_to(lx, 0, lm);
                      addq_to(lx, 3, le);
                  });
    }
    for (int iso = 0; iso < 2; ++iso) {
        const V J = iso ? mkv(2.5e-9, 2.5e-9, 2.5e-9) : mkv(2.0e-9, 3.0e-9, 4.5e-9);
        Vec x(11);
        putq(x, 0, rand_unit_q());
        putq(x, 4, mkq(30 * nrm(), 30 * nrm(), 30 * nrm(), 30 * nrm()));
        putv(x, 8, mkv(1e-6 * nrm(), 1e-6 * nrm(), 1e-6 * nrm()));
        Vec sc(11, 1.0);
        for (int i = 4; i < 8; ++i) sc[i] = 30.0;
        for (int i = 8; i < 11; ++i) sc[i] = 1e-6;
        check(iso ? "uceom_isotropic" : "uceom", x, sc, 4,
              [J](const Vec& x, Vec& y) { putq(y, 0, uceom(J, getq(x, 0), getq(x, 4), getv(x, 8))); },
              [J](const Vec& x, const Vec& ly, Vec& lx) {
                  Q le = mkq(0, 0, 0, 0), ld = mkq(0, 0, 0, 0);
                  V ln = mkv(0, 0, 0);
                  uceom_vjp(J, getq(x, 0), getq(x, 4), getv(x, 8), getq(ly, 0), le, ld, ln);
                  addq_to(lx, 0, le);
                  addq_to(lx, 4, ld);
                  addv_to(lx, 8, ln);
              });
        jvp_check(iso ? "uceom_isotropic" : "uceom", x, sc, 4,
                  [J](const Vec& x, Vec& y) { putq(y, 0, uceom(J, getq(x, 0), getq(x, 4), getv(x, 8))); },
                  [J](const DVec& x, DVec& y) { pq(y, 0, uceom(J, gq(x, 0), gq(x, 4), gv(x, 8))); },
                  [J](const Vec& x, const Vec& ly, Vec& lx) {
                      Q le = mkq(0, 0, 0, 0), ld = mkq(0, 0, 0, 0);
                      V ln = mkv(0, 0, 0);
                      uceom_vjp(J, getq(x, 0), getq(x, 4), getv(x, 8), getq(ly, 0), le, ld, ln);
                      addq_to(lx, 0, le);
                      addq_to(lx, 4, ld);
                      addv_to(lx, 8, ln);
                  });
        // the torque recovered from q
        const Q e = getq(x, 0), d = getq(x, 4);
        const V n = getv(x, 8);
        const V n2 = uceom_torque(J, e, d, uceom(J, e, d, n));
        const double rel = len(n2 - n) / len(n);
        std::printf("%s %.3e\n", iso ? "uceom_torque_isotropic" : "uceom_torque", rel);
    }
    {
        Vec x(4);
        putq(x, 0, 1.3 * rand_unit_q());
        check("normalize", x, Vec(4, 1.0), 4, [](const Vec& x, Vec& y) { putq(y, 0, normalize(getq(x, 0))); },
              [](const Vec& x, const Vec& ly, Vec& lx) {
                  Q le = mkq(0, 0, 0, 0);
                  normalize_vjp(getq(x, 0), getq(ly, 0), le);
                  addq_to(lx, 0, le);
              });
        jvp_check("normalize", x, Vec(4, 1.0), 4, [](const Vec& x, Vec& y) { putq(y, 0, normalize(getq(x, 0))); },
                  [](const DVec& x, DVec& y) { pq(y, 0, normalize(gq(x, 0))); },
                  [](const Vec& x, const Vec& ly, Vec& lx) {
                      Q le = mkq(0, 0, 0, 0);
                      normalize_vjp(getq(x, 0), getq(ly, 0), le);
                      addq_to(lx, 0, le);
                  });
    }
}

// ------------------------------------------------------------ contacts
static const double kE = 1e7, kNu = 0.3, kRest = 0.3;

static Mat material(int model)
{
    Mat m;
    m.Eeq = (kE * kE) / (kE * (1 - kNu * kNu) + kE * (1 - kNu * kNu));
    const double Seq = 1.0 / (2.0 * (2.0 * (2.0 - kNu) * (1.0 + kNu) / kE));
    m.Seq8 = 8.0 * Seq;
    const double lne = std::log(kRest);
    m.beta = -lne * std::sqrt(1.0 / (lne * lne + M_PI * M_PI));
    m.sratio = 0.3;
    m.vs1 = model == 1 ? 2.0 * std::sqrt(5.0 / 6.0) * m.beta : m.beta * m.sratio;
    m.fric = 0.4;
    return m;
}
static void put_mat(Vec& x, int o, const Mat& m)
{
    x[o] = m.Eeq; x[o + 1] = m.Seq8; x[o + 2] = m.beta; x[o + 3] = m.vs1; x[o + 4] = m.fric;
}
static Mat get_mat(const Vec& x, int o, double sratio)
{
    Mat m;
    m.Eeq = x[o]; m.Seq8 = x[o + 1]; m.beta = x[o + 2]; m.vs1 = x[o + 3]; m.fric = x[o + 4]; m.sratio = sratio;
    return m;
}
static void add_mat(Vec& lx, int o, const MatGrad& g)
{
    lx[o] += g.Eeq; lx[o + 1] += g.Seq8; lx[o + 2] += g.beta; lx[o + 3] += g.vs1; lx[o + 4] += g.fric;
}
static double sphere_mass(double r) { return 2500.0 * 4.0 / 3.0 * M_PI * r * r * r; }

// x = [xi vi wi | per partner: xj vj wj ds0 dots0 | Eeq Seq8 beta vs1 fric]
struct PPCase {
    int model, n;
    double ri;
    std::vector<double> rj;
};
static void pp_unpack(const PPCase& pc, const Vec& x, Body& bi, Body* nb, double* ds0, double* dots0)
{
    bi.x = getv(x, 0); bi.v = getv(x, 3); bi.w = getv(x, 6);
    bi.r = pc.ri; bi.m = sphere_mass(pc.ri);
    for (int s = 0; s < pc.n; ++s) {
        const int o = 9 + 11 * s;
        nb[s].x = getv(x, o); nb[s].v = getv(x, o + 3); nb[s].w = getv(x, o + 6);
        nb[s].r = pc.rj[s]; nb[s].m = sphere_mass(pc.rj[s]);
        ds0[s] = x[o + 9]; dots0[s] = x[o + 10];
    }
}

// pp_sphere_fwd on x in the scalar type T (the layout of pp_unpack).
template <class T>
static void pp_eval(const PPCase& pc, int model, double dt, const std::vector<T>& x, std::vector<T>& y)
{
    BodyT<T> bi, nb[kMaxPairs];
    T ds0[kMaxPairs], dots0[kMaxPairs], ds1[kMaxPairs], dots1[kMaxPairs];
    bi.x = gv(x, 0); bi.v = gv(x, 3); bi.w = gv(x, 6);
    bi.r = pc.ri; bi.m = sphere_mass(pc.ri);
    for (int s = 0; s < pc.n; ++s) {
        const int o = 9 + 11 * s;
        nb[s].x = gv(x, o); nb[s].v = gv(x, o + 3); nb[s].w = gv(x, o + 6);
        nb[s].r = pc.rj[s]; nb[s].m = sphere_mass(pc.rj[s]);
        ds0[s] = x[o + 9]; dots0[s] = x[o + 10];
    }
    const int k = 9 + 11 * pc.n;
    MatT<T> m;
    m.Eeq = x[k]; m.Seq8 = x[k + 1]; m.beta = x[k + 2]; m.vs1 = x[k + 3]; m.fric = x[k + 4]; m.sratio = T(0.3);
    VT<T> F = vzero<T>(), M = vzero<T>();
    pp_sphere_fwd(model, dt, m, bi, nb, ds0, dots0, pc.n, F, M, ds1, dots1);
    pv(y, 0, F);
    pv(y, 3, M);
    for (int s = 0; s < pc.n; ++s) { y[6 + s] = ds1[s]; y[6 + pc.n + s] = dots1[s]; }
}

static void pp_check(const char* name, int model, bool carry)
{
    PPCase pc;
    pc.model = model;
    pc.n = 5;
    pc.ri = 1e-3;
    const int nx = 9 + 11 * pc.n + 5;
    Vec x(nx, 0.0), sc(nx, 0.0);
    putv(x, 0, mkv(0.01, 0.02, 0.03));
    putv(x, 3, mkv(0.2 * nrm(), 0.2 * nrm(), 0.2 * nrm()));
    putv(x, 6, carry ? mkv(0, 0, 0) : mkv(20 * nrm(), 20 * nrm(), 20 * nrm()));
    for (int s = 0; s < pc.n; ++s) {
        const double rj = uni(1e-3, 2e-3);
        pc.rj.push_back(rj);
        V u = mkv(nrm(), nrm(), nrm());
        u = u / len(u);
        const double delta = s == 1 ? 1.2e-4 : uni(2e-6, 4e-5);
        const int o = 9 + 11 * s;
        putv(x, o, getv(x, 0) + (pc.ri + rj - delta) * u);
        const bool still = carry && s == 2;
        putv(x, o + 3, still ? getv(x, 3) : mkv(0.2 * nrm(), 0.2 * nrm(), 0.2 * nrm()));
        putv(x, o + 6, carry ? mkv(0, 0, 0) : mkv(20 * nrm(), 20 * nrm(), 20 * nrm()));
        x[o + 9] = s == 3 ? 2e-3 : uni(0.0, 5e-5);
        x[o + 10] = uni(0.0, 0.1);
    }
    const Mat m0 = material(model);
    put_mat(x, 9 + 11 * pc.n, m0);
    // directions: positions on the contact scale, velocities, spins, history;
    // with a kept force the velocities that make it exactly zero stay fixed
    for (int i = 0; i < 3; ++i) { sc[i] = 1e-5; sc[3 + i] = carry ? 0.0 : 0.1; sc[6 + i] = carry ? 0.0 : 10.0; }
    for (int s = 0; s < pc.n; ++s) {
        const int o = 9 + 11 * s;
        const bool still = carry && s == 2;
        for (int i = 0; i < 3; ++i) {
            sc[o + i] = 1e-5;
            sc[o + 3 + i] = still ? 0.0 : 0.1;
            sc[o + 6 + i] = carry ? 0.0 : 10.0;
        }
        sc[o + 9] = 1e-5;
        sc[o + 10] = 0.01;
    }
    for (int i = 0; i < 5; ++i) sc[9 + 11 * pc.n + i] = x[9 + 11 * pc.n + i];
    const int nout = 6 + 2 * pc.n;
    const double dt = 5e-6;
    auto f = [pc, model, dt](const Vec& x, Vec& y) {
        Body bi, nb[kMaxPairs];
        double ds0[kMaxPairs], dots0[kMaxPairs], ds1[kMaxPairs], dots1[kMaxPairs];
        pp_unpack(pc, x, bi, nb, ds0, dots0);
        const Mat m = get_mat(x, 9 + 11 * pc.n, 0.3);
        V F = mkv(0, 0, 0), M = mkv(0, 0, 0);
        pp_sphere_fwd(model, dt, m, bi, nb, ds0, dots0, pc.n, F, M, ds1, dots1);
        putv(y, 0, F);
        putv(y, 3, M);
        for (int s = 0; s < pc.n; ++s) { y[6 + s] = ds1[s]; y[6 + pc.n + s] = dots1[s]; }
    };
    auto vjp = [pc, model, dt](const Vec& x, const Vec& ly, Vec& lx) {
        Body bi, nb[kMaxPairs];
        double ds0[kMaxPairs], dots0[kMaxPairs], lds1[kMaxPairs], ldots1[kMaxPairs];
        double lds0[kMaxPairs] = {}, ldots0[kMaxPairs] = {};
        V lxj[kMaxPairs] = {}, lvj[kMaxPairs] = {}, lwj[kMaxPairs] = {};
        pp_unpack(pc, x, bi, nb, ds0, dots0);
        const Mat m = get_mat(x, 9 + 11 * pc.n, 0.3);
        for (int s = 0; s < pc.n; ++s) { lds1[s] = ly[6 + s]; ldots1[s] = ly[6 + pc.n + s]; }
        V lxi = mkv(0, 0, 0), lvi = mkv(0, 0, 0), lwi = mkv(0, 0, 0);
        MatGrad g{0, 0, 0, 0, 0};
        pp_sphere_vjp(model, dt, m, bi, nb, ds0, dots0, pc.n, getv(ly, 0), getv(ly, 3), lds1, ldots1, lxi, lvi, lwi,
                      lxj, lvj, lwj, lds0, ldots0, g);
        addv_to(lx, 0, lxi); addv_to(lx, 3, lvi); addv_to(lx, 6, lwi);
        for (int s = 0; s < pc.n; ++s) {
            const int o = 9 + 11 * s;
            addv_to(lx, o, lxj[s]); addv_to(lx, o + 3, lvj[s]); addv_to(lx, o + 6, lwj[s]);
            lx[o + 9] += lds0[s]; lx[o + 10] += ldots0[s];
        }
        add_mat(lx, 9 + 11 * pc.n, g);
    };
    // report the regimes the case covers (stick a < b, slip, kept Ft)
    {
        Body bi, nb[kMaxPairs];
        double ds0[kMaxPairs], dots0[kMaxPairs];
        pp_unpack(pc, x, bi, nb, ds0, dots0);
        int stick = 0, slip = 0, kept = 0;
        for (int s = 0; s < pc.n; ++s) {
            PairGeom pg;
            pair_geom(bi.x, nb[s].x, bi.r, nb[s].r, pg);
            Core c;
            core_consts(m0, model, bi.r, nb[s].r, bi.m, nb[s].m, c);
            c.delta = pg.delta; c.u = pg.u;
            c.rv = rel_vel(bi.v, bi.w, pg.di, nb[s].v, nb[s].w, pg.dj);
            c.ds0 = ds0[s]; c.dots0 = dots0[s];
            core_fwd(model, dt, c);
            if (!c.tang) kept++;
            else if (c.a < c.b) stick++;
            else slip++;
        }
        std::printf("# %s stick %d slip %d kept %d\n", name, stick, slip, kept);
    }
    check(name, x, sc, nout, f, vjp);
    jvp_check(name, x, sc, nout, f, [pc, model, dt](const DVec& x, DVec& y) { pp_eval(pc, model, dt, x, y); }, vjp);
}

// plane_contact_fwd_t on x in the scalar type T (the layout of plane_check).
template <class T>
static void plane_eval(const PlaneContact& pc, int model, double r, double dt, const std::vector<T>& x,
                       std::vector<T>& y)
{
    MatT<T> m;
    m.Eeq = x[11]; m.Seq8 = x[12]; m.beta = x[13]; m.vs1 = x[14]; m.fric = x[15]; m.sratio = T(0.3);
    BodyT<T> bi{gv(x, 0), gv(x, 3), gv(x, 6), r, sphere_mass(r)};
    VT<T> F = vzero<T>(), M = vzero<T>();
    T ds1, dots1;
    plane_contact_fwd_t(model, dt, pc, m, bi, x[9], x[10], F, M, ds1, dots1);
    pv(y, 0, F);
    pv(y, 3, M);
    y[6] = ds1;
    y[7] = dots1;
}

static void plane_check(const char* name, int model, V pos)
{
    PlaneContact pc;
    pc.rect.xw = mkv(0, 0, 0);
    pc.rect.u1 = mkv(0, 0, 1);
    pc.rect.u2 = mkv(1, 0, 0);
    pc.rect.uw = mkv(0, 1, 0);
    pc.rect.l1 = 0.1;
    pc.rect.l2 = 0.1;
    pc.rect.w2 = mkv(0, 0, 0.1);
    pc.rect.w3 = mkv(0.1, 0, 0.1);
    pc.rect.w4 = mkv(0.1, 0, 0);
    pc.bp = mkv(0.05, 0.0, 0.05);
    pc.bv = mkv(0.01, 0.0, -0.02);
    pc.bw = mkv(0.0, 0.5, 0.0);
    pc.mat = material(model);
    const double r = 1e-3, dt = 5e-6;
    Vec x(16, 0.0), sc(16, 0.0);
    putv(x, 0, pos);
    putv(x, 3, mkv(0.2 * nrm(), 0.2 * nrm(), 0.2 * nrm()));
    putv(x, 6, mkv(20 * nrm(), 20 * nrm(), 20 * nrm()));
    x[9] = uni(0.0, 5e-5);
    x[10] = uni(0.0, 0.1);
    put_mat(x, 11, pc.mat);
    for (int i = 0; i < 3; ++i) { sc[i] = 1e-5; sc[3 + i] = 0.1; sc[6 + i] = 10.0; }
    sc[9] = 1e-5;
    sc[10] = 0.01;
    for (int i = 0; i < 5; ++i) sc[11 + i] = x[11 + i];
    PlaneGeom pg;
    plane_geom(pc.rect, pos, r, pg);
    std::printf("# %s region %d delta %.3e\n", name, pg.region, pg.delta);
    auto f = [pc, model, r, dt](const Vec& x, Vec& y) {
        PlaneContact p = pc;
        p.mat = get_mat(x, 11, 0.3);
        Body bi{getv(x, 0), getv(x, 3), getv(x, 6), r, sphere_mass(r)};
        V F = mkv(0, 0, 0), M = mkv(0, 0, 0);
        double ds1, dots1;
        plane_contact_fwd(model, dt, p, bi, x[9], x[10], F, M, ds1, dots1);
        putv(y, 0, F);
        putv(y, 3, M);
        y[6] = ds1;
        y[7] = dots1;
    };
    auto vjp = [pc, model, r, dt](const Vec& x, const Vec& ly, Vec& lx) {
        PlaneContact p = pc;
        p.mat = get_mat(x, 11, 0.3);
        Body bi{getv(x, 0), getv(x, 3), getv(x, 6), r, sphere_mass(r)};
        V l0 = mkv(0, 0, 0), l1 = mkv(0, 0, 0), l2 = mkv(0, 0, 0);
        double lds0 = 0.0, ldots0 = 0.0;
        MatGrad g{0, 0, 0, 0, 0};
        plane_contact_vjp(model, dt, p, bi, x[9], x[10], getv(ly, 0), getv(ly, 3), ly[6], ly[7], l0, l1, l2, lds0,
                          ldots0, g);
        addv_to(lx, 0, l0); addv_to(lx, 3, l1); addv_to(lx, 6, l2);
        lx[9] += lds0; lx[10] += ldots0;
        add_mat(lx, 11, g);
    };
    check(name, x, sc, 8, f, vjp);
    jvp_check(name, x, sc, 8, f, [pc, model, r, dt](const DVec& x, DVec& y) { plane_eval(pc, model, r, dt, x, y); },
              vjp);
}

int main()
{
    euler_checks();
    pp_check("pp_hm", 1, false);
    pp_check("pp_dhs", 0, false);
    pp_check("pp_hm_kept_ft", 1, true);
    plane_check("plane_face_hm", 1, mkv(0.05, 1e-3 - 1.5e-5, 0.04));
    plane_check("plane_face_dhs", 0, mkv(0.05, 1e-3 - 1.5e-5, 0.04));
    plane_check("plane_edge_hm", 1, mkv(-0.0006, std::sqrt(9.9e-4 * 9.9e-4 - 0.0006 * 0.0006), 0.05));
    plane_check("plane_corner_hm", 1, mkv(-0.0004, 0.0007, -0.0004));
    return 0;
}
