/*
 * xdem_oracle.c -- CPU oracle of the xdynamics DEM step (test infrastructure).
 *
 * Restates include/xdynamics_parallel/xParallelDEM_impl.cuh ("impl") and the
 * launch order of source/xdynamics_simulation/xIntegratorVV.cpp of
 * miniwooki/xdynamics_dll in plain C.  Build with -ffp-contract=off so that
 * every product and sum is rounded on its own, in the order written; the
 * classification arithmetic of the GPU library (cell ids, distance tests,
 * plane and triangle regions) is written in the same order without FMA and
 * agrees bit for bit.
 */
#include "xdem_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------- vectors */
typedef struct { double x, y, z; } v3;
typedef struct { double x, y, z, w; } v4;

static inline v3 mk3(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v4 mk4(double x, double y, double z, double w) { v4 r = {x, y, z, w}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(double s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline v3 div3(v3 a, double s) { return mk3(a.x / s, a.y / s, a.z / s); }
static inline v3 neg3(v3 a) { return mk3(-a.x, -a.y, -a.z); }
static inline double dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double len3(v3 a) { return sqrt(dot3(a, a)); }
static inline v3 cross3(v3 a, v3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v4 add4(v4 a, v4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline v4 sub4(v4 a, v4 b) { return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline v4 mul4(double s, v4 a) { return mk4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline double dot4(v4 a, v4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

static inline v3 ld3(const double* a, size_t i) { return mk3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
static inline v4 ld4(const double* a, size_t i) { return mk4(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]); }
static inline v3 ld4xyz(const double* a, size_t i) { return mk3(a[4 * i], a[4 * i + 1], a[4 * i + 2]); }
static inline void st3(double* a, size_t i, v3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
static inline void st4(double* a, size_t i, v4 v) { a[4 * i] = v.x; a[4 * i + 1] = v.y; a[4 * i + 2] = v.z; a[4 * i + 3] = v.w; }
static inline void addto3(double* a, size_t i, v3 v) { a[3 * i] += v.x; a[3 * i + 1] += v.y; a[3 * i + 2] += v.z; }
static inline v3 dv3(xdem_double3 d) { return mk3(d.x, d.y, d.z); }

static void raise_status(unsigned int* status, unsigned int bits)
{
    if (!status || !bits) return;
#ifdef _OPENMP
#pragma omp atomic update
#endif
    *status |= bits;
}

int xo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void xo_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------ Euler parameters (impl:8-52) */
/* Rotation matrix rows of ep = (e0,e1,e2,e3) stored as (x,y,z,w). */
static inline void rot_rows(v4 e, v3* r0, v3* r1, v3* r2)
{
    *r0 = mk3(2.0 * (e.x * e.x + e.y * e.y - 0.5), 2.0 * (e.y * e.z - e.x * e.w), 2.0 * (e.y * e.w + e.x * e.z));
    *r1 = mk3(2.0 * (e.y * e.z + e.x * e.w), 2.0 * (e.x * e.x + e.z * e.z - 0.5), 2.0 * (e.z * e.w - e.x * e.y));
    *r2 = mk3(2.0 * (e.y * e.w - e.x * e.z), 2.0 * (e.z * e.w + e.x * e.y), 2.0 * (e.x * e.x + e.w * e.w - 0.5));
}
/* impl:8-18: A v */
static v3 to_global(v3 v, v4 e)
{
    v3 r0, r1, r2; rot_rows(e, &r0, &r1, &r2);
    return mk3(r0.x * v.x + r0.y * v.y + r0.z * v.z,
               r1.x * v.x + r1.y * v.y + r1.z * v.z,
               r2.x * v.x + r2.y * v.y + r2.z * v.z);
}
/* impl:20-30: A^T v */
static v3 to_local(v3 v, v4 e)
{
    v3 r0, r1, r2; rot_rows(e, &r0, &r1, &r2);
    return mk3(r0.x * v.x + r1.x * v.y + r2.x * v.z,
               r0.y * v.x + r1.y * v.y + r2.y * v.z,
               r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
/* impl:32-41: global angular velocity 2 G(e) e_dot */
static v3 ang_vel(v4 e, v4 d)
{
    v3 o = mk3(-e.y * d.x + e.x * d.y - e.w * d.z + e.z * d.w,
               -e.z * d.x + e.w * d.y + e.x * d.z - e.y * d.w,
               -e.w * d.x - e.z * d.y + e.y * d.z + e.x * d.w);
    return mul3(2.0, o);
}

/* ------------------------------------------------ grid (impl:54-72) */
static inline int floor_to_int(double v)
{
    double f = floor(v);
    if (f != f) return 0;                    /* NaN -> 0, as cvt.rzi */
    if (f >= 2147483647.0) return 2147483647;
    if (f <= -2147483648.0) return (-2147483647 - 1);
    return (int)f;
}
static inline void grid_pos(const device_dem_parameters* prm, v3 p, int g[3])
{
    g[0] = floor_to_int((p.x - prm->world_origin.x) / prm->cell_size);
    g[1] = floor_to_int((p.y - prm->world_origin.y) / prm->cell_size);
    g[2] = floor_to_int((p.z - prm->world_origin.z) / prm->cell_size);
}
static inline unsigned int grid_hash(const device_dem_parameters* prm, int gx, int gy, int gz)
{
    unsigned int x = (unsigned int)(gx & (int)(prm->grid_size.x - 1));
    unsigned int y = (unsigned int)(gy & (int)(prm->grid_size.y - 1));
    unsigned int z = (unsigned int)(gz & (int)(prm->grid_size.z - 1));
    return (z * prm->grid_size.y) * prm->grid_size.x + y * prm->grid_size.x + x;
}

/* ------------------------------------------------ uceom (impl:74-133) */
/* Solves [2 J_i L_i(e) ; e^T] q = rhs for the Euler-parameter acceleration,
 * by the explicit inverse (adjugate / determinant) as the reference does. */
static double det3(const double m[4][4], int r0, int r1, int r2, int c0, int c1, int c2)
{
    return m[r0][c0] * (m[r1][c1] * m[r2][c2] - m[r1][c2] * m[r2][c1])
         - m[r0][c1] * (m[r1][c0] * m[r2][c2] - m[r1][c2] * m[r2][c0])
         + m[r0][c2] * (m[r1][c0] * m[r2][c1] - m[r1][c1] * m[r2][c0]);
}
static v4 uceom(v3 J, v4 ep, v4 ev, v3 n)
{
    double l[4][4] = {
        {2.0 * J.x * (-ep.y), 2.0 * J.x * ep.x, 2.0 * J.x * ep.w, 2.0 * J.x * (-ep.z)},
        {2.0 * J.y * (-ep.z), 2.0 * J.y * (-ep.w), 2.0 * J.y * ep.x, 2.0 * J.y * ep.y},
        {2.0 * J.z * (-ep.w), 2.0 * J.z * ep.z, 2.0 * J.z * (-ep.y), 2.0 * J.z * ep.x},
        {ep.x, ep.y, ep.z, ep.w}};
    v3 T = mk3(J.x * (-ep.y * ev.x + ep.x * ev.y + ep.w * ev.z - ep.z * ev.w),
               J.y * (-ep.z * ev.x - ep.w * ev.y + ep.x * ev.z + ep.y * ev.w),
               J.z * (-ep.w * ev.x + ep.z * ev.y - ep.y * ev.z + ep.x * ev.w));
    v4 lh0 = mk4(4.0 * (-ev.y * T.x - ev.z * T.y - ev.w * T.z),
                 4.0 * (ev.x * T.x - ev.w * T.y + ev.z * T.z),
                 4.0 * (ev.w * T.x + ev.x * T.y - ev.y * T.z),
                 4.0 * (-ev.z * T.x + ev.y * T.y + ev.x * T.z));
    v3 lh = mk3(-ep.y * lh0.x + ep.x * lh0.y + ep.w * lh0.z - ep.z * lh0.w,
                -ep.z * lh0.x - ep.w * lh0.y + ep.x * lh0.z + ep.y * lh0.w,
                -ep.w * lh0.x + ep.z * lh0.y - ep.y * lh0.z + ep.x * lh0.w);
    double rhs[4] = {n.x - lh.x, n.y - lh.y, n.z - lh.z, 0.0 - dot4(ev, ev)};
    /* adjugate: adj[c][r] = (-1)^(r+c) minor(r,c) */
    double adj[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            int rr[3], cc[3], a = 0, b = 0;
            for (int i = 0; i < 4; ++i) if (i != r) rr[a++] = i;
            for (int j = 0; j < 4; ++j) if (j != c) cc[b++] = j;
            double m = det3(l, rr[0], rr[1], rr[2], cc[0], cc[1], cc[2]);
            adj[c][r] = ((r + c) & 1) ? -m : m;
        }
    double det = l[0][0] * adj[0][0] + l[0][1] * adj[1][0] + l[0][2] * adj[2][0] + l[0][3] * adj[3][0];
    double s = 1.0 / det;
    double q[4];
    for (int i = 0; i < 4; ++i)
        q[i] = s * (adj[i][0] * rhs[0] + adj[i][1] * rhs[1] + adj[i][2] * rhs[2] + adj[i][3] * rhs[3]);
    return mk4(q[0], q[1], q[2], q[3]);
}

/* ------------------------------------------------ contact constants (impl:362-386) */
typedef struct { double kn, vn, ks, vs, mu, mu_s, ms, eq_r, eq_m; } fconst;

static fconst get_constant(int model, double ir, double jr, double im, double jm,
                           double iE, double jE, double ip, double jp,
                           double rest, double fric, double s_fric, double rfric, double sratio)
{
    fconst c;
    double Meq = jm ? (im * jm) / (im + jm) : im;
    double Req = jr ? (ir * jr) / (ir + jr) : ir;
    double Eeq = (iE * jE) / (iE * (1 - jp * jp) + jE * (1 - ip * ip));
    double Seq = (2.0 * (2.0 - ip) * (1.0 + ip) / iE) + (2.0 * (2.0 - jp) * (1.0 + jp) / jE);
    Seq = 1.0 / Seq;
    double lne = log(rest);
    double beta = -lne * sqrt(1.0 / (lne * lne + M_PI * M_PI));
    c.eq_m = Meq;
    c.eq_r = Req;
    c.kn = (4.0 / 3.0) * Eeq * sqrt(Req);
    c.vn = beta;
    c.ks = model == 1 ? 8.0 * Seq : c.kn * sratio;
    c.vs = model == 1 ? 2.0 * sqrt(5.0 / 6.0) * beta : c.vn * sratio;
    c.mu = fric;
    c.mu_s = s_fric;
    c.ms = rfric;
    return c;
}

/* impl:388-413 */
static double cohesion_force(double ri, double rj, double Ei, double Ej, double pri, double prj,
                             double coh, double Fn)
{
    double cf = 0.0;
    if (coh) {
        double Req = rj ? (ri * rj) / (ri + rj) : ri;
        double Eeq = 1.0 / (((1.0 - pri * pri) / Ei) + ((1.0 - prj * prj) / Ej));
        double c0 = 3.0 * coh * M_PI * Req;
        double eq = 2.0 * c0 * Fn + c0 * c0;
        if (eq <= 0) Fn = -0.5 * c0;
        double a3 = (3.0 * Req) * (Fn + c0 + sqrt(fabs(2.0 * c0 * Fn + c0 * c0))) / (4.0 * Eeq);
        cf = -sqrt(8.0 * M_PI * coh * Eeq * a3);
    }
    return cf;
}
/* impl:415-423 */
static double limit_cohesion_depth(double ir, double jr, double iE, double jE, double ip, double jp, double coh)
{
    double Req = jr ? (ir * jr) / (ir + jr) : ir;
    double Eeq = 1.0 / (((1.0 - ip * ip) / iE) + ((1.0 - jp * jp) / jE));
    double c1 = (M_PI * M_PI * coh * coh * Req) / (Eeq * Eeq);
    return -(3.0 / 4.0) * pow(c1, 1.0 / 3.0);
}
/* impl:425-430 */
static double jkr_separation_force(double ir, double jr, double coh)
{
    double Req = jr ? (ir * jr) / (ir + jr) : ir;
    return -(3.0 / 2.0) * M_PI * coh * Req;
}

/* impl:432-474: Hertz-Mindlin (model 1) and DHS (model 0).  Ft is only
 * written when the tangential relative velocity is non-zero; callers keep the
 * previous value otherwise, as the reference kernels do. */
static void contact_model(int model, fconst c, double ir, double jr, const device_contact_property* cp,
                          double dt, double cdist, double* ds_io, double* dots_io,
                          v3 dv, v3 unit, v3* Ft, v3* Fn)
{
    double fsn = -c.kn * pow(cdist, 1.5);
    double fdn = c.vn * dot3(dv, unit);
    double fca = -cohesion_force(ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, fsn + fdn);
    *Fn = mul3(fsn + fca + fdn, unit);
    v3 e = sub3(dv, mul3(dot3(dv, unit), unit));
    double mag_e = len3(e);
    if (mag_e) {
        v3 s_hat = div3(e, mag_e);
        double s_dot = dot3(dv, s_hat);
        double ds = *ds_io + dt * (s_dot + *dots_io);
        *ds_io = ds;
        *dots_io = s_dot;
        double ft;
        if (model == 1) {
            double S_t = c.ks * sqrt(c.eq_r * cdist);
            double a = S_t * ds + c.vs * sqrt(S_t * c.eq_m);
            double b = c.mu * len3(*Fn);
            ft = a < b ? a : b;
        } else {
            double a = c.ks * ds + c.vs * (dot3(dv, s_hat));
            double b = c.mu * len3(*Fn);
            ft = a < b ? a : b;
        }
        *Ft = mul3(ft, s_hat);
    }
}

/* impl:476-483 */
static void rolling_accumulate(double rf, double ir, double jr, v3 rc, v3 Fn, v3 Ft, double* Mr, v3* Tmax)
{
    *Tmax = add3(*Tmax, cross3(rc, add3(Fn, Ft)));
    double Rij = jr ? ir * jr / (ir + jr) : ir;
    *Mr += Rij * rf * len3(Fn);
}

/* ======================================================================== */
/* VV                                                                        */
/* ======================================================================== */
void xo_vv_update_position(const device_dem_parameters* prm, double* pos, double* ep,
                           const double* vel, const double* ev, const double* acc,
                           const double* ea, unsigned int np)
{
    const double dt = prm->dt, h = prm->half2dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < (long)np; ++i) {
        v4 e = add4(add4(ld4(ep, i), mul4(dt, ld4(ev, i))), mul4(h, ld4(ea, i)));
        double l = sqrt(dot4(e, e));
        st4(ep, i, mk4(e.x / l, e.y / l, e.z / l, e.w / l));
        v3 d = add3(mul3(dt, ld3(vel, i)), mul3(h, ld3(acc, i)));
        pos[4 * i] += d.x; pos[4 * i + 1] += d.y; pos[4 * i + 2] += d.z;
    }
}

/* impl:192-222.  The reference GPU kernel writes `vel[id] = v` unchanged
 * (impl:208,218), so a free sphere never gains speed there.  vel_compat=1
 * reproduces that; vel_compat=0 applies the same trapezoid the kernel applies
 * to ev (impl:216) to the linear velocity, which is the velocity-Verlet update
 * of the CPU path (xIntegratorVV.cpp:143-149) and of the cluster kernel
 * (impl:279-284). */
void xo_vv_update_velocity(const device_dem_parameters* prm, double* vel, double* acc,
                           const double* ep, double* ev, double* ea, double* force,
                           double* moment, const double* mass, const double* iner,
                           unsigned int np, int vel_compat)
{
    const double hdt = 0.5 * prm->dt;
    const v3 g = dv3(prm->gravity);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < (long)np; ++i) {
        double m = mass[i];
        v3 v = ld3(vel, i);
        v4 e = ld4(ep, i);
        v4 av = ld4(ev, i);
        double inv = 1.0 / m;
        v3 F = ld3(force, i);
        v3 a = mul3(inv, add3(F, mul3(m, g)));
        v3 J = ld3(iner, i);
        v3 n = to_local(ld3(moment, i), e);
        v4 q = uceom(J, e, av, n);
        av = add4(av, mul4(hdt, add4(ld4(ea, i), q)));
        st3(force, i, mk3(0, 0, 0));
        st3(moment, i, mk3(0, 0, 0));
        if (!vel_compat) v = add3(v, mul3(hdt, add3(ld3(acc, i), a)));
        st3(vel, i, v);
        st4(ev, i, av);
        st3(acc, i, a);
        st4(ea, i, q);
    }
}

/* ======================================================================== */
/* Grid                                                                      */
/* ======================================================================== */
void xo_hash(const device_dem_parameters* prm, unsigned int* hash, unsigned int* index,
             const double* pos, unsigned int sid, unsigned int np, unsigned int* status)
{
    unsigned int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (long i = 0; i < (long)np; ++i) {
        v3 p = ld4xyz(pos, i);
        if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) bad |= XDEM_ERR_NONFINITE;
        int g[3]; grid_pos(prm, p, g);
        hash[sid + i] = grid_hash(prm, g[0], g[1], g[2]);
        index[sid + i] = sid + (unsigned int)i;
    }
    raise_status(status, bad);
}

/* Stable LSD radix sort of (key, value) by key, 8-bit digits. */
static void stable_sort_pairs(unsigned int* key, unsigned int* val, unsigned int n)
{
    if (n < 2) return;
    unsigned int* k2 = (unsigned int*)malloc(sizeof(unsigned int) * n);
    unsigned int* v2 = (unsigned int*)malloc(sizeof(unsigned int) * n);
    unsigned int maxk = 0;
    for (unsigned int i = 0; i < n; ++i) if (key[i] > maxk) maxk = key[i];
    unsigned int *ks = key, *vs = val, *kd = k2, *vd = v2;
    for (int shift = 0; shift < 32 && (shift == 0 || (maxk >> shift)); shift += 8) {
        size_t cnt[257] = {0};
        for (unsigned int i = 0; i < n; ++i) cnt[((ks[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (unsigned int i = 0; i < n; ++i) {
            size_t o = cnt[(ks[i] >> shift) & 255u]++;
            kd[o] = ks[i]; vd[o] = vs[i];
        }
        unsigned int* t;
        t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    if (ks != key) { memcpy(key, ks, sizeof(unsigned int) * n); memcpy(val, vs, sizeof(unsigned int) * n); }
    free(k2); free(v2);
}

void xo_reorder_cellstart(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                          unsigned int* cend, unsigned int* sorted_index, unsigned int n,
                          unsigned int ncell)
{
    stable_sort_pairs(hash, index, n);
    memset(cstart, 0xff, sizeof(unsigned int) * (size_t)ncell);
    memset(cend, 0, sizeof(unsigned int) * (size_t)ncell);
    for (unsigned int id = 0; id < n; ++id) {
        unsigned int h = hash[id];
        if (id == 0 || h != hash[id - 1]) {
            cstart[h] = id;
            if (id > 0) cend[hash[id - 1]] = id;
        }
        if (id == n - 1) cend[h] = id + 1;
        sorted_index[id] = index[id];
    }
}

/* ======================================================================== */
/* Particle-particle (impl:613-733)                                          */
/* ======================================================================== */
void xo_p2p(const device_dem_parameters* prm, const double* pos, const double* ep,
            const double* vel, const double* ev, double* force, double* moment,
            const double* mass, double* tmax, double* rres, unsigned int* pair_count,
            unsigned int* pair_id, double* tsd, const unsigned int* sorted_index,
            const unsigned int* cstart, const unsigned int* cend,
            const device_contact_property* cp, unsigned int np, unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2P_COUNT;
        unsigned int old_id[MAX_P2P_COUNT];
        double old_sd[MAX_P2P_COUNT][2];
        for (int i = 0; i < MAX_P2P_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        unsigned int old_count = pair_count[id];
        if (old_count > MAX_P2P_COUNT) old_count = MAX_P2P_COUNT;
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        v3 ivel = ld3(vel, id);
        v3 iom = ang_vel(ld4(ep, id), ld4(ev, id));
        int g[3]; grid_pos(prm, ipos, g);
        double ir = ip4.w, im = mass[id];
        v3 Ft = mk3(0, 0, 0), Fn = mk3(0, 0, 0);
        v3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = 0, bits = 0;
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    unsigned int h = grid_hash(prm, g[0] + x, g[1] + y, g[2] + z);
                    unsigned int start = cstart[h];
                    if (start == 0xffffffffu) continue;
                    unsigned int end = cend[h];
                    for (unsigned int j = start; j < end; ++j) {
                        unsigned int k = sorted_index[j];
                        if (id == k || k >= np) continue;
                        v4 jp4 = ld4(pos, k);
                        v3 jvel = ld3(vel, k);
                        v3 jom = ang_vel(ld4(ep, k), ld4(ev, k));
                        double jr = jp4.w, jm = mass[k];
                        v3 rp = mk3(jp4.x - ip4.x, jp4.y - ip4.y, jp4.z - ip4.z);
                        double dist = len3(rp);
                        double cdist = (ir + jr) - dist;
                        double coh_s = 0;
                        if (cp->coh) coh_s = limit_cohesion_depth(ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
                        double sd0 = 0.0, sd1 = 0.0;
                        v3 unit = div3(rp, dist);
                        v3 cpt = add3(ipos, mul3(ir, unit));
                        int store = 0;
                        if (cdist > 0) {
                            for (unsigned int i = 0; i < old_count; ++i)
                                if (old_id[i] == k) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
                            v3 dcpr = sub3(cpt, ipos);
                            v3 dcpr_j = sub3(cpt, mk3(jp4.x, jp4.y, jp4.z));
                            v3 rv = sub3(add3(jvel, cross3(jom, dcpr_j)), add3(ivel, cross3(iom, dcpr)));
                            fconst c = get_constant(model, ir, jr, im, jm, cp->Ei, cp->Ej, cp->pri, cp->prj,
                                                    cp->rest, cp->fric, cp->s_fric, cp->rfric, cp->sratio);
                            contact_model(model, c, ir, jr, cp, dt, cdist, &sd0, &sd1, rv, unit, &Ft, &Fn);
                            rolling_accumulate(cp->rfric, ir, jr, dcpr, Fn, Ft, &res, &tma);
                            sumF = add3(sumF, add3(Fn, Ft));
                            sumM = add3(sumM, cross3(dcpr, add3(Fn, Ft)));
                            store = 1;
                        } else if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
                            double f = jkr_separation_force(ir, jr, cp->coh);
                            double cf = cohesion_force(ir, jr, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, f);
                            sumF = sub3(sumF, mul3(cf, unit));
                            store = 1;
                        }
                        if (store) {
                            if (cnt < MAX_P2P_COUNT) {
                                tsd[2 * (sid + cnt)] = sd0; tsd[2 * (sid + cnt) + 1] = sd1;
                                pair_id[sid + cnt] = k;
                                cnt++;
                            } else bits |= XDEM_ERR_P2P_OVERFLOW;
                        }
                    }
                }
        addto3(force, id, sumF);
        addto3(moment, id, sumM);
        pair_count[id] = cnt;
        addto3(tmax, id, tma);
        rres[id] += res;
        raise_status(status, bits);
    }
}

/* ======================================================================== */
/* Planes                                                                    */
/* ======================================================================== */
/* impl:735-815.  Regions of the finite rectangle: corners, edges (the third
 * edge test can never hold, impl:787), face.  Returns the overlap and sets
 * the unit vector; 0 when nothing is hit. */
static double plane_detection(const device_plane_info* pe, v3 xp, v3 wp, v3* u, double r)
{
    double a_l1 = (wp.x - pe->l1) * (wp.x - pe->l1);
    double b_l2 = (wp.y - pe->l2) * (wp.y - pe->l2);
    double sqa = wp.x * wp.x, sqb = wp.y * wp.y, sqc = wp.z * wp.z, sqr = r * r;
    v3 xw = dv3(pe->xw), w2 = dv3(pe->w2), w3 = dv3(pe->w3), w4 = dv3(pe->w4);
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        v3 X = sub3(xp, xw); double h = len3(X); *u = div3(X, h); return r - h;
    } else if (wp.x > pe->l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        v3 X = sub3(xp, w2); double h = len3(X); *u = div3(X, h); return r - h;
    } else if (wp.x > pe->l1 && wp.y > pe->l2 && (a_l1 + b_l2 + sqc) < sqr) {
        v3 X = sub3(xp, w3); double h = len3(X); *u = div3(X, h); return r - h;
    } else if (wp.x < 0 && wp.y > pe->l2 && (sqa + b_l2 + sqc) < sqr) {
        v3 X = sub3(xp, w4); double h = len3(X); *u = div3(X, h); return r - h;
    }
    if ((wp.x > 0 && wp.x < pe->l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        v3 X = sub3(xp, xw); v3 e = sub3(w2, xw); v3 us = div3(e, len3(e));
        v3 hs = sub3(X, mul3(dot3(X, us), us)); double h = len3(hs);
        *u = div3(neg3(hs), h); return r - h;
    } else if ((wp.x > 0 && wp.x < pe->l1) && wp.y > pe->l2 && (b_l2 + sqc) < sqr) {
        v3 X = sub3(xp, w4); v3 e = sub3(w3, w4); v3 us = div3(e, len3(e));
        v3 hs = sub3(X, mul3(dot3(X, us), us)); double h = len3(hs);
        *u = div3(neg3(hs), h); return r - h;
    } else if ((wp.x > 0 && wp.y < pe->l2) && wp.x < 0 && (sqr + sqc) < sqr) {
        /* unreachable in the reference (wp.x > 0 && wp.x < 0) */
        v3 X = sub3(xp, xw); v3 e = sub3(w4, xw); v3 us = div3(e, len3(e));
        v3 hs = sub3(X, mul3(dot3(X, us), us)); double h = len3(hs);
        *u = div3(neg3(hs), h); return r - h;
    } else if ((wp.x > 0 && wp.y < pe->l2) && wp.x > pe->l1 && (a_l1 + sqc) < sqr) {
        v3 X = sub3(xp, w2); v3 e = sub3(w3, w2); v3 us = div3(e, len3(e));
        v3 hs = sub3(X, mul3(dot3(X, us), us)); double h = len3(hs);
        *u = div3(neg3(hs), h); return r - h;
    } else if ((wp.x > 0 && wp.x < pe->l1) && (wp.y > 0 && wp.y < pe->l2)) {
        v3 dp = sub3(xp, xw);
        v3 uw = dv3(pe->uw);
        v3 uu = div3(uw, len3(uw));
        *u = neg3(uu);
        return r - fabs(dot3(dp, *u));
    }
    return 0;
}

static inline void body_rec(const double* dbi, v3* p, v3* v, v3* om, double* m)
{
    *p = mk3(dbi[XDEM_PX], dbi[XDEM_PY], dbi[XDEM_PZ]);
    *v = mk3(dbi[XDEM_VX], dbi[XDEM_VY], dbi[XDEM_VZ]);
    *om = ang_vel(mk4(dbi[XDEM_E0], dbi[XDEM_E1], dbi[XDEM_E2], dbi[XDEM_E3]),
                  mk4(dbi[XDEM_ED0], dbi[XDEM_ED1], dbi[XDEM_ED2], dbi[XDEM_ED3]));
    *m = dbi[XDEM_MM];
}

/* impl:950-1080.  Plane k = plane->id: k == 0 restarts the particle's plane
 * list, k > 0 appends after the count left by plane k-1 in this step
 * (impl:970).  The history lookup scans all MAX_P2PL_COUNT slots, stale ones
 * included (impl:989). */
void xo_plane(const device_dem_parameters* prm, const device_plane_info* plane,
              const double* dbi, const device_contact_property* cp, double* fx, double* fy,
              double* fz, double* mx, double* my, double* mz, const double* pos,
              const double* ep, const double* vel, const double* ev, double* force,
              double* moment, const double* mass, double* tmax, double* rres,
              unsigned int* pair_count, unsigned int* pair_id, double* tsd, unsigned int np,
              unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
    v3 bp, bv, bom; double bm;
    body_rec(dbi, &bp, &bv, &bom, &bm);
    (void)bm;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2PL_COUNT;
        unsigned int old_id[MAX_P2PL_COUNT];
        double old_sd[MAX_P2PL_COUNT][2];
        for (int i = 0; i < MAX_P2PL_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        fx[id] = fy[id] = fz[id] = 0.0;
        mx[id] = my[id] = mz[id] = 0.0;
        unsigned int old_count = pair_count[id];
        double m = mass[id];
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        double r = ip4.w;
        unsigned int k = plane->id;
        v3 ivel = ld3(vel, id);
        v3 iom = ang_vel(ld4(ep, id), ld4(ev, id));
        v3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
        v3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = k ? old_count : 0, bits = 0;
        double coh_s = 0;
        v3 dp = sub3(ipos, dv3(plane->xw));
        v3 unit = mk3(0, 0, 0);
        v3 wp = mk3(dot3(dp, dv3(plane->u1)), dot3(dp, dv3(plane->u2)), dot3(dp, dv3(plane->uw)));
        double cdist = plane_detection(plane, ipos, wp, &unit, r);
        if (cp->coh) coh_s = limit_cohesion_depth(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
        double sd0 = 0.0, sd1 = 0.0;
        v3 mf = mk3(0, 0, 0);
        v3 cpt = add3(ipos, mul3(r, unit));
        v3 dcpr_j = sub3(cpt, bp);
        int store = 0;
        if (cdist > 0) {
            for (int i = 0; i < MAX_P2PL_COUNT; ++i)
                if (old_id[i] == k) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
            v3 dcpr = sub3(cpt, ipos);
            v3 dv = sub3(add3(bv, cross3(bom, dcpr_j)), add3(ivel, cross3(iom, dcpr)));
            fconst c = get_constant(model, r, 0.0, m, 0.0, cp->Ei, cp->Ej, cp->pri, cp->prj,
                                    cp->rest, cp->fric, cp->s_fric, cp->rfric, cp->sratio);
            contact_model(model, c, r, 0, cp, dt, cdist, &sd0, &sd1, dv, unit, &Ft, &Fn);
            rolling_accumulate(cp->rfric, r, 0, dcpr, Fn, Ft, &res, &tma);
            mf = add3(Fn, Ft);
            sumF = add3(sumF, mf);
            sumM = add3(sumM, cross3(dcpr, mf));
            fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
            v3 bmo = neg3(cross3(dcpr_j, mf));
            mx[id] += bmo.x; my[id] += bmo.y; mz[id] += bmo.z;
            store = 1;
        } else if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
            double f = jkr_separation_force(r, 0, cp->coh);
            double cf = cohesion_force(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, f);
            mf = mul3(-cf, unit);
            sumF = add3(sumF, mf);
            fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
            v3 bmo = neg3(cross3(dcpr_j, mf));
            mx[id] += bmo.x; my[id] += bmo.y; mz[id] += bmo.z;
            store = 1;
        }
        if (store) {
            if (cnt < MAX_P2PL_COUNT) {
                tsd[2 * (sid + cnt)] = sd0; tsd[2 * (sid + cnt) + 1] = sd1;
                pair_id[sid + cnt] = k;
                cnt++;
            } else bits |= XDEM_ERR_P2PL_OVERFLOW;
        }
        addto3(force, id, sumF);
        addto3(moment, id, sumM);
        pair_count[id] = cnt;
        addto3(tmax, id, tma);
        rres[id] += res;
        raise_status(status, bits);
    }
}

/* ======================================================================== */
/* Triangle meshes                                                           */
/* ======================================================================== */
/* impl:1655-1705 (Ericson's closest point; later tests override earlier
 * ones; t: 0 vertex, 1 edge, 2 face; -1 and the origin when none holds). */
static v3 closest_pt_triangle(const device_triangle_info* tri, v3 p, int* ct)
{
    v3 a = dv3(tri->P), b = dv3(tri->Q), c = dv3(tri->R);
    v3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a), bp = sub3(p, b), cp = sub3(p, c);
    double d1 = dot3(ab, ap), d2 = dot3(ac, ap), d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    double va = d3 * d6 - d5 * d4, vb = d5 * d2 - d1 * d6, vc = d1 * d4 - d3 * d2;
    v3 cpt = mk3(0, 0, 0);
    if (d1 <= 0.0 && d2 <= 0.0) { *ct = 0; cpt = a; }
    if (d3 >= 0.0 && d4 <= d3) { *ct = 0; cpt = b; }
    if (d6 >= 0.0 && d5 <= d6) { *ct = 0; cpt = c; }
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) { *ct = 1; cpt = add3(a, mul3(d1 / (d1 - d3), ab)); }
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) { *ct = 1; cpt = add3(a, mul3(d2 / (d2 - d6), ac)); }
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        *ct = 1; cpt = add3(b, mul3((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub3(c, b)));
    }
    if (va >= 0 && vb >= 0 && vc >= 0) {
        double denom = 1.0 / (va + vb + vc);
        v3 v = mul3(vb * denom, ab);
        v3 w = mul3(vc * denom, ac);
        cpt = add3(add3(a, v), w);
        *ct = 2;
    }
    return cpt;
}

/* impl:1729-1746 */
static int check_overlap(v3 p, v3 c)
{
    int b0 = (p.x >= c.x - 1e-9 && p.x <= c.x + 1e-9);
    int b1 = (p.y >= c.y - 1e-9 && p.y <= c.y + 1e-9);
    int b2 = (p.z >= c.z - 1e-9 && p.z <= c.z + 1e-9);
    return b0 && b1 && b2;
}

typedef struct { unsigned int id; v3 cpt; } tri_hit;

typedef struct {
    tri_hit face[XDEM_MAX_TRI_CANDIDATES], line[XDEM_MAX_TRI_CANDIDATES], point[XDEM_MAX_TRI_CANDIDATES];
    unsigned int nf, nl, npt;
} tri_sets;

/* Candidate search shared by the sphere and cluster mesh kernels
 * (impl:1983-2050 and 2183-2238). */
static void collect_triangles(const device_dem_parameters* prm, const device_triangle_info* dti,
                              const device_contact_property* cp, v3 ipos, double ir,
                              const unsigned int* sorted_index, const unsigned int* cstart,
                              const unsigned int* cend, unsigned int lo, unsigned int ntriangle,
                              tri_sets* s, unsigned int* bits)
{
    int g[3]; grid_pos(prm, ipos, g);
    s->nf = s->nl = s->npt = 0;
    v3 prev_line = mk3(0, 0, 0), prev_point = mk3(0, 0, 0);
    double coh_s = 0;
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                unsigned int h = grid_hash(prm, g[0] + x, g[1] + y, g[2] + z);
                unsigned int start = cstart[h];
                if (start == 0xffffffffu) continue;
                unsigned int end = cend[h];
                for (unsigned int j = start; j < end; ++j) {
                    unsigned int tk = sorted_index[j];
                    if (!(tk >= lo && tk < lo + ntriangle)) continue;
                    tk -= lo;
                    int t = -1;
                    v3 cpt = closest_pt_triangle(&dti[tk], ipos, &t);
                    double cdist = ir - len3(sub3(ipos, cpt));
                    if (cp->coh) coh_s = limit_cohesion_depth(ir, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
                    int take = 0;
                    if (cdist > 0) {
                        if (t == 1) {
                            if (check_overlap(prev_line, cpt)) continue;
                            prev_line = cpt;
                        } else if (t == 0) {
                            if (check_overlap(prev_point, cpt)) continue;
                            prev_point = cpt;
                        }
                        take = 1;
                    } else if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
                        take = 1;
                    }
                    if (!take) continue;
                    tri_hit hit; hit.id = tk; hit.cpt = cpt;
                    if (t == 2) { if (s->nf < XDEM_MAX_TRI_CANDIDATES) s->face[s->nf++] = hit; else *bits |= XDEM_ERR_TRI_CANDIDATES; }
                    else if (t == 1) { if (s->nl < XDEM_MAX_TRI_CANDIDATES) s->line[s->nl++] = hit; else *bits |= XDEM_ERR_TRI_CANDIDATES; }
                    else if (t == 0) { if (s->npt < XDEM_MAX_TRI_CANDIDATES) s->point[s->npt++] = hit; else *bits |= XDEM_ERR_TRI_CANDIDATES; }
                }
            }
}

typedef struct {
    v3 sum_force, sum_moment, tma;
    double res;
    unsigned int cnt;
    double bf[6];
} tri_acc;

/* impl:1748-1835 (sphere) and impl:1837-1928 (cluster: icpos != NULL). */
static void triangle_force(int model, double dt, const tri_hit* hit, const device_contact_property* cp,
                           const double* dbi, v3 ipos, const v3* icpos, v3 ivel, v3 iom,
                           const unsigned int* old_id, double (*old_sd)[2], unsigned int* pair_id,
                           double* tsd, unsigned int sid, double r, double m, tri_acc* acc,
                           unsigned int* bits)
{
    v3 bp, bv, bom; double bm;
    body_rec(dbi, &bp, &bv, &bom, &bm);
    double sd0 = 0.0, sd1 = 0.0;
    v3 po2cp = sub3(hit->cpt, bp);
    v3 unit;
    double cdist;
    if (!icpos) {
        v3 rp = sub3(hit->cpt, ipos);
        double dist = len3(rp);
        unit = div3(rp, dist);
        cdist = r - dist;
    } else {
        unit = sub3(hit->cpt, ipos);
        cdist = r - len3(sub3(ipos, hit->cpt));
    }
    double coh_s = 0;
    if (cp->coh) coh_s = limit_cohesion_depth(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
    int store = 0;
    if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
        double f = jkr_separation_force(r, 0, cp->coh);
        double cf = cohesion_force(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, f);
        acc->sum_force = sub3(acc->sum_force, mul3(cf, unit));
        store = 1;
    } else {
        v3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
        v3 rc;
        if (!icpos) {
            rc = sub3(hit->cpt, ipos);
        } else {
            rc = sub3(hit->cpt, *icpos);
            unit = div3(unit, len3(unit));
        }
        for (int i = 0; i < MAX_P2MS_COUNT; ++i)
            if (old_id[i] == hit->id) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
        v3 dv = sub3(add3(bv, cross3(bom, po2cp)), add3(ivel, cross3(iom, rc)));
        fconst c = get_constant(model, r, 0, m, bm, cp->Ei, cp->Ej, cp->pri, cp->prj,
                                cp->rest, cp->fric, cp->s_fric, cp->rfric, cp->sratio);
        contact_model(model, c, r, 0, cp, dt, cdist, &sd0, &sd1, dv, unit, &Ft, &Fn);
        rolling_accumulate(cp->rfric, r, 0, rc, Fn, Ft, &acc->res, &acc->tma);
        v3 mf = add3(Fn, Ft);
        acc->sum_force = add3(acc->sum_force, mf);
        acc->sum_moment = add3(acc->sum_moment, cross3(rc, mf));
        acc->bf[0] += -mf.x; acc->bf[1] += -mf.y; acc->bf[2] += -mf.z;
        v3 mm = neg3(cross3(po2cp, mf));
        acc->bf[3] += mm.x; acc->bf[4] += mm.y; acc->bf[5] += mm.z;
        store = 1;
    }
    if (store) {
        if (acc->cnt < MAX_P2MS_COUNT) {
            tsd[2 * (sid + acc->cnt)] = sd0; tsd[2 * (sid + acc->cnt) + 1] = sd1;
            pair_id[sid + acc->cnt] = hit->id;
            acc->cnt++;
        } else *bits |= XDEM_ERR_P2MS_OVERFLOW;
    }
}

static void mesh_common(const device_dem_parameters* prm, const device_triangle_info* dti,
                        const double* dbi, double* fx, double* fy, double* fz, double* mx,
                        double* my, double* mz, const double* pos, const double* cpos,
                        const double* ep, const double* vel, const double* ev, double* force,
                        double* moment, const double* mass, double* tmax, double* rres,
                        unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                        const unsigned int* sorted_index, const unsigned int* cstart,
                        const unsigned int* cend, const device_contact_property* cp,
                        const xClusterInformation* xci, unsigned int np, unsigned int ntriangle,
                        unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
    /* sphere kernel: sk = dti[0].tid and the range uses cte.np (impl:1970,
       1994); cluster kernel: sk = dti[0].id and the argument np (impl:2180,
       2193). */
    unsigned int lo = cpos ? np + (unsigned int)dti[0].id : prm->np + dti[0].tid;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2MS_COUNT;
        unsigned int old_id[MAX_P2MS_COUNT];
        double old_sd[MAX_P2MS_COUNT][2];
        for (int i = 0; i < MAX_P2MS_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        unsigned int ci = id, bits = 0;
        if (cpos) {
            unsigned int neach = 0;
            for (unsigned int i = 0; i < prm->nClusterObject; ++i)
                if (id >= xci[i].sid && id < xci[i].sid + xci[i].count * xci[i].neach) { neach = xci[i].neach; break; }
            ci = neach ? id / neach : 0;
        }
        double im = mass[ci];
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        v3 icp = cpos ? ld4xyz(cpos, ci) : mk3(0, 0, 0);
        v3 ivel = ld3(vel, ci);
        v3 iom = ang_vel(ld4(ep, ci), ld4(ev, ci));
        double ir = ip4.w;
        tri_sets s;
        collect_triangles(prm, dti, cp, ipos, ir, sorted_index, cstart, cend, lo, ntriangle, &s, &bits);
        tri_acc acc;
        memset(&acc, 0, sizeof(acc));
        const v3* icpp = cpos ? &icp : NULL;
        for (unsigned int k = 0; k < s.nf; ++k)
            triangle_force(model, dt, &s.face[k], cp, dbi, ipos, icpp, ivel, iom, old_id, old_sd, pair_id, tsd, sid, ir, im, &acc, &bits);
        if (!s.nf)
            for (unsigned int k = 0; k < s.nl; ++k)
                triangle_force(model, dt, &s.line[k], cp, dbi, ipos, icpp, ivel, iom, old_id, old_sd, pair_id, tsd, sid, ir, im, &acc, &bits);
        if (!s.nf && !s.nl)
            for (unsigned int k = 0; k < s.npt; ++k)
                triangle_force(model, dt, &s.point[k], cp, dbi, ipos, icpp, ivel, iom, old_id, old_sd, pair_id, tsd, sid, ir, im, &acc, &bits);
        fx[id] = acc.bf[0]; fy[id] = acc.bf[1]; fz[id] = acc.bf[2];
        mx[id] = acc.bf[3]; my[id] = acc.bf[4]; mz[id] = acc.bf[5];
        addto3(force, id, acc.sum_force);
        addto3(moment, id, acc.sum_moment);
        pair_count[id] = acc.cnt;
        addto3(tmax, id, acc.tma);
        rres[id] += acc.res;
        raise_status(status, bits);
    }
}

void xo_mesh(const device_dem_parameters* prm, const device_triangle_info* dti, const double* dbi,
             double* fx, double* fy, double* fz, double* mx, double* my, double* mz,
             const double* pos, const double* ep, const double* vel, const double* ev,
             double* force, double* moment, const double* mass, double* tmax, double* rres,
             unsigned int* pair_count, unsigned int* pair_id, double* tsd,
             const unsigned int* sorted_index, const unsigned int* cstart, const unsigned int* cend,
             const device_contact_property* cp, unsigned int np, unsigned int ntriangle,
             unsigned int* status)
{
    mesh_common(prm, dti, dbi, fx, fy, fz, mx, my, mz, pos, NULL, ep, vel, ev, force, moment, mass,
                tmax, rres, pair_count, pair_id, tsd, sorted_index, cstart, cend, cp, NULL, np,
                ntriangle, status);
}

void xo_cluster_mesh(const device_dem_parameters* prm, const device_triangle_info* dti,
                     const double* dbi, double* fx, double* fy, double* fz, double* mx, double* my,
                     double* mz, const double* pos, const double* cpos, const double* ep,
                     const double* vel, const double* ev, double* force, double* moment,
                     const device_contact_property* cp, const double* mass, double* tmax,
                     double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                     const unsigned int* sorted_index, const unsigned int* cstart,
                     const unsigned int* cend, const xClusterInformation* xci, unsigned int np,
                     unsigned int ntriangle, unsigned int* status)
{
    mesh_common(prm, dti, dbi, fx, fy, fz, mx, my, mz, pos, cpos, ep, vel, ev, force, moment, mass,
                tmax, rres, pair_count, pair_id, tsd, sorted_index, cstart, cend, cp, xci, np,
                ntriangle, status);
}

/* ======================================================================== */
/* Rolling resistance (impl:2420-2454, 2456-2500)                            */
/* ======================================================================== */
void xo_rolling(const device_dem_parameters* prm, double* tmax, double* rres, const double* inertia,
                const double* ep, const double* ev, double* moment, unsigned int np)
{
    xo_rolling_ex(prm, tmax, rres, inertia, ep, ev, moment, np, 0);
}

/* per_sphere = 1 reads the sphere's own inertia, inertia[3 i] (the three
 * entries are equal for a sphere), instead of the flat inertia[i]. */
void xo_rolling_ex(const device_dem_parameters* prm, double* tmax, double* rres, const double* inertia,
                   const double* ep, const double* ev, double* moment, unsigned int np, int per_sphere)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < (long)np; ++i) {
        double Tr = rres[i];
        if (!Tr) continue;
        v3 Tmax = ld3(tmax, i);
        double J = per_sphere ? inertia[3 * i] : inertia[i];  /* impl:2434 reads the flat entry i */
        v3 om = ang_vel(ld4(ep, i), ld4(ev, i));
        v3 T = sub3(mul3(J * prm->dt, om), Tmax);
        double lT = len3(T);
        if (lT && Tr) {
            v3 Tr3 = mul3(Tr, div3(T, lT));
            if (len3(Tr3) >= lT) Tr3 = T;
            addto3(moment, i, Tr3);
        }
        st3(tmax, i, mk3(0, 0, 0));
        rres[i] = 0.0;
    }
}

void xo_cluster_rolling(const device_dem_parameters* prm, double* tmax, double* rres,
                        const double* inertia, const double* ep, const double* ev, double* moment,
                        const xClusterInformation* xci, unsigned int np)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < (long)np; ++i) {
        double Tr = rres[i];
        if (!Tr) continue;
        unsigned int id = (unsigned int)i, neach = 0;
        for (unsigned int k = 0; k < prm->nClusterObject; ++k)
            if (id >= xci[k].sid && id < xci[k].sid + xci[k].count * xci[k].neach) { neach = xci[k].neach; break; }
        unsigned int cid = neach ? id / neach : 0;
        v3 Tmax = ld3(tmax, i);
        v3 J = ld3(inertia, cid);
        v3 om = ang_vel(ld4(ep, cid), ld4(ev, cid));
        v3 Jw = mk3(J.x * om.x, J.y * om.y, J.z * om.z);
        v3 T = sub3(mul3(prm->dt, Jw), Tmax);
        double lT = len3(T);
        if (lT && Tr) {
            v3 Tr3 = mul3(Tr, div3(T, lT));
            if (len3(Tr3) >= lT) Tr3 = T;
            v3 m = ld3(moment, i);
            st3(moment, i, sub3(m, Tr3));
        }
        st3(tmax, i, mk3(0, 0, 0));
        rres[i] = 0.0;
    }
}

/* ======================================================================== */
/* Mesh pose (impl:2544-2601)                                                */
/* ======================================================================== */
void xo_update_mesh(const double* dbi, const double* vList, double* sphere, const double* dlocal,
                    device_triangle_info* dpi, unsigned int ntriangle)
{
    v3 p = mk3(dbi[XDEM_PX], dbi[XDEM_PY], dbi[XDEM_PZ]);
    v4 e = mk4(dbi[XDEM_E0], dbi[XDEM_E1], dbi[XDEM_E2], dbi[XDEM_E3]);
    for (unsigned int i = 0; i < ntriangle; ++i) {
        const double* v = vList + 9 * (size_t)i;
        v3 P = add3(p, to_global(mk3(v[0], v[1], v[2]), e));
        v3 Q = add3(p, to_global(mk3(v[3], v[4], v[5]), e));
        v3 R = add3(p, to_global(mk3(v[6], v[7], v[8]), e));
        v3 c = add3(p, to_global(ld3(dlocal, i), e));
        sphere[4 * i] = c.x; sphere[4 * i + 1] = c.y; sphere[4 * i + 2] = c.z;
        dpi[i].P.x = P.x; dpi[i].P.y = P.y; dpi[i].P.z = P.z;
        dpi[i].Q.x = Q.x; dpi[i].Q.y = Q.y; dpi[i].Q.z = Q.z;
        dpi[i].R.x = R.x; dpi[i].R.y = R.y; dpi[i].R.z = R.z;
    }
}

/* ======================================================================== */
/* Clusters                                                                  */
/* ======================================================================== */
/* impl:485-611.  Pairs with |id - k| <= neach are skipped (impl:556-558),
 * which also skips members of neighbouring clusters one index apart. */
void xo_clusters_p2p(const device_dem_parameters* prm, const double* pos, const double* cpos,
                     const double* ep, const double* vel, const double* ev, double* force,
                     double* moment, const double* mass, double* tmax, double* rres,
                     unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                     const unsigned int* sorted_index, const unsigned int* cstart,
                     const unsigned int* cend, const device_contact_property* cp,
                     const xClusterInformation* xci, unsigned int np, unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2P_COUNT;
        unsigned int old_id[MAX_P2P_COUNT];
        double old_sd[MAX_P2P_COUNT][2];
        for (int i = 0; i < MAX_P2P_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        unsigned int neach = 0;
        for (unsigned int i = 0; i < prm->nClusterObject; ++i)
            if (id >= xci[i].sid && id < xci[i].sid + xci[i].count * xci[i].neach) { neach = xci[i].neach; break; }
        unsigned int old_count = pair_count[id];
        if (old_count > MAX_P2P_COUNT) old_count = MAX_P2P_COUNT;
        unsigned int cid = neach ? id / neach : 0;
        v3 icpos = ld4xyz(cpos, cid);
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        v3 ivel = ld3(vel, cid);
        v3 iom = ang_vel(ld4(ep, cid), ld4(ev, cid));
        int g[3]; grid_pos(prm, ipos, g);
        double ir = ip4.w, im = mass[cid];
        v3 Ft = mk3(0, 0, 0), Fn = mk3(0, 0, 0);
        v3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        double res = 0.0;
        unsigned int cnt = 0, bits = 0;
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    unsigned int h = grid_hash(prm, g[0] + x, g[1] + y, g[2] + z);
                    unsigned int start = cstart[h];
                    if (start == 0xffffffffu) continue;
                    unsigned int end = cend[h];
                    for (unsigned int j = start; j < end; ++j) {
                        unsigned int k = sorted_index[j];
                        unsigned int di = id >= k ? id - k : k - id;
                        if (id == k || k >= np || di <= neach) continue;
                        unsigned int ck = k / neach;
                        v4 jp4 = ld4(pos, k);
                        v3 jvel = ld3(vel, ck);
                        v3 jom = ang_vel(ld4(ep, ck), ld4(ev, ck));
                        double jr = jp4.w, jm = mass[ck];
                        v3 jcpos = ld4xyz(cpos, ck);
                        v3 rp = mk3(jp4.x - ip4.x, jp4.y - ip4.y, jp4.z - ip4.z);
                        double dist = len3(rp);
                        double cdist = (ir + jr) - dist;
                        if (cdist > 0) {
                            double sd0 = 0.0, sd1 = 0.0;
                            for (unsigned int i = 0; i < old_count; ++i)
                                if (old_id[i] == k) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
                            v3 unit = div3(rp, dist);
                            v3 cpt = add3(ipos, mul3(ir, unit));
                            v3 dcpr = sub3(cpt, icpos);
                            v3 dcpr_j = sub3(cpt, jcpos);
                            v3 rv = sub3(add3(jvel, cross3(jom, dcpr_j)), add3(ivel, cross3(iom, dcpr)));
                            fconst c = get_constant(model, ir, jr, im, jm, cp->Ei, cp->Ej, cp->pri, cp->prj,
                                                    cp->rest, cp->fric, cp->s_fric, cp->rfric, cp->sratio);
                            contact_model(model, c, ir, jr, cp, dt, cdist, &sd0, &sd1, rv, unit, &Ft, &Fn);
                            rolling_accumulate(cp->rfric, ir, jr, dcpr, Fn, Ft, &res, &tma);
                            sumF = add3(sumF, add3(Fn, Ft));
                            sumM = add3(sumM, cross3(dcpr, add3(Fn, Ft)));
                            if (cnt < MAX_P2P_COUNT) {
                                tsd[2 * (sid + cnt)] = sd0; tsd[2 * (sid + cnt) + 1] = sd1;
                                pair_id[sid + cnt] = k;
                                cnt++;
                            } else bits |= XDEM_ERR_P2P_OVERFLOW;
                        }
                    }
                }
        addto3(force, id, sumF);
        addto3(moment, id, sumM);
        pair_count[id] = cnt;
        addto3(tmax, id, tma);
        rres[id] += res;
        raise_status(status, bits);
    }
}

/* impl:817-948.  Differences from the sphere plane kernel kept here: the
 * body lever arm dcpr_j is taken before the contact normal is known, i.e.
 * from the particle centre (impl:881-882); the friction passed to the model is
 * s_fric (arguments swapped at impl:898-901); the plane's mass enters the
 * effective mass. */
void xo_cluster_plane(const device_dem_parameters* prm, const device_plane_info* plane,
                      const double* dbi, double* fx, double* fy, double* fz, double* mx,
                      double* my, double* mz, const double* pos, const double* cpos,
                      const double* ep, const double* vel, const double* ev, double* force,
                      double* moment, const device_contact_property* cp, const double* mass,
                      double* tmax, double* rres, unsigned int* pair_count, unsigned int* pair_id,
                      double* tsd, const xClusterInformation* xci, unsigned int np,
                      unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
    v3 bp, bv, bom; double bm;
    body_rec(dbi, &bp, &bv, &bom, &bm);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2PL_COUNT;
        unsigned int old_id[MAX_P2PL_COUNT];
        double old_sd[MAX_P2PL_COUNT][2];
        for (int i = 0; i < MAX_P2PL_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        unsigned int neach = 0;
        for (unsigned int i = 0; i < prm->nClusterObject; ++i)
            if (id >= xci[i].sid && id < xci[i].sid + xci[i].count * xci[i].neach) { neach = xci[i].neach; break; }
        unsigned int cid = neach ? id / neach : 0;
        unsigned int old_count = pair_count[id];
        double m = mass[cid];
        fx[id] = fy[id] = fz[id] = 0.0;
        mx[id] = my[id] = mz[id] = 0.0;
        v3 icpos = ld4xyz(cpos, cid);
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        double r = ip4.w;
        v3 ivel = ld3(vel, cid);
        v3 iom = ang_vel(ld4(ep, cid), ld4(ev, cid));
        v3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
        v3 sumF = mk3(0, 0, 0), sumM = mk3(0, 0, 0), tma = mk3(0, 0, 0);
        unsigned int k = plane->id;
        unsigned int cnt = k ? old_count : 0, bits = 0;
        double res = 0.0;
        v3 dp = sub3(ipos, dv3(plane->xw));
        v3 unit = mk3(0, 0, 0);
        v3 wp = mk3(dot3(dp, dv3(plane->u1)), dot3(dp, dv3(plane->u2)), dot3(dp, dv3(plane->uw)));
        v3 mf = mk3(0, 0, 0);
        v3 cpt0 = add3(ipos, mul3(r, unit));
        v3 dcpr_j = sub3(cpt0, bp);
        double coh_s = 0;
        double cdist = plane_detection(plane, ipos, wp, &unit, r);
        double sd0 = 0.0, sd1 = 0.0;
        if (cp->coh) coh_s = limit_cohesion_depth(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
        int store = 0;
        if (cdist > 0) {
            for (int i = 0; i < MAX_P2PL_COUNT; ++i)
                if (old_id[i] == k) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
            v3 cpt = add3(ipos, mul3(r, unit));
            v3 dcpr = sub3(cpt, icpos);
            v3 dv = sub3(add3(bv, cross3(bom, dcpr_j)), add3(ivel, cross3(iom, dcpr)));
            fconst c = get_constant(model, r, 0.0, m, bm, cp->Ei, cp->Ej, cp->pri, cp->prj,
                                    cp->rest, cp->s_fric, cp->fric, cp->rfric, cp->sratio);
            contact_model(model, c, r, 0, cp, dt, cdist, &sd0, &sd1, dv, unit, &Ft, &Fn);
            rolling_accumulate(cp->rfric, r, 0, dcpr, Fn, Ft, &res, &tma);
            mf = add3(Fn, Ft);
            sumF = add3(sumF, mf);
            sumM = add3(sumM, cross3(dcpr, mf));
            fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
            v3 bmo = neg3(cross3(dcpr_j, mf));
            mx[id] += bmo.x; my[id] += bmo.y; mz[id] += bmo.z;
            store = 1;
        } else if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
            double f = jkr_separation_force(r, 0, cp->coh);
            double cf = cohesion_force(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, f);
            mf = mul3(-cf, unit);
            sumF = add3(sumF, mf);
            fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
            v3 bmo = neg3(cross3(dcpr_j, mf));
            mx[id] += bmo.x; my[id] += bmo.y; mz[id] += bmo.z;
            store = 1;
        }
        if (store) {
            if (cnt < MAX_P2PL_COUNT) {
                tsd[2 * (sid + cnt)] = sd0; tsd[2 * (sid + cnt) + 1] = sd1;
                pair_id[sid + cnt] = k;
                cnt++;
            } else bits |= XDEM_ERR_P2PL_OVERFLOW;
        }
        addto3(force, id, sumF);
        addto3(moment, id, sumM);
        pair_count[id] = cnt;
        addto3(tmax, id, tma);
        rres[id] += res;
        raise_status(status, bits);
    }
}

/* ======================================================================== */
/* Cylinders (impl:1083-1600)                                                */
/* ======================================================================== */
/* Base and top centres of the cylinder at its body pose. */
static void cylinder_ends(const device_cylinder_info* cy, const double* bi, v3* pos, v4* e, v3* base, v3* top)
{
    *pos = mk3(bi[XDEM_PX], bi[XDEM_PY], bi[XDEM_PZ]);
    *e = mk4(bi[XDEM_E0], bi[XDEM_E1], bi[XDEM_E2], bi[XDEM_E3]);
    *base = add3(*pos, to_global(dv3(cy->pbase), *e));
    *top = add3(*pos, to_global(dv3(cy->ptop), *e));
}

/* impl:1189-1288.  Depth of sphere (p, r) against the cylinder and the unit
 * vector of the contact: on the side (the axis parameter t in [0, 1]) the
 * radial direction, the depth measured against len_rr.y and the inside test
 * against len_rr.z (an inside contact flips the normal); beyond the ends the
 * annulus of the wall thickness, else the rim point found through the angle
 * atan(x / z) of the local offset, as the reference forms it. */
static double cylinder_detection(const device_cylinder_info* cy, const double* bi, v3 p, v3* u, double r,
                                 int* inner)
{
    v3 cyl_pos, base, top;
    v4 e;
    cylinder_ends(cy, bi, &cyl_pos, &e, &base, &top);
    v3 ab = sub3(top, base);
    double t = dot3(sub3(p, base), ab) / dot3(ab, ab);
    v3 c = add3(base, mul3(t, ab));
    double dist = len3(sub3(p, c));
    if (t >= 0 && t <= 1) {
        if (dist == 0) {
            *inner = 1;
            return 0;
        }
        *u = div3(sub3(c, p), dist);
        if (dist < cy->len_rr.z) {
            *inner = 1;
            *u = neg3(*u);
            return dist + r - cy->len_rr.y;
        }
        return cy->len_rr.y + r - dist;
    }
    double thick = cy->thickness;
    int one = thick != 0.0 ? 1 : 0;
    if (dist < cy->len_rr.z + thick && dist > one * cy->len_rr.z) {
        v3 o2c = sub3(cyl_pos, c);
        double l = len3(o2c);
        *u = div3(o2c, l);
        return cy->len_rr.x * 0.5 + r - l;
    }
    v3 at = to_local(sub3(p, top), e);
    v3 cp = top;
    if (fabs(at.y) > cy->len_rr.x) {
        at = to_local(sub3(p, base), e);
        cp = base;
    }
    double pi = atan(at.x / at.z);
    v3 q = mk3(0, 0, 0);
    if (pi < 0 && at.z < 0) q.x = cy->len_rr.z * sin(-pi);
    else if (pi > 0 && at.x < 0 && at.z < 0) q.x = cy->len_rr.z * sin(-pi);
    else q.x = cy->len_rr.z * sin(pi);
    q.z = cy->len_rr.z * cos(pi);
    if (at.z < 0 && q.z > 0) q.z = -q.z;
    else if (at.z > 0 && q.z < 0) q.z = -q.z;
    q.y = 0.;
    cp = add3(cp, to_global(q, e));
    v3 dv = sub3(cp, p);
    dist = len3(dv);
    *u = div3(dv, dist);
    if (dist < r) return r - dist;
    return -1.0;
}

/* impl:1290-1322.  Inside a cylinder, the cap the sphere faces: none near
 * an open end (empty 1: top, t > 0.6; empty 2: base, t < 0.4). */
static double cylinder_inner_cap(const device_cylinder_info* cy, const double* bi, v3 p, v3* u, v3* cpt,
                                 unsigned int empty, double r)
{
    v3 cyl_pos, base, top;
    v4 e;
    cylinder_ends(cy, bi, &cyl_pos, &e, &base, &top);
    v3 ab = sub3(top, base);
    double t = dot3(sub3(p, base), ab) / dot3(ab, ab);
    v3 c = add3(base, mul3(t, ab));
    double dist = len3(sub3(p, c));
    if (empty == 1 && t > 0.6) return 0.0;
    if (empty == 2 && t < 0.4) return 0.0;
    double gab = -1.0;
    if (dist < cy->len_rr.z) {
        v3 o2c = sub3(cyl_pos, c);
        double l = len3(o2c);
        *u = neg3(div3(o2c, l));
        *cpt = add3(p, mul3(r, *u));
        gab = r + l - cy->len_rr.x * 0.5;
    }
    return gab;
}

typedef struct {
    v3 sum_f, sum_m, tma;
    double res;
    unsigned int cnt;   /* slots used (the reference's new_count - sid) */
} cyl_acc;

/* One stored cylinder pair (slots without the reference's missing bound:
 * a contact past MAX_P2CY_COUNT is dropped and flagged). */
static void cylinder_store(unsigned int* pair_id, double* tsd, unsigned int sid, cyl_acc* a, unsigned int pid,
                           double sd0, double sd1, unsigned int* bits)
{
    if (a->cnt < MAX_P2CY_COUNT) {
        tsd[2 * (sid + a->cnt)] = sd0;
        tsd[2 * (sid + a->cnt) + 1] = sd1;
        pair_id[sid + a->cnt] = pid;
        a->cnt++;
    } else {
        *bits |= XDEM_ERR_P2CY_OVERFLOW;
    }
}

/* impl:1111-1187: the contact force of one cylinder contact.  `ipos` is the
 * sphere's centre, or for a cluster member its cluster's centre (the lever
 * arm rc = cpt - ipos); the body's mass does not enter the effective mass. */
static void cylinder_force(int model, double dt, const device_contact_property* cp, const double* bi, v3 ipos,
                           v3 ivel, v3 iom, v3 cpt, v3 unit, double cdist, unsigned int id, unsigned int pid,
                           const unsigned int* old_id, double (*old_sd)[2], unsigned int* pair_id, double* tsd,
                           unsigned int sid, double r, double m, double* fx, double* fy, double* fz, double* mx,
                           double* my, double* mz, cyl_acc* a, unsigned int* bits)
{
    double sd0 = 0.0, sd1 = 0.0;
    v3 bp, bv, bom;
    double bm;
    body_rec(bi, &bp, &bv, &bom, &bm);
    v3 po2cp = sub3(cpt, bp);
    v3 Fn = mk3(0, 0, 0), Ft = mk3(0, 0, 0);
    for (int i = 0; i < MAX_P2CY_COUNT; ++i)
        if (old_id[i] == pid) { sd0 = old_sd[i][0]; sd1 = old_sd[i][1]; break; }
    v3 rc = sub3(cpt, ipos);
    v3 dv = sub3(add3(bv, cross3(bom, po2cp)), add3(ivel, cross3(iom, rc)));
    fconst c = get_constant(model, r, 0.0, m, 0.0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->rest, cp->fric,
                            cp->s_fric, cp->rfric, cp->sratio);
    contact_model(model, c, r, 0.0, cp, dt, cdist, &sd0, &sd1, dv, unit, &Ft, &Fn);
    rolling_accumulate(cp->rfric, r, 0.0, rc, Fn, Ft, &a->res, &a->tma);
    v3 mf = add3(Fn, Ft);
    a->sum_f = add3(a->sum_f, mf);
    a->sum_m = add3(a->sum_m, cross3(rc, mf));
    fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
    v3 bmo = neg3(cross3(po2cp, mf));
    mx[id] += bmo.x; my[id] += bmo.y; mz[id] += bmo.z;
    cylinder_store(pair_id, tsd, sid, a, pid, sd0, sd1, bits);
}

/* impl:1324-1601.  One launch for one cylinder over all particles: the side
 * (or annulus, or rim) contact with pair id k = cyl->id, then, for a sphere
 * inside, the cap it faces with pair id k + 1000.  Slots follow the plane
 * rule (k == 0 restarts the list, k > 0 appends to it).  cpos == NULL: free
 * spheres (cylinder_contact_force_kernel); else cluster members
 * (cluster_cylinder_contact_force_kernel: cluster mass, velocity, spin, and
 * lever arms from the cluster centre). */
void xo_cylinder(const device_dem_parameters* prm, const device_cylinder_info* cyl, const double* bi,
                 const device_contact_property* cp, double* fx, double* fy, double* fz, double* mx, double* my,
                 double* mz, const double* pos, const double* cpos, const double* ep, const double* vel,
                 const double* ev, double* force, double* moment, const double* mass, double* tmax, double* rres,
                 unsigned int* pair_count, unsigned int* pair_id, double* tsd, const xClusterInformation* xci,
                 unsigned int np, unsigned int* status)
{
    const int model = prm->contact_model;
    const double dt = prm->dt;
    v3 bp, bv, bom;
    double bm;
    body_rec(bi, &bp, &bv, &bom, &bm);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long ii = 0; ii < (long)np; ++ii) {
        unsigned int id = (unsigned int)ii;
        unsigned int sid = id * MAX_P2CY_COUNT;
        unsigned int old_id[MAX_P2CY_COUNT];
        double old_sd[MAX_P2CY_COUNT][2];
        for (int i = 0; i < MAX_P2CY_COUNT; ++i) {
            old_id[i] = pair_id[sid + i];
            old_sd[i][0] = tsd[2 * (sid + i)];
            old_sd[i][1] = tsd[2 * (sid + i) + 1];
        }
        unsigned int ci = id;
        if (cpos) {
            unsigned int neach = 0;
            for (unsigned int i = 0; i < prm->nClusterObject; ++i)
                if (id >= xci[i].sid && id < xci[i].sid + xci[i].count * xci[i].neach) { neach = xci[i].neach; break; }
            ci = neach ? id / neach : 0;
        }
        fx[id] = fy[id] = fz[id] = 0.0;
        mx[id] = my[id] = mz[id] = 0.0;
        unsigned int old_count = pair_count[id];
        unsigned int k = cyl->id;
        double m = mass[ci];
        v4 ip4 = ld4(pos, id);
        v3 ipos = mk3(ip4.x, ip4.y, ip4.z);
        double r = ip4.w;
        v3 ivel = ld3(vel, ci);
        v3 iom = ang_vel(ld4(ep, ci), ld4(ev, ci));
        v3 arm0 = cpos ? ld4xyz(cpos, ci) : ipos;
        cyl_acc a;
        memset(&a, 0, sizeof(a));
        a.cnt = k ? old_count : 0;
        unsigned int bits = 0;
        int inner = 0;
        double coh_s = 0;
        v3 unit = mk3(0, 0, 0);
        double cdist = cylinder_detection(cyl, bi, ipos, &unit, r, &inner);
        if (cp->coh) coh_s = limit_cohesion_depth(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh);
        v3 cpt = add3(ipos, mul3(r, unit));
        for (int pass = 0; pass < 2; ++pass) {
            unsigned int pid = pass ? k + 1000 : k;
            if (pass) {
                if (!inner) break;
                cdist = cylinder_inner_cap(cyl, bi, ipos, &unit, &cpt, cyl->empty_part, r);
            }
            if (cdist > 0) {
                cylinder_force(model, dt, cp, bi, arm0, ivel, iom, cpt, unit, cdist, id, pid, old_id, old_sd,
                               pair_id, tsd, sid, r, m, fx, fy, fz, mx, my, mz, &a, &bits);
            } else if (cdist <= 0 && fabs(cdist) < fabs(coh_s)) {
                double f = jkr_separation_force(r, 0, cp->coh);
                double cf = cohesion_force(r, 0, cp->Ei, cp->Ej, cp->pri, cp->prj, cp->coh, f);
                v3 mf = mul3(-cf, unit);
                a.sum_f = add3(a.sum_f, mf);
                fx[id] += -mf.x; fy[id] += -mf.y; fz[id] += -mf.z;
                v3 mo = neg3(cross3(sub3(cpt, bp), mf));
                mx[id] += mo.x; my[id] += mo.y; mz[id] += mo.z;
                cylinder_store(pair_id, tsd, sid, &a, pid, 0.0, 0.0, &bits);
            }
        }
        addto3(force, id, a.sum_f);
        addto3(moment, id, a.sum_m);
        pair_count[id] = a.cnt;
        addto3(tmax, id, a.tma);
        rres[id] += a.res;
        raise_status(status, bits);
    }
}

/* Locates cluster id i in the cluster-object table (impl:158-172). */
static void cluster_slot(const xClusterInformation* xci, unsigned int nco, unsigned int i,
                         unsigned int* neach, unsigned int* seach, unsigned int* sbegin,
                         unsigned int* scluster)
{
    *neach = 0; *seach = 0; *sbegin = 0; *scluster = 0;
    for (unsigned int k = 0; k < nco; ++k) {
        if (i >= xci[k].scid && i < xci[k].scid + xci[k].count) {
            *scluster = xci[k].scid; *neach = xci[k].neach; return;
        }
        *seach += xci[k].neach;
        *sbegin += xci[k].count * xci[k].neach;
    }
}

void xo_vv_cluster_position(const device_dem_parameters* prm, double* pos, double* cpos, double* ep,
                            const double* rloc, const double* vel, const double* acc,
                            const double* ev, const double* ea, const xClusterInformation* xci,
                            unsigned int ns)
{
    const double dt = prm->dt, h = prm->half2dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long ii = 0; ii < (long)ns; ++ii) {
        unsigned int id = (unsigned int)ii, neach, seach, sbegin, scl;
        cluster_slot(xci, prm->nClusterObject, id, &neach, &seach, &sbegin, &scl);
        v4 cp = ld4(cpos, id);
        v4 w = ld4(ev, id), wd = ld4(ea, id);
        v3 np_ = add3(add3(mk3(cp.x, cp.y, cp.z), mul3(dt, ld3(vel, id))), mul3(h, ld3(acc, id)));
        st4(cpos, id, mk4(np_.x, np_.y, np_.z, cp.w));
        v4 e = add4(add4(ld4(ep, id), mul4(dt, w)), mul4(h, wd));
        double l = sqrt(dot4(e, e));
        e = mk4(e.x / l, e.y / l, e.z / l, e.w / l);
        st4(ep, id, e);
        unsigned int sid = sbegin + (id - scl) * neach;
        for (unsigned int j = 0; j < neach; ++j) {
            v3 mp = add3(np_, to_global(ld3(rloc, seach + j), e));
            pos[4 * (size_t)(sid + j)] = mp.x; pos[4 * (size_t)(sid + j) + 1] = mp.y;
            pos[4 * (size_t)(sid + j) + 2] = mp.z;
        }
    }
}

void xo_vv_cluster_velocity(const device_dem_parameters* prm, const double* cpos, const double* ep,
                            double* vel, double* acc, double* ev, double* ea, double* force,
                            double* moment, const double* rloc, const double* mass, const double* iner,
                            const xClusterInformation* xci, unsigned int ns)
{
    (void)cpos; (void)rloc;
    const double hdt = 0.5 * prm->dt;
    const v3 g = dv3(prm->gravity);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long ii = 0; ii < (long)ns; ++ii) {
        unsigned int id = (unsigned int)ii, neach, seach, sbegin, scl;
        cluster_slot(xci, prm->nClusterObject, id, &neach, &seach, &sbegin, &scl);
        double m = mass[id];
        v3 v = ld3(vel, id), a = ld3(acc, id);
        v4 av = ld4(ev, id), aa = ld4(ea, id), e = ld4(ep, id);
        double inv_m = 1.0 / m;
        v3 in = ld3(iner, id);
        v3 F = mk3(0, 0, 0), T = mk3(0, 0, 0);
        unsigned int sid = sbegin + (id - scl) * neach;
        for (unsigned int j = 0; j < neach; ++j) {
            F = add3(F, ld3(force, sid + j));
            T = add3(T, ld3(moment, sid + j));
            st3(force, sid + j, mk3(0, 0, 0));
            st3(moment, sid + j, mk3(0, 0, 0));
        }
        F = add3(F, mul3(m, g));
        v3 n = to_local(T, e);
        v4 q = uceom(in, e, av, n);
        v = add3(v, mul3(hdt, a));
        av = add4(av, mul4(hdt, aa));
        a = mul3(inv_m, F);
        aa = q;
        st3(vel, id, add3(v, mul3(hdt, a)));
        st4(ev, id, add4(av, mul4(hdt, aa)));
        st3(acc, id, a);
        st4(ea, id, aa);
    }
}

/* ======================================================================== */
/* Setup helpers                                                             */
/* ======================================================================== */
void xo_fit_sphere_to_triangle(const double Pa[3], const double Qa[3], const double Ra[3], double ft,
                               double out[4])
{
    v3 P = mk3(Pa[0], Pa[1], Pa[2]), Q = mk3(Qa[0], Qa[1], Qa[2]), R = mk3(Ra[0], Ra[1], Ra[2]);
    v3 V = sub3(Q, P), W = sub3(R, P);
    v3 N = cross3(V, W);
    N = div3(N, len3(N));
    v3 M1 = div3(add3(Q, P), 2), M2 = div3(add3(R, P), 2);
    v3 D1 = cross3(N, V), D2 = cross3(N, W);
    double t = 0.0;
    if (fabs(D1.x * D2.y - D1.y * D2.x) > 1E-13)
        t = (D2.x * (M1.y - M2.y)) / (D1.x * D2.y - D1.y * D2.x) - (D2.y * (M1.x - M2.x)) / (D1.x * D2.y - D1.y * D2.x);
    else if (fabs(D1.x * D2.z - D1.z * D2.x) > 1E-13)
        t = (D2.x * (M1.z - M2.z)) / (D1.x * D2.z - D1.z * D2.x) - (D2.z * (M1.x - M2.x)) / (D1.x * D2.z - D1.z * D2.x);
    else if (fabs(D1.y * D2.z - D1.z * D2.y) > 1E-13)
        t = (D2.y * (M1.z - M2.z)) / (D1.y * D2.z - D1.z * D2.y) - (D2.z * (M1.y - M2.y)) / (D1.y * D2.z - D1.z * D2.y);
    v3 Ctri = add3(M1, mul3(t, D1));
    v3 Csph = mk3(0, 0, 0);
    double fc = 0, tol = 1e-4;
    double r = len3(sub3(P, Ctri));
    for (int it = 0; fabs(fc - ft) > tol && it < 1000; ++it) {
        double d = ft * r;
        double p = d / len3(N);
        Csph = sub3(Ctri, mul3(p, N));
        r = len3(sub3(P, Csph));
        fc = d / r;
    }
    out[0] = Csph.x; out[1] = Csph.y; out[2] = Csph.z; out[3] = r;
}

double xo_sum(const double* in, unsigned int n)
{
    double s = 0.0;
    for (unsigned int i = 0; i < n; ++i) s += in[i];
    return s;
}

/* ======================================================================== */
/* Whole step                                                                */
/* ======================================================================== */
unsigned int xo_step(xo_scene* s)
{
    device_dem_parameters* prm = &s->prm;
    const int clusters = s->ns != s->np;
    unsigned int st = 0;
    /* xIntegratorVV.cpp:66-100 */
    if (clusters)
        xo_vv_cluster_position(prm, s->pos, s->cpos, s->ep, s->rloc, s->vel, s->acc, s->ev, s->ea, s->xci, s->ns);
    else
        xo_vv_update_position(prm, s->pos, s->ep, s->vel, s->ev, s->acc, s->ea, s->np);
    /* xIntegratorVV.cpp:30-44 */
    xo_hash(prm, s->hash, s->index, s->pos, 0, s->np, &st);
    for (unsigned int m = 0; m < s->nmesh; ++m)
        xo_hash(prm, s->hash, s->index, s->tri_sphere + 4 * (size_t)s->tri_begin[m], s->np + s->tri_begin[m],
                s->ntri[m], &st);
    xo_reorder_cellstart(s->hash, s->index, s->cstart, s->cend, s->sorted_index, s->nentry, s->ncell);
    /* xContactManager.cpp:458-472: particle-particle, planes in id order,
       meshes, then the rolling pass */
    if (s->has_pp) {
        if (clusters)
            xo_clusters_p2p(prm, s->pos, s->cpos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax,
                            s->rres, s->pp_count, s->pp_id, s->pp_tsd, s->sorted_index, s->cstart, s->cend,
                            &s->pp_cp, s->xci, s->np, &st);
        else
            xo_p2p(prm, s->pos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax, s->rres,
                   s->pp_count, s->pp_id, s->pp_tsd, s->sorted_index, s->cstart, s->cend, &s->pp_cp, s->np, &st);
    }
    for (unsigned int k = 0; k < s->nplane; ++k) {
        if (clusters)
            xo_cluster_plane(prm, &s->plane[k], s->plane_body + 15 * k, s->bfx, s->bfy, s->bfz, s->bmx, s->bmy,
                             s->bmz, s->pos, s->cpos, s->ep, s->vel, s->ev, s->force, s->moment, &s->plane_cp[k],
                             s->mass, s->tmax, s->rres, s->pl_count, s->pl_id, s->pl_tsd, s->xci, s->np, &st);
        else
            xo_plane(prm, &s->plane[k], s->plane_body + 15 * k, &s->plane_cp[k], s->bfx, s->bfy, s->bfz, s->bmx,
                     s->bmy, s->bmz, s->pos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax,
                     s->rres, s->pl_count, s->pl_id, s->pl_tsd, s->np, &st);
        double* w = s->wrench + 6 * k;
        w[0] = xo_sum(s->bfx, s->np); w[1] = xo_sum(s->bfy, s->np); w[2] = xo_sum(s->bfz, s->np);
        w[3] = xo_sum(s->bmx, s->np); w[4] = xo_sum(s->bmy, s->np); w[5] = xo_sum(s->bmz, s->np);
    }
    for (unsigned int m = 0; m < s->nmesh; ++m) {
        const device_triangle_info* dti = s->tri + s->tri_begin[m];
        if (clusters)
            xo_cluster_mesh(prm, dti, s->mesh_body + 15 * m, s->bfx, s->bfy, s->bfz, s->bmx, s->bmy, s->bmz,
                            s->pos, s->cpos, s->ep, s->vel, s->ev, s->force, s->moment, &s->mesh_cp[m], s->mass,
                            s->tmax, s->rres, s->ms_count, s->ms_id, s->ms_tsd, s->sorted_index, s->cstart,
                            s->cend, s->xci, s->np, s->ntri[m], &st);
        else
            xo_mesh(prm, dti, s->mesh_body + 15 * m, s->bfx, s->bfy, s->bfz, s->bmx, s->bmy, s->bmz, s->pos,
                    s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax, s->rres, s->ms_count, s->ms_id,
                    s->ms_tsd, s->sorted_index, s->cstart, s->cend, &s->mesh_cp[m], s->np, s->ntri[m], &st);
        double* w = s->wrench + 6 * (s->nplane + m);
        w[0] = xo_sum(s->bfx, s->np); w[1] = xo_sum(s->bfy, s->np); w[2] = xo_sum(s->bfz, s->np);
        w[3] = xo_sum(s->bmx, s->np); w[4] = xo_sum(s->bmy, s->np); w[5] = xo_sum(s->bmz, s->np);
    }
    /* The reference runs the sphere rolling pass also for clusters, indexing
       per-cluster arrays by sphere id (xContactManager.cpp:471); clusters use
       the cluster pass here. */
    if (clusters)
        xo_cluster_rolling(prm, s->tmax, s->rres, s->inertia, s->ep, s->ev, s->moment, s->xci, s->np);
    else
        xo_rolling(prm, s->tmax, s->rres, s->inertia, s->ep, s->ev, s->moment, s->np);
    /* xIntegratorVV.cpp:102-154 */
    if (clusters)
        xo_vv_cluster_velocity(prm, s->cpos, s->ep, s->vel, s->acc, s->ev, s->ea, s->force, s->moment, s->rloc,
                               s->mass, s->inertia, s->xci, s->ns);
    else
        xo_vv_update_velocity(prm, s->vel, s->acc, s->ep, s->ev, s->ea, s->force, s->moment, s->mass, s->inertia,
                              s->np, s->vel_compat);
    s->status |= st;
    return st;
}
