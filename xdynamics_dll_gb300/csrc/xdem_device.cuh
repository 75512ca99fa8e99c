// xdem_device.cuh -- device-side math of the DEM step (FP64 form).
//
// Restates the helpers of include/xdynamics_parallel/xParallelDEM_impl.cuh of
// the reference ("impl") as device functions.  Translation units that include
// this header for the FP64 path are compiled with -fmad=false, so sums and
// products round one by one in the order written: cell ids, distance tests and
// plane/triangle region tests then agree bit for bit with the CPU oracle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xdem_c.h"

namespace xdem {

#ifndef XDEM_PI
#define XDEM_PI 3.14159265358979323846
#endif

struct d3 { double x, y, z; };
struct d4 { double x, y, z, w; };

__device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__device__ __forceinline__ d4 mk4(double x, double y, double z, double w) { return d4{x, y, z, w}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ d3 operator-(d3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ d3 operator/(d3 a, double s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ d4 operator+(d4 a, d4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ d4 operator*(double s, d4 a) { return mk4(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double dot(d4 a, d4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ double length(d3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ d3 cross(d3 a, d3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Reference layouts: double4 arrays are 32-byte aligned (cudaMalloc), double3
// arrays are packed 24-byte records.
__device__ __forceinline__ d4 ld4(const double* a, size_t i)
{
    const double4_32a v = reinterpret_cast<const double4_32a*>(a)[i];
    return mk4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ d3 ld4xyz(const double* a, size_t i)
{
    const double2 v = reinterpret_cast<const double2*>(a)[2 * i];
    return mk3(v.x, v.y, a[4 * i + 2]);
}
__device__ __forceinline__ d3 ld3(const double* a, size_t i) { return mk3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
__device__ __forceinline__ void st3(double* a, size_t i, d3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
__device__ __forceinline__ void st4(double* a, size_t i, d4 v)
{
    reinterpret_cast<double4_32a*>(a)[i] = make_double4_32a(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void add3to(double* a, size_t i, d3 v)
{
    a[3 * i] += v.x; a[3 * i + 1] += v.y; a[3 * i + 2] += v.z;
}
__device__ __forceinline__ d3 dv3(const xdem_double3& v) { return mk3(v.x, v.y, v.z); }

// ---------------------------------------------------------------- Euler parameters
// Rotation matrix rows of e = (e0,e1,e2,e3) held as (x,y,z,w) (impl:8-30).
__device__ __forceinline__ void rot_rows(d4 e, d3& r0, d3& r1, d3& r2)
{
    r0 = mk3(2.0 * (e.x * e.x + e.y * e.y - 0.5), 2.0 * (e.y * e.z - e.x * e.w), 2.0 * (e.y * e.w + e.x * e.z));
    r1 = mk3(2.0 * (e.y * e.z + e.x * e.w), 2.0 * (e.x * e.x + e.z * e.z - 0.5), 2.0 * (e.z * e.w - e.x * e.y));
    r2 = mk3(2.0 * (e.y * e.w - e.x * e.z), 2.0 * (e.z * e.w + e.x * e.y), 2.0 * (e.x * e.x + e.w * e.w - 0.5));
}
__device__ __forceinline__ d3 to_global(d3 v, d4 e)
{
    d3 r0, r1, r2; rot_rows(e, r0, r1, r2);
    return mk3(r0.x * v.x + r0.y * v.y + r0.z * v.z, r1.x * v.x + r1.y * v.y + r1.z * v.z,
               r2.x * v.x + r2.y * v.y + r2.z * v.z);
}
__device__ __forceinline__ d3 to_local(d3 v, d4 e)
{
    d3 r0, r1, r2; rot_rows(e, r0, r1, r2);
    return mk3(r0.x * v.x + r1.x * v.y + r2.x * v.z, r0.y * v.x + r1.y * v.y + r2.y * v.z,
               r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
// impl:32-41: omega = 2 G(e) e_dot
__device__ __forceinline__ d3 ang_vel(d4 e, d4 d)
{
    d3 o = mk3(-e.y * d.x + e.x * d.y - e.w * d.z + e.z * d.w, -e.z * d.x + e.w * d.y + e.x * d.z - e.y * d.w,
               -e.w * d.x - e.z * d.y + e.y * d.z + e.x * d.w);
    return 2.0 * o;
}

// Euler-parameter acceleration of impl:74-133.  The 4x4 system is
// [2 J_i L_i(e); e^T] q = [n' - L(e) 4 L(e_dot)^T (J L(e) e_dot); -e_dot.e_dot]
// with L_0 = (-e1, e0, e3, -e2), L_1 = (-e2, -e3, e0, e1),
// L_2 = (-e3, e2, -e1, e0).  The rows L_i(e) are orthogonal to e and to each
// other with norm |e|, so the inverse is [L_i^T / (2 J_i |e|^2), e / |e|^2]:
// closed form, no determinant.
__device__ __forceinline__ d4 uceom(d3 J, d4 e, d4 ev, d3 n)
{
    const double T0 = J.x * (-e.y * ev.x + e.x * ev.y + e.w * ev.z - e.z * ev.w);
    const double T1 = J.y * (-e.z * ev.x - e.w * ev.y + e.x * ev.z + e.y * ev.w);
    const double T2 = J.z * (-e.w * ev.x + e.z * ev.y - e.y * ev.z + e.x * ev.w);
    const d4 h = mk4(4.0 * (-ev.y * T0 - ev.z * T1 - ev.w * T2), 4.0 * (ev.x * T0 - ev.w * T1 + ev.z * T2),
                     4.0 * (ev.w * T0 + ev.x * T1 - ev.y * T2), 4.0 * (-ev.z * T0 + ev.y * T1 + ev.x * T2));
    const double r0 = n.x - (-e.y * h.x + e.x * h.y + e.w * h.z - e.z * h.w);
    const double r1 = n.y - (-e.z * h.x - e.w * h.y + e.x * h.z + e.y * h.w);
    const double r2 = n.z - (-e.w * h.x + e.z * h.y - e.y * h.z + e.x * h.w);
    const double r3 = -dot(ev, ev);
    const double e2 = dot(e, e);
    const double a0 = r0 / (2.0 * J.x * e2), a1 = r1 / (2.0 * J.y * e2), a2 = r2 / (2.0 * J.z * e2);
    const double a3 = r3 / e2;
    return mk4(-e.y * a0 - e.z * a1 - e.w * a2 + e.x * a3, e.x * a0 - e.w * a1 + e.z * a2 + e.y * a3,
               e.w * a0 + e.x * a1 - e.y * a2 + e.z * a3, -e.z * a0 + e.y * a1 + e.x * a2 + e.w * a3);
}

// ---------------------------------------------------------------- grid (impl:54-72)
__device__ __forceinline__ int floor_to_int(double v) { return __double2int_rz(floor(v)); }
struct int3v { int x, y, z; };
__device__ __forceinline__ int3v grid_pos(const device_dem_parameters& p, d3 q)
{
    return int3v{floor_to_int((q.x - p.world_origin.x) / p.cell_size),
                 floor_to_int((q.y - p.world_origin.y) / p.cell_size),
                 floor_to_int((q.z - p.world_origin.z) / p.cell_size)};
}
__device__ __forceinline__ unsigned int grid_hash(const device_dem_parameters& p, int gx, int gy, int gz)
{
    const unsigned int x = (unsigned int)(gx & (int)(p.grid_size.x - 1));
    const unsigned int y = (unsigned int)(gy & (int)(p.grid_size.y - 1));
    const unsigned int z = (unsigned int)(gz & (int)(p.grid_size.z - 1));
    return (z * p.grid_size.y) * p.grid_size.x + y * p.grid_size.x + x;
}

// ---------------------------------------------------------------- contact constants (impl:362-386)
struct fconst { double kn, vn, ks, vs, mu, eq_r, eq_m; };

// Terms of getConstant that depend only on the material pair, evaluated once
// per launch instead of once per contact (log, sqrt and four divisions).
struct mat_pair {
    double Eeq, Seq8, beta, vs1, sratio, fric, s_fric, rfric, coh;
    double Ei, Ej, pri, prj;
};

__host__ __device__ inline mat_pair make_mat_pair(const device_contact_property& cp, int model, bool swap_fric)
{
    mat_pair m;
    const double iE = cp.Ei, jE = cp.Ej, ip = cp.pri, jp = cp.prj;
    m.Eeq = (iE * jE) / (iE * (1 - jp * jp) + jE * (1 - ip * ip));
    double Seq = (2.0 * (2.0 - ip) * (1.0 + ip) / iE) + (2.0 * (2.0 - jp) * (1.0 + jp) / jE);
    Seq = 1.0 / Seq;
    m.Seq8 = 8.0 * Seq;
    const double lne = log(cp.rest);
    m.beta = -lne * sqrt(1.0 / (lne * lne + XDEM_PI * XDEM_PI));
    m.vs1 = model == 1 ? 2.0 * sqrt(5.0 / 6.0) * m.beta : m.beta * cp.sratio;
    m.sratio = cp.sratio;
    // impl:898-901: the cluster-plane kernel passes s_fric where fric goes
    m.fric = swap_fric ? cp.s_fric : cp.fric;
    m.s_fric = swap_fric ? cp.fric : cp.s_fric;
    m.rfric = cp.rfric;
    m.coh = cp.coh;
    m.Ei = cp.Ei; m.Ej = cp.Ej; m.pri = cp.pri; m.prj = cp.prj;
    return m;
}

__device__ __forceinline__ fconst get_constant(const mat_pair& m, int model, double ir, double jr, double im,
                                               double jm)
{
    fconst c;
    c.eq_m = jm ? (im * jm) / (im + jm) : im;
    c.eq_r = jr ? (ir * jr) / (ir + jr) : ir;
    c.kn = (4.0 / 3.0) * m.Eeq * sqrt(c.eq_r);
    c.vn = m.beta;
    c.ks = model == 1 ? m.Seq8 : c.kn * m.sratio;
    c.vs = m.vs1;
    c.mu = m.fric;
    return c;
}

// impl:388-430 (cohesion terms; zero when coh == 0)
__device__ __forceinline__ double cohesion_force(const mat_pair& m, double ri, double rj, double Fn)
{
    double cf = 0.0;
    if (m.coh) {
        const double Req = rj ? (ri * rj) / (ri + rj) : ri;
        const double Eeq = 1.0 / (((1.0 - m.pri * m.pri) / m.Ei) + ((1.0 - m.prj * m.prj) / m.Ej));
        const double c0 = 3.0 * m.coh * XDEM_PI * Req;
        const double eq = 2.0 * c0 * Fn + c0 * c0;
        if (eq <= 0) Fn = -0.5 * c0;
        const double a3 = (3.0 * Req) * (Fn + c0 + sqrt(fabs(2.0 * c0 * Fn + c0 * c0))) / (4.0 * Eeq);
        cf = -sqrt(8.0 * XDEM_PI * m.coh * Eeq * a3);
    }
    return cf;
}
__device__ __forceinline__ double limit_cohesion_depth(const mat_pair& m, double ir, double jr)
{
    const double Req = jr ? (ir * jr) / (ir + jr) : ir;
    const double Eeq = 1.0 / (((1.0 - m.pri * m.pri) / m.Ei) + ((1.0 - m.prj * m.prj) / m.Ej));
    const double c1 = (XDEM_PI * XDEM_PI * m.coh * m.coh * Req) / (Eeq * Eeq);
    return -(3.0 / 4.0) * pow(c1, 1.0 / 3.0);
}
__device__ __forceinline__ double jkr_separation_force(const mat_pair& m, double ir, double jr)
{
    const double Req = jr ? (ir * jr) / (ir + jr) : ir;
    return -(3.0 / 2.0) * XDEM_PI * m.coh * Req;
}

// impl:432-474.  Ft is written only when the tangential relative velocity is
// non-zero; otherwise the caller's previous Ft stays, as in the reference.
__device__ __forceinline__ void contact_model(int model, const fconst& c, const mat_pair& m, double ir, double jr,
                                              double dt, double cdist, double& ds_io, double& dots_io, d3 dv,
                                              d3 unit, d3& Ft, d3& Fn)
{
    const double fsn = -c.kn * (cdist * sqrt(cdist));
    const double fdn = c.vn * dot(dv, unit);
    const double fca = -cohesion_force(m, ir, jr, fsn + fdn);
    Fn = (fsn + fca + fdn) * unit;
    const d3 e = dv - dot(dv, unit) * unit;
    const double mag_e = length(e);
    if (mag_e) {
        const d3 s_hat = e / mag_e;
        const double s_dot = dot(dv, s_hat);
        const double ds = ds_io + dt * (s_dot + dots_io);
        ds_io = ds;
        dots_io = s_dot;
        double a;
        if (model == 1) {
            const double S_t = c.ks * sqrt(c.eq_r * cdist);
            a = S_t * ds + c.vs * sqrt(S_t * c.eq_m);
        } else {
            a = c.ks * ds + c.vs * dot(dv, s_hat);
        }
        const double b = c.mu * length(Fn);
        Ft = (a < b ? a : b) * s_hat;
    }
}

// impl:476-483
__device__ __forceinline__ void rolling_accumulate(double rf, double ir, double jr, d3 rc, d3 Fn, d3 Ft, double& Mr,
                                                   d3& Tmax)
{
    Tmax = Tmax + cross(rc, Fn + Ft);
    const double Rij = jr ? ir * jr / (ir + jr) : ir;
    Mr += Rij * rf * length(Fn);
}

// ---------------------------------------------------------------- cylinder regions (impl:1083-1322)
// Shared by the launcher kernel (xdem_kernels.cu) and the mixed step's body
// kernel, so both classify a sphere against a cylinder with the same FP64
// arithmetic.
// Base and top centres of a cylinder at its body pose.
__device__ __forceinline__ void cylinder_ends(const device_cylinder_info& cy, const double* bi, d3& pos, d4& e,
                                              d3& base, d3& top)
{
    pos = mk3(bi[XDEM_PX], bi[XDEM_PY], bi[XDEM_PZ]);
    e = mk4(bi[XDEM_E0], bi[XDEM_E1], bi[XDEM_E2], bi[XDEM_E3]);
    base = pos + to_global(dv3(cy.pbase), e);
    top = pos + to_global(dv3(cy.ptop), e);
}

// impl:1189-1288: depth and unit vector of sphere (p, r) against the
// cylinder -- side (axis parameter in [0, 1]; an inside contact flips the
// normal and sets `inner`), the wall annulus beyond the ends, else the rim
// point through the angle atan(x / z) of the local offset, as the reference
// forms it.
__device__ inline double cylinder_detection(const device_cylinder_info& cy, const double* bi, d3 p, d3& u, double r,
                                     bool& inner)
{
    d3 cyl_pos, base, top;
    d4 e;
    cylinder_ends(cy, bi, cyl_pos, e, base, top);
    const d3 ab = top - base;
    const double t = dot(p - base, ab) / dot(ab, ab);
    const d3 c = base + t * ab;
    double dist = length(p - c);
    if (t >= 0 && t <= 1) {
        if (dist == 0) {
            inner = true;
            return 0;
        }
        u = (c - p) / dist;
        if (dist < cy.len_rr.z) {
            inner = true;
            u = -u;
            return dist + r - cy.len_rr.y;
        }
        return cy.len_rr.y + r - dist;
    }
    const double thick = cy.thickness;
    const int one = thick != 0.0 ? 1 : 0;
    if (dist < cy.len_rr.z + thick && dist > one * cy.len_rr.z) {
        const d3 o2c = cyl_pos - c;
        const double l = length(o2c);
        u = o2c / l;
        return cy.len_rr.x * 0.5 + r - l;
    }
    d3 at = to_local(p - top, e);
    d3 cp = top;
    if (fabs(at.y) > cy.len_rr.x) {
        at = to_local(p - base, e);
        cp = base;
    }
    const double pi = atan(at.x / at.z);
    d3 q = mk3(0, 0, 0);
    if (pi < 0 && at.z < 0) q.x = cy.len_rr.z * sin(-pi);
    else if (pi > 0 && at.x < 0 && at.z < 0) q.x = cy.len_rr.z * sin(-pi);
    else q.x = cy.len_rr.z * sin(pi);
    q.z = cy.len_rr.z * cos(pi);
    if (at.z < 0 && q.z > 0) q.z = -q.z;
    else if (at.z > 0 && q.z < 0) q.z = -q.z;
    q.y = 0.;
    cp = cp + to_global(q, e);
    const d3 dv = cp - p;
    dist = length(dv);
    u = dv / dist;
    if (dist < r) return r - dist;
    return -1.0;
}

// impl:1290-1322: the cap a sphere inside the cylinder faces (none near an
// open end: empty 1 top for t > 0.6, empty 2 base for t < 0.4).
__device__ inline double cylinder_inner_cap(const device_cylinder_info& cy, const double* bi, d3 p, d3& u, d3& cpt,
                                     unsigned int empty, double r)
{
    d3 cyl_pos, base, top;
    d4 e;
    cylinder_ends(cy, bi, cyl_pos, e, base, top);
    const d3 ab = top - base;
    const double t = dot(p - base, ab) / dot(ab, ab);
    const d3 c = base + t * ab;
    const double dist = length(p - c);
    if (empty == 1 && t > 0.6) return 0.0;
    if (empty == 2 && t < 0.4) return 0.0;
    double gab = -1.0;
    if (dist < cy.len_rr.z) {
        const d3 o2c = cyl_pos - c;
        const double l = length(o2c);
        u = -(o2c / l);
        cpt = p + r * u;
        gab = r + l - cy.len_rr.x * 0.5;
    }
    return gab;
}

// ---------------------------------------------------------------- plane (impl:735-815)
__device__ __forceinline__ double plane_detection(const device_plane_info& pe, d3 xp, d3 wp, d3& u, double r)
{
    const double a_l1 = (wp.x - pe.l1) * (wp.x - pe.l1);
    const double b_l2 = (wp.y - pe.l2) * (wp.y - pe.l2);
    const double sqa = wp.x * wp.x, sqb = wp.y * wp.y, sqc = wp.z * wp.z, sqr = r * r;
    const d3 xw = dv3(pe.xw), w2 = dv3(pe.w2), w3 = dv3(pe.w3), w4 = dv3(pe.w4);
    if (wp.x < 0 && wp.y < 0 && (sqa + sqb + sqc) < sqr) {
        const d3 X = xp - xw; const double h = length(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y < 0 && (a_l1 + sqb + sqc) < sqr) {
        const d3 X = xp - w2; const double h = length(X); u = X / h; return r - h;
    } else if (wp.x > pe.l1 && wp.y > pe.l2 && (a_l1 + b_l2 + sqc) < sqr) {
        const d3 X = xp - w3; const double h = length(X); u = X / h; return r - h;
    } else if (wp.x < 0 && wp.y > pe.l2 && (sqa + b_l2 + sqc) < sqr) {
        const d3 X = xp - w4; const double h = length(X); u = X / h; return r - h;
    }
    if ((wp.x > 0 && wp.x < pe.l1) && wp.y < 0 && (sqb + sqc) < sqr) {
        const d3 X = xp - xw; const d3 e = w2 - xw; const d3 us = e / length(e);
        const d3 hs = X - dot(X, us) * us; const double h = length(hs);
        u = (-hs) / h; return r - h;
    } else if ((wp.x > 0 && wp.x < pe.l1) && wp.y > pe.l2 && (b_l2 + sqc) < sqr) {
        const d3 X = xp - w4; const d3 e = w3 - w4; const d3 us = e / length(e);
        const d3 hs = X - dot(X, us) * us; const double h = length(hs);
        u = (-hs) / h; return r - h;
    } else if ((wp.x > 0 && wp.y < pe.l2) && wp.x > pe.l1 && (a_l1 + sqc) < sqr) {
        // (the edge test of impl:787 can never hold and is left out)
        const d3 X = xp - w2; const d3 e = w3 - w2; const d3 us = e / length(e);
        const d3 hs = X - dot(X, us) * us; const double h = length(hs);
        u = (-hs) / h; return r - h;
    } else if ((wp.x > 0 && wp.x < pe.l1) && (wp.y > 0 && wp.y < pe.l2)) {
        const d3 dp = xp - xw;
        const d3 uw = dv3(pe.uw);
        const d3 uu = uw / length(uw);
        u = -uu;
        return r - fabs(dot(dp, u));
    }
    return 0;
}

// ---------------------------------------------------------------- triangle (impl:1655-1746)
__device__ __forceinline__ d3 closest_pt_triangle(const device_triangle_info& t, d3 p, int& ct)
{
    const d3 a = dv3(t.P), b = dv3(t.Q), c = dv3(t.R);
    const d3 ab = b - a, ac = c - a, ap = p - a, bp = p - b, cp = p - c;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap), d3_ = dot(ab, bp), d4 = dot(ac, bp);
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    const double va = d3_ * d6 - d5 * d4, vb = d5 * d2 - d1 * d6, vc = d1 * d4 - d3_ * d2;
    d3 cpt = mk3(0, 0, 0);
    if (d1 <= 0.0 && d2 <= 0.0) { ct = 0; cpt = a; }
    if (d3_ >= 0.0 && d4 <= d3_) { ct = 0; cpt = b; }
    if (d6 >= 0.0 && d5 <= d6) { ct = 0; cpt = c; }
    if (vc <= 0.0 && d1 >= 0.0 && d3_ <= 0.0) { ct = 1; cpt = a + (d1 / (d1 - d3_)) * ab; }
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) { ct = 1; cpt = a + (d2 / (d2 - d6)) * ac; }
    if (va <= 0.0 && (d4 - d3_) >= 0.0 && (d5 - d6) >= 0.0) {
        ct = 1; cpt = b + ((d4 - d3_) / ((d4 - d3_) + (d5 - d6))) * (c - b);
    }
    if (va >= 0 && vb >= 0 && vc >= 0) {
        const double denom = 1.0 / (va + vb + vc);
        const d3 v = (vb * denom) * ab;
        const d3 w = (vc * denom) * ac;
        cpt = (a + v) + w;
        ct = 2;
    }
    return cpt;
}

__device__ __forceinline__ bool check_overlap(d3 p, d3 c)
{
    return (p.x >= c.x - 1e-9 && p.x <= c.x + 1e-9) && (p.y >= c.y - 1e-9 && p.y <= c.y + 1e-9) &&
           (p.z >= c.z - 1e-9 && p.z <= c.z + 1e-9);
}

struct body_state { d3 p, v, om; double m; };
__device__ __forceinline__ body_state load_body(const double* dbi)
{
    body_state b;
    b.m = dbi[XDEM_MM];
    b.p = mk3(dbi[XDEM_PX], dbi[XDEM_PY], dbi[XDEM_PZ]);
    b.v = mk3(dbi[XDEM_VX], dbi[XDEM_VY], dbi[XDEM_VZ]);
    b.om = ang_vel(mk4(dbi[XDEM_E0], dbi[XDEM_E1], dbi[XDEM_E2], dbi[XDEM_E3]),
                   mk4(dbi[XDEM_ED0], dbi[XDEM_ED1], dbi[XDEM_ED2], dbi[XDEM_ED3]));
    return b;
}

// Cluster object lookup (impl:500-510): members of object k are
// [sid, sid + count*neach).
__device__ __forceinline__ unsigned int cluster_neach(const xClusterInformation* xci, unsigned int nco,
                                                      unsigned int id)
{
    for (unsigned int i = 0; i < nco; ++i) {
        const xClusterInformation c = xci[i];
        if (id >= c.sid && id < c.sid + c.count * c.neach) return c.neach;
    }
    return 0;
}

}  // namespace xdem
