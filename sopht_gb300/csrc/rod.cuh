// Discrete Cosserat rod dynamics, one position-Verlet sub-step split into passes over nodes,
// elements and Voronoi regions (Gazzola, Dudte, McCormick & Mahadevan 2018, "Forward and inverse
// problems in the mechanics of soft filaments", R. Soc. Open Sci. 5:171628: the model pyelastica
// 0.3.3 implements and SophT couples its rods through).
//
// Every function here is __host__ __device__ and free of CUDA runtime calls: the batched kernel
// (rod.cu) runs the passes with one CTA per rod and barriers between them, and a host driver
// compiled from this same header runs them in sequence, which is how the arithmetic is checked
// against the numpy model on a machine without a GPU.
//
// Per sub-step (h = dt / 2):  drift x += h v and rotate Q <- exp(-h [w]x) Q;  element pass
// (tangent, dilatation e, strain sigma = e Q t - e3, stress n = S (sigma - sigma0), the lab force
// Q^T n / e, the shear couple (Q t x n) l0, the transport term (J w / e) x w and the dilatation
// term (J w / e^2) de/dt);  Voronoi pass (kappa = -log(Q_{k+1} Q_k^T) / D0, eps, m = B (kappa -
// kappa0), m / eps^3 and (kappa x m) D0 / eps^3);  node update (force differences, v += dt a) and
// element update (couple differences and averages, w += dt e J^-1 (couple + C_ext));  drift and
// rotate again.  A clamped rod keeps node 0 and the directors of element 0 fixed.
#pragma once

#include <math.h>

#include "../../include/sopht_gb300.h"

#ifdef __CUDACC__
#define SG_ROD_FN __host__ __device__ inline
#else
#define SG_ROD_FN inline
#endif

namespace sg {
namespace rod {

// One rod of a batch: its slices of the batch arrays (C order, as sg_rod_batch documents).
struct View {
    int n;
    double* x;
    double* v;
    double* q;
    double* w;
    const double* mass;
    const double* l0;
    const double* d0;
    const double* shear;
    const double* bend;
    const double* inertia;
    const double* inv_inertia;
    const double* sigma0;
    const double* kappa0;
    const double* f_ext;
    const double* c_ext;
    int clamped;
    const double* clamp_x;
    const double* clamp_q;
    const double* clamp_w;  // angular velocity of a driven clamp (local frame), or null: at rest
    // 1 / mass, 1 / l0, 1 / d0 computed once by the caller, or null: divided where used (the same
    // values either way)
    const double* inv_mass;
    const double* inv_l0;
    const double* inv_d0;
};

SG_ROD_FN View view_of(const sg_rod_batch& b, int r) {
    const int n = b.n_elems;
    const int64_t nn = n + 1, ne = n, nv = n - 1;
    View v;
    v.n = n;
    v.x = b.position + r * 3 * nn;
    v.v = b.velocity + r * 3 * nn;
    v.q = b.directors + r * 9 * ne;
    v.w = b.omega + r * 3 * ne;
    v.mass = b.mass + r * nn;
    v.l0 = b.rest_lengths + r * ne;
    v.d0 = b.rest_voronoi_lengths + r * nv;
    v.shear = b.shear_matrix + r * 9 * ne;
    v.bend = b.bend_matrix + r * 9 * nv;
    v.inertia = b.mass_second_moment + r * 9 * ne;
    v.inv_inertia = b.inv_mass_second_moment + r * 9 * ne;
    v.sigma0 = b.rest_sigma + r * 3 * ne;
    v.kappa0 = b.rest_kappa + r * 3 * nv;
    v.f_ext = b.external_forces + r * 3 * nn;
    v.c_ext = b.external_torques + r * 3 * ne;
    v.clamped = b.clamped ? b.clamped[r] : 0;
    v.clamp_x = b.clamp_position + r * 3;
    v.clamp_q = b.clamp_directors + r * 9;
    v.clamp_w = nullptr;
    v.inv_mass = nullptr;
    v.inv_l0 = nullptr;
    v.inv_d0 = nullptr;
    return v;
}

// Work arrays of one rod (shared memory on the GPU): 16 n + 6 (n - 1) doubles.
struct Scratch {
    double* nlab;       // (3, n)  Q^T n / e
    double* shear_c;    // (3, n)  (Q t x n) l0
    double* transport;  // (3, n)  (J w / e) x w
    double* dil_c;      // (3, n)  (J w / e^2) de/dt
    double* e;          // (n)
    double* len;        // (n)
    double* bend_c;     // (3, n-1) m / eps^3
    double* twist_c;    // (3, n-1) (kappa x m) D0 / eps^3
};

SG_ROD_FN int scratch_doubles(int n) { return 16 * n + 6 * (n > 1 ? n - 1 : 0); }

SG_ROD_FN Scratch carve(double* base, int n) {
    Scratch s;
    const int nv = n > 1 ? n - 1 : 0;
    s.nlab = base;
    s.shear_c = s.nlab + 3 * n;
    s.transport = s.shear_c + 3 * n;
    s.dil_c = s.transport + 3 * n;
    s.e = s.dil_c + 3 * n;
    s.len = s.e + n;
    s.bend_c = s.len + n;
    s.twist_c = s.bend_c + 3 * nv;
    return s;
}

// ---------------------------------------------------------------- rotations

// exp([a]x) by Rodrigues' formula, row-major 3x3: I + (sin t / t) [a]x + ((1 - cos t) / t^2) [a]x^2,
// t = |a|.  The rotations of a sub-step are small (t = |omega| dt / 2), and for t < 0.1 both
// coefficients come from their Taylor series in t^2 (the omitted terms are below 3e-18 relative):
// no square root, division, sine or cosine, which cost tens of operations each on this GPU's
// narrow double-precision pipe.
SG_ROD_FN void rotation_exp(const double a[3], double r[9]) {
    const double t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    double sa, ca;  // sin t / t and (1 - cos t) / t^2
    if (t2 < 0.01) {
        sa = 1.0 + t2 * (-1.0 / 6.0 + t2 * (1.0 / 120.0 + t2 * (-1.0 / 5040.0 + t2 * (1.0 / 362880.0))));
        ca = 0.5 + t2 * (-1.0 / 24.0 + t2 * (1.0 / 720.0 + t2 * (-1.0 / 40320.0 + t2 * (1.0 / 3628800.0))));
    } else {
        const double t = sqrt(t2);
        sa = sin(t) / t;
        ca = (1.0 - cos(t)) / t2;
    }
    // [a]x = (0, -a2, a1; a2, 0, -a0; -a1, a0, 0) and [a]x^2 = a a^T - t^2 I, written out: 21
    // operations where the 3x3 products with their zero entries take 45
    const double p01 = a[0] * a[1], p02 = a[0] * a[2], p12 = a[1] * a[2];
    const double s0 = sa * a[0], s1 = sa * a[1], s2 = sa * a[2];
    r[0] = 1.0 + ca * -(a[1] * a[1] + a[2] * a[2]);
    r[4] = 1.0 + ca * -(a[0] * a[0] + a[2] * a[2]);
    r[8] = 1.0 + ca * -(a[0] * a[0] + a[1] * a[1]);
    r[1] = ca * p01 - s2;
    r[3] = ca * p01 + s2;
    r[2] = ca * p02 + s1;
    r[6] = ca * p02 - s1;
    r[5] = ca * p12 - s0;
    r[7] = ca * p12 + s0;
}

// The rotation vector of r (angle below pi), the angle taken from the trace as the rod model does
// (the trace and the antisymmetric part give different angles once r drifts from orthogonality):
// f (r - r^T) with f = theta / (2 sin theta), theta = arccos(c), c the clamped (trace - 1) / 2.
// For u = 1 - c below 0.01 (theta below 0.1415, the Voronoi rotations of a sub-step) f is the
// Taylor series of that same function of c in u, 1/2 + u/6 + u^2/15 + u^3/35 + 4u^4/315 +
// 4u^5/693 + 8u^6/3003 + 8u^7/6435 + 64u^8/109395 (the next term is below 3e-20 of f there), with
// no arccosine, sine or division on the narrow double-precision pipe; above it, sin theta is
// sqrt(u (1 + c)).  u is exact (Sterbenz) for c in [1/2, 1].
SG_ROD_FN void rotation_log(const double r[9], double a[3]) {
    double cosv = (r[0] + r[4] + r[8] - 1.0) / 2.0;
    cosv = cosv < -1.0 ? -1.0 : (cosv > 1.0 ? 1.0 : cosv);
    const double u = 1.0 - cosv;
    double f;
    if (u < 0.01) {
        f = 0.5 + u * (1.0 / 6.0 + u * (1.0 / 15.0 + u * (1.0 / 35.0 + u * (4.0 / 315.0 + u * (4.0 / 693.0 +
            u * (8.0 / 3003.0 + u * (8.0 / 6435.0 + u * (64.0 / 109395.0))))))));
    } else {
        const double theta = acos(cosv);
        const double s = sqrt(u * (1.0 + cosv));
        f = theta / (2.0 * (s == 0.0 ? 1.0 : s));
    }
    a[0] = f * (r[7] - r[5]);
    a[1] = f * (r[2] - r[6]);
    a[2] = f * (r[3] - r[1]);
}

SG_ROD_FN void cross(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// m (3, 3, count) at column e times v.
SG_ROD_FN void matvec(const double* m, int count, int e, const double v[3], double out[3]) {
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc += m[(i * 3 + j) * count + e] * v[j];
        out[i] = acc;
    }
}

// --------------------------------------------------------------- the passes

SG_ROD_FN void clamp_node0(View& r) {
    for (int a = 0; a < 3; ++a) {
        r.x[a * (r.n + 1)] = r.clamp_x[a];
        r.v[a * (r.n + 1)] = 0.0;
    }
}

SG_ROD_FN void clamp_element0(View& r) {
    for (int a = 0; a < 9; ++a) r.q[a * r.n] = r.clamp_q[a];
    for (int a = 0; a < 3; ++a) r.w[a * r.n] = r.clamp_w ? r.clamp_w[a] : 0.0;
}

// A clamp driven by a rotation of the rod's base: element 0's directors at time t are Q0 R^T, with
// R = exp([theta a]x) the turn of the lab frame by theta(t) = A sin(2 pi f t + phi) about the unit lab
// axis a (each director d_i -> R d_i), and its angular velocity in the local frame Q0 R^T (theta' a).
SG_ROD_FN void driven_clamp(const double* q0, const double axis[3], double amp, double freq, double phase,
                            double t, double q[9], double w[3]) {
    const double two_pi = 6.283185307179586476925286766559;
    const double arg = two_pi * freq * t + phase;
    const double theta = amp * sin(arg), rate = amp * two_pi * freq * cos(arg);
    const double a[3] = {theta * axis[0], theta * axis[1], theta * axis[2]};
    double rot[9];
    rotation_exp(a, rot);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int m = 0; m < 3; ++m) acc += q0[i * 3 + m] * rot[j * 3 + m];
            q[i * 3 + j] = acc;
        }
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc += q[i * 3 + j] * axis[j] * rate;
        w[i] = acc;
    }
}

SG_ROD_FN void drift_node(View& r, int i, double h) {
    const int nn = r.n + 1;
    for (int a = 0; a < 3; ++a) r.x[a * nn + i] += h * r.v[a * nn + i];
    if (r.clamped && i == 0) clamp_node0(r);
}

SG_ROD_FN void rotate_element(View& r, int e, double h) {
    const int n = r.n;
    double a[3], rot[9], q[9];
    for (int k = 0; k < 3; ++k) a[k] = -h * r.w[k * n + e];
    rotation_exp(a, rot);
    for (int k = 0; k < 9; ++k) q[k] = r.q[k * n + e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int m = 0; m < 3; ++m) acc += rot[i * 3 + m] * q[m * 3 + j];
            r.q[(i * 3 + j) * n + e] = acc;
        }
    if (r.clamped && e == 0) clamp_element0(r);
}

// Two consecutive half drifts with the same velocity (the closing one of a sub-step and the opening
// one of the next: nothing changes v or w between them), computed as the two separately are --
// two additions, one rotation exp(-h [w]x) applied twice -- so the result is bitwise that of
// drift_node and rotate_element called twice, without the second rotation's exponential.  A
// clamped node 0 and element 0 end at the clamp as they would.
SG_ROD_FN void drift_node_twice(View& r, int i, double h) {
    const int nn = r.n + 1;
    for (int a = 0; a < 3; ++a) {
        r.x[a * nn + i] += h * r.v[a * nn + i];
        r.x[a * nn + i] += h * r.v[a * nn + i];
    }
    if (r.clamped && i == 0) clamp_node0(r);
}

SG_ROD_FN void rotate_element_twice(View& r, int e, double h) {
    const int n = r.n;
    double a[3], rot[9], q[9], p[9];
    for (int k = 0; k < 3; ++k) a[k] = -h * r.w[k * n + e];
    rotation_exp(a, rot);
    for (int k = 0; k < 9; ++k) q[k] = r.q[k * n + e];
    for (int rep = 0; rep < 2; ++rep) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int m = 0; m < 3; ++m) acc += rot[i * 3 + m] * q[m * 3 + j];
                p[i * 3 + j] = acc;
            }
        for (int k = 0; k < 9; ++k) q[k] = p[k];
    }
    for (int k = 0; k < 9; ++k) r.q[k * n + e] = q[k];
    if (r.clamped && e == 0) clamp_element0(r);
}

SG_ROD_FN void element_pass(const View& r, const Scratch& s, int e) {
    const int n = r.n, nn = n + 1;
    double d[3], t[3], qt[3], sig[3], stress[3];
    for (int a = 0; a < 3; ++a) d[a] = r.x[a * nn + e + 1] - r.x[a * nn + e];
    // divisions by their reciprocals: a double division is an iteration of many operations here
    const double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double inv_len = 1.0 / len, inv_l0 = r.inv_l0 ? r.inv_l0[e] : 1.0 / r.l0[e];
    for (int a = 0; a < 3; ++a) t[a] = d[a] * inv_len;
    const double dil = len * inv_l0, inv_dil = 1.0 / dil;
    matvec(r.q, n, e, t, qt);
    for (int a = 0; a < 3; ++a) sig[a] = dil * qt[a] - (a == 2 ? 1.0 : 0.0) - r.sigma0[a * n + e];
    matvec(r.shear, n, e, sig, stress);
    for (int a = 0; a < 3; ++a) {  // Q^T n / e
        double acc = 0.0;
        for (int b = 0; b < 3; ++b) acc += r.q[(b * 3 + a) * n + e] * stress[b];
        s.nlab[a * n + e] = acc * inv_dil;
    }
    double sc[3];
    cross(qt, stress, sc);
    for (int a = 0; a < 3; ++a) s.shear_c[a * n + e] = sc[a] * r.l0[e];
    double w[3], jw[3], tr[3];
    for (int a = 0; a < 3; ++a) w[a] = r.w[a * n + e];
    matvec(r.inertia, n, e, w, jw);
    cross(jw, w, tr);
    double rate = 0.0;
    for (int a = 0; a < 3; ++a) rate += t[a] * (r.v[a * nn + e + 1] - r.v[a * nn + e]);
    rate *= inv_l0;
    for (int a = 0; a < 3; ++a) {
        s.transport[a * n + e] = tr[a] * inv_dil;
        s.dil_c[a * n + e] = jw[a] * (inv_dil * inv_dil) * rate;
    }
    s.e[e] = dil;
    s.len[e] = len;
}

SG_ROD_FN void voronoi_pass(const View& r, const Scratch& s, int k) {
    const int n = r.n, nv = n - 1;
    double rel[9], lg[3], kappa[3], m[3], km[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {  // Q_{k+1} Q_k^T
            double acc = 0.0;
            for (int c = 0; c < 3; ++c) acc += r.q[(i * 3 + c) * n + k + 1] * r.q[(j * 3 + c) * n + k];
            rel[i * 3 + j] = acc;
        }
    rotation_log(rel, lg);
    const double inv_d0 = r.inv_d0 ? r.inv_d0[k] : 1.0 / r.d0[k];
    for (int a = 0; a < 3; ++a) kappa[a] = -lg[a] * inv_d0;
    const double eps = 0.5 * (s.len[k + 1] + s.len[k]) * inv_d0;
    const double inv_eps3 = 1.0 / (eps * eps * eps);
    double dk[3];
    for (int a = 0; a < 3; ++a) dk[a] = kappa[a] - r.kappa0[a * nv + k];
    matvec(r.bend, nv, k, dk, m);
    cross(kappa, m, km);
    for (int a = 0; a < 3; ++a) {
        s.bend_c[a * nv + k] = m[a] * inv_eps3;
        s.twist_c[a * nv + k] = km[a] * r.d0[k] * inv_eps3;
    }
}

SG_ROD_FN void node_update(View& r, const Scratch& s, int i, double dt, double decay) {
    const int n = r.n, nn = n + 1;
    const double inv_m = r.inv_mass ? r.inv_mass[i] : 1.0 / r.mass[i];
    for (int a = 0; a < 3; ++a) {
        double f = 0.0;
        if (i < n) f += s.nlab[a * n + i];
        if (i > 0) f -= s.nlab[a * n + i - 1];
        r.v[a * nn + i] += dt * (f + r.f_ext[a * nn + i]) * inv_m;
        if (decay != 1.0) r.v[a * nn + i] *= decay;  // (x * 1 is x: no multiply without damping)
    }
    if (r.clamped && i == 0) clamp_node0(r);
}

SG_ROD_FN void element_update(View& r, const Scratch& s, int e, double dt, double decay) {
    const int n = r.n, nv = n - 1;
    double c[3];
    for (int a = 0; a < 3; ++a) {
        double acc = 0.0;
        if (e < nv) acc += s.bend_c[a * nv + e];
        if (e > 0) acc -= s.bend_c[a * nv + e - 1];
        if (e < nv) acc += 0.5 * s.twist_c[a * nv + e];
        if (e > 0) acc += 0.5 * s.twist_c[a * nv + e - 1];
        acc += s.shear_c[a * n + e];
        acc += s.transport[a * n + e];
        acc += s.dil_c[a * n + e];
        c[a] = acc + r.c_ext[a * n + e];
    }
    double alpha[3];
    matvec(r.inv_inertia, n, e, c, alpha);
    for (int a = 0; a < 3; ++a) {
        r.w[a * n + e] += dt * s.e[e] * alpha[a];
        if (decay != 1.0) r.w[a * n + e] *= decay;
    }
    if (r.clamped && e == 0) clamp_element0(r);
}

// ------------------------------------------- the element-centric forcing grid of a batch
// cosserat_rod_forcing_grids.py:82-130 for every rod at once, in the marker layout of one
// VirtualBoundaryForcing over the whole batch: (dim, n_rods * n), marker r * n + e.

// Marker (r, e): position (x_e + x_{e+1}) / 2 and the mass-weighted velocity of its two nodes.
// Separately rounded product and sum: device code would otherwise contract a * b + c into one
// fused multiply-add, which rounds once where numpy rounds twice.
SG_ROD_FN double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
SG_ROD_FN double add_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}

SG_ROD_FN void element_marker_at(const View& r, int e, int dim, double* pos, double* vel) {
    const int n = r.n, nn = n + 1;
    const double m0 = r.mass[e], m1 = r.mass[e + 1];
    for (int d = 0; d < dim; ++d) {
        pos[d] = (r.x[d * nn + e + 1] + r.x[d * nn + e]) / 2.0;
        // products rounded before the sum, as numpy does (no fused multiply-add on the device)
        vel[d] = add_rn(mul_rn(m1, r.v[d * nn + e + 1]), mul_rn(m0, r.v[d * nn + e])) / (m1 + m0);
    }
}

SG_ROD_FN void element_marker(const View& r, int rod, int e, int dim, int64_t n_markers, double* pos,
                              double* vel) {
    const int64_t m = (int64_t)rod * r.n + e;
    double p[3], u[3];
    element_marker_at(r, e, dim, p, u);
    for (int d = 0; d < dim; ++d) {
        pos[d * n_markers + m] = p[d];
        vel[d * n_markers + m] = u[d];
    }
}

// Node i of rod `rod`: the reaction -F/2 of each neighbouring element's marker (the element
// before first), into external_forces (components past dim are 0), external_torques 0.
template <typename F>
SG_ROD_FN void element_reaction(View& r, int rod, int i, int dim, int64_t n_markers, const F* forcing,
                                double* f_ext, double* c_ext) {
    const int n = r.n, nn = n + 1;
    for (int d = 0; d < 3; ++d) {
        double f = 0.0;
        if (d < dim) {
            if (i > 0) f -= 0.5 * (double)forcing[d * n_markers + (int64_t)rod * n + i - 1];
            if (i < n) f -= 0.5 * (double)forcing[d * n_markers + (int64_t)rod * n + i];
        }
        f_ext[d * nn + i] = f;
        if (i < n) c_ext[d * n + i] = 0.0;
    }
}

}  // namespace rod
}  // namespace sg
