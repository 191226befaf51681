// Per-element and per-contact FP64 math of the GB300 solver.
//
// Everything here is __host__ __device__ so the same source runs in the
// sm_103a kernels and in host-side unit tests.  It evaluates the Cosserat rod
// strains of the reference (src/cuda_backend.cu:234-245), their energy, the
// gradient and the Gauss-Newton Hessian blocks (src/cuda_backend.cu:899-919)
// with closed-form derivatives of the SO(3) exponential (left Jacobian)
// and of the regularised Cayley map instead of the reference's Dual<12>
// forward-mode AD, plus the log-barrier contact term
// (src/cuda_backend.cu:255-265, 920-938) and the device segment-triangle
// distance (src/cuda_backend.cu:200-223).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define KHS_HD __host__ __device__ __forceinline__
#else
#define KHS_HD inline
#endif

namespace khs {
namespace dm {

constexpr double kPi = 3.1415926535897932384626433832795;

struct V {
    double x, y, z;
};

KHS_HD V v(double x, double y, double z) { V r; r.x = x; r.y = y; r.z = z; return r; }
KHS_HD V operator+(V a, V b) { return v(a.x + b.x, a.y + b.y, a.z + b.z); }
KHS_HD V operator-(V a, V b) { return v(a.x - b.x, a.y - b.y, a.z - b.z); }
KHS_HD V operator*(V a, double s) { return v(a.x * s, a.y * s, a.z * s); }
KHS_HD double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KHS_HD V cross(V a, V b) { return v(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
KHS_HD double norm(V a) { return sqrt(dot(a, a)); }
KHS_HD V vmin(V a, V b) { return v(fmin(a.x, b.x), fmin(a.y, b.y), fmin(a.z, b.z)); }
KHS_HD V vmax(V a, V b) { return v(fmax(a.x, b.x), fmax(a.y, b.y), fmax(a.z, b.z)); }
KHS_HD double at(V a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// 3x3 row-major.
struct M {
    double m[9];
};

KHS_HD M mmul(const M &a, const M &b)
{
    M r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
// a^T b
KHS_HD M mtmul(const M &a, const M &b)
{
    M r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[i] * b.m[j] + a.m[3 + i] * b.m[3 + j] + a.m[6 + i] * b.m[6 + j];
    return r;
}
// a^T x
KHS_HD V mtvec(const M &a, V x)
{
    return v(a.m[0] * x.x + a.m[3] * x.y + a.m[6] * x.z, a.m[1] * x.x + a.m[4] * x.y + a.m[7] * x.z,
             a.m[2] * x.x + a.m[5] * x.y + a.m[8] * x.z);
}
KHS_HD V mvec(const M &a, V x)
{
    return v(a.m[0] * x.x + a.m[1] * x.y + a.m[2] * x.z, a.m[3] * x.x + a.m[4] * x.y + a.m[5] * x.z,
             a.m[6] * x.x + a.m[7] * x.y + a.m[8] * x.z);
}

// Rotation R = exp([u]x) Ref with the reference's Rodrigues coefficients and
// small-angle Taylor branch below theta^2 = 1e-10 (cuda_backend.cu:130-136).
// Also returns the left Jacobian Jl(u), defined by
// exp(u + du) = exp([Jl du]x) exp(u) + O(du^2), as I + p W + r W^2 with
// p = 2 sin^2(t/2) / t^2 (cancellation-free form of (1 - cos t) / t^2) and
// r = (t - sin t) / t^3, both from their Taylor series below t^2 = 1e-4.
KHS_HD void rotation_and_jacobian(V u, const double *ref, M &R, M *Jl)
{
    const double t2 = dot(u, u);
    double a, b;
    double s;
    if (t2 < 1.0e-10) {
        a = 1.0 - t2 / 6.0 + t2 * t2 / 120.0;
        b = 0.5 - t2 / 24.0 + t2 * t2 / 720.0;
        s = 0.0;
    } else {
        // Half-angle form: one sincos, and 1 - cos t = 2 sin^2(t/2) without
        // cancellation (it is also the left Jacobian's coefficient p).
        const double t = sqrt(t2), it = 1.0 / t;
        double sh, ch;
        sincos(0.5 * t, &sh, &ch);
        s = 2.0 * sh * ch;
        a = s * it;
        b = 2.0 * sh * sh * (it * it);
    }
    // E = I + a W + b W^2 with W = [u]x.
    const double wx = u.x, wy = u.y, wz = u.z;
    const double w2[9] = {-(wy * wy + wz * wz), wx * wy, wx * wz,
                          wx * wy, -(wx * wx + wz * wz), wy * wz,
                          wx * wz, wy * wz, -(wx * wx + wy * wy)};
    M E;
    E.m[0] = 1.0 + b * w2[0]; E.m[1] = -a * wz + b * w2[1]; E.m[2] = a * wy + b * w2[2];
    E.m[3] = a * wz + b * w2[3]; E.m[4] = 1.0 + b * w2[4]; E.m[5] = -a * wx + b * w2[5];
    E.m[6] = -a * wy + b * w2[6]; E.m[7] = a * wx + b * w2[7]; E.m[8] = 1.0 + b * w2[8];
    M Rf;
#pragma unroll
    for (int k = 0; k < 9; ++k) Rf.m[k] = ref[k];
    R = mmul(E, Rf);
    if (Jl) {
        double p, r;  // Jl = I + p W + r W^2
        if (t2 < 1.0e-4) {
            p = 0.5 - t2 / 24.0 + t2 * t2 / 720.0 - t2 * t2 * t2 / 40320.0;
            r = 1.0 / 6.0 - t2 / 120.0 + t2 * t2 / 5040.0 - t2 * t2 * t2 / 362880.0;
        } else {
            const double t = sqrt(t2), it = 1.0 / t;
            p = b;
            r = (t - s) * (it * it * it);
        }
        M &J = *Jl;
        J.m[0] = 1.0 + r * w2[0]; J.m[1] = -p * wz + r * w2[1]; J.m[2] = p * wy + r * w2[2];
        J.m[3] = p * wz + r * w2[3]; J.m[4] = 1.0 + r * w2[4]; J.m[5] = -p * wx + r * w2[5];
        J.m[6] = -p * wy + r * w2[6]; J.m[7] = p * wx + r * w2[7]; J.m[8] = 1.0 + r * w2[8];
    }
}

// Material weights of the six strains (cuda_backend.cu:905-907):
// shear, shear, stretch, bend, bend, twist.
struct Weights {
    double w[6];
};

KHS_HD Weights strain_weights(double radius, double young, double poisson, double shear_correction)
{
    const double area = kPi * radius * radius;
    const double inertia = kPi * radius * radius * radius * radius / 4.0;
    const double G = young / (2.0 * (1.0 + poisson));
    Weights r;
    r.w[0] = shear_correction * G * area;
    r.w[1] = r.w[0];
    r.w[2] = young * area;
    r.w[3] = young * inertia;
    r.w[4] = r.w[3];
    r.w[5] = 2.0 * G * inertia;
    return r;
}

// Strain of one element and, optionally, its Jacobian.
//   gamma = 0.5 (Ri^T + Rj^T) t - gamma0,    t = (xj - xi) / L0
//   kappa = cay(Ri^T Rj) / L0 - kappa0
// Jacobian (per 3x3 block; [.]x = cross-product matrix):
//   d gamma / d xj = -d gamma / d xi = A = 0.5 (Ri^T + Rj^T) / L0
//   d gamma / d ui = 0.5 Ri^T [t]x Jl(ui),  d gamma / d uj = 0.5 Rj^T [t]x Jl(uj)
//   d kappa / d uj = -d kappa / d ui|_(Jl(ui) -> Jl(uj)) = K Ri^T Jl(uj) / L0
//   with K = ((tr Q) I - Q) / s + 2 c c^T / s^2, Q = Ri^T Rj, c = axial(Q),
//   s = 1 + (tr Q - 1) / 2 + 1e-12 (differential of the regularised Cayley
//   map along dQ = [w]x Q).
struct ElementJacobian {
    M A, Sgi, Sgj, Kki, Kkj;
};

KHS_HD void element_strain(const M &Ri, const M &Rj, V xi, V xj, double L0, V gamma0, V kappa0, double eps[6],
                           ElementJacobian *J, const M *Jli, const M *Jlj)
{
    const double invL = 1.0 / L0;
    const V t = (xj - xi) * invL;
    M S;  // Ri^T + Rj^T
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) S.m[3 * r + c] = Ri.m[3 * c + r] + Rj.m[3 * c + r];
    const V shear = mvec(S, t) * 0.5;
    const M Q = mtmul(Ri, Rj);
    const V ax = v((Q.m[7] - Q.m[5]) * 0.5, (Q.m[2] - Q.m[6]) * 0.5, (Q.m[3] - Q.m[1]) * 0.5);
    const double trQ = Q.m[0] + Q.m[4] + Q.m[8];
    const double s = 1.0 + (trQ - 1.0) * 0.5 + 1.0e-12;
    const double f = 2.0 / s;
    eps[0] = shear.x - gamma0.x;
    eps[1] = shear.y - gamma0.y;
    eps[2] = shear.z - gamma0.z;
    eps[3] = ax.x * f * invL - kappa0.x;
    eps[4] = ax.y * f * invL - kappa0.y;
    eps[5] = ax.z * f * invL - kappa0.z;
    if (!J) return;
    // A = 0.5 (Ri + Rj)^T / L0
    const double hl = 0.5 * invL;
#pragma unroll
    for (int k = 0; k < 9; ++k) J->A.m[k] = S.m[k] * hl;
    // [t]x Jl: column k = t x Jl_col(k)
    M TJi, TJj;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const V ci = cross(t, v(Jli->m[k], Jli->m[3 + k], Jli->m[6 + k]));
        const V cj = cross(t, v(Jlj->m[k], Jlj->m[3 + k], Jlj->m[6 + k]));
        TJi.m[k] = ci.x; TJi.m[3 + k] = ci.y; TJi.m[6 + k] = ci.z;
        TJj.m[k] = cj.x; TJj.m[3 + k] = cj.y; TJj.m[6 + k] = cj.z;
    }
    J->Sgi = mtmul(Ri, TJi);
    J->Sgj = mtmul(Rj, TJj);
#pragma unroll
    for (int k = 0; k < 9; ++k) { J->Sgi.m[k] *= 0.5; J->Sgj.m[k] *= 0.5; }
    // K
    M K;
    const double is = 1.0 / s, is2 = 2.0 * is * is;
    const double axv[3] = {ax.x, ax.y, ax.z};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) K.m[3 * r + c] = ((r == c ? trQ : 0.0) - Q.m[3 * r + c]) * is + is2 * axv[r] * axv[c];
    const M RJi = mtmul(Ri, *Jli), RJj = mtmul(Ri, *Jlj);
    J->Kki = mmul(K, RJi);
    J->Kkj = mmul(K, RJj);
#pragma unroll
    for (int k = 0; k < 9; ++k) { J->Kki.m[k] *= -invL; J->Kkj.m[k] *= invL; }
}

// Elastic energy 0.5 L0 sum w eps^2.
KHS_HD double element_energy(const double eps[6], const Weights &w, double L0)
{
    double e = 0.0;
#pragma unroll
    for (int s = 0; s < 6; ++s) e += (0.5 * L0 * w.w[s]) * eps[s] * eps[s];
    return e;
}

// Gradient of the element energy: gi, gj (6 each; translation then
// rotation) = L0 J^T diag(w) eps.
KHS_HD void element_gradient(const ElementJacobian &J, const double eps[6], const Weights &w, double L0, double gi[6],
                             double gj[6])
{
    double se[3], ke[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { se[k] = L0 * w.w[k] * eps[k]; ke[k] = L0 * w.w[3 + k] * eps[3 + k]; }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double ax = J.A.m[c] * se[0] + J.A.m[3 + c] * se[1] + J.A.m[6 + c] * se[2];
        gi[c] = -ax;
        gj[c] = ax;
        gi[3 + c] = J.Sgi.m[c] * se[0] + J.Sgi.m[3 + c] * se[1] + J.Sgi.m[6 + c] * se[2] +
                    J.Kki.m[c] * ke[0] + J.Kki.m[3 + c] * ke[1] + J.Kki.m[6 + c] * ke[2];
        gj[3 + c] = J.Sgj.m[c] * se[0] + J.Sgj.m[3 + c] * se[1] + J.Sgj.m[6 + c] * se[2] +
                    J.Kkj.m[c] * ke[0] + J.Kkj.m[3 + c] * ke[1] + J.Kkj.m[6 + c] * ke[2];
    }
}

// X^T diag(d) Y for 3x3 X, Y.
KHS_HD void xtdy(const M &X, const double d[3], const M &Y, double *out, int ld, bool accumulate, double sign)
{
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double h = X.m[r] * d[0] * Y.m[c] + X.m[3 + r] * d[1] * Y.m[3 + c] + X.m[6 + r] * d[2] * Y.m[6 + c];
            if (accumulate) out[ld * r + c] += sign * h;
            else out[ld * r + c] = sign * h;
        }
}

// Gauss-Newton Hessian blocks L0 J^T diag(w) J of one element, as 6x6
// row-major blocks: Hii, Hjj (diagonal blocks of the two nodes) and Hij
// (rows of node i, columns of node j).  With the strain Jacobian's
// structure (shear/stretch rows -A, Sgi, A, Sgj; curvature rows 0, Kki, 0,
// Kkj) the blocks reduce to six 3x3 products:
//   P = A^T Wg A, Xi = A^T Wg Sgi, Xj = A^T Wg Sgj,
//   Rii = Sgi^T Wg Sgi + Kki^T Wk Kki, Rjj likewise, Rij = Sgi^T Wg Sgj + Kki^T Wk Kkj,
//   Hii = [P, -Xi; -Xi^T, Rii], Hjj = [P, Xj; Xj^T, Rjj], Hij = [-P, -Xj; Xi^T, Rij],
// with the symmetric ones (P, Rii, Rjj) evaluated on one triangle and mirrored.
KHS_HD double dot3w(const M &X, int r, const M &WY, int c)
{
    return X.m[r] * WY.m[c] + X.m[3 + r] * WY.m[3 + c] + X.m[6 + r] * WY.m[6 + c];
}

KHS_HD void element_hessian(const ElementJacobian &J, const Weights &w, double L0, double *Hii, double *Hjj, double *Hij)
{
    M WA, WSi, WSj, WKi, WKj;  // rows scaled by L0 w
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double g = L0 * w.w[k], kk = L0 * w.w[3 + k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            WA.m[3 * k + c] = g * J.A.m[3 * k + c];
            WSi.m[3 * k + c] = g * J.Sgi.m[3 * k + c];
            WSj.m[3 * k + c] = g * J.Sgj.m[3 * k + c];
            WKi.m[3 * k + c] = kk * J.Kki.m[3 * k + c];
            WKj.m[3 * k + c] = kk * J.Kkj.m[3 * k + c];
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double xi = dot3w(J.A, r, WSi, c), xj = dot3w(J.A, r, WSj, c);
            Hii[6 * r + 3 + c] = -xi;
            Hii[6 * (3 + c) + r] = -xi;
            Hjj[6 * r + 3 + c] = xj;
            Hjj[6 * (3 + c) + r] = xj;
            Hij[6 * r + 3 + c] = -xj;
            Hij[6 * (3 + c) + r] = xi;
            Hij[6 * (3 + r) + 3 + c] = dot3w(J.Sgi, r, WSj, c) + dot3w(J.Kki, r, WKj, c);
            if (c < r) continue;
            const double p = dot3w(J.A, r, WA, c);
            const double rii = dot3w(J.Sgi, r, WSi, c) + dot3w(J.Kki, r, WKi, c);
            const double rjj = dot3w(J.Sgj, r, WSj, c) + dot3w(J.Kkj, r, WKj, c);
            Hii[6 * r + c] = p; Hii[6 * c + r] = p;
            Hjj[6 * r + c] = p; Hjj[6 * c + r] = p;
            Hij[6 * r + c] = -p; Hij[6 * c + r] = -p;
            Hii[6 * (3 + r) + 3 + c] = rii; Hii[6 * (3 + c) + 3 + r] = rii;
            Hjj[6 * (3 + r) + 3 + c] = rjj; Hjj[6 * (3 + c) + 3 + r] = rjj;
        }
    }
}

// ---- geometry (device flavour, cuda_backend.cu:200-223) ----------------
//
// The proximity tests decide integer outputs (candidate sets, closest
// triangle, active flags), so they are evaluated without FMA contraction:
// every product and sum is rounded on its own (__dmul_rn / __dadd_rn on the
// device, plain operations in host code built with -ffp-contract=off).
// Given the same inputs the device then produces the same bits as a
// correctly rounded host evaluation, including exact-distance ties.

#if defined(__CUDA_ARCH__)
KHS_HD double xm(double a, double b) { return __dmul_rn(a, b); }
KHS_HD double xa(double a, double b) { return __dadd_rn(a, b); }
KHS_HD double xs(double a, double b) { return __dsub_rn(a, b); }
#else
KHS_HD double xm(double a, double b) { return a * b; }
KHS_HD double xa(double a, double b) { return a + b; }
KHS_HD double xs(double a, double b) { return a - b; }
#endif
KHS_HD V gadd(V a, V b) { return v(xa(a.x, b.x), xa(a.y, b.y), xa(a.z, b.z)); }
KHS_HD V gsub(V a, V b) { return v(xs(a.x, b.x), xs(a.y, b.y), xs(a.z, b.z)); }
KHS_HD V gmul(V a, double s) { return v(xm(a.x, s), xm(a.y, s), xm(a.z, s)); }
KHS_HD double gdot(V a, V b) { return xa(xa(xm(a.x, b.x), xm(a.y, b.y)), xm(a.z, b.z)); }
KHS_HD double gnorm(V a) { return sqrt(gdot(a, a)); }

struct ClosestPair {
    double distance, t;
    V bary;
};

KHS_HD V closest_point_triangle(V p, V a, V b, V c, V &bary)
{
    const V ab = gsub(b, a), ac = gsub(c, a), ap = gsub(p, a);
    const double d1 = gdot(ab, ap), d2 = gdot(ac, ap);
    if (d1 <= 0 && d2 <= 0) { bary = v(1, 0, 0); return a; }
    const V bp = gsub(p, b);
    const double d3 = gdot(ab, bp), d4 = gdot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { bary = v(0, 1, 0); return b; }
    const double vc = xs(xm(d1, d4), xm(d3, d2));
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        const double w = d1 / xs(d1, d3);
        bary = v(xs(1.0, w), w, 0);
        return gadd(a, gmul(ab, w));
    }
    const V cp = gsub(p, c);
    const double d5 = gdot(ab, cp), d6 = gdot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { bary = v(0, 0, 1); return c; }
    const double vb = xs(xm(d5, d2), xm(d1, d6));
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        const double w = d2 / xs(d2, d6);
        bary = v(xs(1.0, w), 0, w);
        return gadd(a, gmul(ac, w));
    }
    const double va = xs(xm(d3, d6), xm(d5, d4));
    if (va <= 0 && xs(d4, d3) >= 0 && xs(d5, d6) >= 0) {
        const double w = xs(d4, d3) / xa(xs(d4, d3), xs(d5, d6));
        bary = v(0, xs(1.0, w), w);
        return gadd(b, gmul(gsub(c, b), w));
    }
    const double inv = 1.0 / xa(xa(va, vb), vc), vv = xm(vb, inv), ww = xm(vc, inv);
    bary = v(xs(xs(1.0, vv), ww), vv, ww);
    return gadd(gadd(a, gmul(ab, vv)), gmul(ac, ww));
}

KHS_HD void segment_segment_params(V p1, V q1, V p2, V q2, double &s, double &t)
{
    const V d1 = gsub(q1, p1), d2 = gsub(q2, p2), r = gsub(p1, p2);
    const double a = gdot(d1, d1), e = gdot(d2, d2), f = gdot(d2, r);
    s = 0.0; t = 0.0;
    if (a <= 1e-14 && e <= 1e-14) return;
    if (a <= 1e-14) { t = fmin(1.0, fmax(0.0, f / e)); return; }
    const double c = gdot(d1, r);
    if (e <= 1e-14) { s = fmin(1.0, fmax(0.0, -c / a)); return; }
    const double b = gdot(d1, d2), den = xs(xm(a, e), xm(b, b));
    if (den != 0) s = fmin(1.0, fmax(0.0, xs(xm(b, f), xm(c, e)) / den));
    t = xa(xm(b, s), f) / e;
    if (t < 0) { t = 0; s = fmin(1.0, fmax(0.0, -c / a)); }
    else if (t > 1) { t = 1; s = fmin(1.0, fmax(0.0, xs(b, c) / a)); }
}

// Closest pair between segment p0-p1 and triangle abc: end points against
// the face, then the segment against the three edges, keeping the first
// strictly smaller distance.  No interior-crossing test (device semantics of
// the reference).
KHS_HD ClosestPair closest_segment_triangle(V p0, V p1, V a, V b, V c)
{
    ClosestPair out;
    out.distance = 1.0e300; out.t = 0.0; out.bary = v(1, 0, 0);
    V bary;
    V cp = closest_point_triangle(p0, a, b, c, bary);
    double d = gnorm(gsub(p0, cp));
    if (d < out.distance) { out.distance = d; out.t = 0.0; out.bary = bary; }
    cp = closest_point_triangle(p1, a, b, c, bary);
    d = gnorm(gsub(p1, cp));
    if (d < out.distance) { out.distance = d; out.t = 1.0; out.bary = bary; }
    const V d1 = gsub(p1, p0);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const V p2 = e == 0 ? a : (e == 1 ? b : c);
        const V q2 = e == 0 ? b : (e == 1 ? c : a);
        double s, t;
        segment_segment_params(p0, p1, p2, q2, s, t);
        const double dd = gnorm(gsub(gadd(p0, gmul(d1, s)), gadd(p2, gmul(gsub(q2, p2), t))));
        if (dd < out.distance) {
            out.distance = dd;
            out.t = s;
            if (e == 0) out.bary = v(xs(1.0, t), t, 0);
            else if (e == 1) out.bary = v(0, xs(1.0, t), t);
            else out.bary = v(t, 0, xs(1.0, t));
        }
    }
    return out;
}

// ---- FP32 filters for the mixed form -----------------------------------
//
// Single-precision segment-triangle distance on coordinates taken relative
// to a local origin (the segment start, subtracted in FP64).  Used only to
// discard candidates that provably cannot be the closest one, with a
// relative margin far above the FP32 rounding of these few operations; the
// decision among the survivors is taken in FP64 with the exact code above.
struct F3 {
    float x, y, z;
};
KHS_HD F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
KHS_HD F3 fsub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
KHS_HD F3 fadd(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
KHS_HD F3 fmulv(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
KHS_HD float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KHS_HD F3 to_local(V p, V origin) { return f3(float(p.x - origin.x), float(p.y - origin.y), float(p.z - origin.z)); }

KHS_HD F3 closest_point_triangle_f(F3 p, F3 a, F3 b, F3 c)
{
    const F3 ab = fsub(b, a), ac = fsub(c, a), ap = fsub(p, a);
    const float d1 = fdot(ab, ap), d2 = fdot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) return a;
    const F3 bp = fsub(p, b);
    const float d3 = fdot(ab, bp), d4 = fdot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) return b;
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return fadd(a, fmulv(ab, d1 / (d1 - d3)));
    const F3 cp = fsub(p, c);
    const float d5 = fdot(ab, cp), d6 = fdot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) return c;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return fadd(a, fmulv(ac, d2 / (d2 - d6)));
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
        return fadd(b, fmulv(fsub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    const float inv = 1.f / (va + vb + vc);
    return fadd(fadd(a, fmulv(ab, vb * inv)), fmulv(ac, vc * inv));
}

KHS_HD float segment_segment_distance_f(F3 p1, F3 q1, F3 p2, F3 q2)
{
    const F3 d1 = fsub(q1, p1), d2 = fsub(q2, p2), r = fsub(p1, p2);
    const float a = fdot(d1, d1), e = fdot(d2, d2), f = fdot(d2, r);
    float s = 0.f, t = 0.f;
    if (!(a <= 1e-20f && e <= 1e-20f)) {
        if (a <= 1e-20f) t = fminf(1.f, fmaxf(0.f, f / e));
        else {
            const float c = fdot(d1, r);
            if (e <= 1e-20f) s = fminf(1.f, fmaxf(0.f, -c / a));
            else {
                const float b = fdot(d1, d2), den = a * e - b * b;
                if (den > 0.f) s = fminf(1.f, fmaxf(0.f, (b * f - c * e) / den));
                t = (b * s + f) / e;
                if (t < 0.f) { t = 0.f; s = fminf(1.f, fmaxf(0.f, -c / a)); }
                else if (t > 1.f) { t = 1.f; s = fminf(1.f, fmaxf(0.f, (b - c) / a)); }
            }
        }
    }
    const F3 w = fsub(fadd(p1, fmulv(d1, s)), fadd(p2, fmulv(d2, t)));
    return sqrtf(fdot(w, w));
}

// FP32 segment-triangle distance (local coordinates) and the absolute
// margin that bounds its deviation from the FP64 distance.
KHS_HD float segment_triangle_distance_f(F3 p0, F3 p1, F3 a, F3 b, F3 c, float &margin)
{
    F3 w = fsub(p0, closest_point_triangle_f(p0, a, b, c));
    float dist = sqrtf(fdot(w, w));
    w = fsub(p1, closest_point_triangle_f(p1, a, b, c));
    dist = fminf(dist, sqrtf(fdot(w, w)));
    dist = fminf(dist, segment_segment_distance_f(p0, p1, a, b));
    dist = fminf(dist, segment_segment_distance_f(p0, p1, b, c));
    dist = fminf(dist, segment_segment_distance_f(p0, p1, c, a));
    const float scale = fmaxf(fmaxf(fabsf(p1.x), fmaxf(fabsf(p1.y), fabsf(p1.z))),
                              fmaxf(fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z))),
                                    fmaxf(fmaxf(fabsf(b.x), fmaxf(fabsf(b.y), fabsf(b.z))),
                                          fmaxf(fabsf(c.x), fmaxf(fabsf(c.y), fabsf(c.z))))));
    margin = 1.0e-4f * (scale + dist) + 1.0e-9f;
    return dist;
}

KHS_HD bool boxes_overlap(V al, V au, V bl, V bu, double p)
{
    return al.x <= bu.x + p && bl.x <= au.x + p && al.y <= bu.y + p && bl.y <= au.y + p && al.z <= bu.z + p &&
           bl.z <= au.z + p;
}

// Log barrier b(g) = -kc (dh - g)^2 ln(g / dh) of the contact gap and its
// gradient with respect to the two segment end points at fixed (t, bary)
// (cuda_backend.cu:255-265: the distance is regularised by 1e-30 inside the
// square root).  Returns the energy; g0, g1 get the gradients.
KHS_HD double barrier_energy_gradient(V x0, V x1, double t, V body_point, double radius_offset, double dh, double kc,
                                      double g0[3], double g1[3])
{
    const V p = x0 * (1.0 - t) + x1 * t;
    const V diff = p - body_point;
    const double dist = sqrt(dot(diff, diff) + 1e-30);
    const double gap = dist - radius_offset;
    if (gap >= dh) {
        g0[0] = g0[1] = g0[2] = g1[0] = g1[1] = g1[2] = 0.0;
        return 0.0;
    }
    const double aa = dh - gap, lg = log(gap / dh);
    const double energy = -kc * aa * aa * lg;
    const double db = kc * (2.0 * aa * lg - aa * aa / gap);  // d energy / d gap
    const double s = db / dist;
    g0[0] = s * diff.x * (1.0 - t); g0[1] = s * diff.y * (1.0 - t); g0[2] = s * diff.z * (1.0 - t);
    g1[0] = s * diff.x * t; g1[1] = s * diff.y * t; g1[2] = s * diff.z * t;
    return energy;
}

// ---- root targets (src/solver.cpp:416-447, src/math.hpp:26-58) -----------
//
// Frames of the driven nodes: a frame per node whose third column is the
// unit tangent, the first column carried from node to node by the minimal
// rotation between consecutive tangents, and the rotation vector of
// frame * reference^T (src/solver.cpp:19-26 goes through Eigen's AngleAxis;
// restated with Shepperd's method, J. Guidance and Control 1(3), 1978).
// Written with the non-contracting operations above and correctly rounded
// division and square root, so the device rounds like host code built with
// -ffp-contract=off: positions, tangents and frames agree bit for bit and the
// rotation vectors differ only through atan2.

#if defined(__CUDA_ARCH__)
KHS_HD bool gfinite(double x) { return isfinite(x); }
#else
KHS_HD bool gfinite(double x) { return std::isfinite(x); }
#endif

KHS_HD V gcross(V a, V b)
{
    return v(xs(xm(a.y, b.z), xm(a.z, b.y)), xs(xm(a.z, b.x), xm(a.x, b.z)), xs(xm(a.x, b.y), xm(a.y, b.x)));
}

// Unit vector with Eigen's normalized() semantics: a zero (or NaN) squared
// norm leaves the vector unchanged; each component is divided.
KHS_HD V gunit(V a)
{
    const double n2 = gdot(a, a);
    if (!(n2 > 0.0)) return a;
    const double n = sqrt(n2);
    return v(a.x / n, a.y / n, a.z / n);
}

// (1 - t) a + t b, each product and the sum rounded on its own.
KHS_HD V glerp(V a, V b, double t)
{
    const double u = xs(1.0, t);
    return v(xa(xm(a.x, u), xm(b.x, t)), xa(xm(a.y, u), xm(b.y, t)), xa(xm(a.z, u), xm(b.z, t)));
}

// Frame (row-major, columns d1 d2 d3) from d3 = the normalised tangent and
// d1 the hint made orthogonal to it (math.hpp:26-43).
KHS_HD M frame_from_d3(V d3, V hint)
{
    V d1 = gsub(hint, gmul(d3, gdot(hint, d3)));
    if (gdot(d1, d1) < 1.0e-16) {
        const V axis = fabs(d3.x) < 0.8 ? v(1.0, 0.0, 0.0) : v(0.0, 1.0, 0.0);
        d1 = gsub(axis, gmul(d3, gdot(axis, d3)));
    }
    d1 = gunit(d1);
    const V d2 = gunit(gcross(d3, d1));
    d1 = gunit(gcross(d2, d3));
    M r;
    r.m[0] = d1.x; r.m[1] = d2.x; r.m[2] = d3.x;
    r.m[3] = d1.y; r.m[4] = d2.y; r.m[5] = d3.y;
    r.m[6] = d1.z; r.m[7] = d2.z; r.m[8] = d3.z;
    return r;
}

KHS_HD M frame_from_tangent(V tangent, V hint) { return frame_from_d3(gunit(tangent), hint); }

// A unit vector orthogonal to s, chosen like Eigen's unitOrthogonal.
KHS_HD V unit_orthogonal(V s)
{
    const double eps = 1e-12;
    if (!(fabs(s.x) <= xm(fabs(s.z), eps)) || !(fabs(s.y) <= xm(fabs(s.z), eps))) {
        const double inv = 1.0 / sqrt(xa(xm(s.x, s.x), xm(s.y, s.y)));
        return v(xm(-s.y, inv), xm(s.x, inv), 0.0);
    }
    const double inv = 1.0 / sqrt(xa(xm(s.y, s.y), xm(s.z, s.z)));
    return v(0.0, xm(-s.z, inv), xm(s.y, inv));
}

// The minimal rotation taking `from` to `to` (math.hpp:45-58), split into
// the part that depends on the two tangents only and its application to a
// director: Rodrigues' formula about n = from x to / |from x to| (kind 0),
// the identity for parallel tangents (kind 1), a half turn about an
// orthogonal axis n for opposite ones (kind 2).
struct Transport {
    V n;
    double s, c;
    int kind;
};

KHS_HD Transport transport_between(V from, V to)
{
    const V a = gunit(from), b = gunit(to);
    const V axis = gcross(a, b);
    Transport t;
    t.s = sqrt(gdot(axis, axis));
    const double c = gdot(a, b);
    t.c = c < -1.0 ? -1.0 : (1.0 < c ? 1.0 : c);
    t.kind = 0;
    if (t.s < 1.0e-12) {
        t.kind = t.c > 0.0 ? 1 : 2;
        t.n = t.kind == 2 ? unit_orthogonal(a) : v(0.0, 0.0, 0.0);
    } else {
        t.n = v(axis.x / t.s, axis.y / t.s, axis.z / t.s);
    }
    return t;
}

KHS_HD V transport_apply(const Transport &t, V director)
{
    if (t.kind == 1) return director;
    if (t.kind == 2) return gsub(gmul(gmul(t.n, 2.0), gdot(t.n, director)), director);
    return gadd(gadd(gmul(director, t.c), gmul(gcross(t.n, director), t.s)), gmul(gmul(t.n, gdot(t.n, director)), xs(1.0, t.c)));
}

KHS_HD V parallel_transport(V director, V from, V to) { return transport_apply(transport_between(from, to), director); }

// a * b^T for row-major 3x3 matrices.
KHS_HD M times_transpose(const M &a, const M &b)
{
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = xa(xa(xm(a.m[3 * i], b.m[3 * j]), xm(a.m[3 * i + 1], b.m[3 * j + 1])), xm(a.m[3 * i + 2], b.m[3 * j + 2]));
    return r;
}

// Rotation vector (axis * angle, angle in (-pi, pi]) of a rotation matrix:
// the quaternion from the largest of its four squared components, then
// angle = 2 atan2(|v|, |w|) with the axis carrying the sign of w.
KHS_HD V rotation_vector(const M &r)
{
    double q[4];  // x y z w
    const double tr = xa(xa(r.m[0], r.m[4]), r.m[8]);
    if (tr > 0.0) {
        double s = sqrt(xa(tr, 1.0));
        q[3] = xm(0.5, s);
        s = 0.5 / s;
        q[0] = xm(xs(r.m[7], r.m[5]), s);
        q[1] = xm(xs(r.m[2], r.m[6]), s);
        q[2] = xm(xs(r.m[3], r.m[1]), s);
    } else {
        int i = 0;
        if (r.m[4] > r.m[0]) i = 1;
        if (r.m[8] > r.m[4 * i]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        double s = sqrt(xa(xs(xs(r.m[4 * i], r.m[4 * j]), r.m[4 * k]), 1.0));
        q[i] = xm(0.5, s);
        s = 0.5 / s;
        q[3] = xm(xs(r.m[3 * k + j], r.m[3 * j + k]), s);
        q[j] = xm(xa(r.m[3 * j + i], r.m[3 * i + j]), s);
        q[k] = xm(xa(r.m[3 * k + i], r.m[3 * i + k]), s);
    }
    double n = sqrt(xa(xa(xm(q[0], q[0]), xm(q[1], q[1])), xm(q[2], q[2])));
    if (!(n != 0.0)) return v(0.0, 0.0, 0.0);
    double angle = xm(2.0, atan2(n, fabs(q[3])));
    if (q[3] < 0.0) n = -n;
    const V axis = v(q[0] / n, q[1] / n, q[2] / n);
    if (!gfinite(angle) || !gfinite(axis.x) || !gfinite(axis.y) || !gfinite(axis.z)) return v(0.0, 0.0, 0.0);
    if (angle > kPi) angle = xs(angle, xm(2.0, kPi));
    return gmul(axis, angle);
}

// ---- correctly rounded reciprocal on the integer pipes -----------------
//
// 1/x rounded to nearest, computed without FP64 instructions: on GB300 one
// FP64 warp instruction occupies a sub-partition's pipe for ~64 cycles, and
// the block solve's pivot warp is bound by its FP64 instruction count.
// For x = (-1)^s * M * 2^(E-1075) with M the 53-bit significand,
// 1/x = (-1)^s * (2^105 / M) * 2^(970-E).  T = 2^105 / M lies in
// (2^52, 2^53]:
// * seed: an FP32 reciprocal of the top 24 bits of M, scaled to T0 ~ T
//   (relative error below 2^-21);
// * one residual step of order three: e = (2^105 - T0 M) / 2^105 in 64-bit
//   fixed point, T1 = T0 (1 + e + e^2), error of order e^3 plus truncation
//   (a few units);
// * exact remainder R = 2^105 - T1 M (the low 64 bits suffice: |R| < 2^63)
//   brings T1 to floor(T) with 0 <= R < M; the nearest integer is floor(T)
//   + (2R > M) (no ties: M > 1 is odd or a power of two);
// * reciprocals below the normal range (|x| >= 2^1022) are rounded from
//   floor(T) and R to nearest-even.
// The result equals the IEEE division 1.0 / x for every finite nonzero x
// (checked bit for bit against __drcp_rn on 2^31 values on GB300 and
// against 1.0 / x on the host, tests/native/test_recip.cpp); zero,
// subnormal and non-finite inputs give an unspecified finite bit pattern
// (the block solve fails such pivots before using the result).
#if defined(__CUDA_ARCH__)
KHS_HD uint64_t umulhi64(uint64_t a, uint64_t b) { return __umul64hi(a, b); }
KHS_HD int64_t smulhi64(int64_t a, int64_t b) { return __mul64hi(a, b); }
KHS_HD float recip_seed(float m)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(m));
    return r;
}
KHS_HD uint64_t bits_of(double x) { return uint64_t(__double_as_longlong(x)); }
KHS_HD double double_of(uint64_t b) { return __longlong_as_double((long long)b); }
KHS_HD uint32_t bits_of(float x) { return __float_as_uint(x); }
KHS_HD float float_of(uint32_t b) { return __uint_as_float(b); }
#else
KHS_HD uint64_t umulhi64(uint64_t a, uint64_t b) { return uint64_t((unsigned __int128)a * b >> 64); }
KHS_HD int64_t smulhi64(int64_t a, int64_t b) { return int64_t((__int128)a * b >> 64); }
// Host seed: the correctly rounded float reciprocal (tests may substitute a
// perturbed one through KHS_RECIP_SEED_HOST).
#ifndef KHS_RECIP_SEED_HOST
#define KHS_RECIP_SEED_HOST(m) (1.0f / (m))
#endif
KHS_HD float recip_seed(float m) { return KHS_RECIP_SEED_HOST(m); }
KHS_HD uint64_t bits_of(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }
KHS_HD double double_of(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }
KHS_HD uint32_t bits_of(float x) { uint32_t b; std::memcpy(&b, &x, 4); return b; }
KHS_HD float float_of(uint32_t b) { float x; std::memcpy(&x, &b, 4); return x; }
#endif

KHS_HD double recip_rn(double x)
{
    const uint64_t b = bits_of(x);
    const uint64_t sign = b & 0x8000000000000000ull;
    const int E = int((b >> 52) & 0x7ff);
    const uint64_t M = (b & 0xfffffffffffffull) | (1ull << 52);
    const uint32_t rb = bits_of(recip_seed(float_of((127u << 23) | uint32_t((M >> 29) & 0x7fffff))));
    const int er = int((rb >> 23) & 0xff) - 127;  // the seed lies in (0.5, 1]: -1 or 0
    const uint64_t T0 = uint64_t((rb & 0x7fffff) | 0x800000) << (30 + er);
    const uint64_t Plo = T0 * M, Phi = umulhi64(T0, M);
    const uint64_t Rlo = 0 - Plo;
    const uint64_t Rhi = (1ull << 41) - Phi - uint64_t(Plo != 0);
    const int64_t e = int64_t((Rhi << 23) | (Rlo >> 41));  // (2^105 - T0 M) / 2^41
    const uint64_t ae = e < 0 ? uint64_t(-e) : uint64_t(e);
    const int64_t s = e + int64_t(umulhi64(ae, ae));
    uint64_t T1 = T0 + uint64_t(smulhi64(int64_t(T0), s));
    int64_t R = int64_t(0 - T1 * M);
    for (int k = 0; k < 2; ++k) {
        const bool low = R < 0;
        T1 -= uint64_t(low);
        R += low ? int64_t(M) : 0;
    }
    for (int k = 0; k < 2; ++k) {
        const bool high = R >= int64_t(M);
        T1 += uint64_t(high);
        R -= high ? int64_t(M) : 0;
    }
    int bexp = 2045 - E;
    uint64_t out;
    if (bexp >= 1) {
        uint64_t Q = T1 + uint64_t(2 * uint64_t(R) > M);
        const bool carry = (Q >> 53) != 0;
        Q = carry ? Q >> 1 : Q;
        bexp += int(carry);
        out = sign | (uint64_t(bexp) << 52) | (Q & 0xfffffffffffffull);
    } else {
        const int k = 1 - bexp < 63 ? 1 - bexp : 63;
        const uint64_t mant = T1 >> k;
        const uint64_t dropped = T1 & ((1ull << k) - 1), half = 1ull << (k - 1);
        const bool up = dropped > half || (dropped == half && (R > 0 || (mant & 1)));
        out = sign | (mant + uint64_t(up));
    }
    return double_of(out);
}

}  // namespace dm
}  // namespace khs
