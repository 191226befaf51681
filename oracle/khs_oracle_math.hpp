// ORACLE — test infrastructure only.  Small FP64 vector/matrix and
// forward-mode dual-number library used by the CPU restatement of the
// reference solver (khs_oracle.cpp).  Nothing in the product library links
// or includes this file.
//
// The dual numbers restate the reference's forward-mode AD used for the
// element gradient and Gauss-Newton Jacobian (src/cuda_backend.cu:59-96), so
// the oracle differentiates exactly like the reference does; the product's
// CUDA kernels use closed-form derivatives instead and are checked against
// this.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace khs_oracle {

constexpr double kPi = 3.1415926535897932384626433832795;

struct V3 {
    double x = 0.0, y = 0.0, z = 0.0;
    double &operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
    double operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};

inline V3 v3(double x, double y, double z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double norm2(V3 a) { return dot(a, a); }
inline double norm(V3 a) { return std::sqrt(norm2(a)); }
inline V3 vmin(V3 a, V3 b) { return v3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline bool finite3(V3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

// Two flavours of "divide a vector by a scalar" exist in the reference and
// they round differently: the host (Eigen) code divides each component, the
// device DVec3 operator/ multiplies by the reciprocal (cuda_backend.cu:40).
inline V3 div_each(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 div_recip(V3 a, double s) { return a * (1.0 / s); }

// Eigen-style normalized(): unchanged when the squared norm is zero.
inline V3 normalized(V3 a)
{
    const double z = norm2(a);
    return z > 0.0 ? div_each(a, std::sqrt(z)) : a;
}

// 3x3 row-major: m[3*row + col].
struct M3 {
    double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double &operator()(int r, int c) { return m[3 * r + c]; }
    double operator()(int r, int c) const { return m[3 * r + c]; }
    V3 col(int c) const { return v3(m[c], m[3 + c], m[6 + c]); }
    V3 row(int r) const { return v3(m[3 * r], m[3 * r + 1], m[3 * r + 2]); }
    void set_col(int c, V3 v) { m[c] = v.x; m[3 + c] = v.y; m[6 + c] = v.z; }
};

inline M3 transpose(const M3 &a)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = a(j, i);
    return r;
}
inline M3 matmul(const M3 &a, const M3 &b)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = (a(i, 0) * b(0, j) + a(i, 1) * b(1, j)) + a(i, 2) * b(2, j);
    return r;
}
inline V3 matvec(const M3 &a, V3 v)
{
    return v3((a(0, 0) * v.x + a(0, 1) * v.y) + a(0, 2) * v.z,
              (a(1, 0) * v.x + a(1, 1) * v.y) + a(1, 2) * v.z,
              (a(2, 0) * v.x + a(2, 1) * v.y) + a(2, 2) * v.z);
}

// Rotation-matrix relative rotation vector with the 1e-12 regularised
// Cayley map (math.hpp:14-24; device copy cuda_backend.cu:138-143).
inline V3 cayley_vector(const M3 &q)
{
    const V3 v = v3((q(2, 1) - q(1, 2)) * 0.5, (q(0, 2) - q(2, 0)) * 0.5, (q(1, 0) - q(0, 1)) * 0.5);
    const double c = (((q(0, 0) + q(1, 1)) + q(2, 2)) - 1.0) * 0.5;
    return (2.0 / (1.0 + c + 1.0e-12)) * v;
}

// Eigen's unitOrthogonal for 3-vectors (used only on a 180 degree fold).
inline V3 unit_orthogonal(V3 s)
{
    const double prec = 1e-12;
    const bool x_small = std::fabs(s.x) <= std::fabs(s.z) * prec;
    const bool y_small = std::fabs(s.y) <= std::fabs(s.z) * prec;
    if (!x_small || !y_small) {
        const double inv = 1.0 / std::sqrt(s.x * s.x + s.y * s.y);
        return v3(-s.y * inv, s.x * inv, 0.0);
    }
    const double inv = 1.0 / std::sqrt(s.y * s.y + s.z * s.z);
    return v3(0.0, -s.z * inv, s.y * inv);
}

// One triangle of the ray-parity inside test (solver.cpp:608-632): whether
// the ray p + t (1, 1.2345e-6, 2.3456e-6), t > 1e-12, crosses the triangle
// (Moller-Trumbore with the reference's thresholds).
inline bool ray_crosses_triangle(V3 p, V3 a, V3 b, V3 c)
{
    const V3 dir = v3(1.0, 0.0000012345, 0.0000023456);
    const V3 e1 = b - a, e2 = c - a, h = cross(dir, e2);
    const double det = dot(e1, h);
    if (std::fabs(det) < 1.0e-14) return false;
    const double inv = 1.0 / det;
    const V3 s = p - a;
    const double u = inv * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const V3 q = cross(s, e1);
    const double v = inv * dot(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    return inv * dot(e2, q) > 1.0e-12;
}

// Orthonormal frame whose third column is the tangent (math.hpp:26-43).
inline M3 frame_from_tangent(V3 tangent, V3 hint)
{
    const V3 d3 = normalized(tangent);
    V3 d1 = hint - d3 * dot(hint, d3);
    if (norm2(d1) < 1.0e-16) {
        const V3 axis = std::fabs(d3.x) < 0.8 ? v3(1, 0, 0) : v3(0, 1, 0);
        d1 = axis - d3 * dot(axis, d3);
    }
    d1 = normalized(d1);
    const V3 d2 = normalized(cross(d3, d1));
    d1 = normalized(cross(d2, d3));
    M3 r;
    r.set_col(0, d1);
    r.set_col(1, d2);
    r.set_col(2, d3);
    return r;
}

// Rotates a director from one tangent to the next (math.hpp:45-58).
inline V3 parallel_transport(V3 director, V3 from, V3 to)
{
    const V3 a = normalized(from);
    const V3 b = normalized(to);
    const V3 axis = cross(a, b);
    const double s = norm(axis);
    const double c = std::clamp(dot(a, b), -1.0, 1.0);
    if (s < 1.0e-12) {
        if (c > 0.0) return director;
        const V3 n = unit_orthogonal(a);
        return (2.0 * n) * dot(n, director) - director;
    }
    const V3 n = div_each(axis, s);
    return (director * c + cross(n, director) * s) + (n * dot(n, director)) * (1.0 - c);
}

// Rotation vector of a rotation matrix (solver.cpp:19-26 through Eigen's
// AngleAxis).  Restated with Shepperd's method (S. W. Shepperd, "Quaternion
// from rotation matrix", J. Guidance and Control 1(3), 1978): pick the
// largest of the four quaternion magnitudes to take the square root of, then
// angle = 2 atan2(|v|, |w|) and axis = v / |v| with the sign of w.
inline V3 rotation_vector(const M3 &r)
{
    double q[4];  // x, y, z, w
    const double t = (r(0, 0) + r(1, 1)) + r(2, 2);
    if (t > 0.0) {
        double s = std::sqrt(t + 1.0);
        q[3] = 0.5 * s;
        s = 0.5 / s;
        q[0] = (r(2, 1) - r(1, 2)) * s;
        q[1] = (r(0, 2) - r(2, 0)) * s;
        q[2] = (r(1, 0) - r(0, 1)) * s;
    } else {
        int i = 0;
        if (r(1, 1) > r(0, 0)) i = 1;
        if (r(2, 2) > r(i, i)) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        double s = std::sqrt(r(i, i) - r(j, j) - r(k, k) + 1.0);
        q[i] = 0.5 * s;
        s = 0.5 / s;
        q[3] = (r(k, j) - r(j, k)) * s;
        q[j] = (r(j, i) + r(i, j)) * s;
        q[k] = (r(k, i) + r(i, k)) * s;
    }
    double n = std::sqrt((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]);
    if (!(n != 0.0)) return V3{};
    double angle = 2.0 * std::atan2(n, std::fabs(q[3]));
    if (q[3] < 0.0) n = -n;
    const V3 axis = v3(q[0] / n, q[1] / n, q[2] / n);
    if (!std::isfinite(angle) || !finite3(axis)) return V3{};
    if (angle > kPi) angle -= 2.0 * kPi;
    return axis * angle;
}

// ---------------------------------------------------------------------------
// Forward-mode dual numbers (cuda_backend.cu:59-96).
template<int N> struct Dual {
    double v;
    double d[N];
    Dual(double value = 0.0) : v(value) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
    static Dual var(double value, int index) { Dual r(value); r.d[index] = 1.0; return r; }
};
template<int N> Dual<N> operator+(const Dual<N> &a, const Dual<N> &b)
{ Dual<N> r(a.v + b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template<int N> Dual<N> operator-(const Dual<N> &a, const Dual<N> &b)
{ Dual<N> r(a.v - b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template<int N> Dual<N> operator-(const Dual<N> &a)
{ Dual<N> r(-a.v); for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template<int N> Dual<N> operator*(const Dual<N> &a, const Dual<N> &b)
{ Dual<N> r(a.v * b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template<int N> Dual<N> operator/(const Dual<N> &a, const Dual<N> &b)
{
    const double inv = 1.0 / b.v; Dual<N> r(a.v * inv);
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
template<int N> Dual<N> dsqrt(const Dual<N> &a)
{
    const double s = std::sqrt(a.v); Dual<N> r(s); const double f = 0.5 / std::fmax(s, 1.0e-300);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * f;
    return r;
}
template<int N> Dual<N> dsin(const Dual<N> &a)
{ Dual<N> r(std::sin(a.v)); const double c = std::cos(a.v); for (int i = 0; i < N; ++i) r.d[i] = c * a.d[i]; return r; }
template<int N> Dual<N> dcos(const Dual<N> &a)
{ Dual<N> r(std::cos(a.v)); const double s = -std::sin(a.v); for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i]; return r; }
template<int N> Dual<N> dlog(const Dual<N> &a)
{ Dual<N> r(std::log(a.v)); const double inv = 1.0 / a.v; for (int i = 0; i < N; ++i) r.d[i] = inv * a.d[i]; return r; }

template<int N> struct DV3 { Dual<N> x, y, z; };
template<int N> struct DM3 { Dual<N> m[9]; };

template<int N> DV3<N> dvadd(const DV3<N> &a, const DV3<N> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template<int N> DV3<N> dvsub(const DV3<N> &a, const DV3<N> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template<int N> DV3<N> dvscale(const DV3<N> &a, const Dual<N> &s) { return {a.x * s, a.y * s, a.z * s}; }
template<int N> Dual<N> dvdot(const DV3<N> &a, const DV3<N> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

template<int N> DM3<N> dm_identity() { DM3<N> r; r.m[0] = Dual<N>(1); r.m[4] = Dual<N>(1); r.m[8] = Dual<N>(1); return r; }
template<int N> DM3<N> dm_add(const DM3<N> &a, const DM3<N> &b) { DM3<N> r; for (int i = 0; i < 9; ++i) r.m[i] = a.m[i] + b.m[i]; return r; }
template<int N> DM3<N> dm_scale(const DM3<N> &a, const Dual<N> &s) { DM3<N> r; for (int i = 0; i < 9; ++i) r.m[i] = a.m[i] * s; return r; }
template<int N> DM3<N> dm_mul(const DM3<N> &a, const DM3<N> &b)
{
    DM3<N> r;
    for (int y = 0; y < 3; ++y)
        for (int x = 0; x < 3; ++x)
            for (int k = 0; k < 3; ++k) r.m[3 * y + x] = r.m[3 * y + x] + a.m[3 * y + k] * b.m[3 * k + x];
    return r;
}
template<int N> DM3<N> dm_transpose(const DM3<N> &a)
{ DM3<N> r; for (int y = 0; y < 3; ++y) for (int x = 0; x < 3; ++x) r.m[3 * y + x] = a.m[3 * x + y]; return r; }
template<int N> DV3<N> dm_vec(const DM3<N> &a, const DV3<N> &b)
{
    return {a.m[0] * b.x + a.m[1] * b.y + a.m[2] * b.z,
            a.m[3] * b.x + a.m[4] * b.y + a.m[5] * b.z,
            a.m[6] * b.x + a.m[7] * b.y + a.m[8] * b.z};
}
template<int N> DM3<N> dskew(const DV3<N> &w)
{
    DM3<N> r;
    r.m[1] = -w.z; r.m[2] = w.y; r.m[3] = w.z; r.m[5] = -w.x; r.m[6] = -w.y; r.m[7] = w.x;
    return r;
}

// Rodrigues exponential with the small-angle Taylor branch below
// theta^2 = 1e-10 (cuda_backend.cu:130-136).
template<int N> DM3<N> dexp_so3(const DV3<N> &w)
{
    const Dual<N> t2 = dvdot(w, w);
    Dual<N> a, b;
    if (t2.v < 1.0e-10) {
        a = Dual<N>(1) - t2 / Dual<N>(6) + t2 * t2 / Dual<N>(120);
        b = Dual<N>(0.5) - t2 / Dual<N>(24) + t2 * t2 / Dual<N>(720);
    } else {
        const Dual<N> t = dsqrt(t2);
        a = dsin(t) / t;
        b = (Dual<N>(1) - dcos(t)) / t2;
    }
    const DM3<N> W = dskew(w);
    return dm_add(dm_identity<N>(), dm_add(dm_scale(W, a), dm_scale(dm_mul(W, W), b)));
}

template<int N> DV3<N> dcayley(const DM3<N> &q)
{
    DV3<N> v{(q.m[7] - q.m[5]) * Dual<N>(0.5), (q.m[2] - q.m[6]) * Dual<N>(0.5), (q.m[3] - q.m[1]) * Dual<N>(0.5)};
    const Dual<N> c = (q.m[0] + q.m[4] + q.m[8] - Dual<N>(1)) * Dual<N>(0.5);
    return dvscale(v, Dual<N>(2) / (Dual<N>(1) + c + Dual<N>(1.0e-12)));
}

}  // namespace khs_oracle
