// Checks the product's root-target math (csrc/khs_device_math.cuh, compiled
// for the host) against the oracle's restatement of the reference's root
// frames (src/solver.cpp:416-447, src/math.hpp:26-58): unit tangents,
// frame_from_tangent, parallel_transport and the rotation vector of
// frame * reference^T, walked along random curves exactly as the reference
// walks a strand.  Host code built with -ffp-contract=off must agree bit for
// bit, so every comparison here is exact.  Built and run by
// tests/test_root_targets_math.py.
#include "khs_device_math.cuh"
#include "khs_oracle_math.hpp"

#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

using namespace khs_oracle;
namespace dm = khs::dm;

static dm::V to_dm(V3 a) { return dm::v(a.x, a.y, a.z); }

static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }
static bool same3(dm::V a, V3 b) { return same(a.x, b.x) && same(a.y, b.y) && same(a.z, b.z); }
static bool same9(const dm::M &a, const M3 &b)
{
    for (int k = 0; k < 9; ++k)
        if (!same(a.m[k], b.m[k])) return false;
    return true;
}

// Rodrigues' formula, for test rotations only.
static M3 rotation(V3 axis, double angle)
{
    const double c = std::cos(angle), s = std::sin(angle), t = 1.0 - c;
    M3 r;
    r(0, 0) = c + t * axis.x * axis.x; r(0, 1) = t * axis.x * axis.y - s * axis.z; r(0, 2) = t * axis.x * axis.z + s * axis.y;
    r(1, 0) = t * axis.y * axis.x + s * axis.z; r(1, 1) = c + t * axis.y * axis.y; r(1, 2) = t * axis.y * axis.z - s * axis.x;
    r(2, 0) = t * axis.z * axis.x - s * axis.y; r(2, 1) = t * axis.z * axis.y + s * axis.x; r(2, 2) = c + t * axis.z * axis.z;
    return r;
}

static dm::M to_dm(const M3 &a)
{
    dm::M r;
    for (int k = 0; k < 9; ++k) r.m[k] = a.m[k];
    return r;
}

int main()
{
    std::mt19937_64 g(4242);
    std::normal_distribution<double> n(0.0, 1.0);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long checked = 0, bad = 0;
    for (int curve = 0; curve < 400; ++curve) {
        // A random curve: kinks from gentle to sharp, some straight runs
        // (parallel tangents), and a few exact reversals (a half turn).
        const int count = 2 + int(u(g) * 120);
        const double bend = curve % 4 == 0 ? 1e-9 : (curve % 4 == 1 ? 0.05 : (curve % 4 == 2 ? 0.5 : 2.0));
        std::vector<V3> x(count);
        x[0] = v3(n(g), n(g), n(g));
        V3 dir = normalized(v3(n(g), n(g), n(g)));
        for (int k = 1; k < count; ++k) {
            if (curve % 7 == 3 && k % 9 == 4) dir = dir * -1.0;
            else if (!(curve % 5 == 1 && k % 3 == 0)) dir = normalized(dir + v3(n(g), n(g), n(g)) * bend);
            x[k] = x[k - 1] + dir * (0.002 * (0.5 + u(g)));
        }
        // Reference frames of the nodes (any rotations).
        std::vector<M3> ref(count);
        for (int k = 0; k < count; ++k)
            ref[k] = frame_from_tangent(normalized(v3(n(g), n(g), n(g))), v3(n(g), n(g), n(g)));
        // Binding of the node positions to two source points.
        for (int k = 0; k < count; ++k) {
            const double t = u(g);
            const V3 a = x[k] + v3(n(g), n(g), n(g)) * 1e-3, b = x[k] + v3(n(g), n(g), n(g)) * 1e-3;
            const V3 o = (1.0 - t) * a + t * b;
            const dm::V p = dm::glerp(to_dm(a), to_dm(b), t);
            ++checked;
            if (!same3(p, o)) ++bad;
        }
        // Tangents (solver.cpp:324-331 with the zero check).
        std::vector<V3> tan(count);
        std::vector<dm::V> tan_dm(count);
        for (int k = 0; k < count; ++k) {
            V3 d;
            if (k == 0) d = x[1] - x[0];
            else if (k + 1 == count) d = x[k] - x[k - 1];
            else d = x[k + 1] - x[k - 1];
            tan[k] = normalized(d);
            dm::V dd;
            if (k == 0) dd = dm::gsub(to_dm(x[1]), to_dm(x[0]));
            else if (k + 1 == count) dd = dm::gsub(to_dm(x[k]), to_dm(x[k - 1]));
            else dd = dm::gsub(to_dm(x[k + 1]), to_dm(x[k - 1]));
            tan_dm[k] = dm::gunit(dd);
            ++checked;
            if (!same3(tan_dm[k], tan[k])) ++bad;
        }
        // The strand walk of compute_root_targets.
        M3 f = frame_from_tangent(tan[0], ref[0].col(0));
        dm::M fd = dm::frame_from_tangent(tan_dm[0], dm::v(ref[0].m[0], ref[0].m[3], ref[0].m[6]));
        for (int k = 0; k < count; ++k) {
            if (k > 0) {
                const V3 d1 = parallel_transport(f.col(0), tan[k - 1], tan[k]);
                f = frame_from_tangent(tan[k], d1);
                const dm::V d1d = dm::parallel_transport(dm::v(fd.m[0], fd.m[3], fd.m[6]), tan_dm[k - 1], tan_dm[k]);
                fd = dm::frame_from_tangent(tan_dm[k], d1d);
                ++checked;
                if (!same3(d1d, d1)) ++bad;
            }
            ++checked;
            if (!same9(fd, f)) ++bad;
            const V3 r = rotation_vector(matmul(f, transpose(ref[k])));
            const dm::V rd = dm::rotation_vector(dm::times_transpose(fd, to_dm(ref[k])));
            ++checked;
            if (!same3(rd, r)) ++bad;
        }
    }
    // Rotation vectors of the branches of Shepperd's method and near a half turn.
    for (int k = 0; k < 20000; ++k) {
        const double angle = k % 3 == 0 ? 3.14159265358979 - 1e-9 * u(g) : (k % 3 == 1 ? 1e-8 * u(g) : 3.0 * u(g));
        const V3 axis = normalized(v3(n(g), n(g), n(g)));
        const M3 r = rotation(axis, angle);
        ++checked;
        if (!same3(dm::rotation_vector(to_dm(r)), rotation_vector(r))) ++bad;
    }
    std::printf("root-target math: %ld checks, %ld mismatches\n", checked, bad);
    std::printf(bad == 0 ? "PASS\n" : "FAIL\n");
    return bad == 0 ? 0 : 1;
}
