// ORACLE — test infrastructure only.
//
// A CPU FP64 restatement of the reference solver's per-substep
// incremental-potential solve and of the host model builder that feeds it.
// It exports the same C ABI (include/kami_hair_solver.h) as the GB300
// product library so tests can drive both with identical calls and compare
// results.  Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
// legs load it; the product library never links, loads or calls it.
//
// What it follows, function by function (paths inside the reference project):
//   host builder         src/solver.cpp:121-556 (set_hair, set_collider,
//                        make_internal_mesh, frames/elements, masses, root
//                        targets, collider topology, host BVH, feasibility)
//   device BVH build     src/cuda_backend.cu:294-311 (HostBvh)
//   refit                src/cuda_backend.cu:776-792, 596-602
//   geometry             src/cuda_backend.cu:200-232 (device flavour, no
//                        interior-crossing test) and src/geometry.hpp (host
//                        flavour, used only by the build-time feasibility check)
//   energy/grad/GN       src/cuda_backend.cu:234-265, 883-939 (Dual<12>/<6>)
//   block solve          src/cuda_backend.cu:855-881
//   preconditioner etc.  src/cuda_backend.cu:794-853
//   sweep / CCD          src/cuda_backend.cu:966-1000
//   friction             src/cuda_backend.cu:941-964, 615-621
//   control flow         src/cuda_backend.cu:482-498, 604-723
//   C ABI wrapper        src/api.cpp:16-304
//
// Parallel work (OpenMP) writes into per-element / per-node / per-strand
// slots and every reduction then runs serially in index order, so results
// are independent of the thread count.  Where the reference reduces with
// unordered double atomics, the oracle fixes the order as: node term first,
// then each incident element in increasing element index (elastic part,
// then contact part).  cuBLAS level-1 reductions are replaced by plain
// sequential sums.  Where the reference records "the first" failure through
// a compare-and-swap race, the oracle records the lowest element index and,
// within it, the first triangle in traversal order.
//
// Pinning: the reference ships no golden trajectories.  This oracle is
// checked against every known-answer invariant the reference's own tests
// hold (tests/test_solver.cpp, tests/test_c_api.c) in
// tests/test_oracle_reference_invariants.py.

#include "kami_hair_solver.h"
#include "khs_oracle_math.hpp"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace khs_oracle {

constexpr int kBvhStack = 64;                        // cuda_backend.cu:26
constexpr uint64_t kCheckpointMagic = 0x3154504348534bULL;  // cuda_backend.cu:27
constexpr uint32_t kNone = 0xffffffffu;

// Bounded-sample knob for CPU timing: when non-zero, a frame stops after
// this many substeps (no adaptive retry).  Oracle-only; 0 = whole frames.
static uint32_t g_substep_limit = 0;

// ---------------------------------------------------------------------------
// Strand partition (the sharded-solve design, on CPU ranks).
//
// Strands are independent in assembly, factorisation and contact; the solve
// couples them only through global scalars: energies, the gradient norm, the
// slope g.d, the direction norm, the CCD step bound, the largest node
// translation, the candidate and active-contact counts, feasibility and
// failure flags.  A partitioned solver works on strands [s0, s1) only and
// combines those scalars with a caller-supplied all-reduce over int64
// arrays.  Sums are exact (ExactSum: a fixed-point accumulator whose limbs
// add as integers, rounded once to the nearest double), so the result does
// not depend on how the strands are split: N ranks give the bits of one.

// all-reduce in place over `count` int64 values; op 0 = sum, 1 = min, 2 = max.
using ReduceFn = void (*)(void *ctx, int64_t *values, uint32_t count, int op);

struct ExactSum {
    static constexpr int kLimbs = 68;     // 32-bit limbs from 2^-1088 up: every finite double fits
    static constexpr int kBase = -1088;
    static constexpr int kSize = kLimbs + 3;  // + counts of NaN, +inf, -inf terms
    int64_t v[kSize] = {};

    void add(double x)
    {
        if (std::isnan(x)) { ++v[kLimbs]; return; }
        if (std::isinf(x)) { ++v[x > 0 ? kLimbs + 1 : kLimbs + 2]; return; }
        if (x == 0.0) return;
        int e = 0;
        const double m = std::frexp(std::fabs(x), &e);   // |x| = m 2^e, m in [0.5, 1)
        uint64_t M = uint64_t(std::ldexp(m, 53));         // |x| = M 2^(e - 53), exactly
        int lo = e - 53;
        if (lo < -1074) { M >>= (-1074 - lo); lo = -1074; }  // subnormal: exact multiple of 2^-1074
        const int p = lo - kBase, i = p / 32, o = p % 32;
        const unsigned __int128 w = (unsigned __int128)M << o;
        const int64_t s = x < 0 ? -1 : 1;
        v[i] += s * int64_t(uint64_t(w) & 0xffffffffull);
        v[i + 1] += s * int64_t(uint64_t(w >> 32) & 0xffffffffull);
        v[i + 2] += s * int64_t(uint64_t(w >> 64));
    }

    // The exact sum rounded to the nearest double (ties to even).
    double value() const
    {
        if (v[kLimbs] || (v[kLimbs + 1] && v[kLimbs + 2])) return std::numeric_limits<double>::quiet_NaN();
        if (v[kLimbs + 1]) return std::numeric_limits<double>::infinity();
        if (v[kLimbs + 2]) return -std::numeric_limits<double>::infinity();
        int64_t a[kLimbs];
        std::copy(v, v + kLimbs, a);
        auto normalise = [&]() {
            for (int i = 0; i + 1 < kLimbs; ++i) {
                const int64_t c = a[i] >> 32;  // floor division by 2^32
                a[i] -= c * (int64_t(1) << 32);
                a[i + 1] += c;
            }
        };
        normalise();
        const bool neg = a[kLimbs - 1] < 0;
        if (neg) {
            for (int64_t &x : a) x = -x;
            normalise();
        }
        int t = kLimbs - 1;
        while (t >= 0 && a[t] == 0) --t;
        if (t < 0) return 0.0;
        auto limb = [&](int i) { return i >= 0 ? uint64_t(a[i]) : 0ull; };
        const unsigned __int128 X = ((unsigned __int128)limb(t) << 64) | ((unsigned __int128)limb(t - 1) << 32) | limb(t - 2);
        bool sticky = false;
        for (int i = 0; i < t - 2; ++i) sticky = sticky || a[i] != 0;
        const int lsb = 32 * (t - 2) + kBase;  // exponent of X's lowest bit
        int L = 127;
        while (!((X >> L) & 1)) --L;
        const int keep = std::max(L + lsb - 52, -1074);  // exponent of the lowest kept bit
        const int sh = keep - lsb;
        unsigned __int128 mant;
        if (sh <= 0) {
            mant = X << (-sh);
        } else {
            mant = X >> sh;
            const unsigned __int128 rem = X & ((((unsigned __int128)1) << sh) - 1);
            const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
            if (rem > half || (rem == half && (sticky || (mant & 1)))) ++mant;
        }
        const double r = std::ldexp(double(uint64_t(mant)), keep);
        return neg ? -r : r;
    }
};

// Order-preserving int64 key of a double (for min/max all-reduce).
inline int64_t order_key(double x)
{
    int64_t b;
    std::memcpy(&b, &x, 8);
    return b >= 0 ? b : b ^ std::numeric_limits<int64_t>::max();
}
inline double from_order_key(int64_t k)
{
    const int64_t b = k >= 0 ? k : k ^ std::numeric_limits<int64_t>::max();
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}

// ---------------------------------------------------------------------------
// Geometry.

struct Pair { double distance, t; V3 bary; };

// Ericson-style closest point on a triangle (cuda_backend.cu:200-209,
// geometry.hpp:15-50; both flavours perform identical arithmetic).
inline V3 closest_point_triangle(V3 p, V3 a, V3 b, V3 c, V3 &bary)
{
    const V3 ab = b - a, ac = c - a, ap = p - a;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) { bary = v3(1, 0, 0); return a; }
    const V3 bp = p - b;
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { bary = v3(0, 1, 0); return b; }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { const double v = d1 / (d1 - d3); bary = v3(1 - v, v, 0); return a + ab * v; }
    const V3 cp = p - c;
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { bary = v3(0, 0, 1); return c; }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { const double w = d2 / (d2 - d6); bary = v3(1 - w, 0, w); return a + ac * w; }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary = v3(0, 1 - w, w);
        return b + (c - b) * w;
    }
    const double inv = 1.0 / (va + vb + vc), v = vb * inv, w = vc * inv;
    bary = v3(1 - v - w, v, w);
    return a + ab * v + ac * w;
}

// Clamped segment-segment parameters (cuda_backend.cu:210-216,
// geometry.hpp:59-87).
inline void segment_params(V3 p1, V3 q1, V3 p2, V3 q2, double &s, double &t)
{
    const V3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    const double a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    s = 0; t = 0;
    if (a <= 1e-14 && e <= 1e-14) return;
    if (a <= 1e-14) { t = std::fmin(1.0, std::fmax(0.0, f / e)); return; }
    const double c = dot(d1, r);
    if (e <= 1e-14) { s = std::fmin(1.0, std::fmax(0.0, -c / a)); return; }
    const double b = dot(d1, d2), den = a * e - b * b;
    if (den != 0) s = std::fmin(1.0, std::fmax(0.0, (b * f - c * e) / den));
    t = (b * s + f) / e;
    if (t < 0) { t = 0; s = std::fmin(1.0, std::fmax(0.0, -c / a)); }
    else if (t > 1) { t = 1; s = std::fmin(1.0, std::fmax(0.0, (b - c) / a)); }
}

// Device flavour: no interior-crossing test (cuda_backend.cu:217-223).
inline Pair closest_segment_triangle_device(V3 p0, V3 p1, V3 a, V3 b, V3 c)
{
    Pair out{1.0e300, 0.0, v3(1, 0, 0)};
    V3 bary;
    V3 cp = closest_point_triangle(p0, a, b, c, bary);
    double d = norm(p0 - cp);
    if (d < out.distance) out = {d, 0.0, bary};
    cp = closest_point_triangle(p1, a, b, c, bary);
    d = norm(p1 - cp);
    if (d < out.distance) out = {d, 1.0, bary};
    const V3 tv[3] = {a, b, c};
    for (int e = 0; e < 3; ++e) {
        const V3 p2 = tv[e], q2 = tv[(e + 1) % 3];
        double s, t;
        segment_params(p0, p1, p2, q2, s, t);
        const V3 d1 = p1 - p0, d2 = q2 - p2;
        const double dd = norm((p0 + d1 * s) - (p2 + d2 * t));
        if (dd < out.distance) {
            out.distance = dd;
            out.t = s;
            out.bary = V3{};
            if (e == 0) { out.bary.x = 1 - t; out.bary.y = t; }
            else if (e == 1) { out.bary.y = 1 - t; out.bary.z = t; }
            else { out.bary.z = 1 - t; out.bary.x = t; }
        }
    }
    return out;
}

// Host flavour with the Moller-Trumbore crossing test (geometry.hpp:89-151);
// used only by the build-time feasibility check.
inline bool segment_triangle_hit(V3 p0, V3 p1, V3 a, V3 b, V3 c)
{
    const V3 d = p1 - p0, e1 = b - a, e2 = c - a, h = cross(d, e2);
    const double det = dot(e1, h);
    if (std::fabs(det) < 1.0e-14) return false;
    const double inv = 1.0 / det;
    const V3 s = p0 - a;
    const double u = inv * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const V3 q = cross(s, e1);
    const double v = inv * dot(d, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = inv * dot(e2, q);
    return !(t < 0.0 || t > 1.0);
}

inline double closest_segment_triangle_host(V3 p0, V3 p1, V3 a, V3 b, V3 c)
{
    if (segment_triangle_hit(p0, p1, a, b, c)) return 0.0;
    double best = std::numeric_limits<double>::infinity();
    V3 bary;
    best = std::min(best, norm(p0 - closest_point_triangle(p0, a, b, c, bary)));
    best = std::min(best, norm(p1 - closest_point_triangle(p1, a, b, c, bary)));
    const V3 tv[3] = {a, b, c};
    for (int e = 0; e < 3; ++e) {
        const V3 p2 = tv[e], q2 = tv[(e + 1) % 3];
        double s, t;
        segment_params(p0, p1, p2, q2, s, t);
        const double dd = norm((p0 + s * (p1 - p0)) - (p2 + t * (q2 - p2)));
        best = std::min(best, dd);
    }
    return best;
}

inline bool overlap(V3 al, V3 au, V3 bl, V3 bu, double p)
{
    return al.x <= bu.x + p && bl.x <= au.x + p && al.y <= bu.y + p && bl.y <= au.y + p &&
           al.z <= bu.z + p && bl.z <= au.z + p;
}

struct Tri { uint32_t i0, i1, i2; };

// ---------------------------------------------------------------------------
// BVHs.

struct BvhNode { V3 lower, upper; uint32_t begin = 0, count = 0; int left = -1, right = -1; };

// Device BVH: median split on the centroid span's largest axis, <= 8
// triangles per leaf, nodes in creation (pre-)order, per-depth level lists
// for the bottom-up refit (cuda_backend.cu:294-311).
struct DeviceBvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order, leaves;
    std::vector<std::vector<uint32_t>> levels;
    const std::vector<V3> *vertices = nullptr;
    const std::vector<Tri> *triangles = nullptr;

    V3 centroid(uint32_t t) const
    {
        const Tri &tr = (*triangles)[t];
        return div_recip(((*vertices)[tr.i0] + (*vertices)[tr.i1]) + (*vertices)[tr.i2], 3.0);
    }
    int build_node(uint32_t begin, uint32_t end, uint32_t depth)
    {
        const int idx = int(nodes.size());
        nodes.push_back({});
        if (levels.size() <= depth) levels.resize(depth + 1);
        levels[depth].push_back(uint32_t(idx));
        V3 lo = v3(1e300, 1e300, 1e300), hi = v3(-1e300, -1e300, -1e300), cl = lo, cu = hi;
        for (uint32_t k = begin; k < end; ++k) {
            const Tri &t = (*triangles)[order[k]];
            const V3 a = (*vertices)[t.i0], b = (*vertices)[t.i1], c = (*vertices)[t.i2];
            lo = vmin(lo, vmin(a, vmin(b, c)));
            hi = vmax(hi, vmax(a, vmax(b, c)));
            const V3 ce = div_recip((a + b) + c, 3.0);
            cl = vmin(cl, ce);
            cu = vmax(cu, ce);
        }
        nodes[idx].lower = lo; nodes[idx].upper = hi;
        nodes[idx].begin = begin; nodes[idx].count = end - begin;
        nodes[idx].left = nodes[idx].right = -1;
        if (end - begin <= 8) { leaves.push_back(uint32_t(idx)); return idx; }
        const V3 span = cu - cl;
        const int axis = span.y > span.x ? (span.z > span.y ? 2 : 1) : (span.z > span.x ? 2 : 0);
        const uint32_t mid = begin + (end - begin) / 2;
        std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + end,
                         [&](uint32_t l, uint32_t r) { return centroid(l)[axis] < centroid(r)[axis]; });
        const int left = build_node(begin, mid, depth + 1);
        const int right = build_node(mid, end, depth + 1);
        nodes[idx].left = left; nodes[idx].right = right; nodes[idx].count = 0;
        return idx;
    }
    void build(const std::vector<V3> &v, const std::vector<Tri> &t)
    {
        vertices = &v; triangles = &t;
        nodes.clear(); leaves.clear(); levels.clear();
        order.resize(t.size());
        std::iota(order.begin(), order.end(), 0u);
        if (!t.empty()) build_node(0, uint32_t(t.size()), 0);
    }
    // Leaves then levels bottom-up (cuda_backend.cu:776-792).
    void refit(const std::vector<Tri> &tris, const std::vector<V3> &cur, const std::vector<V3> &old, bool swept)
    {
        for (uint32_t leaf : leaves) {
            BvhNode &n = nodes[leaf];
            V3 lo = v3(1e300, 1e300, 1e300), hi = v3(-1e300, -1e300, -1e300);
            for (uint32_t j = n.begin; j < n.begin + n.count; ++j) {
                const Tri &t = tris[order[j]];
                const uint32_t ids[3] = {t.i0, t.i1, t.i2};
                for (int c = 0; c < 3; ++c) {
                    lo = vmin(lo, cur[ids[c]]); hi = vmax(hi, cur[ids[c]]);
                    if (swept) { lo = vmin(lo, old[ids[c]]); hi = vmax(hi, old[ids[c]]); }
                }
            }
            n.lower = lo; n.upper = hi;
        }
        for (int depth = int(levels.size()) - 2; depth >= 0; --depth) {
            for (uint32_t idx : levels[depth]) {
                BvhNode &n = nodes[idx];
                if (n.left < 0) continue;
                n.lower = vmin(nodes[n.left].lower, nodes[n.right].lower);
                n.upper = vmax(nodes[n.left].upper, nodes[n.right].upper);
            }
        }
    }
    // DFS with a 64-entry stack that pushes left then right, so the right
    // child is visited first (cuda_backend.cu:229-232).
    template<class F> void query(V3 lo, V3 hi, double padding, F &&f) const
    {
        if (nodes.empty()) return;
        int stack[kBvhStack], top = 0;
        stack[top++] = 0;
        while (top) {
            const BvhNode &n = nodes[stack[--top]];
            if (!overlap(lo, hi, n.lower, n.upper, padding)) continue;
            if (n.left >= 0) {
                if (top + 2 <= kBvhStack) { stack[top++] = n.left; stack[top++] = n.right; }
            } else {
                for (uint32_t k = n.begin; k < n.begin + n.count; ++k) f(order[k]);
            }
        }
    }
};

// Host BVH used by the build-time feasibility check (solver.cpp:36-109):
// same median split but +-inf initial bounds, per-axis centroid divided by
// 3 and the first largest axis.
struct HostBvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
    int build_node(uint32_t begin, uint32_t end, const std::vector<V3> &v, const std::vector<Tri> &t)
    {
        const int index = int(nodes.size());
        nodes.push_back({});
        const double inf = std::numeric_limits<double>::infinity();
        V3 lower = v3(inf, inf, inf), upper = v3(-inf, -inf, -inf), cl = lower, cu = upper;
        for (uint32_t k = begin; k < end; ++k) {
            const Tri &tr = t[order[k]];
            const V3 a = v[tr.i0], b = v[tr.i1], c = v[tr.i2];
            lower = vmin(vmin(vmin(lower, a), b), c);
            upper = vmax(vmax(vmax(upper, a), b), c);
            const V3 centroid = div_each((a + b) + c, 3.0);
            cl = vmin(cl, centroid);
            cu = vmax(cu, centroid);
        }
        nodes[index].lower = lower; nodes[index].upper = upper;
        nodes[index].begin = begin; nodes[index].count = end - begin;
        if (end - begin <= 8) return index;
        const V3 span = cu - cl;
        int axis = 0;
        if (span.y > span[axis]) axis = 1;
        if (span.z > span[axis]) axis = 2;
        const uint32_t middle = begin + (end - begin) / 2;
        std::nth_element(order.begin() + begin, order.begin() + middle, order.begin() + end,
                         [&](uint32_t l, uint32_t r) {
                             const Tri &a = t[l], &b = t[r];
                             const double lc = (v[a.i0][axis] + v[a.i1][axis] + v[a.i2][axis]) / 3.0;
                             const double rc = (v[b.i0][axis] + v[b.i1][axis] + v[b.i2][axis]) / 3.0;
                             return lc < rc;
                         });
        const int left = build_node(begin, middle, v, t);
        const int right = build_node(middle, end, v, t);
        nodes[index].left = left; nodes[index].right = right; nodes[index].count = 0;
        return index;
    }
    void build(const std::vector<V3> &v, const std::vector<Tri> &t)
    {
        order.resize(t.size());
        std::iota(order.begin(), order.end(), 0u);
        nodes.clear();
        if (!t.empty()) build_node(0, uint32_t(t.size()), v, t);
    }
    void query(V3 lower, V3 upper, double padding, std::vector<uint32_t> &out) const
    {
        out.clear();
        if (nodes.empty()) return;
        std::vector<int> stack{0};
        while (!stack.empty()) {
            const int index = stack.back();
            stack.pop_back();
            const BvhNode &node = nodes[index];
            if (!overlap(lower, upper, node.lower, node.upper, padding)) continue;
            if (node.left >= 0) { stack.push_back(node.left); stack.push_back(node.right); }
            else for (uint32_t k = node.begin; k < node.begin + node.count; ++k) out.push_back(order[k]);
        }
    }
};

// ---------------------------------------------------------------------------
// Model.

struct Binding { uint32_t left = 0, right = 0; double t = 0.0; };
struct Node {
    V3 x, rotation;
    M3 ref;  // row-major reference frame (columns d1, d2, d3)
    double mass = 0, rmass = 0;
    bool fixed = false, virt = false;
    uint32_t strand = 0;
    Binding binding;
};
struct Element {
    uint32_t i = 0, j = 0, strand = 0;
    bool contact = true;
    double L0 = 0;
    V3 rest_shear, rest_curv;
};
struct Strand { uint32_t first, count, fixed_count; };

struct Stats {
    double objective = 0, elastic = 0, contact = 0, friction = 0, kinetic = 0;
    double minimum_gap = std::numeric_limits<double>::infinity();
    uint64_t candidates = 0, active = 0;
    bool feasible = true;
};

struct SweepFailure {
    bool claimed = false;
    uint32_t strand = 0, element = 0, triangle = 0;
    double distance = 0, required = 0, clearance = 0, displacement = 0;
    V3 hair_start, hair_end, collider_point;
};

class Solver {
public:
    explicit Solver(const KhsSolverDesc &d) : desc_(d)
    {
        step_stats_ = {};
        step_stats_.struct_size = sizeof(KhsStepStats);
        step_stats_.phase = KHS_PHASE_IDLE;
        clear_failure();
    }

    std::string error_;

    // ---- input (solver.cpp:121-225) ----
    KhsResult set_hair(const KhsVec3 *points, uint32_t point_count, const uint32_t *offsets,
                       uint32_t strand_count, const KhsHairMaterial &m)
    {
        if (!points || !offsets || point_count < 2 || strand_count == 0 || offsets[0] != 0 ||
            offsets[strand_count] != point_count) {
            error_ = "invalid hair points or strand offsets";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        for (uint32_t s = 0; s < strand_count; ++s)
            if (offsets[s + 1] <= offsets[s] || offsets[s + 1] > point_count) {
                error_ = "strand offsets are not increasing";
                return KHS_ERROR_INVALID_HAIR;
            }
        if (!(m.density > 0.0 && m.radius > 0.0 && m.young_modulus > 0.0 && m.poisson_ratio > -1.0 &&
              m.poisson_ratio < 0.5 && m.shear_correction > 0.0 && m.contact_stiffness > 0.0 &&
              m.barrier_distance > 0.0 && m.friction >= 0.0 && m.friction_smoothing > 0.0)) {
            error_ = "hair material out of range";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        std::vector<V3> conv(point_count);
        for (uint32_t i = 0; i < point_count; ++i) {
            conv[i] = v3(points[i].x, points[i].y, points[i].z);
            if (!finite3(conv[i])) { error_ = "non-finite hair point"; return KHS_ERROR_INVALID_HAIR; }
        }
        clear_built();
        input_points_ = conv;
        input_offsets_.assign(offsets, offsets + strand_count + 1);
        material_ = m;
        has_hair_ = true;
        error_.clear();
        return KHS_OK;
    }

    KhsResult set_collider(const KhsVec3 *vertices, uint32_t vertex_count, const KhsTriangle *tris,
                           uint32_t tri_count)
    {
        if (tri_count == 0) {
            has_collider_ = false;
            collider_pending_.clear(); collider_current_.clear(); triangles_.clear();
            excluded_ = 0; built_ = false;
            return KHS_OK;
        }
        if (!vertices || !tris || vertex_count < 3) { error_ = "invalid collider arrays"; return KHS_ERROR_INVALID_ARGUMENT; }
        collider_pending_.resize(vertex_count);
        for (uint32_t i = 0; i < vertex_count; ++i) collider_pending_[i] = v3(vertices[i].x, vertices[i].y, vertices[i].z);
        triangles_.clear();
        excluded_ = 0;
        for (uint32_t k = 0; k < tri_count; ++k) {
            const KhsTriangle &s = tris[k];
            if (s.i0 >= vertex_count || s.i1 >= vertex_count || s.i2 >= vertex_count || s.i0 == s.i1 ||
                s.i1 == s.i2 || s.i2 == s.i0 || !finite3(collider_pending_[s.i0]) ||
                !finite3(collider_pending_[s.i1]) || !finite3(collider_pending_[s.i2])) { ++excluded_; continue; }
            const V3 c = cross(collider_pending_[s.i1] - collider_pending_[s.i0], collider_pending_[s.i2] - collider_pending_[s.i0]);
            if (norm2(c) <= 1.0e-24) { ++excluded_; continue; }
            triangles_.push_back({s.i0, s.i1, s.i2});
        }
        if (triangles_.empty()) { error_ = "no valid collider triangle"; return KHS_ERROR_INVALID_COLLIDER; }
        collider_current_ = collider_pending_;
        has_collider_ = true;
        built_ = false;
        error_.clear();
        return KHS_OK;
    }

    // ---- build (solver.cpp:449-556) ----
    KhsResult build()
    {
        if (!has_hair_) { error_ = "set hair curves first"; return KHS_ERROR_INVALID_STATE; }
        step_stats_.phase = KHS_PHASE_PREPARING;
        if (!make_internal_mesh()) { step_stats_.phase = KHS_PHASE_FAILED; return KHS_ERROR_INVALID_HAIR; }
        init_frames_and_elements();
        init_masses();
        free_dofs_ = 0;
        for (const Node &n : nodes_) if (!n.fixed) free_dofs_ += 6;
        if (!compute_root_targets(input_points_, root_x_, root_r_)) {
            error_ = "cannot build initial root directions";
            step_stats_.phase = KHS_PHASE_FAILED;
            return KHS_ERROR_INVALID_HAIR;
        }
        if (has_collider_) {
            validate_topology();
            collider_current_ = collider_pending_;
            host_bvh_.build(collider_current_, triangles_);
            if (!initial_feasibility()) { step_stats_.phase = KHS_PHASE_FAILED; return KHS_ERROR_INITIAL_INTERSECTION; }
        }
        initialize_backend();
        built_ = true;
        build_stats_ = {};
        build_stats_.struct_size = sizeof(KhsBuildStats);
        build_stats_.strand_count = uint32_t(strand_nodes_.size());
        build_stats_.original_point_count = uint32_t(input_points_.size());
        build_stats_.internal_node_count = uint32_t(nodes_.size());
        build_stats_.element_count = uint32_t(elements_.size());
        build_stats_.fixed_node_count = uint32_t(std::count_if(nodes_.begin(), nodes_.end(), [](const Node &n) { return n.fixed; }));
        build_stats_.collider_vertex_count = uint32_t(collider_current_.size());
        build_stats_.collider_triangle_count = uint32_t(triangles_.size());
        build_stats_.excluded_collider_triangle_count = excluded_;
        build_stats_.collider_boundary_edge_count = boundary_;
        build_stats_.collider_nonmanifold_edge_count = nonmanifold_;
        build_stats_.collider_inconsistent_edge_count = inconsistent_;
        build_stats_.collider_inverted_closed_component_count = inverted_;
        build_stats_.merged_zero_length_segment_count = merged_;
        build_stats_.virtual_extension_strand_count = vext_strands_;
        build_stats_.virtual_extension_node_count = vext_nodes_;
        build_stats_.virtual_extension_rest_length = vext_length_;
        build_stats_.degree_of_freedom_count = free_dofs_;
        build_stats_.estimated_bytes = nodes_.size() * 200 + elements_.size() * 80 + collider_current_.size() * 24 * 4 +
                                       triangles_.size() * 12;
        build_stats_.initial_minimum_gap = has_collider_ ? current_minimum_gap(nullptr) : std::numeric_limits<double>::infinity();
        step_stats_.phase = KHS_PHASE_IDLE;
        error_.clear();
        return KHS_OK;
    }

    KhsResult update_runtime(const KhsSolverDesc &d, const KhsHairMaterial &m)
    {
        if (!built_) { error_ = "build before updating runtime parameters"; return KHS_ERROR_INVALID_STATE; }
        if (d.maximum_element_length != desc_.maximum_element_length ||
            d.minimum_dynamic_length != desc_.minimum_dynamic_length || d.fixed_root_nodes != desc_.fixed_root_nodes) {
            error_ = "topology-defining parameters cannot change after build";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        if (!(m.density > 0.0 && m.radius > 0.0 && m.young_modulus > 0.0 && m.poisson_ratio > -1.0 &&
              m.poisson_ratio < 0.5 && m.shear_correction > 0.0 && m.mass_damping >= 0.0 &&
              m.contact_stiffness > 0.0 && m.barrier_distance > 0.0 && m.friction >= 0.0 &&
              m.friction_smoothing > 0.0 && m.collider_offset >= 0.0)) {
            error_ = "runtime material out of range";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        desc_ = d;
        material_ = m;
        init_masses();
        trust_radius_ = std::fmax(0.25 * max_rest_length_, 8.0 * (material_.radius + material_.collider_offset + material_.barrier_distance));
        error_.clear();
        return KHS_OK;
    }

    KhsResult update_collider(const KhsVec3 *v, uint32_t n)
    {
        if (!built_ || !has_collider_) { error_ = "no built collider"; return KHS_ERROR_INVALID_STATE; }
        if (!v || n != collider_pending_.size()) { error_ = "collider vertex count changed"; return KHS_ERROR_INVALID_COLLIDER; }
        for (uint32_t i = 0; i < n; ++i) {
            collider_pending_[i] = v3(v[i].x, v[i].y, v[i].z);
            if (!finite3(collider_pending_[i])) { error_ = "non-finite collider vertex"; return KHS_ERROR_INVALID_COLLIDER; }
        }
        d_collider_pending_ = collider_pending_;
        return KHS_OK;
    }

    KhsResult update_roots(const KhsVec3 *p, uint32_t n)
    {
        if (!built_ || !p || n != input_points_.size()) { error_ = "root target count mismatch"; return KHS_ERROR_INVALID_ARGUMENT; }
        std::vector<V3> conv(n);
        for (uint32_t i = 0; i < n; ++i) {
            conv[i] = v3(p[i].x, p[i].y, p[i].z);
            if (!finite3(conv[i])) { error_ = "non-finite root target"; return KHS_ERROR_INVALID_HAIR; }
        }
        std::vector<V3> pos, rot;
        if (!compute_root_targets(conv, pos, rot)) { error_ = "cannot compute root directions"; return KHS_ERROR_INVALID_HAIR; }
        root_pending_x_ = pos;
        root_pending_r_ = rot;
        return KHS_OK;
    }

    // Extension khsxComputeRootTargets: the targets update_roots computes,
    // copied out instead of stored.
    KhsResult roots_to_host(const KhsVec3 *p, uint32_t n, KhsVec3 *pos_out, KhsVec3 *rot_out, uint32_t capacity)
    {
        if (!built_ || !p || n != input_points_.size()) { error_ = "root target count mismatch"; return KHS_ERROR_INVALID_ARGUMENT; }
        std::vector<V3> conv(n);
        for (uint32_t i = 0; i < n; ++i) {
            conv[i] = v3(p[i].x, p[i].y, p[i].z);
            if (!finite3(conv[i])) { error_ = "non-finite root target"; return KHS_ERROR_INVALID_HAIR; }
        }
        if (!pos_out || !rot_out || capacity < N()) { error_ = "root target output too small"; return KHS_ERROR_INVALID_ARGUMENT; }
        std::vector<V3> pos, rot;
        if (!compute_root_targets(conv, pos, rot)) { error_ = "cannot compute root directions"; return KHS_ERROR_INVALID_HAIR; }
        for (size_t k = 0; k < N(); ++k) {
            pos_out[k] = {pos[k].x, pos[k].y, pos[k].z};
            rot_out[k] = {rot[k].x, rot[k].y, rot[k].z};
        }
        return KHS_OK;
    }

    KhsResult step(double frame_dt)
    {
        if (!built_) { error_ = "prepare the solver first"; return KHS_ERROR_INVALID_STATE; }
        if (!(frame_dt > 0.0) || !std::isfinite(frame_dt)) { error_ = "time step must be positive and finite"; return KHS_ERROR_INVALID_ARGUMENT; }
        const KhsResult r = run_frame(frame_dt, root_current_x_.data(), root_current_r_.data(), root_pending_x_.data(),
                                      root_pending_r_.data(), d_collider_frame_start_.data(), d_collider_pending_.data(), 0, 0);
        if (r == KHS_OK) error_.clear();
        return r;
    }

    // ---- animation (cuda_backend.cu:447-498) ----
    KhsResult allocate_animation(uint32_t frames)
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        if (frames < 1) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid animation frame count");
        anim_frames_ = frames;
        anim_root_x_.assign(size_t(frames) * N(), V3{});
        anim_root_r_.assign(size_t(frames) * N(), V3{});
        anim_collider_.assign(size_t(frames) * collider_current_.size(), V3{});
        root_set_.assign(frames, false);
        collider_set_.assign(frames, collider_current_.empty());
        return KHS_OK;
    }
    KhsResult set_root_frame(uint32_t f, const KhsVec3 *p, uint32_t n)
    {
        if (!built_ || !p || n != input_points_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        std::vector<V3> conv(n);
        for (uint32_t i = 0; i < n; ++i) { conv[i] = v3(p[i].x, p[i].y, p[i].z); if (!finite3(conv[i])) return KHS_ERROR_INVALID_HAIR; }
        std::vector<V3> pos, rot;
        if (!compute_root_targets(conv, pos, rot)) return KHS_ERROR_INVALID_HAIR;
        if (f >= anim_frames_) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid root animation frame");
        std::copy(pos.begin(), pos.end(), anim_root_x_.begin() + size_t(f) * N());
        std::copy(rot.begin(), rot.end(), anim_root_r_.begin() + size_t(f) * N());
        root_set_[f] = true;
        return KHS_OK;
    }
    KhsResult set_collider_frame(uint32_t f, const KhsVec3 *v, uint32_t n)
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        if (f >= anim_frames_ || n != collider_current_.size()) return fail(KHS_ERROR_INVALID_COLLIDER, "invalid collider animation frame");
        for (uint32_t i = 0; i < n; ++i) anim_collider_[size_t(f) * n + i] = v3(v[i].x, v[i].y, v[i].z);
        collider_set_[f] = true;
        return KHS_OK;
    }
    KhsResult finalize_animation()
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        if (anim_frames_ < 1 || std::find(root_set_.begin(), root_set_.end(), false) != root_set_.end() ||
            std::find(collider_set_.begin(), collider_set_.end(), false) != collider_set_.end())
            return fail(KHS_ERROR_INVALID_STATE, "animation has missing frames");
        animation_ready_ = true;
        current_frame_ = 0;
        return KHS_OK;
    }
    KhsResult step_animation_frame(uint32_t frame, double dt)
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        if (!animation_ready_ || frame >= anim_frames_) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid animation frame index");
        if (frame == 0) { current_frame_ = 0; return KHS_OK; }
        if (frame != current_frame_ + 1) return fail(KHS_ERROR_INVALID_STATE, "animation frames must be stepped in order");
        const uint32_t a = frame - 1, b = frame;
        const size_t nv = collider_current_.size();
        const KhsResult r = run_frame(dt, &anim_root_x_[size_t(a) * N()], &anim_root_r_[size_t(a) * N()],
                                      &anim_root_x_[size_t(b) * N()], &anim_root_r_[size_t(b) * N()],
                                      nv ? &anim_collider_[size_t(a) * nv] : nullptr,
                                      nv ? &anim_collider_[size_t(b) * nv] : nullptr, frame, anim_frames_);
        if (r == KHS_OK) { current_frame_ = frame; error_.clear(); }
        return r;
    }

    // ---- checkpoints (cuda_backend.cu:500-537) ----
    struct CkptHeader { uint64_t magic; uint32_t abi; uint32_t frame; uint64_t dof; };
    uint64_t checkpoint_size() const
    {
        if (!built_ || !animation_ready_) return 0;
        return sizeof(CkptHeader) + uint64_t(2 * dof() * sizeof(double));
    }
    KhsResult save_checkpoint(void *data, uint64_t cap)
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        const uint64_t req = checkpoint_size();
        if (!data || !req || cap < req) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid checkpoint output buffer");
        CkptHeader h{kCheckpointMagic, KHS_ABI_VERSION, current_frame_, uint64_t(dof())};
        auto *out = static_cast<unsigned char *>(data);
        std::memcpy(out, &h, sizeof(h));
        std::memcpy(out + sizeof(h), q_.data(), dof() * 8);
        std::memcpy(out + sizeof(h) + dof() * 8, v_.data(), dof() * 8);
        error_.clear();
        return KHS_OK;
    }
    KhsResult restore_checkpoint(const void *data, uint64_t size)
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        const uint64_t req = checkpoint_size();
        if (!data || !req || size != req) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid checkpoint size");
        CkptHeader h{};
        std::memcpy(&h, data, sizeof(h));
        if (h.magic != kCheckpointMagic || h.abi != KHS_ABI_VERSION || h.dof != dof() || h.frame >= anim_frames_)
            return fail(KHS_ERROR_INVALID_ARGUMENT, "checkpoint does not match this solver");
        const auto *in = static_cast<const unsigned char *>(data);
        std::memcpy(q_.data(), in + sizeof(h), dof() * 8);
        std::memcpy(v_.data(), in + sizeof(h) + dof() * 8, dof() * 8);
        old_q_ = q_; snap_q_ = q_; snap_v_ = v_;
        current_frame_ = h.frame;
        cancel_.store(false);
        progress_frame_.store(h.frame);
        progress_substep_.store(0); progress_substep_count_.store(0); progress_iteration_.store(0);
        progress_phase_.store(KHS_PHASE_FINISHED);
        step_stats_ = {};
        step_stats_.struct_size = sizeof(step_stats_);
        step_stats_.phase = KHS_PHASE_FINISHED;
        clear_failure();
        error_.clear();
        return KHS_OK;
    }

    // ---- readback ----
    uint32_t original_count() const { return uint32_t(input_points_.size()); }
    uint32_t internal_count() const { return uint32_t(nodes_.size()); }
    KhsResult copy_original(KhsVec3 *out, uint32_t cap) const
    {
        if (!built_ || !out || cap < mapping_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        for (size_t i = 0; i < mapping_.size(); ++i) { const size_t n = mapping_[i]; out[i] = {q_[6 * n], q_[6 * n + 1], q_[6 * n + 2]}; }
        return KHS_OK;
    }
    KhsResult copy_internal(KhsVec3 *out, uint32_t cap) const
    {
        if (!built_ || !out || cap < nodes_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        for (size_t n = 0; n < nodes_.size(); ++n) out[n] = {q_[6 * n], q_[6 * n + 1], q_[6 * n + 2]};
        return KHS_OK;
    }
    KhsResult copy_mapping(uint32_t *out, uint32_t cap) const
    {
        if (!built_ || !out || cap < mapping_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        std::copy(mapping_.begin(), mapping_.end(), out);
        return KHS_OK;
    }
    KhsResult copy_state(double *q, double *v, uint64_t cap) const
    {
        if (!built_ || cap < dof()) return KHS_ERROR_INVALID_ARGUMENT;
        if (q) std::copy(q_.begin(), q_.end(), q);
        if (v) std::copy(v_.begin(), v_.end(), v);
        return KHS_OK;
    }
    KhsResult copy_contacts(KhsxContactRecord *out, uint32_t cap) const
    {
        if (!built_ || !out || cap < elements_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        for (size_t e = 0; e < elements_.size(); ++e) out[e] = contact_records_.empty() ? KhsxContactRecord{0, kNone, 0, 0, 0.0} : contact_records_[e];
        return KHS_OK;
    }
    // Contact classification of every element at positions q (the contact
    // part of cuda_backend.cu:920-929 without energy).
    KhsResult query_contacts(const double *q, uint64_t dof_count, KhsxContactRecord *out, uint32_t cap) const
    {
        if (!built_ || !q || dof_count < dof() || !out || cap < E()) return KHS_ERROR_INVALID_ARGUMENT;
        const KhsHairMaterial &m = material_;
        for (size_t ei = 0; ei < E(); ++ei) {
            const Element &e = elements_[ei];
            KhsxContactRecord r{0, kNone, 0, 0, std::numeric_limits<double>::infinity()};
            if (has_collider() && !nodes_[e.i].fixed && e.contact) {
                const V3 p0 = v3(q[6 * e.i], q[6 * e.i + 1], q[6 * e.i + 2]), p1 = v3(q[6 * e.j], q[6 * e.j + 1], q[6 * e.j + 2]);
                Pair pair{1.0e300, 0.0, v3(1, 0, 0)};
                uint32_t closest = kNone, cands = 0;
                dev_bvh_.query(vmin(p0, p1), vmax(p0, p1), m.radius + m.collider_offset + m.barrier_distance, [&](uint32_t ti) {
                    ++cands;
                    const Tri &t = triangles_[ti];
                    const Pair c = closest_segment_triangle_device(p0, p1, d_collider_current_[t.i0], d_collider_current_[t.i1], d_collider_current_[t.i2]);
                    if (c.distance < pair.distance) { pair = c; closest = ti; }
                });
                r.candidate_count = cands;
                if (closest != kNone) {
                    r.closest_triangle = closest;
                    r.gap = pair.distance - m.radius - m.collider_offset;
                    r.active = (r.gap > desc_.minimum_gap && r.gap < m.barrier_distance) ? 1u : 0u;
                }
            }
            out[ei] = r;
        }
        return KHS_OK;
    }

    KhsResult build_stats(KhsBuildStats *s) const
    {
        if (!built_ || !s || s->struct_size < sizeof(KhsBuildStats)) return KHS_ERROR_INVALID_ARGUMENT;
        *s = build_stats_;
        return KHS_OK;
    }
    KhsResult get_step_stats(KhsStepStats *s) const
    {
        if (!s || s->struct_size < sizeof(KhsStepStats)) return KHS_ERROR_INVALID_ARGUMENT;
        *s = step_stats_;
        return KHS_OK;
    }
    KhsResult gpu_stats(KhsGpuStats *s) const
    {
        if (!built_ || !s || s->struct_size < sizeof(KhsGpuStats)) return KHS_ERROR_INVALID_ARGUMENT;
        KhsGpuStats g{};
        g.struct_size = sizeof(g);
        g.animation_frame_count = anim_frames_;
        g.resident_bytes = uint64_t(dof()) * 8 * 12 + uint64_t(N()) * 36 * 8 * 3 + anim_root_x_.size() * 48 + anim_collider_.size() * 24;
        g.last_frame_milliseconds = last_frame_ms_;
        *s = g;
        return KHS_OK;
    }
    KhsResult progress(KhsProgress *p) const
    {
        if (!built_ || !p || p->struct_size < sizeof(KhsProgress)) return KHS_ERROR_INVALID_ARGUMENT;
        KhsProgress r{};
        r.struct_size = sizeof(r);
        r.phase = progress_phase_.load(); r.frame_index = progress_frame_.load(); r.frame_count = progress_frame_count_.load();
        r.substep = progress_substep_.load(); r.substep_count = progress_substep_count_.load();
        r.nonlinear_iteration = progress_iteration_.load(); r.nonlinear_iteration_limit = desc_.newton_iterations;
        r.cancelled = cancel_.load() ? 1u : 0u;
        r.frame_elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - frame_clock_).count();
        *p = r;
        return KHS_OK;
    }
    KhsResult failure(KhsFailureDiagnostics *d) const
    {
        if (!built_ || !d || d->struct_size < sizeof(KhsFailureDiagnostics)) return KHS_ERROR_INVALID_ARGUMENT;
        *d = failure_;
        return KHS_OK;
    }
    KhsResult request_cancel()
    {
        if (!built_) return KHS_ERROR_INVALID_STATE;
        cancel_.store(true);
        return KHS_OK;
    }
    // Test hook: the Gauss-Newton system of the most recent gradient
    // evaluation (FP64 blocks, gradient) and the strand layout.
    void export_system(double *diag, double *upper, double *grad, uint32_t *strands) const
    {
        if (diag) std::copy(diag_.begin(), diag_.end(), diag);
        if (upper) std::copy(upper_.begin(), upper_.end(), upper);
        if (grad) std::copy(grad_.begin(), grad_.end(), grad);
        if (strands)
            for (size_t s = 0; s < strands_.size(); ++s) {
                strands[3 * s] = strands_[s].first; strands[3 * s + 1] = strands_[s].count; strands[3 * s + 2] = strands_[s].fixed_count;
            }
    }
    // Test hook: the built rod model in the form the reference's CUDA backend
    // takes it (CudaNodeInit / CudaElementInit / strand node lists, the
    // original-to-internal map and the collider; cuda_backend.hpp:14-55,
    // filled as solver.cpp:485-517 fills them).  sizes = {nodes, elements,
    // strands, original points, collider vertices, triangles}.  Per node:
    // 18 doubles (position, rotation vector, reference frame rows 0-2, mass,
    // rotational mass, binding t) and 4 u32 (strand, binding left, binding
    // right, fixed).  Per element: 7 doubles (rest length, rest shear, rest
    // curvature) and 4 u32 (i, j, strand, collider contact).  Per strand: its
    // first node and node count (the nodes of a strand are consecutive).
    void model_sizes(uint32_t *sizes) const
    {
        sizes[0] = uint32_t(nodes_.size()); sizes[1] = uint32_t(elements_.size());
        sizes[2] = uint32_t(strand_nodes_.size()); sizes[3] = uint32_t(mapping_.size());
        sizes[4] = has_collider_ ? uint32_t(collider_current_.size()) : 0u;
        sizes[5] = has_collider_ ? uint32_t(triangles_.size()) : 0u;
    }
    void export_model(double *node_f, uint32_t *node_u, double *elem_f, uint32_t *elem_u, uint32_t *strand_u,
                      uint32_t *mapping, double *collider, uint32_t *tris) const
    {
        for (size_t i = 0; i < nodes_.size(); ++i) {
            const Node &n = nodes_[i];
            double *f = node_f + 18 * i;
            f[0] = n.x.x; f[1] = n.x.y; f[2] = n.x.z;
            f[3] = n.rotation.x; f[4] = n.rotation.y; f[5] = n.rotation.z;
            for (int k = 0; k < 9; ++k) f[6 + k] = n.ref.m[k];
            f[15] = n.mass; f[16] = n.rmass; f[17] = n.binding.t;
            uint32_t *u = node_u + 4 * i;
            u[0] = n.strand; u[1] = n.binding.left; u[2] = n.binding.right; u[3] = n.fixed ? 1u : 0u;
        }
        for (size_t e = 0; e < elements_.size(); ++e) {
            const Element &el = elements_[e];
            double *f = elem_f + 7 * e;
            f[0] = el.L0;
            f[1] = el.rest_shear.x; f[2] = el.rest_shear.y; f[3] = el.rest_shear.z;
            f[4] = el.rest_curv.x; f[5] = el.rest_curv.y; f[6] = el.rest_curv.z;
            uint32_t *u = elem_u + 4 * e;
            u[0] = el.i; u[1] = el.j; u[2] = el.strand; u[3] = el.contact ? 1u : 0u;
        }
        for (size_t s = 0; s < strand_nodes_.size(); ++s) {
            strand_u[2 * s] = strand_nodes_[s].front();
            strand_u[2 * s + 1] = uint32_t(strand_nodes_[s].size());
        }
        std::copy(mapping_.begin(), mapping_.end(), mapping);
        if (has_collider_) {
            for (size_t v = 0; v < collider_current_.size(); ++v) {
                collider[3 * v] = collider_current_[v].x; collider[3 * v + 1] = collider_current_[v].y;
                collider[3 * v + 2] = collider_current_[v].z;
            }
            for (size_t t = 0; t < triangles_.size(); ++t) {
                tris[3 * t] = triangles_[t].i0; tris[3 * t + 1] = triangles_[t].i1; tris[3 * t + 2] = triangles_[t].i2;
            }
        }
    }
    void set_substep_limit(uint32_t n) { substep_limit_ = n; }

    // Strand partition (see ReduceFn): from now on this solver steps only
    // strands [s0, s1) and combines global quantities with `fn`.  Requires a
    // built solver.
    KhsResult set_partition(uint32_t s0, uint32_t s1, ReduceFn fn, void *ctx)
    {
        if (!built_ || !fn || s0 >= s1 || s1 > strands_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        part_ = true;
        reduce_ = fn;
        reduce_ctx_ = ctx;
        s_lo_ = s0; s_hi_ = s1;
        n_lo_ = strands_[s0].first;
        n_hi_ = size_t(strands_[s1 - 1].first) + strands_[s1 - 1].count;
        e_lo_ = 0;
        while (e_lo_ < E() && elements_[e_lo_].strand < s0) ++e_lo_;
        e_hi_ = e_lo_;
        while (e_hi_ < E() && elements_[e_hi_].strand < s1) ++e_hi_;
        return KHS_OK;
    }
    uint32_t record_count() const { return uint32_t(records_.size()); }
    KhsResult copy_records(KhsxSubstepRecord *out, uint32_t cap) const
    {
        if (!out || cap < records_.size()) return KHS_ERROR_INVALID_ARGUMENT;
        std::copy(records_.begin(), records_.end(), out);
        return KHS_OK;
    }

private:
    size_t N() const { return nodes_.size(); }
    size_t E() const { return elements_.size(); }
    size_t dof() const { return 6 * nodes_.size(); }

    KhsResult fail(KhsResult r, const char *msg)
    {
        error_ = msg;
        step_stats_.phase = KHS_PHASE_FAILED;
        progress_phase_.store(KHS_PHASE_FAILED);
        return r;
    }

    void clear_built()
    {
        built_ = false;
        nodes_.clear(); elements_.clear(); strand_nodes_.clear(); mapping_.clear();
        merged_ = 0; vext_strands_ = 0; vext_nodes_ = 0; vext_length_ = 0.0;
        animation_ready_ = false; anim_frames_ = 0;
    }

    void clear_failure()
    {
        failure_ = {};
        failure_.struct_size = sizeof(failure_);
        failure_.strand_index = kNone;
        failure_.element_index = kNone;
        failure_.collider_triangle_index = kNone;
    }

    // solver.cpp:227-318
    bool make_internal_mesh()
    {
        nodes_.clear(); elements_.clear();
        strand_nodes_.assign(input_offsets_.size() - 1, {});
        mapping_.assign(input_points_.size(), 0);
        const double hmax = desc_.maximum_element_length, zero_tol = 1.0e-12;
        vext_strands_ = 0; vext_nodes_ = 0; vext_length_ = 0.0; merged_ = 0;
        for (uint32_t s = 0; s + 1 < input_offsets_.size(); ++s) {
            const uint32_t begin = input_offsets_[s], end = input_offsets_[s + 1];
            Node first;
            first.x = input_points_[begin];
            first.strand = s;
            first.binding = {begin, begin, 0.0};
            nodes_.push_back(first);
            strand_nodes_[s].push_back(uint32_t(nodes_.size() - 1));
            mapping_[begin] = uint32_t(nodes_.size() - 1);
            V3 previous = input_points_[begin];
            uint32_t unique = 0, term_left = begin, term_right = begin;
            double strand_len = 0.0, term_len = 0.0;
            V3 term_dir;
            for (uint32_t p = begin + 1; p < end; ++p) {
                const V3 target = input_points_[p];
                const double length = norm(target - previous);
                if (length <= zero_tol) {
                    mapping_[p] = strand_nodes_[s].back();
                    ++merged_;
                    previous = target;
                    continue;
                }
                const uint32_t divisions = std::max(1u, uint32_t(std::ceil(length / hmax)));
                for (uint32_t d = 1; d <= divisions; ++d) {
                    const double t = double(d) / divisions;
                    Node node;
                    node.x = (1.0 - t) * previous + t * target;
                    node.strand = s;
                    node.binding = {p - 1, p, t};
                    nodes_.push_back(node);
                    strand_nodes_[s].push_back(uint32_t(nodes_.size() - 1));
                }
                mapping_[p] = strand_nodes_[s].back();
                previous = target;
                strand_len += length;
                term_left = p - 1;
                term_right = p;
                term_len = length;
                term_dir = div_each(target - input_points_[p - 1], length);
                ++unique;
            }
            if (unique == 0 || strand_nodes_[s].size() < 2) {
                std::ostringstream ss;
                ss << "strand " << s << " has all points coincident";
                error_ = ss.str();
                return false;
            }
            if (desc_.minimum_dynamic_length > strand_len + zero_tol) {
                const double ext = desc_.minimum_dynamic_length - strand_len;
                const uint32_t divisions = std::max(1u, uint32_t(std::ceil(ext / hmax)));
                const V3 tip = input_points_[end - 1];
                for (uint32_t d = 1; d <= divisions; ++d) {
                    const double distance = ext * double(d) / divisions;
                    Node node;
                    node.x = tip + distance * term_dir;
                    node.strand = s;
                    node.virt = true;
                    node.binding = {term_left, term_right, 1.0 + distance / term_len};
                    nodes_.push_back(node);
                    strand_nodes_[s].push_back(uint32_t(nodes_.size() - 1));
                }
                ++vext_strands_;
                vext_nodes_ += divisions;
                vext_length_ += ext;
            }
            const uint32_t fixed = std::min<uint32_t>(desc_.fixed_root_nodes, uint32_t(strand_nodes_[s].size()));
            for (uint32_t k = 0; k < fixed; ++k) nodes_[strand_nodes_[s][k]].fixed = true;
        }
        return true;
    }

    // Central-difference unit tangents along a strand (solver.cpp:324-331).
    static bool strand_tangents(const std::vector<uint32_t> &idx, const std::vector<V3> &x, std::vector<V3> &t, bool check)
    {
        t.resize(idx.size());
        for (size_t k = 0; k < idx.size(); ++k) {
            V3 d;
            if (k == 0) d = x[idx[1]] - x[idx[0]];
            else if (k + 1 == idx.size()) d = x[idx[k]] - x[idx[k - 1]];
            else d = x[idx[k + 1]] - x[idx[k - 1]];
            if (check && norm2(d) < 1.0e-24) return false;
            t[k] = normalized(d);
        }
        return true;
    }

    // solver.cpp:320-356
    void init_frames_and_elements()
    {
        elements_.clear();
        std::vector<V3> x(N());
        for (size_t n = 0; n < N(); ++n) x[n] = nodes_[n].x;
        for (uint32_t s = 0; s < strand_nodes_.size(); ++s) {
            const auto &idx = strand_nodes_[s];
            std::vector<V3> tangents;
            strand_tangents(idx, x, tangents, false);
            M3 frame = frame_from_tangent(tangents[0], v3(1, 0, 0));
            nodes_[idx[0]].ref = frame;
            for (size_t k = 1; k < idx.size(); ++k) {
                const V3 d1 = parallel_transport(frame.col(0), tangents[k - 1], tangents[k]);
                frame = frame_from_tangent(tangents[k], d1);
                nodes_[idx[k]].ref = frame;
            }
            for (size_t k = 0; k + 1 < idx.size(); ++k) {
                Element e;
                e.i = idx[k]; e.j = idx[k + 1]; e.strand = s;
                e.contact = !nodes_[e.j].virt;
                e.L0 = norm(nodes_[e.j].x - nodes_[e.i].x);
                const M3 &ri = nodes_[e.i].ref, &rj = nodes_[e.j].ref;
                const V3 tangent = div_each(nodes_[e.j].x - nodes_[e.i].x, e.L0);
                M3 half;
                const M3 rit = transpose(ri), rjt = transpose(rj);
                for (int k2 = 0; k2 < 9; ++k2) half.m[k2] = 0.5 * (rit.m[k2] + rjt.m[k2]);
                e.rest_shear = matvec(half, tangent);
                e.rest_curv = div_each(cayley_vector(matmul(rit, rj)), e.L0);
                elements_.push_back(e);
            }
        }
    }

    // solver.cpp:358-373
    void init_masses()
    {
        const double pi = 3.14159265358979323846;
        const double area = pi * material_.radius * material_.radius;
        const double inertia = pi * std::pow(material_.radius, 4.0) / 4.0;
        const double polar = 2.0 * inertia;
        for (Node &n : nodes_) { n.mass = 0.0; n.rmass = 0.0; }
        for (const Element &e : elements_) {
            const double mass = material_.density * area * e.L0;
            const double rmass = material_.density * (2.0 * inertia + polar) / 3.0 * e.L0;
            nodes_[e.i].mass += 0.5 * mass; nodes_[e.j].mass += 0.5 * mass;
            nodes_[e.i].rmass += 0.5 * rmass; nodes_[e.j].rmass += 0.5 * rmass;
        }
    }

    // solver.cpp:416-447
    bool compute_root_targets(const std::vector<V3> &points, std::vector<V3> &pos, std::vector<V3> &rot) const
    {
        if (points.size() != input_points_.size()) return false;
        pos.resize(N()); rot.resize(N());
        for (size_t n = 0; n < N(); ++n) {
            const Binding &b = nodes_[n].binding;
            pos[n] = (1.0 - b.t) * points[b.left] + b.t * points[b.right];
            rot[n] = nodes_[n].rotation;
        }
        for (const auto &idx : strand_nodes_) {
            std::vector<V3> tangents;
            if (!strand_tangents(idx, pos, tangents, true)) return false;
            M3 frame = frame_from_tangent(tangents[0], nodes_[idx[0]].ref.col(0));
            rot[idx[0]] = rotation_vector(matmul(frame, transpose(nodes_[idx[0]].ref)));
            for (size_t k = 1; k < idx.size(); ++k) {
                const V3 d1 = parallel_transport(frame.col(0), tangents[k - 1], tangents[k]);
                frame = frame_from_tangent(tangents[k], d1);
                rot[idx[k]] = rotation_vector(matmul(frame, transpose(nodes_[idx[k]].ref)));
            }
        }
        return true;
    }

    // solver.cpp:381-414
    void validate_topology()
    {
        boundary_ = nonmanifold_ = inconsistent_ = inverted_ = 0;
        struct Use { uint32_t count = 0; int dir = 0; };
        std::map<uint64_t, Use> uses;
        for (const Tri &t : triangles_) {
            const std::pair<uint32_t, uint32_t> es[3] = {{t.i0, t.i1}, {t.i1, t.i2}, {t.i2, t.i0}};
            for (const auto &e : es) {
                const uint32_t a = std::min(e.first, e.second), b = std::max(e.first, e.second);
                Use &u = uses[(uint64_t(a) << 32) | b];
                ++u.count;
                u.dir += e.first < e.second ? 1 : -1;
            }
        }
        for (const auto &kv : uses) {
            if (kv.second.count == 1) ++boundary_;
            else if (kv.second.count > 2) ++nonmanifold_;
            else if (kv.second.dir != 0) ++inconsistent_;
        }
        closed_ = boundary_ == 0 && nonmanifold_ == 0 && inconsistent_ == 0;
        if (closed_) {
            double vol = 0.0;
            for (const Tri &t : triangles_) vol += dot(collider_current_[t.i0], cross(collider_current_[t.i1], collider_current_[t.i2]));
            if (vol < 0.0) inverted_ = 1;
        }
    }

    // Ray parity (solver.cpp:608-632).
    bool point_inside(V3 p) const
    {
        uint32_t hits = 0;
        for (const Tri &t : triangles_)
            if (ray_crosses_triangle(p, collider_current_[t.i0], collider_current_[t.i1], collider_current_[t.i2])) ++hits;
        return (hits & 1u) != 0;
    }

    // solver.cpp:634-657
    bool initial_feasibility()
    {
        if (closed_) {
            for (size_t n = 0; n < N(); ++n) {
                if (nodes_[n].fixed || nodes_[n].virt) continue;
                if (point_inside(nodes_[n].x)) {
                    std::ostringstream ss;
                    ss << "initial intersection: internal node " << n << " is inside the closed collider";
                    error_ = ss.str();
                    return false;
                }
            }
        }
        uint64_t count = 0;
        const double gap = current_minimum_gap(&count);
        if (gap <= desc_.minimum_gap) {
            std::ostringstream ss;
            ss << "initial intersection or negative gap: minimum gap=" << gap << " m, candidates=" << count;
            error_ = ss.str();
            return false;
        }
        return true;
    }

    // solver.cpp:659-681
    double current_minimum_gap(uint64_t *count_out) const
    {
        double minimum = std::numeric_limits<double>::infinity();
        uint64_t count = 0;
        std::vector<uint32_t> cands;
        const double pad = material_.radius + material_.collider_offset + material_.barrier_distance;
        for (const Element &e : elements_) {
            if (nodes_[e.i].fixed || !e.contact) continue;
            host_bvh_.query(vmin(nodes_[e.i].x, nodes_[e.j].x), vmax(nodes_[e.i].x, nodes_[e.j].x), pad, cands);
            for (uint32_t ti : cands) {
                const Tri &t = triangles_[ti];
                const double d = closest_segment_triangle_host(nodes_[e.i].x, nodes_[e.j].x, collider_current_[t.i0],
                                                               collider_current_[t.i1], collider_current_[t.i2]);
                minimum = std::min(minimum, d - material_.radius - material_.collider_offset);
                ++count;
            }
        }
        if (count_out) *count_out = count;
        return minimum;
    }

    // ---- backend state (cuda_backend.cu:341-407) ----
    void initialize_backend()
    {
        const size_t n = N();
        q_.assign(6 * n, 0.0); v_.assign(6 * n, 0.0);
        for (size_t i = 0; i < n; ++i) {
            q_[6 * i] = nodes_[i].x.x; q_[6 * i + 1] = nodes_[i].x.y; q_[6 * i + 2] = nodes_[i].x.z;
            q_[6 * i + 3] = nodes_[i].rotation.x; q_[6 * i + 4] = nodes_[i].rotation.y; q_[6 * i + 5] = nodes_[i].rotation.z;
        }
        old_q_ = q_; snap_q_ = q_; snap_v_ = v_; base_q_ = q_;
        grad_.assign(6 * n, 0.0); dir_.assign(6 * n, 0.0); precond_.assign(6 * n, 0.0);
        diag_.assign(36 * n, 0.0); upper_.assign(36 * n, 0.0);
        cprime_.assign(36 * n, 0.0); dprime_.assign(6 * n, 0.0);
        max_rest_length_ = 0.0;
        for (const Element &e : elements_) max_rest_length_ = std::fmax(max_rest_length_, e.L0);
        trust_radius_ = std::fmax(0.25 * max_rest_length_, 8.0 * (material_.radius + material_.collider_offset + material_.barrier_distance));
        strands_.clear();
        for (const auto &idx : strand_nodes_) {
            uint32_t fixed = 0;
            while (fixed < idx.size() && nodes_[idx[fixed]].fixed) ++fixed;
            strands_.push_back({idx.front(), uint32_t(idx.size()), fixed});
        }
        root_current_x_ = root_x_; root_current_r_ = root_r_;
        root_pending_x_ = root_x_; root_pending_r_ = root_r_;
        d_collider_current_ = collider_current_;
        d_collider_old_ = collider_current_;
        d_collider_frame_start_ = collider_current_;
        d_collider_pending_ = collider_current_;
        if (!triangles_.empty()) dev_bvh_.build(d_collider_current_, triangles_);
        contact_records_.assign(E(), KhsxContactRecord{0, kNone, 0, 0, 0.0});
        animation_ready_ = false;
        anim_frames_ = 0;
        current_frame_ = 0;
        clear_failure();
    }

    bool has_collider() const { return !triangles_.empty(); }

    // Per-element evaluation output.
    struct ElemOut {
        double elastic = 0, contact = 0;
        double gi[6], gj[6], ci[3], cj[3];
        double hii[36], hjj[36], hij[36];
        double chii[9], chjj[9], chij[9];
        uint32_t candidates = 0, closest = kNone;
        double gap = std::numeric_limits<double>::infinity();
        bool feasible = true, active = false, has_contact_terms = false;
    };

    // Strains (cuda_backend.cu:234-245).
    void strains12(const Element &e, Dual<12> strain[6]) const
    {
        Dual<12> dq[12];
        for (int d = 0; d < 6; ++d) {
            dq[d] = Dual<12>::var(q_[6 * e.i + d], d);
            dq[6 + d] = Dual<12>::var(q_[6 * e.j + d], 6 + d);
        }
        DV3<12> xi{dq[0], dq[1], dq[2]}, ui{dq[3], dq[4], dq[5]}, xj{dq[6], dq[7], dq[8]}, uj{dq[9], dq[10], dq[11]};
        DM3<12> refi, refj;
        for (int k = 0; k < 9; ++k) { refi.m[k] = Dual<12>(nodes_[e.i].ref.m[k]); refj.m[k] = Dual<12>(nodes_[e.j].ref.m[k]); }
        const DM3<12> ri = dm_mul(dexp_so3(ui), refi), rj = dm_mul(dexp_so3(uj), refj);
        const DV3<12> tangent = dvscale(dvsub(xj, xi), Dual<12>(1.0 / e.L0));
        const DV3<12> shear = dvscale(dm_vec(dm_add(dm_transpose(ri), dm_transpose(rj)), tangent), Dual<12>(0.5));
        const DV3<12> curvature = dvscale(dcayley(dm_mul(dm_transpose(ri), rj)), Dual<12>(1.0 / e.L0));
        const DV3<12> ds = dvsub(shear, DV3<12>{Dual<12>(e.rest_shear.x), Dual<12>(e.rest_shear.y), Dual<12>(e.rest_shear.z)});
        const DV3<12> dk = dvsub(curvature, DV3<12>{Dual<12>(e.rest_curv.x), Dual<12>(e.rest_curv.y), Dual<12>(e.rest_curv.z)});
        strain[0] = ds.x; strain[1] = ds.y; strain[2] = ds.z; strain[3] = dk.x; strain[4] = dk.y; strain[5] = dk.z;
    }

    V3 pos(size_t n) const { return v3(q_[6 * n], q_[6 * n + 1], q_[6 * n + 2]); }

    // Element energy, gradient, GN Hessian and barrier contact
    // (cuda_backend.cu:899-939).
    void eval_element(size_t ei, bool grad, ElemOut &o) const
    {
        const Element &e = elements_[ei];
        const KhsHairMaterial &m = material_;
        Dual<12> strain[6];
        strains12(e, strain);
        const double area = kPi * m.radius * m.radius, inertia = kPi * m.radius * m.radius * m.radius * m.radius / 4.0;
        const double G = m.young_modulus / (2.0 * (1.0 + m.poisson_ratio));
        const double w[6] = {m.shear_correction * G * area, m.shear_correction * G * area, m.young_modulus * area,
                             m.young_modulus * inertia, m.young_modulus * inertia, 2.0 * G * inertia};
        Dual<12> re(0.0);
        for (int s = 0; s < 6; ++s) re = re + Dual<12>(0.5 * e.L0 * w[s]) * strain[s] * strain[s];
        o.elastic = re.v;
        const bool fi = nodes_[e.i].fixed, fj = nodes_[e.j].fixed;
        for (int d = 0; d < 6; ++d) { o.gi[d] = fi ? 0.0 : re.d[d]; o.gj[d] = fj ? 0.0 : re.d[6 + d]; }
        std::fill(o.hii, o.hii + 36, 0.0); std::fill(o.hjj, o.hjj + 36, 0.0); std::fill(o.hij, o.hij + 36, 0.0);
        if (grad) {
            for (int a = 0; a < 12; ++a)
                for (int b = 0; b < 12; ++b) {
                    double h = 0.0;
                    for (int s = 0; s < 6; ++s) h += e.L0 * w[s] * strain[s].d[a] * strain[s].d[b];
                    if (a < 6 && b < 6 && !fi) o.hii[6 * a + b] = h;
                    else if (a >= 6 && b >= 6 && !fj) o.hjj[6 * (a - 6) + (b - 6)] = h;
                    else if (a < 6 && b >= 6 && !fi && !fj) o.hij[6 * a + (b - 6)] = h;
                }
        }
        o.contact = 0.0;
        o.has_contact_terms = false;
        o.candidates = 0; o.closest = kNone; o.active = false; o.feasible = true;
        o.gap = std::numeric_limits<double>::infinity();
        if (!has_collider() || fi || !e.contact) return;
        const V3 p0 = pos(e.i), p1 = pos(e.j);
        const double padding = m.radius + m.collider_offset + m.barrier_distance;
        uint32_t closest = kNone;
        Pair pair{1.0e300, 0.0, v3(1, 0, 0)};
        uint32_t cands = 0;
        dev_bvh_.query(vmin(p0, p1), vmax(p0, p1), padding, [&](uint32_t ti) {
            ++cands;
            const Tri &t = triangles_[ti];
            const Pair c = closest_segment_triangle_device(p0, p1, d_collider_current_[t.i0], d_collider_current_[t.i1], d_collider_current_[t.i2]);
            if (c.distance < pair.distance) { pair = c; closest = ti; }
        });
        o.candidates = cands;
        if (closest == kNone) return;
        o.closest = closest;
        const Tri &t = triangles_[closest];
        const double gap = pair.distance - m.radius - m.collider_offset;
        o.gap = gap;
        if (gap <= desc_.minimum_gap) { o.feasible = false; return; }
        if (gap >= m.barrier_distance) return;
        o.active = true;
        const V3 a = d_collider_current_[t.i0], b = d_collider_current_[t.i1], c = d_collider_current_[t.i2];
        // contact_energy_dual (cuda_backend.cu:255-265) with Dual<6>.
        Dual<6> cq[6];
        for (int d = 0; d < 3; ++d) { cq[d] = Dual<6>::var(q_[6 * e.i + d], d); cq[3 + d] = Dual<6>::var(q_[6 * e.j + d], 3 + d); }
        DV3<6> x0{cq[0], cq[1], cq[2]}, x1{cq[3], cq[4], cq[5]};
        const Dual<6> tt(pair.t);
        const DV3<6> p = dvadd(dvscale(x0, Dual<6>(1) - tt), dvscale(x1, tt));
        const V3 bp = (a * pair.bary.x + b * pair.bary.y) + c * pair.bary.z;
        const DV3<6> diff = dvsub(p, DV3<6>{Dual<6>(bp.x), Dual<6>(bp.y), Dual<6>(bp.z)});
        const Dual<6> dist = dsqrt(dvdot(diff, diff) + Dual<6>(1e-30));
        const Dual<6> dgap = dist - Dual<6>(m.radius + m.collider_offset);
        Dual<6> ce(0.0);
        if (dgap.v >= m.barrier_distance) {
            ce = cq[0] * Dual<6>(0);
        } else {
            const Dual<6> aa = Dual<6>(m.barrier_distance) - dgap, lg = dlog(dgap / Dual<6>(m.barrier_distance));
            ce = -Dual<6>(m.contact_stiffness) * aa * aa * lg;
        }
        if (!std::isfinite(ce.v)) { o.feasible = false; return; }
        o.contact = ce.v;
        o.has_contact_terms = true;
        for (int d = 0; d < 3; ++d) { o.ci[d] = ce.d[d]; o.cj[d] = ce.d[3 + d]; }
        std::fill(o.chii, o.chii + 9, 0.0); std::fill(o.chjj, o.chjj + 9, 0.0); std::fill(o.chij, o.chij + 9, 0.0);
        if (grad) {
            const V3 normal = div_recip((p0 * (1.0 - pair.t) + p1 * pair.t) - bp, std::fmax(pair.distance, 1e-15));
            const double aa = m.barrier_distance - gap;
            const double curv = m.contact_stiffness * (-2.0 * std::log(gap / m.barrier_distance) + 4.0 * aa / gap + aa * aa / (gap * gap));
            const double dg[6] = {normal.x * (1.0 - pair.t), normal.y * (1.0 - pair.t), normal.z * (1.0 - pair.t),
                                  normal.x * pair.t, normal.y * pair.t, normal.z * pair.t};
            for (int a2 = 0; a2 < 6; ++a2)
                for (int b2 = 0; b2 < 6; ++b2) {
                    const double h = curv * dg[a2] * dg[b2];
                    if (a2 < 3 && b2 < 3) o.chii[3 * a2 + b2] = h;
                    else if (a2 >= 3 && b2 >= 3) o.chjj[3 * (a2 - 3) + (b2 - 3)] = h;
                    else if (a2 < 3 && b2 >= 3) o.chij[3 * a2 + (b2 - 3)] = h;
                }
        }
    }

    // evaluate (cuda_backend.cu:604-613 + 883-939) with ordered reductions.
    Stats evaluate(bool grad, double dt)
    {
        const size_t n = N(), ne = E();
        std::vector<ElemOut> &eo = elem_out_;
        eo.resize(ne);
        std::vector<double> node_obj(n, 0.0), node_kin(n, 0.0);
        const KhsHairMaterial &m = material_;
        const double inv = 1.0 / dt, inv2 = inv * inv;
#pragma omp parallel for schedule(static)
        for (long long ni = (long long)nlo(); ni < (long long)nhi(); ++ni) {
            const size_t k = size_t(ni);
            if (grad) for (int z = 0; z < 36; ++z) diag_[36 * k + z] = 0.0;
            if (grad) for (int d = 0; d < 6; ++d) grad_[6 * k + d] = 0.0;
            if (nodes_[k].fixed) continue;
            const double kx = nodes_[k].mass * inv2, kr = nodes_[k].rmass * inv2;
            const double cx = nodes_[k].mass * m.mass_damping * inv, cr = nodes_[k].rmass * m.mass_damping * inv;
            double obj = 0, kin = 0;
            for (int d = 0; d < 6; ++d) {
                const double g = d < 3 ? (&desc_.gravity.x)[d] * dt * dt : 0.0;
                const double predicted = old_q_[6 * k + d] + dt * v_[6 * k + d] + g;
                const double delta = q_[6 * k + d] - predicted;
                const double damp = q_[6 * k + d] - old_q_[6 * k + d], kk = d < 3 ? kx : kr, c = d < 3 ? cx : cr;
                obj += 0.5 * kk * delta * delta + 0.5 * c * damp * damp;
                if (d < 3) kin += 0.5 * nodes_[k].mass * damp * damp * inv2;
                if (grad) { grad_[6 * k + d] = kk * delta + c * damp; diag_[36 * k + d * 6 + d] = kk + c; }
            }
            node_obj[k] = obj;
            node_kin[k] = kin;
        }
        if (grad) std::fill(upper_.begin(), upper_.end(), 0.0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long ei = (long long)elo(); ei < (long long)ehi(); ++ei) eval_element(size_t(ei), grad, eo[size_t(ei)]);
        // Ordered scatter: node term, then incident elements by index.
        if (grad) {
#pragma omp parallel for schedule(static)
            for (long long ei = (long long)elo(); ei < (long long)ehi(); ++ei) {
                // upper block of node i belongs to element (i, j) only.
                const Element &e = elements_[size_t(ei)];
                const ElemOut &o = eo[size_t(ei)];
                for (int z = 0; z < 36; ++z) upper_[36 * e.i + z] = o.hij[z];
                if (o.has_contact_terms)
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) upper_[36 * e.i + 6 * a + b] += o.chij[3 * a + b];
            }
            for (size_t ei = elo(); ei < ehi(); ++ei) {
                const Element &e = elements_[ei];
                const ElemOut &o = eo[ei];
                for (int d = 0; d < 6; ++d) { grad_[6 * e.i + d] += o.gi[d]; }
                for (int z = 0; z < 36; ++z) diag_[36 * e.i + z] += o.hii[z];
                if (o.has_contact_terms) {
                    for (int d = 0; d < 3; ++d) grad_[6 * e.i + d] += o.ci[d];
                    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) diag_[36 * e.i + 6 * a + b] += o.chii[3 * a + b];
                }
                for (int d = 0; d < 6; ++d) { grad_[6 * e.j + d] += o.gj[d]; }
                for (int z = 0; z < 36; ++z) diag_[36 * e.j + z] += o.hjj[z];
                if (o.has_contact_terms) {
                    for (int d = 0; d < 3; ++d) grad_[6 * e.j + d] += o.cj[d];
                    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) diag_[36 * e.j + 6 * a + b] += o.chjj[3 * a + b];
                }
            }
        }
        Stats st;
        double node_sum = 0, kin = 0, el = 0, co = 0;
        if (part_) {
            // Exact sums over this range, combined across the ranks.
            ExactSum sn, sk, se, sc;
            for (size_t k = nlo(); k < nhi(); ++k) { sn.add(node_obj[k]); sk.add(node_kin[k]); }
            int64_t counts[2] = {0, 0};
            for (size_t ei = elo(); ei < ehi(); ++ei) {
                const ElemOut &o = eo[ei];
                se.add(o.elastic);
                counts[0] += o.candidates;
                if (o.closest != kNone) {
                    st.minimum_gap = std::fmin(st.minimum_gap, o.gap);
                    if (!o.feasible) st.feasible = false;
                    if (o.active) ++counts[1];
                    if (o.has_contact_terms) sc.add(o.contact);
                }
            }
            // One sum all-reduce (four exact sums, two counts) and one
            // min all-reduce (minimum gap, feasibility) per evaluation.
            constexpr int K = ExactSum::kSize;
            std::vector<int64_t> sums(4 * K + 2);
            std::copy(sn.v, sn.v + K, sums.begin());
            std::copy(sk.v, sk.v + K, sums.begin() + K);
            std::copy(se.v, se.v + K, sums.begin() + 2 * K);
            std::copy(sc.v, sc.v + K, sums.begin() + 3 * K);
            sums[4 * K] = counts[0];
            sums[4 * K + 1] = counts[1];
            reduce_(reduce_ctx_, sums.data(), uint32_t(sums.size()), 0);
            std::copy(sums.begin(), sums.begin() + K, sn.v);
            std::copy(sums.begin() + K, sums.begin() + 2 * K, sk.v);
            std::copy(sums.begin() + 2 * K, sums.begin() + 3 * K, se.v);
            std::copy(sums.begin() + 3 * K, sums.begin() + 4 * K, sc.v);
            node_sum = sn.value(); kin = sk.value(); el = se.value(); co = sc.value();
            st.candidates = uint64_t(sums[4 * K]);
            st.active = uint64_t(sums[4 * K + 1]);
            int64_t mins[2] = {order_key(st.minimum_gap), st.feasible ? 1 : 0};
            reduce_(reduce_ctx_, mins, 2, 1);
            st.minimum_gap = from_order_key(mins[0]);
            st.feasible = mins[1] != 0;
        } else {
            for (size_t k = 0; k < n; ++k) { node_sum += node_obj[k]; kin += node_kin[k]; }
            for (size_t ei = 0; ei < ne; ++ei) {
                const ElemOut &o = eo[ei];
                el += o.elastic;
                st.candidates += o.candidates;
                if (o.closest != kNone) {
                    st.minimum_gap = std::fmin(st.minimum_gap, o.gap);
                    if (!o.feasible) st.feasible = false;
                    if (o.active) ++st.active;
                    if (o.has_contact_terms) co += o.contact;
                }
            }
        }
        st.objective = (node_sum + el) + co;
        st.kinetic = kin; st.elastic = el; st.contact = co;
        if (grad) {
            for (size_t ei = elo(); ei < ehi(); ++ei) {
                const ElemOut &o = eo[ei];
                contact_records_[ei] = KhsxContactRecord{o.candidates, o.closest, o.active ? 1u : 0u, 0u, o.gap};
            }
        }
        return st;
    }

    // Gauss-Jordan 6x6 inverse with partial pivoting and a relative
    // diagonal shift (cuda_backend.cu:855-864).
    static bool inverse6(const double *src, double *inverse)
    {
        double a[36];
        for (int i = 0; i < 36; ++i) { a[i] = src[i]; inverse[i] = 0.0; }
        for (int i = 0; i < 6; ++i) inverse[6 * i + i] = 1.0;
        double scale = 0.0;
        for (int i = 0; i < 6; ++i) scale = std::fmax(scale, std::fabs(a[6 * i + i]));
        for (int i = 0; i < 6; ++i) a[6 * i + i] += std::fmax(1.0e-12 * scale, 1.0e-24);
        for (int col = 0; col < 6; ++col) {
            int pivot = col;
            double best = std::fabs(a[6 * col + col]);
            for (int row = col + 1; row < 6; ++row)
                if (std::fabs(a[6 * row + col]) > best) { best = std::fabs(a[6 * row + col]); pivot = row; }
            if (best < 1.0e-30 || !std::isfinite(best)) return false;
            if (pivot != col)
                for (int k = 0; k < 6; ++k) {
                    std::swap(a[6 * col + k], a[6 * pivot + k]);
                    std::swap(inverse[6 * col + k], inverse[6 * pivot + k]);
                }
            const double invp = 1.0 / a[6 * col + col];
            for (int k = 0; k < 6; ++k) { a[6 * col + k] *= invp; inverse[6 * col + k] *= invp; }
            for (int row = 0; row < 6; ++row)
                if (row != col) {
                    const double f = a[6 * row + col];
                    for (int k = 0; k < 6; ++k) { a[6 * row + k] -= f * a[6 * col + k]; inverse[6 * row + k] -= f * inverse[6 * col + k]; }
                }
        }
        return true;
    }

    // Block Thomas per strand (cuda_backend.cu:866-881).
    bool block_solve()
    {
        std::fill(dir_.begin(), dir_.end(), 0.0);
        std::atomic<int> failed{0};
#pragma omp parallel for schedule(dynamic, 16)
        for (long long si = (long long)slo(); si < (long long)shi(); ++si) {
            const Strand st = strands_[size_t(si)];
            const uint32_t begin = st.first + st.fixed_count, end = st.first + st.count;
            if (begin >= end) continue;
            bool ok = true;
            for (uint32_t n = begin; n < end && ok; ++n) {
                double b[36], inv[36], rhs[6];
                for (int i = 0; i < 36; ++i) b[i] = diag_[36 * size_t(n) + i];
                for (int i = 0; i < 6; ++i) rhs[i] = -grad_[6 * size_t(n) + i];
                if (n > begin) {
                    const double *lower = &upper_[36 * size_t(n - 1)];
                    const double *pc = &cprime_[36 * size_t(n - 1)];
                    const double *pd = &dprime_[6 * size_t(n - 1)];
                    for (int r = 0; r < 6; ++r) {
                        for (int c = 0; c < 6; ++c) {
                            double sum = 0;
                            for (int k = 0; k < 6; ++k) sum += lower[6 * k + r] * pc[6 * k + c];
                            b[6 * r + c] -= sum;
                        }
                        double sum = 0;
                        for (int k = 0; k < 6; ++k) sum += lower[6 * k + r] * pd[k];
                        rhs[r] -= sum;
                    }
                }
                if (!inverse6(b, inv)) { failed.store(1); ok = false; break; }
                double *cc = &cprime_[36 * size_t(n)];
                double *cd = &dprime_[6 * size_t(n)];
                if (n + 1 < end) {
                    const double *up = &upper_[36 * size_t(n)];
                    for (int r = 0; r < 6; ++r)
                        for (int c = 0; c < 6; ++c) {
                            double sum = 0;
                            for (int k = 0; k < 6; ++k) sum += inv[6 * r + k] * up[6 * k + c];
                            cc[6 * r + c] = sum;
                        }
                } else for (int i = 0; i < 36; ++i) cc[i] = 0.0;
                for (int r = 0; r < 6; ++r) {
                    double sum = 0;
                    for (int k = 0; k < 6; ++k) sum += inv[6 * r + k] * rhs[k];
                    cd[r] = sum;
                }
            }
            if (!ok) continue;
            for (uint32_t n = end; n-- > begin;) {
                for (int r = 0; r < 6; ++r) {
                    double value = dprime_[6 * size_t(n) + r];
                    if (n + 1 < end)
                        for (int k = 0; k < 6; ++k) value -= cprime_[36 * size_t(n) + 6 * r + k] * dir_[6 * size_t(n + 1) + k];
                    dir_[6 * size_t(n) + r] = value;
                }
            }
        }
        return all_int(failed.load(), 2) == 0;
    }

    static double dotv(const std::vector<double> &a, const std::vector<double> &b)
    {
        double s = 0.0;
        for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
        return s;
    }
    static double nrm2(const std::vector<double> &a) { return std::sqrt(dotv(a, a)); }
    // Global dot product / norm: the serial sum, or over a partition the
    // exact sum of this range's products across the ranks.
    double gdot(const std::vector<double> &a, const std::vector<double> &b)
    {
        if (!part_) return dotv(a, b);
        ExactSum s;
        for (size_t i = 6 * nlo(); i < 6 * nhi(); ++i) s.add(a[i] * b[i]);
        return all_sum(s);
    }
    double gnorm(const std::vector<double> &a) { return std::sqrt(gdot(a, a)); }

    // cuda_backend.cu:815-841
    void build_preconditioner(double dt)
    {
        const KhsHairMaterial &m = material_;
        const double inv = 1.0 / dt, inv2 = inv * inv;
        for (size_t n = nlo(); n < nhi(); ++n) {
            const double p = nodes_[n].mass * (inv2 + m.mass_damping * inv);
            const double r = nodes_[n].rmass * (inv2 + m.mass_damping * inv);
            for (int d = 0; d < 3; ++d) { precond_[6 * n + d] = p; precond_[6 * n + 3 + d] = r; }
        }
        const double area = kPi * m.radius * m.radius;
        const double inertia = kPi * m.radius * m.radius * m.radius * m.radius / 4.0;
        const double G = m.young_modulus / (2.0 * (1.0 + m.poisson_ratio));
        for (size_t ei = elo(); ei < ehi(); ++ei) {
            const Element &e = elements_[ei];
            const double tr = std::fmax(m.young_modulus * area, m.shear_correction * G * area) / e.L0;
            const double rot = m.shear_correction * G * area * e.L0 + std::fmax(m.young_modulus * inertia, 2.0 * G * inertia) / e.L0;
            for (int d = 0; d < 3; ++d) {
                precond_[6 * e.i + d] += tr; precond_[6 * e.j + d] += tr;
                precond_[6 * e.i + 3 + d] += rot; precond_[6 * e.j + 3 + d] += rot;
            }
        }
        for (size_t n = nlo(); n < nhi(); ++n)
            for (int d = 0; d < 6; ++d) precond_[6 * n + d] = nodes_[n].fixed ? 0.0 : 1.0 / std::fmax(precond_[6 * n + d], 1.0e-30);
    }

    // cuda_backend.cu:623-630, 848-853
    void limit_direction()
    {
        double mx = 0.0;
        for (size_t n = nlo(); n < nhi(); ++n) {
            if (nodes_[n].fixed) continue;
            mx = std::fmax(mx, norm(v3(dir_[6 * n], dir_[6 * n + 1], dir_[6 * n + 2])));
        }
        mx = all_max(mx);
        if (mx > trust_radius_) {
            const double scale = trust_radius_ / mx;
            for (size_t i = 6 * nlo(); i < 6 * nhi(); ++i) dir_[i] *= scale;
            ++trust_;
        }
    }

    // cuda_backend.cu:632-638
    void make_steepest()
    {
        for (size_t i = 6 * nlo(); i < 6 * nhi(); ++i) dir_[i] = -grad_[i] * precond_[i];
        for (size_t n = nlo(); n < nhi(); ++n) if (nodes_[n].fixed) for (int d = 0; d < 6; ++d) dir_[6 * n + d] = 0.0;
        limit_direction();
    }

    // cuda_backend.cu:640-648
    bool make_direction()
    {
        const bool ok = block_solve();
        bool used = false;
        if (ok) { const double slope = gdot(grad_, dir_); used = slope < 0 && std::isfinite(slope); }
        if (!used) { ++steepest_; make_steepest(); return false; }
        limit_direction();
        return true;
    }

    // Line-search CCD bound (cuda_backend.cu:989-1000).
    double ccd_limit()
    {
        const KhsHairMaterial &m = material_;
        const double target = m.radius + m.collider_offset + desc_.minimum_gap;
        std::vector<double> lim(E(), 1.0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long ei = (long long)elo(); ei < (long long)ehi(); ++ei) {
            const Element &e = elements_[size_t(ei)];
            if (nodes_[e.i].fixed || !e.contact) continue;
            const V3 p0 = pos(e.i), p1 = pos(e.j);
            const V3 d0 = v3(dir_[6 * e.i], dir_[6 * e.i + 1], dir_[6 * e.i + 2]), d1 = v3(dir_[6 * e.j], dir_[6 * e.j + 1], dir_[6 * e.j + 2]);
            const V3 lo = vmin(vmin(p0, p1), vmin(p0 + d0, p1 + d1)), hi = vmax(vmax(p0, p1), vmax(p0 + d0, p1 + d1));
            double local = 1.0;
            dev_bvh_.query(lo, hi, target, [&](uint32_t ti) {
                const Tri &t = triangles_[ti];
                const double speed = std::fmax(norm(d0), norm(d1));
                if (speed < 1e-30) return;
                double alpha = 0;
                for (int k = 0; k < 80; ++k) {
                    const double dist = closest_segment_triangle_device(p0 + d0 * alpha, p1 + d1 * alpha, d_collider_current_[t.i0],
                                                                        d_collider_current_[t.i1], d_collider_current_[t.i2]).distance;
                    const double clear = dist - target;
                    if (clear <= 0) { local = std::fmin(local, std::fmax(0.0, alpha * 0.9)); return; }
                    const double advance = 0.8 * clear / speed;
                    if (alpha + advance >= 1) return;
                    if (advance < 1e-12) { local = std::fmin(local, alpha); return; }
                    alpha += advance;
                }
                local = std::fmin(local, alpha);
            });
            lim[size_t(ei)] = local;
        }
        double alpha = 1.0;
        for (double l : lim) alpha = std::fmin(alpha, l);
        return all_min(alpha);
    }

    // Partitioned sweep result: the failure with the lowest element index
    // over all ranks, its record sent by the rank that owns the element
    // (every other rank adds zeros to the integer sum of the record's bits).
    bool sweep_result(const std::vector<SweepFailure> &per, SweepFailure &fail_out)
    {
        int64_t first = std::numeric_limits<int64_t>::max();
        for (size_t ei = elo(); ei < ehi(); ++ei)
            if (per[ei].claimed) { first = int64_t(ei); break; }
        first = all_int(first, 1);
        if (first == std::numeric_limits<int64_t>::max()) return true;
        const bool mine = size_t(first) >= elo() && size_t(first) < ehi();
        const SweepFailure &f = per[mine ? size_t(first) : 0];
        const double d[13] = {f.distance, f.required, f.clearance, f.displacement, f.hair_start.x, f.hair_start.y,
                              f.hair_start.z, f.hair_end.x, f.hair_end.y, f.hair_end.z, f.collider_point.x,
                              f.collider_point.y, f.collider_point.z};
        int64_t rec[16] = {};
        if (mine) {
            rec[0] = f.strand; rec[1] = f.element; rec[2] = f.triangle;
            std::memcpy(rec + 3, d, sizeof(d));
        }
        reduce_(reduce_ctx_, rec, 16, 0);
        double o[13];
        std::memcpy(o, rec + 3, sizeof(o));
        fail_out.claimed = true;
        fail_out.strand = uint32_t(rec[0]); fail_out.element = uint32_t(rec[1]); fail_out.triangle = uint32_t(rec[2]);
        fail_out.distance = o[0]; fail_out.required = o[1]; fail_out.clearance = o[2]; fail_out.displacement = o[3];
        fail_out.hair_start = v3(o[4], o[5], o[6]); fail_out.hair_end = v3(o[7], o[8], o[9]);
        fail_out.collider_point = v3(o[10], o[11], o[12]);
        return false;
    }

    // Moving-collider conservative advancement (cuda_backend.cu:966-987).
    bool moving_sweep(SweepFailure &fail_out)
    {
        const KhsHairMaterial &m = material_;
        const double target = m.radius + m.collider_offset + desc_.minimum_gap;
        std::vector<SweepFailure> per(E());
#pragma omp parallel for schedule(dynamic, 64)
        for (long long ei = (long long)elo(); ei < (long long)ehi(); ++ei) {
            const Element &e = elements_[size_t(ei)];
            if (nodes_[e.i].fixed || !e.contact) continue;
            const V3 p0 = pos(e.i), p1 = pos(e.j);
            SweepFailure &f = per[size_t(ei)];
            dev_bvh_.query(vmin(p0, p1), vmax(p0, p1), target, [&](uint32_t ti) {
                const Tri &t = triangles_[ti];
                const V3 oa = d_collider_old_[t.i0], ob = d_collider_old_[t.i1], oc = d_collider_old_[t.i2];
                const V3 da = d_collider_current_[t.i0] - oa, db = d_collider_current_[t.i1] - ob, dc = d_collider_current_[t.i2] - oc;
                const double speed = std::fmax(norm(da), std::fmax(norm(db), norm(dc)));
                if (speed < 1e-30) return;
                double alpha = 0;
                bool end = false;
                Pair pair{};
                V3 a, b, c;
                auto record = [&]() {
                    if (f.claimed) return;
                    f.claimed = true;
                    f.strand = e.strand; f.element = uint32_t(ei); f.triangle = ti;
                    f.distance = pair.distance; f.required = target; f.clearance = pair.distance - target; f.displacement = speed;
                    f.hair_start = p0; f.hair_end = p1;
                    f.collider_point = (a * pair.bary.x + b * pair.bary.y) + c * pair.bary.z;
                };
                for (int k = 0; k < 80; ++k) {
                    a = oa + da * alpha; b = ob + db * alpha; c = oc + dc * alpha;
                    pair = closest_segment_triangle_device(p0, p1, a, b, c);
                    const double clearance = pair.distance - target;
                    if (clearance <= 0) { record(); return; }
                    const double advance = 0.8 * clearance / speed;
                    if (alpha + advance >= 1) { end = true; break; }
                    if (advance < 1e-12) { record(); return; }
                    alpha += advance;
                }
                if (!end) record();
            });
        }
        if (part_) return sweep_result(per, fail_out);
        for (size_t ei = 0; ei < E(); ++ei)
            if (per[ei].claimed) { fail_out = per[ei]; return false; }
        return true;
    }

    // cuda_backend.cu:615-621, 941-964
    void apply_friction(double dt)
    {
        const KhsHairMaterial &m = material_;
        if (!has_collider() || !(m.friction > 0.0)) return;
        struct Imp { bool any = false; double di[3] = {0, 0, 0}, dj[3] = {0, 0, 0}; };
        std::vector<Imp> imp(E());
#pragma omp parallel for schedule(dynamic, 64)
        for (long long ei = (long long)elo(); ei < (long long)ehi(); ++ei) {
            const Element &e = elements_[size_t(ei)];
            if (!e.contact) continue;
            if (nodes_[e.i].fixed && nodes_[e.j].fixed) continue;
            const V3 p0 = pos(e.i), p1 = pos(e.j);
            const double padding = m.radius + m.collider_offset + m.barrier_distance;
            uint32_t closest = kNone;
            Pair pair{1.0e300, 0.0, v3(1, 0, 0)};
            dev_bvh_.query(vmin(p0, p1), vmax(p0, p1), padding, [&](uint32_t ti) {
                const Tri &t = triangles_[ti];
                const Pair c = closest_segment_triangle_device(p0, p1, d_collider_current_[t.i0], d_collider_current_[t.i1], d_collider_current_[t.i2]);
                if (c.distance < pair.distance) { pair = c; closest = ti; }
            });
            if (closest == kNone) continue;
            const double gap = pair.distance - m.radius - m.collider_offset;
            if (!(gap > 0.0 && gap < m.barrier_distance)) continue;
            const Tri &t = triangles_[closest];
            const double w0 = 1.0 - pair.t, w1 = pair.t;
            const V3 hair = p0 * w0 + p1 * w1;
            const V3 body = (d_collider_current_[t.i0] * pair.bary.x + d_collider_current_[t.i1] * pair.bary.y) + d_collider_current_[t.i2] * pair.bary.z;
            const V3 obody = (d_collider_old_[t.i0] * pair.bary.x + d_collider_old_[t.i1] * pair.bary.y) + d_collider_old_[t.i2] * pair.bary.z;
            const V3 normal = div_recip(hair - body, std::fmax(pair.distance, 1.0e-15));
            const V3 v0 = v3(v_[6 * e.i], v_[6 * e.i + 1], v_[6 * e.i + 2]), v1 = v3(v_[6 * e.j], v_[6 * e.j + 1], v_[6 * e.j + 2]);
            const V3 rel = (v0 * w0 + v1 * w1) - div_recip(body - obody, dt);
            const V3 tangent = rel - normal * dot(normal, rel);
            const double ts = norm(tangent);
            if (ts < 1.0e-15) continue;
            double im = 0.0;
            if (!nodes_[e.i].fixed) im += w0 * w0 / std::fmax(nodes_[e.i].mass, 1.0e-30);
            if (!nodes_[e.j].fixed) im += w1 * w1 / std::fmax(nodes_[e.j].mass, 1.0e-30);
            if (!(im > 0.0)) continue;
            const double aa = m.barrier_distance - gap, lg = std::log(gap / m.barrier_distance);
            const double fn = m.contact_stiffness * (aa * aa / gap - 2.0 * aa * lg), required = ts / im;
            const double mag = std::fmin(required, m.friction * fn * dt), smooth = m.friction_smoothing / dt;
            const V3 impulse = tangent * (-mag / std::fmax(std::sqrt(ts * ts + smooth * smooth), 1.0e-30));
            Imp &o = imp[size_t(ei)];
            o.any = true;
            if (!nodes_[e.i].fixed) { const double s = w0 / std::fmax(nodes_[e.i].mass, 1.0e-30); o.di[0] = impulse.x * s; o.di[1] = impulse.y * s; o.di[2] = impulse.z * s; }
            if (!nodes_[e.j].fixed) { const double s = w1 / std::fmax(nodes_[e.j].mass, 1.0e-30); o.dj[0] = impulse.x * s; o.dj[1] = impulse.y * s; o.dj[2] = impulse.z * s; }
        }
        std::vector<double> dv(dof(), 0.0);
        for (size_t ei = elo(); ei < ehi(); ++ei) {
            const Imp &o = imp[ei];
            if (!o.any) continue;
            const Element &e = elements_[ei];
            for (int d = 0; d < 3; ++d) { dv[6 * e.i + d] += o.di[d]; dv[6 * e.j + d] += o.dj[d]; }
        }
        for (size_t i = 6 * nlo(); i < 6 * nhi(); ++i) v_[i] += dv[i];
    }

    void update_velocity(double dt)
    {
        const double inv_dt = 1.0 / dt;
        for (size_t n = nlo(); n < nhi(); ++n) {
            if (nodes_[n].fixed) continue;
            for (int d = 0; d < 6; ++d) v_[6 * n + d] = (q_[6 * n + d] - old_q_[6 * n + d]) * inv_dt;
        }
    }

    // Gauss-Newton loop (cuda_backend.cu:650-688).
    KhsResult optimize_substep(double dt, KhsxSubstepRecord &rec)
    {
        build_preconditioner(dt);
        Stats current = evaluate(true, dt);
        if (!current.feasible) return fail(KHS_ERROR_NOT_CONVERGED, "state is outside the barrier feasible region");
        const double initial = gnorm(grad_);
        step_stats_.initial_residual_norm = std::fmax(step_stats_.initial_residual_norm, initial);
        for (uint32_t it = 0; it <= desc_.newton_iterations; ++it) {
            progress_iteration_.store(it);
            if (all_int(cancel_.load() ? 1 : 0, 2)) return fail(KHS_ERROR_INVALID_STATE, "solve cancelled");
            const double residual = gnorm(grad_);
            const double relative = residual / std::fmax(initial, 1e-30);
            step_stats_.final_residual_norm = residual;
            step_stats_.relative_residual_norm = relative;
            step_stats_.minimum_gap = std::fmin(step_stats_.minimum_gap, current.minimum_gap);
            step_stats_.contact_candidate_count += current.candidates;
            step_stats_.active_contact_count += current.active;
            step_stats_.kinetic_energy = current.kinetic;
            step_stats_.elastic_energy = current.elastic;
            step_stats_.contact_energy = current.contact;
            step_stats_.friction_energy = current.friction;
            rec.final_residual_norm = residual;
            rec.minimum_gap = std::fmin(rec.minimum_gap, current.minimum_gap);
            rec.contact_candidates += current.candidates;
            rec.active_contacts += current.active;
            const double floor = 1.0e-5 * std::sqrt(double(dof()));
            if (residual <= std::fmax(desc_.absolute_tolerance, floor) || relative <= std::fmax(desc_.relative_tolerance, 1.0e-4)) {
                update_velocity(dt);
                return KHS_OK;
            }
            if (it == desc_.newton_iterations) break;
            progress_phase_.store(KHS_PHASE_LINEAR_SOLVE);
            bool block_direction = make_direction();
            ++step_stats_.linear_solves;
            base_q_ = q_;
            bool accepted = false;
            double alpha = 1.0;
            for (int attempt = 0; attempt < 2; ++attempt) {
                const double slope = gdot(grad_, dir_);
                alpha = 1.0;
                if (has_collider()) {
                    progress_phase_.store(KHS_PHASE_CCD);
                    alpha = ccd_limit();
                    if (alpha < 1.0) alpha *= 0.9;
                    step_stats_.ccd_step_limit = std::fmin(step_stats_.ccd_step_limit, alpha);
                }
                accepted = false;
                progress_phase_.store(KHS_PHASE_LINE_SEARCH);
                if (alpha >= desc_.minimum_line_search_step)
                    for (uint32_t s = 0; s < desc_.line_search_iterations; ++s) {
                        for (size_t i = 6 * nlo(); i < 6 * nhi(); ++i) q_[i] = base_q_[i] + alpha * dir_[i];
                        const Stats trial = evaluate(false, dt);
                        ++step_stats_.line_search_evaluations;
                        ++rec.line_search_evaluations;
                        if (trial.feasible && std::isfinite(trial.objective) && trial.objective <= current.objective + 1e-4 * alpha * slope) {
                            accepted = true;
                            break;
                        }
                        alpha *= 0.5;
                        if (alpha < desc_.minimum_line_search_step) break;
                    }
                if (accepted) break;
                if (!block_direction) break;
                q_ = base_q_;
                ++steepest_;
                make_steepest();
                block_direction = false;
            }
            if (!accepted) { q_ = base_q_; return fail(KHS_ERROR_NOT_CONVERGED, "Gauss-Newton line search failed"); }
            current = evaluate(true, dt);
            const double dnorm = gnorm(dir_);
            step_stats_.increment_norm = alpha * dnorm;
            step_stats_.accepted_step_length = alpha;
            ++step_stats_.newton_iterations;
            ++rec.newton_iterations;
            progress_phase_.store(KHS_PHASE_ASSEMBLING);
            const double rms = step_stats_.increment_norm / std::sqrt(double(dof()));
            if (rms <= 2.0 * desc_.increment_tolerance) { update_velocity(dt); return KHS_OK; }
        }
        update_velocity(dt);
        return KHS_OK;
    }

    void set_failure_context(uint32_t kind, uint32_t frame, uint32_t sub, uint32_t attempted, uint32_t maximum, uint32_t attempts)
    {
        failure_.kind = kind; failure_.frame_index = frame; failure_.substep = sub;
        failure_.requested_substeps = desc_.substeps; failure_.attempted_substeps = attempted;
        failure_.maximum_substeps = maximum; failure_.adaptive_attempt_count = attempts;
    }

    // Frame driver with adaptive substep doubling (cuda_backend.cu:690-723).
    KhsResult run_frame(double frame_dt, const V3 *root_a, const V3 *rot_a, const V3 *root_b, const V3 *rot_b,
                        const V3 *col_a, const V3 *col_b, uint32_t frame, uint32_t frame_count)
    {
        const auto t0 = std::chrono::steady_clock::now();
        if (!(frame_dt > 0 && std::isfinite(frame_dt))) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid time step");
        cancel_.store(false);
        clear_failure();
        frame_clock_ = std::chrono::steady_clock::now();
        progress_frame_.store(frame); progress_frame_count_.store(frame_count); progress_iteration_.store(0);
        snap_q_ = q_; snap_v_ = v_;
        // Copy the interpolation endpoints first: for khsStep col_a aliases
        // the frame-start buffer which this function overwrites.
        const size_t nv = d_collider_current_.size();
        std::vector<V3> ca(col_a ? col_a : nullptr, col_a ? col_a + nv : nullptr), cb(col_b ? col_b : nullptr, col_b ? col_b + nv : nullptr);
        uint32_t substeps = desc_.substeps;
        const uint32_t maximum = has_collider() ? desc_.maximum_substeps : desc_.substeps;
        uint32_t attempts = 0;
        for (;;) {
            ++attempts;
            q_ = snap_q_; v_ = snap_v_;
            clear_failure();
            error_.clear();
            records_.clear();
            progress_phase_.store(KHS_PHASE_ASSEMBLING);
            progress_substep_count_.store(substeps);
            progress_iteration_.store(0);
            step_stats_ = {};
            step_stats_.struct_size = sizeof(step_stats_);
            step_stats_.substeps = substeps;
            step_stats_.minimum_gap = std::numeric_limits<double>::infinity();
            step_stats_.ccd_step_limit = 1.0;
            if (has_collider()) { d_collider_current_ = ca; d_collider_frame_start_ = ca; }
            const double dt = frame_dt / substeps;
            bool crossed = false;
            KhsResult result = KHS_OK;
            for (uint32_t sub = 1; sub <= substeps; ++sub) {
                if (g_substep_limit && sub > g_substep_limit) break;
                if (substep_limit_ && sub > substep_limit_) break;
                progress_substep_.store(sub);
                progress_iteration_.store(0);
                KhsxSubstepRecord rec{};
                rec.struct_size = sizeof(rec);
                rec.substep = sub;
                rec.minimum_gap = std::numeric_limits<double>::infinity();
                steepest_ = 0;
                trust_ = 0;
                old_q_ = q_;
                const double f = double(sub) / substeps;
                for (size_t n = nlo(); n < nhi(); ++n) {
                    if (!nodes_[n].fixed) continue;
                    const V3 p = root_a[n] * (1.0 - f) + root_b[n] * f, r = rot_a[n] * (1.0 - f) + rot_b[n] * f;
                    const double vals[6] = {p.x, p.y, p.z, r.x, r.y, r.z};
                    for (int d = 0; d < 6; ++d) { q_[6 * n + d] = vals[d]; v_[6 * n + d] = (vals[d] - old_q_[6 * n + d]) / dt; }
                }
                if (has_collider()) {
                    d_collider_old_ = d_collider_current_;
                    for (size_t i = 0; i < nv; ++i) d_collider_current_[i] = ca[i] * (1.0 - f) + cb[i] * f;
                    dev_bvh_.refit(triangles_, d_collider_current_, d_collider_old_, true);
                    progress_phase_.store(KHS_PHASE_CCD);
                    SweepFailure sf;
                    if (!moving_sweep(sf)) {
                        set_failure_context(KHS_FAILURE_MOVING_COLLIDER_SWEEP, frame, sub, substeps, maximum, attempts);
                        if (sf.claimed) {
                            failure_.strand_index = sf.strand; failure_.element_index = sf.element; failure_.collider_triangle_index = sf.triangle;
                            failure_.distance = sf.distance; failure_.required_distance = sf.required; failure_.clearance = sf.clearance;
                            failure_.collider_substep_displacement = sf.displacement;
                            failure_.collider_frame_displacement = sf.displacement * substeps;
                            failure_.hair_start = {sf.hair_start.x, sf.hair_start.y, sf.hair_start.z};
                            failure_.hair_end = {sf.hair_end.x, sf.hair_end.y, sf.hair_end.z};
                            failure_.collider_point = {sf.collider_point.x, sf.collider_point.y, sf.collider_point.z};
                        }
                        crossed = true;
                        break;
                    }
                    dev_bvh_.refit(triangles_, d_collider_current_, d_collider_old_, false);
                }
                progress_phase_.store(KHS_PHASE_ASSEMBLING);
                result = optimize_substep(dt, rec);
                rec.steepest_fallbacks = steepest_;
                rec.trust_scalings = trust_;
                records_.push_back(rec);
                if (result != KHS_OK) {
                    if (!cancel_.load()) {
                        const uint32_t kind = error_.find("outside the barrier") != std::string::npos ? KHS_FAILURE_BARRIER_INFEASIBLE : KHS_FAILURE_NONLINEAR_SOLVE;
                        set_failure_context(kind, frame, sub, substeps, maximum, attempts);
                    }
                    break;
                }
                apply_friction(dt);
                ++step_stats_.converged_substeps;
            }
            if (!crossed && result == KHS_OK) break;
            q_ = snap_q_; v_ = snap_v_;
            if (cancel_.load()) return result;
            if (substeps >= maximum) {
                if (crossed) return fail(KHS_ERROR_NOT_CONVERGED, "animated collider crossed hair after adaptive substepping");
                return result;
            }
            substeps = std::min(maximum, substeps * 2);
        }
        if (!animation_ready_) {
            root_current_x_ = root_pending_x_; root_current_r_ = root_pending_r_;
            if (has_collider()) d_collider_frame_start_ = d_collider_pending_;
        }
        clear_failure();
        step_stats_.phase = KHS_PHASE_FINISHED;
        progress_phase_.store(KHS_PHASE_FINISHED);
        last_frame_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        error_.clear();
        return KHS_OK;
    }

    // ---- members ----
    KhsSolverDesc desc_{};
    KhsHairMaterial material_{};
    bool has_hair_ = false, has_collider_ = false, built_ = false, closed_ = false;
    std::vector<V3> input_points_;
    std::vector<uint32_t> input_offsets_, mapping_;
    std::vector<Node> nodes_;
    std::vector<Element> elements_;
    std::vector<std::vector<uint32_t>> strand_nodes_;
    std::vector<Strand> strands_;
    uint64_t free_dofs_ = 0;
    std::vector<V3> root_x_, root_r_;
    std::vector<V3> collider_pending_, collider_current_;
    std::vector<Tri> triangles_;
    HostBvh host_bvh_;
    uint32_t excluded_ = 0, boundary_ = 0, nonmanifold_ = 0, inconsistent_ = 0, inverted_ = 0;
    uint32_t merged_ = 0, vext_strands_ = 0, vext_nodes_ = 0;
    double vext_length_ = 0.0;
    KhsBuildStats build_stats_{};
    KhsStepStats step_stats_{};

    std::vector<double> q_, old_q_, snap_q_, v_, snap_v_, base_q_, grad_, dir_, precond_;
    std::vector<double> diag_, upper_, cprime_, dprime_;
    std::vector<V3> root_current_x_, root_current_r_, root_pending_x_, root_pending_r_;
    std::vector<V3> d_collider_current_, d_collider_old_, d_collider_frame_start_, d_collider_pending_;
    DeviceBvh dev_bvh_;
    std::vector<ElemOut> elem_out_;
    std::vector<KhsxContactRecord> contact_records_;
    std::vector<KhsxSubstepRecord> records_;
    uint32_t substep_limit_ = 0;  // khsxSetSubstepLimit (0: whole frames)
    // Strand partition (set_partition): the node, element and strand ranges
    // stepped here, and the all-reduce that combines the global scalars.
    bool part_ = false;
    size_t n_lo_ = 0, n_hi_ = 0, e_lo_ = 0, e_hi_ = 0, s_lo_ = 0, s_hi_ = 0;
    ReduceFn reduce_ = nullptr;
    void *reduce_ctx_ = nullptr;
    size_t nlo() const { return part_ ? n_lo_ : 0; }
    size_t nhi() const { return part_ ? n_hi_ : N(); }
    size_t elo() const { return part_ ? e_lo_ : 0; }
    size_t ehi() const { return part_ ? e_hi_ : E(); }
    size_t slo() const { return part_ ? s_lo_ : 0; }
    size_t shi() const { return part_ ? s_hi_ : strands_.size(); }
    int64_t all_int(int64_t x, int op)
    {
        if (part_) reduce_(reduce_ctx_, &x, 1, op);
        return x;
    }
    double all_min(double x)
    {
        if (!part_) return x;
        int64_t k = order_key(x);
        reduce_(reduce_ctx_, &k, 1, 1);
        return from_order_key(k);
    }
    double all_max(double x)
    {
        if (!part_) return x;
        int64_t k = order_key(x);
        reduce_(reduce_ctx_, &k, 1, 2);
        return from_order_key(k);
    }
    double all_sum(ExactSum &s)
    {
        reduce_(reduce_ctx_, s.v, ExactSum::kSize, 0);
        return s.value();
    }
    uint32_t steepest_ = 0, trust_ = 0;  // per substep: steepest fallbacks, trust-radius scalings
    double max_rest_length_ = 0.0, trust_radius_ = 0.0, last_frame_ms_ = 0.0;
    bool animation_ready_ = false;
    uint32_t anim_frames_ = 0, current_frame_ = 0;
    std::vector<V3> anim_root_x_, anim_root_r_, anim_collider_;
    std::vector<bool> root_set_, collider_set_;
    KhsFailureDiagnostics failure_{};
    std::atomic<bool> cancel_{false};
    std::atomic<uint32_t> progress_phase_{KHS_PHASE_IDLE}, progress_frame_{0}, progress_frame_count_{0},
        progress_substep_{0}, progress_substep_count_{0}, progress_iteration_{0};
    std::chrono::steady_clock::time_point frame_clock_ = std::chrono::steady_clock::now();
};

}  // namespace khs_oracle

// ---------------------------------------------------------------------------
// C ABI (api.cpp:9-306).

struct KhsSolver {
    explicit KhsSolver(const KhsSolverDesc &d) : impl(d) {}
    khs_oracle::Solver impl;
};

namespace {

template<class F> KhsResult guarded(KhsSolver *s, F &&f)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    try { return f(); }
    catch (const std::bad_alloc &) { s->impl.error_ = "out of memory"; return KHS_ERROR_OUT_OF_MEMORY; }
    catch (const std::exception &e) { s->impl.error_ = std::string("internal exception: ") + e.what(); return KHS_ERROR_INTERNAL; }
    catch (...) { s->impl.error_ = "unknown internal exception"; return KHS_ERROR_INTERNAL; }
}

bool valid_desc(const KhsSolverDesc *d)
{
    return d && d->struct_size >= sizeof(KhsSolverDesc) && d->substeps > 0 && d->maximum_substeps >= d->substeps &&
           d->newton_iterations > 0 && d->line_search_iterations > 0 && d->absolute_tolerance > 0.0 &&
           d->relative_tolerance > 0.0 && d->increment_tolerance > 0.0 && d->minimum_line_search_step > 0.0 &&
           d->minimum_gap > 0.0 && d->maximum_element_length > 0.0 && d->minimum_dynamic_length >= 0.0 &&
           std::isfinite(d->minimum_dynamic_length) && d->fixed_root_nodes > 0;
}

bool valid_material(const KhsHairMaterial *m)
{
    return m && m->struct_size >= sizeof(KhsHairMaterial) && m->density > 0.0 && m->radius > 0.0 &&
           m->young_modulus > 0.0 && m->poisson_ratio > -1.0 && m->poisson_ratio < 0.5 && m->shear_correction > 0.0 &&
           m->mass_damping >= 0.0 && m->contact_stiffness > 0.0 && m->barrier_distance > 0.0 && m->friction >= 0.0 &&
           m->friction_smoothing > 0.0 && m->collider_offset >= 0.0;
}

}  // namespace

extern "C" {

KHS_API uint32_t khsGetAbiVersion(void) { return KHS_ABI_VERSION; }

KHS_API KhsResult khsGetGpuInfo(KhsGpuInfo *info)
{
    if (!info || info->struct_size < sizeof(KhsGpuInfo)) return KHS_ERROR_INVALID_ARGUMENT;
    KhsGpuInfo r{};
    r.struct_size = sizeof(r);
    std::strncpy(r.device_name, "CPU oracle", sizeof(r.device_name) - 1);
    *info = r;
    return KHS_ERROR_INVALID_STATE;
}

KHS_API void khsDefaultSolverDesc(KhsSolverDesc *d)
{
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->struct_size = sizeof(*d);
    d->gravity = {0.0, 0.0, -9.81};
    d->substeps = 8; d->maximum_substeps = 32; d->newton_iterations = 24; d->line_search_iterations = 20;
    d->absolute_tolerance = 1.0e-8; d->relative_tolerance = 1.0e-5; d->increment_tolerance = 1.0e-8;
    d->minimum_line_search_step = 1.0e-9; d->minimum_gap = 1.0e-7; d->maximum_element_length = 0.01;
    d->minimum_dynamic_length = 0.0; d->fixed_root_nodes = 2; d->thread_count = 0;
}

KHS_API void khsDefaultHairMaterial(KhsHairMaterial *m)
{
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->struct_size = sizeof(*m);
    m->density = 1300.0; m->radius = 4.0e-5; m->young_modulus = 4.0e9; m->poisson_ratio = 0.38;
    m->shear_correction = 0.9; m->mass_damping = 8.0; m->contact_stiffness = 1.0e4; m->barrier_distance = 2.0e-4;
    m->friction = 0.35; m->friction_smoothing = 1.0e-6; m->collider_offset = 0.0;
}

KHS_API KhsSolver *khsCreate(const KhsSolverDesc *d)
{
    if (!valid_desc(d)) return nullptr;
    try { return new KhsSolver(*d); } catch (...) { return nullptr; }
}

KHS_API void khsDestroy(KhsSolver *s) { delete s; }

KHS_API KhsResult khsSetHairCurves(KhsSolver *s, const KhsVec3 *p, uint32_t n, const uint32_t *o, uint32_t sc, const KhsHairMaterial *m)
{
    if (!m || m->struct_size < sizeof(KhsHairMaterial)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { return s->impl.set_hair(p, n, o, sc, *m); });
}
KHS_API KhsResult khsSetColliderMesh(KhsSolver *s, const KhsVec3 *v, uint32_t nv, const KhsTriangle *t, uint32_t nt)
{ return guarded(s, [&] { return s->impl.set_collider(v, nv, t, nt); }); }
KHS_API KhsResult khsBuild(KhsSolver *s) { return guarded(s, [&] { return s->impl.build(); }); }
KHS_API KhsResult khsUpdateRuntimeParameters(KhsSolver *s, const KhsSolverDesc *d, const KhsHairMaterial *m)
{
    if (!valid_desc(d) || !valid_material(m)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { return s->impl.update_runtime(*d, *m); });
}
KHS_API KhsResult khsUpdateColliderVertices(KhsSolver *s, const KhsVec3 *v, uint32_t n) { return guarded(s, [&] { return s->impl.update_collider(v, n); }); }
KHS_API KhsResult khsUpdateRootTargets(KhsSolver *s, const KhsVec3 *p, uint32_t n) { return guarded(s, [&] { return s->impl.update_roots(p, n); }); }
KHS_API KhsResult khsStep(KhsSolver *s, double dt) { return guarded(s, [&] { return s->impl.step(dt); }); }
KHS_API KhsResult khsAllocateAnimation(KhsSolver *s, uint32_t f) { return guarded(s, [&] { return s->impl.allocate_animation(f); }); }
KHS_API KhsResult khsSetRootAnimationFrame(KhsSolver *s, uint32_t f, const KhsVec3 *p, uint32_t n) { return guarded(s, [&] { return s->impl.set_root_frame(f, p, n); }); }
KHS_API KhsResult khsSetColliderAnimationFrame(KhsSolver *s, uint32_t f, const KhsVec3 *v, uint32_t n) { return guarded(s, [&] { return s->impl.set_collider_frame(f, v, n); }); }
KHS_API KhsResult khsFinalizeAnimation(KhsSolver *s) { return guarded(s, [&] { return s->impl.finalize_animation(); }); }
KHS_API KhsResult khsStepAnimationFrame(KhsSolver *s, uint32_t f, double dt) { return guarded(s, [&] { return s->impl.step_animation_frame(f, dt); }); }
KHS_API uint64_t khsGetAnimationCheckpointSize(const KhsSolver *s) { return s ? s->impl.checkpoint_size() : 0; }
KHS_API KhsResult khsSaveAnimationCheckpoint(KhsSolver *s, void *d, uint64_t c) { return guarded(s, [&] { return s->impl.save_checkpoint(d, c); }); }
KHS_API KhsResult khsRestoreAnimationCheckpoint(KhsSolver *s, const void *d, uint64_t n) { return guarded(s, [&] { return s->impl.restore_checkpoint(d, n); }); }
KHS_API uint32_t khsGetOriginalPointCount(const KhsSolver *s) { return s ? s->impl.original_count() : 0; }
KHS_API uint32_t khsGetInternalNodeCount(const KhsSolver *s) { return s ? s->impl.internal_count() : 0; }
KHS_API KhsResult khsCopyOriginalPositions(const KhsSolver *s, KhsVec3 *p, uint32_t c) { return s ? s->impl.copy_original(p, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsCopyInternalPositions(const KhsSolver *s, KhsVec3 *p, uint32_t c) { return s ? s->impl.copy_internal(p, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsCopyOriginalToInternalMap(const KhsSolver *s, uint32_t *i, uint32_t c) { return s ? s->impl.copy_mapping(i, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsGetBuildStats(const KhsSolver *s, KhsBuildStats *b) { return s ? s->impl.build_stats(b) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsGetLastStepStats(const KhsSolver *s, KhsStepStats *b) { return s ? s->impl.get_step_stats(b) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsGetGpuStats(const KhsSolver *s, KhsGpuStats *g) { return s ? s->impl.gpu_stats(g) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsGetProgress(const KhsSolver *s, KhsProgress *p) { return s ? s->impl.progress(p) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsGetFailureDiagnostics(const KhsSolver *s, KhsFailureDiagnostics *d) { return s ? s->impl.failure(d) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsRequestCancel(KhsSolver *s) { return guarded(s, [&] { return s->impl.request_cancel(); }); }
KHS_API const char *khsGetLastError(const KhsSolver *s)
{
    static const char *invalid = "no solver";
    return s ? s->impl.error_.c_str() : invalid;
}

KHS_API KhsResult khsxSetSolveMode(KhsSolver *s, uint32_t mode) { return s && mode <= 2 ? KHS_OK : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API uint32_t khsxGetSolveMode(const KhsSolver *) { return 0; }
KHS_API KhsResult khsxSetSubstepLimit(KhsSolver *s, uint32_t n)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    s->impl.set_substep_limit(n);
    return KHS_OK;
}
KHS_API KhsResult khsxCopyState(const KhsSolver *s, double *q, double *v, uint64_t cap) { return s ? s->impl.copy_state(q, v, cap) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API uint32_t khsxGetSubstepRecordCount(const KhsSolver *s) { return s ? s->impl.record_count() : 0; }
KHS_API KhsResult khsxCopySubstepRecords(const KhsSolver *s, KhsxSubstepRecord *r, uint32_t c) { return s ? s->impl.copy_records(r, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsxCopyContactRecords(const KhsSolver *s, KhsxContactRecord *r, uint32_t c) { return s ? s->impl.copy_contacts(r, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsxQueryContacts(KhsSolver *s, const double *q, uint64_t n, KhsxContactRecord *r, uint32_t c) { return s ? s->impl.query_contacts(q, n, r, c) : KHS_ERROR_INVALID_ARGUMENT; }
KHS_API KhsResult khsxComputeRootTargets(KhsSolver *s, const KhsVec3 *p, uint32_t n, KhsVec3 *pos, KhsVec3 *rot, uint32_t cap)
{ return guarded(s, [&] { return s->impl.roots_to_host(p, n, pos, rot, cap); }); }

// Oracle-only test hook (see Solver::export_system).
KHS_API void khsOracleExportSystem(const KhsSolver *s, double *diag, double *upper, double *grad, uint32_t *strands)
{
    if (s) s->impl.export_system(diag, upper, grad, strands);
}

// Oracle-only test hooks (see Solver::model_sizes / export_model): the built
// model as the reference's CUDA backend takes it.
KHS_API void khsOracleModelSizes(const KhsSolver *s, uint32_t *sizes)
{
    if (s && sizes) s->impl.model_sizes(sizes);
}
KHS_API void khsOracleExportModel(const KhsSolver *s, double *node_f, uint32_t *node_u, double *elem_f, uint32_t *elem_u,
                                  uint32_t *strand_u, uint32_t *mapping, double *collider, uint32_t *tris)
{
    if (s) s->impl.export_model(node_f, node_u, elem_f, elem_u, strand_u, mapping, collider, tris);
}

// Oracle-only test hook (see Solver::set_partition): step only strands
// [s0, s1) and combine the global scalars through `reduce`.
KHS_API KhsResult khsOracleSetPartition(KhsSolver *s, uint32_t s0, uint32_t s1, khs_oracle::ReduceFn reduce, void *ctx)
{
    return s ? s->impl.set_partition(s0, s1, reduce, ctx) : KHS_ERROR_INVALID_ARGUMENT;
}

// Oracle-only: stop every frame after n substeps (0 = whole frames).
KHS_API void khsOracleSetSubstepLimit(uint32_t n) { khs_oracle::g_substep_limit = n; }

// Oracle-only: thread count used by the OpenMP loops (0 = library default).
KHS_API int khsOracleSetThreads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
