// Host-side rod model builder (see khs_model.hpp).
#include "khs_model.hpp"
#include "khs_device_math.cuh"

#include <algorithm>
#include <exception>
#include <limits>
#include <numeric>
#include <sstream>
#include <thread>
#include <unordered_map>

namespace khs {
namespace {

constexpr double kPiHost = 3.14159265358979323846;

// Host threads for the build-time passes (the machine's cores, at most 32).
inline unsigned host_threads()
{
    const unsigned n = std::thread::hardware_concurrency();
    return std::max(1u, std::min(n ? n : 1u, 32u));
}

// f(begin, end, chunk) over contiguous chunks of [0, count), one per host
// thread (the caller runs the first); exceptions reach the caller.
template<class F> void parallel_chunks(size_t count, unsigned chunks, F &&f)
{
    chunks = unsigned(std::max<size_t>(1, std::min<size_t>(chunks, count)));
    std::vector<std::exception_ptr> errors(chunks);
    auto run = [&](unsigned c) {
        try {
            f(count * c / chunks, count * (c + 1) / chunks, c);
        } catch (...) {
            errors[c] = std::current_exception();
        }
    };
    std::vector<std::thread> pool;
    for (unsigned c = 1; c < chunks; ++c) pool.emplace_back(run, c);
    run(0);
    for (std::thread &t : pool) t.join();
    for (const std::exception_ptr &e : errors)
        if (e) std::rethrow_exception(e);
}

inline Vec mk(double x, double y, double z) { Vec v; v.x = x; v.y = y; v.z = z; return v; }
inline Vec add(Vec a, Vec b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec sub(Vec a, Vec b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec mul(Vec a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
inline Vec divs(Vec a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
inline double dot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec cross(Vec a, Vec b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline double sq(Vec a) { return dot(a, a); }
inline double len(Vec a) { return std::sqrt(sq(a)); }
inline double comp(Vec a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
inline Vec vmin(Vec a, Vec b) { return mk(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline Vec vmax(Vec a, Vec b) { return mk(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline bool finite(Vec a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }
// Unit vector; a zero vector stays zero (Eigen normalized()).
inline Vec unit(Vec a)
{
    const double n2 = sq(a);
    return n2 > 0.0 ? divs(a, std::sqrt(n2)) : a;
}
// (1 - t) a + t b with the reference's evaluation order.
inline Vec lerp(Vec a, Vec b, double t) { return add(mul(a, 1.0 - t), mul(b, t)); }

inline Vec column(const Mat &m, int c) { return mk(m.m[c], m.m[3 + c], m.m[6 + c]); }
inline Mat from_columns(Vec a, Vec b, Vec c)
{
    Mat r;
    r.m[0] = a.x; r.m[1] = b.x; r.m[2] = c.x;
    r.m[3] = a.y; r.m[4] = b.y; r.m[5] = c.y;
    r.m[6] = a.z; r.m[7] = b.z; r.m[8] = c.z;
    return r;
}
inline Mat transpose_times(const Mat &a, const Mat &b)  // a^T * b
{
    Mat r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = (a.m[i] * b.m[j] + a.m[3 + i] * b.m[3 + j]) + a.m[6 + i] * b.m[6 + j];
    return r;
}

// Regularised Cayley rotation vector (math.hpp:14-24).
Vec cayley(const Mat &q)
{
    const Vec v = mk((q.m[7] - q.m[5]) * 0.5, (q.m[2] - q.m[6]) * 0.5, (q.m[3] - q.m[1]) * 0.5);
    const double c = (((q.m[0] + q.m[4]) + q.m[8]) - 1.0) * 0.5;
    const double s = 2.0 / (1.0 + c + 1.0e-12);
    return mk(s * v.x, s * v.y, s * v.z);
}

// Root and reference frames (math.hpp:26-58, solver.cpp:19-26) use the
// same functions as the device root-target kernels (khs_device_math.cuh,
// compiled here for the host), so the two round identically.
inline dm::V to_dm(Vec a) { return dm::v(a.x, a.y, a.z); }
inline Vec from_dm(dm::V a) { return mk(a.x, a.y, a.z); }
inline dm::M to_dm(const Mat &a)
{
    dm::M r;
    for (int k = 0; k < 9; ++k) r.m[k] = a.m[k];
    return r;
}
inline Mat from_dm(const dm::M &a)
{
    Mat r;
    for (int k = 0; k < 9; ++k) r.m[k] = a.m[k];
    return r;
}

// Frame with the tangent as third column, first column from the hint.
Mat tangent_frame(Vec tangent, Vec hint) { return from_dm(dm::frame_from_tangent(to_dm(tangent), to_dm(hint))); }

// Minimal rotation of a director between consecutive tangents.
Vec transport(Vec director, Vec from, Vec to) { return from_dm(dm::parallel_transport(to_dm(director), to_dm(from), to_dm(to))); }

// Rotation vector of a rotation matrix.
Vec rotation_vector(const Mat &r) { return from_dm(dm::rotation_vector(to_dm(r))); }

// Unit central-difference tangents along one strand (solver.cpp:324-331).
bool strand_tangents(const std::vector<Vec> &x, uint32_t first, uint32_t count, std::vector<Vec> &t, bool reject_zero)
{
    t.resize(count);
    for (uint32_t k = 0; k < count; ++k) {
        Vec d;
        if (k == 0) d = sub(x[first + 1], x[first]);
        else if (k + 1 == count) d = sub(x[first + k], x[first + k - 1]);
        else d = sub(x[first + k + 1], x[first + k - 1]);
        if (reject_zero && sq(d) < 1.0e-24) return false;
        t[k] = unit(d);
    }
    return true;
}

// ---- BVH construction (two flavours of the same median split) ----------

struct TreeNode {
    Vec lo, hi;
    uint32_t begin = 0, count = 0;
    int left = -1, right = -1;
};

struct TreeBuilder {
    const std::vector<Vec> &v;
    const std::vector<uint32_t> &tri;
    bool device_flavour;
    std::vector<TreeNode> nodes;
    std::vector<uint32_t> order;

    Vec vert(uint32_t t, int c) const { return v[tri[3 * t + c]]; }
    // Device flavour multiplies by 1/3 (cuda_backend.cu:40,303); host
    // flavour divides each component by 3 (solver.cpp:65,78-79).
    double centroid(uint32_t t, int axis) const
    {
        const Vec s = add(add(vert(t, 0), vert(t, 1)), vert(t, 2));
        return device_flavour ? comp(s, axis) * (1.0 / 3.0) : comp(s, axis) / 3.0;
    }
    // Builds [begin, end) of `order` into `out` (root first, then the left
    // subtree, then the right one) and returns the root's index there.  Up to
    // `spawn` levels down, the right half is built on another thread into a
    // vector of its own and appended after the left one, which gives the same
    // nodes in the same order as the one-thread build: the two halves touch
    // disjoint ranges of `order`.
    int build(std::vector<TreeNode> &out, uint32_t begin, uint32_t end, int spawn)
    {
        std::vector<TreeNode> &nodes = out;
        const int idx = int(nodes.size());
        nodes.push_back({});
        const double big = device_flavour ? 1e300 : std::numeric_limits<double>::infinity();
        Vec lo = mk(big, big, big), hi = mk(-big, -big, -big), cl = lo, cu = hi;
        for (uint32_t k = begin; k < end; ++k) {
            const uint32_t t = order[k];
            const Vec a = vert(t, 0), b = vert(t, 1), c = vert(t, 2);
            lo = vmin(lo, vmin(a, vmin(b, c)));
            hi = vmax(hi, vmax(a, vmax(b, c)));
            const Vec s = add(add(a, b), c);
            const Vec ce = device_flavour ? mul(s, 1.0 / 3.0) : divs(s, 3.0);
            cl = vmin(cl, ce);
            cu = vmax(cu, ce);
        }
        nodes[idx].lo = lo; nodes[idx].hi = hi;
        nodes[idx].begin = begin; nodes[idx].count = end - begin;
        if (end - begin <= 8) return idx;
        const Vec span = sub(cu, cl);
        int axis;
        if (device_flavour) axis = span.y > span.x ? (span.z > span.y ? 2 : 1) : (span.z > span.x ? 2 : 0);
        else { axis = 0; if (span.y > comp(span, axis)) axis = 1; if (span.z > comp(span, axis)) axis = 2; }
        const uint32_t mid = begin + (end - begin) / 2;
        std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + end,
                         [&](uint32_t l, uint32_t r) { return centroid(l, axis) < centroid(r, axis); });
        int left, right;
        if (spawn > 0 && end - begin >= 16384) {
            std::vector<TreeNode> right_nodes;
            std::exception_ptr error;
            std::thread worker([&] {
                try {
                    build(right_nodes, mid, end, spawn - 1);
                } catch (...) {
                    error = std::current_exception();
                }
            });
            left = build(nodes, begin, mid, spawn - 1);
            worker.join();
            if (error) std::rethrow_exception(error);
            right = int(nodes.size());
            for (TreeNode n : right_nodes) {
                if (n.left >= 0) { n.left += right; n.right += right; }
                nodes.push_back(n);
            }
        } else {
            left = build(nodes, begin, mid, 0);
            right = build(nodes, mid, end, 0);
        }
        nodes[idx].left = left; nodes[idx].right = right; nodes[idx].count = 0;
        return idx;
    }
    void run()
    {
        order.resize(tri.size() / 3);
        std::iota(order.begin(), order.end(), 0u);
        nodes.clear();
        int spawn = 0;
        while ((2u << spawn) <= host_threads()) ++spawn;
        if (!order.empty()) build(nodes, 0, uint32_t(order.size()), spawn);
    }
};

inline bool boxes_touch(Vec al, Vec au, Vec bl, Vec bu, double p)
{
    return al.x <= bu.x + p && bl.x <= au.x + p && al.y <= bu.y + p && bl.y <= au.y + p && al.z <= bu.z + p &&
           bl.z <= au.z + p;
}

// ---- host closest-distance (geometry.hpp flavour) -----------------------

Vec triangle_point(Vec p, Vec a, Vec b, Vec c)
{
    const Vec ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    const Vec bp = sub(p, b);
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) return b;
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return add(a, mul(ab, d1 / (d1 - d3)));
    const Vec cp = sub(p, c);
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return add(a, mul(ac, d2 / (d2 - d6)));
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
        return add(b, mul(sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    const double inv = 1.0 / (va + vb + vc);
    return add(add(a, mul(ab, vb * inv)), mul(ac, vc * inv));
}

double segment_segment(Vec p1, Vec q1, Vec p2, Vec q2)
{
    const Vec d1 = sub(q1, p1), d2 = sub(q2, p2), r = sub(p1, p2);
    const double a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    double s = 0.0, t = 0.0;
    if (!(a <= 1e-14 && e <= 1e-14)) {
        if (a <= 1e-14) t = std::clamp(f / e, 0.0, 1.0);
        else {
            const double c = dot(d1, r);
            if (e <= 1e-14) s = std::clamp(-c / a, 0.0, 1.0);
            else {
                const double b = dot(d1, d2), den = a * e - b * b;
                if (den != 0.0) s = std::clamp((b * f - c * e) / den, 0.0, 1.0);
                t = (b * s + f) / e;
                if (t < 0.0) { t = 0.0; s = std::clamp(-c / a, 0.0, 1.0); }
                else if (t > 1.0) { t = 1.0; s = std::clamp((b - c) / a, 0.0, 1.0); }
            }
        }
    }
    return len(sub(add(p1, mul(d1, s)), add(p2, mul(d2, t))));
}

bool segment_crosses(Vec p0, Vec p1, Vec a, Vec b, Vec c)
{
    const Vec d = sub(p1, p0), e1 = sub(b, a), e2 = sub(c, a), h = cross(d, e2);
    const double det = dot(e1, h);
    if (std::fabs(det) < 1.0e-14) return false;
    const double inv = 1.0 / det;
    const Vec s = sub(p0, a);
    const double u = inv * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const Vec q = cross(s, e1);
    const double v = inv * dot(d, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = inv * dot(e2, q);
    return !(t < 0.0 || t > 1.0);
}

double segment_triangle_distance(Vec p0, Vec p1, Vec a, Vec b, Vec c)
{
    if (segment_crosses(p0, p1, a, b, c)) return 0.0;
    double best = std::min(len(sub(p0, triangle_point(p0, a, b, c))), len(sub(p1, triangle_point(p1, a, b, c))));
    best = std::min(best, segment_segment(p0, p1, a, b));
    best = std::min(best, segment_segment(p0, p1, b, c));
    best = std::min(best, segment_segment(p0, p1, c, a));
    return best;
}

// Whether the ray p + t (1, 1.2345e-6, 2.3456e-6), t > 1e-12, crosses the
// triangle: the per-triangle test of the reference's ray-parity inside test
// (solver.cpp:608-632), Moller-Trumbore with its thresholds.
constexpr double kRayDy = 0.0000012345, kRayDz = 0.0000023456;

inline bool ray_crosses(Vec p, Vec a, Vec b, Vec c)
{
    const Vec dir = mk(1.0, kRayDy, kRayDz);
    const Vec e1 = sub(b, a), e2 = sub(c, a), h = cross(dir, e2);
    const double det = dot(e1, h);
    if (std::fabs(det) < 1.0e-14) return false;
    const double inv = 1.0 / det;
    const Vec s = sub(p, a);
    const double u = inv * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const Vec q = cross(s, e1);
    const double v = inv * dot(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    return inv * dot(e2, q) > 1.0e-12;
}

// The reference loops over every triangle per point (O(points x
// triangles): minutes for a 1.8M-node request on a 20k-triangle body).  Here
// a host BVH skips triangles that loop cannot count, and the hit count is
// otherwise the same test on the same values, so the parity is identical:
//   a counted triangle's exact ray-plane point Q lies within `pad` of the
//   triangle (the rounding of its barycentric test is at most about
//   0.1 E^2 (S + 2E) with E the longest edge and S the scene diagonal, since
//   |det| >= 1e-14; `pad` takes 20 times that), at a ray parameter above
//   -pad; the walk visits every node whose box grown by `pad` the ray
//   crosses for x >= p.x - pad, which includes Q's leaf.
struct InsideTester {
    const Model &m;
    TreeBuilder tb;
    double pad = 0.0;

    // `points`: every point that will be tested (they bound S).
    InsideTester(const Model &model, const std::vector<Vec> &points) : m(model), tb{model.collider, model.tri, false, {}, {}}
    {
        tb.run();
        double edge2 = 0.0;
        for (size_t t = 0; t < m.tri.size() / 3; ++t)
            for (int e = 0; e < 3; ++e)
                edge2 = std::max(edge2, sq(sub(m.collider[m.tri[3 * t + e]], m.collider[m.tri[3 * t + (e + 1) % 3]])));
        Vec lo = mk(1e300, 1e300, 1e300), hi = mk(-1e300, -1e300, -1e300);
        for (const Vec &v : m.collider) { lo = vmin(lo, v); hi = vmax(hi, v); }
        for (const Vec &v : points) { lo = vmin(lo, v); hi = vmax(hi, v); }
        const double scene = points.empty() && m.collider.empty() ? 0.0 : len(sub(hi, lo));
        const double edge = std::sqrt(edge2);
        pad = 2.0 * edge2 * (scene + 2.0 * edge) + 1.0e-9;
    }

    // The ray meets the box grown by pad at some x >= p.x - pad.
    bool ray_meets(Vec p, const TreeNode &nd) const
    {
        const double x0 = std::max(nd.lo.x, p.x) - pad, x1 = nd.hi.x + pad;
        if (x1 < x0) return false;
        const double y0 = p.y + (x0 - p.x) * kRayDy, y1 = p.y + (x1 - p.x) * kRayDy;
        const double z0 = p.z + (x0 - p.x) * kRayDz, z1 = p.z + (x1 - p.x) * kRayDz;
        return y1 >= nd.lo.y - pad && y0 <= nd.hi.y + pad && z1 >= nd.lo.z - pad && z0 <= nd.hi.z + pad;
    }

    bool inside(Vec p, std::vector<int> &stack) const
    {
        if (tb.nodes.empty()) return false;
        uint32_t hits = 0;
        stack.assign(1, 0);
        while (!stack.empty()) {
            const TreeNode &nd = tb.nodes[stack.back()];
            stack.pop_back();
            if (!ray_meets(p, nd)) continue;
            if (nd.left >= 0) { stack.push_back(nd.left); stack.push_back(nd.right); continue; }
            for (uint32_t k = nd.begin; k < nd.begin + nd.count; ++k) {
                const uint32_t t = tb.order[k];
                if (ray_crosses(p, m.collider[m.tri[3 * t]], m.collider[m.tri[3 * t + 1]], m.collider[m.tri[3 * t + 2]])) ++hits;
            }
        }
        return (hits & 1u) != 0;
    }
};

}  // namespace

bool build_rod_model(const SceneInput &in, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                     Model &m, std::string &error)
{
    m = Model{};
    const uint32_t strand_count = uint32_t(in.offsets.size() - 1);
    const double hmax = desc.maximum_element_length, zero_tol = 1.0e-12;
    m.mapping.assign(in.points.size(), 0);
    auto push_node = [&](Vec x, uint32_t s, NodeBinding b, bool virt) {
        m.x.push_back(x);
        m.node_strand.push_back(s);
        m.binding.push_back(b);
        m.virtual_extension.push_back(virt ? 1 : 0);
        return uint32_t(m.x.size() - 1);
    };
    for (uint32_t s = 0; s < strand_count; ++s) {
        const uint32_t begin = in.offsets[s], end = in.offsets[s + 1];
        const uint32_t first = uint32_t(m.x.size());
        m.mapping[begin] = push_node(in.points[begin], s, {begin, begin, 0.0}, false);
        Vec prev = in.points[begin];
        uint32_t unique = 0, tip_left = begin, tip_right = begin;
        double rest = 0.0, tip_len = 0.0;
        Vec tip_dir;
        for (uint32_t p = begin + 1; p < end; ++p) {
            const Vec target = in.points[p];
            const double seg = len(sub(target, prev));
            if (seg <= zero_tol) {  // zero-length segment: merge (solver.cpp:263-268)
                m.mapping[p] = uint32_t(m.x.size() - 1);
                ++m.merged_segments;
                prev = target;
                continue;
            }
            const uint32_t div = std::max(1u, uint32_t(std::ceil(seg / hmax)));
            for (uint32_t d = 1; d <= div; ++d) {
                const double t = double(d) / div;
                push_node(lerp(prev, target, t), s, {p - 1, p, t}, false);
            }
            m.mapping[p] = uint32_t(m.x.size() - 1);
            prev = target;
            rest += seg;
            tip_left = p - 1;
            tip_right = p;
            tip_len = seg;
            tip_dir = divs(sub(target, in.points[p - 1]), seg);
            ++unique;
        }
        if (unique == 0 || m.x.size() - first < 2) {
            std::ostringstream ss;
            ss << "strand " << s << " has all points at one position (points " << begin << ".." << (end - 1) << ")";
            error = ss.str();
            return false;
        }
        if (desc.minimum_dynamic_length > rest + zero_tol) {  // invisible extension (solver.cpp:292-311)
            const double ext = desc.minimum_dynamic_length - rest;
            const uint32_t div = std::max(1u, uint32_t(std::ceil(ext / hmax)));
            const Vec tip = in.points[end - 1];
            for (uint32_t d = 1; d <= div; ++d) {
                const double dist = ext * double(d) / div;
                push_node(add(tip, mul(tip_dir, dist)), s, {tip_left, tip_right, 1.0 + dist / tip_len}, true);
            }
            ++m.extension_strands;
            m.extension_nodes += div;
            m.extension_length += ext;
        }
        const uint32_t count = uint32_t(m.x.size()) - first;
        const uint32_t fixed = std::min<uint32_t>(desc.fixed_root_nodes, count);
        m.strand_first.push_back(first);
        m.strand_count.push_back(count);
        m.strand_fixed.push_back(fixed);
    }
    const size_t n = m.x.size();
    m.fixed.assign(n, 0);
    for (size_t s = 0; s < m.strands(); ++s)
        for (uint32_t k = 0; k < m.strand_fixed[s]; ++k) m.fixed[m.strand_first[s] + k] = 1;

    // Parallel-transported reference frames and rest strains
    // (solver.cpp:320-356).
    m.frame.assign(n, Mat{});
    std::vector<Vec> tangents;
    for (size_t s = 0; s < m.strands(); ++s) {
        const uint32_t first = m.strand_first[s], count = m.strand_count[s];
        strand_tangents(m.x, first, count, tangents, false);
        Mat f = tangent_frame(tangents[0], mk(1, 0, 0));
        m.frame[first] = f;
        for (uint32_t k = 1; k < count; ++k) {
            f = tangent_frame(tangents[k], transport(column(f, 0), tangents[k - 1], tangents[k]));
            m.frame[first + k] = f;
        }
        for (uint32_t k = 0; k + 1 < count; ++k) {
            const uint32_t i = first + k, j = first + k + 1;
            m.elem_i.push_back(i);
            m.elem_j.push_back(j);
            m.elem_strand.push_back(uint32_t(s));
            m.elem_contact.push_back(m.virtual_extension[j] ? 0 : 1);
            const double L = len(sub(m.x[j], m.x[i]));
            m.rest_length.push_back(L);
            const Vec t = divs(sub(m.x[j], m.x[i]), L);
            const Mat &ri = m.frame[i], &rj = m.frame[j];
            // 0.5 (Ri^T + Rj^T) t
            Vec shear;
            double *out[3] = {&shear.x, &shear.y, &shear.z};
            for (int r = 0; r < 3; ++r) {
                const double h0 = 0.5 * (ri.m[r] + rj.m[r]), h1 = 0.5 * (ri.m[3 + r] + rj.m[3 + r]),
                             h2 = 0.5 * (ri.m[6 + r] + rj.m[6 + r]);
                *out[r] = (h0 * t.x + h1 * t.y) + h2 * t.z;
            }
            m.rest_shear.push_back(shear);
            m.rest_curvature.push_back(divs(cayley(transpose_times(ri, rj)), L));
        }
    }
    assign_masses(m, material);
    (void)error;
    return true;
}

void assign_masses(Model &m, const KhsHairMaterial &material)
{
    const double area = kPiHost * material.radius * material.radius;
    const double inertia = kPiHost * std::pow(material.radius, 4.0) / 4.0;
    const double polar = 2.0 * inertia;
    m.mass.assign(m.nodes(), 0.0);
    m.rotational_mass.assign(m.nodes(), 0.0);
    for (size_t e = 0; e < m.elements(); ++e) {
        const double mass = material.density * area * m.rest_length[e];
        const double rmass = material.density * (2.0 * inertia + polar) / 3.0 * m.rest_length[e];
        m.mass[m.elem_i[e]] += 0.5 * mass;
        m.mass[m.elem_j[e]] += 0.5 * mass;
        m.rotational_mass[m.elem_i[e]] += 0.5 * rmass;
        m.rotational_mass[m.elem_j[e]] += 0.5 * rmass;
    }
}

bool root_targets(const Model &m, const std::vector<Vec> &points, std::vector<Vec> &pos, std::vector<Vec> &rot)
{
    const size_t n = m.nodes();
    pos.resize(n);
    rot.assign(n, Vec{});
    for (size_t k = 0; k < n; ++k) {
        const NodeBinding &b = m.binding[k];
        pos[k] = add(mul(points[b.left], 1.0 - b.t), mul(points[b.right], b.t));
    }
    std::vector<Vec> tangents;
    for (size_t s = 0; s < m.strands(); ++s) {
        const uint32_t first = m.strand_first[s], count = m.strand_count[s];
        if (!strand_tangents(pos, first, count, tangents, true)) return false;
        Mat f = tangent_frame(tangents[0], column(m.frame[first], 0));
        rot[first] = rotation_vector(from_dm(dm::times_transpose(to_dm(f), to_dm(m.frame[first]))));
        for (uint32_t k = 1; k < count; ++k) {
            f = tangent_frame(tangents[k], transport(column(f, 0), tangents[k - 1], tangents[k]));
            rot[first + k] = rotation_vector(from_dm(dm::times_transpose(to_dm(f), to_dm(m.frame[first + k]))));
        }
    }
    return true;
}

void collider_topology(Model &m)
{
    m.boundary_edges = m.nonmanifold_edges = m.inconsistent_edges = m.inverted_components = 0;
    struct Use { uint32_t count = 0; int direction = 0; };
    std::unordered_map<uint64_t, Use> uses;
    uses.reserve(m.tri.size());
    for (size_t t = 0; t < m.tri.size() / 3; ++t)
        for (int e = 0; e < 3; ++e) {
            const uint32_t a = m.tri[3 * t + e], b = m.tri[3 * t + (e + 1) % 3];
            Use &u = uses[(uint64_t(std::min(a, b)) << 32) | std::max(a, b)];
            ++u.count;
            u.direction += a < b ? 1 : -1;
        }
    for (const auto &kv : uses) {
        if (kv.second.count == 1) ++m.boundary_edges;
        else if (kv.second.count > 2) ++m.nonmanifold_edges;
        else if (kv.second.direction != 0) ++m.inconsistent_edges;
    }
    m.closed_manifold = m.boundary_edges == 0 && m.nonmanifold_edges == 0 && m.inconsistent_edges == 0;
    if (m.closed_manifold) {
        double six_volume = 0.0;
        for (size_t t = 0; t < m.tri.size() / 3; ++t)
            six_volume += dot(m.collider[m.tri[3 * t]], cross(m.collider[m.tri[3 * t + 1]], m.collider[m.tri[3 * t + 2]]));
        if (six_volume < 0.0) m.inverted_components = 1;
    }
}

double minimum_gap_host(const Model &m, const KhsHairMaterial &material, uint64_t *candidates)
{
    TreeBuilder tb{m.collider, m.tri, false, {}, {}};
    tb.run();
    const double pad = material.radius + material.collider_offset + material.barrier_distance;
    // Elements in chunks on the host threads: the minimum and the count do
    // not depend on the order the elements are visited in.
    const unsigned chunks = host_threads();
    std::vector<double> chunk_best(chunks, std::numeric_limits<double>::infinity());
    std::vector<uint64_t> chunk_count(chunks, 0);
    parallel_chunks(m.elements(), chunks, [&](size_t begin, size_t end, unsigned c) {
        double best = std::numeric_limits<double>::infinity();
        uint64_t count = 0;
        std::vector<int> stack;
        for (size_t e = begin; e < end; ++e) {
            const uint32_t i = m.elem_i[e], j = m.elem_j[e];
            if (m.fixed[i] || !m.elem_contact[e] || tb.nodes.empty()) continue;
            const Vec lo = vmin(m.x[i], m.x[j]), hi = vmax(m.x[i], m.x[j]);
            stack.assign(1, 0);
            while (!stack.empty()) {
                const TreeNode &nd = tb.nodes[stack.back()];
                stack.pop_back();
                if (!boxes_touch(lo, hi, nd.lo, nd.hi, pad)) continue;
                if (nd.left >= 0) { stack.push_back(nd.left); stack.push_back(nd.right); continue; }
                for (uint32_t k = nd.begin; k < nd.begin + nd.count; ++k) {
                    const uint32_t t = tb.order[k];
                    const double d = segment_triangle_distance(m.x[i], m.x[j], m.collider[m.tri[3 * t]],
                                                               m.collider[m.tri[3 * t + 1]], m.collider[m.tri[3 * t + 2]]);
                    best = std::min(best, d - material.radius - material.collider_offset);
                    ++count;
                }
            }
        }
        chunk_best[c] = best;
        chunk_count[c] = count;
    });
    double best = std::numeric_limits<double>::infinity();
    uint64_t count = 0;
    for (unsigned c = 0; c < chunks; ++c) {
        best = std::min(best, chunk_best[c]);
        count += chunk_count[c];
    }
    if (candidates) *candidates = count;
    return best;
}

bool initial_feasibility(const Model &m, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                         double &minimum_gap, std::string &error)
{
    if (m.closed_manifold) {
        const InsideTester tester(m, m.x);
        // Nodes in chunks on the host threads; the error names the lowest
        // inside node, as the one-thread scan would.
        const unsigned chunks = host_threads();
        std::vector<size_t> first_inside(chunks, m.nodes());
        parallel_chunks(m.nodes(), chunks, [&](size_t begin, size_t end, unsigned c) {
            std::vector<int> stack;
            for (size_t k = begin; k < end; ++k) {
                if (m.fixed[k] || m.virtual_extension[k]) continue;
                if (tester.inside(m.x[k], stack)) { first_inside[c] = k; return; }
            }
        });
        const size_t k = *std::min_element(first_inside.begin(), first_inside.end());
        if (k < m.nodes()) {
            std::ostringstream ss;
            ss << "initial intersection: internal node " << k << " lies inside the closed collider";
            error = ss.str();
            return false;
        }
    }
    uint64_t candidates = 0;
    minimum_gap = minimum_gap_host(m, material, &candidates);
    if (minimum_gap <= desc.minimum_gap) {
        std::ostringstream ss;
        ss << "initial intersection or negative gap: minimum gap " << minimum_gap << " m over " << candidates
           << " candidates";
        error = ss.str();
        return false;
    }
    return true;
}

void inside_closed_collider(const Model &m, const std::vector<Vec> &points, std::vector<uint8_t> &inside)
{
    inside.assign(points.size(), 0);
    const InsideTester tester(m, points);
    parallel_chunks(points.size(), host_threads(), [&](size_t begin, size_t end, unsigned) {
        std::vector<int> stack;
        for (size_t k = begin; k < end; ++k) inside[k] = tester.inside(points[k], stack) ? 1 : 0;
    });
}

void build_device_bvh(Model &m)
{
    TreeBuilder tb{m.collider, m.tri, true, {}, {}};
    tb.run();
    FlatBvh &f = m.bvh;
    f = FlatBvh{};
    f.order = tb.order;
    if (tb.nodes.empty()) return;
    const size_t count = tb.nodes.size();
    std::vector<uint32_t> slot(count, 0);
    f.lower.resize(3 * count); f.upper.resize(3 * count);
    f.escape.resize(count); f.first.resize(count); f.count.resize(count);
    f.parent.assign(count, -1); f.left_child.assign(count, 0); f.right_child.assign(count, 0);
    // Right-first preorder: iterative DFS that pushes left below right.
    struct Item { int tree; int parent_slot; uint32_t depth; };
    std::vector<Item> stack{{0, -1, 0}};
    uint32_t next = 0;
    std::vector<int> tree_of_slot(count, -1);
    while (!stack.empty()) {
        const Item it = stack.back();
        stack.pop_back();
        const uint32_t s = next++;
        slot[it.tree] = s;
        tree_of_slot[s] = it.tree;
        f.parent[s] = it.parent_slot;
        f.depth = std::max(f.depth, it.depth);
        const TreeNode &t = tb.nodes[it.tree];
        f.lower[3 * s] = t.lo.x; f.lower[3 * s + 1] = t.lo.y; f.lower[3 * s + 2] = t.lo.z;
        f.upper[3 * s] = t.hi.x; f.upper[3 * s + 1] = t.hi.y; f.upper[3 * s + 2] = t.hi.z;
        f.first[s] = t.begin;
        f.count[s] = t.left >= 0 ? 0 : t.count;
        if (t.left >= 0) {
            stack.push_back({t.left, int(s), it.depth + 1});
            stack.push_back({t.right, int(s), it.depth + 1});
        } else {
            f.leaves.push_back(s);
        }
    }
    // Escape index: the slot after the last slot of the subtree.
    std::vector<uint32_t> subtree_end(count, 0);
    for (size_t s = count; s-- > 0;) {
        const TreeNode &t = tb.nodes[tree_of_slot[s]];
        if (t.left < 0) subtree_end[s] = uint32_t(s + 1);
        else {
            const uint32_t l = slot[t.left], r = slot[t.right];
            f.left_child[s] = l;
            f.right_child[s] = r;
            subtree_end[s] = std::max(subtree_end[l], subtree_end[r]);
        }
    }
    for (size_t s = 0; s < count; ++s) f.escape[s] = subtree_end[s];
}

}  // namespace khs
