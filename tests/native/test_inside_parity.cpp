// Checks the product's BVH-walked ray-parity inside test
// (khs::inside_closed_collider, csrc/khs_model.cpp) against the reference's
// all-triangle loop (src/solver.cpp:608-632) as the oracle restates it
// (ray_crosses_triangle, oracle/khs_oracle_math.hpp): the inside flag of
// every point must be the same.  Usage:
//   test_inside_parity vertices.bin triangles.bin points.bin [sample]
// (FP64 [V][3], uint32 [T][3], FP64 [P][3]).  With `sample`, the BVH walk
// is timed over every point and the all-triangle loop over every sample-th
// point only (its time is scaled to all points); the flags of the sampled
// points are compared.  Built and run by tests/test_inside_parity.py.
#include "khs_model.hpp"
#include "khs_oracle_math.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

template<class T> static std::vector<T> read_all(const char *path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    const size_t bytes = size_t(f.tellg());
    f.seekg(0);
    std::vector<T> v(bytes / sizeof(T));
    f.read(reinterpret_cast<char *>(v.data()), std::streamsize(v.size() * sizeof(T)));
    return v;
}

int main(int argc, char **argv)
{
    if (argc != 4 && argc != 5) {
        std::printf("usage: %s vertices.bin triangles.bin points.bin [sample]\n", argv[0]);
        return 2;
    }
    const size_t sample = argc == 5 ? size_t(std::atol(argv[4])) : 1;
    const std::vector<double> verts = read_all<double>(argv[1]), pts = read_all<double>(argv[3]);
    const std::vector<uint32_t> tris = read_all<uint32_t>(argv[2]);
    khs::Model m;
    m.collider.resize(verts.size() / 3);
    for (size_t k = 0; k < m.collider.size(); ++k) m.collider[k] = {verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]};
    m.tri = tris;
    std::vector<khs::Vec> points(pts.size() / 3);
    for (size_t k = 0; k < points.size(); ++k) points[k] = {pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};

    std::vector<uint8_t> fast;
    const auto t0 = std::chrono::steady_clock::now();
    khs::inside_closed_collider(m, points, fast);
    const auto t1 = std::chrono::steady_clock::now();

    using khs_oracle::v3;
    long mismatches = 0, inside = 0;
    size_t checked = 0;
    for (size_t k = 0; k < points.size(); k += sample) {
        ++checked;
        const khs_oracle::V3 p = v3(points[k].x, points[k].y, points[k].z);
        uint32_t hits = 0;
        for (size_t t = 0; t < tris.size() / 3; ++t) {
            const khs::Vec &a = m.collider[tris[3 * t]], &b = m.collider[tris[3 * t + 1]], &c = m.collider[tris[3 * t + 2]];
            if (khs_oracle::ray_crosses_triangle(p, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z))) ++hits;
        }
        const uint8_t brute = (hits & 1u) ? 1 : 0;
        inside += brute;
        if (brute != fast[k]) {
            if (mismatches < 10) std::printf("point %zu: all-triangle loop %d, BVH walk %d\n", k, int(brute), int(fast[k]));
            ++mismatches;
        }
    }
    const auto t2 = std::chrono::steady_clock::now();
    const double bvh_s = std::chrono::duration<double>(t1 - t0).count();
    const double loop_s = std::chrono::duration<double>(t2 - t1).count() * double(points.size()) / double(checked);
    std::printf("inside parity: %zu points checked (%ld inside), %zu triangles, %ld mismatches\n", checked, inside,
                tris.size() / 3, mismatches);
    std::printf("time for all %zu points: BVH walk %.3f s, all-triangle loop %.1f s%s\n", points.size(), bvh_s, loop_s,
                sample > 1 ? " (scaled from the sample)" : "");
    std::printf(mismatches == 0 ? "PASS\n" : "FAIL\n");
    return mismatches == 0 ? 0 : 1;
}
