// The device BVH layout of csrc/khs_model.cpp (build_device_bvh): nodes in
// right-first preorder, each node's escape index the end of its subtree.
// The device walks rely on it: the index after a skipped subtree always
// advances (so a walk visits each node at most once), the root's escape is
// the node count, a leaf's escape is the next node, and an internal node's
// subtree is its own index, its right child's subtree, then its left
// child's.  Usage: test_bvh_layout vertices.bin triangles.bin (FP64 [V][3],
// uint32 [T][3]).  Built and run by tests/test_bvh_layout.py.
#include "khs_model.hpp"

#include <cstdio>
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
    if (argc != 3) {
        std::printf("usage: %s vertices.bin triangles.bin\n", argv[0]);
        return 2;
    }
    const std::vector<double> verts = read_all<double>(argv[1]);
    khs::Model m;
    m.collider.resize(verts.size() / 3);
    for (size_t k = 0; k < m.collider.size(); ++k) m.collider[k] = {verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]};
    m.tri = read_all<uint32_t>(argv[2]);
    khs::build_device_bvh(m);
    const khs::FlatBvh &b = m.bvh;
    const size_t n = b.size();
    long bad = 0;
    if (n == 0 || b.escape[0] != n) ++bad;
    size_t leaf_triangles = 0;
    for (size_t i = 0; i < n; ++i) {
        if (b.escape[i] <= i || b.escape[i] > n) ++bad;
        if (b.count[i]) {
            leaf_triangles += b.count[i];
            if (b.escape[i] != i + 1) ++bad;
        } else {
            const uint32_t r = b.right_child[i], l = b.left_child[i];
            if (r != i + 1 || l != b.escape[r] || b.escape[l] != b.escape[i]) ++bad;
        }
    }
    if (leaf_triangles != m.tri.size() / 3) ++bad;
    std::printf("%zu nodes, %zu triangles, %ld violations\n", n, m.tri.size() / 3, bad);
    if (bad == 0) std::printf("PASS\n");
    return bad != 0;
}
