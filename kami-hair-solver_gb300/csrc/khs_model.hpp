// Host-side rod model builder of the GB300 solver.
//
// Turns the caller's curves and collider into the internal Cosserat rod
// discretisation the device kernels consume.  It follows the reference's
// host preprocessing (src/solver.cpp:121-681, src/math.hpp) step for step,
// because the internal mesh, reference frames, rest strains, masses and root
// targets define the problem being solved; the output, however, is laid out
// for the GPU: node-indexed structure-of-arrays, elements stored at their
// left node, strands as [first, count) ranges and the collider BVH flattened
// into a right-child-first preorder with escape indices for stackless
// traversal.
#pragma once

#include "kami_hair_solver.h"

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace khs {

struct Vec {
    double x = 0.0, y = 0.0, z = 0.0;
};

// 3x3 row-major.
struct Mat {
    double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

struct NodeBinding {
    uint32_t left = 0, right = 0;
    double t = 0.0;
};

// Flattened BVH for the device.  Nodes are stored in DFS preorder visiting
// the right child before the left one, which is the order in which the
// reference's stack traversal visits them (cuda_backend.cu:229-232), so a
// stackless walk "next = overlap && internal ? i + 1 : escape[i]" reproduces
// its candidate order and its first-found closest-triangle tie-break.
struct FlatBvh {
    std::vector<double> lower, upper;       // 3 per node
    std::vector<uint32_t> escape;           // next node index after the subtree (count == end)
    std::vector<uint32_t> first, count;     // leaf triangle range in `order` (count 0 = internal)
    std::vector<int32_t> parent;            // -1 for the root
    std::vector<uint32_t> left_child, right_child;  // internal nodes only
    std::vector<uint32_t> leaves;           // leaf node indices
    std::vector<uint32_t> order;            // triangle permutation
    uint32_t depth = 0;
    size_t size() const { return escape.size(); }
};

struct Model {
    // Nodes (N).
    std::vector<Vec> x;              // rest / initial position
    std::vector<Mat> frame;          // reference frame, columns d1 d2 d3
    std::vector<double> mass, rotational_mass;
    std::vector<uint8_t> fixed, virtual_extension;
    std::vector<uint32_t> node_strand;
    std::vector<NodeBinding> binding;
    // Elements (E), in reference order (strand by strand, root to tip).
    std::vector<uint32_t> elem_i, elem_j, elem_strand;
    std::vector<uint8_t> elem_contact;
    std::vector<double> rest_length;
    std::vector<Vec> rest_shear, rest_curvature;
    // Strands (S): nodes [first, first + count), fixed prefix fixed_count.
    std::vector<uint32_t> strand_first, strand_count, strand_fixed;
    // Original point -> internal node.
    std::vector<uint32_t> mapping;
    // Collider.
    std::vector<Vec> collider;                  // vertex positions at build
    std::vector<uint32_t> tri;                  // 3 per valid triangle
    FlatBvh bvh;

    uint32_t merged_segments = 0, extension_strands = 0, extension_nodes = 0;
    double extension_length = 0.0;
    uint32_t boundary_edges = 0, nonmanifold_edges = 0, inconsistent_edges = 0, inverted_components = 0;
    bool closed_manifold = false;

    size_t nodes() const { return x.size(); }
    size_t elements() const { return elem_i.size(); }
    size_t strands() const { return strand_first.size(); }
};

// Inputs kept by the solver between set_* calls and build.
struct SceneInput {
    std::vector<Vec> points;
    std::vector<uint32_t> offsets;
    std::vector<Vec> collider_vertices;
    std::vector<uint32_t> collider_triangles;   // valid triangles only, 3 per triangle
    uint32_t excluded_triangles = 0;
    bool has_hair = false, has_collider = false;
};

// Internal mesh, frames, elements and masses (solver.cpp:227-373).  Returns
// false with `error` on a strand whose points all coincide.
bool build_rod_model(const SceneInput &in, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                     Model &model, std::string &error);

// Lumped masses from the current material (solver.cpp:358-373).
void assign_masses(Model &model, const KhsHairMaterial &material);

// Root target positions and rotation vectors of every node for evaluated
// source points (solver.cpp:416-447).  Returns false on a degenerate tangent.
bool root_targets(const Model &model, const std::vector<Vec> &points, std::vector<Vec> &positions,
                  std::vector<Vec> &rotations);

// Edge-use diagnostics and closed-mesh orientation (solver.cpp:381-414).
void collider_topology(Model &model);

// Build-time feasibility (solver.cpp:608-681): ray-parity inside test of free
// visible nodes on a closed collider, then the minimum gap over the host
// BVH.  Returns false with `error` when the start state is infeasible.
bool initial_feasibility(const Model &model, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                         double &minimum_gap, std::string &error);

// Ray-parity inside flags of points against the collider, with the
// reference's per-triangle test and parity rule (solver.cpp:608-632) walked
// over a host BVH; the same flags as the reference's all-triangle loop.
void inside_closed_collider(const Model &model, const std::vector<Vec> &points, std::vector<uint8_t> &inside);

// Minimum gap of contact-enabled elements (solver.cpp:659-681).
double minimum_gap_host(const Model &model, const KhsHairMaterial &material, uint64_t *candidates);

// The device BVH of the reference (cuda_backend.cu:294-311) flattened for
// stackless traversal.
void build_device_bvh(Model &model);

}  // namespace khs
