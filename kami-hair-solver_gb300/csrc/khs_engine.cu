// GB300 device engine (see khs_engine.hpp).
//
// Device data layout (one arena allocation, 256-byte aligned sub-arrays):
//   node state     q, q_old, v, q_snap, v_snap, q_base   [N][6] FP64
//   solver vectors grad, dir, precond, dprime            [N][6] FP64
//   block matrices diag, upper, cprime                   [N][36] FP64
//   rotation cache R = exp(u) Ref, left Jacobian Jl      [N][9] FP64
//   element parts  contributions of the element whose left node is n
//                  (as_i_*) and whose right node is n (as_j_*) so every
//                  node sums its two incident elements in a fixed order
//                  without atomics
//   elements       (i, j, contact flag, L0, gamma0, kappa0), energies,
//                  contact records                        [E]
//   strands        first, count, fixed prefix, length-sorted order [S]
//   collider       triangles [T][3], current/old/frame-start/pending
//                  vertices [V][3], BVH in right-first preorder with escape
//                  indices (stackless traversal) and parent links (one-launch
//                  bottom-up refit)
//
// Kernels (thread per node / element / BVH leaf unless noted):
//   per substep   k_begin_substep, k_collider_interp, k_tri32, k_refit,
//                 k_sweep(+record), k_precond, k_update_velocity,
//                 k_friction(+apply)
//   evaluation    k_node_eval, [mixed: k_contact_filter, k_contact_near (warp
//                 per element with cached leaves), k_contact_exact (thread per
//                 FP32 survivor), k_contact_select], k_elem_eval, k_node_sum
//                 (thread per block entry), k_reduce_eval (both levels: the
//                 last block to finish reduces the partials)
//   direction     k_block_solve_aug<H> / k_block_solve_hybrid (persistent
//                 warps, strand groups from a longest-first queue),
//                 [float-float form: k_ff_factor, k_ff_residual, k_ff_correct],
//                 k_steepest, k_scale, k_reduce_dir, k_final_dir
//   CCD           k_ccd (plain), k_ccd_collect + k_ccd_pairs (mixed)
//   queries       k_contact, k_contact_query_records, k_gather
//   root targets  k_root_tangents, k_root_transport, k_root_frames (thread
//                 per strand), k_root_rotations: per call of
//                 khsUpdateRootTargets / khsSetRootAnimationFrame
// Reductions are two-level (fixed per-block trees, then one block over the
// partials) and therefore deterministic.
#include "khs_engine.hpp"
#include "khs_device_math.cuh"
#include "khs_ff.cuh"

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <mutex>
#include <numeric>
#include <stdexcept>

namespace khs {
namespace {

#define KHS_CUDA(call)                                                                         \
    do {                                                                                       \
        const cudaError_t khs_err = (call);                                                    \
        if (khs_err != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(khs_err)); \
    } while (0)

using dm::V;
using dm::M;

constexpr int kBlock = 256;
constexpr int kPartials = 304;  // 2 reduction blocks per SM on a 152-SM GB300
constexpr uint32_t kNone = 0xffffffffu;
constexpr uint64_t kCheckpointMagic = 0x3154504348534bULL;  // same blob header as the reference
constexpr uint8_t kFlagActive = 1, kFlagInfeasible = 2, kFlagEnergy = 4, kFlagClosest = 8;

inline unsigned grid_for(size_t n) { return unsigned((n + kBlock - 1) / kBlock); }
// Every solver runs on device 0 (Engine::initialize selects it).
constexpr int kDevice = 0;

// Scalars produced by one evaluation / direction pass (host-mapped).
struct Mailbox {
    double objective, elastic, contact, kinetic, minimum_gap, grad_norm2;
    unsigned long long candidates, active;
    int feasible;
    int solve_failed;
    double slope, dir_norm2, max_translation;
    unsigned long long ccd_bits;
    uint32_t sweep_fail;
    uint32_t pair_count;
    uint32_t refine_bits;
    uint32_t pad;
    // The direction pass's values (every k_final_dir but the CCD pass of a
    // pipelined iteration, which reduces the already limited direction).
    double dir_slope, dir_max_translation;
    int dir_solve_failed;
    int dir_pad;
};

// Atomic targets live in device memory; the publishing kernels copy them to
// the host-mapped mailbox and reset them for the next use.
struct Scalars {
    unsigned long long ccd_bits;
    uint32_t sweep_fail;
    int solve_failed;
    uint32_t pair_count;
    uint32_t surv_count;  // entries of the mixed contact pass's FP64 work list
    uint32_t solve_next;  // next strand group of the block-solve work queue
    uint32_t refine_bits; // largest relative refinement correction (FP32 bits)
    uint32_t near_count;  // elements queued for the warp-cooperative contact pass
    uint32_t ccd_near;    // elements queued for the warp-cooperative CCD pass
    uint32_t eval_done;   // blocks of k_reduce_eval finished (the last one reduces the partials)
    uint32_t pool_used;   // entries of the leaf pool handed out since the last cache rebuild
    double trial_alpha;   // first line-search step from the last CCD bound (k_final_dir)
    double max_translation;  // largest free-node translation of the last reduced direction (k_final_dir)
};

struct Partial {
    double node_energy, kinetic, elastic, contact, min_gap, grad2;
    unsigned long long candidates, active;
    int infeasible;
    int pad;
};

struct DirPartial {
    double slope, dnorm2, max_translation;
};

struct SweepRecord {
    uint32_t claimed, strand, element, triangle;
    double distance, required, clearance, displacement;
    double hair_start[3], hair_end[3], collider_point[3];
};

// POD view of every device array (passed by value to kernels).
struct View {
    uint32_t N, E, S, V, T, B;
    double *q, *q_old, *v, *q_base, *grad, *dir, *precond;
    double *inertia;  // inertia + damping diagonal of each node's block [N][6]
    float *q32;       // FP32 copy of the node positions [N][3] (mixed contact filter)
    double *rot, *jl, *node_energy, *node_kinetic;
    double *diag, *upper, *cprime, *dprime;
    double *as_i_g, *as_j_g, *as_i_h, *as_j_h, *as_i_f, *as_j_f;
    const double *ref, *mass, *rmass;
    const uint8_t *fixed;
    const int32_t *elem_left, *elem_right;
    const uint32_t *ei, *ej, *estrand;
    const uint8_t *econtact;
    const double *L0, *gamma0, *kappa0;
    double *e_el, *e_co, *c_gap;
    uint32_t *c_cand, *c_tri;
    uint8_t *c_flags;
    const uint32_t *sfirst, *scount, *sfixed, *sorder;
    const uint32_t *tri;
    double *col_cur, *col_old;
    float *col32;  // FP32 copy of col_cur for the mixed form's filters
    double *blo, *bhi;
    float *blo32, *bhi32;  // outward-rounded copies for the mixed form
    // Mixed form: each BVH node packed in 32 bytes (FP32 outward-rounded box,
    // escape index, leaf range), the per-element contact result of the
    // separate contact pass, and the CCD (element, triangle) work list.
    float4 *bnode;
    double *c_t, *c_bary, *c_dist;
    uint32_t *pair_elem, *pair_tri;
    uint32_t pair_capacity;
    // Per-substep leaf cache of the mixed contact pass: the leaves (DFS
    // order) whose FP32 box overlaps the element box grown by kCacheSlack,
    // and the element's node positions when they were collected.
    uint32_t *cache_leaf;
    uint8_t *cache_n;
    // Leaf lists of elements with more than kCacheLeaves leaves: a bump
    // pool (reset at each cache rebuild); such an element's first two
    // cache_leaf slots hold its offset and count.
    uint32_t *leaf_pool;
    uint32_t leaf_pool_capacity;
    float *cache_x32;  // FP32 node positions when the leaves were collected [E][6]
    // Mixed contact pass in three launches: FP32 vertex records of every
    // triangle in leaf order (a, b, c as three float4, the triangle index in
    // the first .w), the survivors of the FP32 filter per element (at most
    // kSurvivors, in traversal order), their FP64 closest pairs (distance,
    // t, barycentrics) and the (element, slot) work list of the FP64 pass.
    float4 *tri32, *tri32_old;  // FP32 records of col_cur and col_old
    // Mixed-form factors in float-float (hi, lo): B_n^-1 and C_n rows [N][36],
    // d'_n [N][6], and the diagonal shift used at each node.
    float2 *ff_inv, *ff_c, *ff_d;
    float *ff_shift;
    uint32_t *surv_tri, *surv_list;
    uint32_t *near_list;  // elements with cached leaves, one warp each in k_contact_near
    uint8_t *surv_n;
    double *surv_res;
    const uint32_t *besc, *bfirst, *bcount, *border, *bleaves;
    const int32_t *bparent;
    const uint32_t *bleft, *bright;
    uint32_t *brefit;
    uint32_t L;
    Partial *partials;
    DirPartial *dpartials;
    Scalars *sc;          // device
    Mailbox *mail;        // host-mapped
    SweepRecord *sweep;   // host-mapped
    // material / desc
    double radius, offset, dhat, kc, friction, smoothing, damping, min_gap;
    double gx, gy, gz;
    dm::Weights w;
    double young, poisson, shear_corr;
    int has_collider;
};

// Next free slot of a work list whose length is *count, for every lane that
// calls it: the lanes that arrive together take consecutive slots with one
// atomic (a per-lane atomic on one address serialises at L2 when tens of
// thousands of elements append in one launch).  Slot order within a list is
// not meaningful to any of its consumers.
__device__ __forceinline__ uint32_t append_slot(uint32_t *count)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

__device__ __forceinline__ V load3(const double *p) { return dm::v(p[0], p[1], p[2]); }
__device__ __forceinline__ void store3(double *p, V a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
__device__ __forceinline__ M load9(const double *p)
{
    M r;
#pragma unroll
    for (int k = 0; k < 9; ++k) r.m[k] = p[k];
    return r;
}
__device__ __forceinline__ V tri_vertex(const View &d, uint32_t t, int c) { return load3(d.col_cur + 3 * size_t(d.tri[3 * t + c])); }

// Next node of a stackless walk after skipping node i's subtree.  In the
// preorder layout a node's escape index is the end of its subtree, so it is
// always greater than i; anything else (a corrupted or uninitialised tree)
// ends the walk instead of restarting it.
__device__ __forceinline__ uint32_t escape_from(uint32_t i, uint32_t escape) { return escape > i ? escape : 0xffffffffu; }

// Stackless BVH walk in the reference's visiting order.
template<class F> __device__ void bvh_query(const View &d, V lo, V hi, double pad, F &&f)
{
    uint32_t i = 0;
    while (i < d.B) {
        const V nl = load3(d.blo + 3 * size_t(i)), nh = load3(d.bhi + 3 * size_t(i));
        if (!dm::boxes_overlap(lo, hi, nl, nh, pad)) { i = escape_from(i, d.besc[i]); continue; }
        const uint32_t cnt = d.bcount[i];
        if (cnt == 0) { ++i; continue; }
        const uint32_t first = d.bfirst[i];
        for (uint32_t k = first; k < first + cnt; ++k) f(d.border[k]);
        i = escape_from(i, d.besc[i]);
    }
}

// Mixed-form walk: internal nodes are tested on outward-rounded FP32 boxes
// against the outward-rounded FP32 query box (a superset of the FP64 test,
// and an FP64 overlap of a leaf implies FP64 overlap of every ancestor);
// leaves passing the FP32 test are re-tested exactly in FP64.  The
// candidates and their order are therefore exactly those of bvh_query.
template<class F> __device__ void bvh_query_mixed(const View &d, V lo, V hi, double pad, F &&f)
{
    const float lx = __double2float_rd(lo.x), ly = __double2float_rd(lo.y), lz = __double2float_rd(lo.z);
    const float hx = __double2float_ru(hi.x), hy = __double2float_ru(hi.y), hz = __double2float_ru(hi.z);
    const float p = __double2float_ru(pad);
    uint32_t i = 0;
    while (i < d.B) {
        const float *nl = d.blo32 + 3 * size_t(i), *nh = d.bhi32 + 3 * size_t(i);
        const bool hit = lx <= __fadd_ru(nh[0], p) && nl[0] <= __fadd_ru(hx, p) && ly <= __fadd_ru(nh[1], p) &&
                         nl[1] <= __fadd_ru(hy, p) && lz <= __fadd_ru(nh[2], p) && nl[2] <= __fadd_ru(hz, p);
        if (!hit) { i = escape_from(i, d.besc[i]); continue; }
        const uint32_t cnt = d.bcount[i];
        if (cnt == 0) { ++i; continue; }
        if (dm::boxes_overlap(lo, hi, load3(d.blo + 3 * size_t(i)), load3(d.bhi + 3 * size_t(i)), pad)) {
            const uint32_t first = d.bfirst[i];
            for (uint32_t k = first; k < first + cnt; ++k) f(d.border[k]);
        }
        i = escape_from(i, d.besc[i]);
    }
}

// Exact FP64 leaf test of the reference (al <= bu + p && bl <= au + p per
// axis) decided in FP32 when possible: if the query box rounded inwards
// still overlaps the leaf box rounded inwards (one ulp inside the stored
// outward box) with the padding rounded down, the FP64 test is true; if the
// outward FP32 test failed it is false; only inside the rounding band is
// the FP64 test evaluated.
struct QueryBox {
    V lo, hi;
    double pad;
    float olx, oly, olz, ohx, ohy, ohz, opad;  // outward-rounded box and padding
    float ilx, ily, ilz, ihx, ihy, ihz, ipad;  // inward-rounded box and padding
};

__device__ __forceinline__ QueryBox make_query(V lo, V hi, double pad)
{
    QueryBox qb;
    qb.lo = lo; qb.hi = hi; qb.pad = pad;
    qb.olx = __double2float_rd(lo.x); qb.oly = __double2float_rd(lo.y); qb.olz = __double2float_rd(lo.z);
    qb.ohx = __double2float_ru(hi.x); qb.ohy = __double2float_ru(hi.y); qb.ohz = __double2float_ru(hi.z);
    qb.opad = __double2float_ru(pad);
    qb.ilx = __double2float_ru(lo.x); qb.ily = __double2float_ru(lo.y); qb.ilz = __double2float_ru(lo.z);
    qb.ihx = __double2float_rd(hi.x); qb.ihy = __double2float_rd(hi.y); qb.ihz = __double2float_rd(hi.z);
    qb.ipad = __double2float_rd(pad);
    return qb;
}

// The same box from FP32 copies of the segment's end points (lo32, hi32 =
// componentwise min / max of the rounded coordinates): rounding to nearest
// moved each coordinate by at most 2^-24 of its magnitude, so widening by
// 2^-23 of the magnitude (plus 1e-30) bounds the FP64 box from outside and
// narrowing by the same bounds it from inside.  lo and hi (FP64) serve the
// exact leaf test.
__device__ __forceinline__ QueryBox make_query_f(const float lo32[3], const float hi32[3], V lo, V hi, double pad)
{
    QueryBox qb;
    qb.lo = lo; qb.hi = hi; qb.pad = pad;
    const float k = 1.1920929e-7f;  // 2^-23
    qb.olx = __fsub_rd(lo32[0], __fmaf_ru(fabsf(lo32[0]), k, 1e-30f));
    qb.oly = __fsub_rd(lo32[1], __fmaf_ru(fabsf(lo32[1]), k, 1e-30f));
    qb.olz = __fsub_rd(lo32[2], __fmaf_ru(fabsf(lo32[2]), k, 1e-30f));
    qb.ohx = __fadd_ru(hi32[0], __fmaf_ru(fabsf(hi32[0]), k, 1e-30f));
    qb.ohy = __fadd_ru(hi32[1], __fmaf_ru(fabsf(hi32[1]), k, 1e-30f));
    qb.ohz = __fadd_ru(hi32[2], __fmaf_ru(fabsf(hi32[2]), k, 1e-30f));
    qb.ilx = __fadd_ru(lo32[0], __fmaf_ru(fabsf(lo32[0]), k, 1e-30f));
    qb.ily = __fadd_ru(lo32[1], __fmaf_ru(fabsf(lo32[1]), k, 1e-30f));
    qb.ilz = __fadd_ru(lo32[2], __fmaf_ru(fabsf(lo32[2]), k, 1e-30f));
    qb.ihx = __fsub_rd(hi32[0], __fmaf_ru(fabsf(hi32[0]), k, 1e-30f));
    qb.ihy = __fsub_rd(hi32[1], __fmaf_ru(fabsf(hi32[1]), k, 1e-30f));
    qb.ihz = __fsub_rd(hi32[2], __fmaf_ru(fabsf(hi32[2]), k, 1e-30f));
    qb.opad = __double2float_ru(pad);
    qb.ipad = __double2float_rd(pad);
    return qb;
}

__device__ __forceinline__ bool maybe_overlap(const QueryBox &q, float4 a, float4 b)
{
    return q.olx <= __fadd_ru(b.x, q.opad) && a.x <= __fadd_ru(q.ohx, q.opad) && q.oly <= __fadd_ru(b.y, q.opad) &&
           a.y <= __fadd_ru(q.ohy, q.opad) && q.olz <= __fadd_ru(b.z, q.opad) && a.z <= __fadd_ru(q.ohz, q.opad);
}

__device__ __forceinline__ bool leaf_overlap_exact(const View &d, uint32_t node, float4 a, float4 b, const QueryBox &q)
{
    const bool surely = q.ilx <= __fadd_rd(nextafterf(b.x, -INFINITY), q.ipad) &&
                        nextafterf(a.x, INFINITY) <= __fadd_rd(q.ihx, q.ipad) &&
                        q.ily <= __fadd_rd(nextafterf(b.y, -INFINITY), q.ipad) &&
                        nextafterf(a.y, INFINITY) <= __fadd_rd(q.ihy, q.ipad) &&
                        q.ilz <= __fadd_rd(nextafterf(b.z, -INFINITY), q.ipad) &&
                        nextafterf(a.z, INFINITY) <= __fadd_rd(q.ihz, q.ipad);
    if (surely) return true;
    return dm::boxes_overlap(q.lo, q.hi, load3(d.blo + 3 * size_t(node)), load3(d.bhi + 3 * size_t(node)), q.pad);
}

// Same walk over the packed 32-byte nodes: one pair of 16-byte loads per
// visited node (box + escape, box + leaf range (first << 4 | count)).
// f receives the position of each candidate in leaf order (index into
// border and tri32).
template<class F> __device__ void bvh_positions_packed(const View &d, const QueryBox &q, F &&f)
{
    uint32_t i = 0;
    while (i < d.B) {
        const float4 a = __ldg(d.bnode + 2 * size_t(i)), b = __ldg(d.bnode + 2 * size_t(i) + 1);
        const uint32_t escape = __float_as_uint(a.w), leaf = __float_as_uint(b.w);
        if (!maybe_overlap(q, a, b)) { i = escape_from(i, escape); continue; }
        if (leaf == 0) { ++i; continue; }
        if (leaf_overlap_exact(d, i, a, b, q)) {
            const uint32_t first = leaf >> 4, cnt = leaf & 15u;
            for (uint32_t k = first; k < first + cnt; ++k) f(k);
        }
        i = escape_from(i, escape);
    }
}

template<class F> __device__ void bvh_query_packed(const View &d, V lo, V hi, double pad, F &&f)
{
    bvh_positions_packed(d, make_query(lo, hi, pad), [&](uint32_t k) { f(d.border[k]); });
}

constexpr int kCacheLeaves = 32;
constexpr double kCacheSlack = 1.0e-3;  // metres each node may move before the cache is bypassed
constexpr uint8_t kCacheInvalid = 0xff;
constexpr uint8_t kCacheBig = 0xfe;     // cache_n of an element whose leaves live in the leaf pool

// Leaves whose FP32 outward box overlaps (lo, hi) padded by pad, in DFS
// order; the first cap are written to out, and the return value is the
// count of all of them.
__device__ uint32_t collect_leaves(const View &d, V lo, V hi, double pad, uint32_t *out, uint32_t cap)
{
    const QueryBox q = make_query(lo, hi, pad);
    uint32_t i = 0, n = 0;
    while (i < d.B) {
        const float4 a = __ldg(d.bnode + 2 * size_t(i)), b = __ldg(d.bnode + 2 * size_t(i) + 1);
        const uint32_t escape = __float_as_uint(a.w), leaf = __float_as_uint(b.w);
        if (!maybe_overlap(q, a, b)) { i = escape_from(i, escape); continue; }
        if (leaf == 0) { ++i; continue; }
        if (n < cap) out[n] = i;
        ++n;
        i = escape_from(i, escape);
    }
    return n;
}

// The cached leaf list of element e with cache state nl (its cache_n):
// the element's own slots, or its range of the leaf pool; nullptr without
// a cache.
__device__ __forceinline__ const uint32_t *cached_leaves(const View &d, uint32_t e, uint8_t nl, uint32_t &count)
{
    const uint32_t *slots = d.cache_leaf + size_t(kCacheLeaves) * e;
    if (nl == kCacheInvalid) { count = 0; return nullptr; }
    if (nl == kCacheBig) { count = slots[1]; return d.leaf_pool + slots[0]; }
    count = nl;
    return slots;
}

// Candidates of leaves given as a list (the cached leaves), with the exact
// per-leaf test: the same candidates in the same order as the full walk,
// provided the list holds every leaf that test can accept.  f receives
// leaf-order positions.
template<class F> __device__ void leaves_positions(const View &d, const uint32_t *leaves, uint32_t n, const QueryBox &q,
                                                   F &&f)
{
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t i = leaves[k];
        const float4 a = __ldg(d.bnode + 2 * size_t(i)), b = __ldg(d.bnode + 2 * size_t(i) + 1);
        if (!maybe_overlap(q, a, b) || !leaf_overlap_exact(d, i, a, b, q)) continue;
        const uint32_t leaf = __float_as_uint(b.w), first = leaf >> 4, cnt = leaf & 15u;
        for (uint32_t t = first; t < first + cnt; ++t) f(t);
    }
}

template<class F> __device__ void leaves_query(const View &d, const uint32_t *leaves, uint32_t n, V lo, V hi, double pad, F &&f)
{
    leaves_positions(d, leaves, n, make_query(lo, hi, pad), [&](uint32_t k) { f(d.border[k]); });
}

template<bool MIXED, class F> __device__ __forceinline__ void bvh_walk(const View &d, V lo, V hi, double pad, F &&f)
{
    if (MIXED) bvh_query_packed(d, lo, hi, pad, f);
    else bvh_query(d, lo, hi, pad, f);
}

// FP32 distance of a candidate from the FP32 vertex copy, relative to an
// FP32 origin (the segment start): no FP64 instruction.  Rounding the
// vertices, the origin and the segment end to FP32 moves each coordinate by
// at most 2^-24 of its magnitude, so the distance moves by at most
// sqrt(3) * 2^-24 * (|vertex| + |origin| + |end|)_inf < 2.5e-7 * M, with M
// bounding the absolute coordinates involved; that term is added to the
// relative margin of the FP32 distance itself.
__device__ __forceinline__ float candidate_distance_f(const View &d, uint32_t t, dm::F3 origin, dm::F3 p0, dm::F3 p1, float &m)
{
    const float *c32 = d.col32;
    const uint32_t i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
    const float ax = c32[3 * i0], ay = c32[3 * i0 + 1], az = c32[3 * i0 + 2];
    const float bx = c32[3 * i1], by = c32[3 * i1 + 1], bz = c32[3 * i1 + 2];
    const float cx = c32[3 * i2], cy = c32[3 * i2 + 1], cz = c32[3 * i2 + 2];
    const dm::F3 a = dm::f3(ax - origin.x, ay - origin.y, az - origin.z);
    const dm::F3 b = dm::f3(bx - origin.x, by - origin.y, bz - origin.z);
    const dm::F3 c = dm::f3(cx - origin.x, cy - origin.y, cz - origin.z);
    const float df = dm::segment_triangle_distance_f(p0, p1, a, b, c, m);
    const float vmax = fmaxf(fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fmaxf(fabsf(az), fabsf(bx))),
                             fmaxf(fmaxf(fabsf(by), fabsf(bz)), fmaxf(fmaxf(fabsf(cx), fabsf(cy)), fabsf(cz))));
    const float omax = fmaxf(fmaxf(fabsf(origin.x), fabsf(origin.y)), fabsf(origin.z));
    const float emax = fmaxf(fmaxf(fabsf(p1.x), fabsf(p1.y)), fabsf(p1.z)) + omax;
    m += 2.5e-7f * (vmax + omax + emax) + 1.0e-9f;
    return df;
}

// ---- per-substep set-up ---------------------------------------------------

__global__ void __launch_bounds__(kBlock) k_begin_substep(View d, const double *root_a, const double *rot_a,
                                                          const double *root_b, const double *rot_b, double f, double dt)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    double q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) { q[k] = d.q[6 * size_t(n) + k]; d.q_old[6 * size_t(n) + k] = q[k]; }
    if (!d.fixed[n]) return;
    // Uncontracted lerps: the root targets and collider vertices feed the
    // integer contact work, so they round exactly like a host evaluation.
    const V p = dm::gadd(dm::gmul(load3(root_a + 3 * size_t(n)), 1.0 - f), dm::gmul(load3(root_b + 3 * size_t(n)), f));
    const V r = dm::gadd(dm::gmul(load3(rot_a + 3 * size_t(n)), 1.0 - f), dm::gmul(load3(rot_b + 3 * size_t(n)), f));
    const double vals[6] = {p.x, p.y, p.z, r.x, r.y, r.z};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        d.q[6 * size_t(n) + k] = vals[k];
        d.v[6 * size_t(n) + k] = (vals[k] - q[k]) / dt;
    }
}

__global__ void __launch_bounds__(kBlock) k_collider_interp(View d, const double *a, const double *b, double f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    const V cur = load3(d.col_cur + 3 * size_t(i));
    store3(d.col_old + 3 * size_t(i), cur);
    const V nv = dm::gadd(dm::gmul(load3(a + 3 * size_t(i)), 1.0 - f), dm::gmul(load3(b + 3 * size_t(i)), f));
    store3(d.col_cur + 3 * size_t(i), nv);
    d.col32[3 * size_t(i)] = float(nv.x); d.col32[3 * size_t(i) + 1] = float(nv.y); d.col32[3 * size_t(i) + 2] = float(nv.z);
}

// Bottom-up refit in one launch: each leaf thread computes its box and walks
// up; the second child to arrive at a parent (atomic counter) merges the two
// children, resets the counter for the next launch and continues.
__global__ void __launch_bounds__(kBlock) k_refit(View d, int swept)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.L) return;
    uint32_t node = d.bleaves[k];
    V lo = dm::v(1e300, 1e300, 1e300), hi = dm::v(-1e300, -1e300, -1e300);
    const uint32_t first = d.bfirst[node], cnt = d.bcount[node];
    for (uint32_t j = first; j < first + cnt; ++j) {
        const uint32_t t = d.border[j];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint32_t vi = d.tri[3 * t + c];
            const V a = load3(d.col_cur + 3 * size_t(vi));
            lo = dm::vmin(lo, a); hi = dm::vmax(hi, a);
            if (swept) { const V o = load3(d.col_old + 3 * size_t(vi)); lo = dm::vmin(lo, o); hi = dm::vmax(hi, o); }
        }
    }
    store3(d.blo + 3 * size_t(node), lo);
    store3(d.bhi + 3 * size_t(node), hi);
    d.blo32[3 * size_t(node)] = __double2float_rd(lo.x); d.blo32[3 * size_t(node) + 1] = __double2float_rd(lo.y);
    d.blo32[3 * size_t(node) + 2] = __double2float_rd(lo.z);
    d.bhi32[3 * size_t(node)] = __double2float_ru(hi.x); d.bhi32[3 * size_t(node) + 1] = __double2float_ru(hi.y);
    d.bhi32[3 * size_t(node) + 2] = __double2float_ru(hi.z);
    if (d.bnode) {
        float4 *pn = d.bnode + 2 * size_t(node);
        pn[0].x = d.blo32[3 * size_t(node)]; pn[0].y = d.blo32[3 * size_t(node) + 1]; pn[0].z = d.blo32[3 * size_t(node) + 2];
        pn[1].x = d.bhi32[3 * size_t(node)]; pn[1].y = d.bhi32[3 * size_t(node) + 1]; pn[1].z = d.bhi32[3 * size_t(node) + 2];
    }
    for (;;) {
        const int32_t p = d.bparent[node];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(&d.brefit[p], 1u) == 0) return;
        d.brefit[p] = 0;
        __threadfence();
        const volatile double *blo = d.blo, *bhi = d.bhi;
        const uint32_t l = d.bleft[p], r = d.bright[p];
        const V llo = dm::v(blo[3 * l], blo[3 * l + 1], blo[3 * l + 2]), rlo = dm::v(blo[3 * r], blo[3 * r + 1], blo[3 * r + 2]);
        const V lhi = dm::v(bhi[3 * l], bhi[3 * l + 1], bhi[3 * l + 2]), rhi = dm::v(bhi[3 * r], bhi[3 * r + 1], bhi[3 * r + 2]);
        const V plo = dm::vmin(llo, rlo), phi = dm::vmax(lhi, rhi);
        store3(d.blo + 3 * size_t(p), plo);
        store3(d.bhi + 3 * size_t(p), phi);
        // Rounding is monotone, so rounding the merged FP64 box equals the
        // merge of the rounded children.
        d.blo32[3 * size_t(p)] = __double2float_rd(plo.x); d.blo32[3 * size_t(p) + 1] = __double2float_rd(plo.y);
        d.blo32[3 * size_t(p) + 2] = __double2float_rd(plo.z);
        d.bhi32[3 * size_t(p)] = __double2float_ru(phi.x); d.bhi32[3 * size_t(p) + 1] = __double2float_ru(phi.y);
        d.bhi32[3 * size_t(p) + 2] = __double2float_ru(phi.z);
        if (d.bnode) {
            float4 *pn = d.bnode + 2 * size_t(p);
            pn[0].x = d.blo32[3 * size_t(p)]; pn[0].y = d.blo32[3 * size_t(p) + 1]; pn[0].z = d.blo32[3 * size_t(p) + 2];
            pn[1].x = d.bhi32[3 * size_t(p)]; pn[1].y = d.bhi32[3 * size_t(p) + 1]; pn[1].z = d.bhi32[3 * size_t(p) + 2];
        }
        node = uint32_t(p);
    }
}

// Conservative advancement of each moving triangle against the stationary
// hair at the start of the substep (cuda_backend.cu:975-987).  Returns the
// first failing triangle of this element in traversal order.
// Mixed form: a candidate whose FP32 lower-bound clearance already lets the
// first advancement step reach alpha = 1 cannot fail and is skipped (the
// 1e-6 relative slack dwarfs the FP64 rounding of that one step).
// FP32 pre-test of the mixed sweep for the candidate at leaf-order position
// p: true when the first conservative-advancement step of the exact pass is
// certain to reach the end of the substep (no failure from this triangle).
// It needs a lower bound of the segment's distance to the triangle at its
// old position (tri32_old records, margins as record_distance_f) and an
// upper bound of the largest vertex displacement (FP32 differences of the
// rounded copies, widened by their rounding).
__device__ __forceinline__ bool sweep_skip_f(const View &d, uint32_t p, dm::F3 origin, dm::F3 f1, float target_ru)
{
    const float4 n0 = __ldg(d.tri32 + 3 * size_t(p)), n1 = __ldg(d.tri32 + 3 * size_t(p) + 1),
                 n2 = __ldg(d.tri32 + 3 * size_t(p) + 2);
    const float4 o0 = __ldg(d.tri32_old + 3 * size_t(p)), o1 = __ldg(d.tri32_old + 3 * size_t(p) + 1),
                 o2 = __ldg(d.tri32_old + 3 * size_t(p) + 2);
    auto disp = [](float4 a, float4 b) {
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float mag = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)), fmaxf(fmaxf(fabsf(b.x), fabsf(b.y)), fabsf(b.z)));
        return __fadd_ru(__fmul_ru(sqrtf(dx * dx + dy * dy + dz * dz), 1.00001f), __fmaf_ru(mag, 5.0e-7f, 1.0e-12f));
    };
    const float speed_ub = fmaxf(disp(n0, o0), fmaxf(disp(n1, o1), disp(n2, o2)));
    const dm::F3 a = dm::f3(o0.x - origin.x, o0.y - origin.y, o0.z - origin.z);
    const dm::F3 b = dm::f3(o1.x - origin.x, o1.y - origin.y, o1.z - origin.z);
    const dm::F3 c = dm::f3(o2.x - origin.x, o2.y - origin.y, o2.z - origin.z);
    float m;
    const float df = dm::segment_triangle_distance_f(dm::f3(0.f, 0.f, 0.f), f1, a, b, c, m);
    const float vmax = fmaxf(fmaxf(fmaxf(fabsf(o0.x), fabsf(o0.y)), fmaxf(fabsf(o0.z), fabsf(o1.x))),
                             fmaxf(fmaxf(fabsf(o1.y), fabsf(o1.z)), fmaxf(fmaxf(fabsf(o2.x), fabsf(o2.y)), fabsf(o2.z))));
    const float omax = fmaxf(fmaxf(fabsf(origin.x), fabsf(origin.y)), fabsf(origin.z));
    const float emax = fmaxf(fmaxf(fabsf(f1.x), fabsf(f1.y)), fabsf(f1.z)) + omax;
    m += 2.5e-7f * (vmax + omax + emax) + 1.0e-9f;
    return __fmul_rd(0.8f, __fsub_rd(__fsub_rd(df, m), target_ru)) >= __fmul_ru(speed_ub, 1.000002f);
}

template<bool MIXED> __device__ bool sweep_element(const View &d, uint32_t e, SweepRecord *rec)
{
    const uint32_t i = d.ei[e], j = d.ej[e];
    const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
    const double target = d.radius + d.offset + d.min_gap;
    const dm::F3 f0 = dm::f3(0.f, 0.f, 0.f), f1 = dm::to_local(p1, p0);
    bool failed = false;
    bvh_walk<MIXED>(d, dm::vmin(p0, p1), dm::vmax(p0, p1), target, [&](uint32_t t) {
        if (failed) return;
        const V oa = load3(d.col_old + 3 * size_t(d.tri[3 * t])), ob = load3(d.col_old + 3 * size_t(d.tri[3 * t + 1])),
                oc = load3(d.col_old + 3 * size_t(d.tri[3 * t + 2]));
        const V da = dm::gsub(tri_vertex(d, t, 0), oa), db = dm::gsub(tri_vertex(d, t, 1), ob),
                dc = dm::gsub(tri_vertex(d, t, 2), oc);
        const double speed = fmax(dm::gnorm(da), fmax(dm::gnorm(db), dm::gnorm(dc)));
        if (speed < 1e-30) return;
        if (MIXED) {
            float m;
            const float df = dm::segment_triangle_distance_f(f0, f1, dm::to_local(oa, p0), dm::to_local(ob, p0),
                                                              dm::to_local(oc, p0), m);
            if (0.8 * (double(df) - double(m) - target) >= speed * (1.0 + 1e-6)) return;
        }
        double alpha = 0.0;
        bool end = false;
        dm::ClosestPair pair;
        V a, b, c;
        for (int k = 0; k < 80; ++k) {
            a = dm::gadd(oa, dm::gmul(da, alpha)); b = dm::gadd(ob, dm::gmul(db, alpha)); c = dm::gadd(oc, dm::gmul(dc, alpha));
            pair = dm::closest_segment_triangle(p0, p1, a, b, c);
            const double clearance = pair.distance - target;
            if (clearance <= 0) { failed = true; break; }
            const double advance = 0.8 * clearance / speed;
            if (alpha + advance >= 1) { end = true; break; }
            if (advance < 1e-12) { failed = true; break; }
            alpha += advance;
        }
        if (!end) failed = true;
        if (failed && rec) {
            rec->claimed = 1; rec->strand = d.estrand[e]; rec->element = e; rec->triangle = t;
            rec->distance = pair.distance; rec->required = target; rec->clearance = pair.distance - target;
            rec->displacement = speed;
            store3(rec->hair_start, p0); store3(rec->hair_end, p1);
            store3(rec->collider_point, dm::gadd(dm::gadd(dm::gmul(a, pair.bary.x), dm::gmul(b, pair.bary.y)), dm::gmul(c, pair.bary.z)));
        }
    });
    return failed;
}

// Mixed sweep of one element: the same candidates in the same order as
// sweep_element, with sweep_skip_f deciding first from FP32 copies, so only
// the triangles that could fail are loaded and advanced in FP64.
__device__ bool sweep_element_f(const View &d, uint32_t e)
{
    const uint32_t i = d.ei[e], j = d.ej[e];
    const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
    const double target = d.radius + d.offset + d.min_gap;
    const float target_ru = __double2float_ru(target);
    const dm::F3 origin = dm::f3(float(p0.x), float(p0.y), float(p0.z));
    const dm::F3 f1 = dm::f3(float(p1.x) - origin.x, float(p1.y) - origin.y, float(p1.z) - origin.z);
    bool failed = false;
    bvh_positions_packed(d, make_query(dm::vmin(p0, p1), dm::vmax(p0, p1), target), [&](uint32_t p) {
        if (failed || sweep_skip_f(d, p, origin, f1, target_ru)) return;
        const uint32_t t = __float_as_uint(__ldg(d.tri32 + 3 * size_t(p)).w);
        const V oa = load3(d.col_old + 3 * size_t(d.tri[3 * t])), ob = load3(d.col_old + 3 * size_t(d.tri[3 * t + 1])),
                oc = load3(d.col_old + 3 * size_t(d.tri[3 * t + 2]));
        const V da = dm::gsub(tri_vertex(d, t, 0), oa), db = dm::gsub(tri_vertex(d, t, 1), ob),
                dc = dm::gsub(tri_vertex(d, t, 2), oc);
        const double speed = fmax(dm::gnorm(da), fmax(dm::gnorm(db), dm::gnorm(dc)));
        if (speed < 1e-30) return;
        double alpha = 0.0;
        bool end = false;
        for (int k = 0; k < 80; ++k) {
            const V a = dm::gadd(oa, dm::gmul(da, alpha)), b = dm::gadd(ob, dm::gmul(db, alpha)), c = dm::gadd(oc, dm::gmul(dc, alpha));
            const double clearance = dm::closest_segment_triangle(p0, p1, a, b, c).distance - target;
            if (clearance <= 0) { failed = true; break; }
            const double advance = 0.8 * clearance / speed;
            if (alpha + advance >= 1) { end = true; break; }
            if (advance < 1e-12) { failed = true; break; }
            alpha += advance;
        }
        if (!end) failed = true;
    });
    return failed;
}

template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_sweep(View d)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    if (d.fixed[d.ei[e]] || !d.econtact[e]) return;
    const bool failed = MIXED ? sweep_element_f(d, e) : sweep_element<false>(d, e, nullptr);
    if (failed) atomicMin(&d.sc->sweep_fail, e);
}

// Publishes the lowest failing element of k_sweep (with its first failing
// triangle in traversal order) and re-arms the atomic.
__global__ void k_sweep_record(View d)
{
    if (threadIdx.x || blockIdx.x) return;
    const uint32_t e = d.sc->sweep_fail;
    d.sc->sweep_fail = kNone;
    d.mail->sweep_fail = e;
    if (e == kNone) return;
    SweepRecord rec{};
    sweep_element<false>(d, e, &rec);
    *d.sweep = rec;
}

// Diagonal preconditioner (cuda_backend.cu:815-841): node term then the
// left and right incident elements, inverted; 0 at fixed nodes.
__global__ void __launch_bounds__(kBlock) k_precond(View d, double dt)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    const double inv = 1.0 / dt, inv2 = inv * inv;
    double t = d.mass[n] * (inv2 + d.damping * inv), r = d.rmass[n] * (inv2 + d.damping * inv);
    const double area = dm::kPi * d.radius * d.radius;
    const double inertia = dm::kPi * d.radius * d.radius * d.radius * d.radius / 4.0;
    const double G = d.young / (2.0 * (1.0 + d.poisson));
    const int32_t es[2] = {d.elem_left[n], d.elem_right[n]};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (es[k] < 0) continue;
        const double L = d.L0[es[k]];
        t += fmax(d.young * area, d.shear_corr * G * area) / L;
        r += d.shear_corr * G * area * L + fmax(d.young * inertia, 2.0 * G * inertia) / L;
    }
    const bool fx = d.fixed[n];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        d.precond[6 * size_t(n) + k] = fx ? 0.0 : 1.0 / fmax(t, 1.0e-30);
        d.precond[6 * size_t(n) + 3 + k] = fx ? 0.0 : 1.0 / fmax(r, 1.0e-30);
    }
}

// ---- energy / gradient / Gauss-Newton Hessian -----------------------------

// Per node: optional line-search update q = q_base + alpha dir, rotation
// cache, inertia + damping energy, gradient and diagonal
// (cuda_backend.cu:883-897).
// Trial state q = q_base + alpha dir (trial) and the FP32 position copy.
// alpha_dev (if set) holds the trial step in device memory (the pipelined
// first trial of an iteration, whose step the host has not read yet).
__device__ __forceinline__ void node_positions(const View &d, uint32_t n, int trial, double alpha, double q[6])
{
    const size_t o = 6 * size_t(n);
    if (trial) {
#pragma unroll
        for (int k = 0; k < 6; ++k) { q[k] = d.q_base[o + k] + alpha * d.dir[o + k]; d.q[o + k] = q[k]; }
    } else {
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = d.q[o + k];
    }
    d.q32[3 * size_t(n)] = float(q[0]); d.q32[3 * size_t(n) + 1] = float(q[1]); d.q32[3 * size_t(n) + 2] = float(q[2]);
}

// The positions alone, so that the contact passes (which read q and the
// FP32 copy) can run beside the rest of k_node_eval.
__global__ void __launch_bounds__(kBlock) k_positions(View d, int trial, double alpha, const double *alpha_dev)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    double q[6];
    node_positions(d, n, trial, alpha_dev ? *alpha_dev : alpha, q);
}

// positions_done: k_positions has written q and the FP32 copy.
__global__ void __launch_bounds__(kBlock) k_node_eval(View d, int gradient, int trial, double alpha, double dt,
                                                      const double *alpha_dev, int positions_done)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    if (alpha_dev) alpha = *alpha_dev;
    double q[6];
    const size_t o = 6 * size_t(n);
    if (positions_done) {
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = d.q[o + k];
    } else {
        node_positions(d, n, trial, alpha, q);
    }
    M R, J;
    dm::rotation_and_jacobian(dm::v(q[3], q[4], q[5]), d.ref + 9 * size_t(n), R, gradient ? &J : nullptr);
#pragma unroll
    for (int k = 0; k < 9; ++k) d.rot[9 * size_t(n) + k] = R.m[k];
    if (gradient) {
#pragma unroll
        for (int k = 0; k < 9; ++k) d.jl[9 * size_t(n) + k] = J.m[k];
    }
    if (d.fixed[n]) {
        d.node_energy[n] = 0.0;
        d.node_kinetic[n] = 0.0;
        if (gradient) {
#pragma unroll
            for (int k = 0; k < 6; ++k) { d.grad[o + k] = 0.0; d.inertia[o + k] = 0.0; }
        }
        return;
    }
    const double inv = 1.0 / dt, inv2 = inv * inv, m = d.mass[n], mr = d.rmass[n];
    const double kx = m * inv2, kr = mr * inv2, cx = m * d.damping * inv, cr = mr * d.damping * inv;
    const double grav[3] = {d.gx, d.gy, d.gz};
    double obj = 0.0, kin = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double g = k < 3 ? grav[k] * dt * dt : 0.0;
        const double qo = d.q_old[o + k];
        const double predicted = qo + dt * d.v[o + k] + g;
        const double delta = q[k] - predicted, damp = q[k] - qo;
        const double kk = k < 3 ? kx : kr, c = k < 3 ? cx : cr;
        obj += 0.5 * kk * delta * delta + 0.5 * c * damp * damp;
        if (k < 3) kin += 0.5 * m * damp * damp * inv2;
        if (gradient) {
            d.grad[o + k] = kk * delta + c * damp;
            d.inertia[o + k] = kk + c;
        }
    }
    d.node_energy[n] = obj;
    d.node_kinetic[n] = kin;
}

// Two-pass closest search of the mixed form over a candidate source
// (source(fn) calls fn(triangle) for each candidate in traversal order):
// FP32 distances with margins bound the FP64 minimum, then FP64 is evaluated
// only for candidates whose lower bound does not exceed that bound.
template<class Source>
__device__ __forceinline__ uint32_t closest_triangle_in(const View &d, V xi, V xj, uint32_t &cand, dm::ClosestPair &pair,
                                                        Source &&source)
{
    uint32_t closest = kNone;
    cand = 0;
    pair.distance = 1.0e300; pair.t = 0.0; pair.bary = dm::v(1, 0, 0);
    const dm::F3 origin = dm::f3(float(xi.x), float(xi.y), float(xi.z));
    const dm::F3 p0 = dm::f3(0.f, 0.f, 0.f), p1 = dm::f3(float(xj.x) - origin.x, float(xj.y) - origin.y, float(xj.z) - origin.z);
    float bound = 3.0e38f;
    source([&](uint32_t t) {
        ++cand;
        float m;
        const float df = candidate_distance_f(d, t, origin, p0, p1, m);
        bound = fminf(bound, df + m);
    });
    if (cand == 0) return kNone;
    source([&](uint32_t t) {
        float m;
        const float df = candidate_distance_f(d, t, origin, p0, p1, m);
        if (df - m > bound) return;
        const dm::ClosestPair c = dm::closest_segment_triangle(xi, xj, tri_vertex(d, t, 0), tri_vertex(d, t, 1), tri_vertex(d, t, 2));
        if (c.distance < pair.distance) { pair = c; closest = t; }
    });
    return closest;
}

// Broad + narrow phase of one element: every candidate in traversal order,
// the first strictly closest triangle kept (cuda_backend.cu:920-926).
// Mixed form: a first pass bounds the FP64 minimum by FP32 distances with
// margins; the second pass evaluates in FP64 only the candidates whose lower
// bound does not exceed that bound, in the same order, so the result (and
// the first-found tie-break) equals the all-FP64 search.
template<bool MIXED>
__device__ __forceinline__ uint32_t closest_triangle(const View &d, V xi, V xj, double pad, uint32_t &cand,
                                                     dm::ClosestPair &pair)
{
    uint32_t closest = kNone;
    cand = 0;
    pair.distance = 1.0e300; pair.t = 0.0; pair.bary = dm::v(1, 0, 0);
    const V lo = dm::vmin(xi, xj), hi = dm::vmax(xi, xj);
    if (!MIXED) {
        bvh_query(d, lo, hi, pad, [&](uint32_t t) {
            ++cand;
            const dm::ClosestPair c = dm::closest_segment_triangle(xi, xj, tri_vertex(d, t, 0), tri_vertex(d, t, 1), tri_vertex(d, t, 2));
            if (c.distance < pair.distance) { pair = c; closest = t; }
        });
        return closest;
    }
    return closest_triangle_in(d, xi, xj, cand, pair, [&](auto &&fn) { bvh_query_packed(d, lo, hi, pad, fn); });
}

// Contact classification of every element at a caller-provided state
// (positions of q_probe); used to check the integer contact work.
// Contact classification of every element at the state q: candidate count,
// closest triangle with its closest pair, gap and flags.  The mixed form runs
// this as its own low-register pass before the element energy (and for the
// contact-query entry point); the plain form searches inside k_elem_eval.
template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_contact(View d, const double *q)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    uint32_t cand = 0, closest = kNone;
    uint8_t flags = 0;
    double gap = 0.0;
    dm::ClosestPair pair;
    pair.distance = 1.0e300; pair.t = 0.0; pair.bary = dm::v(1, 0, 0);
    if (d.has_collider && !d.fixed[i] && d.econtact[e]) {
        const V xi = load3(q + 6 * size_t(i)), xj = load3(q + 6 * size_t(j));
        closest = closest_triangle<MIXED>(d, xi, xj, d.radius + d.offset + d.dhat, cand, pair);
        if (closest != kNone) {
            flags |= kFlagClosest;
            gap = pair.distance - d.radius - d.offset;
            if (gap <= d.min_gap) flags |= kFlagInfeasible;
            else if (gap < d.dhat) flags |= kFlagActive;
        }
    }
    d.c_cand[e] = cand;
    d.c_tri[e] = closest;
    d.c_flags[e] = flags;
    d.c_gap[e] = gap;
    d.c_t[e] = pair.t;
    d.c_dist[e] = pair.distance;
    store3(d.c_bary + 3 * size_t(e), pair.bary);
}

// ---- mixed contact pass in three launches ---------------------------------
//
// k_contact_filter (per element): candidate count and the FP32 filter over
// the triangle records in leaf order; the survivors (every candidate whose
// FP32 lower bound does not exceed the smallest FP32 upper bound, in
// traversal order) go to per-element slots and to a compact work list.
// k_contact_exact (per survivor): the FP64 closest pair, with every lane of
// a warp on the same code path.  k_contact_select (per element): the first
// strictly closest survivor in traversal order.  Candidates that are not
// survivors are strictly farther in FP64 than the minimum, so the result,
// tie-break included, equals k_contact's and the all-FP64 search.

constexpr int kSurvivors = 8;
constexpr int kLeafTriangles = 8;  // BVH leaves hold at most 8 triangles (cuda_backend.cu:305)
constexpr uint8_t kSurvOverflow = 0xff;

// FP32 vertex records of every triangle in leaf order, of col_cur and of
// col_old; run whenever they change (after k_collider_interp and at set-up).
__global__ void __launch_bounds__(kBlock) k_tri32(View d)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.T) return;
    const uint32_t t = d.border[p];
    const V a = tri_vertex(d, t, 0), b = tri_vertex(d, t, 1), c = tri_vertex(d, t, 2);
    d.tri32[3 * size_t(p)] = make_float4(float(a.x), float(a.y), float(a.z), __uint_as_float(t));
    d.tri32[3 * size_t(p) + 1] = make_float4(float(b.x), float(b.y), float(b.z), 0.0f);
    d.tri32[3 * size_t(p) + 2] = make_float4(float(c.x), float(c.y), float(c.z), 0.0f);
    const V oa = load3(d.col_old + 3 * size_t(d.tri[3 * t])), ob = load3(d.col_old + 3 * size_t(d.tri[3 * t + 1])),
            oc = load3(d.col_old + 3 * size_t(d.tri[3 * t + 2]));
    d.tri32_old[3 * size_t(p)] = make_float4(float(oa.x), float(oa.y), float(oa.z), __uint_as_float(t));
    d.tri32_old[3 * size_t(p) + 1] = make_float4(float(ob.x), float(ob.y), float(ob.z), 0.0f);
    d.tri32_old[3 * size_t(p) + 2] = make_float4(float(oc.x), float(oc.y), float(oc.z), 0.0f);
}

// candidate_distance_f on the record at leaf-order position p (one 48-byte
// record instead of an index triple and three vertex reads).
__device__ __forceinline__ float record_distance_f(const View &d, uint32_t p, dm::F3 origin, dm::F3 p0, dm::F3 p1, float &m,
                                                   uint32_t &t)
{
    const float4 r0 = __ldg(d.tri32 + 3 * size_t(p)), r1 = __ldg(d.tri32 + 3 * size_t(p) + 1),
                 r2 = __ldg(d.tri32 + 3 * size_t(p) + 2);
    t = __float_as_uint(r0.w);
    const dm::F3 a = dm::f3(r0.x - origin.x, r0.y - origin.y, r0.z - origin.z);
    const dm::F3 b = dm::f3(r1.x - origin.x, r1.y - origin.y, r1.z - origin.z);
    const dm::F3 c = dm::f3(r2.x - origin.x, r2.y - origin.y, r2.z - origin.z);
    const float df = dm::segment_triangle_distance_f(p0, p1, a, b, c, m);
    const float vmax = fmaxf(fmaxf(fmaxf(fabsf(r0.x), fabsf(r0.y)), fmaxf(fabsf(r0.z), fabsf(r1.x))),
                             fmaxf(fmaxf(fabsf(r1.y), fabsf(r1.z)), fmaxf(fmaxf(fabsf(r2.x), fabsf(r2.y)), fabsf(r2.z))));
    const float omax = fmaxf(fmaxf(fabsf(origin.x), fabsf(origin.y)), fabsf(origin.z));
    const float emax = fmaxf(fmaxf(fabsf(p1.x), fabsf(p1.y)), fabsf(p1.z)) + omax;
    m += 2.5e-7f * (vmax + omax + emax) + 1.0e-9f;
    return df;
}

// Filter of one element over a position source; returns the survivor count
// (kSurvivors + 1 or more on overflow; the first kSurvivors are stored).
template<class Source>
__device__ __forceinline__ uint32_t filter_survivors(const View &d, uint32_t e, dm::F3 xi32, dm::F3 xj32, uint32_t &cand,
                                                     Source &&source)
{
    const dm::F3 origin = xi32;
    const dm::F3 p0 = dm::f3(0.f, 0.f, 0.f), p1 = dm::f3(xj32.x - origin.x, xj32.y - origin.y, xj32.z - origin.z);
    float bound = 3.0e38f;
    cand = 0;
    source([&](uint32_t p) {
        ++cand;
        float m;
        uint32_t t;
        const float df = record_distance_f(d, p, origin, p0, p1, m, t);
        bound = fminf(bound, df + m);
    });
    if (cand == 0) return 0;
    uint32_t n = 0;
    uint32_t *slots = d.surv_tri + size_t(kSurvivors) * e;
    source([&](uint32_t p) {
        float m;
        uint32_t t;
        const float df = record_distance_f(d, p, origin, p0, p1, m, t);
        if (df - m > bound) return;
        if (n < uint32_t(kSurvivors)) slots[n] = t;
        ++n;
    });
    return n;
}

__device__ __forceinline__ void write_contact(const View &d, uint32_t e, uint32_t closest, const dm::ClosestPair &pair)
{
    uint8_t flags = 0;
    double gap = 0.0;
    if (closest != kNone) {
        flags |= kFlagClosest;
        gap = pair.distance - d.radius - d.offset;
        if (gap <= d.min_gap) flags |= kFlagInfeasible;
        else if (gap < d.dhat) flags |= kFlagActive;
    }
    d.c_tri[e] = closest;
    d.c_flags[e] = flags;
    d.c_gap[e] = gap;
    d.c_t[e] = pair.t;
    d.c_dist[e] = pair.distance;
    store3(d.c_bary + 3 * size_t(e), pair.bary);
}

// Slack test of the leaf cache on the FP32 copies: the copies differ from
// the FP64 positions by at most 2^-24 of a coordinate's magnitude, so the
// margin of 1e-5 m keeps every accepted displacement within kCacheSlack
// for coordinates below a few hundred metres.
__device__ __forceinline__ bool within_cache_slack(const float *c, dm::F3 xi, dm::F3 xj)
{
    const float s = float(kCacheSlack) - 1.0e-5f;
    return fabsf(xi.x - c[0]) <= s && fabsf(xi.y - c[1]) <= s && fabsf(xi.z - c[2]) <= s && fabsf(xj.x - c[3]) <= s &&
           fabsf(xj.y - c[4]) <= s && fabsf(xj.z - c[5]) <= s;
}

// q must be d.q (its FP32 copy d.q32 is read).
__global__ void __launch_bounds__(kBlock) k_contact_filter(View d, const double *q, int cache)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = e < d.E;
    uint32_t append = 0;
    if (live) {
        const uint32_t i = d.ei[e], j = d.ej[e];
        uint32_t cand = 0, n = 0;
        bool deferred = false;  // finished by k_contact_near
        const bool enabled = d.has_collider && !d.fixed[i] && d.econtact[e];
        if (enabled) {
            const dm::F3 xi32 = dm::f3(d.q32[3 * size_t(i)], d.q32[3 * size_t(i) + 1], d.q32[3 * size_t(i) + 2]);
            const dm::F3 xj32 = dm::f3(d.q32[3 * size_t(j)], d.q32[3 * size_t(j) + 1], d.q32[3 * size_t(j) + 2]);
            const double pad = d.radius + d.offset + d.dhat;
            float *c32 = d.cache_x32 + 6 * size_t(e);
            uint8_t nl = cache >= 0 ? d.cache_n[e] : kCacheInvalid;
            bool inside = cache == 0 && nl != kCacheInvalid && within_cache_slack(c32, xi32, xj32);
            // FP64 positions only where a walk is needed.
            V xi = dm::v(0, 0, 0), xj = xi;
            if (!inside) { xi = load3(q + 6 * size_t(i)); xj = load3(q + 6 * size_t(j)); }
            if (cache == 1 || (cache == 0 && !inside)) {
                // (Re)collect the leaves around the element box grown by the
                // slack: one walk, after which both filter passes read the
                // short leaf list (an element that left its slack would
                // otherwise walk the tree twice in every evaluation).
                const V s3 = dm::v(kCacheSlack, kCacheSlack, kCacheSlack);
                const V clo = dm::vmin(xi, xj) - s3, chi = dm::vmax(xi, xj) + s3;
                uint32_t *slots = d.cache_leaf + size_t(kCacheLeaves) * e;
                const uint32_t c = collect_leaves(d, clo, chi, pad, slots, kCacheLeaves);
                if (c <= uint32_t(kCacheLeaves)) {
                    nl = uint8_t(c);
                } else {
                    // A dense patch of the collider (a mesh pole, a seam):
                    // the list goes to the pool, and k_contact_near works
                    // through it 32 leaves at a time.
                    const uint32_t off = atomicAdd(&d.sc->pool_used, c);
                    nl = kCacheInvalid;
                    if (size_t(off) + c <= d.leaf_pool_capacity) {
                        collect_leaves(d, clo, chi, pad, d.leaf_pool + off, c);
                        slots[0] = off;
                        slots[1] = c;
                        nl = kCacheBig;
                    }
                }
                d.cache_n[e] = nl;
                c32[0] = xi32.x; c32[1] = xi32.y; c32[2] = xi32.z; c32[3] = xj32.x; c32[4] = xj32.y; c32[5] = xj32.z;
                inside = nl != kCacheInvalid;
            }
            if (inside) {
                if (nl > 0) {
                    // k_contact_near finishes the element, one warp over its leaves.
                    d.near_list[append_slot(&d.sc->near_count)] = e;
                    deferred = true;
                }
            } else {
                // More than kCacheLeaves leaves around the element: walk.
                const float lo32[3] = {fminf(xi32.x, xj32.x), fminf(xi32.y, xj32.y), fminf(xi32.z, xj32.z)};
                const float hi32[3] = {fmaxf(xi32.x, xj32.x), fmaxf(xi32.y, xj32.y), fmaxf(xi32.z, xj32.z)};
                const QueryBox qb = make_query_f(lo32, hi32, dm::vmin(xi, xj), dm::vmax(xi, xj), pad);
                n = filter_survivors(d, e, xi32, xj32, cand, [&](auto &&fn) { bvh_positions_packed(d, qb, fn); });
            }
        }
        if (!deferred) {
            d.c_cand[e] = cand;
            if (n > uint32_t(kSurvivors)) {
                // Rare: more near-equal candidates than slots; k_contact_select
                // finishes the element with the in-thread search.
                d.surv_n[e] = kSurvOverflow;
            } else {
                d.surv_n[e] = uint8_t(n);
                append = n;
                if (n == 0) {
                    dm::ClosestPair pair;
                    pair.distance = 1.0e300; pair.t = 0.0; pair.bary = dm::v(1, 0, 0);
                    write_contact(d, e, kNone, pair);
                }
            }
        }
    }
    // Warp-aggregated append of (element, slot) entries to the work list.
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint32_t incl = append;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(&d.sc->surv_count, total);
    base = __shfl_sync(FULL, base, 31);
    const uint32_t start = base + incl - append;
    for (uint32_t k = 0; k < append; ++k) d.surv_list[start + k] = uint32_t(kSurvivors) * e + k;
}

// One warp per element with cached leaves: lane l tests cached leaf l
// (DFS order) and evaluates the FP32 distances of that leaf's triangles, so
// the element's candidates are examined in parallel instead of one after
// another by a single lane.  The candidate order is leaf order, then
// triangle order within the leaf, as in the single-lane filter; survivors
// are compacted in that order (a prefix over lanes, then ascending within a
// lane), so slots, the FP64 pass and the ordered selection are unchanged.
// Triangle range (first, cnt) of cached leaf k of a list of `count` when
// its box passes the query's exact per-leaf test; cnt = 0 otherwise.
__device__ __forceinline__ void near_leaf(const View &d, const uint32_t *leaves, uint32_t k, uint32_t count, const QueryBox &qb,
                                          uint32_t &first, uint32_t &cnt)
{
    first = 0;
    cnt = 0;
    if (k >= count) return;
    const uint32_t node = leaves[k];
    const float4 a = __ldg(d.bnode + 2 * size_t(node)), b = __ldg(d.bnode + 2 * size_t(node) + 1);
    if (maybe_overlap(qb, a, b) && leaf_overlap_exact(d, node, a, b, qb)) {
        const uint32_t leaf = __float_as_uint(b.w);
        first = leaf >> 4;
        cnt = leaf & 15u;
    }
}

__device__ __forceinline__ uint32_t warp_inclusive_sum(uint32_t v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Result of one element of the warp-cooperative contact pass (lane 0
// writes): candidate count, survivor count or overflow, the no-contact
// record, and the survivors' entries in the FP64 work list.
__device__ __forceinline__ void near_finish(const View &d, uint32_t e, uint32_t total, uint32_t n, int lane)
{
    uint32_t base = 0;
    if (lane == 0) {
        d.c_cand[e] = total;
        if (n > uint32_t(kSurvivors)) {
            d.surv_n[e] = kSurvOverflow;
        } else {
            d.surv_n[e] = uint8_t(n);
            if (n == 0) {
                dm::ClosestPair pair;
                pair.distance = 1.0e300; pair.t = 0.0; pair.bary = dm::v(1, 0, 0);
                write_contact(d, e, kNone, pair);
            } else {
                base = atomicAdd(&d.sc->surv_count, n);
            }
        }
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    if (n <= uint32_t(kSurvivors) && uint32_t(lane) < n) d.surv_list[base + lane] = uint32_t(kSurvivors) * e + lane;
}

// An element whose cached leaves live in the leaf pool (more than 32): the
// list is taken 32 leaves at a time, once for the FP32 bound and once more
// for the survivors, which are written in leaf order.  Kept out of line so
// the common one-round path keeps its registers.
__device__ __noinline__ void near_pool_element(const View &d, uint32_t e, const QueryBox &qb, dm::F3 origin, dm::F3 p1)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const dm::F3 p0 = dm::f3(0.f, 0.f, 0.f);
    uint32_t nleaves = 0;
    const uint32_t *leaves = cached_leaves(d, e, kCacheBig, nleaves);
    uint32_t total = 0;
    float ub = 3.0e38f;
    for (uint32_t r0 = 0; r0 < nleaves; r0 += 32) {
        uint32_t first, cnt;
        near_leaf(d, leaves, r0 + lane, nleaves, qb, first, cnt);
        for (uint32_t r = 0; r < cnt; ++r) {
            float m;
            uint32_t t;
            const float df = record_distance_f(d, first + r, origin, p0, p1, m, t);
            ub = fminf(ub, df + m);
        }
        total += __shfl_sync(FULL, warp_inclusive_sum(cnt, lane), 31);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ub = fminf(ub, __shfl_xor_sync(FULL, ub, o));
    uint32_t *slots = d.surv_tri + size_t(kSurvivors) * e;
    uint32_t n = 0;
    for (uint32_t r0 = 0; r0 < nleaves; r0 += 32) {
        uint32_t first, cnt;
        near_leaf(d, leaves, r0 + lane, nleaves, qb, first, cnt);
        uint32_t mine = 0;
        for (uint32_t r = 0; r < cnt; ++r) {
            float m;
            uint32_t t;
            const float df = record_distance_f(d, first + r, origin, p0, p1, m, t);
            mine += !(df - m > ub) ? 1u : 0u;
        }
        const uint32_t sincl = warp_inclusive_sum(mine, lane);
        uint32_t slot = n + sincl - mine;
        for (uint32_t r = 0; r < cnt && mine; ++r) {
            float m;
            uint32_t t;
            const float df = record_distance_f(d, first + r, origin, p0, p1, m, t);
            if (df - m > ub) continue;
            if (slot < uint32_t(kSurvivors)) slots[slot] = t;
            ++slot;
        }
        n += __shfl_sync(FULL, sincl, 31);
    }
    near_finish(d, e, total, n, lane);
}

// One warp per element queued by k_contact_filter (leaves cached and the
// element within its slack): lane l tests cached leaf l and the FP32
// distances of its triangles; the smallest upper bound is reduced across
// the warp and the survivors are written in traversal order (leaf, then
// triangle), so the first-found tie-break is kept.
__global__ void __launch_bounds__(kBlock) k_contact_near(View d)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t count = d.sc->near_count;
    const double pad = d.radius + d.offset + d.dhat;
    for (uint32_t k = warp; k < count; k += nwarps) {
        const uint32_t e = d.near_list[k];
        const uint32_t i = d.ei[e], j = d.ej[e];
        const dm::F3 xi32 = dm::f3(d.q32[3 * size_t(i)], d.q32[3 * size_t(i) + 1], d.q32[3 * size_t(i) + 2]);
        const dm::F3 xj32 = dm::f3(d.q32[3 * size_t(j)], d.q32[3 * size_t(j) + 1], d.q32[3 * size_t(j) + 2]);
        const V xi = load3(d.q + 6 * size_t(i)), xj = load3(d.q + 6 * size_t(j));
        const float lo32[3] = {fminf(xi32.x, xj32.x), fminf(xi32.y, xj32.y), fminf(xi32.z, xj32.z)};
        const float hi32[3] = {fmaxf(xi32.x, xj32.x), fmaxf(xi32.y, xj32.y), fmaxf(xi32.z, xj32.z)};
        const QueryBox qb = make_query_f(lo32, hi32, dm::vmin(xi, xj), dm::vmax(xi, xj), pad);
        const dm::F3 origin = xi32, p0 = dm::f3(0.f, 0.f, 0.f);
        const dm::F3 p1 = dm::f3(xj32.x - origin.x, xj32.y - origin.y, xj32.z - origin.z);
        const uint8_t nl = d.cache_n[e];
        if (nl == kCacheBig) {
            near_pool_element(d, e, qb, origin, p1);
            continue;
        }
        uint32_t first, cnt;
        near_leaf(d, d.cache_leaf + size_t(kCacheLeaves) * e, lane, nl, qb, first, cnt);
        const uint32_t total = __shfl_sync(FULL, warp_inclusive_sum(cnt, lane), 31);
        float lb[kLeafTriangles];
        uint32_t tri[kLeafTriangles];
        float ub = 3.0e38f;
#pragma unroll
        for (int r = 0; r < kLeafTriangles; ++r) {
            lb[r] = 3.0e38f;
            tri[r] = 0;
            if (uint32_t(r) < cnt) {
                float m;
                const float df = record_distance_f(d, first + r, origin, p0, p1, m, tri[r]);
                lb[r] = df - m;
                ub = fminf(ub, df + m);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ub = fminf(ub, __shfl_xor_sync(FULL, ub, o));
        uint32_t mine = 0;
#pragma unroll
        for (int r = 0; r < kLeafTriangles; ++r) mine += (uint32_t(r) < cnt && !(lb[r] > ub)) ? 1u : 0u;
        const uint32_t sincl = warp_inclusive_sum(mine, lane);
        const uint32_t n = __shfl_sync(FULL, sincl, 31);
        uint32_t slot = sincl - mine;
        uint32_t *slots = d.surv_tri + size_t(kSurvivors) * e;
#pragma unroll
        for (int r = 0; r < kLeafTriangles; ++r) {
            if (uint32_t(r) < cnt && !(lb[r] > ub)) {
                if (slot < uint32_t(kSurvivors)) slots[slot] = tri[r];
                ++slot;
            }
        }
        near_finish(d, e, total, n, lane);
    }
}

__global__ void __launch_bounds__(kBlock) k_contact_exact(View d, const double *q)
{
    const uint32_t count = d.sc->surv_count;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const uint32_t slot = d.surv_list[k], e = slot / uint32_t(kSurvivors), t = d.surv_tri[slot];
        const uint32_t i = d.ei[e], j = d.ej[e];
        const V xi = load3(q + 6 * size_t(i)), xj = load3(q + 6 * size_t(j));
        const dm::ClosestPair c = dm::closest_segment_triangle(xi, xj, tri_vertex(d, t, 0), tri_vertex(d, t, 1), tri_vertex(d, t, 2));
        double *r = d.surv_res + 5 * size_t(slot);
        r[0] = c.distance; r[1] = c.t; r[2] = c.bary.x; r[3] = c.bary.y; r[4] = c.bary.z;
    }
}

__global__ void __launch_bounds__(kBlock) k_contact_select(View d, const double *q)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0) {  // k_contact_near and k_contact_exact, their only readers, have completed
        d.sc->surv_count = 0;
        d.sc->near_count = 0;
    }
    if (e >= d.E) return;
    const uint32_t n = d.surv_n[e];
    if (n == 0) return;
    if (n == kSurvOverflow) {
        // The two-pass search over the same candidates (the cached leaves
        // when the filter used them, else the full walk).
        const uint32_t i = d.ei[e], j = d.ej[e];
        const V xi = load3(q + 6 * size_t(i)), xj = load3(q + 6 * size_t(j));
        const double pad = d.radius + d.offset + d.dhat;
        const uint8_t nl = d.cache_n[e];
        const dm::F3 xi32 = dm::f3(d.q32[3 * size_t(i)], d.q32[3 * size_t(i) + 1], d.q32[3 * size_t(i) + 2]);
        const dm::F3 xj32 = dm::f3(d.q32[3 * size_t(j)], d.q32[3 * size_t(j) + 1], d.q32[3 * size_t(j) + 2]);
        const bool inside = nl != kCacheInvalid && within_cache_slack(d.cache_x32 + 6 * size_t(e), xi32, xj32);
        uint32_t nleaves = 0;
        const uint32_t *leaves = cached_leaves(d, e, nl, nleaves);
        const V lo = dm::vmin(xi, xj), hi = dm::vmax(xi, xj);
        uint32_t c2 = 0;
        dm::ClosestPair pair;
        const uint32_t closest =
            inside ? closest_triangle_in(d, xi, xj, c2, pair, [&](auto &&fn) { leaves_query(d, leaves, nleaves, lo, hi, pad, fn); })
                   : closest_triangle<true>(d, xi, xj, pad, c2, pair);
        write_contact(d, e, closest, pair);
        return;
    }
    uint32_t best = 0;
    double bd = 1.0e300;
    for (uint32_t k = 0; k < n; ++k) {
        const double dist = d.surv_res[5 * (size_t(kSurvivors) * e + k)];
        if (dist < bd) { bd = dist; best = k; }
    }
    const size_t slot = size_t(kSurvivors) * e + best;
    const double *r = d.surv_res + 5 * slot;
    dm::ClosestPair pair;
    pair.distance = r[0]; pair.t = r[1]; pair.bary = dm::v(r[2], r[3], r[4]);
    write_contact(d, e, d.surv_tri[slot], pair);
}

// ---- contact query without allocation -------------------------------------
//
// Scratch of khsxQueryContactsNoAlloc: the caller's state (48 bytes per
// node) followed by the records (24 bytes per element), in a file-scope
// device array of KHSX_NO_ALLOC_SCRATCH_BYTES.  One array per device and
// process, shared by every solver on that device: calls that overlap in
// time on one device race on it.
__device__ __align__(256) unsigned char g_no_alloc_scratch[KHSX_NO_ALLOC_SCRATCH_BYTES];

// k_contact without the leaf cache, writing the caller-facing record of each
// element straight into the scratch instead of the solver's contact arrays
// (the solver's own records are left as they are).  Every record below E is
// written in full, so nothing in the scratch has to start at zero.
template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_contact_query_records(View d, const double *q,
                                                                                        KhsxContactRecord *out)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    uint32_t cand = 0, closest = kNone, active = 0;
    double gap = __longlong_as_double(0x7ff0000000000000LL);  // +infinity
    dm::ClosestPair pair;
    if (d.has_collider && !d.fixed[i] && d.econtact[e]) {
        const V xi = load3(q + 6 * size_t(i)), xj = load3(q + 6 * size_t(j));
        closest = closest_triangle<MIXED>(d, xi, xj, d.radius + d.offset + d.dhat, cand, pair);
        if (closest != kNone) {
            gap = pair.distance - d.radius - d.offset;
            active = gap > d.min_gap && gap < d.dhat ? 1u : 0u;
        }
    }
    KhsxContactRecord r;
    r.candidate_count = cand;
    r.closest_triangle = closest;
    r.active = active;
    r.reserved = 0;
    r.gap = gap;
    out[e] = r;
}

// Per element: elastic energy (+ gradient and GN blocks) and barrier contact
// against the closest BVH candidate (cuda_backend.cu:899-939).
template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_elem_eval(View d, int gradient)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    const bool fi = d.fixed[i], fj = d.fixed[j];
    const V xi = load3(d.q + 6 * size_t(i)), xj = load3(d.q + 6 * size_t(j));
    const M Ri = load9(d.rot + 9 * size_t(i)), Rj = load9(d.rot + 9 * size_t(j));
    const double L0 = d.L0[e];
    double eps[6];
    double *gi = d.as_i_g + 6 * size_t(i), *gj = d.as_j_g + 6 * size_t(j);
    double *Hii = d.as_i_h + 36 * size_t(i), *Hjj = d.as_j_h + 36 * size_t(j), *Hij = d.upper + 36 * size_t(i);
    if (gradient) {
        const M Jli = load9(d.jl + 9 * size_t(i)), Jlj = load9(d.jl + 9 * size_t(j));
        dm::ElementJacobian J;
        dm::element_strain(Ri, Rj, xi, xj, L0, load3(d.gamma0 + 3 * size_t(e)), load3(d.kappa0 + 3 * size_t(e)), eps, &J,
                           &Jli, &Jlj);
        double a[6], b[6];
        dm::element_gradient(J, eps, d.w, L0, a, b);
        // 16-byte stores: every block starts on a 16-byte boundary (36 and
        // 6 doubles per node from 256-byte aligned arrays).
        double2 *gi2 = reinterpret_cast<double2 *>(gi), *gj2 = reinterpret_cast<double2 *>(gj);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            gi2[k] = fi ? make_double2(0.0, 0.0) : make_double2(a[2 * k], a[2 * k + 1]);
            gj2[k] = fj ? make_double2(0.0, 0.0) : make_double2(b[2 * k], b[2 * k + 1]);
        }
        double hii[36], hjj[36], hij[36];
        dm::element_hessian(J, d.w, L0, hii, hjj, hij);
        double2 *Hii2 = reinterpret_cast<double2 *>(Hii), *Hjj2 = reinterpret_cast<double2 *>(Hjj);
        double2 *Hij2 = reinterpret_cast<double2 *>(Hij);
        const bool fij = fi || fj;
#pragma unroll
        for (int k = 0; k < 18; ++k) {
            Hii2[k] = fi ? make_double2(0.0, 0.0) : make_double2(hii[2 * k], hii[2 * k + 1]);
            Hjj2[k] = fj ? make_double2(0.0, 0.0) : make_double2(hjj[2 * k], hjj[2 * k + 1]);
            Hij2[k] = fij ? make_double2(0.0, 0.0) : make_double2(hij[2 * k], hij[2 * k + 1]);
        }
    } else {
        dm::element_strain(Ri, Rj, xi, xj, L0, load3(d.gamma0 + 3 * size_t(e)), load3(d.kappa0 + 3 * size_t(e)), eps,
                           nullptr, nullptr, nullptr);
    }
    d.e_el[e] = dm::element_energy(eps, d.w, L0);

    uint32_t cand = 0, closest = kNone;
    uint8_t flags = 0;
    double gap = 0.0, ce = 0.0;
    if (d.has_collider && !fi && d.econtact[e]) {
        dm::ClosestPair pair;
        if (MIXED) {
            // Result of the contact pass at this same state.
            cand = d.c_cand[e]; closest = d.c_tri[e]; flags = d.c_flags[e]; gap = d.c_gap[e];
            pair.t = d.c_t[e]; pair.distance = d.c_dist[e]; pair.bary = load3(d.c_bary + 3 * size_t(e));
        } else {
            closest = closest_triangle<false>(d, xi, xj, d.radius + d.offset + d.dhat, cand, pair);
            if (closest != kNone) {
                flags |= kFlagClosest;
                gap = pair.distance - d.radius - d.offset;
                if (gap <= d.min_gap) flags |= kFlagInfeasible;
                else if (gap < d.dhat) flags |= kFlagActive;
            }
        }
        if (closest != kNone) {
            if (flags & kFlagActive) {
                const V a = tri_vertex(d, closest, 0), b = tri_vertex(d, closest, 1), c = tri_vertex(d, closest, 2);
                const V bp = a * pair.bary.x + b * pair.bary.y + c * pair.bary.z;
                double g0[3], g1[3];
                const double energy = dm::barrier_energy_gradient(xi, xj, pair.t, bp, d.radius + d.offset, d.dhat, d.kc, g0, g1);
                if (!isfinite(energy)) flags |= kFlagInfeasible;
                else {
                    flags |= kFlagEnergy;
                    ce = energy;
                    if (gradient) {
#pragma unroll
                        for (int k = 0; k < 3; ++k) { gi[k] += g0[k]; gj[k] += g1[k]; }
                        const V normal = (xi * (1.0 - pair.t) + xj * pair.t - bp) * (1.0 / fmax(pair.distance, 1e-15));
                        const double aa = d.dhat - gap;
                        const double curv = d.kc * (-2.0 * log(gap / d.dhat) + 4.0 * aa / gap + aa * aa / (gap * gap));
                        const double dg[6] = {normal.x * (1.0 - pair.t), normal.y * (1.0 - pair.t), normal.z * (1.0 - pair.t),
                                              normal.x * pair.t, normal.y * pair.t, normal.z * pair.t};
#pragma unroll
                        for (int r = 0; r < 3; ++r)
#pragma unroll
                            for (int c2 = 0; c2 < 3; ++c2) {
                                Hii[6 * r + c2] += curv * dg[r] * dg[c2];
                                Hjj[6 * r + c2] += curv * dg[3 + r] * dg[3 + c2];
                                Hij[6 * r + c2] += curv * dg[r] * dg[3 + c2];
                            }
                    }
                }
            }
        }
    }
    d.e_co[e] = ce;
    d.c_cand[e] = cand;
    d.c_tri[e] = closest;
    d.c_flags[e] = flags;
    d.c_gap[e] = gap;
}

// Node sums in a fixed order: inertia, then the element on the left (this
// node as its right end), then the element on the right.
// One thread per entry (36 N diagonal-block entries, then 6 N gradient
// entries) so every access is coalesced.  Diagonal block = inertia diagonal
// + the contribution of the element whose right node is n + that of the
// element whose left node is n, in that order.
__global__ void __launch_bounds__(kBlock) k_node_sum(View d)
{
    const size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t nh = 36 * size_t(d.N);
    if (idx < nh) {
        const size_t n = idx / 36, k = idx % 36;
        const double base = (k % 7 == 0) ? d.inertia[6 * n + k / 7] : 0.0;
        d.diag[idx] = (base + d.as_j_h[idx]) + d.as_i_h[idx];
    } else if (idx < nh + 6 * size_t(d.N)) {
        const size_t i = idx - nh;
        d.grad[i] = (d.grad[i] + d.as_j_g[i]) + d.as_i_g[i];
    }
}

// K block-level tree reductions (sums, minima or maxima, by Op) at once,
// one value per thread each (blockDim == kBlock), in the order of the plain
// shared-memory tree sh[t] = f(sh[t], sh[t + s]) for s = 128, 64, ..., 1:
// levels 128, 64 and 32 in shared memory, then 16 ... 1 by shuffles in the
// first warp (lane t combines lane t + s exactly as the tree would), with 4
// barriers for all K values.  Every thread receives the results.
struct OpSum { template<class T> __device__ static T f(T a, T b) { return a + b; } };
struct OpMin { __device__ static double f(double a, double b) { return fmin(a, b); } };
struct OpMax { __device__ static double f(double a, double b) { return fmax(a, b); } };

template<class Op, int K, class T> __device__ void block_tree(T (&x)[K], T (*sh)[kBlock])
{
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][t] = x[k];
    __syncthreads();
#pragma unroll
    for (int s = kBlock / 2; s >= 32; s >>= 1) {
        if (t < s) {
#pragma unroll
            for (int k = 0; k < K; ++k) sh[k][t] = Op::f(sh[k][t], sh[k][t + s]);
        }
        __syncthreads();
    }
    if (t < 32) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            T v = sh[k][t];
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) v = Op::f(v, __shfl_down_sync(0xffffffffu, v, s));
            if (t == 0) sh[k][0] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) x[k] = sh[k][0];
    __syncthreads();
}

__device__ __forceinline__ void chunk(uint32_t count, uint32_t &begin, uint32_t &end)
{
    const uint64_t b = uint64_t(blockIdx.x) * count / gridDim.x, e = uint64_t(blockIdx.x + 1) * count / gridDim.x;
    begin = uint32_t(b);
    end = uint32_t(e);
}

// First reduction level over nodes and elements of this block's chunk.
// Final level of the evaluation sums over the per-block partials, in block
// order, published to the host mailbox (run by the last block of
// k_reduce_eval to finish).
__device__ void final_eval(const View &d, double (*sh)[kBlock], unsigned long long (*shu)[kBlock])
{
    double v[6] = {0, 0, 0, 0, 0, 0};  // energy, kinetic, grad2, elastic, contact, and min gap below
    v[5] = __longlong_as_double(0x7ff0000000000000LL);
    unsigned long long u[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < kPartials; b += kBlock) {
        const Partial *p = d.partials + b;
        v[0] += __ldcg(&p->node_energy); v[1] += __ldcg(&p->kinetic); v[2] += __ldcg(&p->grad2);
        v[3] += __ldcg(&p->elastic); v[4] += __ldcg(&p->contact);
        v[5] = fmin(v[5], __ldcg(&p->min_gap));
        u[0] += __ldcg(&p->candidates); u[1] += __ldcg(&p->active); u[2] += (unsigned long long)__ldcg(&p->infeasible);
    }
    double sums[5] = {v[0], v[1], v[2], v[3], v[4]}, mins[1] = {v[5]};
    block_tree<OpSum>(sums, sh);
    block_tree<OpMin>(mins, sh);
    block_tree<OpSum>(u, shu);
    if (threadIdx.x == 0) {
        Mailbox *m = d.mail;
        m->objective = (sums[0] + sums[3]) + sums[4];
        m->elastic = sums[3]; m->contact = sums[4]; m->kinetic = sums[1]; m->minimum_gap = mins[0]; m->grad_norm2 = sums[2];
        m->candidates = u[0]; m->active = u[1]; m->feasible = u[2] ? 0 : 1;
    }
}

// Both reduction levels of an evaluation in one launch: each block sums its
// chunk of nodes and elements into a partial; the last block to finish
// (counted with an atomic after a fence) reduces the partials in block
// order, so the result does not depend on which block that is.
__global__ void __launch_bounds__(kBlock) k_reduce_eval(View d, int gradient)
{
    __shared__ double sh[5][kBlock];
    __shared__ unsigned long long shu[3][kBlock];
    __shared__ bool last;
    uint32_t nb, ne, eb, ee;
    chunk(d.N, nb, ne);
    chunk(d.E, eb, ee);
    double en = 0.0, ki = 0.0, g2 = 0.0, el = 0.0, co = 0.0, mg = __longlong_as_double(0x7ff0000000000000LL);
    unsigned long long cand = 0, act = 0;
    int inf = 0;
    for (uint32_t n = nb + threadIdx.x; n < ne; n += kBlock) {
        en += d.node_energy[n];
        ki += d.node_kinetic[n];
        if (gradient)
            for (int k = 0; k < 6; ++k) { const double g = d.grad[6 * size_t(n) + k]; g2 += g * g; }
    }
    for (uint32_t e = eb + threadIdx.x; e < ee; e += kBlock) {
        el += d.e_el[e];
        co += d.e_co[e];
        cand += d.c_cand[e];
        const uint8_t f = d.c_flags[e];
        if (f & kFlagClosest) mg = fmin(mg, d.c_gap[e]);
        if (f & kFlagActive) ++act;
        if (f & kFlagInfeasible) inf = 1;
    }
    double sums[5] = {en, ki, g2, el, co}, mins[1] = {mg};
    unsigned long long u[3] = {cand, act, (unsigned long long)inf};
    block_tree<OpSum>(sums, sh);
    block_tree<OpMin>(mins, sh);
    block_tree<OpSum>(u, shu);
    if (threadIdx.x == 0) {
        Partial p;
        p.node_energy = sums[0]; p.kinetic = sums[1]; p.grad2 = sums[2]; p.elastic = sums[3]; p.contact = sums[4];
        p.min_gap = mins[0];
        p.candidates = u[0]; p.active = u[1]; p.infeasible = int(u[2] != 0); p.pad = 0;
        d.partials[blockIdx.x] = p;
        __threadfence();
        last = atomicAdd(&d.sc->eval_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    final_eval(d, sh, shu);
    if (threadIdx.x == 0) d.sc->eval_done = 0;
}

// ---- direction ----------------------------------------------------------

// Block-tridiagonal Thomas solve per strand (cuda_backend.cu:866-881) with
// the reference's Gauss-Jordan elimination, partial pivoting on the first
// largest |pivot|, after the relative diagonal shift max(1e-12 max|a_ii|,
// 1e-24) (cuda_backend.cu:855-864).  Strands are taken in length-sorted
// order, longest first, by persistent warps from a work queue, so the
// strands of a warp have similar lengths and the long strands that bound
// the solve start first.
constexpr int kSolveGroup = 6, kSolveGroupsPerWarp = 5;  // float-float kernels: 6 lanes per strand, 5 per warp

// Block Thomas solve with Gauss-Jordan elimination on the augmented block
// [B_n | U_n | rhs_n]: the elimination leaves C_n = B_n^-1 U_n and
// d'_n = B_n^-1 rhs_n in place of U_n and rhs_n (the reference forms
// B_n^-1 first and multiplies; the operations per result entry differ in
// order only).  Finished pivot columns are not updated.  A group of 6 H lanes
// owns one strand: lane (r, h) holds row r, columns [6h/H, 6(h+1)/H) of B_n
// and U_n; every lane of row r holds rhs_n[r].  H = 1 puts 5 strands in a
// warp, H = 2 puts 2 strands in a warp and halves the instructions on each
// strand's sequential chain, H = 3 gives one strand 18 lanes.  Every entry is computed by the same sequence
// of operations in both layouts, so the results are identical bit for bit
// and the launch tuner may pick either.
template<int H> struct AugLayout {
    static constexpr int kCols = 6 / H;              // columns per lane
    static constexpr int kLanes = 6 * H;             // lanes per strand
    static constexpr int kStrands = 32 / kLanes;     // strands per warp
};

// Group g of the strands in solve order [first, end) (end 0: to the last).
template<int H> __device__ __forceinline__ void solve_group_aug(const View &d, uint32_t g, uint32_t first = 0,
                                                                uint32_t end = 0)
{
    using L = AugLayout<H>;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int grp = lane / L::kLanes, gl = lane % L::kLanes, r = gl % 6, h = gl / 6;
    const int base = grp * L::kLanes;
    const int c0 = h * L::kCols;  // first column of this lane
    const uint32_t k = first + g * L::kStrands + uint32_t(grp);
    const bool member = grp < L::kStrands && k < (end ? end : d.S);
    uint32_t begin = 0, len = 0;
    if (member) {
        const uint32_t s = d.sorder[k];
        begin = d.sfirst[s] + d.sfixed[s];
        const uint32_t end = d.sfirst[s] + d.scount[s];
        len = end > begin ? end - begin : 0;
    }
    uint32_t maxlen = len;
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(FULL, maxlen, o));
    double nd[L::kCols], nu[L::kCols], nuc[6], ng = 0.0;
    auto fetch = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) nd[j] = on ? d.diag[36 * n + 6 * r + c0 + j] : 0.0;
        ng = on ? d.grad[6 * n + r] : 0.0;
        const bool up = on && t + 1 < len;
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) nu[j] = up ? d.upper[36 * n + 6 * r + c0 + j] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) nuc[q] = (on && t > 0) ? d.upper[36 * (n - 1) + 6 * q + r] : 0.0;
    };
    fetch(0);
    double Cprev[L::kCols], dprev = 0.0;
#pragma unroll
    for (int j = 0; j < L::kCols; ++j) Cprev[j] = 0.0;
    bool failed = false;
    for (uint32_t t = 0; t < maxlen; ++t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        double a[L::kCols], u[L::kCols], ucol[6], rhs = -ng;
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) { a[j] = nd[j]; u[j] = nu[j]; }
#pragma unroll
        for (int q = 0; q < 6; ++q) ucol[q] = nuc[q];
        if (t + 1 < maxlen) fetch(t + 1);
        if (t > 0) {
            // B = D - U_{n-1}^T C_{n-1}, rhs = -g - U_{n-1}^T d'_{n-1}
#pragma unroll
            for (int q = 0; q < 6; ++q) {
#pragma unroll
                for (int j = 0; j < L::kCols; ++j) a[j] = __fma_rn(-ucol[q], __shfl_sync(FULL, Cprev[j], base + 6 * h + q), a[j]);
                rhs = __fma_rn(-ucol[q], __shfl_sync(FULL, dprev, base + q), rhs);
            }
        }
        // Relative diagonal shift max(1e-12 max|b_ii|, 1e-24).
        double diag_r = 0.0;
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) if (c0 + j == r) diag_r = a[j];
        unsigned long long smax = 0ull;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int owner = base + 6 * (q / L::kCols) + q;
            const unsigned long long b = (unsigned long long)__double_as_longlong(__shfl_sync(FULL, diag_r, owner)) & 0x7fffffffffffffffull;
            smax = b > smax ? b : smax;
        }
        const double shift = fmax(__dmul_rn(1.0e-12, __longlong_as_double((long long)smax)), 1.0e-24);
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) if (c0 + j == r) a[j] = __dadd_rn(a[j], shift);
        // Gauss-Jordan with the pivot rows left unscaled: row r is divided
        // by its pivot (the value at column r when it became the pivot row)
        // once at the end, so each column costs one reciprocal, one product
        // and one fused multiply-add per live entry.
        bool ok = true;
        double ipiv = 1.0;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            const int hc = col / L::kCols, jc = col % L::kCols;
            const int owner_half = base + 6 * hc;
            double acol = 0.0;
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) if (j == jc && h == hc) acol = a[j];
            const unsigned long long mb = (unsigned long long)__double_as_longlong(acol) & 0x7fffffffffffffffull;
            int pivot = col;
            unsigned long long best = __shfl_sync(FULL, mb, owner_half + col);
#pragma unroll
            for (int row = col + 1; row < 6; ++row) {
                const unsigned long long vrow = __shfl_sync(FULL, mb, owner_half + row);
                if (vrow > best) { best = vrow; pivot = row; }
            }
            // best < 1e-30 or not finite (exponent all ones) => failure.
            if (best < 0x39b4484bfeebc2a0ull || best >= 0x7ff0000000000000ull) ok = false;
            const int partner = r == col ? pivot : (r == pivot ? col : r);
            const int src = base + 6 * h + partner;
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) {
                a[j] = __shfl_sync(FULL, a[j], src);
                u[j] = __shfl_sync(FULL, u[j], src);
            }
            rhs = __shfl_sync(FULL, rhs, src);
            acol = 0.0;
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) if (j == jc && h == hc) acol = a[j];
            const double ip = __drcp_rn(__shfl_sync(FULL, acol, owner_half + col));
            const double fp = __dmul_rn(__shfl_sync(FULL, acol, owner_half + r), ip);
            if (r == col) ipiv = ip;
            const int prow = base + 6 * h + col;
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) {
                if (L::kCols * (H - 1) + j <= col) continue;  // finished in every lane
                const double x = __shfl_sync(FULL, a[j], prow);
                a[j] = (r == col) ? a[j] : __fma_rn(-fp, x, a[j]);
            }
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) {
                const double x = __shfl_sync(FULL, u[j], prow);
                u[j] = (r == col) ? u[j] : __fma_rn(-fp, x, u[j]);
            }
            const double xr = __shfl_sync(FULL, rhs, prow);
            rhs = (r == col) ? rhs : __fma_rn(-fp, xr, rhs);
        }
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) u[j] = __dmul_rn(u[j], ipiv);
        rhs = __dmul_rn(rhs, ipiv);
        if (on && !ok) {
            failed = true;
            if (gl == 0) atomicExch(&d.sc->solve_failed, 1);
        }
        // u now holds row r of C_n (zero at the strand tip), rhs = d'_n[r].
#pragma unroll
        for (int j = 0; j < L::kCols; ++j) Cprev[j] = u[j];
        dprev = rhs;
        if (on && !failed) {
#pragma unroll
            for (int j = 0; j < L::kCols; ++j) d.cprime[36 * n + 6 * r + c0 + j] = u[j];
            if (h == 0) d.dprime[6 * n + r] = rhs;
        }
    }
    // Back substitution d_n = d'_n - C_n d_{n+1} (full C row in every lane).
    double next = 0.0;
    double pc[6], pd = 0.0;
    auto fetch_back = [&](uint32_t t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        pd = on ? d.dprime[6 * n + r] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = on ? d.cprime[36 * n + 6 * r + q] : 0.0;
    };
    if (maxlen) fetch_back(maxlen - 1);
    for (uint32_t t = maxlen; t-- > 0;) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        double value = pd, crow[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) crow[q] = pc[q];
        if (t > 0) fetch_back(t - 1);
        const bool coupled = on && t + 1 < len;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double dq = __shfl_sync(FULL, next, base + q);
            if (coupled) value = __fma_rn(-crow[q], dq, value);
        }
        if (on && h == 0) d.dir[6 * n + r] = value;
        next = on ? value : 0.0;
    }
}

// Hybrid schedule: the `long_strands` longest strands one per warp with
// 18 lanes each (the shortest chain per node), then the rest five per warp
// with 6 lanes each (the fewest instructions per node overall).  Both
// layouts compute every entry identically, so the split point does not
// change the result.
__global__ void __launch_bounds__(128) k_block_solve_hybrid(View d, uint32_t long_strands)
{
    const uint32_t rest = d.S > long_strands ? d.S - long_strands : 0;
    const uint32_t groups = long_strands + (rest + AugLayout<1>::kStrands - 1) / AugLayout<1>::kStrands;
    for (;;) {
        uint32_t g = 0;
        if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= groups) break;
        if (g < long_strands) solve_group_aug<3>(d, g);
        else solve_group_aug<1>(d, g - long_strands, long_strands);
    }
}

// ---- long strands on a pair of warps ------------------------------------
//
// On GB300 one FP64 warp instruction holds a sub-partition's FP64 pipe for
// about 64 cycles whatever the number of active lanes, so a strand solved by
// one warp is bound by the FP64 instructions of its per-node chain (about 110
// per node with 18 lanes).  Here the longest strands are solved by two warps
// of one block, which the SM places on two sub-partitions:
// * the B warp holds the Schur complement B_n (lane (r, h): row r, columns
//   2h, 2h+1), adds the relative shift and runs the six pivot steps --
//   pivot search, row swap, pivot reciprocal, row factors, update of the
//   remaining columns -- and publishes each step's pivot row, reciprocal
//   and row factors in shared memory;
// * the U warp holds [U_n | rhs_n] in the same lane layout, applies each
//   published step to it one step behind, scales the rows, stores C_n and
//   d'_n, and forms the next Schur complement B_{n+1} = D_{n+1} - U_n^T C_n
//   and right-hand side, which it hands to the B warp; it also runs the back
//   substitution.
// Every entry goes through the same operations in the same order as in
// solve_group_aug<3>, so the directions are identical bit for bit.  The two
// warps meet at a named barrier (bar.sync, 64 threads) once per pivot step
// and once per node; both execute the same number of barriers by
// construction (same strand length, six steps per node, no early exit).
struct PairShared {
    double B[36];      // B_n, row-major, from the U warp to the B warp
    double fp[2][6];   // row factors a[r][col] * (1 / pivot) of a step (double-buffered by step parity)
    double ip[2];      // the step's pivot reciprocal
    int pivot[2];      // the step's pivot row
    int ok[2];         // no pivot failure in this node up to and including the step
    uint32_t item;     // work item, from the B warp to the U warp
};

__device__ __forceinline__ void pair_barrier(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }

__device__ __forceinline__ void pair_strand_range(const View &d, uint32_t k, uint32_t &begin, uint32_t &len)
{
    const uint32_t s = d.sorder[k];
    begin = d.sfirst[s] + d.sfixed[s];
    const uint32_t end = d.sfirst[s] + d.scount[s];
    len = end > begin ? end - begin : 0;
}

// B warp of a pair (see above): pivot steps on the Schur complements.
__device__ void solve_pair_b(const View &d, uint32_t k, PairShared &sh, int bar)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gl = lane < 18 ? lane : lane - 18;  // lanes 18-31 shadow lanes 0-13 and write nothing
    const int r = gl % 6, h = gl / 6, c0 = 2 * h;
    uint32_t begin, len;
    pair_strand_range(d, k, begin, len);
    for (uint32_t t = 0; t < len; ++t) {
        pair_barrier(bar);  // B_t is in shared memory
        double a[2] = {sh.B[6 * r + c0], sh.B[6 * r + c0 + 1]};
        double diag_r = 0.0;
#pragma unroll
        for (int j = 0; j < 2; ++j) if (c0 + j == r) diag_r = a[j];
        unsigned long long smax = 0ull;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(__shfl_sync(FULL, diag_r, 6 * (q / 2) + q)) &
                                         0x7fffffffffffffffull;
            smax = b > smax ? b : smax;
        }
        const double shift = fmax(__dmul_rn(1.0e-12, __longlong_as_double((long long)smax)), 1.0e-24);
#pragma unroll
        for (int j = 0; j < 2; ++j) if (c0 + j == r) a[j] = __dadd_rn(a[j], shift);
        bool ok = true;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            const int hc = col / 2, jc = col % 2, owner_half = 6 * hc;
            double acol = 0.0;
#pragma unroll
            for (int j = 0; j < 2; ++j) if (j == jc && h == hc) acol = a[j];
            const unsigned long long mb = (unsigned long long)__double_as_longlong(acol) & 0x7fffffffffffffffull;
            int pivot = col;
            unsigned long long best = __shfl_sync(FULL, mb, owner_half + col);
#pragma unroll
            for (int row = col + 1; row < 6; ++row) {
                const unsigned long long vrow = __shfl_sync(FULL, mb, owner_half + row);
                if (vrow > best) { best = vrow; pivot = row; }
            }
            if (best < 0x39b4484bfeebc2a0ull || best >= 0x7ff0000000000000ull) ok = false;
            const int partner = r == col ? pivot : (r == pivot ? col : r);
#pragma unroll
            for (int j = 0; j < 2; ++j) a[j] = __shfl_sync(FULL, a[j], 6 * h + partner);
            acol = 0.0;
#pragma unroll
            for (int j = 0; j < 2; ++j) if (j == jc && h == hc) acol = a[j];
            const double ip = __drcp_rn(__shfl_sync(FULL, acol, owner_half + col));
            const double fp = __dmul_rn(__shfl_sync(FULL, acol, owner_half + r), ip);
            const int prow = 6 * h + col;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                if (2 * 2 + j <= col) continue;  // finished in every lane
                const double x = __shfl_sync(FULL, a[j], prow);
                a[j] = (r == col) ? a[j] : __fma_rn(-fp, x, a[j]);
            }
            const int slot = col & 1;
            if (lane < 6) sh.fp[slot][lane] = fp;
            if (lane == 0) {
                sh.ip[slot] = ip;
                sh.pivot[slot] = pivot;
                sh.ok[slot] = ok ? 1 : 0;
            }
            pair_barrier(bar);  // step published
        }
    }
}

// U warp of a pair (see above): the published steps applied to [U_n | rhs_n],
// the next Schur complement, and the back substitution.
__device__ void solve_pair_u(const View &d, uint32_t k, PairShared &sh, int bar)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gl = lane < 18 ? lane : lane - 18;
    const int r = gl % 6, h = gl / 6, c0 = 2 * h;
    const bool writer = lane < 18;
    uint32_t begin, len;
    pair_strand_range(d, k, begin, len);
    double nd[2], nu[2], nuc[6], ng = 0.0;
    auto fetch = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
#pragma unroll
        for (int j = 0; j < 2; ++j) nd[j] = on ? d.diag[36 * n + 6 * r + c0 + j] : 0.0;
        ng = on ? d.grad[6 * n + r] : 0.0;
        const bool up = on && t + 1 < len;
#pragma unroll
        for (int j = 0; j < 2; ++j) nu[j] = up ? d.upper[36 * n + 6 * r + c0 + j] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) nuc[q] = (on && t > 0) ? d.upper[36 * (n - 1) + 6 * q + r] : 0.0;
    };
    fetch(0);
    double Cprev[2] = {0.0, 0.0}, dprev = 0.0;
    bool failed = false;
    for (uint32_t t = 0; t < len; ++t) {
        const bool on = !failed;
        const size_t n = begin + t;
        double a[2] = {nd[0], nd[1]}, u[2] = {nu[0], nu[1]}, ucol[6], rhs = -ng;
#pragma unroll
        for (int q = 0; q < 6; ++q) ucol[q] = nuc[q];
        if (t + 1 < len) fetch(t + 1);
        if (t > 0) {
#pragma unroll
            for (int q = 0; q < 6; ++q) {
#pragma unroll
                for (int j = 0; j < 2; ++j) a[j] = __fma_rn(-ucol[q], __shfl_sync(FULL, Cprev[j], 6 * h + q), a[j]);
                rhs = __fma_rn(-ucol[q], __shfl_sync(FULL, dprev, q), rhs);
            }
        }
        if (writer) {
            sh.B[6 * r + c0] = a[0];
            sh.B[6 * r + c0 + 1] = a[1];
        }
        pair_barrier(bar);  // hand B_t over
        double ipiv = 1.0;
        bool ok = true;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            pair_barrier(bar);  // step published
            const int slot = col & 1;
            const int pivot = sh.pivot[slot];
            const double fp = sh.fp[slot][r], ip = sh.ip[slot];
            ok = sh.ok[slot] != 0;
            const int partner = r == col ? pivot : (r == pivot ? col : r);
            const int src = 6 * h + partner;
#pragma unroll
            for (int j = 0; j < 2; ++j) u[j] = __shfl_sync(FULL, u[j], src);
            rhs = __shfl_sync(FULL, rhs, src);
            if (r == col) ipiv = ip;
            const int prow = 6 * h + col;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const double x = __shfl_sync(FULL, u[j], prow);
                u[j] = (r == col) ? u[j] : __fma_rn(-fp, x, u[j]);
            }
            const double xr = __shfl_sync(FULL, rhs, prow);
            rhs = (r == col) ? rhs : __fma_rn(-fp, xr, rhs);
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) u[j] = __dmul_rn(u[j], ipiv);
        rhs = __dmul_rn(rhs, ipiv);
        if (on && !ok) {
            failed = true;
            if (lane == 0) atomicExch(&d.sc->solve_failed, 1);
        }
        Cprev[0] = u[0];
        Cprev[1] = u[1];
        dprev = rhs;
        if (on && !failed && writer) {
#pragma unroll
            for (int j = 0; j < 2; ++j) d.cprime[36 * n + 6 * r + c0 + j] = u[j];
            if (h == 0) d.dprime[6 * n + r] = rhs;
        }
    }
    __syncwarp();  // C_n and d'_n written by the other lanes of this warp
    double next = 0.0, pc[6], pd = 0.0;
    auto fetch_back = [&](uint32_t t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        pd = on ? d.dprime[6 * n + r] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = on ? d.cprime[36 * n + 6 * r + q] : 0.0;
    };
    if (len) fetch_back(len - 1);
    for (uint32_t t = len; t-- > 0;) {
        const bool on = !failed;
        const size_t n = begin + t;
        double value = pd, crow[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) crow[q] = pc[q];
        if (t > 0) fetch_back(t - 1);
        const bool coupled = on && t + 1 < len;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double dq = __shfl_sync(FULL, next, q);
            if (coupled) value = __fma_rn(-crow[q], dq, value);
        }
        if (on && h == 0 && writer) d.dir[6 * n + r] = value;
        next = on ? value : 0.0;
    }
}

// Pair schedule: the `long_strands` longest strands each on a pair of
// warps (solve_pair_b / solve_pair_u), then the rest five per warp.  Blocks
// of four warps hold two pairs.  A pair takes work items together while
// they are long strands; at the first item past them both warps go on alone
// through the five-strand groups.
__global__ void __launch_bounds__(128) k_block_solve_pairs(View d, uint32_t long_strands)
{
    __shared__ PairShared shared[2];
    const int warp = threadIdx.x >> 5, pair = warp >> 1, role = warp & 1;
    const int bar = 1 + pair;
    PairShared &sh = shared[pair];
    const uint32_t rest = d.S > long_strands ? d.S - long_strands : 0;
    const uint32_t items = long_strands + (rest + AugLayout<1>::kStrands - 1) / AugLayout<1>::kStrands;
    bool paired = true;
    for (;;) {
        uint32_t g = 0;
        if (paired) {
            if (role == 0 && (threadIdx.x & 31) == 0) sh.item = atomicAdd(&d.sc->solve_next, 1u);
            pair_barrier(bar);
            g = sh.item;
            if (g < long_strands) {
                if (role == 0) solve_pair_b(d, g, sh, bar);
                else solve_pair_u(d, g, sh, bar);
                continue;
            }
            paired = false;  // every later item is a five-strand group
            if (role == 1) {
                if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
                g = __shfl_sync(0xffffffffu, g, 0);
            }
        } else {
            if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
            g = __shfl_sync(0xffffffffu, g, 0);
        }
        if (g >= items) break;
        solve_group_aug<1>(d, g - long_strands, long_strands);
    }
}

// ---- long strands on four warps ------------------------------------------
//
// One warp issues at most one FP64 instruction per ~64 cycles, so a strand
// is bound by the FP64 instructions its busiest warp issues per node (about
// 84 with 18 lanes, 45 on the pair's pivot warp, plus its reciprocals).  A
// quad spreads a strand over the four warps of a block (four sub-partitions):
// * the pivot warp (warp 0) holds B_n in the 18-lane layout, adds the shift
//   and runs the six pivot steps; the reciprocal of every candidate of the
//   step's column is taken on the integer pipes (dm::recip_rn, equal to the
//   FP64 division) while the pivot search runs, so the step's FP64 work is
//   one product and the update of the remaining columns;
// * column warps 1-3 hold columns 2(w-1), 2(w-1)+1 of [U_n], one entry per
//   lane (slots 0-11), and the right-hand side (slots 12-17, used in warp
//   3); they apply each published step one behind, scale the rows, store
//   C_n and d'_n, and form their two columns of the next Schur complement
//   B_{n+1} = D_{n+1} - U_n^T C_n (column c of B needs column c of C only)
//   and, in warp 3, the next right-hand side; warp 1 then runs the back
//   substitution.
// Each entry goes through the same operations in the same order as in
// solve_group_aug<3>, so the directions are identical bit for bit.  The four
// warps meet at a named barrier (128 threads) once per pivot step and once
// per node; all execute the same number by construction (same strand, six
// steps per node, no early exit).  Lanes 18-31 shadow lanes 0-13 (full-warp
// shuffles; they write nothing).
struct QuadShared {
    double B[36];      // B_n, row-major, from the column warps to the pivot warp
    double fp[2][6];   // row factors of a step (double-buffered by step parity)
    double ip[2];      // the step's pivot reciprocal
    int pivot[2];      // the step's pivot row
    int ok[2];         // no pivot failure in this node up to and including the step
    uint32_t item[2];  // work item (double-buffered by fetch parity)
};

__device__ __forceinline__ void quad_barrier(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

__device__ void solve_quad_pivot(const View &d, uint32_t k, QuadShared &sh, int bar)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gl = lane < 18 ? lane : lane - 18;
    const int r = gl % 6, h = gl / 6, c0 = 2 * h;
    uint32_t begin, len;
    pair_strand_range(d, k, begin, len);
    for (uint32_t t = 0; t < len; ++t) {
        quad_barrier(bar);  // B_t is in shared memory
        double a[2] = {sh.B[6 * r + c0], sh.B[6 * r + c0 + 1]};
        double diag_r = 0.0;
#pragma unroll
        for (int j = 0; j < 2; ++j) if (c0 + j == r) diag_r = a[j];
        unsigned long long smax = 0ull;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(__shfl_sync(FULL, diag_r, 6 * (q / 2) + q)) &
                                         0x7fffffffffffffffull;
            smax = b > smax ? b : smax;
        }
        const double shift = fmax(__dmul_rn(1.0e-12, __longlong_as_double((long long)smax)), 1.0e-24);
#pragma unroll
        for (int j = 0; j < 2; ++j) if (c0 + j == r) a[j] = __dadd_rn(a[j], shift);
        bool ok = true;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            const int hc = col / 2, jc = col % 2, owner_half = 6 * hc;
            double acol = 0.0;
#pragma unroll
            for (int j = 0; j < 2; ++j) if (j == jc && h == hc) acol = a[j];
            // Every candidate's reciprocal, alongside the pivot search; the
            // pivot's is the one the 18-lane layout takes after the swap.
            const double rc = dm::recip_rn(acol);
            const unsigned long long mb = (unsigned long long)__double_as_longlong(acol) & 0x7fffffffffffffffull;
            int pivot = col;
            unsigned long long best = __shfl_sync(FULL, mb, owner_half + col);
#pragma unroll
            for (int row = col + 1; row < 6; ++row) {
                const unsigned long long vrow = __shfl_sync(FULL, mb, owner_half + row);
                if (vrow > best) { best = vrow; pivot = row; }
            }
            if (best < 0x39b4484bfeebc2a0ull || best >= 0x7ff0000000000000ull) ok = false;
            const double ip = __shfl_sync(FULL, rc, owner_half + pivot);
            const int partner = r == col ? pivot : (r == pivot ? col : r);
#pragma unroll
            for (int j = 0; j < 2; ++j) a[j] = __shfl_sync(FULL, a[j], 6 * h + partner);
            acol = 0.0;
#pragma unroll
            for (int j = 0; j < 2; ++j) if (j == jc && h == hc) acol = a[j];
            const double fp = __dmul_rn(__shfl_sync(FULL, acol, owner_half + r), ip);
            const int prow = 6 * h + col;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                if (2 * 2 + j <= col) continue;  // finished in every lane
                const double x = __shfl_sync(FULL, a[j], prow);
                a[j] = (r == col) ? a[j] : __fma_rn(-fp, x, a[j]);
            }
            const int slot = col & 1;
            if (lane < 6) sh.fp[slot][lane] = fp;
            if (lane == 0) {
                sh.ip[slot] = ip;
                sh.pivot[slot] = pivot;
                sh.ok[slot] = ok ? 1 : 0;
            }
            quad_barrier(bar);  // step published
        }
    }
}

__device__ void solve_quad_columns(const View &d, uint32_t k, QuadShared &sh, int bar, int w)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int s = lane < 18 ? lane : lane - 18;
    const int r = s % 6, jj = s / 6;                 // jj 0, 1: a column of U; 2: the right-hand side
    const int c = 2 * (w - 1) + (jj < 2 ? jj : 0);
    const bool writer = lane < 18;
    uint32_t begin, len;
    pair_strand_range(d, k, begin, len);
    double nd = 0.0, nu = 0.0, nuc[6], ng = 0.0;
    auto fetch = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
        nd = on ? d.diag[36 * n + 6 * r + c] : 0.0;
        ng = on ? d.grad[6 * n + r] : 0.0;
        nu = (on && t + 1 < len) ? d.upper[36 * n + 6 * r + c] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) nuc[q] = (on && t > 0) ? d.upper[36 * (n - 1) + 6 * q + r] : 0.0;
    };
    fetch(0);
    double prev = 0.0;  // C_{t-1}[r][c] or d'_{t-1}[r]
    bool failed = false;
    for (uint32_t t = 0; t < len; ++t) {
        const bool on = !failed;
        const size_t n = begin + t;
        double acc = jj < 2 ? nd : -ng, ucol[6];
        const double u_next = nu;
#pragma unroll
        for (int q = 0; q < 6; ++q) ucol[q] = nuc[q];
        if (t + 1 < len) fetch(t + 1);
        if (t > 0) {
            // B = D - U_{t-1}^T C_{t-1} (column c), rhs = -g - U_{t-1}^T d'_{t-1}
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                acc = __fma_rn(-ucol[q], __shfl_sync(FULL, prev, 6 * jj + q), acc);
            }
        }
        if (writer && jj < 2) sh.B[6 * r + c] = acc;
        double v = jj < 2 ? u_next : acc;
        quad_barrier(bar);  // hand B_t over
        double ipiv = 1.0;
        bool ok = true;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            quad_barrier(bar);  // step published
            const int slot = col & 1;
            const int pivot = sh.pivot[slot];
            const double fp = sh.fp[slot][r], ip = sh.ip[slot];
            ok = sh.ok[slot] != 0;
            const int partner = r == col ? pivot : (r == pivot ? col : r);
            v = __shfl_sync(FULL, v, 6 * jj + partner);
            if (r == col) ipiv = ip;
            const double x = __shfl_sync(FULL, v, 6 * jj + col);
            v = (r == col) ? v : __fma_rn(-fp, x, v);
        }
        v = __dmul_rn(v, ipiv);
        if (on && !ok) {
            failed = true;
            if (w == 1 && lane == 0) atomicExch(&d.sc->solve_failed, 1);
        }
        prev = v;
        if (on && !failed && writer) {
            if (jj < 2) d.cprime[36 * n + 6 * r + c] = v;
            else if (w == 3) d.dprime[6 * n + r] = v;
        }
    }
    // Back substitution d_n = d'_n - C_n d_{n+1} in warp 1, once the three
    // column warps have stored C and d' (barrier bar + 1, 96 threads).
    asm volatile("bar.sync %0, 96;" ::"r"(bar + 1) : "memory");
    if (w != 1) return;
    double next = 0.0, pc[6], pd = 0.0;
    auto fetch_back = [&](uint32_t t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        pd = on ? d.dprime[6 * n + r] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = on ? d.cprime[36 * n + 6 * r + q] : 0.0;
    };
    if (len) fetch_back(len - 1);
    for (uint32_t t = len; t-- > 0;) {
        const bool on = !failed;
        const size_t n = begin + t;
        double value = pd, crow[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) crow[q] = pc[q];
        if (t > 0) fetch_back(t - 1);
        const bool coupled = on && t + 1 < len;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double dq = __shfl_sync(FULL, next, q);
            if (coupled) value = __fma_rn(-crow[q], dq, value);
        }
        if (on && lane < 6) d.dir[6 * n + r] = value;
        next = on ? value : 0.0;
    }
}

// Tiered schedule over one longest-first queue: the `quads` longest strands
// on a block of four warps each, the next `singles` one per warp (18 lanes),
// the next `doubles` two per warp (12 lanes each), the rest five per warp.
// A block takes queue items together while they are quads; at the first
// item past them its warps go on alone.  Every tier computes each entry
// with the same operations, so the split changes no result.
// The tiers are inlined: as separate functions they would take the View by
// reference, which places the kernel's parameter block in local memory.
__device__ __forceinline__ void tier_quad(const View &d, uint32_t g, QuadShared &sh, int warp)
{
    if (warp == 0) solve_quad_pivot(d, g, sh, 1);
    else solve_quad_columns(d, g, sh, 1, warp);
}
__device__ __forceinline__ void tier_single(const View &d, uint32_t g, uint32_t first) { solve_group_aug<3>(d, g, first); }
__device__ __forceinline__ void tier_double(const View &d, uint32_t g, uint32_t first, uint32_t end)
{
    solve_group_aug<2>(d, g, first, end);
}
__device__ __forceinline__ void tier_five(const View &d, uint32_t g, uint32_t first) { solve_group_aug<1>(d, g, first); }

__global__ void __launch_bounds__(128) k_block_solve_tiers(View d, uint32_t quads, uint32_t singles, uint32_t doubles)
{
    __shared__ QuadShared sh;
    const int warp = threadIdx.x >> 5;
    const uint32_t end1 = quads + singles, end2 = end1 + doubles;
    const uint32_t i2 = end1 + (doubles + 1) / 2;  // first five-strand item
    const uint32_t rest = d.S > end2 ? d.S - end2 : 0;
    const uint32_t items = i2 + (rest + AugLayout<1>::kStrands - 1) / AugLayout<1>::kStrands;
    bool together = quads > 0;
    uint32_t parity = 0;
    for (;;) {
        uint32_t g = 0;
        if (together) {
            if (threadIdx.x == 0) sh.item[parity] = atomicAdd(&d.sc->solve_next, 1u);
            quad_barrier(1);
            g = sh.item[parity];
            parity ^= 1u;
            if (g < quads) {
                tier_quad(d, g, sh, warp);
                continue;
            }
            together = false;  // every later item is a one-warp item
            if (warp != 0) {
                if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
                g = __shfl_sync(0xffffffffu, g, 0);
            }
        } else {
            if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
            g = __shfl_sync(0xffffffffu, g, 0);
        }
        if (g >= items) break;
        if (g < end1) tier_single(d, g - quads, quads);
        else if (g < i2) tier_double(d, g - end1, end1, end2);
        else tier_five(d, g - i2, end2);
    }
}

template<int H> __global__ void __launch_bounds__(128) k_block_solve_aug(View d)
{
    const uint32_t groups = (d.S + AugLayout<H>::kStrands - 1) / AugLayout<H>::kStrands;
    for (;;) {
        uint32_t g = 0;
        if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= groups) break;
        solve_group_aug<H>(d, g);
    }
}

// ---- mixed form: float-float block solve with FP64 refinement -------------
//
// The same block Thomas recurrence as the FP64 solve (per strand, one lane
// per block row, Gauss-Jordan with partial pivoting on the first largest
// |pivot|, relative diagonal shift) evaluated in float-float arithmetic:
// k_ff_factor stores B_n^-1, C_n = B_n^-1 U_n and d'_n and writes the first
// direction; k_ff_residual forms r = -g - A x in FP64 (one thread per row,
// no sequential chain), with the shifts the factorisation used; k_ff_correct
// solves A delta = r with the stored factors and adds delta to the direction
// in FP64.  The float-float factor has about 48 significant bits, so a sweep
// contracts the error by about cond(B) * 2^-48 and one sweep recovers the
// accuracy of the FP64 solve for the condition numbers of these systems
// (block condition numbers up to about 1e10); further sweeps run while the
// largest relative correction of any strand exceeds kRefineRatio.  A pivot
// below 1e-30 or a value outside the FP32 exponent range sets the solve
// failure flag and the host falls back to the FP64 block solve.

constexpr float kRefineRatio = 1.0e-4f;
constexpr int kRefineSweepsMax = 3;

__device__ __forceinline__ void group_range(const View &d, uint32_t warp, int lane, int &r, int &base, uint32_t &begin,
                                            uint32_t &len, uint32_t &maxlen)
{
    const int grp = lane / kSolveGroup;
    r = lane % kSolveGroup;
    base = grp * kSolveGroup;
    const uint32_t k = warp * kSolveGroupsPerWarp + uint32_t(grp);
    const bool member = grp < kSolveGroupsPerWarp && k < d.S;
    begin = 0; len = 0;
    if (member) {
        const uint32_t s = d.sorder[k];
        begin = d.sfirst[s] + d.sfixed[s];
        const uint32_t end = d.sfirst[s] + d.scount[s];
        len = end > begin ? end - begin : 0;
    }
    maxlen = len;
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
}

__device__ __forceinline__ float2 f2(ff::FF a) { return make_float2(a.hi, a.lo); }
__device__ __forceinline__ ff::FF fromf2(float2 a) { return ff::make(a.x, a.y); }

__device__ __forceinline__ void ff_factor_group(const View &d, uint32_t warp)
{
    const int lane = threadIdx.x & 31;
    int r, base;
    uint32_t begin, len, maxlen;
    group_range(d, warp, lane, r, base, begin, len, maxlen);
    double nd[6], nu[6], nuc[6], ng = 0.0;
    auto fetch = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
#pragma unroll
        for (int c = 0; c < 6; ++c) nd[c] = on ? d.diag[36 * n + 6 * r + c] : 0.0;
        ng = on ? d.grad[6 * n + r] : 0.0;
        const bool up = on && t + 1 < len;
#pragma unroll
        for (int c = 0; c < 6; ++c) nu[c] = up ? d.upper[36 * n + 6 * r + c] : 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) nuc[q] = (on && t > 0) ? d.upper[36 * (n - 1) + 6 * q + r] : 0.0;
    };
    fetch(0);
    ff::FF Crow[6], dprev = ff::make(0.0f);
#pragma unroll
    for (int c = 0; c < 6; ++c) Crow[c] = ff::make(0.0f);
    bool failed = false;
    for (uint32_t t = 0; t < maxlen; ++t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        bool bad = false;
        ff::FF a[6], inv[6], urow[6], ucol[6];
        ff::FF rhs = ff::neg(ff::split(ng, bad));
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            a[c] = ff::split(nd[c], bad);
            inv[c] = ff::make(c == r ? 1.0f : 0.0f);
            ucol[c] = ff::split(nuc[c], bad);
            urow[c] = ff::split(nu[c], bad);
        }
        if (t + 1 < maxlen) fetch(t + 1);
        if (t > 0) {
            // B = D - U_{n-1}^T C_{n-1}, rhs = -g - U_{n-1}^T d'_{n-1}
#pragma unroll
            for (int q = 0; q < 6; ++q) {
#pragma unroll
                for (int c = 0; c < 6; ++c) a[c] = ff::fms(a[c], ucol[q], ff::shfl(Crow[c], base + q));
                rhs = ff::fms(rhs, ucol[q], ff::shfl(dprev, base + q));
            }
        }
        // Relative diagonal shift max(1e-12 max|b_ii|, 1e-24); the value used
        // is stored for the FP64 residual.
        ff::FF diag_r = ff::make(0.0f);
#pragma unroll
        for (int c = 0; c < 6; ++c) if (c == r) diag_r = a[c];
        unsigned smax = 0u;
#pragma unroll
        for (int q = 0; q < 6; ++q) smax = max(smax, __shfl_sync(0xffffffffu, ff::abs_bits(diag_r), base + q));
        const float shift = fmaxf(__fmul_rn(1.0e-12f, __uint_as_float(smax)), 1.0e-24f);
#pragma unroll
        for (int c = 0; c < 6; ++c) if (c == r) a[c] = ff::add(a[c], ff::make(shift));
        if (on && r == 0) d.ff_shift[n] = shift;
        bool ok = !bad;
#pragma unroll
        for (int col = 0; col < 6; ++col) {
            ff::FF mine = ff::make(0.0f);
#pragma unroll
            for (int c = 0; c < 6; ++c) if (c == col) mine = a[c];
            const unsigned mb = ff::abs_bits(mine);
            int pivot = col;
            unsigned best = __shfl_sync(0xffffffffu, mb, base + col);
#pragma unroll
            for (int row = col + 1; row < 6; ++row) {
                const unsigned vrow = __shfl_sync(0xffffffffu, mb, base + row);
                if (vrow > best) { best = vrow; pivot = row; }
            }
            // best < 1e-30 or not finite => failure.
            if (best < 0x0da24260u || best >= 0x7f800000u) ok = false;
            const int partner = r == col ? pivot : (r == pivot ? col : r);
#pragma unroll
            for (int c = col; c < 6; ++c) a[c] = ff::shfl(a[c], base + partner);
#pragma unroll
            for (int c = 0; c < 6; ++c) inv[c] = ff::shfl(inv[c], base + partner);
            ff::FF pv = ff::make(1.0f);
#pragma unroll
            for (int c = 0; c < 6; ++c) if (c == col) pv = a[c];
            const ff::FF ip = ff::rcp(ff::shfl(pv, base + col));
            ff::FF f = ff::make(0.0f);
#pragma unroll
            for (int c = 0; c < 6; ++c) if (c == col) f = a[c];
#pragma unroll
            for (int c = col + 1; c < 6; ++c) {
                const ff::FF p = ff::mul(ff::shfl(a[c], base + col), ip);
                a[c] = (r == col) ? p : ff::fms(a[c], f, p);
            }
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const ff::FF p = ff::mul(ff::shfl(inv[c], base + col), ip);
                inv[c] = (r == col) ? p : ff::fms(inv[c], f, p);
            }
        }
        if (on && !ok) {
            failed = true;
            if (r == 0) atomicExch(&d.sc->solve_failed, 1);
        }
        // C_n = B^-1 U_n, d'_n = B^-1 rhs (row q of U_n in lane q).
        ff::FF dn = ff::make(0.0f);
#pragma unroll
        for (int c = 0; c < 6; ++c) Crow[c] = ff::make(0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
#pragma unroll
            for (int c = 0; c < 6; ++c) Crow[c] = ff::fma(Crow[c], inv[q], ff::shfl(urow[c], base + q));
            dn = ff::fma(dn, inv[q], ff::shfl(rhs, base + q));
        }
        dprev = dn;
        if (on && !failed) {
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                d.ff_inv[36 * n + 6 * r + c] = f2(inv[c]);
                d.ff_c[36 * n + 6 * r + c] = f2(Crow[c]);
            }
            d.ff_d[6 * n + r] = f2(dn);
        }
    }
    // Back substitution x_n = d'_n - C_n x_{n+1}.
    ff::FF next = ff::make(0.0f), pc[6], pd = ff::make(0.0f);
    auto fetch_back = [&](uint32_t t) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        pd = on ? fromf2(d.ff_d[6 * n + r]) : ff::make(0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = on ? fromf2(d.ff_c[36 * n + 6 * r + q]) : ff::make(0.0f);
    };
    if (maxlen) fetch_back(maxlen - 1);
    for (uint32_t t = maxlen; t-- > 0;) {
        const bool on = t < len && !failed;
        const size_t n = begin + t;
        ff::FF value = pd, crow[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) crow[q] = pc[q];
        if (t > 0) fetch_back(t - 1);
        const bool coupled = on && t + 1 < len;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const ff::FF xq = ff::shfl(next, base + q);
            if (coupled) value = ff::fms(value, crow[q], xq);
        }
        if (on) d.dir[6 * n + r] = ff::to_double(value);
        next = on ? value : ff::make(0.0f);
    }
}

__global__ void __launch_bounds__(128) k_ff_factor(View d)
{
    const uint32_t groups = (d.S + kSolveGroupsPerWarp - 1) / kSolveGroupsPerWarp;
    for (;;) {
        uint32_t g = 0;
        if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= groups) break;
        ff_factor_group(d, g);
    }
}

// r = -g - (A + shifts) x in FP64, one thread per row of a free node.
__global__ void __launch_bounds__(kBlock) k_ff_residual(View d)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) d.sc->solve_next = 0;  // k_ff_factor has completed
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 6 * d.N) return;
    const uint32_t n = idx / 6, r = idx % 6;
    if (d.fixed[n]) { d.dprime[idx] = 0.0; return; }
    const double *x = d.dir + 6 * size_t(n);
    const double *D = d.diag + 36 * size_t(n) + 6 * r;
    double res = -d.grad[idx] - double(d.ff_shift[n]) * x[r];
#pragma unroll
    for (int c = 0; c < 6; ++c) res -= D[c] * x[c];
    if (d.elem_right[n] >= 0) {
        const double *U = d.upper + 36 * size_t(n) + 6 * r, *xn = x + 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) res -= U[c] * xn[c];
    }
    if (d.elem_left[n] >= 0 && !d.fixed[n - 1]) {
        const double *U = d.upper + 36 * size_t(n - 1) + r, *xp = x - 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) res -= U[6 * c] * xp[c];
    }
    d.dprime[idx] = res;
}

__device__ __forceinline__ void ff_correct_group(const View &d, uint32_t warp)
{
    const int lane = threadIdx.x & 31;
    int r, base;
    uint32_t begin, len, maxlen;
    group_range(d, warp, lane, r, base, begin, len, maxlen);
    double nres = 0.0, nuc[6];
    float2 ninv[6];
    auto fetch = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
        nres = on ? d.dprime[6 * n + r] : 0.0;
#pragma unroll
        for (int c = 0; c < 6; ++c) ninv[c] = on ? d.ff_inv[36 * n + 6 * r + c] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) nuc[q] = (on && t > 0) ? d.upper[36 * (n - 1) + 6 * q + r] : 0.0;
    };
    fetch(0);
    ff::FF dprev = ff::make(0.0f);
    for (uint32_t t = 0; t < maxlen; ++t) {
        const bool on = t < len;
        const size_t n = begin + t;
        bool bad = false;
        ff::FF rhs = ff::split(nres, bad), inv[6], ucol[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) { inv[c] = fromf2(ninv[c]); ucol[c] = ff::split(nuc[c], bad); }
        if (t + 1 < maxlen) fetch(t + 1);
#pragma unroll
        for (int q = 0; q < 6; ++q) rhs = ff::fms(rhs, ucol[q], ff::shfl(dprev, base + q));
        ff::FF dn = ff::make(0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) dn = ff::fma(dn, inv[q], ff::shfl(rhs, base + q));
        dprev = dn;
        if (on) d.ff_d[6 * n + r] = f2(dn);
    }
    ff::FF next = ff::make(0.0f), pc[6], pd = ff::make(0.0f);
    auto fetch_back = [&](uint32_t t) {
        const bool on = t < len;
        const size_t n = begin + t;
        pd = on ? fromf2(d.ff_d[6 * n + r]) : ff::make(0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = on ? fromf2(d.ff_c[36 * n + 6 * r + q]) : ff::make(0.0f);
    };
    if (maxlen) fetch_back(maxlen - 1);
    float dmax = 0.0f, xmax = 0.0f;
    for (uint32_t t = maxlen; t-- > 0;) {
        const bool on = t < len;
        const size_t n = begin + t;
        ff::FF value = pd, crow[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) crow[q] = pc[q];
        if (t > 0) fetch_back(t - 1);
        const bool coupled = on && t + 1 < len;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const ff::FF xq = ff::shfl(next, base + q);
            if (coupled) value = ff::fms(value, crow[q], xq);
        }
        if (on) {
            const double x = d.dir[6 * n + r] + ff::to_double(value);
            d.dir[6 * n + r] = x;
            dmax = fmaxf(dmax, fabsf(value.hi));
            xmax = fmaxf(xmax, fabsf(float(x)));
        }
        next = on ? value : ff::make(0.0f);
    }
    // Largest relative correction of the strand (over its rows) for the
    // host's sweep decision.
    for (int o = 16; o > 0; o >>= 1) {
        dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        xmax = fmaxf(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
    }
    if (lane == 0 && dmax > 0.0f) {
        const float ratio = xmax > 0.0f ? dmax / xmax : 3.0e38f;
        atomicMax(&d.sc->refine_bits, __float_as_uint(ratio));
    }
}

__global__ void __launch_bounds__(128) k_ff_correct(View d)
{
    const uint32_t groups = (d.S + kSolveGroupsPerWarp - 1) / kSolveGroupsPerWarp;
    for (;;) {
        uint32_t g = 0;
        if ((threadIdx.x & 31) == 0) g = atomicAdd(&d.sc->solve_next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= groups) break;
        ff_correct_group(d, g);
    }
}

// Preconditioned steepest descent d = -P g, zero at fixed nodes
// (cuda_backend.cu:632-638).
__global__ void __launch_bounds__(kBlock) k_steepest(View d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * d.N) return;
    d.dir[i] = d.fixed[i / 6] ? 0.0 : -d.grad[i] * d.precond[i];
}

__global__ void __launch_bounds__(kBlock) k_scale(View d, double s)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * d.N) d.dir[i] *= s;
}

// The trust-radius limit applied on the device (pipelined iteration): the
// same scale trust / max_translation as the host applies after reading the
// reduction, when the direction's largest translation exceeds the radius.
__global__ void __launch_bounds__(kBlock) k_scale_trust(View d, double trust)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const double mt = d.sc->max_translation;
    if (i < 6 * d.N && mt > trust) d.dir[i] *= trust / mt;
}

// g.d, |d|^2 and the largest free-node translation of d.
__global__ void __launch_bounds__(kBlock) k_reduce_dir(View d)
{
    __shared__ double sh2[2][kBlock];
    uint32_t nb, ne;
    chunk(d.N, nb, ne);
    double gd = 0.0, dd = 0.0, mx = 0.0;
    for (uint32_t n = nb + threadIdx.x; n < ne; n += kBlock) {
        for (int k = 0; k < 6; ++k) {
            const double x = d.dir[6 * size_t(n) + k];
            gd += d.grad[6 * size_t(n) + k] * x;
            dd += x * x;
        }
        if (!d.fixed[n]) mx = fmax(mx, dm::norm(load3(d.dir + 6 * size_t(n))));
    }
    double sums[2] = {gd, dd}, maxs[1] = {mx};
    block_tree<OpSum>(sums, sh2);
    block_tree<OpMax>(maxs, sh2);
    if (threadIdx.x == 0) {
        DirPartial p;
        p.slope = sums[0];
        p.dnorm2 = sums[1];
        p.max_translation = maxs[0];
        d.dpartials[blockIdx.x] = p;
    }
}

// ccd_pass: the CCD pass of a pipelined iteration, which leaves the
// direction pass's values (dir_*) in the mailbox.
__global__ void __launch_bounds__(kBlock) k_final_dir(View d, int ccd_pass)
{
    __shared__ double sh2[2][kBlock];
    double gd = 0, dd = 0, mx = 0;
    for (int b = threadIdx.x; b < kPartials; b += kBlock) {
        const DirPartial p = d.dpartials[b];
        gd += p.slope; dd += p.dnorm2; mx = fmax(mx, p.max_translation);
    }
    double sums[2] = {gd, dd}, maxs[1] = {mx};
    block_tree<OpSum>(sums, sh2);
    block_tree<OpMax>(maxs, sh2);
    gd = sums[0]; dd = sums[1]; mx = maxs[0];
    if (threadIdx.x == 0) {
        d.mail->slope = gd; d.mail->dir_norm2 = dd; d.mail->max_translation = mx;
        d.sc->max_translation = mx;
        d.mail->ccd_bits = d.sc->ccd_bits;
        d.mail->solve_failed = d.sc->solve_failed;
        if (!ccd_pass) {
            d.mail->dir_slope = gd; d.mail->dir_max_translation = mx; d.mail->dir_solve_failed = d.sc->solve_failed;
        }
        // The first line-search step as the host forms it: 0.9 x the CCD
        // bound below 1, else 1 (no collider: 1).
        const double lim = __longlong_as_double((long long)d.sc->ccd_bits);
        d.sc->trial_alpha = d.has_collider ? (lim < 1.0 ? __dmul_rn(lim, 0.9) : lim) : 1.0;
        d.mail->pair_count = d.sc->pair_count;
        d.mail->refine_bits = d.sc->refine_bits;
        d.sc->ccd_bits = 0x3ff0000000000000ULL;  // 1.0
        d.sc->solve_failed = 0;
        d.sc->pair_count = 0;
        d.sc->solve_next = 0;
        d.sc->ccd_near = 0;
        d.sc->refine_bits = 0;
    }
}

// Line-search CCD bound (cuda_backend.cu:989-1000); the minimum over all
// elements and candidates is taken with an unsigned atomicMin on the bit
// pattern of the non-negative step.
template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_ccd(View d)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    if (d.fixed[i] || !d.econtact[e]) return;
    const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
    const V d0 = load3(d.dir + 6 * size_t(i)), d1 = load3(d.dir + 6 * size_t(j));
    const V lo = dm::vmin(dm::vmin(p0, p1), dm::vmin(p0 + d0, p1 + d1));
    const V hi = dm::vmax(dm::vmax(p0, p1), dm::vmax(p0 + d0, p1 + d1));
    const double target = d.radius + d.offset + d.min_gap;
    double local = 1.0;
    const dm::F3 f0 = dm::f3(0.f, 0.f, 0.f), f1 = dm::to_local(p1, p0);
    bvh_walk<MIXED>(d, lo, hi, target, [&](uint32_t t) {
        const double speed = fmax(dm::gnorm(d0), dm::gnorm(d1));
        if (speed < 1e-30) return;
        const V a = tri_vertex(d, t, 0), b = tri_vertex(d, t, 1), c = tri_vertex(d, t, 2);
        if (MIXED) {
            // Skip candidates whose first advancement step provably reaches 1.
            float m;
            const float df = dm::segment_triangle_distance_f(f0, f1, dm::to_local(a, p0), dm::to_local(b, p0),
                                                              dm::to_local(c, p0), m);
            if (0.8 * (double(df) - double(m) - target) >= speed * (1.0 + 1e-6)) return;
        }
        double alpha = 0.0;
        // Mixed form: every limit this candidate can still produce is
        // >= 0.9 alpha (alpha only grows), so it stops as soon as that
        // reaches the best limit known (its element's or the global one);
        // the minimum is unchanged.
        double bound = local;
        if (MIXED) bound = fmin(bound, __longlong_as_double(*reinterpret_cast<volatile long long *>(&d.sc->ccd_bits)));
        for (int k = 0; k < 80; ++k) {
            if (MIXED && 0.9 * alpha >= bound) return;
            const double dist = dm::closest_segment_triangle(dm::gadd(p0, dm::gmul(d0, alpha)), dm::gadd(p1, dm::gmul(d1, alpha)), a, b, c).distance;
            const double clear = dist - target;
            if (clear <= 0) { local = fmin(local, fmax(0.0, alpha * 0.9)); return; }
            const double advance = 0.8 * clear / speed;
            if (alpha + advance >= 1) return;
            if (advance < 1e-12) { local = fmin(local, alpha); return; }
            alpha += advance;
        }
        local = fmin(local, alpha);
    });
    if (local < 1.0) atomicMin(&d.sc->ccd_bits, (unsigned long long)__double_as_longlong(local));
}

// Mixed-form CCD, load balanced: k_ccd_collect lists every (element,
// triangle) candidate whose FP32 lower-bound clearance does not already let
// the first advancement step reach alpha = 1; k_ccd_pairs runs the exact FP64
// conservative advancement of cuda_backend.cu:989-1000 per listed pair and
// stops a pair once 0.9 alpha reaches the global minimum found so far (every
// limit the pair could still produce is >= 0.9 alpha).  The minimum equals
// the per-element kernel's.
// Candidates of the swept element box (positions at step 0 and 1) whose
// FP32 lower-bound distance does not rule out a limit below 1: a pair is
// skipped only when even the lower bound of 0.8 (dist - target) reaches the
// speed, so the first advancement step of the exact pass would leave the
// step unlimited anyway.  When all four swept end points stay within the
// slack of the element's leaf cache, the cached leaves (collected with the
// contact padding, which is at least the CCD target) hold every leaf the
// swept box can touch and replace the tree walk.
__global__ void __launch_bounds__(kBlock) k_ccd_collect(View d)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    if (d.fixed[i] || !d.econtact[e]) return;
    const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
    const V d0 = load3(d.dir + 6 * size_t(i)), d1 = load3(d.dir + 6 * size_t(j));
    const double speed = fmax(dm::gnorm(d0), dm::gnorm(d1));
    if (speed < 1e-30) return;
    const V e0 = p0 + d0, e1 = p1 + d1;
    const V lo = dm::vmin(dm::vmin(p0, p1), dm::vmin(e0, e1));
    const V hi = dm::vmax(dm::vmax(p0, p1), dm::vmax(e0, e1));
    const double target = d.radius + d.offset + d.min_gap;
    const dm::F3 origin = dm::f3(d.q32[3 * size_t(i)], d.q32[3 * size_t(i) + 1], d.q32[3 * size_t(i) + 2]);
    const dm::F3 f0 = dm::f3(0.f, 0.f, 0.f);
    const dm::F3 f1 = dm::f3(d.q32[3 * size_t(j)] - origin.x, d.q32[3 * size_t(j) + 1] - origin.y,
                             d.q32[3 * size_t(j) + 2] - origin.z);
    const float target_ru = __double2float_ru(target);
    const float speed_ru = __fmul_ru(__double2float_ru(speed), 1.000002f);
    const QueryBox qb = make_query(lo, hi, target);
    auto test = [&](uint32_t p) {
        float m;
        uint32_t t;
        const float df = record_distance_f(d, p, origin, f0, f1, m, t);
        if (__fmul_rd(0.8f, __fsub_rd(__fsub_rd(df, m), target_ru)) >= speed_ru) return;
        const uint32_t slot = append_slot(&d.sc->pair_count);
        if (slot < d.pair_capacity) { d.pair_elem[slot] = e; d.pair_tri[slot] = t; }
    };
    const uint8_t nl = d.cache_n[e];
    bool cached = nl != kCacheInvalid && d.dhat >= d.min_gap;
    if (cached) {
        const float *c = d.cache_x32 + 6 * size_t(e);
        const dm::F3 xj32 = dm::f3(d.q32[3 * size_t(j)], d.q32[3 * size_t(j) + 1], d.q32[3 * size_t(j) + 2]);
        const dm::F3 a0 = dm::f3(float(e0.x), float(e0.y), float(e0.z)), a1 = dm::f3(float(e1.x), float(e1.y), float(e1.z));
        cached = within_cache_slack(c, origin, xj32) && within_cache_slack(c, a0, a1);
    }
    if (cached) {
        // k_ccd_near tests the cached leaves, one warp per element.
        if (nl > 0) d.near_list[append_slot(&d.sc->ccd_near)] = e;
    } else {
        bvh_positions_packed(d, qb, test);
    }
}

// One warp per element queued by k_ccd_collect: lane l tests cached leaf l
// against the swept box and applies the same FP32 skip bound to that leaf's
// triangles (the pair order does not matter: the bound is a minimum).
__global__ void __launch_bounds__(kBlock) k_ccd_near(View d)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t count = d.sc->ccd_near;
    const double target = d.radius + d.offset + d.min_gap;
    const float target_ru = __double2float_ru(target);
    for (uint32_t k = warp; k < count; k += nwarps) {
        const uint32_t e = d.near_list[k];
        uint32_t nleaves = 0;
        const uint32_t *leaves = cached_leaves(d, e, d.cache_n[e], nleaves);
        if (uint32_t(lane) >= nleaves) continue;
        const uint32_t i = d.ei[e], j = d.ej[e];
        const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
        const V d0 = load3(d.dir + 6 * size_t(i)), d1 = load3(d.dir + 6 * size_t(j));
        const double speed = fmax(dm::gnorm(d0), dm::gnorm(d1));
        const V e0 = p0 + d0, e1 = p1 + d1;
        const QueryBox qb = make_query(dm::vmin(dm::vmin(p0, p1), dm::vmin(e0, e1)), dm::vmax(dm::vmax(p0, p1), dm::vmax(e0, e1)),
                                       target);
        const dm::F3 origin = dm::f3(d.q32[3 * size_t(i)], d.q32[3 * size_t(i) + 1], d.q32[3 * size_t(i) + 2]);
        const dm::F3 f0 = dm::f3(0.f, 0.f, 0.f);
        const dm::F3 f1 = dm::f3(d.q32[3 * size_t(j)] - origin.x, d.q32[3 * size_t(j) + 1] - origin.y,
                                 d.q32[3 * size_t(j) + 2] - origin.z);
        const float speed_ru = __fmul_ru(__double2float_ru(speed), 1.000002f);
        // Lane l takes leaves l, l + 32, ... of the cached list.
        for (uint32_t c = lane; c < nleaves; c += 32) {
            const uint32_t node = leaves[c];
            const float4 a = __ldg(d.bnode + 2 * size_t(node)), b = __ldg(d.bnode + 2 * size_t(node) + 1);
            if (!maybe_overlap(qb, a, b) || !leaf_overlap_exact(d, node, a, b, qb)) continue;
            const uint32_t leaf = __float_as_uint(b.w), first = leaf >> 4, cnt = leaf & 15u;
            for (uint32_t p = first; p < first + cnt; ++p) {
                float m;
                uint32_t t;
                const float df = record_distance_f(d, p, origin, f0, f1, m, t);
                if (__fmul_rd(0.8f, __fsub_rd(__fsub_rd(df, m), target_ru)) >= speed_ru) continue;
                const uint32_t slot = append_slot(&d.sc->pair_count);
                if (slot < d.pair_capacity) { d.pair_elem[slot] = e; d.pair_tri[slot] = t; }
            }
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_ccd_pairs(View d)
{
    const uint32_t count = min(d.sc->pair_count, d.pair_capacity);
    const double target = d.radius + d.offset + d.min_gap;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const uint32_t e = d.pair_elem[k], t = d.pair_tri[k];
        const uint32_t i = d.ei[e], j = d.ej[e];
        const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
        const V d0 = load3(d.dir + 6 * size_t(i)), d1 = load3(d.dir + 6 * size_t(j));
        const double speed = fmax(dm::gnorm(d0), dm::gnorm(d1));
        const V a = tri_vertex(d, t, 0), b = tri_vertex(d, t, 1), c = tri_vertex(d, t, 2);
        double limit = 2.0;  // no limit
        double alpha = 0.0;
        const double bound = __longlong_as_double(*reinterpret_cast<volatile long long *>(&d.sc->ccd_bits));
        bool done = false;
        for (int it = 0; it < 80 && !done; ++it) {
            if (0.9 * alpha >= bound) { done = true; break; }
            const double dist = dm::closest_segment_triangle(dm::gadd(p0, dm::gmul(d0, alpha)), dm::gadd(p1, dm::gmul(d1, alpha)), a, b, c).distance;
            const double clear = dist - target;
            if (clear <= 0) { limit = fmax(0.0, alpha * 0.9); done = true; break; }
            const double advance = 0.8 * clear / speed;
            if (alpha + advance >= 1) { done = true; break; }
            if (advance < 1e-12) { limit = alpha; done = true; break; }
            alpha += advance;
        }
        if (!done) limit = alpha;
        if (limit < 1.0) atomicMin(&d.sc->ccd_bits, (unsigned long long)__double_as_longlong(limit));
    }
}

// ---- end of substep -------------------------------------------------------

__global__ void __launch_bounds__(kBlock) k_update_velocity(View d, double inv_dt)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N || d.fixed[n]) return;
    for (int k = 0; k < 6; ++k) d.v[6 * size_t(n) + k] = (d.q[6 * size_t(n) + k] - d.q_old[6 * size_t(n) + k]) * inv_dt;
}

// Coulomb friction impulse (cuda_backend.cu:941-964); each element writes
// its velocity change into its left/right node slots.
template<bool MIXED> __global__ void __launch_bounds__(kBlock) k_friction(View d, double dt)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const uint32_t i = d.ei[e], j = d.ej[e];
    double di[3] = {0, 0, 0}, dj[3] = {0, 0, 0};
    const bool fi = d.fixed[i], fj = d.fixed[j];
    if (d.econtact[e] && !(fi && fj)) {
        const V p0 = load3(d.q + 6 * size_t(i)), p1 = load3(d.q + 6 * size_t(j));
        uint32_t cand = 0, closest;
        dm::ClosestPair pair;
        if (MIXED && !fi) {
            // The last gradient evaluation ran the contact pass at this q and
            // this collider state: reuse its closest pair.
            closest = d.c_tri[e];
            pair.t = d.c_t[e]; pair.distance = d.c_dist[e]; pair.bary = load3(d.c_bary + 3 * size_t(e));
        } else {
            closest = closest_triangle<MIXED>(d, p0, p1, d.radius + d.offset + d.dhat, cand, pair);
        }
        const double gap = pair.distance - d.radius - d.offset;
        if (closest != kNone && gap > 0.0 && gap < d.dhat) {
            const double w0 = 1.0 - pair.t, w1 = pair.t;
            const V hair = p0 * w0 + p1 * w1;
            const V body = tri_vertex(d, closest, 0) * pair.bary.x + tri_vertex(d, closest, 1) * pair.bary.y +
                           tri_vertex(d, closest, 2) * pair.bary.z;
            const V ob = load3(d.col_old + 3 * size_t(d.tri[3 * closest])) * pair.bary.x +
                         load3(d.col_old + 3 * size_t(d.tri[3 * closest + 1])) * pair.bary.y +
                         load3(d.col_old + 3 * size_t(d.tri[3 * closest + 2])) * pair.bary.z;
            const V normal = (hair - body) * (1.0 / fmax(pair.distance, 1.0e-15));
            const V v0 = load3(d.v + 6 * size_t(i)), v1 = load3(d.v + 6 * size_t(j));
            const V rel = v0 * w0 + v1 * w1 - (body - ob) * (1.0 / dt);
            const V tangent = rel - normal * dm::dot(normal, rel);
            const double ts = dm::norm(tangent);
            double im = 0.0;
            if (!fi) im += w0 * w0 / fmax(d.mass[i], 1.0e-30);
            if (!fj) im += w1 * w1 / fmax(d.mass[j], 1.0e-30);
            if (!(ts < 1.0e-15) && im > 0.0) {
                const double aa = d.dhat - gap, lg = log(gap / d.dhat);
                const double fn = d.kc * (aa * aa / gap - 2.0 * aa * lg), required = ts / im;
                const double mag = fmin(required, d.friction * fn * dt), smooth = d.smoothing / dt;
                const V imp = tangent * (-mag / fmax(sqrt(ts * ts + smooth * smooth), 1.0e-30));
                if (!fi) { const double s = w0 / fmax(d.mass[i], 1.0e-30); di[0] = imp.x * s; di[1] = imp.y * s; di[2] = imp.z * s; }
                if (!fj) { const double s = w1 / fmax(d.mass[j], 1.0e-30); dj[0] = imp.x * s; dj[1] = imp.y * s; dj[2] = imp.z * s; }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) { d.as_i_f[3 * size_t(i) + k] = di[k]; d.as_j_f[3 * size_t(j) + k] = dj[k]; }
}

__global__ void __launch_bounds__(kBlock) k_friction_apply(View d)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) d.v[6 * size_t(n) + k] += d.as_j_f[3 * size_t(n) + k] + d.as_i_f[3 * size_t(n) + k];
}

__global__ void k_init_scalars(View d)
{
    if (threadIdx.x || blockIdx.x) return;
    d.sc->ccd_bits = 0x3ff0000000000000ULL;
    d.sc->sweep_fail = kNone;
    d.sc->solve_failed = 0;
    d.sc->pair_count = 0;
    d.sc->surv_count = 0;
    d.sc->solve_next = 0;
    d.sc->refine_bits = 0;
    d.sc->near_count = 0;
    d.sc->ccd_near = 0;
    d.sc->pool_used = 0;
    d.sc->eval_done = 0;
}

__global__ void __launch_bounds__(kBlock) k_gather(const double *q, const uint32_t *map, uint32_t count, double *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t n = map ? map[i] : i;
    out[3 * size_t(i)] = q[6 * size_t(n)];
    out[3 * size_t(i) + 1] = q[6 * size_t(n) + 1];
    out[3 * size_t(i) + 2] = q[6 * size_t(n) + 2];
}

// ---- root targets (src/solver.cpp:416-447) --------------------------------
//
// Target positions and rotation vectors of every node for one set of
// evaluated source points: positions and unit tangents, the tangent-only
// part of each frame step (thread per node), the frame walk along each
// strand (thread per strand, longest strands first), then the rotation
// vector of frame * reference^T (thread per node).

struct RootArgs {
    uint32_t N, S;
    const double *points;                    // [P][3] evaluated source points
    const uint32_t *bind_l, *bind_r;         // the two source points a node interpolates
    const double *bind_t;
    const uint32_t *node_strand, *sfirst, *scount, *sorder;
    const double *ref;                       // [N][9] reference frames
    double *x, *tangent, *frame, *rot;       // [N][3], [N][3], [N][9], [N][3]
    uint32_t *bad;                           // nonzero after a degenerate tangent
};

__device__ __forceinline__ V root_position(const RootArgs &a, uint32_t n)
{
    return dm::glerp(load3(a.points + 3 * size_t(a.bind_l[n])), load3(a.points + 3 * size_t(a.bind_r[n])), a.bind_t[n]);
}

// Central-difference tangents, one-sided at the strand ends
// (solver.cpp:426-433); a squared length below 1e-24 fails the whole call.
__global__ void __launch_bounds__(kBlock) k_root_tangents(RootArgs a)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const uint32_t s = a.node_strand[n], k = n - a.sfirst[s], count = a.scount[s];
    const V x = root_position(a, n);
    store3(a.x + 3 * size_t(n), x);
    V d;
    if (k == 0) d = dm::gsub(root_position(a, n + 1), x);
    else if (k + 1 == count) d = dm::gsub(x, root_position(a, n - 1));
    else d = dm::gsub(root_position(a, n + 1), root_position(a, n - 1));
    if (dm::gdot(d, d) < 1.0e-24) atomicOr(a.bad, 1u);
    store3(a.tangent + 3 * size_t(n), dm::gunit(d));
}

// Everything of the frame walk that depends on the tangents alone, per node:
// d3 (the tangent normalised once more, as frame_from_tangent does) and the
// minimal rotation from the previous node's tangent, packed into the node's
// frame slot [d3, n, s, c, kind] until k_root_frames replaces it.
__global__ void __launch_bounds__(kBlock) k_root_transport(RootArgs a)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const V t = load3(a.tangent + 3 * size_t(n));
    double *p = a.frame + 9 * size_t(n);
    store3(p, dm::gunit(t));
    dm::Transport tr{};
    tr.kind = 1;
    if (n != a.sfirst[a.node_strand[n]]) tr = dm::transport_between(load3(a.tangent + 3 * size_t(n - 1)), t);
    store3(p + 3, tr.n);
    p[6] = tr.s; p[7] = tr.c; p[8] = double(tr.kind);
}

// The sequential part (solver.cpp:435-443): each frame's first column is the
// previous one carried by the minimal rotation between consecutive tangents.
// One thread per strand, longest strands first.
__global__ void __launch_bounds__(kBlock) k_root_frames(RootArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.S) return;
    const uint32_t s = a.sorder[i], first = a.sfirst[s], count = a.scount[s];
    const double *r0 = a.ref + 9 * size_t(first);
    double *p = a.frame + 9 * size_t(first);
    M f = dm::frame_from_d3(load3(p), dm::v(r0[0], r0[3], r0[6]));
#pragma unroll
    for (int c = 0; c < 9; ++c) p[c] = f.m[c];
    for (uint32_t k = 1; k < count; ++k) {
        p += 9;
        dm::Transport tr;
        tr.n = load3(p + 3); tr.s = p[6]; tr.c = p[7]; tr.kind = int(p[8]);
        f = dm::frame_from_d3(load3(p), dm::transport_apply(tr, dm::v(f.m[0], f.m[3], f.m[6])));
#pragma unroll
        for (int c = 0; c < 9; ++c) p[c] = f.m[c];
    }
}

__global__ void __launch_bounds__(kBlock) k_root_rotations(RootArgs a)
{
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const M r = dm::times_transpose(load9(a.frame + 9 * size_t(n)), load9(a.ref + 9 * size_t(n)));
    store3(a.rot + 3 * size_t(n), dm::rotation_vector(r));
}

// ---- device memory --------------------------------------------------------

struct Arena {
    char *base = nullptr;
    size_t size = 0, used = 0;
    template<class T> T *take(size_t count)
    {
        const size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        T *p = reinterpret_cast<T *>(base + used);
        used += bytes;
        return p;
    }
};

template<class T> size_t padded(size_t count) { return (count * sizeof(T) + 255) & ~size_t(255); }

}  // namespace

struct Engine::Impl {
    View v{};
    Arena arena;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;          // contact passes beside the node kernel
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    Mailbox *mail_host = nullptr;
    SweepRecord *sweep_host = nullptr;
    // Host copies needed by the control flow.
    std::vector<uint32_t> mapping;
    uint32_t original_count = 0;
    double *mapping_gather_out = nullptr;
    uint32_t *mapping_dev = nullptr;
    double *q_snap = nullptr, *v_snap = nullptr;
    double *root_cur_x = nullptr, *root_cur_r = nullptr, *root_pend_x = nullptr, *root_pend_r = nullptr;
    double *col_frame_start = nullptr, *col_pending = nullptr;
    double *anim_root_x = nullptr, *anim_root_r = nullptr, *anim_col = nullptr;
    size_t anim_bytes = 0, ring_bytes = 0;
    double *col_a_copy = nullptr;  // frame-start copy used while stepping
    // Root targets on the device: the two source points each node
    // interpolates and its strand (arena), and the work arrays of one pass
    // (allocated on first use: points [P][3], positions, tangents, frames,
    // rotation vectors, the degenerate-tangent flag).
    uint32_t *bind_l = nullptr, *bind_r = nullptr, *node_strand = nullptr;
    double *bind_t = nullptr;
    char *root_work = nullptr;
    RootArgs root{};
    std::vector<uint8_t> fixed_host;
    uint64_t resident = 0;

    // Per-kernel device-time accounting (CUDA events on this stream).
    struct KernelStat { const char *name; uint64_t launches; double ms; };
    bool profiling = false;
    uint64_t launches = 0;
    unsigned solve_blocks = 0;  // launch shape of the FP64 block solve (0 = not tuned yet)
    // Rollback ring: q and v of the last ring_frame.size() animation frames,
    // slot k holding frame ring_frame[k] (-1 = empty), [slots][2][N][6] FP64.
    double *ring = nullptr;
    std::vector<int64_t> ring_frame;
    // Output ring: the original points' positions of the last
    // out_frame.size() animation frames, gathered on the solver's stream after
    // each frame and copied to pinned host memory on copy_stream, so the copy
    // overlaps the next frame ([slots][P][3] FP64 on both sides).
    cudaStream_t copy_stream = nullptr;
    double *out_dev = nullptr, *out_host = nullptr;
    std::vector<cudaEvent_t> out_gathered, out_copied;
    std::vector<int64_t> out_frame;
    size_t out_bytes = 0;
    uint32_t out_next = 0;
    void release_output()
    {
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (cudaEvent_t e : out_gathered) cudaEventDestroy(e);
        for (cudaEvent_t e : out_copied) cudaEventDestroy(e);
        out_gathered.clear();
        out_copied.clear();
        if (out_dev) cudaFree(out_dev);
        if (out_host) cudaFreeHost(out_host);
        out_dev = out_host = nullptr;
        resident -= out_bytes;
        out_bytes = 0;
        out_frame.clear();
        out_next = 0;
    }
    void (*solve_kernel)(View) = nullptr;
    uint32_t solve_long = 0;  // > 0: k_block_solve_hybrid / k_block_solve_pairs with this many long strands
    bool solve_pairs = false; // the long strands on warp pairs (k_block_solve_pairs)
    bool solve_tiers = false; // k_block_solve_tiers with tier_quads / tier_singles / tier_doubles
    uint32_t tier_quads = 0, tier_singles = 0, tier_doubles = 0;
    std::vector<uint32_t> sorted_len;  // free nodes per strand, in the solve order
    unsigned ff_blocks = 0;     // launch shape of the float-float kernels
    std::vector<KernelStat> kstats;
    std::vector<std::pair<size_t, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> pool;

    cudaEvent_t take_event()
    {
        if (pool.empty()) {
            cudaEvent_t e;
            KHS_CUDA(cudaEventCreate(&e));
            return e;
        }
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    size_t stat_index(const char *name)
    {
        for (size_t k = 0; k < kstats.size(); ++k)
            if (kstats[k].name == name) return k;
        kstats.push_back({name, 0, 0.0});
        return kstats.size() - 1;
    }
    // A launch on stream s (the solver's stream, or the side stream, which
    // is only used while kernels are not timed one by one).
    template<class K, class... A> void launch_on(cudaStream_t s, const char *name, K kernel, unsigned grid, unsigned block,
                                                 A... args)
    {
        if (s == stream) {
            launch(name, kernel, grid, block, args...);
            return;
        }
        ++launches;
        kernel<<<grid, block, 0, s>>>(args...);
    }
    template<class K, class... A> void launch(const char *name, K kernel, unsigned grid, unsigned block, A... args)
    {
        ++launches;
        if (!profiling) {
            kernel<<<grid, block, 0, stream>>>(args...);
            return;
        }
        cudaEvent_t a = take_event(), b = take_event();
        KHS_CUDA(cudaEventRecord(a, stream));
        kernel<<<grid, block, 0, stream>>>(args...);
        KHS_CUDA(cudaEventRecord(b, stream));
        pending.push_back({stat_index(name), {a, b}});
    }
    void resolve()
    {
        for (auto &p : pending) {
            float ms = 0.0f;
            KHS_CUDA(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
            kstats[p.first].launches += 1;
            kstats[p.first].ms += ms;
            pool.push_back(p.second.first);
            pool.push_back(p.second.second);
        }
        pending.clear();
    }

    ~Impl()
    {
        for (auto &p : pending) { pool.push_back(p.second.first); pool.push_back(p.second.second); }
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
        if (arena.base) cudaFree(arena.base);
        if (ring) cudaFree(ring);
        if (anim_root_x) cudaFree(anim_root_x);
        if (root_work) cudaFree(root_work);
        release_output();
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (mail_host) cudaFreeHost(mail_host);
        if (sweep_host) cudaFreeHost(sweep_host);
        if (ev_begin) cudaEventDestroy(ev_begin);
        if (ev_end) cudaEventDestroy(ev_end);
        if (side) cudaStreamDestroy(side);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (stream) cudaStreamDestroy(stream);
    }
    void sync()
    {
        KHS_CUDA(cudaStreamSynchronize(stream));
        if (!pending.empty()) resolve();
    }
    void check() { KHS_CUDA(cudaGetLastError()); }
};

Engine::Engine() : d_(new Impl) {}
Engine::~Engine() = default;

void Engine::initialize(const Model &m, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                        const std::vector<Vec> &root_pos, const std::vector<Vec> &root_rot)
{
    Impl &I = *d_;
    KHS_CUDA(cudaSetDevice(0));
    KHS_CUDA(cudaStreamCreateWithFlags(&I.stream, cudaStreamNonBlocking));
    KHS_CUDA(cudaStreamCreateWithFlags(&I.side, cudaStreamNonBlocking));
    KHS_CUDA(cudaEventCreateWithFlags(&I.fork, cudaEventDisableTiming));
    KHS_CUDA(cudaEventCreateWithFlags(&I.join, cudaEventDisableTiming));
    KHS_CUDA(cudaEventCreate(&I.ev_begin));
    KHS_CUDA(cudaEventCreate(&I.ev_end));
    KHS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&I.mail_host), sizeof(Mailbox), cudaHostAllocMapped));
    KHS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&I.sweep_host), sizeof(SweepRecord), cudaHostAllocMapped));
    std::memset(I.mail_host, 0, sizeof(Mailbox));
    std::memset(I.sweep_host, 0, sizeof(SweepRecord));
    desc_ = desc;
    material_ = material;
    const size_t N = m.nodes(), E = m.elements(), S = m.strands(), Vn = m.collider.size(), T = m.tri.size() / 3,
                 B = m.bvh.size(), L = m.bvh.leaves.size(), O = m.mapping.size();
    // Arena sizing.
    size_t bytes = 0;
    bytes += 13 * padded<double>(6 * N);     // q q_old v q_base grad dir precond dprime as_i_g as_j_g q_snap v_snap inertia
    bytes += 5 * padded<double>(36 * N);     // diag upper cprime as_i_h as_j_h
    bytes += 2 * padded<double>(9 * N) + padded<double>(9 * N);  // rot jl ref
    bytes += 4 * padded<double>(N);          // node_energy kinetic mass rmass
    bytes += 2 * padded<double>(3 * N);      // as_i_f as_j_f
    bytes += padded<uint8_t>(N) + 2 * padded<int32_t>(N);
    bytes += 4 * padded<double>(3 * N);      // root cur/pending x r
    bytes += 3 * padded<uint32_t>(N) + padded<double>(N);  // root bindings, node strand
    bytes += 3 * padded<uint32_t>(E) + padded<uint8_t>(E) + padded<double>(E) + 2 * padded<double>(3 * E);
    bytes += 3 * padded<double>(E) + 2 * padded<uint32_t>(E) + padded<uint8_t>(E);
    bytes += 4 * padded<uint32_t>(S);
    bytes += padded<uint32_t>(3 * T) + 5 * padded<double>(3 * Vn) + padded<float>(3 * Vn);
    bytes += 2 * padded<float>(3 * B) + padded<float4>(2 * B);
    const size_t pair_capacity = std::min<size_t>(std::max<size_t>(size_t(1) << 20, 8 * E), size_t(16) << 20);
    bytes += 2 * padded<double>(E) + padded<double>(3 * E) + 2 * padded<uint32_t>(pair_capacity);
    bytes += padded<uint32_t>(size_t(kCacheLeaves) * E) + padded<uint8_t>(E);
    const size_t leaf_pool = std::min<size_t>(std::max<size_t>(size_t(1) << 20, 4 * E), size_t(16) << 20);
    bytes += padded<uint32_t>(leaf_pool);
    bytes += padded<float>(3 * N) + padded<float>(6 * E);
    bytes += padded<uint32_t>(E);
    bytes += 2 * padded<float2>(36 * N) + padded<float2>(6 * N) + padded<float>(N);
    bytes += 2 * padded<float4>(3 * T) + 2 * padded<uint32_t>(size_t(kSurvivors) * E) + padded<uint8_t>(E) +
             padded<double>(5 * size_t(kSurvivors) * E);
    bytes += 2 * padded<double>(3 * B) + 4 * padded<uint32_t>(B) + padded<int32_t>(B) + 2 * padded<uint32_t>(B) +
             padded<uint32_t>(L) + padded<uint32_t>(T);
    bytes += padded<Partial>(kPartials) + padded<DirPartial>(kPartials) + padded<Scalars>(1);
    bytes += padded<uint32_t>(O) + padded<double>(3 * std::max(N, O));
    KHS_CUDA(cudaMalloc(reinterpret_cast<void **>(&I.arena.base), bytes));
    KHS_CUDA(cudaMemsetAsync(I.arena.base, 0, bytes, I.stream));
    I.arena.size = bytes;
    I.resident = bytes;
    Arena &a = I.arena;
    View &v = I.v;
    v.N = uint32_t(N); v.E = uint32_t(E); v.S = uint32_t(S); v.V = uint32_t(Vn); v.T = uint32_t(T); v.B = uint32_t(B);
    v.L = uint32_t(L);
    v.q = a.take<double>(6 * N); v.q_old = a.take<double>(6 * N); v.v = a.take<double>(6 * N);
    v.q_base = a.take<double>(6 * N); v.grad = a.take<double>(6 * N); v.dir = a.take<double>(6 * N);
    v.precond = a.take<double>(6 * N); v.dprime = a.take<double>(6 * N); v.inertia = a.take<double>(6 * N);
    v.q32 = a.take<float>(3 * N);
    v.as_i_g = a.take<double>(6 * N); v.as_j_g = a.take<double>(6 * N);
    I.q_snap = a.take<double>(6 * N); I.v_snap = a.take<double>(6 * N);
    v.diag = a.take<double>(36 * N); v.upper = a.take<double>(36 * N); v.cprime = a.take<double>(36 * N);
    v.as_i_h = a.take<double>(36 * N); v.as_j_h = a.take<double>(36 * N);
    v.rot = a.take<double>(9 * N); v.jl = a.take<double>(9 * N);
    double *ref = a.take<double>(9 * N);
    v.node_energy = a.take<double>(N); v.node_kinetic = a.take<double>(N);
    double *mass = a.take<double>(N), *rmass = a.take<double>(N);
    v.as_i_f = a.take<double>(3 * N); v.as_j_f = a.take<double>(3 * N);
    uint8_t *fixed = a.take<uint8_t>(N);
    int32_t *eleft = a.take<int32_t>(N), *eright = a.take<int32_t>(N);
    I.root_cur_x = a.take<double>(3 * N); I.root_cur_r = a.take<double>(3 * N);
    I.root_pend_x = a.take<double>(3 * N); I.root_pend_r = a.take<double>(3 * N);
    I.bind_l = a.take<uint32_t>(N); I.bind_r = a.take<uint32_t>(N); I.node_strand = a.take<uint32_t>(N);
    I.bind_t = a.take<double>(N);
    uint32_t *ei = a.take<uint32_t>(E), *ej = a.take<uint32_t>(E), *es = a.take<uint32_t>(E);
    uint8_t *ec = a.take<uint8_t>(E);
    double *L0 = a.take<double>(E), *g0 = a.take<double>(3 * E), *k0 = a.take<double>(3 * E);
    v.e_el = a.take<double>(E); v.e_co = a.take<double>(E); v.c_gap = a.take<double>(E);
    v.c_cand = a.take<uint32_t>(E); v.c_tri = a.take<uint32_t>(E); v.c_flags = a.take<uint8_t>(E);
    uint32_t *sf = a.take<uint32_t>(S), *sc = a.take<uint32_t>(S), *sx = a.take<uint32_t>(S), *so = a.take<uint32_t>(S);
    uint32_t *tri = a.take<uint32_t>(3 * T);
    v.col_cur = a.take<double>(3 * Vn); v.col_old = a.take<double>(3 * Vn);
    v.col32 = a.take<float>(3 * Vn);
    I.col_frame_start = a.take<double>(3 * Vn); I.col_pending = a.take<double>(3 * Vn); I.col_a_copy = a.take<double>(3 * Vn);
    v.blo = a.take<double>(3 * B); v.bhi = a.take<double>(3 * B);
    v.blo32 = a.take<float>(3 * B); v.bhi32 = a.take<float>(3 * B);
    v.bnode = B ? a.take<float4>(2 * B) : nullptr;
    v.c_t = a.take<double>(E); v.c_dist = a.take<double>(E); v.c_bary = a.take<double>(3 * E);
    v.pair_elem = a.take<uint32_t>(pair_capacity); v.pair_tri = a.take<uint32_t>(pair_capacity);
    v.pair_capacity = uint32_t(pair_capacity);
    v.cache_leaf = a.take<uint32_t>(size_t(kCacheLeaves) * E); v.cache_n = a.take<uint8_t>(E);
    v.leaf_pool = a.take<uint32_t>(leaf_pool); v.leaf_pool_capacity = uint32_t(leaf_pool);
    v.cache_x32 = a.take<float>(6 * E);
    v.tri32 = a.take<float4>(3 * T); v.tri32_old = a.take<float4>(3 * T);
    v.ff_inv = a.take<float2>(36 * N); v.ff_c = a.take<float2>(36 * N); v.ff_d = a.take<float2>(6 * N);
    v.ff_shift = a.take<float>(N);
    v.surv_tri = a.take<uint32_t>(size_t(kSurvivors) * E); v.surv_list = a.take<uint32_t>(size_t(kSurvivors) * E);
    v.surv_n = a.take<uint8_t>(E); v.surv_res = a.take<double>(5 * size_t(kSurvivors) * E);
    v.near_list = a.take<uint32_t>(E);
    if (E) KHS_CUDA(cudaMemsetAsync(v.cache_n, kCacheInvalid, E, I.stream));
    uint32_t *besc = a.take<uint32_t>(B), *bfirst = a.take<uint32_t>(B), *bcount = a.take<uint32_t>(B);
    v.brefit = a.take<uint32_t>(B);
    int32_t *bparent = a.take<int32_t>(B);
    uint32_t *bleft = a.take<uint32_t>(B), *bright = a.take<uint32_t>(B), *bleaves = a.take<uint32_t>(L);
    uint32_t *border = a.take<uint32_t>(T);
    v.partials = a.take<Partial>(kPartials);
    v.dpartials = a.take<DirPartial>(kPartials);
    v.sc = a.take<Scalars>(1);
    I.mapping_dev = a.take<uint32_t>(O);
    I.mapping_gather_out = a.take<double>(3 * std::max(N, O));
    if (a.used > a.size) throw std::runtime_error("device arena overflow");

    // Host staging.
    auto up = [&](void *dst, const void *src, size_t bytes2) {
        if (bytes2) KHS_CUDA(cudaMemcpyAsync(dst, src, bytes2, cudaMemcpyHostToDevice, I.stream));
    };
    std::vector<double> hq(6 * N, 0.0), href(9 * N);
    std::vector<int32_t> hl(N, -1), hr(N, -1);
    for (size_t n = 0; n < N; ++n) {
        hq[6 * n] = m.x[n].x; hq[6 * n + 1] = m.x[n].y; hq[6 * n + 2] = m.x[n].z;
        std::memcpy(&href[9 * n], m.frame[n].m, 9 * sizeof(double));
    }
    for (size_t e = 0; e < E; ++e) { hr[m.elem_i[e]] = int32_t(e); hl[m.elem_j[e]] = int32_t(e); }
    std::vector<double> hg0(3 * E), hk0(3 * E);
    for (size_t e = 0; e < E; ++e) {
        hg0[3 * e] = m.rest_shear[e].x; hg0[3 * e + 1] = m.rest_shear[e].y; hg0[3 * e + 2] = m.rest_shear[e].z;
        hk0[3 * e] = m.rest_curvature[e].x; hk0[3 * e + 1] = m.rest_curvature[e].y; hk0[3 * e + 2] = m.rest_curvature[e].z;
    }
    std::vector<uint32_t> order(S);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t l, uint32_t r) {
        return m.strand_count[l] - m.strand_fixed[l] > m.strand_count[r] - m.strand_fixed[r];
    });
    I.sorted_len.resize(S);
    for (size_t k = 0; k < S; ++k) I.sorted_len[k] = m.strand_count[order[k]] - m.strand_fixed[order[k]];
    std::vector<double> hcol(3 * Vn);
    for (size_t k = 0; k < Vn; ++k) { hcol[3 * k] = m.collider[k].x; hcol[3 * k + 1] = m.collider[k].y; hcol[3 * k + 2] = m.collider[k].z; }
    std::vector<double> hrx(3 * N), hrr(3 * N);
    for (size_t n = 0; n < N; ++n) {
        hrx[3 * n] = root_pos[n].x; hrx[3 * n + 1] = root_pos[n].y; hrx[3 * n + 2] = root_pos[n].z;
        hrr[3 * n] = root_rot[n].x; hrr[3 * n + 1] = root_rot[n].y; hrr[3 * n + 2] = root_rot[n].z;
    }
    up(v.q, hq.data(), 6 * N * 8); up(v.q_old, hq.data(), 6 * N * 8); up(I.q_snap, hq.data(), 6 * N * 8);
    up(v.q_base, hq.data(), 6 * N * 8);
    up(ref, href.data(), 9 * N * 8);
    up(mass, m.mass.data(), N * 8); up(rmass, m.rotational_mass.data(), N * 8);
    up(fixed, m.fixed.data(), N);
    up(eleft, hl.data(), N * 4); up(eright, hr.data(), N * 4);
    up(I.root_cur_x, hrx.data(), 3 * N * 8); up(I.root_cur_r, hrr.data(), 3 * N * 8);
    up(I.root_pend_x, hrx.data(), 3 * N * 8); up(I.root_pend_r, hrr.data(), 3 * N * 8);
    std::vector<uint32_t> hbl(N), hbr(N);
    std::vector<double> hbt(N);
    for (size_t n = 0; n < N; ++n) { hbl[n] = m.binding[n].left; hbr[n] = m.binding[n].right; hbt[n] = m.binding[n].t; }
    up(I.bind_l, hbl.data(), N * 4); up(I.bind_r, hbr.data(), N * 4); up(I.bind_t, hbt.data(), N * 8);
    up(I.node_strand, m.node_strand.data(), N * 4);
    I.root.N = uint32_t(N); I.root.S = uint32_t(S);
    I.root.bind_l = I.bind_l; I.root.bind_r = I.bind_r; I.root.bind_t = I.bind_t; I.root.node_strand = I.node_strand;
    I.root.sfirst = sf; I.root.scount = sc; I.root.sorder = so; I.root.ref = ref;
    up(ei, m.elem_i.data(), E * 4); up(ej, m.elem_j.data(), E * 4); up(es, m.elem_strand.data(), E * 4);
    up(ec, m.elem_contact.data(), E);
    up(L0, m.rest_length.data(), E * 8); up(g0, hg0.data(), 3 * E * 8); up(k0, hk0.data(), 3 * E * 8);
    up(sf, m.strand_first.data(), S * 4); up(sc, m.strand_count.data(), S * 4); up(sx, m.strand_fixed.data(), S * 4);
    up(so, order.data(), S * 4);
    up(tri, m.tri.data(), 3 * T * 4);
    up(v.col_cur, hcol.data(), 3 * Vn * 8); up(v.col_old, hcol.data(), 3 * Vn * 8);
    std::vector<float> hcol32(hcol.begin(), hcol.end());
    up(v.col32, hcol32.data(), 3 * Vn * 4);
    up(I.col_frame_start, hcol.data(), 3 * Vn * 8); up(I.col_pending, hcol.data(), 3 * Vn * 8);
    if (B) {
        up(v.blo, m.bvh.lower.data(), 3 * B * 8); up(v.bhi, m.bvh.upper.data(), 3 * B * 8);
        std::vector<float> lo32(3 * B), hi32(3 * B);
        for (size_t k = 0; k < 3 * B; ++k) {
            lo32[k] = std::nextafter(float(m.bvh.lower[k]), -std::numeric_limits<float>::infinity());
            hi32[k] = std::nextafter(float(m.bvh.upper[k]), std::numeric_limits<float>::infinity());
        }
        up(v.blo32, lo32.data(), 3 * B * 4); up(v.bhi32, hi32.data(), 3 * B * 4);
        std::vector<float4> packed(2 * B);
        for (size_t k = 0; k < B; ++k) {
            const uint32_t leaf = m.bvh.count[k] ? (m.bvh.first[k] << 4) | m.bvh.count[k] : 0u;
            uint32_t esc = m.bvh.escape[k];
            float e_f, l_f;
            std::memcpy(&e_f, &esc, 4);
            std::memcpy(&l_f, &leaf, 4);
            packed[2 * k] = make_float4(lo32[3 * k], lo32[3 * k + 1], lo32[3 * k + 2], e_f);
            packed[2 * k + 1] = make_float4(hi32[3 * k], hi32[3 * k + 1], hi32[3 * k + 2], l_f);
        }
        up(v.bnode, packed.data(), 2 * B * sizeof(float4));
        up(besc, m.bvh.escape.data(), B * 4); up(bfirst, m.bvh.first.data(), B * 4); up(bcount, m.bvh.count.data(), B * 4);
        up(bparent, m.bvh.parent.data(), B * 4); up(bleft, m.bvh.left_child.data(), B * 4);
        up(bright, m.bvh.right_child.data(), B * 4); up(bleaves, m.bvh.leaves.data(), L * 4);
        up(border, m.bvh.order.data(), T * 4);
    }
    up(I.mapping_dev, m.mapping.data(), O * 4);
    v.ref = ref; v.mass = mass; v.rmass = rmass; v.fixed = fixed; v.elem_left = eleft; v.elem_right = eright;
    v.ei = ei; v.ej = ej; v.estrand = es; v.econtact = ec; v.L0 = L0; v.gamma0 = g0; v.kappa0 = k0;
    v.sfirst = sf; v.scount = sc; v.sfixed = sx; v.sorder = so; v.tri = tri;
    v.besc = besc; v.bfirst = bfirst; v.bcount = bcount; v.border = border; v.bleaves = bleaves; v.bparent = bparent;
    v.bleft = bleft; v.bright = bright;
    KHS_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&v.mail), I.mail_host, 0));
    KHS_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&v.sweep), I.sweep_host, 0));
    v.has_collider = T > 0 ? 1 : 0;
    I.launch("k_init_scalars", k_init_scalars, 1, 1, v);
    if (T) I.launch("k_tri32", k_tri32, grid_for(T), kBlock, v);
    KHS_CUDA(cudaGetLastError());
    I.original_count = uint32_t(O);
    I.fixed_host = m.fixed;
    max_rest_length_ = 0.0;
    for (double L : m.rest_length) max_rest_length_ = std::fmax(max_rest_length_, L);
    update_runtime(desc, material, m.mass, m.rotational_mass);
    I.sync();
    clear_failure();
    step_stats_ = {};
    step_stats_.struct_size = sizeof(step_stats_);
    gpu_stats_ = {};
    gpu_stats_.struct_size = sizeof(gpu_stats_);
    gpu_stats_.resident_bytes = I.resident;
    initialized_ = true;
}

void Engine::update_runtime(const KhsSolverDesc &desc, const KhsHairMaterial &material, const std::vector<double> &mass,
                            const std::vector<double> &rotational_mass)
{
    Impl &I = *d_;
    desc_ = desc;
    material_ = material;
    View &v = I.v;
    if (initialized_ || !mass.empty()) {
        KHS_CUDA(cudaMemcpyAsync(const_cast<double *>(v.mass), mass.data(), mass.size() * 8, cudaMemcpyHostToDevice, I.stream));
        KHS_CUDA(cudaMemcpyAsync(const_cast<double *>(v.rmass), rotational_mass.data(), rotational_mass.size() * 8,
                                 cudaMemcpyHostToDevice, I.stream));
        I.sync();
    }
    v.radius = material.radius; v.offset = material.collider_offset; v.dhat = material.barrier_distance;
    v.kc = material.contact_stiffness; v.friction = material.friction; v.smoothing = material.friction_smoothing;
    v.damping = material.mass_damping; v.min_gap = desc.minimum_gap;
    v.gx = desc.gravity.x; v.gy = desc.gravity.y; v.gz = desc.gravity.z;
    v.young = material.young_modulus; v.poisson = material.poisson_ratio; v.shear_corr = material.shear_correction;
    v.w = dm::strain_weights(material.radius, material.young_modulus, material.poisson_ratio, material.shear_correction);
    trust_radius_ = std::fmax(0.25 * max_rest_length_, 8.0 * (material.radius + material.collider_offset + material.barrier_distance));
}

KhsResult Engine::run_root_pass(const KhsVec3 *points, uint32_t count)
{
    Impl &I = *d_;
    const size_t N = I.v.N;
    if (!points || count != I.original_count) return fail(KHS_ERROR_INVALID_ARGUMENT, "the root target point count does not match the source curves");
    if (!I.root_work) {
        const size_t bytes = padded<double>(3 * size_t(count)) + 3 * padded<double>(3 * N) + padded<double>(9 * N) +
                             padded<uint32_t>(1);
        char *base = nullptr;
        if (cudaMalloc(reinterpret_cast<void **>(&base), bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(KHS_ERROR_OUT_OF_MEMORY, "cannot allocate the device root-target arrays");
        }
        I.root_work = base;
        I.resident += bytes;
        gpu_stats_.resident_bytes = I.resident;
        size_t off = 0;
        auto take = [&](size_t doubles) { double *p = reinterpret_cast<double *>(base + off); off += padded<double>(doubles); return p; };
        I.root.points = take(3 * size_t(count));
        I.root.x = take(3 * N); I.root.tangent = take(3 * N); I.root.rot = take(3 * N); I.root.frame = take(9 * N);
        I.root.bad = reinterpret_cast<uint32_t *>(base + off);
    }
    KHS_CUDA(cudaMemcpyAsync(const_cast<double *>(I.root.points), points, size_t(count) * 24, cudaMemcpyHostToDevice, I.stream));
    KHS_CUDA(cudaMemsetAsync(I.root.bad, 0, sizeof(uint32_t), I.stream));
    I.launch("k_root_tangents", k_root_tangents, grid_for(N), kBlock, I.root);
    I.launch("k_root_transport", k_root_transport, grid_for(N), kBlock, I.root);
    I.launch("k_root_frames", k_root_frames, grid_for(I.v.S), kBlock, I.root);
    I.launch("k_root_rotations", k_root_rotations, grid_for(N), kBlock, I.root);
    I.check();
    uint32_t bad = 0;
    KHS_CUDA(cudaMemcpyAsync(&bad, I.root.bad, sizeof(bad), cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    if (bad) return fail(KHS_ERROR_INVALID_HAIR, "cannot compute root directions from the root targets");
    return KHS_OK;
}

KhsResult Engine::set_pending_root_points(const KhsVec3 *points, uint32_t count)
{
    Impl &I = *d_;
    const KhsResult r = run_root_pass(points, count);
    if (r != KHS_OK) return r;
    const size_t bytes = 3 * size_t(I.v.N) * 8;
    KHS_CUDA(cudaMemcpyAsync(I.root_pend_x, I.root.x, bytes, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.root_pend_r, I.root.rot, bytes, cudaMemcpyDeviceToDevice, I.stream));
    return KHS_OK;
}

KhsResult Engine::root_targets_to_host(const KhsVec3 *points, uint32_t count, KhsVec3 *positions, KhsVec3 *rotations)
{
    Impl &I = *d_;
    const KhsResult r = run_root_pass(points, count);
    if (r != KHS_OK) return r;
    const size_t bytes = 3 * size_t(I.v.N) * 8;
    KHS_CUDA(cudaMemcpyAsync(positions, I.root.x, bytes, cudaMemcpyDeviceToHost, I.stream));
    KHS_CUDA(cudaMemcpyAsync(rotations, I.root.rot, bytes, cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    return KHS_OK;
}

void Engine::set_pending_collider(const std::vector<Vec> &vertices)
{
    Impl &I = *d_;
    KHS_CUDA(cudaMemcpyAsync(I.col_pending, vertices.data(), vertices.size() * sizeof(Vec), cudaMemcpyHostToDevice, I.stream));
    I.sync();
}

KhsResult Engine::allocate_animation(uint32_t frames)
{
    Impl &I = *d_;
    if (!initialized_ || frames < 1) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid animation frame count");
    if (I.anim_root_x) { cudaFree(I.anim_root_x); I.anim_root_x = nullptr; I.resident -= I.anim_bytes; }
    const size_t N = I.v.N, Vn = I.v.V;
    const size_t root_bytes = size_t(frames) * 3 * N * 8, col_bytes = size_t(frames) * 3 * Vn * 8;
    const size_t total = 2 * padded<char>(root_bytes) + padded<char>(col_bytes);
    char *base = nullptr;
    if (cudaMalloc(reinterpret_cast<void **>(&base), total) != cudaSuccess) {
        cudaGetLastError();
        return fail(KHS_ERROR_OUT_OF_MEMORY, "cannot allocate device animation storage");
    }
    I.anim_root_x = reinterpret_cast<double *>(base);
    I.anim_root_r = reinterpret_cast<double *>(base + padded<char>(root_bytes));
    I.anim_col = reinterpret_cast<double *>(base + 2 * padded<char>(root_bytes));
    I.anim_bytes = total;
    I.resident += total;
    animation_frames_ = frames;
    animation_ready_ = false;
    root_frame_set_.assign(frames, false);
    collider_frame_set_.assign(frames, Vn == 0);
    gpu_stats_.animation_frame_count = frames;
    gpu_stats_.resident_bytes = I.resident;
    return KHS_OK;
}

KhsResult Engine::set_root_animation_frame(uint32_t frame, const KhsVec3 *points, uint32_t count)
{
    Impl &I = *d_;
    const size_t N = I.v.N;
    // Targets first, then the frame index, in the reference's order
    // (solver.cpp:802-824 computes before the backend checks the frame).
    const KhsResult r = run_root_pass(points, count);
    if (r != KHS_OK) return r;
    if (frame >= animation_frames_) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid root animation frame");
    KHS_CUDA(cudaMemcpyAsync(I.anim_root_x + size_t(frame) * 3 * N, I.root.x, 3 * N * 8, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.anim_root_r + size_t(frame) * 3 * N, I.root.rot, 3 * N * 8, cudaMemcpyDeviceToDevice, I.stream));
    root_frame_set_[frame] = true;
    return KHS_OK;
}

KhsResult Engine::set_collider_animation_frame(uint32_t frame, const KhsVec3 *vertices, uint32_t count)
{
    Impl &I = *d_;
    if (frame >= animation_frames_ || count != I.v.V) return fail(KHS_ERROR_INVALID_COLLIDER, "invalid collider animation frame");
    if (count) {
        KHS_CUDA(cudaMemcpyAsync(I.anim_col + size_t(frame) * 3 * I.v.V, vertices, size_t(count) * 24, cudaMemcpyHostToDevice, I.stream));
        I.sync();
    }
    collider_frame_set_[frame] = true;
    return KHS_OK;
}

KhsResult Engine::finalize_animation()
{
    if (animation_frames_ < 1 || std::find(root_frame_set_.begin(), root_frame_set_.end(), false) != root_frame_set_.end() ||
        std::find(collider_frame_set_.begin(), collider_frame_set_.end(), false) != collider_frame_set_.end())
        return fail(KHS_ERROR_INVALID_STATE, "animation has missing frames");
    animation_ready_ = true;
    current_frame_ = 0;
    return KHS_OK;
}

KhsResult Engine::fail(KhsResult r, const std::string &message)
{
    error_ = message;
    step_stats_.phase = KHS_PHASE_FAILED;
    progress_phase_.store(KHS_PHASE_FAILED);
    return r;
}

void Engine::clear_failure()
{
    failure_ = {};
    failure_.struct_size = sizeof(failure_);
    failure_.strand_index = kNone;
    failure_.element_index = kNone;
    failure_.collider_triangle_index = kNone;
}

void Engine::set_failure_context(uint32_t kind, uint32_t frame, uint32_t sub, uint32_t attempted, uint32_t maximum,
                                 uint32_t attempts)
{
    failure_.kind = kind; failure_.frame_index = frame; failure_.substep = sub;
    failure_.requested_substeps = desc_.substeps; failure_.attempted_substeps = attempted;
    failure_.maximum_substeps = maximum; failure_.adaptive_attempt_count = attempts;
}

KhsProgress Engine::progress() const
{
    KhsProgress p{};
    p.struct_size = sizeof(p);
    p.phase = progress_phase_.load(); p.frame_index = progress_frame_.load(); p.frame_count = progress_frame_count_.load();
    p.substep = progress_substep_.load(); p.substep_count = progress_substep_count_.load();
    p.nonlinear_iteration = progress_iteration_.load(); p.nonlinear_iteration_limit = desc_.newton_iterations;
    p.cancelled = cancel_.load() ? 1u : 0u;
    p.frame_elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - frame_clock_).count();
    return p;
}

EvalStats Engine::evaluate(bool gradient, double dt, double alpha, const double *alpha_dev)
{
    Impl &I = *d_;
    const View &v = I.v;
    const bool trial = alpha >= 0.0 || alpha_dev;
    const double a = alpha >= 0.0 ? alpha : 0.0;
    if (mode_ && v.has_collider) {
        // The mixed form's contact passes read only q and its FP32 copy: once
        // k_positions has written them, the passes run on a second stream
        // beside the node kernel (on one stream while kernels are timed one by
        // one).  The same kernels see the same inputs either way.
        I.launch("k_positions", k_positions, grid_for(v.N), kBlock, v, trial ? 1 : 0, a, alpha_dev);
        const bool side = !I.profiling;
        const cudaStream_t cs = side ? I.side : I.stream;
        if (side) {
            KHS_CUDA(cudaEventRecord(I.fork, I.stream));
            KHS_CUDA(cudaStreamWaitEvent(I.side, I.fork, 0));
        }
        const double *q = v.q;
        if (rebuild_cache_) KHS_CUDA(cudaMemsetAsync(&v.sc->pool_used, 0, sizeof(uint32_t), cs));
        I.launch_on(cs, rebuild_cache_ ? "k_contact_filter_rebuild" : trial ? "k_contact_filter_trial" : "k_contact_filter",
                    k_contact_filter, grid_for(v.E), kBlock, v, q, rebuild_cache_ ? 1 : 0);
        I.launch_on(cs, "k_contact_near", k_contact_near, 152 * 8, kBlock, v);
        I.launch_on(cs, "k_contact_exact", k_contact_exact, 152 * 4, kBlock, v, q);
        I.launch_on(cs, "k_contact_select", k_contact_select, grid_for(v.E), kBlock, v, q);
        if (side) KHS_CUDA(cudaEventRecord(I.join, I.side));
        I.launch(gradient ? "k_node_eval_grad" : "k_node_eval_energy", k_node_eval, grid_for(v.N), kBlock, v,
                 gradient ? 1 : 0, trial ? 1 : 0, a, dt, alpha_dev, 1);
        if (side) KHS_CUDA(cudaStreamWaitEvent(I.stream, I.join, 0));
    } else {
        I.launch(gradient ? "k_node_eval_grad" : "k_node_eval_energy", k_node_eval, grid_for(v.N), kBlock, v,
                 gradient ? 1 : 0, trial ? 1 : 0, a, dt, alpha_dev, 0);
    }
    rebuild_cache_ = false;
    I.launch(gradient ? "k_elem_eval_grad" : "k_elem_eval_energy", mode_ ? k_elem_eval<true> : k_elem_eval<false>, grid_for(v.E),
             kBlock, v, gradient ? 1 : 0);
    if (gradient) I.launch("k_node_sum", k_node_sum, grid_for(42 * size_t(v.N)), kBlock, v);
    I.launch("k_reduce_eval", k_reduce_eval, kPartials, kBlock, v, gradient ? 1 : 0);
    I.check();
    I.sync();
    const Mailbox &mb = *I.mail_host;
    EvalStats s;
    s.objective = mb.objective; s.elastic = mb.elastic; s.contact = mb.contact; s.kinetic = mb.kinetic;
    s.minimum_gap = mb.minimum_gap; s.grad_norm2 = mb.grad_norm2; s.candidates = mb.candidates; s.active = mb.active;
    s.feasible = mb.feasible;
    return s;
}

bool Engine::limit_direction(double max_translation)
{
    Impl &I = *d_;
    if (max_translation > trust_radius_) {
        I.launch("k_scale", k_scale, grid_for(6 * size_t(I.v.N)), kBlock, I.v, trust_radius_ / max_translation);
        return true;
    }
    return false;
}

bool Engine::make_steepest()
{
    Impl &I = *d_;
    I.launch("k_steepest", k_steepest, grid_for(6 * size_t(I.v.N)), kBlock, I.v);
    I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, I.v);
    I.launch("k_final_dir", k_final_dir, 1, kBlock, I.v, 0);
    I.check();
    I.sync();
    return limit_direction(I.mail_host->max_translation);
}

// Launch shape of the persistent FP64 block solve: the layout (H = 1: five
// strands of 6 lanes per warp; H = 2: two strands of 12 lanes; H = 3: one
// strand of 18 lanes) and 1-4
// blocks of four warps per SM, chosen once by timing each on the first
// system.  The choice does not change the result: both layouts compute every
// entry with the same operations, and each strand is solved by one group.
KhsResult Engine::set_block_solve_schedule(uint32_t strands_per_warp, uint32_t blocks_per_sm, uint32_t long_strands)
{
    Impl &I = *d_;
    if (strands_per_warp == 0) {
        I.solve_blocks = 0; I.solve_kernel = nullptr; I.solve_long = 0; I.solve_pairs = false; I.solve_tiers = false;
        return KHS_OK;
    }
    if ((strands_per_warp != 5 && strands_per_warp != 2 && strands_per_warp != 1) || blocks_per_sm < 1 || blocks_per_sm > 8 ||
        (long_strands && ((strands_per_warp != 5 && strands_per_warp != 1) || long_strands >= I.v.S)))
        return KHS_ERROR_INVALID_ARGUMENT;
    int sms = 0;
    KHS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, kDevice));
    const unsigned groups = long_strands ? long_strands + unsigned((I.v.S - long_strands + 4) / 5)
                                         : unsigned((I.v.S + strands_per_warp - 1) / strands_per_warp);
    I.solve_kernel = long_strands ? nullptr
                     : strands_per_warp == 5 ? k_block_solve_aug<1>
                     : strands_per_warp == 2 ? k_block_solve_aug<2>
                                             : k_block_solve_aug<3>;
    I.solve_long = long_strands;
    I.solve_pairs = long_strands && strands_per_warp == 1;
    I.solve_tiers = false;
    I.solve_blocks = std::min(std::max(1u, (groups + 3) / 4), blocks_per_sm * unsigned(sms));
    const unsigned ff_groups = unsigned((I.v.S + kSolveGroupsPerWarp - 1) / kSolveGroupsPerWarp);
    I.ff_blocks = std::min(std::max(1u, (ff_groups + 3) / 4), 2u * unsigned(sms));
    return KHS_OK;
}

// Queue items of the tiered schedule: one per quad strand and per single,
// one per two doubles, one per five of the rest.
static unsigned tier_items(uint32_t S, uint32_t quads, uint32_t singles, uint32_t doubles)
{
    const uint32_t head = quads + singles + doubles;
    return quads + singles + (doubles + 1) / 2 + (S > head ? (S - head + 4) / 5 : 0);
}

// Tiered launch shape (k_block_solve_tiers): the `quads` longest strands on
// four warps each, the next `singles` on one warp of 18 lanes, the next
// `doubles` two per warp, the rest five per warp; blocks_per_sm 1-8.  The
// shape does not change the result.
KhsResult Engine::set_block_solve_tiers(uint32_t quads, uint32_t singles, uint32_t doubles, uint32_t blocks_per_sm)
{
    Impl &I = *d_;
    if (blocks_per_sm < 1 || blocks_per_sm > 8 || uint64_t(quads) + singles + doubles > I.v.S)
        return KHS_ERROR_INVALID_ARGUMENT;
    int sms = 0;
    KHS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, kDevice));
    I.solve_kernel = nullptr;
    I.solve_long = 0;
    I.solve_pairs = false;
    I.solve_tiers = true;
    I.tier_quads = quads; I.tier_singles = singles; I.tier_doubles = doubles;
    const unsigned items = tier_items(I.v.S, quads, singles, doubles);
    I.solve_blocks = std::min(std::max(1u, (items + 3) / 4), blocks_per_sm * unsigned(sms));
    const unsigned ff_groups = unsigned((I.v.S + kSolveGroupsPerWarp - 1) / kSolveGroupsPerWarp);
    I.ff_blocks = std::min(std::max(1u, (ff_groups + 3) / 4), 2u * unsigned(sms));
    return KHS_OK;
}

void Engine::tune_block_solve()
{
    Impl &I = *d_;
    int sms = 0;
    KHS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, kDevice));
    cudaEvent_t ev[2];
    KHS_CUDA(cudaEventCreate(&ev[0]));
    KHS_CUDA(cudaEventCreate(&ev[1]));
    auto time_it = [&](void (*kernel)(View), unsigned blocks, uint32_t nlong, bool pairs = false,
                       const uint32_t *tiers = nullptr) {
        float best = 3.0e38f;
        for (int rep = 0; rep < 2; ++rep) {
            KHS_CUDA(cudaMemsetAsync(&I.v.sc->solve_next, 0, sizeof(uint32_t), I.stream));
            KHS_CUDA(cudaEventRecord(ev[0], I.stream));
            if (tiers) k_block_solve_tiers<<<blocks, 128, 0, I.stream>>>(I.v, tiers[0], tiers[1], tiers[2]);
            else if (kernel) kernel<<<blocks, 128, 0, I.stream>>>(I.v);
            else if (pairs) k_block_solve_pairs<<<blocks, 128, 0, I.stream>>>(I.v, nlong);
            else k_block_solve_hybrid<<<blocks, 128, 0, I.stream>>>(I.v, nlong);
            ++I.launches;
            KHS_CUDA(cudaEventRecord(ev[1], I.stream));
            KHS_CUDA(cudaEventSynchronize(ev[1]));
            float ms = 0.0f;
            KHS_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
            best = std::min(best, ms);
        }
        return best;
    };
    struct Candidate { void (*kernel)(View); unsigned strands_per_warp; };
    const Candidate layouts[3] = {{k_block_solve_aug<1>, 5u}, {k_block_solve_aug<2>, 2u}, {k_block_solve_aug<3>, 1u}};
    float best_ms = 3.0e38f;
    for (const Candidate &c : layouts) {
        const unsigned groups = unsigned((I.v.S + c.strands_per_warp - 1) / c.strands_per_warp);
        const unsigned most = std::max(1u, (groups + 3) / 4);
        for (unsigned per_sm = 1; per_sm <= 4; ++per_sm) {
            const unsigned blocks = std::min(most, per_sm * unsigned(sms));
            const float ms = time_it(c.kernel, blocks, 0);
            if (ms < best_ms) {
                best_ms = ms; I.solve_kernel = c.kernel; I.solve_blocks = blocks; I.solve_long = 0; I.solve_pairs = false;
                I.solve_tiers = false;
            }
            if (blocks == most) break;
        }
    }
    // Hybrid: the strands of at least `cut` free nodes one per warp (18
    // lanes) or on a pair of warps, the rest five per warp.
    uint32_t last_long = 0;
    for (uint32_t cut : {160u, 128u, 96u, 64u, 48u}) {
        const uint32_t nlong = uint32_t(std::count_if(I.sorted_len.begin(), I.sorted_len.end(),
                                                       [&](uint32_t len) { return len >= cut; }));
        if (nlong == 0 || nlong == last_long || nlong >= I.v.S) continue;
        last_long = nlong;
        const unsigned groups = nlong + unsigned((I.v.S - nlong + 4) / 5);
        const unsigned most = std::max(1u, (groups + 3) / 4);
        for (unsigned per_sm = 1; per_sm <= 3; ++per_sm) {
            const unsigned blocks = std::min(most, per_sm * unsigned(sms));
            for (bool pairs : {false, true}) {
                const float ms = time_it(nullptr, blocks, nlong, pairs);
                if (ms < best_ms) {
                    best_ms = ms; I.solve_kernel = nullptr; I.solve_blocks = blocks; I.solve_long = nlong; I.solve_pairs = pairs;
                    I.solve_tiers = false;
                }
            }
            if (blocks == most) break;
        }
    }
    // Tiered: quads for the longest ~0.5-2% of the strands, then singles,
    // doubles and five per warp, two blocks per SM (its 255 registers per
    // thread leave no room for a third).
    for (uint32_t qd : {110u, 75u, 55u})
        for (uint32_t sd : {70u, 35u, 25u})
            for (uint32_t dd : {34u, 17u}) {
                const uint32_t tiers[3] = {I.v.S / qd, I.v.S / sd, (I.v.S / dd) & ~1u};
                if (tiers[0] == 0 || uint64_t(tiers[0]) + tiers[1] + tiers[2] >= I.v.S) continue;
                const unsigned items = tier_items(I.v.S, tiers[0], tiers[1], tiers[2]);
                const unsigned most = std::max(1u, (items + 3) / 4);
                const unsigned blocks = std::min(most, 2u * unsigned(sms));
                const float ms = time_it(nullptr, blocks, 0, false, tiers);
                if (ms < best_ms) {
                    best_ms = ms; I.solve_kernel = nullptr; I.solve_blocks = blocks; I.solve_long = 0;
                    I.solve_pairs = false; I.solve_tiers = true;
                    I.tier_quads = tiers[0]; I.tier_singles = tiers[1]; I.tier_doubles = tiers[2];
                }
            }
    // Float-float kernels (5 strands of 6 lanes per warp).
    {
        const unsigned groups = unsigned((I.v.S + kSolveGroupsPerWarp - 1) / kSolveGroupsPerWarp);
        I.ff_blocks = std::min(std::max(1u, (groups + 3) / 4), 2u * unsigned(sms));
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    KHS_CUDA(cudaMemsetAsync(&I.v.sc->solve_next, 0, sizeof(uint32_t), I.stream));
    KHS_CUDA(cudaMemsetAsync(&I.v.sc->solve_failed, 0, sizeof(int), I.stream));
}

void Engine::launch_block_solve()
{
    Impl &I = *d_;
    if (I.solve_kernel) I.launch("k_block_solve", I.solve_kernel, I.solve_blocks, 128, I.v);
    else if (I.solve_tiers)
        I.launch("k_block_solve", k_block_solve_tiers, I.solve_blocks, 128, I.v, I.tier_quads, I.tier_singles,
                 I.tier_doubles);
    else if (I.solve_pairs) I.launch("k_block_solve", k_block_solve_pairs, I.solve_blocks, 128, I.v, I.solve_long);
    else I.launch("k_block_solve", k_block_solve_hybrid, I.solve_blocks, 128, I.v, I.solve_long);
}

bool Engine::make_direction(KhsxSubstepRecord &rec, double grad_norm2)
{
    Impl &I = *d_;
    (void)grad_norm2;
    if (!I.solve_blocks) tune_block_solve();
    const Mailbox &mb = *I.mail_host;
    bool fp64 = mode_ != KHSX_MODE_MIXED_FF;
    if (!fp64) {
        I.launch("k_ff_factor", k_ff_factor, I.ff_blocks, 128, I.v);
        uint32_t sweeps = 0;
        for (;;) {
            I.launch("k_ff_residual", k_ff_residual, grid_for(6 * size_t(I.v.N)), kBlock, I.v);
            I.launch("k_ff_correct", k_ff_correct, I.ff_blocks, 128, I.v);
            ++sweeps;
            I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, I.v);
            I.launch("k_final_dir", k_final_dir, 1, kBlock, I.v, 0);
            I.check();
            I.sync();
            if (mb.solve_failed) break;
            float ratio;
            std::memcpy(&ratio, &mb.refine_bits, sizeof(ratio));
            if (!(ratio > kRefineRatio) || sweeps >= uint32_t(kRefineSweepsMax)) break;
        }
        rec.refinement_sweeps += sweeps;
        if (mb.solve_failed) {
            ++rec.fp64_fallbacks;
            fp64 = true;
        }
    }
    if (fp64) {
        launch_block_solve();
        I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, I.v);
        I.launch("k_final_dir", k_final_dir, 1, kBlock, I.v, 0);
        I.check();
        I.sync();
    }
    const bool used = !mb.solve_failed && mb.slope < 0 && std::isfinite(mb.slope);
    if (!used) {
        ++rec.steepest_fallbacks;
        if (make_steepest()) ++rec.trust_scalings;
        return false;
    }
    if (limit_direction(mb.max_translation)) ++rec.trust_scalings;
    return true;
}

// The line-search CCD bound of the current direction (the mixed form's
// FP32-filtered pair list, or the per-element FP64 kernel).
void Engine::launch_ccd_bound()
{
    Impl &I = *d_;
    const View &v = I.v;
    if (mode_) {
        I.launch("k_ccd_collect", k_ccd_collect, grid_for(v.E), kBlock, v);
        I.launch("k_ccd_near", k_ccd_near, 152u * 8u, kBlock, v);
        I.launch("k_ccd_pairs", k_ccd_pairs, 152u * 8u, kBlock, v);
    } else {
        I.launch("k_ccd", k_ccd<false>, grid_for(v.E), kBlock, v);
    }
}

KhsResult Engine::optimize_substep(double dt, KhsxSubstepRecord &rec)
{
    Impl &I = *d_;
    last_dt_ = dt;
    const View &v = I.v;
    I.launch("k_precond", k_precond, grid_for(v.N), kBlock, v, dt);
    EvalStats current = evaluate(true, dt, -1.0);
    if (!current.feasible) return fail(KHS_ERROR_NOT_CONVERGED, "state is outside the barrier feasible region");
    const double initial = std::sqrt(current.grad_norm2);
    step_stats_.initial_residual_norm = std::fmax(step_stats_.initial_residual_norm, initial);
    const double dof = 6.0 * double(v.N);
    for (uint32_t it = 0; it <= desc_.newton_iterations; ++it) {
        progress_iteration_.store(it);
        if (cancel_.load()) return fail(KHS_ERROR_INVALID_STATE, "solve cancelled");
        const double residual = std::sqrt(current.grad_norm2);
        const double relative = residual / std::fmax(initial, 1e-30);
        step_stats_.final_residual_norm = residual;
        step_stats_.relative_residual_norm = relative;
        step_stats_.minimum_gap = std::fmin(step_stats_.minimum_gap, current.minimum_gap);
        step_stats_.contact_candidate_count += current.candidates;
        step_stats_.active_contact_count += current.active;
        step_stats_.kinetic_energy = current.kinetic;
        step_stats_.elastic_energy = current.elastic;
        step_stats_.contact_energy = current.contact;
        step_stats_.friction_energy = 0.0;
        rec.final_residual_norm = residual;
        rec.minimum_gap = std::fmin(rec.minimum_gap, current.minimum_gap);
        rec.contact_candidates += current.candidates;
        rec.active_contacts += current.active;
        if (residual <= std::fmax(desc_.absolute_tolerance, 1.0e-5 * std::sqrt(dof)) ||
            relative <= std::fmax(desc_.relative_tolerance, 1.0e-4)) {
            I.launch("k_update_velocity", k_update_velocity, grid_for(v.N), kBlock, v, 1.0 / dt);
            return KHS_OK;
        }
        if (it == desc_.newton_iterations) break;
        progress_phase_.store(KHS_PHASE_LINEAR_SOLVE);
        // FP64 solve: the direction, its CCD bound and the first line-search
        // trial (at the step k_final_dir leaves in device memory) are enqueued
        // together, with one host synchronisation instead of three.  The
        // device runs the same kernels in the same order as step by step.
        // The trust-radius limit is applied on the device (k_scale_trust, the
        // host's scale when it applies, else nothing).  When the direction is
        // not used as is (steepest fallback, CCD work-list overflow, step
        // below the minimum) the trial is discarded: the iterate is restored
        // and evaluated again, and the iteration goes on step by step.
        bool block_direction;
        bool pipelined = false;
        EvalStats first{};
        double first_alpha = 1.0, first_slope = 0.0;
        if (mode_ != KHSX_MODE_MIXED_FF) {
            if (!I.solve_blocks) tune_block_solve();
            launch_block_solve();
            I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, v);
            I.launch("k_final_dir", k_final_dir, 1, kBlock, v, 0);
            I.launch("k_scale", k_scale_trust, grid_for(6 * size_t(v.N)), kBlock, v, trust_radius_);
            KHS_CUDA(cudaMemcpyAsync(v.q_base, v.q, 6 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
            I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, v);
            if (v.has_collider) launch_ccd_bound();
            I.launch("k_final_dir", k_final_dir, 1, kBlock, v, 1);
            first = evaluate(true, dt, -1.0, &v.sc->trial_alpha);
            const Mailbox &mb = *I.mail_host;
            const bool used = !mb.dir_solve_failed && mb.dir_slope < 0 && std::isfinite(mb.dir_slope);
            const double max_translation = mb.dir_max_translation;
            first_slope = mb.slope;  // of the (possibly limited) direction, from the CCD pass
            if (v.has_collider) {
                unsigned long long bits = mb.ccd_bits;
                double lim;
                std::memcpy(&lim, &bits, sizeof(lim));
                first_alpha = lim;
                if (first_alpha < 1.0) first_alpha *= 0.9;
            }
            const bool overflow = mode_ && v.has_collider && mb.pair_count > v.pair_capacity;
            // The direction was limited to the trust radius on the device.
            const bool scaled = max_translation > trust_radius_;
            pipelined = used && !overflow && first_alpha >= desc_.minimum_line_search_step;
            block_direction = used;
            if (used && scaled) ++rec.trust_scalings;
            if (!pipelined) {
                KHS_CUDA(cudaMemcpyAsync(v.q, v.q_base, 6 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
                evaluate(true, dt, -1.0);
                if (!used) {
                    ++rec.steepest_fallbacks;
                    if (make_steepest()) ++rec.trust_scalings;
                }
            }
        } else {
            block_direction = make_direction(rec, current.grad_norm2);
            KHS_CUDA(cudaMemcpyAsync(v.q_base, v.q, 6 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
        }
        ++step_stats_.linear_solves;
        bool accepted = false;
        // The first trial of the Gauss-Newton direction also evaluates the
        // gradient, the Hessian blocks and the rotation Jacobians (its
        // energy is computed by the same operations as an energy-only
        // evaluation).  When it is accepted -- most iterations -- that
        // evaluation is the next iterate's, and the separate evaluation at
        // the accepted state is skipped: same values, one evaluation fewer.
        bool graded_trial = false;     // a trial evaluated the gradient at its own state
        bool accepted_graded = false;  // ... and it was the accepted one
        EvalStats graded{};
        double alpha = 1.0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            const bool reuse = pipelined && attempt == 0;  // bound and first trial already evaluated
            double slope;
            if (reuse) {
                slope = first_slope;
                alpha = first_alpha;
            } else {
                // Slope of the (possibly scaled) direction, and the CCD bound.
                I.launch("k_reduce_dir", k_reduce_dir, kPartials, kBlock, v);
                if (v.has_collider) {
                    progress_phase_.store(KHS_PHASE_CCD);
                    launch_ccd_bound();
                }
                I.launch("k_final_dir", k_final_dir, 1, kBlock, v, 0);
                I.check();
                I.sync();
                if (mode_ && v.has_collider && I.mail_host->pair_count > v.pair_capacity) {
                    // Work list overflow: redo the bound with the per-element kernel.
                    I.launch("k_ccd", k_ccd<true>, grid_for(v.E), kBlock, v);
                    I.launch("k_final_dir", k_final_dir, 1, kBlock, v, 0);
                    I.check();
                    I.sync();
                }
                slope = I.mail_host->slope;
                alpha = 1.0;
                if (v.has_collider) {
                    unsigned long long bits = I.mail_host->ccd_bits;
                    double lim;
                    std::memcpy(&lim, &bits, sizeof(lim));
                    alpha = lim;
                    if (alpha < 1.0) alpha *= 0.9;
                }
            }
            if (v.has_collider) step_stats_.ccd_step_limit = std::fmin(step_stats_.ccd_step_limit, alpha);
            accepted = false;
            progress_phase_.store(KHS_PHASE_LINE_SEARCH);
            if (alpha >= desc_.minimum_line_search_step)
                for (uint32_t s = 0; s < desc_.line_search_iterations; ++s) {
                    const bool with_gradient = attempt == 0 && s == 0;
                    const EvalStats trial = reuse && s == 0 ? first : evaluate(with_gradient, dt, alpha);
                    graded_trial = graded_trial || with_gradient;
                    ++step_stats_.line_search_evaluations;
                    ++rec.line_search_evaluations;
                    if (trial.feasible && std::isfinite(trial.objective) &&
                        trial.objective <= current.objective + 1e-4 * alpha * slope) {
                        accepted = true;
                        accepted_graded = with_gradient;
                        if (with_gradient) graded = trial;
                        break;
                    }
                    alpha *= 0.5;
                    if (alpha < desc_.minimum_line_search_step) break;
                }
            if (accepted) break;
            if (!block_direction) break;
            KHS_CUDA(cudaMemcpyAsync(v.q, v.q_base, 6 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
            // The trials left their own gradient, blocks, rotations and FP32
            // positions behind; the steepest direction (gradient) and the
            // mixed form's CCD filter (FP32 positions) need the iterate's.
            if (graded_trial) evaluate(true, dt, -1.0);
            ++rec.steepest_fallbacks;
            if (make_steepest()) ++rec.trust_scalings;
            block_direction = false;
        }
        if (!accepted) {
            KHS_CUDA(cudaMemcpyAsync(v.q, v.q_base, 6 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
            I.sync();
            return fail(KHS_ERROR_NOT_CONVERGED, "Gauss-Newton line search failed");
        }
        current = accepted_graded ? graded : evaluate(true, dt, -1.0);
        const double dnorm = std::sqrt(I.mail_host->dir_norm2);
        step_stats_.increment_norm = alpha * dnorm;
        step_stats_.accepted_step_length = alpha;
        ++step_stats_.newton_iterations;
        ++rec.newton_iterations;
        progress_phase_.store(KHS_PHASE_ASSEMBLING);
        if (step_stats_.increment_norm / std::sqrt(dof) <= 2.0 * desc_.increment_tolerance) {
            I.launch("k_update_velocity", k_update_velocity, grid_for(v.N), kBlock, v, 1.0 / dt);
            return KHS_OK;
        }
    }
    I.launch("k_update_velocity", k_update_velocity, grid_for(v.N), kBlock, v, 1.0 / dt);
    return KHS_OK;
}

KhsResult Engine::run_frame(double frame_dt, const double *root_a, const double *rot_a, const double *root_b,
                            const double *rot_b, const double *col_a, const double *col_b, uint32_t frame,
                            uint32_t frame_count)
{
    Impl &I = *d_;
    View &v = I.v;
    if (!(frame_dt > 0 && std::isfinite(frame_dt))) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid time step");
    cancel_.store(false);
    clear_failure();
    frame_clock_ = std::chrono::steady_clock::now();
    progress_frame_.store(frame); progress_frame_count_.store(frame_count); progress_iteration_.store(0);
    const size_t q_bytes = 6 * size_t(v.N) * 8, c_bytes = 3 * size_t(v.V) * 8;
    KHS_CUDA(cudaEventRecord(I.ev_begin, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.q_snap, v.q, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v_snap, v.v, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
    // Keep the frame's start collider: for khsStep it aliases the
    // frame-start buffer that is rewritten on success.
    if (v.V) {
        KHS_CUDA(cudaMemcpyAsync(I.col_a_copy, col_a, c_bytes, cudaMemcpyDeviceToDevice, I.stream));
        if (col_a != I.col_frame_start)
            KHS_CUDA(cudaMemcpyAsync(I.col_frame_start, col_a, c_bytes, cudaMemcpyDeviceToDevice, I.stream));
    }
    uint32_t substeps = desc_.substeps;
    const uint32_t maximum = v.has_collider ? desc_.maximum_substeps : desc_.substeps;
    uint32_t attempts = 0;
    for (;;) {
        ++attempts;
        KHS_CUDA(cudaMemcpyAsync(v.q, I.q_snap, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
        KHS_CUDA(cudaMemcpyAsync(v.v, I.v_snap, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
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
        if (v.V) KHS_CUDA(cudaMemcpyAsync(v.col_cur, I.col_a_copy, c_bytes, cudaMemcpyDeviceToDevice, I.stream));
        const double dt = frame_dt / substeps;
        bool crossed = false;
        KhsResult result = KHS_OK;
        for (uint32_t sub = 1; sub <= substeps; ++sub) {
            if (substep_limit_ && sub > substep_limit_) break;
            progress_substep_.store(sub);
            progress_iteration_.store(0);
            KhsxSubstepRecord rec{};
            rec.struct_size = sizeof(rec);
            rec.substep = sub;
            rec.minimum_gap = std::numeric_limits<double>::infinity();
            const double f = double(sub) / substeps;
            I.launch("k_begin_substep", k_begin_substep, grid_for(v.N), kBlock, v, root_a, rot_a, root_b, rot_b, f, dt);
            if (v.has_collider) {
                I.launch("k_collider_interp", k_collider_interp, grid_for(v.V), kBlock, v, I.col_a_copy, col_b, f);
                I.launch("k_tri32", k_tri32, grid_for(v.T), kBlock, v);
                I.launch("k_refit", k_refit, grid_for(v.L), kBlock, v, 1);
                progress_phase_.store(KHS_PHASE_CCD);
                I.launch("k_sweep", mode_ ? k_sweep<true> : k_sweep<false>, grid_for(v.E), kBlock, v);
                I.launch("k_sweep_record", k_sweep_record, 1, 1, v);
                I.check();
                I.sync();
                if (I.mail_host->sweep_fail != kNone) {
                    const SweepRecord &sr = *I.sweep_host;
                    set_failure_context(KHS_FAILURE_MOVING_COLLIDER_SWEEP, frame, sub, substeps, maximum, attempts);
                    if (sr.claimed) {
                        failure_.strand_index = sr.strand; failure_.element_index = sr.element;
                        failure_.collider_triangle_index = sr.triangle;
                        failure_.distance = sr.distance; failure_.required_distance = sr.required;
                        failure_.clearance = sr.clearance; failure_.collider_substep_displacement = sr.displacement;
                        failure_.collider_frame_displacement = sr.displacement * substeps;
                        failure_.hair_start = {sr.hair_start[0], sr.hair_start[1], sr.hair_start[2]};
                        failure_.hair_end = {sr.hair_end[0], sr.hair_end[1], sr.hair_end[2]};
                        failure_.collider_point = {sr.collider_point[0], sr.collider_point[1], sr.collider_point[2]};
                    }
                    crossed = true;
                    break;
                }
                I.launch("k_refit", k_refit, grid_for(v.L), kBlock, v, 0);
                rebuild_cache_ = true;
            }
            progress_phase_.store(KHS_PHASE_ASSEMBLING);
            result = optimize_substep(dt, rec);
            records_.push_back(rec);
            if (result != KHS_OK) {
                if (!cancel_.load()) {
                    const uint32_t kind = error_.find("outside the barrier") != std::string::npos ? KHS_FAILURE_BARRIER_INFEASIBLE
                                                                                                   : KHS_FAILURE_NONLINEAR_SOLVE;
                    set_failure_context(kind, frame, sub, substeps, maximum, attempts);
                }
                break;
            }
            if (v.has_collider && material_.friction > 0.0) {
                I.launch("k_friction", mode_ ? k_friction<true> : k_friction<false>, grid_for(v.E), kBlock, v, dt);
                I.launch("k_friction_apply", k_friction_apply, grid_for(v.N), kBlock, v);
            }
            ++step_stats_.converged_substeps;
        }
        if (!crossed && result == KHS_OK) break;
        KHS_CUDA(cudaMemcpyAsync(v.q, I.q_snap, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
        KHS_CUDA(cudaMemcpyAsync(v.v, I.v_snap, q_bytes, cudaMemcpyDeviceToDevice, I.stream));
        I.sync();
        if (cancel_.load()) return result;
        if (substeps >= maximum) {
            if (crossed) return fail(KHS_ERROR_NOT_CONVERGED, "animated collider crossed hair after adaptive substepping");
            return result;
        }
        substeps = std::min(maximum, substeps * 2);
    }
    if (!animation_ready_) {
        KHS_CUDA(cudaMemcpyAsync(I.root_cur_x, I.root_pend_x, 3 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
        KHS_CUDA(cudaMemcpyAsync(I.root_cur_r, I.root_pend_r, 3 * size_t(v.N) * 8, cudaMemcpyDeviceToDevice, I.stream));
        if (v.V) KHS_CUDA(cudaMemcpyAsync(I.col_frame_start, I.col_pending, c_bytes, cudaMemcpyDeviceToDevice, I.stream));
    }
    clear_failure();
    step_stats_.phase = KHS_PHASE_FINISHED;
    progress_phase_.store(KHS_PHASE_FINISHED);
    KHS_CUDA(cudaEventRecord(I.ev_end, I.stream));
    KHS_CUDA(cudaEventSynchronize(I.ev_end));
    float ms = 0;
    KHS_CUDA(cudaEventElapsedTime(&ms, I.ev_begin, I.ev_end));
    gpu_stats_.last_frame_milliseconds = ms;
    error_.clear();
    return KHS_OK;
}

KhsResult Engine::step(double frame_dt)
{
    Impl &I = *d_;
    return run_frame(frame_dt, I.root_cur_x, I.root_cur_r, I.root_pend_x, I.root_pend_r, I.col_frame_start, I.col_pending, 0, 0);
}

KhsResult Engine::step_animation_frame(uint32_t frame, double frame_dt)
{
    Impl &I = *d_;
    if (!animation_ready_ || frame >= animation_frames_) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid animation frame index");
    if (frame == 0) {
        current_frame_ = 0;
        push_output(0);
        return KHS_OK;
    }
    if (frame != current_frame_ + 1) return fail(KHS_ERROR_INVALID_STATE, "animation frames must be stepped in order");
    const size_t N3 = 3 * size_t(I.v.N), V3 = 3 * size_t(I.v.V);
    const uint32_t a = frame - 1, b = frame;
    const KhsResult r = run_frame(frame_dt, I.anim_root_x + a * N3, I.anim_root_r + a * N3, I.anim_root_x + b * N3,
                                  I.anim_root_r + b * N3, I.v.V ? I.anim_col + a * V3 : nullptr,
                                  I.v.V ? I.anim_col + b * V3 : nullptr, frame, animation_frames_);
    if (r == KHS_OK) {
        current_frame_ = frame;
        push_ring(frame);
        push_output(frame);
    }
    return r;
}

void Engine::push_output(uint32_t frame)
{
    Impl &I = *d_;
    if (!I.out_dev || !I.original_count) return;
    const uint32_t k = I.out_next;
    I.out_next = uint32_t((k + 1) % I.out_frame.size());
    for (int64_t &held : I.out_frame)
        if (held == int64_t(frame)) held = -1;  // an older pass over this frame (before a rollback)
    const size_t per = 3 * size_t(I.original_count);
    double *dst = I.out_dev + k * per;
    // The slot's previous copy must have finished before the gather
    // overwrites it; an event never recorded does not wait.
    KHS_CUDA(cudaStreamWaitEvent(I.stream, I.out_copied[k], 0));
    I.launch("k_gather", k_gather, grid_for(I.original_count), kBlock, I.v.q, I.mapping_dev, I.original_count, dst);
    KHS_CUDA(cudaEventRecord(I.out_gathered[k], I.stream));
    KHS_CUDA(cudaStreamWaitEvent(I.copy_stream, I.out_gathered[k], 0));
    KHS_CUDA(cudaMemcpyAsync(I.out_host + k * per, dst, per * 8, cudaMemcpyDeviceToHost, I.copy_stream));
    KHS_CUDA(cudaEventRecord(I.out_copied[k], I.copy_stream));
    I.out_frame[k] = int64_t(frame);
}

// Outputs of frames after `frame` belong to a trajectory that a rollback or
// a checkpoint restore has left.
void Engine::drop_outputs_after(uint32_t frame)
{
    for (int64_t &held : d_->out_frame)
        if (held > int64_t(frame)) held = -1;
}

KhsResult Engine::set_output_ring(uint32_t slots)
{
    Impl &I = *d_;
    if (slots > 1024) return fail(KHS_ERROR_INVALID_ARGUMENT, "output ring holds at most 1024 frames");
    I.sync();
    I.release_output();
    if (!slots) return KHS_OK;
    const size_t bytes = size_t(slots) * 3 * size_t(I.original_count) * 8;
    if (!I.copy_stream) KHS_CUDA(cudaStreamCreateWithFlags(&I.copy_stream, cudaStreamNonBlocking));
    if (cudaMalloc(reinterpret_cast<void **>(&I.out_dev), std::max<size_t>(bytes, 256)) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void **>(&I.out_host), std::max<size_t>(bytes, 256), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        if (I.out_dev) cudaFree(I.out_dev);
        I.out_dev = I.out_host = nullptr;
        return fail(KHS_ERROR_OUT_OF_MEMORY, "cannot allocate the output ring");
    }
    I.out_bytes = bytes;
    I.resident += bytes;
    gpu_stats_.resident_bytes = I.resident;
    I.out_gathered.resize(slots);
    I.out_copied.resize(slots);
    for (uint32_t k = 0; k < slots; ++k) {
        KHS_CUDA(cudaEventCreateWithFlags(&I.out_gathered[k], cudaEventDisableTiming));
        KHS_CUDA(cudaEventCreateWithFlags(&I.out_copied[k], cudaEventDisableTiming));
    }
    I.out_frame.assign(slots, -1);
    I.out_next = 0;
    return KHS_OK;
}

KhsResult Engine::output_frame(uint32_t frame, KhsVec3 *out, uint32_t capacity, const KhsVec3 **view)
{
    Impl &I = *d_;
    if (!I.out_dev) return fail(KHS_ERROR_INVALID_STATE, "the output ring is off");
    size_t k = I.out_frame.size();
    for (size_t s = 0; s < I.out_frame.size(); ++s)
        if (I.out_frame[s] == int64_t(frame)) k = s;
    if (k == I.out_frame.size()) return fail(KHS_ERROR_INVALID_ARGUMENT, "the frame is not in the output ring");
    if (out && capacity < I.original_count) return fail(KHS_ERROR_INVALID_ARGUMENT, "output buffer smaller than the point count");
    KHS_CUDA(cudaEventSynchronize(I.out_copied[k]));
    const double *src = I.out_host + k * 3 * size_t(I.original_count);
    if (view) *view = reinterpret_cast<const KhsVec3 *>(src);
    if (out) std::memcpy(out, src, size_t(I.original_count) * 24);
    return KHS_OK;
}

void Engine::push_ring(uint32_t frame)
{
    Impl &I = *d_;
    if (!I.ring) return;
    const size_t slots = I.ring_frame.size(), qn = 6 * size_t(I.v.N);
    const size_t k = frame % slots;
    KHS_CUDA(cudaMemcpyAsync(I.ring + 2 * qn * k, I.v.q, qn * 8, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.ring + 2 * qn * k + qn, I.v.v, qn * 8, cudaMemcpyDeviceToDevice, I.stream));
    I.ring_frame[k] = int64_t(frame);
}

KhsResult Engine::set_rollback_ring(uint32_t slots)
{
    Impl &I = *d_;
    if (slots > 1024) return fail(KHS_ERROR_INVALID_ARGUMENT, "rollback ring holds at most 1024 frames");
    I.sync();
    if (I.ring) { cudaFree(I.ring); I.ring = nullptr; I.resident -= I.ring_bytes; I.ring_bytes = 0; }
    I.ring_frame.clear();
    if (!slots) return KHS_OK;
    const size_t bytes = size_t(slots) * 2 * 6 * size_t(I.v.N) * 8;
    if (cudaMalloc(reinterpret_cast<void **>(&I.ring), bytes) != cudaSuccess) {
        I.ring = nullptr;
        cudaGetLastError();
        return fail(KHS_ERROR_OUT_OF_MEMORY, "cannot allocate the rollback ring");
    }
    I.ring_bytes = bytes;
    I.resident += bytes;
    I.ring_frame.assign(slots, -1);
    gpu_stats_.resident_bytes = I.resident;
    if (animation_ready_) push_ring(current_frame_);
    return KHS_OK;
}

KhsResult Engine::rollback_to_frame(uint32_t frame)
{
    Impl &I = *d_;
    if (!animation_ready_) return fail(KHS_ERROR_INVALID_STATE, "finalize the animation before rolling back");
    const size_t slots = I.ring_frame.size();
    if (!I.ring || !slots || I.ring_frame[frame % slots] != int64_t(frame))
        return fail(KHS_ERROR_INVALID_ARGUMENT, "frame is not held by the rollback ring");
    const size_t qn = 6 * size_t(I.v.N), k = frame % slots, qb = qn * 8;
    KHS_CUDA(cudaMemcpyAsync(I.v.q, I.ring + 2 * qn * k, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v.v, I.ring + 2 * qn * k + qn, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v.q_old, I.v.q, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.q_snap, I.v.q, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v_snap, I.v.v, qb, cudaMemcpyDeviceToDevice, I.stream));
    I.sync();
    // Frames after the restored one are no longer on this trajectory.
    for (size_t j = 0; j < slots; ++j)
        if (I.ring_frame[j] > int64_t(frame)) I.ring_frame[j] = -1;
    drop_outputs_after(frame);
    current_frame_ = frame;
    cancel_.store(false);
    progress_frame_.store(frame);
    progress_substep_.store(0); progress_substep_count_.store(0); progress_iteration_.store(0);
    progress_phase_.store(KHS_PHASE_FINISHED);
    step_stats_ = {};
    step_stats_.struct_size = sizeof(step_stats_);
    step_stats_.phase = KHS_PHASE_FINISHED;
    clear_failure();
    error_.clear();
    return KHS_OK;
}

namespace {
struct CheckpointHeader {
    uint64_t magic;
    uint32_t abi_version;
    uint32_t animation_frame;
    uint64_t dof_count;
};
}  // namespace

uint64_t Engine::checkpoint_size() const
{
    if (!initialized_ || !animation_ready_) return 0;
    return sizeof(CheckpointHeader) + 2 * uint64_t(6) * d_->v.N * sizeof(double);
}

KhsResult Engine::save_checkpoint(void *data, uint64_t capacity)
{
    Impl &I = *d_;
    const uint64_t required = checkpoint_size();
    if (!data || !required || capacity < required) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid checkpoint output buffer");
    CheckpointHeader h{kCheckpointMagic, KHS_ABI_VERSION, current_frame_, uint64_t(6) * I.v.N};
    auto *out = static_cast<unsigned char *>(data);
    std::memcpy(out, &h, sizeof(h));
    const size_t qb = 6 * size_t(I.v.N) * 8;
    KHS_CUDA(cudaMemcpyAsync(out + sizeof(h), I.v.q, qb, cudaMemcpyDeviceToHost, I.stream));
    KHS_CUDA(cudaMemcpyAsync(out + sizeof(h) + qb, I.v.v, qb, cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    error_.clear();
    return KHS_OK;
}

KhsResult Engine::restore_checkpoint(const void *data, uint64_t size)
{
    Impl &I = *d_;
    const uint64_t required = checkpoint_size();
    if (!data || !required || size != required) return fail(KHS_ERROR_INVALID_ARGUMENT, "invalid checkpoint size");
    CheckpointHeader h{};
    std::memcpy(&h, data, sizeof(h));
    if (h.magic != kCheckpointMagic || h.abi_version != KHS_ABI_VERSION || h.dof_count != uint64_t(6) * I.v.N ||
        h.animation_frame >= animation_frames_)
        return fail(KHS_ERROR_INVALID_ARGUMENT, "checkpoint does not match this solver");
    const auto *in = static_cast<const unsigned char *>(data);
    const size_t qb = 6 * size_t(I.v.N) * 8;
    KHS_CUDA(cudaMemcpyAsync(I.v.q, in + sizeof(h), qb, cudaMemcpyHostToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v.v, in + sizeof(h) + qb, qb, cudaMemcpyHostToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v.q_old, I.v.q, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.q_snap, I.v.q, qb, cudaMemcpyDeviceToDevice, I.stream));
    KHS_CUDA(cudaMemcpyAsync(I.v_snap, I.v.v, qb, cudaMemcpyDeviceToDevice, I.stream));
    // The rollback ring must describe the restored trajectory: frames after
    // the checkpoint's are forgotten, and the checkpoint's own frame is
    // replaced by the restored state (the slot may hold another trajectory).
    for (size_t j = 0; j < I.ring_frame.size(); ++j)
        if (I.ring_frame[j] > int64_t(h.animation_frame)) I.ring_frame[j] = -1;
    push_ring(h.animation_frame);
    I.sync();
    current_frame_ = h.animation_frame;
    drop_outputs_after(h.animation_frame);
    cancel_.store(false);
    progress_frame_.store(h.animation_frame);
    progress_substep_.store(0); progress_substep_count_.store(0); progress_iteration_.store(0);
    progress_phase_.store(KHS_PHASE_FINISHED);
    step_stats_ = {};
    step_stats_.struct_size = sizeof(step_stats_);
    step_stats_.phase = KHS_PHASE_FINISHED;
    clear_failure();
    error_.clear();
    return KHS_OK;
}

KhsResult Engine::copy_original_positions(KhsVec3 *out, uint32_t capacity) const
{
    Impl &I = *d_;
    if (!out || capacity < I.original_count) return KHS_ERROR_INVALID_ARGUMENT;
    if (!I.original_count) return KHS_OK;
    I.launch("k_gather", k_gather, grid_for(I.original_count), kBlock, I.v.q, I.mapping_dev, I.original_count, I.mapping_gather_out);
    KHS_CUDA(cudaGetLastError());
    KHS_CUDA(cudaMemcpyAsync(out, I.mapping_gather_out, size_t(I.original_count) * 24, cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    return KHS_OK;
}

KhsResult Engine::copy_internal_positions(KhsVec3 *out, uint32_t capacity) const
{
    Impl &I = *d_;
    if (!out || capacity < I.v.N) return KHS_ERROR_INVALID_ARGUMENT;
    I.launch("k_gather", k_gather, grid_for(I.v.N), kBlock, I.v.q, nullptr, I.v.N, I.mapping_gather_out);
    KHS_CUDA(cudaGetLastError());
    KHS_CUDA(cudaMemcpyAsync(out, I.mapping_gather_out, size_t(I.v.N) * 24, cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    return KHS_OK;
}

KhsResult Engine::copy_state(double *q, double *v, uint64_t capacity) const
{
    Impl &I = *d_;
    const size_t dof = 6 * size_t(I.v.N);
    if (capacity < dof) return KHS_ERROR_INVALID_ARGUMENT;
    if (q) KHS_CUDA(cudaMemcpyAsync(q, I.v.q, dof * 8, cudaMemcpyDeviceToHost, I.stream));
    if (v) KHS_CUDA(cudaMemcpyAsync(v, I.v.v, dof * 8, cudaMemcpyDeviceToHost, I.stream));
    I.sync();
    return KHS_OK;
}

KhsResult Engine::query_contacts(const double *q, uint64_t dof, KhsxContactRecord *out, uint32_t capacity)
{
    Impl &I = *d_;
    if (!q || dof < 6 * uint64_t(I.v.N) || !out || capacity < I.v.E) return KHS_ERROR_INVALID_ARGUMENT;
    KHS_CUDA(cudaMemcpyAsync(I.v.q_base, q, 6 * size_t(I.v.N) * 8, cudaMemcpyHostToDevice, I.stream));
    I.launch("k_contact_query", mode_ ? k_contact<true> : k_contact<false>, grid_for(I.v.E), kBlock, I.v,
             static_cast<const double *>(I.v.q_base));
    KHS_CUDA(cudaGetLastError());
    return copy_contact_records(out, capacity);
}

namespace {

constexpr int kMaxScratchDevices = 64;
std::mutex g_no_alloc_mutex;
void *g_no_alloc_ptr[kMaxScratchDevices] = {};

// Device address of g_no_alloc_scratch on device `device`, looked up once per
// device with that device current (the first call may load the module).
cudaError_t no_alloc_scratch(int device, void **ptr)
{
    if (device < 0 || device >= kMaxScratchDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_no_alloc_mutex);
    if (!g_no_alloc_ptr[device]) {
        int previous = 0;
        cudaError_t err = cudaGetDevice(&previous);
        if (err != cudaSuccess) return err;
        if (previous != device && (err = cudaSetDevice(device)) != cudaSuccess) return err;
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_no_alloc_scratch);
        if (previous != device) {
            const cudaError_t back = cudaSetDevice(previous);
            if (err == cudaSuccess) err = back;
        }
        if (err != cudaSuccess) return err;
        if (!p) return cudaErrorInvalidSymbol;
        g_no_alloc_ptr[device] = p;
    }
    *ptr = g_no_alloc_ptr[device];
    return cudaSuccess;
}

}  // namespace

KhsResult Engine::query_contacts_no_alloc(const double *q, uint64_t dof, KhsxContactRecord *out, uint32_t capacity)
{
    Impl &I = *d_;
    const View &v = I.v;
    if (!q || dof < 6 * uint64_t(v.N) || !out || capacity < v.E) return KHS_ERROR_INVALID_ARGUMENT;
    const uint64_t q_bytes = 6 * uint64_t(v.N) * sizeof(double);
    const uint64_t rec_offset = (q_bytes + 255) / 256 * 256;
    if (rec_offset + uint64_t(v.E) * sizeof(KhsxContactRecord) > KHSX_NO_ALLOC_SCRATCH_BYTES) return KHS_ERROR_INVALID_ARGUMENT;
    if (v.E == 0) return KHS_OK;
    void *base = nullptr;
    if (no_alloc_scratch(kDevice, &base) != cudaSuccess) return KHS_ERROR_INTERNAL;
    double *q_dev = static_cast<double *>(base);
    KhsxContactRecord *rec = reinterpret_cast<KhsxContactRecord *>(static_cast<unsigned char *>(base) + rec_offset);
    if (cudaMemcpyAsync(q_dev, q, q_bytes, cudaMemcpyHostToDevice, I.stream) != cudaSuccess) return KHS_ERROR_INTERNAL;
    if (mode_) k_contact_query_records<true><<<grid_for(v.E), kBlock, 0, I.stream>>>(v, q_dev, rec);
    else k_contact_query_records<false><<<grid_for(v.E), kBlock, 0, I.stream>>>(v, q_dev, rec);
    ++I.launches;
    if (cudaGetLastError() != cudaSuccess) return KHS_ERROR_INTERNAL;
    if (cudaMemcpyAsync(out, rec, size_t(v.E) * sizeof(KhsxContactRecord), cudaMemcpyDeviceToHost, I.stream) != cudaSuccess)
        return KHS_ERROR_INTERNAL;
    return cudaStreamSynchronize(I.stream) == cudaSuccess ? KHS_OK : KHS_ERROR_INTERNAL;
}

KhsResult Engine::copy_contact_records(KhsxContactRecord *out, uint32_t capacity) const
{
    Impl &I = *d_;
    const size_t E = I.v.E;
    if (!out || capacity < E) return KHS_ERROR_INVALID_ARGUMENT;
    std::vector<uint32_t> cand(E), tri(E);
    std::vector<uint8_t> flags(E);
    std::vector<double> gap(E);
    if (E) {
        KHS_CUDA(cudaMemcpyAsync(cand.data(), I.v.c_cand, E * 4, cudaMemcpyDeviceToHost, I.stream));
        KHS_CUDA(cudaMemcpyAsync(tri.data(), I.v.c_tri, E * 4, cudaMemcpyDeviceToHost, I.stream));
        KHS_CUDA(cudaMemcpyAsync(flags.data(), I.v.c_flags, E, cudaMemcpyDeviceToHost, I.stream));
        KHS_CUDA(cudaMemcpyAsync(gap.data(), I.v.c_gap, E * 8, cudaMemcpyDeviceToHost, I.stream));
        I.sync();
    }
    for (size_t e = 0; e < E; ++e) {
        const bool closest = flags[e] & kFlagClosest;
        out[e] = KhsxContactRecord{cand[e], closest ? tri[e] : kNone, (flags[e] & kFlagActive) ? 1u : 0u, 0u,
                                   closest ? gap[e] : std::numeric_limits<double>::infinity()};
    }
    return KHS_OK;
}

void Engine::set_profiling(bool on)
{
    Impl &I = *d_;
    I.sync();
    I.profiling = on;
}

std::vector<KernelTiming> Engine::kernel_timings() const
{
    Impl &I = *d_;
    I.sync();
    std::vector<KernelTiming> out;
    for (const auto &k : I.kstats) out.push_back({k.name, k.launches, k.ms});
    return out;
}

void Engine::reset_kernel_timings()
{
    Impl &I = *d_;
    I.sync();
    I.kstats.clear();
}

uint64_t Engine::kernel_launches() const { return d_->launches; }

bool query_device(KhsGpuInfo &info, std::string &error)
{
    std::memset(&info, 0, sizeof(info));
    info.struct_size = sizeof(info);
    int count = 0;
    const cudaError_t r = cudaGetDeviceCount(&count);
    if (r != cudaSuccess || count < 1) {
        error = r == cudaSuccess ? "no CUDA GPU found" : cudaGetErrorString(r);
        cudaGetLastError();
        return false;
    }
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) { error = "cannot query the CUDA device"; return false; }
    info.available = 1;
    info.device_ordinal = 0;
    info.compute_capability_major = uint32_t(prop.major);
    info.compute_capability_minor = uint32_t(prop.minor);
    info.total_vram_bytes = prop.totalGlobalMem;
    std::strncpy(info.device_name, prop.name, sizeof(info.device_name) - 1);
    return true;
}

}  // namespace khs
