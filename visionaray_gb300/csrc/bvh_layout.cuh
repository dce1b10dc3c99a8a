// HBM layout of a traversal BVH.
//
// Nodes: one 64-byte record per inner node holding BOTH children's boxes, so a
// traversal step is four coalesced 128-bit loads and two slab tests (the node-pair
// layout of Aila & Laine, "Understanding the Efficiency of Ray Traversal on GPUs",
// HPG 2009):
//     xy0  = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//     xy1  = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//     z01  = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//     link = (child0, child1, height, parent)
// child >= 0 is an inner node index; child < 0 is a leaf whose first triangle is
// ~child.  height is the subtree height (leaves 0); parent is the parent inner
// node (-1 for the root) -- both are build-time fields, unused by traversal.
//
// Triangles: 48 bytes, three float4, stored in leaf order so that a leaf is a
// contiguous run; the last triangle of a leaf carries kLastInLeaf.
//     t0 = (v1.x, v1.y, v1.z, prim_id bits)
//     t1 = (e1.x, e1.y, e1.z, geom_id bits)
//     t2 = (e2.x, e2.y, e2.z, flags bits)
#pragma once

#include <cstdint>

namespace gbrt {

struct __align__(16) bvh2_node
{
    float4 xy0;
    float4 xy1;
    float4 z01;
    int4 link;
};
static_assert(sizeof(bvh2_node) == 64, "node is one 64-byte record");

struct __align__(16) tri48
{
    float4 t0;
    float4 t1;
    float4 t2;
};
static_assert(sizeof(tri48) == 48, "triangle is 48 bytes");

constexpr uint32_t kLastInLeaf = 1u;
constexpr int kStackSize = 64;   // traversal stack entries (tree height must stay below)

// 4-wide node (128 bytes = eight 128-bit loads), collapsed from the node pairs: the
// six box planes of the four children in SoA form, so one float4 per plane serves all
// four slab tests.  count[k] > 0: leaf of count[k] contiguous triangles starting at
// child[k]; count[k] == 0: inner child, child[k] indexes the 4-wide nodes; count[k] < 0:
// empty slot.
struct __align__(16) bvh4_node
{
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 child;
    int4 count;
};
static_assert(sizeof(bvh4_node) == 128, "4-wide node is 128 bytes");

// Quantised 4-wide node (64 bytes = four 128-bit loads) in the byte layout of
// visionaray's bvh_compressed_node<4> (bvh.h:319-426): the children's boxes as 8-bit
// offsets from the node's origin in units of 2^e per axis (24 bytes, lo x/y/z then
// hi x/y/z, four children each), the children as packed {int id; short count} (24
// bytes), the origin (12 bytes) and the three exponents (3 bytes).  count > 0: leaf of
// count triangles from id; 0: inner child, id indexes these nodes; -1: empty slot.
// The quantisation rounds outward and the traversal decodes with directed rounding, so
// every decoded box contains its child's true box.
struct __align__(16) bvh4q_node
{
    unsigned char q[24];         // lo.x[4] lo.y[4] lo.z[4] hi.x[4] hi.y[4] hi.z[4]
    unsigned char children[24];  // 4 x {int32 id; int16 count}, packed
    float origin[3];
    signed char e[3];
    unsigned char pad;
};
static_assert(sizeof(bvh4q_node) == 64, "quantised 4-wide node is 64 bytes");

// 8-wide node (256 bytes = eight 256-bit loads): the same SoA planes for eight
// children, each plane two float4; child / count as for bvh4_node.
struct __align__(32) bvh8_node
{
    float4 lox[2], hix[2], loy[2], hiy[2], loz[2], hiz[2];
    int4 child[2];
    int4 count[2];
};
static_assert(sizeof(bvh8_node) == 256, "8-wide node is 256 bytes");

template <int W> struct wide_node;
template <> struct wide_node<4> { using type = bvh4_node; };
template <> struct wide_node<8> { using type = bvh8_node; };

constexpr int kStack4 = 96;        // 4-wide traversal stack entries (up to 3 per level)
constexpr int kStack8 = 160;       // 8-wide traversal stack entries (up to 7 per level)
constexpr int kLeafMax4 = 4;       // triangles per wide leaf (default)

} // namespace gbrt
