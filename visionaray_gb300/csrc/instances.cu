// Two-level instancing: a top-level tree of node pairs over instances, each a bottom-
// level tree (gbrt_bvh) and visionaray's mat4x3 transform (index_bvh_inst_t, bvh.h:
// 678-782).  A query walks the top-level tree; at an instance leaf it maps the ray
// into the instance's space exactly as transform_ray does (bvh.h:748-755: ori' =
// A (ori + trans_inv), dir' = A dir, the 3x3 product in the reference's operation
// order) and traverses the instance's tree with the best distance so far as its bound,
// which accepts the same hits as the reference's per-instance closest hit followed by
// the strict is_closer test (intersect.inl:362-394, update_if.h:45-107).
//
// The top-level tree is built on the host: instance counts are small next to triangle
// counts, and the reference builds its top-level tree on the host too (the viewer's
// index_bvh over bvh_inst, viewer.cpp:647-661).

#include "instances.cuh"

#include <algorithm>
#include <new>
#include <numeric>
#include <vector>


namespace gbrt {
namespace {

constexpr int kBlock = 128;

// The reference's float 3x3 algebra (math/detail/matrix3.inl, math.h:616-621), m[r][c].
struct m3
{
    float m[3][3];
};

inline float det2(float m00, float m01, float m10, float m11) { return m00 * m11 - m10 * m01; }

// inverse(matrix<3,3>) (matrix3.inl:285-305): cofactors over the determinant.
m3 inverse3(m3 const& x)
{
    auto m = [&](int r, int c) { return x.m[r][c]; };
    float a00 = det2(m(1, 1), m(1, 2), m(2, 1), m(2, 2));
    float a01 = det2(m(1, 0), m(1, 2), m(2, 0), m(2, 2));
    float a02 = det2(m(1, 0), m(1, 1), m(2, 0), m(2, 1));
    float a10 = det2(m(0, 1), m(0, 2), m(2, 1), m(2, 2));
    float a11 = det2(m(0, 0), m(0, 2), m(2, 0), m(2, 2));
    float a12 = det2(m(0, 0), m(0, 1), m(2, 0), m(2, 1));
    float a20 = det2(m(0, 1), m(0, 2), m(1, 1), m(1, 2));
    float a21 = det2(m(0, 0), m(0, 2), m(1, 0), m(1, 2));
    float a22 = det2(m(0, 0), m(0, 1), m(1, 0), m(1, 1));
    float det = m(0, 0) * a00 - m(0, 1) * a01 + m(0, 2) * a02;
    // the result's constructor takes its arguments column by column
    m3 r;
    r.m[0][0] = +a00 / det;
    r.m[1][0] = -a01 / det;
    r.m[2][0] = +a02 / det;
    r.m[0][1] = -a10 / det;
    r.m[1][1] = +a11 / det;
    r.m[2][1] = -a12 / det;
    r.m[0][2] = +a20 / det;
    r.m[1][2] = -a21 / det;
    r.m[2][2] = +a22 / det;
    return r;
}

// matrix<3,3> * vector<3> (matrix3.inl:226-234)
inline void mul3(m3 const& a, const float v[3], float out[3])
{
    for (int r = 0; r < 3; ++r) out[r] = a.m[r][0] * v[0] + a.m[r][1] * v[1] + a.m[r][2] * v[2];
}

struct box
{
    float lo[3], hi[3];
};

inline float vmin(float a, float b) { return a < b ? a : b; }
inline float vmax(float a, float b) { return a < b ? b : a; }

// get_bounds(instance) (detail/bvh/get_bounds.inl:30-56): affine = inverse(affine_inv),
// trans = -trans_inv, the 8 corners of the tree's root box (aabb.inl:305-324 order)
// mapped by affine * v + trans and inserted into an invalid box.
box instance_bounds(m3 const& affine_inv, const float trans_inv[3], gbrt_bvh const* blas)
{
    box r;
    for (int a = 0; a < 3; ++a)
    {
        r.lo[a] = FLT_MAX;
        r.hi[a] = -FLT_MAX;
    }
    if (blas->num_prims == 0) return r;
    m3 affine = inverse3(affine_inv);
    float trans[3] = { -trans_inv[0], -trans_inv[1], -trans_inv[2] };
    const float* mn = blas->lo;
    const float* mx = blas->hi;
    const float corners[8][3] = { { mx[0], mx[1], mx[2] }, { mn[0], mx[1], mx[2] }, { mn[0], mn[1], mx[2] },
                                  { mx[0], mn[1], mx[2] }, { mn[0], mx[1], mn[2] }, { mx[0], mx[1], mn[2] },
                                  { mx[0], mn[1], mn[2] }, { mn[0], mn[1], mn[2] } };
    for (auto const& c : corners)
    {
        float w[3];
        mul3(affine, c, w);
        for (int a = 0; a < 3; ++a)
        {
            float v = w[a] + trans[a];
            r.lo[a] = vmin(r.lo[a], v);
            r.hi[a] = vmax(r.hi[a], v);
        }
    }
    return r;
}

box merge(box const& a, box const& b)
{
    box r;
    for (int k = 0; k < 3; ++k)
    {
        r.lo[k] = vmin(a.lo[k], b.lo[k]);
        r.hi[k] = vmax(a.hi[k], b.hi[k]);
    }
    return r;
}

float half_area(box const& b)
{
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Binned SAH split (16 bins per axis over the instance centroids; cost = half area x
// instances on each side), one instance per leaf; the median of the longest centroid
// axis when every centroid falls in one bin, and below `sah_levels` levels, so that the
// tree is at most 31 levels deep (the traversal's top-level stack holds 32 entries).
// An instance box as large as the scene (a room around its furniture) is split off near
// the root instead of widening half of the tree.  Returns the link of the subtree
// (inner index, or ~instance).
int32_t build_top(std::vector<uint32_t>& ids, size_t first, size_t last, std::vector<box> const& boxes,
                  std::vector<bvh2_node>& nodes, box& out_box, int sah_levels)
{
    if (last - first == 1)
    {
        out_box = boxes[ids[first]];
        return ~int32_t(ids[first]);
    }
    auto centroid = [&](uint32_t i, int a) { return 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]); };
    float clo[3] = { FLT_MAX, FLT_MAX, FLT_MAX }, chi[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    for (size_t i = first; i < last; ++i)
        for (int a = 0; a < 3; ++a)
        {
            float c = centroid(ids[i], a);
            clo[a] = vmin(clo[a], c);
            chi[a] = vmax(chi[a], c);
        }
    constexpr int kBins = 16;
    // the bin of a centroid; a non-finite one goes to bin 0
    auto bin_of = [&](uint32_t i, int a, float extent) {
        const float f = float(kBins) * (centroid(i, a) - clo[a]) / extent;
        return f >= 0.0f ? (f < float(kBins) ? int(f) : kBins - 1) : 0;
    };
    int best_axis = -1, best_split = 0;
    float best_cost = FLT_MAX;
    for (int a = 0; a < 3 && sah_levels > 0; ++a)
    {
        const float extent = chi[a] - clo[a];
        if (!(extent > 0.0f)) continue;
        box bb[kBins];
        size_t cnt[kBins] = {};
        for (int k = 0; k < kBins; ++k)
            for (int c = 0; c < 3; ++c)
            {
                bb[k].lo[c] = FLT_MAX;
                bb[k].hi[c] = -FLT_MAX;
            }
        for (size_t i = first; i < last; ++i)
        {
            const int k = bin_of(ids[i], a, extent);
            bb[k] = merge(bb[k], boxes[ids[i]]);
            ++cnt[k];
        }
        // cost of splitting after bin k: left bins [0, k], right bins (k, kBins)
        float right_area[kBins];
        size_t right_cnt[kBins];
        box acc = bb[kBins - 1];
        size_t n_acc = cnt[kBins - 1];
        for (int k = kBins - 2; k >= 0; --k)
        {
            right_area[k] = n_acc ? half_area(acc) : 0.0f;
            right_cnt[k] = n_acc;
            acc = merge(acc, bb[k]);
            n_acc += cnt[k];
        }
        box left = bb[0];
        size_t n_left = cnt[0];
        for (int k = 0; k < kBins - 1; ++k)
        {
            if (k > 0)
            {
                left = merge(left, bb[k]);
                n_left += cnt[k];
            }
            if (n_left == 0 || right_cnt[k] == 0) continue;
            const float cost = half_area(left) * float(n_left) + right_area[k] * float(right_cnt[k]);
            if (cost < best_cost)
            {
                best_cost = cost;
                best_axis = a;
                best_split = k;
            }
        }
    }
    size_t mid;
    if (best_axis >= 0)
    {
        const int a = best_axis;
        const float extent = chi[a] - clo[a];
        auto goes_left = [&](uint32_t i) { return bin_of(i, a, extent) <= best_split; };
        // stable partition: instances keep their relative order on each side
        mid = size_t(std::stable_partition(ids.begin() + first, ids.begin() + last, goes_left) - ids.begin());
    }
    else
    {
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        mid = first + (last - first) / 2;
        std::nth_element(ids.begin() + first, ids.begin() + mid, ids.begin() + last, [&](uint32_t x, uint32_t y) {
            float cx = boxes[x].lo[axis] + boxes[x].hi[axis], cy = boxes[y].lo[axis] + boxes[y].hi[axis];
            return cx < cy || (cx == cy && x < y);
        });
    }
    int32_t self = int32_t(nodes.size());
    nodes.emplace_back();
    box lb, rb;
    int32_t l = build_top(ids, first, mid, boxes, nodes, lb, sah_levels - 1);
    int32_t r = build_top(ids, mid, last, boxes, nodes, rb, sah_levels - 1);
    bvh2_node& nd = nodes[size_t(self)];
    nd.xy0 = make_float4(lb.lo[0], lb.hi[0], lb.lo[1], lb.hi[1]);
    nd.xy1 = make_float4(rb.lo[0], rb.hi[0], rb.lo[1], rb.hi[1]);
    nd.z01 = make_float4(lb.lo[2], lb.hi[2], rb.lo[2], rb.hi[2]);
    nd.link = make_int4(l, r, 0, 0);
    out_box = merge(lb, rb);
    return self;
}

template <bool AnyHit>
__global__ void __launch_bounds__(kBlock) tlas_trace(tlas_view tv, const gbrt_ray* __restrict__ rays, uint32_t n,
                                                     gbrt_hit_inst* __restrict__ hits, uint32_t* __restrict__ status)
{
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    float4 r0 = ldg4(&rays[i]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
    const tlas_result best = traverse_tlas<AnyHit>(tv, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint4 w0, w1;
    if (best.inst >= 0)
    {
        const bvh_view bv = tv.views[best.inst];
        float4 t0 = ldg4(&bv.tris[best.tri].t0), t1 = ldg4(&bv.tris[best.tri].t1);
        w0 = make_uint4(__float_as_uint(t0.w), uint32_t(best.inst), __float_as_uint(best.t), __float_as_uint(best.u));
        w1 = make_uint4(__float_as_uint(best.v), __float_as_uint(t1.w), 0u, 0u);
    }
    else
    {
        w0 = make_uint4(GBRT_NO_HIT, GBRT_NO_HIT, __float_as_uint(FLT_MAX), 0u);
        w1 = make_uint4(0u, 0u, 0u, 0u);
    }
    reinterpret_cast<uint4*>(hits)[2 * size_t(i)] = w0;
    reinterpret_cast<uint4*>(hits)[2 * size_t(i) + 1] = w1;
}

void free_tlas(gbrt_tlas* t)
{
    cudaFree(t->nodes);
    cudaFree(t->records);
    cudaFree(t->forward);
    cudaFree(t->views);
}

} // namespace
} // namespace gbrt

using namespace gbrt;

extern "C" gbrt_status gbrt_tlas_build(gbrt_context* ctx, gbrt_instance const* h_instances, uint32_t num_instances,
                                       gbrt_tlas** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out || (num_instances && !h_instances)) return fail(ctx, GBRT_ERR_INVALID_ARG, "tlas_build: null argument");
    *out = nullptr;
    if (num_instances > (1u << 24)) return fail(ctx, GBRT_ERR_TOO_LARGE, "tlas_build: more than 2^24 instances");
    for (uint32_t k = 0; k < num_instances; ++k)
        if (!h_instances[k].blas) return fail(ctx, GBRT_ERR_INVALID_ARG, "tlas_build: instance without a tree");
    std::vector<float4> records(size_t(num_instances) * 3), forward(size_t(num_instances) * 3);
    std::vector<bvh_view> views(num_instances);
    std::vector<box> boxes(num_instances);
    for (uint32_t k = 0; k < num_instances; ++k)
    {
        gbrt_instance const& in = h_instances[k];
        // index_bvh_inst_t(ref, transform) (bvh.h:694-700): affine_inv =
        // inverse(top_left(transform)), trans_inv = -transform(3)
        m3 tl;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) tl.m[r][c] = in.transform[3 * r + c];
        m3 ainv = inverse3(tl);
        float tinv[3] = { -in.transform[9], -in.transform[10], -in.transform[11] };
        for (int r = 0; r < 3; ++r) records[3 * k + r] = make_float4(ainv.m[r][0], ainv.m[r][1], ainv.m[r][2], tinv[r]);
        // the instance-to-world map as get_bounds forms it (get_bounds.inl:30-56):
        // affine = inverse(affine_inv), trans = -trans_inv
        m3 aff = inverse3(ainv);
        for (int r = 0; r < 3; ++r) forward[3 * k + r] = make_float4(aff.m[r][0], aff.m[r][1], aff.m[r][2], -tinv[r]);
        views[k] = view_of(in.blas);
        boxes[k] = instance_bounds(ainv, tinv, in.blas);
    }
    std::vector<bvh2_node> nodes;
    int32_t root = INT32_MIN;
    if (num_instances > 0)
    {
        std::vector<uint32_t> ids(num_instances);
        std::iota(ids.begin(), ids.end(), 0u);
        nodes.reserve(num_instances);
        box all;
        // SAH levels such that SAH levels + the median split's ceil(log2 n) <= 31
        int log2n = 0;
        while ((uint64_t(1) << log2n) < uint64_t(num_instances)) ++log2n;
        root = build_top(ids, 0, num_instances, boxes, nodes, all, 31 - log2n);
    }
    device_guard g(ctx->device);
    auto* t = new (std::nothrow) gbrt_tlas;
    if (!t) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "tlas_build: host allocation");
    t->device = ctx->device;
    t->num_instances = num_instances;
    t->num_inner = uint32_t(nodes.size());
    t->root = root;
    t->blas.resize(num_instances);
    for (uint32_t k = 0; k < num_instances; ++k) t->blas[k] = h_instances[k].blas;
    cudaError_t e = cudaSuccess;
    if (num_instances > 0)
    {
        if ((e = cudaMalloc(&t->records, records.size() * sizeof(float4))) == cudaSuccess &&
            (e = cudaMalloc(&t->forward, forward.size() * sizeof(float4))) == cudaSuccess &&
            (e = cudaMalloc(&t->views, views.size() * sizeof(bvh_view))) == cudaSuccess)
        {
            e = cudaMemcpy(t->records, records.data(), records.size() * sizeof(float4), cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(t->forward, forward.data(), forward.size() * sizeof(float4), cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(t->views, views.data(), views.size() * sizeof(bvh_view), cudaMemcpyHostToDevice);
        }
        if (e == cudaSuccess && !nodes.empty())
        {
            e = cudaMalloc(&t->nodes, nodes.size() * sizeof(bvh2_node));
            if (e == cudaSuccess)
                e = cudaMemcpy(t->nodes, nodes.data(), nodes.size() * sizeof(bvh2_node), cudaMemcpyHostToDevice);
        }
    }
    if (e != cudaSuccess)
    {
        free_tlas(t);
        delete t;
        return check_cuda(ctx, e, "tlas_build");
    }
    *out = t;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_tlas_destroy(gbrt_tlas* tlas)
{
    if (!tlas) return GBRT_ERR_INVALID_ARG;
    device_guard g(tlas->device);
    free_tlas(tlas);
    delete tlas;
    return GBRT_OK;
}

namespace {

gbrt_status tlas_trace_call(gbrt_context* ctx, gbrt_tlas const* tlas, gbrt_ray const* d_rays, uint32_t n,
                            gbrt_hit_inst* d_hits, bool any_hit)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!tlas || (n && (!d_rays || !d_hits))) return fail(ctx, GBRT_ERR_INVALID_ARG, "tlas_trace: null argument");
    if ((reinterpret_cast<uintptr_t>(d_rays) & 15u) || (reinterpret_cast<uintptr_t>(d_hits) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "tlas_trace: rays and hits must be 16-byte aligned");
    if (n == 0) return GBRT_OK;
    device_guard g(ctx->device);
    tlas_view tv{ tlas->nodes, tlas->records, tlas->views, tlas->num_instances > 0 ? tlas->root : kEmptyLink,
                  int32_t(tlas->num_inner), int32_t(tlas->num_instances) };
    const uint32_t blocks = (n + kBlock - 1) / kBlock;
    if (any_hit)
        tlas_trace<true><<<blocks, kBlock, 0, ctx->stream>>>(tv, d_rays, n, d_hits, ctx->d_status);
    else
        tlas_trace<false><<<blocks, kBlock, 0, ctx->stream>>>(tv, d_rays, n, d_hits, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "tlas_trace");
    return GBRT_OK;
}

} // namespace

extern "C" gbrt_status gbrt_tlas_trace_closest_hit(gbrt_context* ctx, gbrt_tlas const* tlas, gbrt_ray const* d_rays,
                                                   uint32_t n, gbrt_hit_inst* d_hits)
{
    return tlas_trace_call(ctx, tlas, d_rays, n, d_hits, false);
}

extern "C" gbrt_status gbrt_tlas_trace_any_hit(gbrt_context* ctx, gbrt_tlas const* tlas, gbrt_ray const* d_rays,
                                               uint32_t n, gbrt_hit_inst* d_hits)
{
    return tlas_trace_call(ctx, tlas, d_rays, n, d_hits, true);
}
