// CPU restatement of visionaray's ray-tracing hot path -- TEST INFRASTRUCTURE ONLY
// (see oracle.h).  Build with -ffp-contract=off.

#include "oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// math/detail/math.h:118-128: min(x, y) = x < y ? x : y, max(x, y) = x < y ? y : x.
// The NaN behaviour of these forms (not fminf/fmaxf) matters for degenerate inputs.
inline float vmin(float x, float y) { return x < y ? x : y; }
inline float vmax(float x, float y) { return x < y ? y : x; }

struct v3
{
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline v3 load3(const float* p) { return { p[0], p[1], p[2] }; }
inline v3 operator+(v3 a, v3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
inline v3 operator-(v3 a, v3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
inline v3 operator*(v3 a, v3 b) { return { a.x * b.x, a.y * b.y, a.z * b.z }; }
inline v3 operator*(v3 a, float s) { return { a.x * s, a.y * s, a.z * s }; }
inline v3 operator/(v3 a, v3 b) { return { a.x / b.x, a.y / b.y, a.z / b.z }; }
inline v3 vmin3(v3 a, v3 b) { return { vmin(a.x, b.x), vmin(a.y, b.y), vmin(a.z, b.z) }; }
inline v3 vmax3(v3 a, v3 b) { return { vmax(a.x, b.x), vmax(a.y, b.y), vmax(a.z, b.z) }; }

// math/detail/vector3.inl:292-307 (cross, dot), evaluated left to right.
inline v3 cross(v3 u, v3 v)
{
    return { u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x };
}
inline float dot(v3 u, v3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; }

// math/detail/vector.inl:874-884: ties go to the later component.
inline int max_index(v3 u)
{
    int i = u[1] < u[0] ? 0 : 1;
    i = u[2] < u[i] ? i : 2;
    return i;
}

// basic_aabb<float> (math/aabb.h, math/detail/aabb.inl:58-150, 180-230).
struct box
{
    v3 lo, hi;

    void invalidate()
    {
        lo = { FLT_MAX, FLT_MAX, FLT_MAX };
        hi = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    }
    void insert(v3 p)
    {
        lo = vmin3(lo, p);
        hi = vmax3(hi, p);
    }
    void insert(box const& b)
    {
        lo = vmin3(lo, b.lo);
        hi = vmax3(hi, b.hi);
    }
    v3 center() const { return (hi + lo) * 0.5f; }
    v3 size() const { return hi - lo; }
};

inline box combine(box a, box const& b)
{
    a.insert(b);
    return a;
}

// The GPU builder's float atomicMin / atomicMax (detail/bvh/lbvh.h:63-91): a compare-
// and-swap loop from +FLT_MAX / -FLT_MAX that stores a value only when it lies below
// (above) the current one, so NaN, +Inf into a minimum and -Inf into a maximum never
// land.  Folding cas_lo / cas_hi of each value gives those bounds in any order.
inline float cas_lo(float x) { return x < FLT_MAX ? x : FLT_MAX; }
inline float cas_hi(float x) { return x > -FLT_MAX ? x : -FLT_MAX; }

inline void atomic_insert(box& b, v3 p)
{
    b.lo = { vmin(b.lo.x, cas_lo(p.x)), vmin(b.lo.y, cas_lo(p.y)), vmin(b.lo.z, cas_lo(p.z)) };
    b.hi = { vmax(b.hi.x, cas_hi(p.x)), vmax(b.hi.y, cas_hi(p.y)), vmax(b.hi.z, cas_hi(p.z)) };
}

// assign_node_bounds (lbvh.h:332-372): an inner box is the atomic fold of the leaf boxes
// below it.
inline box atomic_combine(box const& a, box const& b)
{
    box r;
    r.lo = { vmin(cas_lo(a.lo.x), cas_lo(b.lo.x)), vmin(cas_lo(a.lo.y), cas_lo(b.lo.y)),
             vmin(cas_lo(a.lo.z), cas_lo(b.lo.z)) };
    r.hi = { vmax(cas_hi(a.hi.x), cas_hi(b.hi.x)), vmax(cas_hi(a.hi.y), cas_hi(b.hi.y)),
             vmax(cas_hi(a.hi.z), cas_hi(b.hi.z)) };
    return r;
}

inline float safe_half_surface_area(box const& b)
{
    v3 s = b.size();
    s.x = vmax(0.0f, s.x);
    s.y = vmax(0.0f, s.y);
    s.z = vmax(0.0f, s.z);
    return s.x * s.y + s.y * s.z + s.z * s.x;
}

inline float surface_area(box const& b)
{
    v3 s = b.size();
    return 2.0f * (s.x * s.y + s.y * s.z + s.z * s.x);
}

// get_bounds(basic_triangle) (math/detail/triangle.inl:43-52).
inline box tri_bounds(gbrt_triangle const& t)
{
    v3 v1 = load3(t.v1);
    box b;
    b.invalidate();
    b.insert(v1);
    b.insert(v1 + load3(t.e1));
    b.insert(v1 + load3(t.e2));
    return b;
}

// morton_encode3D(unsigned, unsigned, unsigned) (morton.h:33-46): bit i of x, y, z
// lands on bit 3i, 3i+1, 3i+2.  Written here as the plain bit loop.
inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t code = 0;
    for (int i = 0; i < 10; ++i)
    {
        code |= ((x >> i) & 1u) << (3 * i);
        code |= ((y >> i) & 1u) << (3 * i + 1);
        code |= ((z >> i) & 1u) << (3 * i + 2);
    }
    return code;
}

// Centroid quantisation of lbvh.h:253-267 (GPU) / :580-593 (CPU), op for op.
inline uint32_t quantise_centroid(v3 c, box const& cb)
{
    v3 cc = cb.center();
    v3 cs = cb.size();
    c = c - cc;
    c = (c + cs * 0.5f) / cs;
    c = c * 1024.0f;
    c = vmin3(vmax3(c, v3{ 0.0f, 0.0f, 0.0f }), v3{ 1023.0f, 1023.0f, 1023.0f });
    return morton3(static_cast<uint32_t>(c.x), static_cast<uint32_t>(c.y),
                   static_cast<uint32_t>(c.z));
}

inline int clz32(uint32_t v) { return v == 0 ? 32 : __builtin_clz(v); }

struct node
{
    box bbox;
    uint32_t first;   // first child or first index
    uint16_t count;   // primitives in a leaf, 0 for inner
    uint8_t axis;
    uint8_t sign;

    void set_inner(box const& b, uint32_t first_child, uint8_t ax, uint8_t sg)
    {
        bbox = b;
        first = first_child;
        count = 0;
        axis = ax;
        sign = sg;
    }
    void set_leaf(box const& b, uint32_t first_prim, uint32_t n)
    {
        bbox = b;
        first = first_prim;
        count = static_cast<uint16_t>(n);
    }
};

} // namespace

struct orc_bvh
{
    std::vector<node> nodes;
    std::vector<uint32_t> indices;
};

namespace {

//--------------------------------------------------------------------------------------
// Top-down build driver (detail/bvh/build_top_down.h:27-80, 149-173): the node is
// turned inner with its two children appended, the RIGHT subtree is built before the
// left one, and leaves append their primitive indices.

template <typename Builder>
void build_top_down(orc_bvh& tree, Builder& builder, typename Builder::leaf_info root,
                    int max_leaf_size)
{
    struct frame
    {
        int index;
        typename Builder::leaf_info leaf;
    };
    // Explicit stack keeps the visiting order of the recursion: right before left.
    std::vector<frame> work;
    tree.nodes.emplace_back();
    work.push_back({ 0, root });
    while (!work.empty())
    {
        frame f = work.back();
        work.pop_back();
        std::array<typename Builder::leaf_info, 2> childs;
        auto sr = builder.split(childs, f.leaf, max_leaf_size);
        if (sr.do_split)
        {
            int first_child = static_cast<int>(tree.nodes.size());
            tree.nodes[f.index].set_inner(builder.bounds_of(f.leaf), uint32_t(first_child),
                                          sr.axis, sr.sign);
            tree.nodes.emplace_back();
            tree.nodes.emplace_back();
            work.push_back({ first_child + 0, childs[0] });   // popped second
            work.push_back({ first_child + 1, childs[1] });   // popped first
        }
        else
        {
            uint32_t first = static_cast<uint32_t>(tree.indices.size());
            int count = builder.insert_indices(tree.indices, f.leaf);
            tree.nodes[f.index].set_leaf(builder.bounds_of(f.leaf), first, uint32_t(count));
        }
    }
}

//--------------------------------------------------------------------------------------
// binned_sah_builder, object splits (detail/bvh/sah.h:176-467, 676-807).

struct sah_builder
{
    static constexpr int kBins = 16;   // sah.h:226

    struct prim_ref
    {
        box bounds;
        int index;
    };
    struct leaf_info
    {
        box prim_bounds;
        box cent_bounds;
        int first;
    };
    struct bin
    {
        box prim_bounds, cent_bounds;
        int enter, leave;
        void clear()
        {
            prim_bounds.invalidate();
            cent_bounds.invalidate();
            enter = leave = 0;
        }
    };
    struct split_result
    {
        box prim_bounds[2];
        box cent_bounds[2];
        int count[2];
        float cost;
        int index;
    };
    struct split_record
    {
        bool do_split;
        uint8_t axis, sign;
    };
    struct projection
    {
        float k0, k1;
        int axis;
        projection(box const& b, int ax)
            : k0(b.lo[ax]), k1(float(kBins) / (b.hi[ax] - b.lo[ax])), axis(ax)
        {
        }
        int project_unsafe(v3 v) const { return static_cast<int>(k1 * (v[axis] - k0)); }
        int project(v3 v) const
        {
            int i = project_unsafe(v);
            if (i < 0) i = 0;
            if (i > kBins - 1) i = kBins - 1;
            return i;
        }
    };

    std::vector<prim_ref> refs;

    static bin merge(bin l, bin const& r)
    {
        l.prim_bounds.insert(r.prim_bounds);
        l.cent_bounds.insert(r.cent_bounds);
        l.enter += r.enter;
        l.leave += r.leave;
        return l;
    }

    // sah.h:315-328
    static float split_cost(box const& bl, int nl, box const& br, int nr, float hsa_parent)
    {
        float hl = safe_half_surface_area(bl);
        float hr = safe_half_surface_area(br);
        return 1.0f + (hl / hsa_parent) * (3.0f * float(nl)) + (hr / hsa_parent) * (3.0f * float(nr));
    }

    // sah.h:344-403: prefix/suffix sweep, strict '<' from the right.
    static split_result find_split(std::array<bin, kBins> const& bins, box const& bounds)
    {
        float hsa_parent = safe_half_surface_area(bounds);
        float best_cost = FLT_MAX;
        int best = -1;
        std::array<bin, kBins> acc_l, acc_r;
        acc_l[0] = bins[0];
        for (int i = 1; i < kBins; ++i) acc_l[i] = merge(acc_l[i - 1], bins[i]);
        acc_r[kBins - 1] = bins[kBins - 1];
        for (int i = kBins - 1; i > 0; --i)
        {
            acc_r[i - 1] = merge(acc_r[i], bins[i - 1]);
            bin const& L = acc_l[i - 1];
            bin const& R = acc_r[i];
            float cost = split_cost(L.prim_bounds, L.enter, R.prim_bounds, R.leave, hsa_parent);
            if (cost < best_cost)
            {
                best_cost = cost;
                best = i;
            }
        }
        split_result sr;
        if (best < 0)
        {
            // every candidate cost was NaN or FLT_MAX: report a cost above any leaf
            sr.cost = FLT_MAX;
            sr.index = 1;
            return sr;
        }
        bin const& L = acc_l[best - 1];
        bin const& R = acc_r[best];
        sr.prim_bounds[0] = L.prim_bounds;
        sr.prim_bounds[1] = R.prim_bounds;
        sr.cent_bounds[0] = L.cent_bounds;
        sr.cent_bounds[1] = R.cent_bounds;
        sr.count[0] = L.enter;
        sr.count[1] = R.leave;
        sr.cost = best_cost;
        sr.index = best;
        return sr;
    }

    leaf_info init(const gbrt_triangle* tris, uint32_t n)
    {
        refs.resize(n);
        box pb, cb;
        pb.invalidate();
        cb.invalidate();
        for (uint32_t i = 0; i < n; ++i)
        {
            refs[i].bounds = tri_bounds(tris[i]);
            refs[i].index = int(i);
            pb.insert(refs[i].bounds);
            cb.insert(refs[i].bounds.center());
        }
        return { pb, cb, 0 };
    }

    static box bounds_of(leaf_info const& l) { return l.prim_bounds; }

    int insert_indices(std::vector<uint32_t>& indices, leaf_info const& leaf)
    {
        int size = int(refs.size()) - leaf.first;
        for (int i = leaf.first; i != int(refs.size()); ++i)
        {
            indices.push_back(uint32_t(refs[i].index));
        }
        refs.resize(size_t(leaf.first));
        return size;
    }

    // sah.h:721-806 without spatial splits (use_spatial_splits defaults to false).
    split_record split(std::array<leaf_info, 2>& childs, leaf_info const& leaf, int max_leaf_size)
    {
        int leaf_size = int(refs.size()) - leaf.first;
        if (leaf_size <= max_leaf_size) return { false, 0, 0 };

        v3 size = leaf.cent_bounds.size();
        int axis = max_index(size);
        if (size[axis] <= 0.0f) return { false, 0, 0 };

        projection pr(leaf.cent_bounds, axis);

        std::array<bin, kBins> bins;
        for (auto& b : bins) b.clear();
        for (size_t i = size_t(leaf.first); i < refs.size(); ++i)
        {
            v3 cen = refs[i].bounds.center();
            bin& b = bins[size_t(pr.project(cen))];
            b.prim_bounds.insert(refs[i].bounds);
            b.cent_bounds.insert(cen);
            b.enter++;
            b.leave++;
        }
        split_result sr = find_split(bins, leaf.prim_bounds);

        if (sr.cost > 3.0f * float(leaf_size)) return { false, 0, 0 };

        childs[0].prim_bounds = sr.prim_bounds[0];
        childs[0].cent_bounds = sr.cent_bounds[0];
        childs[1].prim_bounds = sr.prim_bounds[1];
        childs[1].cent_bounds = sr.cent_bounds[1];
        // The partition order is std::partition's, as in sah.h:450-457.
        auto pivot = std::partition(refs.begin() + leaf.first, refs.end(), [&](prim_ref const& x) {
            return pr.project_unsafe(x.bounds.center()) < sr.index;
        });
        childs[0].first = leaf.first;
        childs[1].first = int(pivot - refs.begin());

        uint8_t sign = sr.prim_bounds[0].lo[axis] < sr.prim_bounds[1].lo[axis] ? 0 : 1;
        return { true, uint8_t(axis), sign };
    }
};

//--------------------------------------------------------------------------------------
// CPU lbvh_builder (detail/bvh/lbvh.h:473-656).

struct cpu_lbvh_builder
{
    struct prim_ref
    {
        int id;
        uint32_t code;
    };
    struct leaf_info
    {
        int first, last;
        box prim_bounds;
    };
    struct split_record
    {
        bool do_split;
        uint8_t axis, sign;
    };

    std::vector<prim_ref> refs;
    std::vector<box> prim_bounds;

    static box bounds_of(leaf_info const& l) { return l.prim_bounds; }

    // lbvh.h:499-532: binary search for the last index sharing the first key's
    // longer-than-common prefix.
    int find_split(int first, int last) const
    {
        uint32_t code_first = refs[size_t(first)].code;
        uint32_t code_last = refs[size_t(last - 1)].code;
        if (code_first == code_last) return (first + last) / 2;
        int common = clz32(code_first ^ code_last);
        int result = first;
        int step = last - first;
        do
        {
            step = (step + 1) / 2;
            int next = result + step;
            if (next < last)
            {
                uint32_t code = refs[size_t(next)].code;
                if (code_first == code || clz32(code_first ^ code) > common) result = next;
            }
        } while (step > 1);
        return result;
    }

    leaf_info init(const gbrt_triangle* tris, uint32_t n)
    {
        box scene, cb;
        scene.invalidate();
        cb.invalidate();
        prim_bounds.resize(n);
        std::vector<v3> centroids(n);
        for (uint32_t i = 0; i < n; ++i)
        {
            prim_bounds[i] = tri_bounds(tris[i]);
            scene.insert(prim_bounds[i]);
            centroids[i] = prim_bounds[i].center();
            cb.insert(centroids[i]);
        }
        refs.resize(n);
        for (uint32_t i = 0; i < n; ++i)
        {
            refs[i].id = int(i);
            refs[i].code = quantise_centroid(centroids[i], cb);
        }
        std::stable_sort(refs.begin(), refs.end(),
                         [](prim_ref const& a, prim_ref const& b) { return a.code < b.code; });
        return { 0, int(n), scene };
    }

    int insert_indices(std::vector<uint32_t>& indices, leaf_info const& leaf)
    {
        for (int i = leaf.first; i < leaf.last; ++i) indices.push_back(uint32_t(refs[size_t(i)].id));
        return leaf.last - leaf.first;
    }

    split_record split(std::array<leaf_info, 2>& childs, leaf_info const& leaf, int max_leaf_size)
    {
        if (leaf.last - leaf.first <= max_leaf_size) return { false, 0, 0 };
        int s = find_split(leaf.first, leaf.last);
        childs[0].first = leaf.first;
        childs[0].last = s + 1;
        childs[0].prim_bounds.invalidate();
        for (int i = childs[0].first; i != childs[0].last; ++i)
            childs[0].prim_bounds = combine(childs[0].prim_bounds, prim_bounds[size_t(refs[size_t(i)].id)]);
        childs[1].first = s + 1;
        childs[1].last = leaf.last;
        childs[1].prim_bounds.invalidate();
        for (int i = childs[1].first; i != childs[1].last; ++i)
            childs[1].prim_bounds = combine(childs[1].prim_bounds, prim_bounds[size_t(refs[size_t(i)].id)]);
        return { true, 0, 0 };
    }
};

//--------------------------------------------------------------------------------------
// Karras (2012) radix-tree split for inner node i (lbvh.h:120-185): the prefix length
// delta(i, j) is clz(code_i ^ code_j), or 32 + clz(i ^ j) for equal codes, and -1
// outside [0, n-1].  The range end is found by exponential then binary search, the
// split by binary search with step ceil(l / 2^k).

struct karras
{
    const uint32_t* codes;
    int n;

    int delta(int i, int j) const
    {
        if (j < 0 || j >= n) return -1;
        uint32_t x = codes[i] ^ codes[j];
        if (x == 0) return 32 + clz32(uint32_t(i) ^ uint32_t(j));
        return clz32(x);
    }

    // Returns [first, last] and the split position.
    void range(int i, int& first, int& last, int& split) const
    {
        int d = delta(i, i + 1) >= delta(i, i - 1) ? 1 : -1;
        int dmin = delta(i, i - d);
        int lmax = 2;
        while (delta(i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
        {
            if (delta(i, i + (l + t) * d) > dmin) l += t;
        }
        int j = i + l * d;
        int dnode = delta(i, j);
        int s = 0;
        int t = l;
        do
        {
            t = (t + 1) >> 1;
            if (delta(i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        split = i + s * d + (d < 0 ? d : 0);
        first = d == 1 ? i : j;
        last = d == 1 ? j : i;
    }
};

//--------------------------------------------------------------------------------------
// Ray / triangle (math/intersect.h:176-229) and ray / box (math/intersect.h:44-62).

struct hit_rec
{
    bool hit;
    uint32_t prim_id;
    float t, u, v;
};

inline hit_rec intersect_tri(gbrt_ray const& r, gbrt_triangle const& tri)
{
    hit_rec res{ false, 0, -1.0f, 0.0f, 0.0f };
    v3 ori = load3(r.ori), dir = load3(r.dir);
    v3 v1 = load3(tri.v1), e1 = load3(tri.e1), e2 = load3(tri.e2);
    v3 s1 = cross(dir, e2);
    float div = dot(s1, e1);
    if (!(div != 0.0f)) return res;
    float inv_div = 1.0f / div;
    v3 d = ori - v1;
    float b1 = dot(d, s1) * inv_div;
    if (!(b1 >= 0.0f && b1 <= 1.0f)) return res;
    v3 s2 = cross(d, e1);
    float b2 = dot(dir, s2) * inv_div;
    if (!(b2 >= 0.0f && b1 + b2 <= 1.0f)) return res;
    res.hit = true;
    res.prim_id = tri.prim_id;
    res.t = dot(e2, s2) * inv_div;
    res.u = b1;
    res.v = b2;
    return res;
}

struct box_rec
{
    bool hit;
    float tnear, tfar;
};

inline box_rec intersect_box(v3 ori, v3 inv_dir, box const& b)
{
    v3 t1 = (b.lo - ori) * inv_dir;
    v3 t2 = (b.hi - ori) * inv_dir;
    box_rec r;
    // min_max(a, b, c) = max(min(a, b), c); max_min(a, b, c) = min(max(a, b), c)
    r.tnear = vmax(vmin(t1.x, t2.x), vmax(vmin(t1.y, t2.y), vmin(t1.z, t2.z)));
    r.tfar = vmin(vmax(t1.x, t2.x), vmin(vmax(t1.y, t2.y), vmax(t1.z, t2.z)));
    r.hit = r.tfar >= r.tnear;
    return r;
}

inline v3 inverse_dir(v3 d)
{
    return { d.x != 0.0f ? 1.0f / d.x : FLT_MAX, d.y != 0.0f ? 1.0f / d.y : FLT_MAX,
             d.z != 0.0f ? 1.0f / d.z : FLT_MAX };
}

inline float dir_component(v3 d, int a) { return a == 0 ? d.x : (a == 1 ? d.y : d.z); }

// detail/bvh/intersect.inl:51-165 for a scalar ray (ordered traversal by the node's
// split axis and sign, full stack of 32 entries).  Returns false on stack overflow.
bool trace_one(gbrt_bvh_node const* nodes, const uint32_t* indices, gbrt_triangle const* tris,
               gbrt_ray const& r, bool any_hit, gbrt_hit& out, uint64_t& nbox, uint64_t& ntri)
{
    hit_rec best{ false, 0, FLT_MAX, 0.0f, 0.0f };
    v3 ori = load3(r.ori), dir = load3(r.dir);
    v3 inv = inverse_dir(dir);
    uint32_t st[32];
    int sp = 0;
    st[sp++] = 0;
    bool ok = true;
    while (sp > 0)
    {
        gbrt_bvh_node const* nd = &nodes[st[--sp]];
        bool reached_leaf = false;
        while (true)
        {
            box b{ load3(nd->bbox_min), load3(nd->bbox_max) };
            box_rec hr = intersect_box(ori, inv, b);
            ++nbox;
            // is_closer(box hit record, result, tmin, tmax) (update_if.h:76-107)
            bool hit = hr.hit && hr.tnear < best.t && hr.tfar >= r.tmin && hr.tnear <= r.tmax;
            if (!hit) break;
            if (nd->num_prims != 0)
            {
                reached_leaf = true;
                break;
            }
            int32_t sign = int32_t(nd->ordered_traversal_sign);
            uint32_t bits;
            float dc = dir_component(dir, nd->ordered_traversal_axis);
            std::memcpy(&bits, &dc, 4);
            int32_t sign_rd = int32_t(bits) >> 31;
            uint32_t near_addr = (sign ^ sign_rd) != 0 ? 1u : 0u;
            uint32_t far_addr = near_addr ? 0u : 1u;
            if (sp == 32)
            {
                ok = false;
                sp = 0;
                break;
            }
            st[sp++] = nd->first_child_or_prim + far_addr;
            nd = &nodes[nd->first_child_or_prim + near_addr];
        }
        if (!reached_leaf) continue;
        for (uint32_t i = nd->first_child_or_prim; i != nd->first_child_or_prim + nd->num_prims; ++i)
        {
            hit_rec h = intersect_tri(r, tris[indices[i]]);
            ++ntri;
            bool closer = h.hit && h.t < best.t && h.t >= r.tmin && h.t <= r.tmax;
            if (!closer) continue;
            best = h;
            if (any_hit)
            {
                sp = 0;
                break;
            }
        }
    }
    out.prim_id = best.hit ? best.prim_id : GBRT_NO_HIT;
    out.t = best.t;
    out.u = best.u;
    out.v = best.v;
    return ok;
}

template <typename F>
void parallel_chunks(uint64_t n, int nthreads, F&& body)
{
    if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
    const uint64_t chunk = 4096;
    std::atomic<uint64_t> next{ 0 };
    auto worker = [&](int tid) {
        for (;;)
        {
            uint64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            body(tid, b, std::min(n, b + chunk));
        }
    };
    if (nthreads == 1)
    {
        worker(0);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
}

uint32_t compute_depth(std::vector<node> const& nodes)
{
    if (nodes.empty()) return 0;
    uint32_t best = 0;
    std::vector<std::pair<uint32_t, uint32_t>> st{ { 0u, 1u } };
    while (!st.empty())
    {
        auto [i, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        if (nodes[i].count == 0)
        {
            st.push_back({ nodes[i].first, d + 1 });
            st.push_back({ nodes[i].first + 1, d + 1 });
        }
    }
    return best;
}

} // namespace

//--------------------------------------------------------------------------------------
// C ABI

extern "C" orc_bvh* orc_build_sah(const gbrt_triangle* tris, uint32_t n, int max_leaf_size)
{
    auto* tree = new orc_bvh;
    if (n == 0) return tree;
    if (max_leaf_size <= 0) max_leaf_size = 4;   // build_top_down.h:151-154
    sah_builder b;
    auto root = b.init(tris, n);
    build_top_down(*tree, b, root, max_leaf_size);
    return tree;
}

extern "C" orc_bvh* orc_build_lbvh_cpu(const gbrt_triangle* tris, uint32_t n, int max_leaf_size)
{
    if (max_leaf_size <= 0) max_leaf_size = 4;
    if (max_leaf_size < 2) return nullptr;
    auto* tree = new orc_bvh;
    if (n == 0) return tree;
    cpu_lbvh_builder b;
    auto root = b.init(tris, n);
    build_top_down(*tree, b, root, max_leaf_size);
    return tree;
}

extern "C" void orc_morton_codes(const gbrt_triangle* tris, uint32_t n, uint32_t* codes)
{
    std::vector<v3> cen(n);
    box cb;
    cb.invalidate();
    for (uint32_t i = 0; i < n; ++i)
    {
        cen[i] = tri_bounds(tris[i]).center();
        atomic_insert(cb, cen[i]);   // lbvh.h:233-238
    }
    for (uint32_t i = 0; i < n; ++i) codes[i] = quantise_centroid(cen[i], cb);
}

extern "C" void orc_karras_children(const uint32_t* codes, uint32_t n, int32_t* left, int32_t* right)
{
    karras k{ codes, int(n) };
    int num_inner = int(n) - 1;
    for (int i = 0; i < num_inner; ++i)
    {
        int first, last, split;
        k.range(i, first, last, split);
        left[i] = split == first ? num_inner + split : split;
        right[i] = split + 1 == last ? num_inner + split + 1 : split + 1;
    }
}

// lbvh.h:215-451 restated: the whole GPU builder's output in cuda_index_bvh layout.
extern "C" orc_bvh* orc_build_karras(const gbrt_triangle* tris, uint32_t n)
{
    auto* tree = new orc_bvh;
    if (n == 0) return tree;
    std::vector<box> pb(n);
    std::vector<v3> cen(n);
    box cb;
    cb.invalidate();
    for (uint32_t i = 0; i < n; ++i)
    {
        pb[i] = tri_bounds(tris[i]);
        cen[i] = pb[i].center();
        atomic_insert(cb, cen[i]);   // lbvh.h:233-238
    }
    struct ref
    {
        int id;
        uint32_t code;
    };
    std::vector<ref> refs(n);
    for (uint32_t i = 0; i < n; ++i) refs[i] = { int(i), quantise_centroid(cen[i], cb) };
    std::stable_sort(refs.begin(), refs.end(), [](ref const& a, ref const& b) { return a.code < b.code; });

    tree->nodes.assign(2 * size_t(n) - 1, node{});
    tree->indices.resize(n);
    for (uint32_t i = 0; i < n; ++i) tree->indices[i] = i;   // lbvh::sequence (lbvh.h:453-466)

    if (n == 1)
    {
        tree->nodes[0].set_leaf(pb[size_t(refs[0].id)], uint32_t(refs[0].id), 1);
        tree->nodes[0].axis = tree->nodes[0].sign = 0;
        return tree;
    }

    int num_inner = int(n) - 1;
    std::vector<uint32_t> codes(n);
    for (uint32_t i = 0; i < n; ++i) codes[i] = refs[i].code;
    std::vector<int32_t> left(static_cast<size_t>(num_inner)), right(static_cast<size_t>(num_inner));
    orc_karras_children(codes.data(), n, left.data(), right.data());

    // Bounds bottom-up: children always have a larger "first index" relation that is
    // not monotone, so compute by explicit post-order from the root.
    std::vector<box> inner_box(static_cast<size_t>(num_inner));
    auto child_box = [&](int c) -> box const& {
        return c >= num_inner ? pb[size_t(refs[size_t(c - num_inner)].id)] : inner_box[size_t(c)];
    };
    {
        std::vector<std::pair<int, bool>> st{ { 0, false } };
        while (!st.empty())
        {
            auto [i, expanded] = st.back();
            st.pop_back();
            if (expanded)
            {
                inner_box[size_t(i)] = atomic_combine(child_box(left[size_t(i)]), child_box(right[size_t(i)]));
                continue;
            }
            st.push_back({ i, true });
            if (right[size_t(i)] < num_inner) st.push_back({ right[size_t(i)], false });
            if (left[size_t(i)] < num_inner) st.push_back({ left[size_t(i)], false });
        }
    }

    // lbvh::collapse (lbvh.h:374-451): children of inner i at 1+2i (left), 2+2i (right).
    tree->nodes[0].set_inner(inner_box[0], 1, 0, 0);
    for (int i = 0; i < num_inner; ++i)
    {
        int ch[2] = { left[size_t(i)], right[size_t(i)] };
        for (int s = 0; s < 2; ++s)
        {
            node& dst = tree->nodes[size_t(1 + 2 * i + s)];
            int c = ch[s];
            if (c >= num_inner)
            {
                int leaf = c - num_inner;
                dst.set_leaf(pb[size_t(refs[size_t(leaf)].id)], uint32_t(refs[size_t(leaf)].id), 1);
                dst.axis = dst.sign = 0;
            }
            else
            {
                dst.set_inner(inner_box[size_t(c)], uint32_t(1 + 2 * c), 0, 0);
            }
        }
    }
    return tree;
}

extern "C" uint32_t orc_bvh_num_nodes(const orc_bvh* b) { return uint32_t(b->nodes.size()); }
extern "C" uint32_t orc_bvh_num_indices(const orc_bvh* b) { return uint32_t(b->indices.size()); }
extern "C" uint32_t orc_bvh_depth(const orc_bvh* b) { return compute_depth(b->nodes); }

extern "C" void orc_bvh_copy(const orc_bvh* b, gbrt_bvh_node* nodes, uint32_t* indices)
{
    for (size_t i = 0; i < b->nodes.size(); ++i)
    {
        node const& s = b->nodes[i];
        gbrt_bvh_node& d = nodes[i];
        d.bbox_min[0] = s.bbox.lo.x;
        d.bbox_min[1] = s.bbox.lo.y;
        d.bbox_min[2] = s.bbox.lo.z;
        d.bbox_max[0] = s.bbox.hi.x;
        d.bbox_max[1] = s.bbox.hi.y;
        d.bbox_max[2] = s.bbox.hi.z;
        d.first_child_or_prim = s.first;
        d.num_prims = s.count;
        d.ordered_traversal_axis = s.count == 0 ? s.axis : 0;
        d.ordered_traversal_sign = s.count == 0 ? s.sign : 0;
    }
    if (indices && !b->indices.empty())
        std::memcpy(indices, b->indices.data(), b->indices.size() * sizeof(uint32_t));
}

extern "C" void orc_bvh_free(orc_bvh* b) { delete b; }

extern "C" float orc_sah_cost(const gbrt_bvh_node* nodes, uint32_t num_nodes, float ci, float cl, float cp)
{
    if (num_nodes == 0) return 0.0f;
    auto boxof = [&](uint32_t i) { return box{ load3(nodes[i].bbox_min), load3(nodes[i].bbox_max) }; };
    float a_r = surface_area(boxof(0));
    float a_l = 0.0f, a_i = 0.0f, a_ln = 0.0f;
    for (uint32_t i = 0; i < num_nodes; ++i)
    {
        float sa = surface_area(boxof(i));
        if (nodes[i].num_prims != 0)
        {
            a_l += sa;
            a_ln += sa * float(nodes[i].num_prims);
        }
        else
        {
            a_i += sa;
        }
    }
    return ci * (a_i / a_r) + cl * (a_l / a_r) + cp * (a_ln / a_r);
}

// bvh_refitter::refit (detail/bvh/refit.h:25-117): every node's box becomes the union of
// its subtree's primitive bounds (the new positions), gathered depth first with child 0
// before child 1 as the reference's per-node walk does; topology, child / primitive
// links and traversal hints are kept.
extern "C" void orc_refit(const gbrt_bvh_node* nodes, uint32_t num_nodes, const uint32_t* indices,
                          const gbrt_triangle* tris, gbrt_bvh_node* out)
{
    for (uint32_t i = 0; i < num_nodes; ++i)
    {
        box b;
        b.invalidate();
        std::vector<uint32_t> stack{ i };
        while (!stack.empty())
        {
            uint32_t a = stack.back();
            stack.pop_back();
            gbrt_bvh_node const& nd = nodes[a];
            if (nd.num_prims == 0)
            {
                stack.push_back(nd.first_child_or_prim + 1);
                stack.push_back(nd.first_child_or_prim);
            }
            else
            {
                for (uint32_t j = nd.first_child_or_prim; j < nd.first_child_or_prim + nd.num_prims; ++j)
                    b.insert(tri_bounds(tris[indices[j]]));
            }
        }
        out[i] = nodes[i];
        out[i].bbox_min[0] = b.lo.x;
        out[i].bbox_min[1] = b.lo.y;
        out[i].bbox_min[2] = b.lo.z;
        out[i].bbox_max[0] = b.hi.x;
        out[i].bbox_max[1] = b.hi.y;
        out[i].bbox_max[2] = b.hi.z;
    }
}

namespace {

// The reference's float 3x3 inverse (math/detail/matrix3.inl:285-305, det2 math.h:
// 616-621): cofactors over the determinant, m[r][c].
void inverse3(const float m[3][3], float r[3][3])
{
    auto det2 = [](float m00, float m01, float m10, float m11) { return m00 * m11 - m10 * m01; };
    float a00 = det2(m[1][1], m[1][2], m[2][1], m[2][2]);
    float a01 = det2(m[1][0], m[1][2], m[2][0], m[2][2]);
    float a02 = det2(m[1][0], m[1][1], m[2][0], m[2][1]);
    float a10 = det2(m[0][1], m[0][2], m[2][1], m[2][2]);
    float a11 = det2(m[0][0], m[0][2], m[2][0], m[2][2]);
    float a12 = det2(m[0][0], m[0][1], m[2][0], m[2][1]);
    float a20 = det2(m[0][1], m[0][2], m[1][1], m[1][2]);
    float a21 = det2(m[0][0], m[0][2], m[1][0], m[1][2]);
    float a22 = det2(m[0][0], m[0][1], m[1][0], m[1][1]);
    float det = m[0][0] * a00 - m[0][1] * a01 + m[0][2] * a02;
    r[0][0] = +a00 / det; r[1][0] = -a01 / det; r[2][0] = +a02 / det;
    r[0][1] = -a10 / det; r[1][1] = +a11 / det; r[2][1] = -a12 / det;
    r[0][2] = +a20 / det; r[1][2] = -a21 / det; r[2][2] = +a22 / det;
}

} // namespace

extern "C" void orc_trace_instances(const orc_instance* instances, uint32_t num_instances, const gbrt_ray* rays,
                                    uint64_t nrays, int any_hit, int nthreads, gbrt_hit_inst* hits)
{
    // index_bvh_inst_t(ref, transform): affine_inv = inverse(top_left(transform)) with
    // top_left's row i = column i; trans_inv = -column 3 (bvh.h:694-700)
    std::vector<std::array<float, 12>> xf(num_instances);
    for (uint32_t k = 0; k < num_instances; ++k)
    {
        float tl[3][3], inv[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) tl[r][c] = instances[k].transform[3 * r + c];
        inverse3(tl, inv);
        for (int r = 0; r < 3; ++r)
        {
            for (int c = 0; c < 3; ++c) xf[k][size_t(4 * r + c)] = inv[r][c];
            xf[k][size_t(4 * r + 3)] = -instances[k].transform[9 + r];
        }
    }
    parallel_chunks(nrays, nthreads, [&](int, uint64_t b, uint64_t e) {
        uint64_t lb = 0, lt = 0;
        for (uint64_t i = b; i < e; ++i)
        {
            gbrt_hit_inst best{ GBRT_NO_HIT, GBRT_NO_HIT, FLT_MAX, 0.0f, 0.0f, 0u, { 0u, 0u } };
            gbrt_ray const& r = rays[i];
            for (uint32_t k = 0; k < num_instances; ++k)
            {
                if (instances[k].num_nodes == 0) continue;
                auto const& a = xf[k];
                // transform_ray (bvh.h:748-755): ori' = A (ori + trans_inv), dir' = A dir
                float p[3] = { r.ori[0] + a[3], r.ori[1] + a[7], r.ori[2] + a[11] };
                gbrt_ray t = r;
                for (int row = 0; row < 3; ++row)
                {
                    t.ori[row] = a[size_t(4 * row)] * p[0] + a[size_t(4 * row + 1)] * p[1] + a[size_t(4 * row + 2)] * p[2];
                    t.dir[row] = a[size_t(4 * row)] * r.dir[0] + a[size_t(4 * row + 1)] * r.dir[1] +
                                 a[size_t(4 * row + 2)] * r.dir[2];
                }
                gbrt_hit h;
                trace_one(instances[k].nodes, instances[k].indices, instances[k].tris, t, any_hit != 0, h, lb, lt);
                if (h.prim_id != GBRT_NO_HIT && h.t < best.t)
                {
                    best.prim_id = h.prim_id;
                    best.inst_id = k;
                    best.t = h.t;
                    best.u = h.u;
                    best.v = h.v;
                    if (any_hit) break;
                }
            }
            hits[i] = best;
        }
    });
}

extern "C" int orc_intersect_triangle(const gbrt_ray* ray, const gbrt_triangle* tri, gbrt_hit* out)
{
    hit_rec h = intersect_tri(*ray, *tri);
    if (out)
    {
        out->prim_id = h.hit ? h.prim_id : GBRT_NO_HIT;
        out->t = h.t;
        out->u = h.u;
        out->v = h.v;
    }
    return h.hit ? 1 : 0;
}

extern "C" int orc_intersect_box(const gbrt_ray* ray, const float bmin[3], const float bmax[3], float* tnear,
                                 float* tfar)
{
    box b{ load3(bmin), load3(bmax) };
    box_rec r = intersect_box(load3(ray->ori), inverse_dir(load3(ray->dir)), b);
    if (tnear) *tnear = r.tnear;
    if (tfar) *tfar = r.tfar;
    return r.hit ? 1 : 0;
}

extern "C" int orc_trace(const gbrt_bvh_node* nodes, uint32_t num_nodes, const uint32_t* indices,
                         const gbrt_triangle* tris, const gbrt_ray* rays, uint64_t nrays, int any_hit,
                         int nthreads, gbrt_hit* hits, uint64_t* counters)
{
    std::atomic<uint64_t> nbox{ 0 }, ntri{ 0 };
    std::atomic<int> overflow{ 0 };
    parallel_chunks(nrays, nthreads, [&](int, uint64_t b, uint64_t e) {
        uint64_t lb = 0, lt = 0;
        for (uint64_t i = b; i < e; ++i)
        {
            if (num_nodes == 0)
            {
                hits[i] = { GBRT_NO_HIT, FLT_MAX, 0.0f, 0.0f };
                continue;
            }
            if (!trace_one(nodes, indices, tris, rays[i], any_hit != 0, hits[i], lb, lt))
                overflow.store(1);
        }
        nbox += lb;
        ntri += lt;
    });
    if (counters)
    {
        counters[0] = nbox.load();
        counters[1] = ntri.load();
    }
    return overflow.load() ? -1 : 0;
}

extern "C" void orc_trace_linear(const gbrt_triangle* tris, uint32_t ntris, const gbrt_ray* rays,
                                 uint64_t nrays, int any_hit, int nthreads, gbrt_hit* hits)
{
    parallel_chunks(nrays, nthreads, [&](int, uint64_t b, uint64_t e) {
        for (uint64_t r = b; r < e; ++r)
        {
            hit_rec best{ false, 0, FLT_MAX, 0.0f, 0.0f };
            for (uint32_t i = 0; i < ntris; ++i)
            {
                hit_rec h = intersect_tri(rays[r], tris[i]);
                if (h.hit && h.t < best.t && h.t >= rays[r].tmin && h.t <= rays[r].tmax)
                {
                    best = h;
                    if (any_hit) break;
                }
            }
            hits[r] = { best.hit ? best.prim_id : GBRT_NO_HIT, best.t, best.u, best.v };
        }
    });
}
