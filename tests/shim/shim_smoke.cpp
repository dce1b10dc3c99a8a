// Compiles the header-only C++ shim as a visionaray caller would include it, links it
// against libgbrt.so, and runs it: without a CUDA device the context constructor throws
// visionaray_gb300::error (exit 0, "no-device"); with one, a two-triangle upload, host-
// buffer closest_hit and a status check run end to end ("ok").
#include <visionaray_gb300/visionaray_gb300.hpp>

#include <cstdio>
#include <vector>

namespace vg = visionaray_gb300;

int main()
{
    try
    {
        vg::context ctx(0, nullptr);
        // two triangles facing -z at z = 1, a single-leaf index_bvh over both
        std::vector<gbrt_triangle> tris(2);
        for (uint32_t i = 0; i < 2; ++i)
        {
            tris[i] = gbrt_triangle{ 0u, i, { float(i), 0.0f, 1.0f }, { 1.0f, 0.0f, 0.0f }, { 0.0f, 1.0f, 0.0f } };
        }
        std::vector<gbrt_bvh_node> nodes(1);
        nodes[0] = gbrt_bvh_node{ { 0.0f, 0.0f, 1.0f }, { 2.0f, 1.0f, 1.0f }, 0u, 2u, 0u, 0u };
        std::vector<uint32_t> indices{ 0u, 1u };
        vg::cuda_index_bvh bvh = vg::cuda_index_bvh::upload(ctx, nodes, indices, tris.data(), tris.size());
        gbrt_ray ray{ { 1.25f, 0.25f, 0.0f }, { 0.0f, 0.0f, 1.0f }, 0.0f, 1e30f };
        gbrt_hit hit{};
        vg::check(gbrt_trace_closest_hit_host(ctx.get(), bvh.get(), &ray, 1, &hit), ctx.get(), "trace");
        ctx.synchronize();
        if (hit.prim_id != 1u || hit.t != 1.0f)
        {
            std::printf("wrong hit %u %g\n", hit.prim_id, double(hit.t));
            return 1;
        }
        std::printf("ok\n");
    }
    catch (vg::error const& e)
    {
        if (e.status == GBRT_ERR_INVALID_ARG)
        {
            std::printf("no-device\n");
            return 0;
        }
        std::printf("error %d: %s\n", int(e.status), e.what());
        return 1;
    }
    return 0;
}
