// Compiles the header-only C++ shim as a visionaray caller would include it, links it
// against libgbrt.so, and runs it: without a CUDA device the context constructor throws
// visionaray_gb300::error (exit 0, "no-device"); with one, a two-triangle upload, host-
// buffer closest_hit and a status check run end to end, then LBVH and PLOC builds of a
// small lit scene and one path-traced frame through make_kernel_params /
// pathtracing::kernel / cuda_sched::frame ("ok").
#include <visionaray_gb300/visionaray_gb300.hpp>

#include <cuda_runtime_api.h>

#include <cmath>
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
        // a floor quad (matte) under a light triangle (emissive, also the area light)
        std::vector<gbrt_triangle> scene(3);
        scene[0] = gbrt_triangle{ 0u, 0u, { 0.0f, 0.0f, 0.0f }, { 1.0f, 0.0f, 0.0f }, { 0.0f, 0.0f, 1.0f } };
        scene[1] = gbrt_triangle{ 0u, 1u, { 1.0f, 0.0f, 1.0f }, { -1.0f, 0.0f, 0.0f }, { 0.0f, 0.0f, -1.0f } };
        scene[2] = gbrt_triangle{ 1u, 2u, { 0.3f, 0.9f, 0.3f }, { 0.4f, 0.0f, 0.0f }, { 0.0f, 0.0f, 0.4f } };
        gbrt_triangle* d_tris = nullptr;
        if (cudaMalloc(reinterpret_cast<void**>(&d_tris), scene.size() * sizeof(gbrt_triangle)) != cudaSuccess ||
            cudaMemcpy(d_tris, scene.data(), scene.size() * sizeof(gbrt_triangle), cudaMemcpyHostToDevice) !=
                cudaSuccess)
        {
            std::printf("cuda alloc failed\n");
            return 1;
        }
        vg::cuda_index_bvh lbvh = vg::lbvh_builder(ctx).build(vg::cuda_index_bvh{}, d_tris, scene.size());
        vg::cuda_index_bvh ploc = vg::ploc_builder(ctx).build(vg::cuda_index_bvh{}, d_tris, scene.size());
        gbrt_ray down{ { 0.5f, 2.0f, 0.5f }, { 0.0f, -1.0f, 0.0f }, 0.0f, 1e30f };
        gbrt_hit h1{}, h2{};
        vg::check(gbrt_trace_closest_hit_host(ctx.get(), lbvh.get(), &down, 1, &h1), ctx.get(), "trace lbvh");
        vg::check(gbrt_trace_closest_hit_host(ctx.get(), ploc.get(), &down, 1, &h2), ctx.get(), "trace ploc");
        if (h1.prim_id != 2u || h2.prim_id != 2u || h1.t != h2.t)
        {
            std::printf("wrong builder hits %u %u\n", h1.prim_id, h2.prim_id);
            return 1;
        }
        std::vector<gbrt_material> mats(2);
        mats[0] = gbrt_material{};
        mats[0].kind = GBRT_MATERIAL_MATTE;
        mats[0].color[0] = mats[0].color[1] = mats[0].color[2] = 0.5f;
        mats[0].scale = 1.0f;
        mats[1] = gbrt_material{};
        mats[1].kind = GBRT_MATERIAL_EMISSIVE;
        mats[1].color[0] = mats[1].color[1] = mats[1].color[2] = 4.0f;
        mats[1].scale = 1.0f;
        std::vector<gbrt_area_light> lights(1);
        lights[0].geometry = scene[2];
        lights[0].cl[0] = lights[0].cl[1] = lights[0].cl[2] = 4.0f;
        lights[0].kl = 1.0f;
        vg::kernel_params kp = vg::make_kernel_params(ctx, lbvh, mats, lights, 4u, 1e-4f, { 0.0f, 0.0f, 0.0f, 1.0f },
                                                      { 0.0f, 0.0f, 0.0f });
        vg::pathtracing::kernel<vg::kernel_params> k;
        k.params = &kp;
        const uint32_t w = 16, hgt = 16;
        float* d_accum = nullptr;
        if (cudaMalloc(reinterpret_cast<void**>(&d_accum), size_t(w) * hgt * 16) != cudaSuccess)
        {
            std::printf("cuda alloc failed\n");
            return 1;
        }
        vg::sched_params sp;
        sp.camera = gbrt_camera{ { 0.5f, 0.6f, -1.0f }, { 0.5f, 0.2f, 0.5f }, { 0.0f, 1.0f, 0.0f }, 45.0f };
        sp.width = w;
        sp.height = hgt;
        sp.spp = 4;
        sp.d_accum = d_accum;
        vg::cuda_sched(ctx).frame(k, sp);
        // a second frame under a 2x1 environment light, blended in
        std::vector<float> texels = { 0.2f, 0.4f, 0.8f, 1.0f, 0.9f, 0.7f, 0.3f, 1.0f };
        float* d_texels = nullptr;
        if (cudaMalloc(reinterpret_cast<void**>(&d_texels), texels.size() * sizeof(float)) != cudaSuccess)
        {
            std::printf("cuda alloc failed\n");
            return 1;
        }
        cudaMemcpy(d_texels, texels.data(), texels.size() * sizeof(float), cudaMemcpyHostToDevice);
        vg::environment_light env;
        env.d_texels = d_texels;
        env.width = 2;
        env.height = 1;
        env.address = GBRT_ADDRESS_WRAP;
        kp.set_environment(env);
        sp.sfactor = 0.5f;
        sp.dfactor = 0.5f;
        vg::cuda_sched(ctx).frame(k, sp);
        ctx.synchronize();
        cudaFree(d_texels);
        std::vector<float> img(size_t(w) * hgt * 4);
        cudaMemcpy(img.data(), d_accum, img.size() * sizeof(float), cudaMemcpyDeviceToHost);
        double sum = 0.0;   // of the color channels (alpha is 1 wherever a ray hit)
        for (size_t i = 0; i < img.size(); ++i)
        {
            if (!std::isfinite(img[i]))
            {
                std::printf("non-finite pixel\n");
                return 1;
            }
            if (i % 4 != 3) sum += img[i];
        }
        cudaFree(d_accum);
        cudaFree(d_tris);
        if (!(sum > 0.0))
        {
            std::printf("black frame\n");
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
