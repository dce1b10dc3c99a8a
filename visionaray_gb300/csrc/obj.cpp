// Wavefront OBJ ingestion into the 44-byte triangle layout (host code, built into
// libgbrt_scenes.so), following the reference viewer's load_obj
// (src/common/obj_loader.cpp, whose boost::spirit grammar is obj_grammar.h):
//   * "v x y z [w]" appends a vertex (w ignored)
//   * "f" with index groups v, v/t, v//n or v/t/n: 1-based, negative indices count from
//     the end of the vertices read so far (remap_index, obj_loader.cpp:40-45); the
//     face is a triangle fan (f0, f[k-1], f[k]) (store_faces, :81-134)
//   * a triangle is v1 = p[i1], e1 = p[i2] - v1, e2 = p[i3] - v1, rejected when
//     length(cross(e1, e2)) == 0 (store_triangle, :51-76); prim_id counts the stored
//     triangles, geom_id is the index of the material last activated
//   * "mtllib a.mtl" reads material names ("newmtl") and Kd / Ke from the named files
//     (next to the OBJ); "usemtl name" with a known name activates a new material slot
//     (:380-470), an unknown name leaves the slot unchanged
// Everything else (vt, vn, g, o, s, comments) is skipped.  Arithmetic in float as the
// reference's vec3 (this file is compiled with -ffp-contract=off).

#include "scenes.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct mtl
{
    float kd[3] = { 0.8f, 0.8f, 0.8f };
    float ke[3] = { 0.0f, 0.0f, 0.0f };
};

struct obj_data
{
    std::vector<gbrt_triangle> tris;
    std::vector<mtl> slots;   // activated materials, in order
};

bool read_file(std::string const& path, std::string& text)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    text.resize(size > 0 ? size_t(size) : 0);
    size_t got = text.empty() ? 0 : std::fread(&text[0], 1, text.size(), f);
    std::fclose(f);
    text.resize(got);
    return true;
}

std::vector<std::string> split_lines(std::string const& text)
{
    std::vector<std::string> lines;
    size_t start = 0;
    for (size_t i = 0; i <= text.size(); ++i)
    {
        if (i == text.size() || text[i] == '\n')
        {
            std::string l = text.substr(start, i - start);
            if (!l.empty() && l.back() == '\r') l.pop_back();
            lines.push_back(l);
            start = i + 1;
        }
    }
    return lines;
}

std::vector<std::string> tokens(std::string const& line)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size())
    {
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
        if (i >= line.size() || line[i] == '#') break;
        size_t j = i;
        while (j < line.size() && line[j] != ' ' && line[j] != '\t') ++j;
        out.push_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

std::string dir_of(std::string const& path)
{
    size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

void read_mtllib(std::string const& path, std::map<std::string, mtl>& lib)
{
    std::string text;
    if (!read_file(path, text)) return;
    mtl* cur = nullptr;
    for (auto const& line : split_lines(text))
    {
        auto t = tokens(line);
        if (t.empty()) continue;
        if (t[0] == "newmtl" && t.size() >= 2)
        {
            cur = &lib[t[1]];
            *cur = mtl{};
        }
        else if (cur && (t[0] == "Kd" || t[0] == "Ke") && t.size() >= 4)
        {
            float* dst = t[0] == "Kd" ? cur->kd : cur->ke;
            for (int a = 0; a < 3; ++a) dst[a] = std::strtof(t[1 + a].c_str(), nullptr);
        }
    }
}

bool load(std::string const& path, obj_data& out)
{
    std::string text;
    if (!read_file(path, text)) return false;
    std::map<std::string, mtl> lib;
    std::vector<float> v;   // xyz per vertex
    uint32_t geom_id = 0;
    for (auto const& line : split_lines(text))
    {
        auto t = tokens(line);
        if (t.empty()) continue;
        if (t[0] == "v" && t.size() >= 4)
        {
            for (int a = 0; a < 3; ++a) v.push_back(std::strtof(t[1 + a].c_str(), nullptr));
        }
        else if (t[0] == "mtllib")
        {
            for (size_t k = 1; k < t.size(); ++k) read_mtllib(dir_of(path) + t[k], lib);
        }
        else if (t[0] == "usemtl" && t.size() >= 2)
        {
            auto it = lib.find(t[1]);
            if (it != lib.end())
            {
                out.slots.push_back(it->second);
                geom_id = uint32_t(out.slots.size() - 1);
            }
        }
        else if (t[0] == "f" && t.size() >= 4)
        {
            const long nv = long(v.size() / 3);
            std::vector<long> idx;
            bool ok = true;
            for (size_t k = 1; k < t.size(); ++k)
            {
                long i = std::strtol(t[k].c_str(), nullptr, 10);   // the vertex index before any '/'
                long r = i < 0 ? nv + i : i - 1;                    // remap_index
                if (i == 0 || r < 0 || r >= nv) ok = false;
                idx.push_back(r);
            }
            if (!ok) continue;   // an index outside the vertices read so far
            for (size_t last = 2; last < idx.size(); ++last)
            {
                const float* p1 = &v[size_t(3 * idx[0])];
                const float* p2 = &v[size_t(3 * idx[last - 1])];
                const float* p3 = &v[size_t(3 * idx[last])];
                gbrt_triangle tri;
                for (int a = 0; a < 3; ++a)
                {
                    tri.v1[a] = p1[a];
                    tri.e1[a] = p2[a] - p1[a];
                    tri.e2[a] = p3[a] - p1[a];
                }
                float cx = tri.e1[1] * tri.e2[2] - tri.e1[2] * tri.e2[1];
                float cy = tri.e1[2] * tri.e2[0] - tri.e1[0] * tri.e2[2];
                float cz = tri.e1[0] * tri.e2[1] - tri.e1[1] * tri.e2[0];
                if (std::sqrt(cx * cx + cy * cy + cz * cz) == 0.0f) continue;   // degenerate
                tri.prim_id = uint32_t(out.tris.size());
                tri.geom_id = geom_id;
                out.tris.push_back(tri);
            }
        }
    }
    return true;
}

} // namespace

extern "C" int64_t gbrt_obj_load(const char* path, gbrt_triangle* out, uint64_t capacity)
{
    if (!path) return -1;
    obj_data d;
    if (!load(path, d)) return -1;
    if (out)
    {
        uint64_t n = d.tris.size() < capacity ? d.tris.size() : capacity;
        if (n) std::memcpy(out, d.tris.data(), n * sizeof(gbrt_triangle));
    }
    return int64_t(d.tris.size());
}

extern "C" int64_t gbrt_obj_materials(const char* path, gbrt_material* out, uint64_t capacity)
{
    if (!path) return -1;
    obj_data d;
    if (!load(path, d)) return -1;
    size_t slots = d.slots.empty() ? 1 : d.slots.size();   // one default slot (geom_id 0)
    if (out)
    {
        for (size_t k = 0; k < slots && k < capacity; ++k)
        {
            mtl m = d.slots.empty() ? mtl{} : d.slots[k];
            out[k] = gbrt_material{};
            bool emits = m.ke[0] > 0.0f || m.ke[1] > 0.0f || m.ke[2] > 0.0f;
            out[k].kind = emits ? GBRT_MATERIAL_EMISSIVE : GBRT_MATERIAL_MATTE;
            for (int a = 0; a < 3; ++a) out[k].color[a] = emits ? m.ke[a] : m.kd[a];
            out[k].scale = 1.0f;
        }
    }
    return int64_t(slots);
}
