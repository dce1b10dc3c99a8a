// Stanford PLY ingestion into the 44-byte triangle layout (host code, built into
// libgbrt_scenes.so), following the reference viewer's load_ply
// (src/common/ply_loader.cpp, which reads the file with tinyply):
//   * the "vertex" element's x, y, z properties are the positions (the reference
//     requires float32; float64 is accepted here and rounded to float)
//   * the "face" element's "vertex_indices" list gives the triangles: v1 = p[i0],
//     e1 = p[i1] - v1, e2 = p[i2] - v1 with no degenerate-face test (ply_loader.cpp:
//     118-140); prim_id counts the triangles, geom_id is 0 (one material per file)
//   * the reference assumes three indices per face; a face with more is split into
//     the fan (f0, f[k-1], f[k]) here, and one with fewer, or an index outside the
//     vertex list, is an error rather than an out-of-bounds read
//   * ascii, binary_little_endian and binary_big_endian bodies, any index type
//     (int8 .. uint32), other elements and properties skipped by their declared sizes
// Arithmetic in float as the reference's vec3 (compiled with -ffp-contract=off).

#include "scenes.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

enum class ptype
{
    i8, u8, i16, u16, i32, u32, f32, f64, none
};

ptype parse_type(std::string const& t)
{
    if (t == "char" || t == "int8") return ptype::i8;
    if (t == "uchar" || t == "uint8") return ptype::u8;
    if (t == "short" || t == "int16") return ptype::i16;
    if (t == "ushort" || t == "uint16") return ptype::u16;
    if (t == "int" || t == "int32") return ptype::i32;
    if (t == "uint" || t == "uint32") return ptype::u32;
    if (t == "float" || t == "float32") return ptype::f32;
    if (t == "double" || t == "float64") return ptype::f64;
    return ptype::none;
}

size_t type_size(ptype t)
{
    switch (t)
    {
    case ptype::i8:
    case ptype::u8: return 1;
    case ptype::i16:
    case ptype::u16: return 2;
    case ptype::i32:
    case ptype::u32:
    case ptype::f32: return 4;
    case ptype::f64: return 8;
    default: return 0;
    }
}

struct property
{
    std::string name;
    bool list = false;
    ptype count_type = ptype::none;   // list: type of the length
    ptype type = ptype::none;         // scalar type, or list item type
};

struct element
{
    std::string name;
    uint64_t count = 0;
    std::vector<property> props;
};

enum class format
{
    ascii, binary_le, binary_be
};

// A cursor over the body: values in declaration order, ascii tokens or binary fields.
struct reader
{
    const unsigned char* p;
    const unsigned char* end;
    format fmt;
    bool ok = true;

    bool token(std::string& out)
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
        const unsigned char* s = p;
        while (p < end && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
        out.assign(reinterpret_cast<const char*>(s), size_t(p - s));
        return !out.empty();
    }

    // Reads one value of type t as a double (integers are exact in a double).
    double value(ptype t)
    {
        if (fmt == format::ascii)
        {
            std::string tok;
            if (!token(tok))
            {
                ok = false;
                return 0.0;
            }
            char* e = nullptr;
            double v = (t == ptype::f32 || t == ptype::f64) ? std::strtod(tok.c_str(), &e)
                                                              : double(std::strtoll(tok.c_str(), &e, 10));
            if (!e || *e != '\0') ok = false;
            return v;
        }
        const size_t n = type_size(t);
        if (n == 0 || size_t(end - p) < n)
        {
            ok = false;
            return 0.0;
        }
        unsigned char b[8];
        for (size_t k = 0; k < n; ++k) b[k] = fmt == format::binary_le ? p[k] : p[n - 1 - k];
        p += n;
        // b now holds the value little-endian; assemble it independently of the host
        uint64_t u = 0;
        for (size_t k = 0; k < n; ++k) u |= uint64_t(b[k]) << (8 * k);
        switch (t)
        {
        case ptype::i8: return double(int8_t(uint8_t(u)));
        case ptype::u8: return double(uint8_t(u));
        case ptype::i16: return double(int16_t(uint16_t(u)));
        case ptype::u16: return double(uint16_t(u));
        case ptype::i32: return double(int32_t(uint32_t(u)));
        case ptype::u32: return double(uint32_t(u));
        case ptype::f32:
        {
            uint32_t w = uint32_t(u);
            float f;
            std::memcpy(&f, &w, 4);
            return double(f);
        }
        case ptype::f64:
        {
            double d;
            std::memcpy(&d, &u, 8);
            return d;
        }
        default: ok = false; return 0.0;
        }
    }
};

bool read_file(std::string const& path, std::vector<unsigned char>& data)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    data.resize(size > 0 ? size_t(size) : 0);
    size_t got = data.empty() ? 0 : std::fread(data.data(), 1, data.size(), f);
    std::fclose(f);
    data.resize(got);
    return true;
}

std::vector<std::string> words(std::string const& line)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size())
    {
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
        size_t j = i;
        while (j < line.size() && !(line[j] == ' ' || line[j] == '\t' || line[j] == '\r')) ++j;
        if (j > i) out.push_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

// Parses the file into triangles; false when it is unreadable or malformed.
bool load(std::string const& path, std::vector<gbrt_triangle>& tris)
{
    std::vector<unsigned char> data;
    if (!read_file(path, data)) return false;
    // header: lines up to "end_header"
    size_t pos = 0;
    auto next_line = [&](std::string& line) {
        if (pos >= data.size()) return false;
        size_t e = pos;
        while (e < data.size() && data[e] != '\n') ++e;
        line.assign(reinterpret_cast<const char*>(data.data()) + pos, e - pos);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        pos = e < data.size() ? e + 1 : e;
        return true;
    };
    std::string line;
    if (!next_line(line) || line != "ply") return false;
    format fmt = format::ascii;
    bool have_format = false, ended = false;
    std::vector<element> elements;
    while (next_line(line))
    {
        auto w = words(line);
        if (w.empty()) continue;
        if (w[0] == "end_header")
        {
            ended = true;
            break;
        }
        if (w[0] == "comment" || w[0] == "obj_info") continue;
        if (w[0] == "format" && w.size() >= 2)
        {
            if (w[1] == "ascii") fmt = format::ascii;
            else if (w[1] == "binary_little_endian") fmt = format::binary_le;
            else if (w[1] == "binary_big_endian") fmt = format::binary_be;
            else return false;
            have_format = true;
        }
        else if (w[0] == "element" && w.size() >= 3)
        {
            element el;
            el.name = w[1];
            char* e = nullptr;
            el.count = std::strtoull(w[2].c_str(), &e, 10);
            if (!e || *e != '\0') return false;
            elements.push_back(el);
        }
        else if (w[0] == "property" && !elements.empty())
        {
            property pr;
            if (w.size() >= 5 && w[1] == "list")
            {
                pr.list = true;
                pr.count_type = parse_type(w[2]);
                pr.type = parse_type(w[3]);
                pr.name = w[4];
                if (pr.count_type == ptype::none || pr.count_type == ptype::f32 || pr.count_type == ptype::f64)
                    return false;
            }
            else if (w.size() >= 3)
            {
                pr.type = parse_type(w[1]);
                pr.name = w[2];
            }
            else
            {
                return false;
            }
            if (pr.type == ptype::none) return false;
            elements.back().props.push_back(pr);
        }
        else
        {
            return false;
        }
    }
    if (!ended || !have_format) return false;

    reader rd{ data.data() + pos, data.data() + data.size(), fmt };
    std::vector<float> verts;   // xyz per vertex
    bool have_vertices = false;
    std::vector<uint32_t> face;
    for (element const& el : elements)
    {
        const bool is_vertex = el.name == "vertex", is_face = el.name == "face";
        int ix = -1, iy = -1, iz = -1, iidx = -1;
        for (size_t k = 0; k < el.props.size(); ++k)
        {
            property const& pr = el.props[k];
            if (is_vertex && !pr.list)
            {
                if (pr.name == "x") ix = int(k);
                if (pr.name == "y") iy = int(k);
                if (pr.name == "z") iz = int(k);
            }
            if (is_face && pr.list && pr.name == "vertex_indices") iidx = int(k);
        }
        if (el.count > uint64_t(data.size())) return false;   // every element takes at least a byte
        if (is_vertex)
        {
            if (ix < 0 || iy < 0 || iz < 0) return false;
            verts.assign(size_t(el.count) * 3, 0.0f);
            have_vertices = true;
        }
        if (is_face && (iidx < 0 || !have_vertices)) return false;
        for (uint64_t i = 0; i < el.count; ++i)
        {
            for (size_t k = 0; k < el.props.size(); ++k)
            {
                property const& pr = el.props[k];
                if (!pr.list)
                {
                    double v = rd.value(pr.type);
                    if (is_vertex && int(k) == ix) verts[size_t(3 * i + 0)] = float(v);
                    if (is_vertex && int(k) == iy) verts[size_t(3 * i + 1)] = float(v);
                    if (is_vertex && int(k) == iz) verts[size_t(3 * i + 2)] = float(v);
                    continue;
                }
                double len = rd.value(pr.count_type);
                if (!rd.ok || len < 0.0 || len > 1e6) return false;
                const size_t m = size_t(len);
                if (is_face && int(k) == iidx)
                {
                    face.resize(m);
                    for (size_t j = 0; j < m; ++j)
                    {
                        double v = rd.value(pr.type);
                        if (v < 0.0 || v >= double(verts.size() / 3)) return false;   // outside the vertex list
                        face[j] = uint32_t(v);
                    }
                    if (m < 3) return false;
                    for (size_t last = 2; last < m; ++last)
                    {
                        const float* p1 = &verts[size_t(3) * face[0]];
                        const float* p2 = &verts[size_t(3) * face[last - 1]];
                        const float* p3 = &verts[size_t(3) * face[last]];
                        gbrt_triangle t;
                        for (int a = 0; a < 3; ++a)
                        {
                            t.v1[a] = p1[a];
                            t.e1[a] = p2[a] - p1[a];
                            t.e2[a] = p3[a] - p1[a];
                        }
                        t.prim_id = uint32_t(tris.size());
                        t.geom_id = 0;
                        tris.push_back(t);
                    }
                }
                else
                {
                    for (size_t j = 0; j < m; ++j) rd.value(pr.type);
                }
            }
            if (!rd.ok) return false;
        }
    }
    return true;
}

} // namespace

extern "C" int64_t gbrt_ply_load(const char* path, gbrt_triangle* out, uint64_t capacity)
{
    if (!path) return -1;
    std::vector<gbrt_triangle> tris;
    if (!load(path, tris)) return -1;
    if (out)
    {
        uint64_t n = tris.size() < capacity ? tris.size() : capacity;
        if (n) std::memcpy(out, tris.data(), n * sizeof(gbrt_triangle));
    }
    return int64_t(tris.size());
}
