// kf_obj.cpp — Wavefront OBJ / MTL loading with the geometry and material mapping of
// kuafu's loadScene (src/core/geometry.cpp:46-237), which reads files through assimp with
// aiProcess_Triangulate | GenNormals | FlipUVs | PreTransformVertices:
//   * every face corner is its own vertex (no vertex sharing between faces); polygons are
//     split into the fan (c0, ci, ci+1); V texture coordinates are flipped (1 - v);
//   * a material group without normals gets flat face normals;
//   * faces are merged per material: one geometry per material used, in the order the
//     materials were first used;
//   * MTL keys: Kd → diffuse, Ke → emission, Ni → ior, d → alpha (Tr → 1 - alpha), Ns →
//     shininess; metallic, specular, transmission and emission strength keep kuafu's
//     defaults (0, 0.5, 0, 1); roughness from shininess (geometry.cpp:110-126):
//     Ns <= 5 → 1, else 1 - sqrt(Ns - 5) * 0.025 (at least 0.001), no Ns → 1;
//   * defaults of a material the file does not define (assimp's OBJ material):
//     diffuse 0.6, alpha 1, ior 1, shininess 0.
// Texture maps (map_Kd ...) are not decoded (no image decoder in this build): register
// textures with kf_texture_create and reference them from the material instead.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "kf_obj.h"
#include "kf_util.h"

namespace kf {
namespace {

struct MtlDef {
    float kd[3] = {0.6f, 0.6f, 0.6f};
    float ke[3] = {0.0f, 0.0f, 0.0f};
    float alpha = 1.0f;
    float ior = 1.0f;
    float shininess = 0.0f;
};

kf_material to_material(const MtlDef& d) {
    kf_material m{};
    for (int k = 0; k < 3; ++k) {
        m.diffuse_color[k] = d.kd[k];
        m.emission[k] = d.ke[k];
    }
    m.alpha = d.alpha;
    m.metallic = 0.0f;
    m.specular = 0.5f;
    m.ior = d.ior;
    m.transmission = 0.0f;
    m.emission_strength = 1.0f;
    // roughness is not an OBJ key: derived from the shininess (geometry.cpp:110-126)
    float roughness = 0.0f;
    if (d.shininess > 0.0f) {
        roughness = d.shininess <= 5.0f ? 1.0f : 1.0f - std::sqrt(d.shininess - 5.0f) * 0.025f;
        if (roughness < 0.001f) roughness = 0.001f;
    } else {
        roughness = 1.0f;
    }
    m.roughness = roughness;
    m.diffuse_tex = m.metallic_tex = m.roughness_tex = m.transmission_tex = -1;
    return m;
}

std::string dir_of(const std::string& p) {
    const size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string() : p.substr(0, s + 1);
}

void parse_mtl(const std::string& path, std::map<std::string, MtlDef>& out) {
    std::ifstream f(path);
    if (!f) return; // a missing library leaves its materials at the defaults, as assimp does
    std::string line, cur;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "newmtl") {
            ss >> cur;
            out[cur] = MtlDef{};
            continue;
        }
        if (cur.empty()) continue;
        MtlDef& d = out[cur];
        if (key == "Kd") ss >> d.kd[0] >> d.kd[1] >> d.kd[2];
        else if (key == "Ke") ss >> d.ke[0] >> d.ke[1] >> d.ke[2];
        else if (key == "Ni") ss >> d.ior;
        else if (key == "Ns") ss >> d.shininess;
        else if (key == "d") ss >> d.alpha;
        else if (key == "Tr") {
            float tr = 0.0f;
            ss >> tr;
            d.alpha = 1.0f - tr;
        }
    }
}

// OBJ index (1-based, or negative = relative to the end) -> 0-based, -1 if absent / invalid
long obj_index(const std::string& s, size_t count) {
    if (s.empty()) return -1;
    char* end = nullptr;
    const long v = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || v == 0) return -1;
    const long i = v > 0 ? v - 1 : (long)count + v;
    return (i >= 0 && (size_t)i < count) ? i : -2;
}

struct Group {
    std::string material;
    std::vector<kf_vertex> v;
    std::vector<uint32_t> idx;
    bool has_normals = false;
};

} // namespace

void load_obj(const std::string& path, std::vector<ObjMesh>& out) {
    out.clear();
    std::ifstream f(path);
    KF_REQUIRE(f.good(), KF_ERR_INVALID_ARGUMENT, "Failed to load scene: cannot open " + path);
    std::vector<float> pos, nrm, uv, col;
    std::map<std::string, MtlDef> mtls;
    std::vector<Group> groups;
    std::map<std::string, size_t> group_of;
    std::string cur_mtl; // "" = assimp's default material
    auto group = [&](const std::string& m) -> Group& {
        auto it = group_of.find(m);
        if (it != group_of.end()) return groups[it->second];
        group_of[m] = groups.size();
        groups.push_back(Group{m, {}, {}, false});
        return groups.back();
    };
    std::string line;
    size_t lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "v") {
            float x = 0, y = 0, z = 0;
            ss >> x >> y >> z;
            pos.insert(pos.end(), {x, y, z});
            float r, g, b;
            if (ss >> r >> g >> b)
                col.insert(col.end(), {r, g, b});
            else
                col.insert(col.end(), {0.0f, 0.0f, 0.0f});
        } else if (key == "vn") {
            float x = 0, y = 0, z = 0;
            ss >> x >> y >> z;
            nrm.insert(nrm.end(), {x, y, z});
        } else if (key == "vt") {
            float u = 0, v = 0;
            ss >> u >> v;
            uv.insert(uv.end(), {u, 1.0f - v}); // aiProcess_FlipUVs
        } else if (key == "mtllib") {
            std::string name;
            std::getline(ss >> std::ws, name);
            parse_mtl(dir_of(path) + name, mtls);
        } else if (key == "usemtl") {
            ss >> cur_mtl;
        } else if (key == "f") {
            Group& g = group(cur_mtl);
            const uint32_t first = (uint32_t)g.v.size();
            std::string tok;
            uint32_t corners = 0;
            while (ss >> tok) {
                std::string a, b, c;
                const size_t s1 = tok.find('/');
                if (s1 == std::string::npos) {
                    a = tok;
                } else {
                    a = tok.substr(0, s1);
                    const size_t s2 = tok.find('/', s1 + 1);
                    if (s2 == std::string::npos) {
                        b = tok.substr(s1 + 1);
                    } else {
                        b = tok.substr(s1 + 1, s2 - s1 - 1);
                        c = tok.substr(s2 + 1);
                    }
                }
                const long pi = obj_index(a, pos.size() / 3), ti = obj_index(b, uv.size() / 2),
                           ni = obj_index(c, nrm.size() / 3);
                KF_REQUIRE(pi >= 0 && ti != -2 && ni != -2, KF_ERR_INVALID_ARGUMENT,
                           "Failed to load scene: bad face index at line " + std::to_string(lineno) + " of " + path);
                kf_vertex vx{};
                for (int k = 0; k < 3; ++k) {
                    vx.pos[k] = pos[3 * pi + k];
                    vx.color[k] = col[3 * pi + k];
                }
                if (ti >= 0) {
                    vx.uv[0] = uv[2 * ti];
                    vx.uv[1] = uv[2 * ti + 1];
                }
                if (ni >= 0) {
                    for (int k = 0; k < 3; ++k) vx.normal[k] = nrm[3 * ni + k];
                    g.has_normals = true;
                }
                g.v.push_back(vx);
                ++corners;
            }
            KF_REQUIRE(corners >= 3, KF_ERR_INVALID_ARGUMENT,
                       "Failed to load scene: face with fewer than 3 vertices at line " + std::to_string(lineno));
            for (uint32_t k = 1; k + 1 < corners; ++k) // aiProcess_Triangulate (convex fan)
                g.idx.insert(g.idx.end(), {first, first + k, first + k + 1});
        }
        // o, g, s, l, p and other keys: grouping by material only (PreTransformVertices)
    }
    for (Group& g : groups) {
        if (g.idx.empty()) continue;
        if (!g.has_normals) { // aiProcess_GenNormals: flat normals of each face
            for (size_t t = 0; t + 2 < g.idx.size(); t += 3) {
                const float* a = g.v[g.idx[t]].pos;
                const float* b = g.v[g.idx[t + 1]].pos;
                const float* c = g.v[g.idx[t + 2]].pos;
                const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                              e1[0] * e2[1] - e1[1] * e2[0]};
                const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                if (len > 0.0f)
                    for (float& x : n) x /= len;
                for (int k = 0; k < 3; ++k)
                    for (int q = 0; q < 3; ++q) g.v[g.idx[t + k]].normal[q] = n[q];
            }
        }
        ObjMesh m;
        auto it = mtls.find(g.material);
        m.material = to_material(it != mtls.end() ? it->second : MtlDef{});
        m.material_name = g.material;
        m.vertices = std::move(g.v);
        m.indices = std::move(g.idx);
        out.push_back(std::move(m));
    }
}

} // namespace kf
