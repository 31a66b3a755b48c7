// kf_mesh.cpp — procedural meshes of kuafu's API (src/core/geometry.cpp:268-537)
// plus the subdivided icosahedron used by the 256-sphere benchmark scene.
#include <cmath>
#include <cstring>
#include <map>
#include <utility>

#include "kf_host.h"

namespace kf {

namespace {
kf_vertex vtx(float px, float py, float pz, float nx = 0, float ny = 0, float nz = 0, float u = 0, float v = 0) {
    kf_vertex o;
    std::memset(&o, 0, sizeof(o));
    o.pos[0] = px; o.pos[1] = py; o.pos[2] = pz;
    o.normal[0] = nx; o.normal[1] = ny; o.normal[2] = nz;
    o.uv[0] = u; o.uv[1] = v;
    return o;
}
// glm::normalize: v * inversesqrt(dot(v, v))
void gnormalize(float v[3]) {
    const float inv = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}
} // namespace

// Geometry::recalculateNormals (geometry.cpp:268-295): area-unweighted sum of
// unit face normals, renormalised; degenerate faces are skipped.
void recalculate_normals(std::vector<kf_vertex>& v, const std::vector<uint32_t>& idx) {
    for (auto& x : v) x.normal[0] = x.normal[1] = x.normal[2] = 0.0f;
    for (size_t i = 0; i + 2 < idx.size(); i += 3) {
        kf_vertex& a = v[idx[i]];
        kf_vertex& b = v[idx[i + 1]];
        kf_vertex& c = v[idx[i + 2]];
        const float e1[3] = {b.pos[0] - a.pos[0], b.pos[1] - a.pos[1], b.pos[2] - a.pos[2]};
        const float e2[3] = {c.pos[0] - a.pos[0], c.pos[1] - a.pos[1], c.pos[2] - a.pos[2]};
        float n[3] = {e1[1] * e2[2] - e2[1] * e1[2], e1[2] * e2[0] - e2[2] * e1[0], e1[0] * e2[1] - e2[0] * e1[1]};
        gnormalize(n);
        if (std::isnan(n[0])) continue;
        for (int k = 0; k < 3; ++k) {
            a.normal[k] += n[k];
            b.normal[k] += n[k];
            c.normal[k] += n[k];
        }
    }
    for (auto& x : v) {
        if (x.normal[0] == 0.0f && x.normal[1] == 0.0f && x.normal[2] == 0.0f) continue;
        gnormalize(x.normal);
    }
}

// createYZPlane (geometry.cpp:297-318): the unit square in x = 0 facing +x.
void mesh_yz_plane(std::vector<kf_vertex>& v, std::vector<uint32_t>& i) {
    v = {vtx(0, 1, 1, 1, 0, 0, 1, 0), vtx(0, -1, 1, 1, 0, 0, 0, 0), vtx(0, -1, -1, 1, 0, 0, 1, 1),
         vtx(0, 1, -1, 1, 0, 0, 0, 1)};
    i = {0, 1, 2, 0, 2, 3};
}

// createCube (geometry.cpp:320-372). The vertex table is kuafu's (a Blender
// export); it is data a drop-in must reproduce, so it is kept as is.
void mesh_cube(std::vector<kf_vertex>& v, std::vector<uint32_t>& i) {
    static const float T[24][8] = {
        {-1, 1, -1, 0, 1, 0, 0.875f, 0.5f},  {1, 1, 1, 0, 1, 0, 0.625f, 0.25f},   {1, 1, -1, 0, 1, 0, 0.625f, 0.5f},
        {1, 1, 1, 0, 0, 1, 0.625f, 0.25f},   {-1, -1, 1, 0, 0, 1, 0.375f, 0.0f},  {1, -1, 1, 0, 0, 1, 0.375f, 0.25f},
        {-1, 1, 1, -1, 0, 0, 0.625f, 1.0f},  {-1, -1, -1, -1, 0, 0, 0.375f, 0.75f}, {-1, -1, 1, -1, 0, 0, 0.375f, 1.0f},
        {1, -1, -1, 0, -1, 0, 0.375f, 0.5f}, {-1, -1, 1, 0, -1, 0, 0.125f, 0.25f}, {-1, -1, -1, 0, -1, 0, 0.125f, 0.5f},
        {1, 1, -1, 1, 0, 0, 0.625f, 0.5f},   {1, -1, 1, 1, 0, 0, 0.375f, 0.25f},  {1, -1, -1, 1, 0, 0, 0.375f, 0.5f},
        {-1, 1, -1, 0, 0, -1, 0.625f, 0.75f}, {1, -1, -1, 0, 0, -1, 0.375f, 0.5f}, {-1, -1, -1, 0, 0, -1, 0.375f, 0.75f},
        {-1, 1, 1, 0, 1, 0, 0.875f, 0.25f},  {-1, 1, 1, 0, 0, 1, 0.625f, 0.0f},   {-1, 1, -1, -1, 0, 0, 0.625f, 0.75f},
        {1, -1, 1, 0, -1, 0, 0.375f, 0.25f}, {1, 1, 1, 1, 0, 0, 0.625f, 0.25f},   {1, 1, -1, 0, 0, -1, 0.625f, 0.5f},
    };
    v.clear();
    for (const auto& r : T) v.push_back(vtx(r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7]));
    i = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17,
         0, 18, 1, 3, 19, 4, 6, 20, 7, 9, 21, 10, 12, 22, 13, 15, 23, 16};
}

// createSphere (geometry.cpp:375-433): 50 stacks x 50 slices, two poles.
void mesh_sphere(std::vector<kf_vertex>& v, std::vector<uint32_t>& idx) {
    const uint32_t stacks = 50, slices = 50;
    const float radius = 1.0f;
    const float pi = 3.14159265358979323846f;
    v.clear();
    idx.clear();
    for (uint32_t i = 1; i < stacks; ++i) {
        const float phi = pi / (float)stacks * (float)i - pi / 2.0f;
        for (uint32_t j = 0; j < slices; ++j) {
            const float theta = pi * 2.0f / (float)slices * (float)j;
            v.push_back(vtx(std::sin(phi) * radius, std::cos(theta) * std::cos(phi) * radius,
                            std::sin(theta) * std::cos(phi) * radius));
        }
    }
    for (uint32_t i = 0; i < (stacks - 2) * slices; ++i) {
        const uint32_t right = (i + 1) % slices + i / slices * slices;
        const uint32_t up = i + slices;
        const uint32_t rightUp = right + slices;
        idx.insert(idx.end(), {i, rightUp, up, i, right, rightUp});
    }
    v.push_back(vtx(-radius, 0, 0));
    v.push_back(vtx(radius, 0, 0));
    for (uint32_t i = 0; i < slices; ++i) {
        const uint32_t right = (i + 1) % slices + i / slices * slices;
        idx.insert(idx.end(), {(uint32_t)v.size() - 2, right, i});
    }
    for (uint32_t i = (stacks - 2) * slices; i < (stacks - 1) * slices; ++i) {
        const uint32_t right = (i + 1) % slices + i / slices * slices;
        idx.insert(idx.end(), {(uint32_t)v.size() - 1, i, right});
    }
    recalculate_normals(v, idx);
}

// createCapsule (geometry.cpp:437-537): 32 segments, 8 half rings, along x.
void mesh_capsule(float halfLength, float radius, std::vector<kf_vertex>& out_v, std::vector<uint32_t>& out_i) {
    const int segments = 32, halfRings = 8, rings = 2 * halfRings;
    const float pi = 3.14159265358979323846f;
    std::vector<kf_vertex> v;
    std::vector<uint32_t> idx;
    for (int s = 0; s < segments; ++s)
        v.push_back(vtx(radius + halfLength, 0, 0, 1, 0, 0, (0.5f + (float)s) / (float)segments, 1.0f));
    for (int r = 1; r <= halfRings; ++r) {
        const float theta = pi * (float)r / (float)rings;
        const float x = std::cos(theta), yz = std::sin(theta);
        for (int s = 0; s < segments + 1; ++s) {
            const float phi = pi * (float)s * 2.0f / (float)segments;
            const float y = yz * std::cos(phi), z = yz * std::sin(phi);
            v.push_back(vtx(x * radius + halfLength, y * radius, z * radius, x, y, z, (float)s / (float)segments,
                            1.0f - 0.5f * (float)r / (float)rings));
        }
    }
    for (int r = halfRings; r < rings; ++r) {
        const float theta = pi * (float)r / (float)rings;
        const float x = std::cos(theta), yz = std::sin(theta);
        for (int s = 0; s < segments + 1; ++s) {
            const float phi = pi * (float)s * 2.0f / (float)segments;
            const float y = yz * std::cos(phi), z = yz * std::sin(phi);
            v.push_back(vtx(x * radius - halfLength, y * radius, z * radius, x, y, z, (float)s / (float)segments,
                            0.5f - 0.5f * (float)r / (float)rings));
        }
    }
    for (int s = 0; s < segments; ++s)
        v.push_back(vtx(-radius - halfLength, 0, 0, -1, 0, 0, (0.5f + (float)s) / (float)segments, 0.0f));
    auto tri = [&](int a, int b, int c) { idx.insert(idx.end(), {(uint32_t)a, (uint32_t)b, (uint32_t)c}); };
    for (int s = 0; s < segments; ++s) tri(s, s + segments, s + segments + 1);
    for (int r = 0; r < rings - 1; ++r)
        for (int s = 0; s < segments; ++s) {
            const int a = segments + (segments + 1) * r + s, b = segments + (segments + 1) * (r + 1) + s;
            tri(a, b, b + 1);
            tri(a, b + 1, a + 1);
        }
    for (int s = 0; s < segments; ++s)
        tri(segments + (segments + 1) * (rings - 1) + s, segments + (segments + 1) * rings + s,
            segments + (segments + 1) * (rings - 1) + s + 1);
    out_v = std::move(v);
    out_i = std::move(idx);
}

// Unit icosphere: the icosahedron with every face split into four, `level` times,
// vertices pushed to the unit sphere; smooth normals as recalculateNormals makes
// them; uv = spherical angles. Level 4 has 5120 triangles.
void mesh_icosphere(int level, std::vector<kf_vertex>& v, std::vector<uint32_t>& idx) {
    KF_REQUIRE(level >= 0 && level <= 8, KF_ERR_INVALID_ARGUMENT, "icosphere level must be in [0, 8]");
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> P = {{-1, t, 0}, {1, t, 0},   {-1, -t, 0}, {1, -t, 0},
                                            {0, -1, t}, {0, 1, t},   {0, -1, -t}, {0, 1, -t},
                                            {t, 0, -1}, {t, 0, 1},   {-t, 0, -1}, {-t, 0, 1}};
    for (auto& p : P) {
        const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        p = {p[0] / n, p[1] / n, p[2] / n};
    }
    std::vector<uint32_t> F = {0, 11, 5, 0, 5, 1,  0, 1, 7,   0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                               11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4,  3, 4, 2,   3, 2, 6, 3, 6, 8,
                               3, 8, 9,  4, 9, 5,  2, 4, 11, 6, 2, 10, 8, 6, 7,   9, 8, 1};
    for (int l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            const auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            std::array<double, 3> m = {(P[a][0] + P[b][0]) * 0.5, (P[a][1] + P[b][1]) * 0.5, (P[a][2] + P[b][2]) * 0.5};
            const double n = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            m = {m[0] / n, m[1] / n, m[2] / n};
            P.push_back(m);
            const uint32_t id = (uint32_t)P.size() - 1;
            mid[key] = id;
            return id;
        };
        std::vector<uint32_t> G;
        G.reserve(F.size() * 4);
        for (size_t f = 0; f < F.size(); f += 3) {
            const uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
            const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            G.insert(G.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
        }
        F.swap(G);
    }
    v.clear();
    const double pi = 3.14159265358979323846;
    for (const auto& p : P) {
        const float u = (float)(0.5 + std::atan2(p[1], p[0]) / (2.0 * pi));
        const float w = (float)(0.5 - std::asin(std::max(-1.0, std::min(1.0, p[2]))) / pi);
        v.push_back(vtx((float)p[0], (float)p[1], (float)p[2], 0, 0, 0, u, w));
    }
    idx = F;
    recalculate_normals(v, idx);
}

} // namespace kf
