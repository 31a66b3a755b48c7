// kf_scene.cu — scene flattening and acceleration-structure upkeep.
//
// Mirrors kuafu's Scene::uploadGeometries / uploadGeometryInstances /
// uploadLightBuffers (src/core/scene.cpp:252-467) and the BLAS/TLAS management
// of RayTracer (src/core/rt/rt.cpp:142-495), with the driver's builder replaced
// by the GPU LBVH of kf_bvh.cu.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "kf_bvh.h"
#include "kf_host.h"

namespace kf {

std::mutex& global_mutex();
extern std::vector<kf_material> g_materials;
extern std::vector<HostTexture> g_textures;
extern uint64_t g_material_version, g_texture_version;

namespace {

// Triangle boxes of one geometry (object space).
__global__ void k_tri_boxes(const float4* __restrict__ verts, const uint32_t* __restrict__ idx, uint32_t vbase,
                            uint32_t tbase, uint32_t n, float4* lo, float4* hi) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float4 p[3];
    for (int k = 0; k < 3; ++k) p[k] = verts[3 * (size_t)(vbase + idx[3 * (size_t)(tbase + t) + k])];
    lo[t] = make_float4(fminf(fminf(p[0].x, p[1].x), p[2].x), fminf(fminf(p[0].y, p[1].y), p[2].y),
                        fminf(fminf(p[0].z, p[1].z), p[2].z), 0.0f);
    hi[t] = make_float4(fmaxf(fmaxf(p[0].x, p[1].x), p[2].x), fmaxf(fmaxf(p[0].y, p[1].y), p[2].y),
                        fmaxf(fmaxf(p[0].z, p[1].z), p[2].z), 0.0f);
}

// Precomputed triangles in BVH leaf order; the primitive id rides in v0.w.
__global__ void k_tri_gather(const float4* __restrict__ verts, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ order, uint32_t vbase, uint32_t tbase, uint32_t n, Tri* out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t prim = order[j];
    float4 p[3];
    for (int k = 0; k < 3; ++k) p[k] = verts[3 * (size_t)(vbase + idx[3 * (size_t)(tbase + prim) + k])];
    Tri t;
    t.v0 = make_float4(p[0].x, p[0].y, p[0].z, __uint_as_float(prim));
    t.v1 = make_float4(p[1].x, p[1].y, p[1].z, 0.0f);
    t.v2 = make_float4(p[2].x, p[2].y, p[2].z, 0.0f);
    out[j] = t;
}

// Rebase a freshly built node array into a pool: inner children += node_base, leaf
// children += leaf_base, instance links (TLAS leaves of one instance) += inst_base.
__global__ void k_rebase(const Node4* __restrict__ in, uint32_t n, uint32_t node_base, uint32_t leaf_base,
                         uint32_t inst_base, Node4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Node4 o = in[i];
    int c[4] = {o.child.x, o.child.y, o.child.z, o.child.w};
    const int k[4] = {o.cnt.x, o.cnt.y, o.cnt.z, o.cnt.w};
    for (int q = 0; q < 4; ++q) {
        if (k[q] == 0) c[q] += (int)node_base;
        else if (k[q] > 0) c[q] += (int)(((uint32_t)c[q] & kInstChildTag) ? inst_base : leaf_base);
    }
    o.child = make_int4(c[0], c[1], c[2], c[3]);
    out[i] = o;
}

// k_tri_gather over every geometry at once: out[j] for j in the triangle pool, the
// geometry found by binary search over the pool offsets of the `ng` geometries
// (geom[g] = {vertex offset, triangle offset, triangles, flags}); order holds each
// geometry's leaf order (geometry-local primitive ids) at its triangle offset.
__global__ void k_tri_gather_all(const float4* __restrict__ verts, const uint32_t* __restrict__ idx,
                                 const uint32_t* __restrict__ order, const uint4* __restrict__ geom, uint32_t ng,
                                 uint32_t n, Tri* out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t lo = 0, hi = ng;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (geom[mid].y <= j) lo = mid;
        else hi = mid;
    }
    const uint4 g = geom[lo];
    if (j - g.y >= g.z) return; // not a triangle of any geometry (cannot happen: the pool is dense)
    const uint32_t prim = order[j];
    float4 p[3];
    for (int k = 0; k < 3; ++k) p[k] = verts[3 * (size_t)(g.x + idx[3 * (size_t)(g.y + prim) + k])];
    Tri t;
    t.v0 = make_float4(p[0].x, p[0].y, p[0].z, __uint_as_float(prim));
    t.v1 = make_float4(p[1].x, p[1].y, p[1].z, 0.0f);
    t.v2 = make_float4(p[2].x, p[2].y, p[2].z, 0.0f);
    out[j] = t;
}

__global__ void k_map_ids(const uint32_t* __restrict__ order, const uint32_t* __restrict__ ids, uint32_t n,
                          uint32_t* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = ids[order[i]];
}

// Object-space bounds of a geometry's triangles for its instances' world boxes (the TLAS
// leaf boxes): the box of the referenced vertices, lo[3] hi[3], and the sphere around the
// box centre through the farthest vertex, centre[3] radius. Both hold every triangle (the
// convex hull of its vertices), so an instance's world box can be the overlap of the
// transformed box's box and the transformed sphere's box: O(1) per instance and update, and
// for a rotated sphere-like mesh as tight as the box of its transformed vertices, where the
// transformed box corners alone give a box up to sqrt(3) times wider per axis.
std::array<double, 10> geometry_bound(const kf_geometry_s* g) {
    const size_t nv = g->vertices.size(), ni = g->indices.size() / 3 * 3;
    std::array<double, 10> b{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0, 0, 0, 0};
    for (size_t i = 0; i < ni; ++i) {
        if (g->indices[i] >= nv) continue;
        const float* p = g->vertices[g->indices[i]].pos;
        for (int k = 0; k < 3; ++k) {
            b[k] = std::min(b[k], (double)p[k]);
            b[3 + k] = std::max(b[3 + k], (double)p[k]);
        }
    }
    if (!(b[0] <= b[3])) return b; // no triangle: the instance is hidden
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) b[6 + k] = 0.5 * (b[k] + b[3 + k]);
    for (size_t i = 0; i < ni; ++i) {
        if (g->indices[i] >= nv) continue;
        const float* p = g->vertices[g->indices[i]].pos;
        double d2 = 0.0;
        for (int k = 0; k < 3; ++k) d2 += ((double)p[k] - b[6 + k]) * ((double)p[k] - b[6 + k]);
        r2 = std::max(r2, d2);
    }
    b[9] = std::sqrt(r2);
    return b;
}

void root_box(const Node4& n, std::array<float, 6>& b) {
    const float lx[4] = {n.lox.x, n.lox.y, n.lox.z, n.lox.w}, hx[4] = {n.hix.x, n.hix.y, n.hix.z, n.hix.w};
    const float ly[4] = {n.loy.x, n.loy.y, n.loy.z, n.loy.w}, hy[4] = {n.hiy.x, n.hiy.y, n.hiy.z, n.hiy.w};
    const float lz[4] = {n.loz.x, n.loz.y, n.loz.z, n.loz.w}, hz[4] = {n.hiz.x, n.hiz.y, n.hiz.z, n.hiz.w};
    const int cn[4] = {n.cnt.x, n.cnt.y, n.cnt.z, n.cnt.w};
    b = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 4; ++c) {
        if (cn[c] < 0) continue;
        b[0] = std::min(b[0], lx[c]); b[1] = std::min(b[1], ly[c]); b[2] = std::min(b[2], lz[c]);
        b[3] = std::max(b[3], hx[c]); b[4] = std::max(b[4], hy[c]); b[5] = std::max(b[5], hz[c]);
    }
}

} // namespace

// Light uniform buffers exactly as Scene::uploadLightBuffers builds them (scene.cpp:252-292).
void scene_light_ubos(const kf_scene_s* s, kf_dir_light_ubo* d, kf_point_lights_ubo* p, kf_active_lights_ubo* a) {
    std::memset(d, 0, sizeof(*d));
    std::memset(p, 0, sizeof(*p));
    std::memset(a, 0, sizeof(*a));
    if (s->has_dir_light) {
        const float* dir = s->dir_light.direction;
        // glm::normalize: v * inversesqrt(dot(v, v))
        const float len2 = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
        const float inv = 1.0f / std::sqrt(len2);
        d->direction[0] = dir[0] * inv;
        d->direction[1] = dir[1] * inv;
        d->direction[2] = dir[2] * inv;
        d->direction[3] = s->dir_light.softness;
        d->rgbs[0] = s->dir_light.color[0];
        d->rgbs[1] = s->dir_light.color[1];
        d->rgbs[2] = s->dir_light.color[2];
        d->rgbs[3] = s->dir_light.strength;
    } else {
        d->rgbs[3] = 0.0f;
    }
    for (size_t i = 0; i < KF_MAX_POINT_LIGHTS; ++i) {
        if (i < s->point_lights.size()) {
            const kf_point_light& l = s->point_lights[i]->point;
            p->posr[i][0] = l.position[0]; p->posr[i][1] = l.position[1]; p->posr[i][2] = l.position[2];
            p->posr[i][3] = l.radius;
            p->rgbs[i][0] = l.color[0]; p->rgbs[i][1] = l.color[1]; p->rgbs[i][2] = l.color[2];
            p->rgbs[i][3] = l.strength;
        } else {
            p->rgbs[i][3] = 0.0f;
        }
    }
    for (size_t i = 0; i < KF_MAX_ACTIVE_LIGHTS; ++i) {
        if (i < s->active_lights.size()) {
            const kf_active_light& l = s->active_lights[i]->active;
            float vinv[16];
            inverse4_d(l.view, vinv);
            std::memcpy(a->view[i], l.view, sizeof(float) * 16);
            perspective(l.fov, 1.0f, 0.01f, 1000.0f, a->proj[i]);
            a->front[i][0] = -vinv[2 * 4 + 0]; a->front[i][1] = -vinv[2 * 4 + 1]; a->front[i][2] = -vinv[2 * 4 + 2];
            a->front[i][3] = 1.0f;
            a->rgbs[i][0] = l.color[0]; a->rgbs[i][1] = l.color[1]; a->rgbs[i][2] = l.color[2];
            a->rgbs[i][3] = l.strength;
            a->position[i][0] = vinv[3 * 4 + 0]; a->position[i][1] = vinv[3 * 4 + 1];
            a->position[i][2] = vinv[3 * 4 + 2]; a->position[i][3] = 0.0f;
            const int tex = (l.tex_id >= 0 && (uint32_t)l.tex_id < g_textures.size()) ? l.tex_id : -1;
            a->sftp[i][0] = l.softness; a->sftp[i][1] = l.fov; a->sftp[i][2] = (float)tex; a->sftp[i][3] = 0.0f;
        } else {
            a->front[i][3] = 0.0f;
        }
    }
}

std::vector<kf_material_gpu> flatten_materials() {
    std::vector<kf_material_gpu> out;
    out.reserve(g_materials.size());
    for (const kf_material& m : g_materials) {
        kf_material_gpu g{};
        g.diffuse[0] = m.diffuse_color[0]; g.diffuse[1] = m.diffuse_color[1]; g.diffuse[2] = m.diffuse_color[2];
        g.diffuse[3] = 0.0f;
        g.emission[0] = m.emission[0]; g.emission[1] = m.emission[1]; g.emission[2] = m.emission[2];
        g.emission[3] = m.emission_strength;
        g.alpha = m.alpha; g.metallic = m.metallic; g.specular = m.specular; g.roughness = m.roughness;
        g.ior = m.ior; g.transmission = m.transmission;
        auto tex = [](int32_t id) { return (id >= 0 && (size_t)id < g_textures.size()) ? id : -1; };
        g.diffuse_tex = tex(m.diffuse_tex);
        g.metallic_tex = tex(m.metallic_tex);
        g.roughness_tex = tex(m.roughness_tex);
        g.transmission_tex = tex(m.transmission_tex);
        out.push_back(g);
    }
    return out;
}

// Bring the device copy of a scene up to date: geometry buffers + BLAS when the
// geometry set changed, TLAS when instances changed, materials / textures when the
// global tables changed, lights every frame (uploadLightBuffers runs every frame).
void scene_sync_gpu(kf_renderer_s* r, kf_scene_s* s) {
    cudaStream_t st = r->stream;
    SceneGpu& G = s->gpu;
    bool rebuilt_geom = false;
    // build timing (bvh_build_ms): events around the update, waited on only when something
    // was built, so that a frame without changes queues behind the previous one unblocked
    struct SyncEvents {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~SyncEvents() {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } ev;
    KF_CUDA_CHECK(cudaEventCreate(&ev.e0));
    KF_CUDA_CHECK(cudaEventCreate(&ev.e1));
    KF_CUDA_CHECK(cudaEventRecord(ev.e0, st));
    bool built_any = false, refitted = false, matidx_changed = false;
    const uint32_t bvh_key = 1u | (r->cfg.bvh_builder << 1) | (r->cfg.blas_leaf_size << 2) |
                             ((r->cfg.blas_share ? 1u : 0u) << 8);
    // a geometry's versions only grow, so their sums change whenever one of them does
    uint64_t vert_sum = 0, flag_sum = 0;
    for (const kf_geometry_s* g : s->geometries) {
        vert_sum += g->vert_version;
        flag_sum += g->version;
    }
    const bool geom_changed =
        G.built_geom_stamp != s->geom_stamp || G.built_bvh_key != bvh_key || G.built_vert_sum != vert_sum;
    if (geom_changed || G.built_material_version != g_material_version) {
        // every triangle must name an existing material (the kernels index the table
        // unchecked); checked before anything is uploaded or marked as built, so that a
        // refused scene leaves no stale index on the device
        for (const kf_geometry_s* g : s->geometries) {
            const size_t ntri = g->indices.size() / 3;
            for (size_t t = 0; t < ntri; ++t)
                KF_REQUIRE(g->mat_index[t] < g_materials.size(), KF_ERR_OUT_OF_RANGE,
                           "a geometry's matIndex names a material that does not exist");
        }
    }
    if (geom_changed) {
        built_any = true;
        rebuilt_geom = true;
        const size_t ng = s->geometries.size();
        std::vector<float4> verts;
        std::vector<uint32_t> idx, mat;
        std::vector<uint4> geom(ng);
        G.vert_offset.assign(ng, 0);
        G.tri_offset.assign(ng, 0);
        size_t nv = 0, nt = 0;
        for (size_t gi = 0; gi < ng; ++gi) {
            nv += s->geometries[gi]->vertices.size();
            nt += s->geometries[gi]->indices.size() / 3;
        }
        verts.resize(nv * 3);
        idx.reserve(nt * 3);
        mat.reserve(nt);
        // traversal stack entries address leaves as 26-bit triangle offsets with a 4-bit count
        KF_REQUIRE(nt < (1ull << 26), KF_ERR_LIMIT, "a scene holds at most 67108863 triangles");
        // geometry records hold 32-bit vertex offsets
        KF_REQUIRE(nv < (1ull << 32), KF_ERR_LIMIT, "a scene holds at most 4294967295 vertices");
        KF_REQUIRE(r->cfg.blas_leaf_size >= 1 && r->cfg.blas_leaf_size <= 16, KF_ERR_INVALID_ARGUMENT,
                   "blas_leaf_size must be in [1, 16]");
        // TLAS leaves are stack entries too: 26-bit offsets into the leaf list, <= 16 instances
        KF_REQUIRE(s->instances.size() < (1ull << 26), KF_ERR_LIMIT, "too many instances");
        KF_REQUIRE(r->cfg.tlas_leaf_size >= 1 && r->cfg.tlas_leaf_size <= 16, KF_ERR_INVALID_ARGUMENT,
                   "tlas_leaf_size must be in [1, 16]");
        size_t vo = 0, to = 0;
        for (size_t gi = 0; gi < ng; ++gi) {
            const kf_geometry_s* g = s->geometries[gi];
            const uint32_t ntri = (uint32_t)(g->indices.size() / 3);
            std::memcpy(&verts[vo * 3], g->vertices.data(), sizeof(kf_vertex) * g->vertices.size());
            idx.insert(idx.end(), g->indices.begin(), g->indices.begin() + 3 * (size_t)ntri);
            mat.insert(mat.end(), g->mat_index.begin(), g->mat_index.begin() + ntri);
            uint32_t flags = (g->opaque ? 1u : 0u) | (g->hide_render ? 2u : 0u);
            geom[gi] = make_uint4((uint32_t)vo, (uint32_t)to, ntri, flags);
            G.vert_offset[gi] = (uint32_t)vo;
            G.tri_offset[gi] = (uint32_t)to;
            vo += g->vertices.size();
            to += ntri;
        }
        G.verts.upload(verts.data(), verts.size(), st);
        G.indices.upload(idx.data(), idx.size(), st);
        G.matidx.upload(mat.data(), mat.size(), st);
        G.geom.upload(geom.data(), geom.size(), st);

        // BLAS per geometry, appended to one node pool and one triangle pool.
        G.blas_root.assign(ng, 0);
        G.blas_box.assign(ng, {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY});
        G.blas_bound.resize(ng);
        for (size_t gi = 0; gi < ng; ++gi) G.blas_bound[gi] = geometry_bound(s->geometries[gi]);
        size_t total_nodes_est = 0;
        for (size_t gi = 0; gi < ng; ++gi) total_nodes_est += std::max<size_t>(1, s->geometries[gi]->indices.size() / 3);
        G.blas_nodes.resize(std::max<size_t>(total_nodes_est, 1), st);
        G.tris.resize(std::max<size_t>(nt, 1), st);
        uint32_t node_base = 0;
        DeviceBuffer<float4> lo, hi;
        DeviceBuffer<Node4> nodes;
        DeviceBuffer<uint32_t> order;
        // host SAH builds of every BLAS, in parallel over geometries (bvh_builder = 1)
        const bool sah = r->cfg.bvh_builder == 1;
        std::vector<std::vector<Node4>> sah_nodes(sah ? ng : 0);
        std::vector<std::vector<uint32_t>> sah_order(sah ? ng : 0);
        // geometries whose triangles are byte-identical (same positions and indices, the
        // materials may differ) share one build; with blas_share they also share one copy
        // of its nodes and triangles (a triangle carries its geometry-local primitive id,
        // the instance names the geometry, so the hit is the same), else each gets its own
        std::vector<size_t> build_of(ng);
        std::vector<size_t> to_build;
        {
            std::unordered_map<uint64_t, std::vector<size_t>> seen;
            auto fnv = [](uint64_t h, const void* p, size_t n) {
                const unsigned char* b = static_cast<const unsigned char*>(p);
                for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
                return h;
            };
            auto same = [&](const kf_geometry_s* a, const kf_geometry_s* b) {
                if (a->indices.size() != b->indices.size() || a->vertices.size() != b->vertices.size()) return false;
                if (std::memcmp(a->indices.data(), b->indices.data(), a->indices.size() * sizeof(uint32_t))) return false;
                for (size_t v = 0; v < a->vertices.size(); ++v)
                    if (std::memcmp(a->vertices[v].pos, b->vertices[v].pos, sizeof(float) * 3)) return false;
                return true;
            };
            for (size_t gi = 0; gi < ng; ++gi) {
                const kf_geometry_s* g = s->geometries[gi];
                uint64_t h = fnv(0xcbf29ce484222325ull, g->indices.data(), g->indices.size() * sizeof(uint32_t));
                for (const kf_vertex& v : g->vertices) h = fnv(h, v.pos, sizeof(float) * 3);
                std::vector<size_t>& cand = seen[h];
                size_t found = SIZE_MAX;
                for (size_t c : cand)
                    if (same(s->geometries[c], g)) found = c;
                if (found == SIZE_MAX) {
                    cand.push_back(gi);
                    to_build.push_back(gi);
                    build_of[gi] = gi;
                } else {
                    build_of[gi] = found;
                }
            }
        }
        if (sah) {
            const int leaf = (int)std::max(1u, r->cfg.blas_leaf_size);
            std::atomic<size_t> next{0};
            auto work = [&]() {
                std::vector<float> blo, bhi;
                for (size_t k; (k = next.fetch_add(1)) < to_build.size();) {
                    const size_t gi = to_build[k];
                    const kf_geometry_s* g = s->geometries[gi];
                    const size_t nt_g = g->indices.size() / 3;
                    blo.resize(3 * nt_g);
                    bhi.resize(3 * nt_g);
                    for (size_t t = 0; t < nt_g; ++t)
                        for (int k = 0; k < 3; ++k) {
                            const float a = g->vertices[g->indices[3 * t + 0]].pos[k];
                            const float b = g->vertices[g->indices[3 * t + 1]].pos[k];
                            const float c = g->vertices[g->indices[3 * t + 2]].pos[k];
                            blo[3 * t + k] = std::min(std::min(a, b), c);
                            bhi[3 * t + k] = std::max(std::max(a, b), c);
                        }
                    build_wide_bvh_sah_host(blo.data(), bhi.data(), (int)nt_g, leaf, sah_nodes[gi], sah_order[gi]);
                }
            };
            const unsigned nthreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
            std::vector<std::thread> pool;
            for (unsigned i = 1; i < nthreads; ++i) pool.emplace_back(work);
            work();
            for (std::thread& t : pool) t.join();
        }
        if (sah) {
            // every BLAS in one pool upload: children rebased on the host (inner links by the
            // BLAS's first node, leaf links by its first triangle), one leaf-order array at the
            // triangle offsets, one gather kernel for the whole triangle pool; no per-BLAS sync
            std::vector<Node4> pool;
            pool.reserve(total_nodes_est);
            std::vector<uint32_t> order_all(std::max<size_t>(nt, 1), 0u);
            const bool share = r->cfg.blas_share != 0;
            for (size_t gi = 0; gi < ng; ++gi) {
                if (geom[gi].z == 0) continue;
                const size_t bi = build_of[gi];
                if (share && bi != gi) { // the first geometry of this build was placed before
                    G.blas_root[gi] = G.blas_root[bi];
                    G.blas_box[gi] = G.blas_box[bi];
                    continue;
                }
                G.blas_root[gi] = (uint32_t)pool.size();
                root_box(sah_nodes[bi][0], G.blas_box[gi]);
                const uint32_t nb = (uint32_t)pool.size(), tb = geom[gi].y;
                for (Node4 nd : sah_nodes[bi]) {
                    int* c = &nd.child.x;
                    const int* k = &nd.cnt.x;
                    for (int q = 0; q < 4; ++q) {
                        if (k[q] == 0) c[q] += (int)nb;
                        else if (k[q] > 0) c[q] += (int)tb;
                    }
                    pool.push_back(nd);
                }
                std::copy(sah_order[bi].begin(), sah_order[bi].end(), order_all.begin() + tb);
            }
            if (!pool.empty()) G.blas_nodes.upload(pool.data(), pool.size(), st);
            order.upload(order_all.data(), order_all.size(), st);
            if (nt > 0) {
                k_tri_gather_all<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
                    G.verts.ptr, G.indices.ptr, order.ptr, G.geom.ptr, (uint32_t)ng, (uint32_t)nt, G.tris.ptr);
                KF_CUDA_CHECK(cudaGetLastError());
            }
            node_base = (uint32_t)pool.size();
        }
        // GPU builds (bvh_builder 0: LBVH, 2: PLOC), one per geometry; with blas_share a geometry
        // identical to an earlier one takes that one's BLAS instead of a build of its own
        for (size_t gi = 0; gi < ng && !sah; ++gi) {
            const uint32_t ntri = geom[gi].z;
            if (ntri == 0) continue;
            if (r->cfg.blas_share && build_of[gi] != gi) {
                G.blas_root[gi] = G.blas_root[build_of[gi]];
                G.blas_box[gi] = G.blas_box[build_of[gi]];
                continue;
            }
            lo.resize(ntri, st);
            hi.resize(ntri, st);
            k_tri_boxes<<<(ntri + 255) / 256, 256, 0, st>>>(G.verts.ptr, G.indices.ptr, geom[gi].x, geom[gi].y, ntri,
                                                            lo.ptr, hi.ptr);
            KF_CUDA_CHECK(cudaGetLastError());
            const int nn =
                build_wide_bvh(lo.ptr, hi.ptr, (int)ntri, (int)std::max(1u, r->cfg.blas_leaf_size), nodes, order, st,
                               r->cfg.bvh_builder == 2);
            k_tri_gather<<<(ntri + 255) / 256, 256, 0, st>>>(G.verts.ptr, G.indices.ptr, order.ptr, geom[gi].x,
                                                             geom[gi].y, ntri, G.tris.ptr + geom[gi].y);
            k_rebase<<<(nn + 127) / 128, 128, 0, st>>>(nodes.ptr, (uint32_t)nn, node_base, geom[gi].y, 0u,
                                                       G.blas_nodes.ptr + node_base);
            KF_CUDA_CHECK(cudaGetLastError());
            Node4 root;
            KF_CUDA_CHECK(cudaMemcpyAsync(&root, nodes.ptr, sizeof(Node4), cudaMemcpyDeviceToHost, st));
            KF_CUDA_CHECK(cudaStreamSynchronize(st));
            root_box(root, G.blas_box[gi]);
            G.blas_root[gi] = node_base;
            node_base += (uint32_t)nn;
        }
        G.blas_node_count = node_base;
        G.built_geom_stamp = s->geom_stamp;
        G.built_bvh_key = bvh_key;
        G.built_vert_sum = vert_sum;
    }
    if (G.built_material_version != g_material_version || rebuilt_geom) {
        std::vector<kf_material_gpu> mats = flatten_materials();
        if (!rebuilt_geom) {
            // the per-triangle material indices follow the geometries' current ones
            // (Geometry::setMaterial after the first upload, or a cleared and refilled table)
            std::vector<uint32_t> mat;
            mat.reserve(G.matidx.count);
            for (const kf_geometry_s* g : s->geometries)
                mat.insert(mat.end(), g->mat_index.begin(), g->mat_index.begin() + g->indices.size() / 3);
            KF_REQUIRE(mat.size() == G.matidx.count, KF_ERR_INTERNAL, "material index count changed");
            G.matidx.upload(mat.data(), mat.size(), st);
            matidx_changed = true;
        }
        if (mats.empty()) mats.push_back(kf_material_gpu{});
        G.materials.upload(mats.data(), mats.size(), st);
        G.built_material_version = g_material_version;
        ++G.generation;
    }
    if (G.built_texture_version != g_texture_version || G.srgb_decode.count == 0) {
        std::vector<uint4> info;
        std::vector<uchar4> texels;
        for (const HostTexture& t : g_textures) {
            // texture records hold 32-bit texel offsets
            KF_REQUIRE(texels.size() + (size_t)t.w * t.h < (1ull << 32), KF_ERR_LIMIT,
                       "the textures hold at most 4294967295 texels in total");
            info.push_back(make_uint4((uint32_t)texels.size(), t.w, t.h, t.srgb));
            const uchar4* p = reinterpret_cast<const uchar4*>(t.rgba.data());
            texels.insert(texels.end(), p, p + (size_t)t.w * t.h);
        }
        if (info.empty()) info.push_back(make_uint4(0, 1, 1, 0));
        if (texels.empty()) texels.push_back(make_uchar4(255, 255, 255, 255));
        G.tex_info.upload(info.data(), info.size(), st);
        G.texels.upload(texels.data(), texels.size(), st);
        const std::vector<float>& dec = srgb_decode_table();
        G.srgb_decode.upload(dec.data(), dec.size(), st);
        G.built_texture_version = g_texture_version;
        ++G.generation;
    }
    if (G.built_env_version != s->env_version) {
        // uploadEnvironmentMap (scene.cpp:294-310)
        if (s->env_size) {
            G.env.upload(reinterpret_cast<const float4*>(s->env_texels.data()), s->env_texels.size() / 4, st);
        } else {
            G.env.release();
        }
        G.built_env_version = s->env_version;
        ++G.generation;
    }
    // Instance records (world->object rows, BLAS root, flags) and padded world boxes of the
    // visible instances; wlo / whi indexed by instance, ids = the visible instances.
    auto instance_records = [&](std::vector<InstanceRec>& recs, std::vector<float4>& wlo,
                                std::vector<float4>& whi, std::vector<uint32_t>& ids) {
        const size_t ni = s->instances.size();
        recs.assign(ni, InstanceRec{});
        wlo.assign(ni, make_float4(0, 0, 0, 0));
        whi.assign(ni, make_float4(0, 0, 0, 0));
        ids.clear();
        for (size_t i = 0; i < ni; ++i) {
            const kf_instance_s* in = s->instances[i];
            size_t gi = 0;
            for (; gi < s->geometries.size(); ++gi)
                if (s->geometries[gi] == in->geometry) break;
            KF_REQUIRE(gi < s->geometries.size(), KF_ERR_STATE,
                       "instance references a geometry not submitted to the scene");
            float rows[12];
            affine_inverse_rows(in->transform, rows);
            InstanceRec& rc = recs[i];
            rc.w2o0 = make_float4(rows[0], rows[1], rows[2], rows[3]);
            rc.w2o1 = make_float4(rows[4], rows[5], rows[6], rows[7]);
            rc.w2o2 = make_float4(rows[8], rows[9], rows[10], rows[11]);
            rc.blas_root = G.blas_root.empty() ? 0 : G.blas_root[gi];
            rc.geometry = (uint32_t)gi;
            const kf_geometry_s* g = s->geometries[gi];
            const bool hidden = g->hide_render || g->indices.size() < 3;
            rc.flags = (g->opaque ? 1u : 0u) | (hidden ? 2u : 0u);
            rc.pad = 0;
            if (hidden) continue;
            // world box (double, padded): the transformed object box's box overlapped with the
            // transformed bounding sphere's box (half extent along axis k: radius x |row k|)
            const std::array<double, 10>& gb = G.blas_bound[gi];
            double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
            const float* m = in->transform;
            for (int c = 0; c < 8; ++c) {
                const double p[3] = {(c & 1) ? gb[3] : gb[0], (c & 2) ? gb[4] : gb[1], (c & 4) ? gb[5] : gb[2]};
                for (int k = 0; k < 3; ++k) {
                    const double v = (double)m[0 * 4 + k] * p[0] + (double)m[1 * 4 + k] * p[1] +
                                     (double)m[2 * 4 + k] * p[2] + (double)m[3 * 4 + k];
                    mn[k] = std::min(mn[k], v);
                    mx[k] = std::max(mx[k], v);
                }
            }
            for (int k = 0; k < 3; ++k) {
                const double c = (double)m[0 * 4 + k] * gb[6] + (double)m[1 * 4 + k] * gb[7] +
                                 (double)m[2 * 4 + k] * gb[8] + (double)m[3 * 4 + k];
                const double row = std::sqrt((double)m[0 * 4 + k] * m[0 * 4 + k] + (double)m[1 * 4 + k] * m[1 * 4 + k] +
                                             (double)m[2 * 4 + k] * m[2 * 4 + k]);
                mn[k] = std::max(mn[k], c - gb[9] * row);
                mx[k] = std::min(mx[k], c + gb[9] * row);
            }
            double mag = 0.0;
            for (int k = 0; k < 3; ++k) mag = std::max(mag, std::max(std::fabs(mn[k]), std::fabs(mx[k])));
            const double pad = mag * 0x1.0p-16 + 1e-6;
            wlo[i] = make_float4((float)(mn[0] - pad), (float)(mn[1] - pad), (float)(mn[2] - pad), 0.0f);
            whi[i] = make_float4((float)(mx[0] + pad), (float)(mx[1] + pad), (float)(mx[2] + pad), 0.0f);
            ids.push_back((uint32_t)i);
        }
    };
    // the instance records carry each geometry's opaque and hidden flags (kuafu reads
    // hideRender when it rebuilds the TLAS every frame, rt.cpp:156): a change rebuilds
    const bool set_changed = rebuilt_geom || G.built_inst_stamp != s->inst_stamp || G.built_flag_sum != flag_sum;
    if (!set_changed && G.built_xform_stamp != s->xform_stamp) {
        // Transforms moved, the instance set did not (RayTracer::updateTlas every frame,
        // context.cpp:334-341): new world->object rows and world boxes; the TLAS keeps its
        // topology and its node boxes are refitted children-first (children are always
        // numbered after their parent). Buffers keep their size: no graph recapture.
        refitted = true;
        std::vector<InstanceRec> recs;
        std::vector<float4> wlo, whi;
        std::vector<uint32_t> ids;
        instance_records(recs, wlo, whi, ids);
        if (!recs.empty()) G.inst.upload(recs.data(), recs.size(), st);
        std::vector<Node4>& nodes = G.tlas_host_nodes;
        for (size_t n = nodes.size(); n-- > 0;) {
            Node4& nd = nodes[n];
            float lx[4], ly[4], lz[4], hx[4], hy[4], hz[4];
            const int ch[4] = {nd.child.x, nd.child.y, nd.child.z, nd.child.w};
            const int cn[4] = {nd.cnt.x, nd.cnt.y, nd.cnt.z, nd.cnt.w};
            for (int c = 0; c < 4; ++c) {
                lx[c] = ly[c] = lz[c] = INFINITY;
                hx[c] = hy[c] = hz[c] = -INFINITY;
                if (cn[c] < 0) continue;
                if (cn[c] == 0) {
                    const Node4& k = nodes[ch[c]];
                    lx[c] = std::min(std::min(k.lox.x, k.lox.y), std::min(k.lox.z, k.lox.w));
                    ly[c] = std::min(std::min(k.loy.x, k.loy.y), std::min(k.loy.z, k.loy.w));
                    lz[c] = std::min(std::min(k.loz.x, k.loz.y), std::min(k.loz.z, k.loz.w));
                    hx[c] = std::max(std::max(k.hix.x, k.hix.y), std::max(k.hix.z, k.hix.w));
                    hy[c] = std::max(std::max(k.hiy.x, k.hiy.y), std::max(k.hiy.z, k.hiy.w));
                    hz[c] = std::max(std::max(k.hiz.x, k.hiz.y), std::max(k.hiz.z, k.hiz.w));
                } else {
                    for (int q = 0; q < cn[c]; ++q) {
                        const uint32_t id = ((uint32_t)ch[c] & kInstChildTag)
                                                ? ((uint32_t)ch[c] & ~kInstChildTag)
                                                : G.tlas_host_inst[leaf_first(ch[c]) + q];
                        lx[c] = std::min(lx[c], wlo[id].x); ly[c] = std::min(ly[c], wlo[id].y);
                        lz[c] = std::min(lz[c], wlo[id].z); hx[c] = std::max(hx[c], whi[id].x);
                        hy[c] = std::max(hy[c], whi[id].y); hz[c] = std::max(hz[c], whi[id].z);
                    }
                }
            }
            nd.lox = make_float4(lx[0], lx[1], lx[2], lx[3]);
            nd.loy = make_float4(ly[0], ly[1], ly[2], ly[3]);
            nd.loz = make_float4(lz[0], lz[1], lz[2], lz[3]);
            nd.hix = make_float4(hx[0], hx[1], hx[2], hx[3]);
            nd.hiy = make_float4(hy[0], hy[1], hy[2], hy[3]);
            nd.hiz = make_float4(hz[0], hz[1], hz[2], hz[3]);
        }
        if (!nodes.empty()) G.tlas_nodes.upload(nodes.data(), nodes.size(), st);
        G.built_xform_stamp = s->xform_stamp;
        ++G.tlas_refits;
    }
    if (set_changed) {
        built_any = true;
        std::vector<InstanceRec> recs;
        std::vector<float4> wlo, whi;
        std::vector<uint32_t> ids;
        instance_records(recs, wlo, whi, ids);
        std::vector<float4> blo, bhi;
        for (uint32_t id : ids) {
            blo.push_back(wlo[id]);
            bhi.push_back(whi[id]);
        }
        G.inst.upload(recs.data(), std::max<size_t>(recs.size(), 0), st);
        if (recs.empty()) G.inst.resize(1, st);
        const uint32_t nv = (uint32_t)ids.size();
        if (nv > 0) {
            DeviceBuffer<float4> dlo, dhi;
            DeviceBuffer<uint32_t> dids, order;
            dlo.upload(blo.data(), nv, st);
            dhi.upload(bhi.data(), nv, st);
            dids.upload(ids.data(), nv, st);
            int nn;
            if (r->cfg.bvh_builder == 1) {
                std::vector<float> flo(3 * (size_t)nv), fhi(3 * (size_t)nv);
                for (uint32_t i = 0; i < nv; ++i) {
                    flo[3 * i] = blo[i].x; flo[3 * i + 1] = blo[i].y; flo[3 * i + 2] = blo[i].z;
                    fhi[3 * i] = bhi[i].x; fhi[3 * i + 1] = bhi[i].y; fhi[3 * i + 2] = bhi[i].z;
                }
                std::vector<Node4> hn;
                std::vector<uint32_t> ho;
                nn = build_wide_bvh_sah_host(flo.data(), fhi.data(), (int)nv,
                                             (int)std::max(1u, r->cfg.tlas_leaf_size), hn, ho);
                G.tlas_nodes.upload(hn.data(), hn.size(), st);
                order.upload(ho.data(), ho.size(), st);
            } else {
                nn = build_wide_bvh(dlo.ptr, dhi.ptr, (int)nv, (int)std::max(1u, r->cfg.tlas_leaf_size),
                                    G.tlas_nodes, order, st, r->cfg.bvh_builder == 2);
            }
            G.tlas_inst.resize(nv, st);
            k_map_ids<<<(nv + 255) / 256, 256, 0, st>>>(order.ptr, dids.ptr, nv, G.tlas_inst.ptr);
            KF_CUDA_CHECK(cudaGetLastError());
            G.tlas_node_count = (uint32_t)nn;
            // host copies of the topology for later refits
            G.tlas_host_nodes.resize(nn);
            G.tlas_host_inst.resize(nv);
            KF_CUDA_CHECK(cudaMemcpyAsync(G.tlas_host_nodes.data(), G.tlas_nodes.ptr, sizeof(Node4) * nn,
                                          cudaMemcpyDeviceToHost, st));
            KF_CUDA_CHECK(cudaMemcpyAsync(G.tlas_host_inst.data(), G.tlas_inst.ptr, sizeof(uint32_t) * nv,
                                          cudaMemcpyDeviceToHost, st));
            KF_CUDA_CHECK(cudaStreamSynchronize(st));
            // a leaf of one instance links the instance itself (the traversal enters it without
            // reading the leaf list)
            for (Node4& nd : G.tlas_host_nodes) {
                int* ch = &nd.child.x;
                const int* cn = &nd.cnt.x;
                for (int c = 0; c < 4; ++c)
                    if (cn[c] == 1) ch[c] = (int)(kInstChildTag | G.tlas_host_inst[leaf_first(ch[c])]);
            }
            G.tlas_nodes.upload(G.tlas_host_nodes.data(), G.tlas_host_nodes.size(), st);
        } else {
            G.tlas_node_count = 0;
            G.tlas_nodes.resize(1, st);
            G.tlas_inst.resize(1, st);
            G.tlas_host_nodes.clear();
            G.tlas_host_inst.clear();
        }
        G.built_inst_stamp = s->inst_stamp;
        G.built_xform_stamp = s->xform_stamp;
        G.built_flag_sum = flag_sum;
    }
    if (built_any || rebuilt_geom) ++G.generation;            // buffers may have moved: recapture graphs
    if (built_any || rebuilt_geom || refitted || matidx_changed) ++G.content_version; // contents changed: recopy batch pools
    if (built_any) {
        KF_CUDA_CHECK(cudaEventRecord(ev.e1, st));
        KF_CUDA_CHECK(cudaEventSynchronize(ev.e1));
        float ms = 0.0f;
        KF_CUDA_CHECK(cudaEventElapsedTime(&ms, ev.e0, ev.e1));
        r->stats.bvh_build_ms += ms;
    }
    // lights: every frame, like uploadUniformBuffers
    kf_dir_light_ubo d;
    kf_point_lights_ubo p;
    kf_active_lights_ubo a;
    scene_light_ubos(s, &d, &p, &a);
    G.dlight.upload(&d, 1, st);
    G.plights.upload(&p, 1, st);
    G.alights.upload(&a, 1, st);

    SceneDev& v = G.view;
    v.verts = G.verts.ptr;
    v.indices = G.indices.ptr;
    v.matidx = G.matidx.ptr;
    v.geom = G.geom.ptr;
    v.materials = G.materials.ptr;
    v.inst = G.inst.ptr;
    v.blas_nodes = G.blas_nodes.ptr;
    v.tris = G.tris.ptr;
    v.tlas_nodes = G.tlas_nodes.ptr;
    v.tlas_inst = G.tlas_inst.ptr;
    v.dlight = G.dlight.ptr;
    v.plights = G.plights.ptr;
    v.alights = G.alights.ptr;
    v.tex_info = G.tex_info.ptr;
    v.texels = G.texels.ptr;
    v.srgb_decode = G.srgb_decode.ptr;
    v.env = s->env_size ? G.env.ptr : nullptr;
    v.env_size = s->env_size;
    v.num_instances = (uint32_t)s->instances.size();
    v.has_tlas = G.tlas_node_count > 0 ? 1u : 0u;
    v.num_textures = (uint32_t)g_textures.size();
    // light slots in the order the shaders sum them: directional, points, actives
    uint32_t ns = 0;
    if (d.rgbs[3] != 0.0f) {
        v.slot_group[ns] = 0;
        v.slot_index[ns] = 0;
        ++ns;
    }
    for (uint32_t i = 0; i < KF_MAX_POINT_LIGHTS; ++i)
        if (p.rgbs[i][3] > 0.0f) {
            v.slot_group[ns] = 1;
            v.slot_index[ns] = (uint8_t)i;
            ++ns;
        }
    for (uint32_t i = 0; i < KF_MAX_ACTIVE_LIGHTS; ++i)
        if (a.front[i][3] > 0.0f) {
            v.slot_group[ns] = 2;
            v.slot_index[ns] = (uint8_t)i;
            ++ns;
        }
    v.num_slots = ns;
    r->stats.blas_nodes = G.blas_node_count;
    r->stats.tlas_nodes = G.tlas_node_count;
    r->stats.tlas_refits = G.tlas_refits;
}

// Concatenates the pools of the batch's scenes: vertex, index, material-index and
// triangle pools are copied as they are (indices are geometry-local, triangle ids too);
// geometry records, instance records, BLAS / TLAS child links and TLAS leaf entries are
// rebased by the sizes of the scenes before them.
void batch_sync(kf_renderer_s* r, const std::vector<kf_scene_s*>& scenes) {
    cudaStream_t st = r->stream;
    for (kf_scene_s* s : scenes) scene_sync_gpu(r, s);
    if (!r->batch) r->batch = std::make_unique<BatchState>();
    BatchState& B = *r->batch;
    std::vector<uint64_t> gens;
    for (kf_scene_s* s : scenes) gens.push_back(s->gpu.content_version);
    if (B.scenes == scenes && B.generations == gens) {
        // lights and slot tables are refreshed by scene_sync_gpu every call; pools are current
        return;
    }
    size_t nv = 0, ni = 0, nt = 0, ng = 0, ninst = 0, nbn = 0, ntn = 0, nti = 0;
    for (kf_scene_s* s : scenes) {
        const SceneGpu& G = s->gpu;
        nv += G.verts.count;
        ni += G.indices.count;
        nt += G.matidx.count;
        ng += s->geometries.size();
        ninst += s->instances.size();
        nbn += G.blas_node_count;
        if (G.tlas_node_count) {
            ntn += G.tlas_node_count;
            nti += G.tlas_inst.count;
        }
    }
    KF_REQUIRE(nt < (1ull << 26), KF_ERR_LIMIT, "a batch holds at most 67108863 distinct triangles");
    KF_REQUIRE(ninst < (1ull << 30), KF_ERR_LIMIT, "too many instances in one batch");
    B.verts.resize(std::max<size_t>(nv, 1), st);
    B.indices.resize(std::max<size_t>(ni, 1), st);
    B.matidx.resize(std::max<size_t>(nt, 1), st);
    // traversal stack entries hold 26-bit triangle and TLAS-leaf offsets
    KF_REQUIRE(nt < (1ull << 26) && nti < (1ull << 26), KF_ERR_LIMIT,
               "a batch holds at most 67108863 triangles and instances");
    B.tris.resize(std::max<size_t>(nt, 1), st);
    B.geom.resize(std::max<size_t>(ng, 1), st);
    B.inst.resize(std::max<size_t>(ninst, 1), st);
    B.blas_nodes.resize(std::max<size_t>(nbn, 1), st);
    B.tlas_nodes.resize(std::max<size_t>(ntn, 1), st);
    B.tlas_inst.resize(std::max<size_t>(nti, 1), st);
    B.roots.assign(scenes.size(), kNoRoot);
    size_t ov = 0, oi = 0, ot = 0, og = 0, oinst = 0, obn = 0, otn = 0, oti = 0;
    std::vector<uint4> geom;
    std::vector<InstanceRec> inst;
    std::vector<uint32_t> tinst;
    for (size_t k = 0; k < scenes.size(); ++k) {
        kf_scene_s* s = scenes[k];
        const SceneGpu& G = s->gpu;
        auto copy = [&](void* dst, const void* src, size_t bytes) {
            if (bytes) KF_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
        };
        copy(B.verts.ptr + ov, G.verts.ptr, G.verts.count * sizeof(float4));
        copy(B.indices.ptr + oi, G.indices.ptr, G.indices.count * sizeof(uint32_t));
        const size_t sct = G.matidx.count;
        copy(B.matidx.ptr + ot, G.matidx.ptr, sct * sizeof(uint32_t));
        copy(B.tris.ptr + ot, G.tris.ptr, sct * sizeof(Tri));
        // geometry records: vertex offsets count vertices (3 float4 each)
        for (size_t gi = 0; gi < s->geometries.size(); ++gi) {
            const kf_geometry_s* g = s->geometries[gi];
            const uint32_t flags = (g->opaque ? 1u : 0u) | (g->hide_render ? 2u : 0u);
            geom.push_back(make_uint4(G.vert_offset[gi] + (uint32_t)(ov / 3), G.tri_offset[gi] + (uint32_t)ot,
                                      (uint32_t)(g->indices.size() / 3), flags));
        }
        const size_t sn = s->instances.size();
        if (sn) {
            std::vector<InstanceRec> recs(sn);
            KF_CUDA_CHECK(cudaMemcpyAsync(recs.data(), G.inst.ptr, sn * sizeof(InstanceRec), cudaMemcpyDeviceToHost, st));
            KF_CUDA_CHECK(cudaStreamSynchronize(st));
            for (InstanceRec& rc : recs) {
                rc.blas_root += (uint32_t)obn;
                rc.geometry += (uint32_t)og;
                inst.push_back(rc);
            }
        }
        if (G.blas_node_count) {
            k_rebase<<<(G.blas_node_count + 127) / 128, 128, 0, st>>>(G.blas_nodes.ptr, G.blas_node_count,
                                                                      (uint32_t)obn, (uint32_t)ot, 0u,
                                                                      B.blas_nodes.ptr + obn);
            KF_CUDA_CHECK(cudaGetLastError());
        }
        if (G.tlas_node_count) {
            k_rebase<<<(G.tlas_node_count + 127) / 128, 128, 0, st>>>(G.tlas_nodes.ptr, G.tlas_node_count,
                                                                      (uint32_t)otn, (uint32_t)oti,
                                                                      (uint32_t)oinst, B.tlas_nodes.ptr + otn);
            KF_CUDA_CHECK(cudaGetLastError());
            std::vector<uint32_t> ti(G.tlas_inst.count);
            KF_CUDA_CHECK(cudaMemcpyAsync(ti.data(), G.tlas_inst.ptr, ti.size() * 4, cudaMemcpyDeviceToHost, st));
            KF_CUDA_CHECK(cudaStreamSynchronize(st));
            for (uint32_t v : ti) tinst.push_back(v + (uint32_t)oinst);
            B.roots[k] = (uint32_t)otn;
            otn += G.tlas_node_count;
            oti += ti.size();
        }
        ov += G.verts.count;
        oi += G.indices.count;
        ot += sct;
        og += s->geometries.size();
        oinst += sn;
        obn += G.blas_node_count;
    }
    if (!geom.empty()) B.geom.upload(geom.data(), geom.size(), st);
    if (!inst.empty()) B.inst.upload(inst.data(), inst.size(), st);
    if (!tinst.empty()) B.tlas_inst.upload(tinst.data(), tinst.size(), st);
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    const SceneDev& v0 = scenes.front()->gpu.view;
    SceneDev& v = B.view;
    v = v0; // materials, textures, sRGB table: process-global, identical in every scene
    v.verts = B.verts.ptr;
    v.indices = B.indices.ptr;
    v.matidx = B.matidx.ptr;
    v.geom = B.geom.ptr;
    v.inst = B.inst.ptr;
    v.blas_nodes = B.blas_nodes.ptr;
    v.tris = B.tris.ptr;
    v.tlas_nodes = B.tlas_nodes.ptr;
    v.tlas_inst = B.tlas_inst.ptr;
    v.num_instances = (uint32_t)ninst;
    v.has_tlas = 0;        // each view starts at its own root
    v.num_slots = 0;       // each view has its own light slots
    v.dlight = nullptr;
    v.plights = nullptr;
    v.alights = nullptr;
    v.env = nullptr;
    v.env_size = 0;
    B.scenes = scenes;
    B.generations = gens;
    ++B.generation;
}

} // namespace kf
