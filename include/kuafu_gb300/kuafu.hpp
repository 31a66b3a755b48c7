// kuafu.hpp — header-only C++ facade re-creating kuafu's public API
// (include/kuafu.hpp, include/core/{config,scene,camera,geometry,light}.hpp of
// jetd1/kuafu) on top of libkf's C-ABI (include/kf.h). Code written against
// kuafu compiles against this header with the same class and method names;
// errors come back as std::runtime_error, as kuafu's KF_ASSERT throws.
//
// Math types: kuafu uses glm. Define KF_WITH_GLM before including this header to
// use glm::vec2/vec3/vec4/mat4 directly; otherwise small layout-compatible
// stand-ins (column-major mat4) are provided in namespace kuafu.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "../kf.h"

#ifdef KF_WITH_GLM
#include <glm/glm.hpp>
namespace kuafu {
using vec2 = glm::vec2;
using vec3 = glm::vec3;
using vec4 = glm::vec4;
using mat4 = glm::mat4;
} // namespace kuafu
#else
namespace kuafu {
struct vec2 {
    float x = 0, y = 0;
};
struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float a) : x(a), y(a), z(a) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct vec4 {
    float x = 0, y = 0, z = 0, w = 0;
    vec4() = default;
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
};
// column-major like glm::mat4: m[col][row]
struct mat4 {
    float m[4][4];
    mat4() : mat4(1.0f) {}
    explicit mat4(float d) {
        std::memset(m, 0, sizeof(m));
        for (int i = 0; i < 4; ++i) m[i][i] = d;
    }
    float* operator[](int c) { return m[c]; }
    const float* operator[](int c) const { return m[c]; }
};
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r(0.0f);
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr)
            r[c][rr] = a[0][rr] * b[c][0] + a[1][rr] * b[c][1] + a[2][rr] * b[c][2] + a[3][rr] * b[c][3];
    return r;
}
} // namespace kuafu
#endif

namespace kuafu {

namespace detail {
inline void check(int status) {
    if (status != KF_OK) throw std::runtime_error(kf_last_error());
}
inline void to_cm(const mat4& m, float out[16]) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}
inline mat4 from_cm(const float in[16]) {
    mat4 m(0.0f);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[c][r] = in[c * 4 + r];
    return m;
}
inline void f3(const vec3& v, float o[3]) {
    o[0] = v[0];
    o[1] = v[1];
    o[2] = v[2];
}
} // namespace detail

// include/core/context/vertex.hpp:28-34
struct Vertex {
    vec3 pos;
    vec3 normal;
    vec3 color;
    vec2 texCoord;
    float padding0 = 0.0f;
};
static_assert(sizeof(Vertex) == sizeof(kf_vertex), "Vertex must match kf_vertex");

// include/core/geometry.hpp:11-30
struct NiceMaterial {
    vec3 diffuseColor = vec3(1.0f);
    float alpha = 1.0f;
    std::string diffuseTexPath, metallicTexPath, roughnessTexPath, transmissionTexPath;
    float metallic = 0.0f;
    float specular = 0.5f;
    float roughness = 0.5f;
    float ior = 1.4f;
    float transmission = 0.0f;
    vec3 emission = vec3(1.0f);
    float emissionStrength = 0.0f;
    // GB300 addition: texture ids from kf_texture_create (kuafu loads files by path)
    int diffuseTex = -1, metallicTex = -1, roughnessTex = -1, transmissionTex = -1;

    kf_material to_c() const {
        kf_material m;
        kf_material_init(&m);
        detail::f3(diffuseColor, m.diffuse_color);
        m.alpha = alpha;
        m.metallic = metallic;
        m.specular = specular;
        m.roughness = roughness;
        m.ior = ior;
        m.transmission = transmission;
        detail::f3(emission, m.emission);
        m.emission_strength = emissionStrength;
        m.diffuse_tex = diffuseTex;
        m.metallic_tex = metallicTex;
        m.roughness_tex = roughnessTex;
        m.transmission_tex = transmissionTex;
        return m;
    }
};

// include/core/geometry.hpp:32-46. The device copy is created when the geometry is
// first submitted; edit the vectors before that (or call markGeometriesChanged).
struct Geometry {
    std::vector<Vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<uint32_t> matIndex;
    std::string path;
    bool initialized = false;
    bool dynamic = false;
    bool isOpaque = true;
    bool hideRender = false;

    void setMaterial(const NiceMaterial& material) { // geometry.cpp:241-249
        isOpaque = material.alpha >= 1.0f;
        const kf_material m = material.to_c();
        uint32_t idx = 0;
        detail::check(kf_material_add(&m, &idx));
        for (auto& it : matIndex) it = idx;
        handle_.reset();
    }
    void recalculateNormals() { // geometry.cpp:268-295
        kf_geometry g = handle();
        detail::check(kf_geometry_recalculate_normals(g));
        detail::check(kf_geometry_get_data(g, reinterpret_cast<kf_vertex*>(vertices.data()), nullptr, nullptr));
    }

    kf_geometry handle() {
        if (!handle_) {
            kf_geometry g = nullptr;
            detail::check(kf_geometry_create(reinterpret_cast<const kf_vertex*>(vertices.data()),
                                             (uint32_t)vertices.size(), indices.data(), (uint32_t)indices.size(),
                                             matIndex.data(), (uint32_t)matIndex.size(), &g));
            detail::check(kf_geometry_set_flags(g, isOpaque, hideRender, dynamic));
            pushed_ = flags();
            handle_.reset(g, [](kf_geometry p) { kf_geometry_release(p); });
            initialized = true;
        }
        return handle_.get();
    }
    // isOpaque / hideRender / dynamic edited after submission reach the next frame, as in
    // kuafu, which reads them when it rebuilds the TLAS every frame (rt.cpp:156)
    void pushFlags() {
        if (handle_ && flags() != pushed_) {
            detail::check(kf_geometry_set_flags(handle_.get(), isOpaque, hideRender, dynamic));
            pushed_ = flags();
        }
    }
    void adopt(kf_geometry g) {
        handle_.reset(g, [](kf_geometry p) { kf_geometry_release(p); });
        uint32_t nv = 0, ni = 0;
        detail::check(kf_geometry_get_info(g, &nv, &ni));
        vertices.resize(nv);
        indices.resize(ni);
        matIndex.resize(ni);
        detail::check(kf_geometry_get_data(g, reinterpret_cast<kf_vertex*>(vertices.data()), indices.data(),
                                           matIndex.data()));
        for (size_t i = ni / 3; i < matIndex.size(); ++i) matIndex[i] = matIndex[0];
    }

  private:
    int flags() const { return (isOpaque ? 1 : 0) | (hideRender ? 2 : 0) | (dynamic ? 4 : 0); }
    std::shared_ptr<struct kf_geometry_s> handle_;
    int pushed_ = -1;
};

// include/core/geometry.hpp:48-54
struct GeometryInstance {
    void setTransform(const mat4& t) {
        transform = t;
        if (handle) {
            float m[16];
            detail::to_cm(t, m);
            detail::check(kf_instance_set_transform(handle, m));
        }
    }
    mat4 transform = mat4(1.0f);
    int geometryIndex = -1;
    std::shared_ptr<Geometry> geometry = nullptr;
    kf_instance handle = nullptr; // set when submitted to a scene
};

inline std::shared_ptr<GeometryInstance> instance(const std::shared_ptr<Geometry>& geometry,
                                                  const mat4& transform = mat4(1.0f)) {
    auto r = std::make_shared<GeometryInstance>();
    r->geometry = geometry;
    r->transform = transform;
    return r;
}

namespace detail {
inline std::shared_ptr<Geometry> builtin(int kind, float p0, float p1, bool dynamic, const NiceMaterial& mat) {
    const kf_material m = mat.to_c();
    kf_geometry g = nullptr;
    detail::check(kf_geometry_create_builtin(kind, p0, p1, &m, &g));
    auto r = std::make_shared<Geometry>();
    r->adopt(g);
    r->dynamic = dynamic;
    r->isOpaque = mat.alpha >= 1.0f;
    return r;
}
} // namespace detail

// geometry.cpp:297-537
inline std::shared_ptr<Geometry> createYZPlane(bool dynamic = true, NiceMaterial mat = {}) {
    return detail::builtin(KF_MESH_YZ_PLANE, 0, 0, dynamic, mat);
}
inline std::shared_ptr<Geometry> createCube(bool dynamic = true, NiceMaterial mat = {}) {
    return detail::builtin(KF_MESH_CUBE, 0, 0, dynamic, mat);
}
inline std::shared_ptr<Geometry> createSphere(bool dynamic = true, NiceMaterial mat = {}) {
    return detail::builtin(KF_MESH_SPHERE, 0, 0, dynamic, mat);
}
inline std::shared_ptr<Geometry> createCapsule(float halfHeight = 1., float radius = 1., bool dynamic = true,
                                               NiceMaterial mat = {}) {
    return detail::builtin(KF_MESH_CAPSULE, halfHeight, radius, dynamic, mat);
}

// loadScene / loadObj (geometry.hpp:56-57): Wavefront OBJ + MTL
inline std::vector<std::shared_ptr<Geometry>> loadScene(std::string_view fname, bool dynamic) {
    const std::string p(fname);
    uint32_t n = 0;
    detail::check(kf_load_scene(p.c_str(), dynamic ? 1 : 0, nullptr, 0, &n));
    std::vector<kf_geometry> hs(n);
    detail::check(kf_load_scene(p.c_str(), dynamic ? 1 : 0, hs.data(), n, &n));
    std::vector<std::shared_ptr<Geometry>> out;
    for (kf_geometry h : hs) {
        auto g = std::make_shared<Geometry>();
        g->adopt(h);
        g->path = p;
        g->dynamic = dynamic;
        if (!g->matIndex.empty()) { // geometry.cpp:226: opaque iff the material's alpha is 1
            kf_material m{};
            detail::check(kf_material_get(g->matIndex.front(), &m));
            g->isOpaque = m.alpha >= 1.0f;
        }
        out.push_back(std::move(g));
    }
    return out;
}
inline std::shared_ptr<Geometry> loadObj(std::string_view path, bool dynamic = false) {
    auto scene = loadScene(path, dynamic);
    if (scene.size() != 1) throw std::runtime_error("complex scene! use loadScene");
    return scene.front();
}

// include/core/light.hpp:9-39
struct DirectionalLight {
    vec3 direction = {0, 0, -1};
    vec3 color = {1, 1, 1};
    float strength = 0.0f;
    float softness = 0.0f;
};
struct PointLight {
    vec3 position = {0, 0, 0};
    vec3 color = {1, 1, 1};
    float radius = 1;
    float strength = 0.0f;
};
struct ActiveLight {
    mat4 viewMat{};
    vec3 color = {1, 1, 1};
    float fov = 0.0f;
    float strength = 0.0f;
    float softness = 0.0f;
    std::string texPath;
    int texID = -1;
};

// include/core/config.hpp:35-177
class Config {
  public:
    Config() { kf_config_init(&c_); }
    void setPathDepth(uint32_t d) { c_.path_depth = d; }
    uint32_t getPathDepth() const { return c_.path_depth; }
    uint32_t getMaxPathDepth() const { return c_.max_path_depth; }
    void setRussianRoulette(bool f) { c_.russian_roulette = f; }
    bool getRussianRoulette() const { return c_.russian_roulette; }
    void setRussianRouletteMinBounces(uint32_t n) { c_.rr_min_bounces = n; }
    uint32_t getRussianRouletteMinBounces() const { return c_.rr_min_bounces; }
    void setNextEventEstimation(bool f) { c_.nee = f; }
    bool getNextEventEstimation() const { return c_.nee; }
    void setNextEventEstimationMinBounces(uint32_t n) { c_.nee_min_bounces = n; }
    void setAssetsPath(std::string_view p) { assets_ = std::string(p); }
    std::string_view getAssetsPath() const { return assets_; }
    void setAutomaticPipelineRefresh(bool) {}
    void setGeometryLimit(size_t n) { c_.max_geometries = (uint32_t)n; }
    void setGeometryInstanceLimit(uint32_t n) { c_.max_instances = n; }
    void setTextureLimit(size_t n) { c_.max_textures = (uint32_t)n; }
    void setMaterialLimit(size_t n) { c_.max_materials = (uint32_t)n; }
    void setPerPixelSampleRate(uint32_t s) { c_.spp = s; }
    uint32_t getPerPixelSampleRate() const { return c_.spp; }
    void setUseDenoiser(bool f = true) { c_.use_denoiser = f; }
    bool isUsingDenoiser() const { return c_.use_denoiser; }
    void setAccumulatingFrames(bool f) { c_.accumulate_frames = f; }
    bool isAccumulatingFrames() const { return c_.accumulate_frames; }
    void setPresent(bool p) { c_.present = p; }
    bool getPresent() const { return c_.present; }
    void setInitialWidth(int w) { c_.initial_width = w; }
    void setInitialHeight(int h) { c_.initial_height = h; }
    // GB300 additions
    void setSeed(uint32_t s) { c_.seed = s; }
    kf_config& raw() { return c_; }
    const kf_config& raw() const { return c_; }

  private:
    kf_config c_;
    std::string assets_;
};

// include/core/camera.hpp:40-174
class Camera {
  public:
    explicit Camera(kf_camera c) : c_(c) {}
    void setPosition(const vec3& p) { float v[3]; detail::f3(p, v); detail::check(kf_camera_set_position(c_, v)); }
    void setFront(const vec3& p) { float v[3]; detail::f3(p, v); detail::check(kf_camera_set_front(c_, v)); }
    void setUp(const vec3& p) { float v[3]; detail::f3(p, v); detail::check(kf_camera_set_up(c_, v)); }
    void setPose(const mat4& pose) { float m[16]; detail::to_cm(pose, m); detail::check(kf_camera_set_pose(c_, m)); }
    mat4 getPose() const { float m[16]; detail::check(kf_camera_get_pose(c_, m)); return detail::from_cm(m); }
    void setFullPerspective(float w, float h, float fx, float fy, float cx, float cy, float skew) {
        detail::check(kf_camera_set_full_perspective(c_, w, h, fx, fy, cx, cy, skew));
    }
    void setSize(int w, int h) { detail::check(kf_camera_set_size(c_, w, h)); }
    void resetView() { detail::check(kf_camera_reset_view(c_)); }
    int getWidth() const { int w, h; detail::check(kf_camera_get_size(c_, &w, &h)); return w; }
    int getHeight() const { int w, h; detail::check(kf_camera_get_size(c_, &w, &h)); return h; }
    mat4 getViewMatrix() const { kf_camera_ubo u; detail::check(kf_camera_get_ubo(c_, &u)); return detail::from_cm(u.view); }
    mat4 getProjectionMatrix() const { kf_camera_ubo u; detail::check(kf_camera_get_ubo(c_, &u)); return detail::from_cm(u.proj); }
    kf_camera raw() const { return c_; }

  private:
    kf_camera c_;
};

class Kuafu;

// include/core/scene.hpp:40-295
class Scene {
  public:
    Scene(kf_scene s) : s_(s) {}
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    const std::vector<std::shared_ptr<Geometry>>& getGeometries() const { return geometries_; }
    const std::vector<std::shared_ptr<GeometryInstance>>& getGeometryInstances() const { return instances_; }
    std::shared_ptr<GeometryInstance> getGeometryInstance(size_t index) const {
        if (index < instances_.size()) return instances_[index];
        throw std::runtime_error("Geometry Instances out of bound.");
    }
    void submitGeometry(std::shared_ptr<Geometry> g) {
        detail::check(kf_scene_submit_geometry(s_, g->handle()));
        geometries_.push_back(std::move(g));
    }
    void submitGeometry(const Geometry& g) { submitGeometry(std::make_shared<Geometry>(g)); }
    void setGeometries(const std::vector<std::shared_ptr<Geometry>>& gs) {
        clearGeometries();
        for (auto& g : gs) submitGeometry(g);
    }
    void removeGeometry(std::shared_ptr<Geometry>) { throw std::runtime_error("Not implemented!"); }
    void removeGeometry(uint32_t) { throw std::runtime_error("Not implemented!"); }
    void clearGeometries() {
        detail::check(kf_scene_clear_geometries(s_));
        geometries_.clear();
        instances_.clear();
    }
    void submitGeometryInstance(std::shared_ptr<GeometryInstance> inst) {
        auto it = std::find(geometries_.begin(), geometries_.end(), inst->geometry);
        if (it == geometries_.end()) throw std::runtime_error("Geometry not submitted!");
        inst->geometryIndex = (int)(it - geometries_.begin());
        float m[16];
        detail::to_cm(inst->transform, m);
        kf_instance h = nullptr;
        detail::check(kf_scene_submit_instance(s_, inst->geometry->handle(), m, &h));
        inst->handle = h;
        instances_.push_back(std::move(inst));
    }
    void submitGeometryInstance(const GeometryInstance& inst) {
        submitGeometryInstance(std::make_shared<GeometryInstance>(inst));
    }
    void setGeometryInstances(const std::vector<std::shared_ptr<GeometryInstance>>& insts) {
        clearGeometryInstances();
        for (auto& i : insts) submitGeometryInstance(i);
    }
    void removeGeometryInstance(const std::shared_ptr<GeometryInstance>& inst) {
        detail::check(kf_scene_remove_instance(s_, inst->handle));
        instances_.erase(std::remove(instances_.begin(), instances_.end(), inst), instances_.end());
        inst->handle = nullptr;
    }
    void removeGeometryInstances(const std::vector<std::shared_ptr<GeometryInstance>>& insts) {
        for (auto& i : insts) removeGeometryInstance(i);
    }
    void clearGeometryInstances() {
        detail::check(kf_scene_clear_instances(s_));
        for (auto& i : instances_) i->handle = nullptr;
        instances_.clear();
    }
    void setClearColor(const vec4& c) {
        const float v[4] = {c.x, c.y, c.z, c.w};
        detail::check(kf_scene_set_clear_color(s_, v));
    }
    vec4 getClearColor() const {
        float v[4];
        detail::check(kf_scene_get_clear_color(s_, v));
        return vec4(v[0], v[1], v[2], v[3]);
    }
    std::shared_ptr<Geometry> findGeometry(std::string_view path) const {
        for (auto& g : geometries_)
            if (g->path == path) return g;
        return nullptr;
    }
    // Scene::setEnvironmentMap (scene.cpp:182-186): a KTX 1.1 cube map file
    void setEnvironmentMap(std::string_view path) {
        const std::string p(path);
        detail::check(kf_scene_set_environment_map_file(s_, p.c_str()));
    }
    void removeEnvironmentMap() { detail::check(kf_scene_remove_environment_map(s_)); }
    Camera* createCamera(int w, int h) {
        kf_camera c = nullptr;
        detail::check(kf_scene_create_camera(s_, w, h, &c));
        cameras_.push_back(std::make_unique<Camera>(c));
        return cameras_.back().get();
    }
    void removeCamera(Camera* cam) {
        detail::check(kf_scene_remove_camera(s_, cam->raw()));
        cameras_.erase(std::remove_if(cameras_.begin(), cameras_.end(), [&](auto& p) { return p.get() == cam; }),
                       cameras_.end());
    }
    void setCamera(Camera* cam) { detail::check(kf_scene_set_camera(s_, cam->raw())); }
    Camera* getCamera() {
        kf_camera c = nullptr;
        detail::check(kf_scene_get_camera(s_, &c));
        for (auto& p : cameras_)
            if (p->raw() == c) return p.get();
        if (!c) return nullptr;
        cameras_.push_back(std::make_unique<Camera>(c));
        return cameras_.back().get();
    }
    size_t getGeometryInstanceCount() const { return geometries_.size(); }
    void markGeometriesChanged() { detail::check(kf_scene_mark_geometries_changed(s_)); }
    void markGeometryInstancesChanged() { detail::check(kf_scene_mark_instances_changed(s_)); }

    void setDirectionalLight(std::shared_ptr<DirectionalLight> l) { dlight_ = std::move(l); }
    void removeDirectionalLight() {
        dlight_ = nullptr;
        detail::check(kf_scene_remove_directional_light(s_));
    }
    void addPointLight(const std::shared_ptr<PointLight>& l) {
        if (plights_.size() >= KF_MAX_POINT_LIGHTS) return; // kuafu warns and drops it
        kf_point_light p = to_c(*l);
        kf_light h = nullptr;
        detail::check(kf_scene_add_point_light(s_, &p, &h));
        plights_.push_back({l, h});
    }
    void removePointLight(const std::shared_ptr<PointLight>& l) {
        for (auto it = plights_.begin(); it != plights_.end(); ++it)
            if (it->first == l) {
                detail::check(kf_scene_remove_light(s_, it->second));
                plights_.erase(it);
                return;
            }
    }
    void addActiveLight(const std::shared_ptr<ActiveLight>& l) {
        if (alights_.size() >= KF_MAX_ACTIVE_LIGHTS) return;
        kf_active_light a = to_c(*l);
        kf_light h = nullptr;
        detail::check(kf_scene_add_active_light(s_, &a, &h));
        alights_.push_back({l, h});
    }
    void removeActiveLight(const std::shared_ptr<ActiveLight>& l) {
        for (auto it = alights_.begin(); it != alights_.end(); ++it)
            if (it->first == l) {
                detail::check(kf_scene_remove_light(s_, it->second));
                alights_.erase(it);
                return;
            }
    }

    void pushGeometryFlags() {
        for (auto& g : geometries_) g->pushFlags();
    }
    // kuafu re-reads the light objects every frame (uploadLightBuffers); so does the facade.
    void pushLights() {
        if (dlight_) {
            kf_directional_light d;
            detail::f3(dlight_->direction, d.direction);
            detail::f3(dlight_->color, d.color);
            d.strength = dlight_->strength;
            d.softness = dlight_->softness;
            detail::check(kf_scene_set_directional_light(s_, &d));
        }
        for (auto& p : plights_) {
            kf_point_light c = to_c(*p.first);
            detail::check(kf_light_update_point(p.second, &c));
        }
        for (auto& a : alights_) {
            kf_active_light c = to_c(*a.first);
            detail::check(kf_light_update_active(a.second, &c));
        }
    }
    kf_scene raw() const { return s_; }

  private:
    static kf_point_light to_c(const PointLight& l) {
        kf_point_light p;
        detail::f3(l.position, p.position);
        detail::f3(l.color, p.color);
        p.radius = l.radius;
        p.strength = l.strength;
        return p;
    }
    static kf_active_light to_c(const ActiveLight& l) {
        kf_active_light a;
        detail::to_cm(l.viewMat, a.view);
        detail::f3(l.color, a.color);
        a.fov = l.fov;
        a.strength = l.strength;
        a.softness = l.softness;
        a.tex_id = l.texID;
        return a;
    }
    kf_scene s_;
    std::vector<std::shared_ptr<Geometry>> geometries_;
    std::vector<std::shared_ptr<GeometryInstance>> instances_;
    std::vector<std::unique_ptr<Camera>> cameras_;
    std::shared_ptr<DirectionalLight> dlight_;
    std::vector<std::pair<std::shared_ptr<PointLight>, kf_light>> plights_;
    std::vector<std::pair<std::shared_ptr<ActiveLight>, kf_light>> alights_;
};

// include/kuafu.hpp:31-93
class Kuafu {
  public:
    explicit Kuafu(std::shared_ptr<Config> config = nullptr) {
        cfg_ = config ? std::make_shared<Config>(*config) : std::make_shared<Config>();
        detail::check(kf_renderer_create(&cfg_->raw(), &r_));
        kf_scene s = nullptr;
        detail::check(kf_renderer_get_scene(r_, &s));
        scenes_.push_back(std::make_unique<Scene>(s));
        current_ = scenes_.back().get();
    }
    ~Kuafu() {
        if (r_) kf_renderer_destroy(r_);
    }
    Kuafu(const Kuafu&) = delete;
    Kuafu& operator=(const Kuafu&) = delete;

    void run() {
        current_->pushGeometryFlags();
        current_->pushLights();
        detail::check(kf_renderer_run(r_));
    }
    bool isRunning() const {
        int v = 0;
        detail::check(kf_renderer_is_running(r_, &v));
        return v != 0;
    }
    std::vector<uint8_t> downloadLatestFrame(Camera* cam) {
        std::vector<uint8_t> out((size_t)cam->getWidth() * cam->getHeight() * 4);
        detail::check(kf_renderer_download_latest_frame(r_, cam->raw(), out.data(), out.size()));
        return out;
    }
    Config& getConfig() { return *cfg_; }
    void applyConfig() { detail::check(kf_renderer_set_config(r_, &cfg_->raw())); }
    Scene* getScene() { return current_; }
    Scene* createScene() {
        kf_scene s = nullptr;
        detail::check(kf_renderer_create_scene(r_, &s));
        scenes_.push_back(std::make_unique<Scene>(s));
        return scenes_.back().get();
    }
    void setScene(Scene* scene) {
        if (!scene) throw std::runtime_error("Trying to set an invalid scene!");
        detail::check(kf_renderer_set_scene(r_, scene->raw()));
        current_ = scene;
    }
    void removeScene(Scene* scene) {
        if (!scene) throw std::runtime_error("Trying to remove an invalid scene!");
        detail::check(kf_renderer_remove_scene(r_, scene->raw()));
        if (current_ == scene) current_ = nullptr;
        scenes_.erase(std::remove_if(scenes_.begin(), scenes_.end(), [&](auto& p) { return p.get() == scene; }),
                      scenes_.end());
    }
    kf_renderer raw() const { return r_; }

  private:
    std::shared_ptr<Config> cfg_;
    kf_renderer r_ = nullptr;
    std::vector<std::unique_ptr<Scene>> scenes_;
    Scene* current_ = nullptr;
};

} // namespace kuafu
