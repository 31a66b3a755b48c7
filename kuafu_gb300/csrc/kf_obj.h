// kf_obj.h — Wavefront OBJ / MTL loading (kf_obj.cpp).
#pragma once

#include <string>
#include <vector>

#include "../../include/kf.h"

namespace kf {

// One geometry per material used by the file (kuafu's loadScene after assimp's
// PreTransformVertices): triangle list over per-corner vertices, and its material.
struct ObjMesh {
    std::vector<kf_vertex> vertices;
    std::vector<uint32_t> indices;
    kf_material material;
    std::string material_name;
};

void load_obj(const std::string& path, std::vector<ObjMesh>& out);

} // namespace kf
