// cornell_facade.cpp — renders the procedural Cornell box through the kuafu-shaped
// C++ facade (include/kuafu_gb300/kuafu.hpp), the way an application written
// against kuafu would, and writes the downloaded B8G8R8A8 frame to a file.
//
//   cornell_facade <width> <height> <spp> <frames> <out.bgra>
//
// The scene is built exactly like kuafu_gb300.scenes.cornell (same transforms in
// FP64 rounded to float), so its frame is comparable byte for byte.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kuafu_gb300/kuafu.hpp"

namespace {
struct M4 {
    double a[4][4]; // row-major [row][col]
};
M4 eye() {
    M4 m{};
    for (int i = 0; i < 4; ++i) m.a[i][i] = 1.0;
    return m;
}
M4 mul(const M4& x, const M4& y) {
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += x.a[i][k] * y.a[k][j];
            r.a[i][j] = s;
        }
    return r;
}
M4 translate(double x, double y, double z) {
    M4 m = eye();
    m.a[0][3] = x;
    m.a[1][3] = y;
    m.a[2][3] = z;
    return m;
}
M4 scale(double x, double y, double z) {
    M4 m = eye();
    m.a[0][0] = x;
    m.a[1][1] = y;
    m.a[2][2] = z;
    return m;
}
M4 rot(char axis, double deg) {
    const double r = deg * (3.141592653589793 / 180.0), c = std::cos(r), s = std::sin(r);
    M4 m = eye();
    int i = 0, j = 1;
    if (axis == 'x') { i = 1; j = 2; }
    if (axis == 'y') { i = 2; j = 0; }
    m.a[i][i] = c; m.a[i][j] = -s; m.a[j][i] = s; m.a[j][j] = c;
    return m;
}
kuafu::mat4 to_mat4(const M4& m) {
    kuafu::mat4 o(0.0f);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) o[c][r] = (float)m.a[r][c];
    return o;
}
} // namespace

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s width height spp frames out.bgra\n", argv[0]);
        return 2;
    }
    const int W = std::atoi(argv[1]), H = std::atoi(argv[2]), spp = std::atoi(argv[3]), frames = std::atoi(argv[4]);
    try {
        auto config = std::make_shared<kuafu::Config>();
        config->setPerPixelSampleRate(spp);
        config->setPathDepth(5);
        config->setRussianRoulette(false);
        config->setPresent(false);
        config->setAccumulatingFrames(true);
        kuafu::Kuafu renderer(config);
        kuafu::Scene* scene = renderer.getScene();

        auto wall = [](float r, float g, float b) {
            kuafu::NiceMaterial m;
            m.diffuseColor = kuafu::vec3(r, g, b);
            return m;
        };
        struct Item {
            std::shared_ptr<kuafu::Geometry> g;
            M4 m;
        };
        std::vector<Item> items = {
            {kuafu::createYZPlane(true, wall(0.73f, 0.73f, 0.73f)), mul(translate(1, 0, 0), rot('z', 180))},
            {kuafu::createYZPlane(true, wall(0.73f, 0.73f, 0.73f)), mul(translate(0, 0, -1), rot('y', -90))},
            {kuafu::createYZPlane(true, wall(0.73f, 0.73f, 0.73f)), mul(translate(0, 0, 1), rot('y', 90))},
            {kuafu::createYZPlane(true, wall(0.63f, 0.065f, 0.05f)), mul(translate(0, 1, 0), rot('z', -90))},
            {kuafu::createYZPlane(true, wall(0.14f, 0.45f, 0.09f)), mul(translate(0, -1, 0), rot('z', 90))},
        };
        kuafu::NiceMaterial box = wall(0.73f, 0.73f, 0.73f);
        box.roughness = 1.0f;
        items.push_back({kuafu::createCube(true, box),
                         mul(mul(translate(-0.25, -0.35, -0.7), rot('z', -17)), scale(0.3, 0.3, 0.3))});
        items.push_back({kuafu::createCube(true, box),
                         mul(mul(translate(0.35, 0.35, -0.4), rot('z', 17)), scale(0.3, 0.3, 0.6))});
        kuafu::NiceMaterial light = wall(0.0f, 0.0f, 0.0f);
        light.emission = kuafu::vec3(1.0f);
        light.emissionStrength = 15.0f;
        items.push_back({kuafu::createYZPlane(true, light),
                         mul(mul(translate(0, 0, 0.999), rot('y', 90)), scale(1.0, 0.25, 0.2))});
        for (auto& it : items) scene->submitGeometry(it.g);
        for (auto& it : items) scene->submitGeometryInstance(kuafu::instance(it.g, to_mat4(it.m)));
        scene->setClearColor(kuafu::vec4(0.0f, 0.0f, 0.0f, 1.0f));

        kuafu::Camera* cam = scene->createCamera(W, H);
        scene->setCamera(cam);
        const double t = std::tan(20.0 * (3.141592653589793 / 180.0));
        cam->setPosition(kuafu::vec3((float)(-1.0 - 1.0 / t - 0.02), 0.0f, 0.0f));
        cam->setFront(kuafu::vec3(1.0f, 0.0f, 0.0f));
        cam->setUp(kuafu::vec3(0.0f, 0.0f, 1.0f));
        const double fy = (H / 2.0) / t;
        cam->setFullPerspective((float)W, (float)H, (float)fy, (float)fy, (float)(W / 2.0), (float)(H / 2.0), 0.0f);

        for (int f = 0; f < frames; ++f) renderer.run();
        std::vector<uint8_t> frame = renderer.downloadLatestFrame(cam);
        FILE* fp = std::fopen(argv[5], "wb");
        if (!fp) return 3;
        std::fwrite(frame.data(), 1, frame.size(), fp);
        std::fclose(fp);
        std::printf("wrote %zu bytes\n", frame.size());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
