// Drives the C++ class layer of include/lightgraph.hpp (tests/test_cpp_classes.py
// builds and runs it).
//   nodevice : constructing a Context on a machine without a GPU throws
//              lightgraph::Error with LG_ERR_NODEVICE; prints "error <status>"
//   frame    : a small frame through the classes -- two dart-thrown LightGraph
//              iterations in a 32^3 sphere-fBm volume, the scatter grid, a
//              24 x 24 render -- and the same frame through the lg_* calls
//              made directly; prints "match ..." when every gather, scatter
//              grid value and film agrees bit for bit
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lightgraph.hpp"
#include "lightgraph_scene.h"

namespace {

struct Scene {
    std::vector<float> density;
    lg_grid_desc grid{};
    lg_shader shader{};
    lg_settings settings{};
    std::vector<lg_light> lights;
    lg_camera camera{};
    lg_scatter_opts scatter{};
};

Scene make_scene() {
    Scene s;
    const int res = 32;
    const double voxel = 1.28 / res;
    s.density.resize((size_t)res * res * res);
    lgs_volume(LGS_VOLUME_SPHERE_FBM, res, 4, 0, 1.0, nullptr, s.density.data());
    for (int a = 0; a < 3; ++a) {
        s.grid.dims[a] = res;
        s.grid.origin[a] = -res / 2;
        s.grid.world_origin[a] = 0.0;
    }
    s.grid.voxel_size = voxel;
    lg_shader_default(&s.shader);
    const double k = 10.0 * voxel;  // extinction 10 per world unit
    const double absorption[3] = {0.1 * k, 0.1 * k, 0.1 * k}, scattering[3] = {0.9 * k, 0.9 * k, 0.9 * k},
                 color[3] = {1.0, 1.0, 1.0};
    lg_shader_set_coefficients(&s.shader, absorption, scattering, color);
    lg_settings_default(&s.settings);
    s.settings.iter = 2;
    lg_light light;
    if (lg_parse_light("dir:0:1,1,1:1.0:-35,25,0", &light) != LG_OK) std::printf("light parse failed\n");
    s.lights.push_back(light);
    lg_camera_default(&s.camera);
    s.camera.width = 24;
    s.camera.height = 24;
    s.camera.samples = 1;
    s.camera.translate[2] = 2.2;
    lg_scatter_opts_default(&s.scatter);
    return s;
}

struct Result {
    std::vector<float> points, diffuse, grid, films;
};

Result through_classes(const Scene& s) {
    lightgraph::Context ctx(0);
    ctx.uploadGrid(LG_GRID_DENSITY, s.grid, s.density.data());
    ctx.setShader(s.shader);
    ctx.setSettings(s.settings);
    ctx.setLights(s.lights);
    std::vector<std::vector<lightgraph::Vec3R>> pointCloudGather(s.settings.iter), diffusePointGather(s.settings.iter);
    lightgraph::LightGraph lg(ctx, s.scatter, 12, pointCloudGather, diffusePointGather);
    lg(lightgraph::Range(0, (size_t)s.settings.iter));
    lightgraph::ScatterGrid::buildScatterGrid(ctx);
    const lightgraph::ScatterGrid::Values sg = lightgraph::ScatterGrid::values(ctx);
    lightgraph::VolumeRender renderer(ctx, s.camera);
    renderer.render(true);
    Result r;
    for (int i = 0; i < s.settings.iter; ++i)
        for (size_t p = 0; p < pointCloudGather[i].size(); ++p)
            for (int c = 0; c < 3; ++c) {
                r.points.push_back((float)pointCloudGather[i][p][c]);
                r.diffuse.push_back((float)diffusePointGather[i][p][c]);
            }
    r.grid = sg.rgb;
    for (const lightgraph::Film* f : {&renderer.rgba(), &renderer.direct(), &renderer.scatter(), &renderer.emission()})
        r.films.insert(r.films.end(), f->pixels.begin(), f->pixels.end());
    return r;
}

#define CALL(x)                                                       \
    do {                                                              \
        const lg_status st_ = (x);                                    \
        if (st_ != LG_OK) {                                           \
            std::printf("%s failed: %s\n", #x, lg_last_error(h));     \
            lg_destroy(h);                                            \
            return false;                                             \
        }                                                             \
    } while (0)

bool through_c_abi(const Scene& s, Result& r) {
    lg_ctx* h = nullptr;
    if (lg_create(0, &h) != LG_OK) return false;
    CALL(lg_upload_grid(h, LG_GRID_DENSITY, &s.grid, s.density.data(), LG_DTYPE_F32));
    CALL(lg_set_shader(h, &s.shader));
    CALL(lg_set_settings(h, &s.settings));
    CALL(lg_set_lights(h, s.lights.data(), (int)s.lights.size(), nullptr, 0, 0));
    const int n = s.settings.iter;
    const size_t cap = s.scatter.hard_limit;
    std::vector<float> pts((size_t)n * cap * 3), r2(n);
    std::vector<int32_t> counts(n);
    CALL(lg_scatter_points(h, &s.scatter, 0, n, pts.data(), counts.data(), r2.data()));
    std::vector<int64_t> offsets(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        offsets[i + 1] = offsets[i] + counts[i];
        r.points.insert(r.points.end(), pts.begin() + (long)(i * cap * 3), pts.begin() + (long)(i * cap * 3 + 3 * counts[i]));
    }
    CALL(lg_build_graphs(h, n, r.points.data(), offsets.data(), r2.data(), 12, nullptr, nullptr));
    r.diffuse.resize(r.points.size());
    CALL(lg_solve_graphs(h, r.diffuse.data()));
    CALL(lg_splat(h, 0.0));
    int32_t dims[3], origin[3];
    CALL(lg_get_scatter_grid(h, dims, origin, nullptr));
    r.grid.resize((size_t)dims[0] * dims[1] * dims[2] * 3);
    CALL(lg_get_scatter_grid(h, dims, origin, r.grid.data()));
    const size_t px = (size_t)s.camera.width * s.camera.height * 4;
    r.films.resize(4 * px);
    CALL(lg_render(h, &s.camera, r.films.data(), r.films.data() + px, r.films.data() + 2 * px,
                   r.films.data() + 3 * px));
    lg_destroy(h);
    return true;
}

bool same_bits(const std::vector<float>& a, const std::vector<float>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), sizeof(float) * a.size()) == 0;
}

}  // namespace

int main(int argc, char** argv) {
    const char* mode = argc > 1 ? argv[1] : "frame";
    if (std::strcmp(mode, "nodevice") == 0) {
        try {
            lightgraph::Context ctx(0);
            std::printf("a device is present\n");
            return 3;
        } catch (const lightgraph::Error& e) {
            std::printf("error %d: %s\n", e.status(), e.what());
            return e.status() == LG_ERR_NODEVICE ? 0 : 4;
        }
    }
    const Scene s = make_scene();
    Result a, b;
    try {
        a = through_classes(s);
    } catch (const lightgraph::Error& e) {
        std::printf("classes: %s\n", e.what());
        return 2;
    }
    if (!through_c_abi(s, b)) return 2;
    const size_t px = (size_t)s.camera.width * s.camera.height * 4;
    float alpha_max = 0.f;
    bool alpha_ok = true;
    for (size_t p = 3; p < px; p += 4) {
        alpha_ok = alpha_ok && a.films[p] >= 0.f && a.films[p] <= 1.f;
        alpha_max = std::fmax(alpha_max, a.films[p]);
    }
    float grid_max = 0.f;
    for (float v : a.grid) grid_max = std::fmax(grid_max, v);
    const bool ok = same_bits(a.points, b.points) && same_bits(a.diffuse, b.diffuse) && same_bits(a.grid, b.grid) &&
                    same_bits(a.films, b.films) && !a.points.empty() && alpha_ok && alpha_max > 0.f &&
                    grid_max > 0.f;
    std::printf("%s points=%zu grid=%zu alpha_max=%g grid_max=%g\n", ok ? "match" : "mismatch", a.points.size() / 3,
                a.grid.size() / 3, alpha_max, grid_max);
    return ok ? 0 : 1;
}
