/*
 * lightgraph.hpp -- the reference's three hot-path classes for C++ callers,
 * over the C ABI of lightgraph_c.h (header only, C++17, no CUDA headers).
 *
 * The reference compiles LightGraph (src/LightGraph.h:32-153), ScatterGrid
 * (src/ScatterGrid.h:20-56) and VolumeRender (src/Renderer.h:403-448) into its
 * executable and drives them from main() in three stages:
 *   tbb::parallel_for(blocked_range(0, iter), LightGraph(...))  src/main.cc:534-538
 *   ScatterGrid::buildScatterGrid + tools::foreach(ScatterGrid)  src/main.cc:571-586
 *   VolumeRender(...).render(threaded)                           src/main.cc:111-121
 * The classes below keep those names, that call sequence and the meaning of
 * the arguments, with OpenVDB types replaced by plain arrays: grids are dense
 * boxes uploaded once into a Context, points and colours are Vec3R (double
 * triples, as the reference's gathers hold them). Failures are exceptions,
 * as the reference raises them (OPENVDB_THROW, asserts): lightgraph::Error
 * carries the lg_status and the library's message.
 *
 * Differences a caller sees:
 *  - LightGraph's body runs all the iterations of its range on the GPU at
 *    once. Call it once over every iteration whose vertices the ScatterGrid
 *    stage splats (in place of tbb::parallel_for, which would hand it
 *    sub-ranges): the splat reads the vertices of the last call.
 *  - The scatter grid lives in the Context; ScatterGrid::values copies it out.
 *  - A Context serialises its calls, and each class method here makes its
 *    C-ABI calls under the Context's own lock, so methods of one Context may
 *    be called from several threads.
 * Link with -llightgraph_gb300 -llightgraph_host.
 */
#ifndef LIGHTGRAPH_HPP_
#define LIGHTGRAPH_HPP_

#include <array>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "lightgraph_c.h"

namespace lightgraph {

using Vec3R = std::array<double, 3>;

class Error : public std::runtime_error {
public:
    Error(lg_status status, const std::string& what) : std::runtime_error(what), mStatus(status) {}
    lg_status status() const { return mStatus; }

private:
    lg_status mStatus;
};

inline void check(lg_status s, const lg_ctx* ctx, const char* call) {
    if (s == LG_OK) return;
    std::string msg = std::string(call) + " failed (status " + std::to_string(s) + ")";
    if (ctx) msg += ": " + std::string(lg_last_error(ctx));
    throw Error(s, msg);
}

/* One GPU and the scene the reference hands every class by reference: the
 * density and temperature grids (src/main.cc:486-502), the Shader, the
 * SceneSettings and the lights. */
class Context {
public:
    explicit Context(int device = 0) { check(lg_create(device, &mCtx), nullptr, "lg_create"); }
    ~Context() {
        if (mCtx) lg_destroy(mCtx);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    lg_ctx* handle() const { return mCtx; }
    std::mutex& mutex() const { return mMutex; }

    /* which: LG_GRID_DENSITY or LG_GRID_TEMPERATURE; values as lg_grid_desc
     * describes them (x fastest); storage: LG_DTYPE_F32/F16/BF16. */
    void uploadGrid(int which, const lg_grid_desc& desc, const float* values, int storage = LG_DTYPE_F32) {
        std::lock_guard<std::mutex> lk(mMutex);
        check(lg_upload_grid(mCtx, which, &desc, values, storage), mCtx, "lg_upload_grid");
    }
    void setShader(const lg_shader& shader) {
        std::lock_guard<std::mutex> lk(mMutex);
        check(lg_set_shader(mCtx, &shader), mCtx, "lg_set_shader");
    }
    void setSettings(const lg_settings& settings) {
        std::lock_guard<std::mutex> lk(mMutex);
        check(lg_set_settings(mCtx, &settings), mCtx, "lg_set_settings");
    }
    /* env_rgb (env_h x env_w x RGB) is the map of the environment lights. */
    void setLights(const std::vector<lg_light>& lights, const float* env_rgb = nullptr, int env_w = 0,
                   int env_h = 0) {
        std::lock_guard<std::mutex> lk(mMutex);
        check(lg_set_lights(mCtx, lights.data(), (int)lights.size(), env_rgb, env_w, env_h), mCtx,
              "lg_set_lights");
    }

private:
    lg_ctx* mCtx = nullptr;
    mutable std::mutex mMutex;
};

/* tbb::blocked_range<std::size_t> for the LightGraph body. */
struct Range {
    std::size_t mBegin, mEnd;
    Range(std::size_t b, std::size_t e) : mBegin(b), mEnd(e) {}
    std::size_t begin() const { return mBegin; }
    std::size_t end() const { return mEnd; }
};

/* LightGraph (src/LightGraph.h:32-153). Per iteration i of the range, the
 * body of src/LightGraph.h:158-196: scatterPoints (the reference's dart
 * throwing with iteration i's RandGen stream, src/LightGraph.h:206-274),
 * buildGraph, raymarchConnection, floydAlgo, computeLighting and
 * diffuseLight, leaving the points in pointCloudGather[i] and their diffused
 * radiance in diffusePointGather[i] (both sized by the caller to the
 * iteration count, as src/main.cc:527-528 does). */
class LightGraph {
public:
    LightGraph(Context& ctx, const lg_scatter_opts& scatter, uint32_t maxConnect,
               std::vector<std::vector<Vec3R>>& pointCloudGather,
               std::vector<std::vector<Vec3R>>& diffusePointGather)
        : mCtx(ctx),
          mScatter(scatter),
          mMaxConnect(maxConnect),
          mPointCloudGather(pointCloudGather),
          mDiffusePointGather(diffusePointGather) {}

    void operator()(const Range& r) const {
        if (r.end() <= r.begin()) return;
        if (r.end() > mPointCloudGather.size() || r.end() > mDiffusePointGather.size())
            throw Error(LG_ERR_INVALID, "LightGraph: the gathers hold fewer entries than the range's end");
        const int first = (int)r.begin(), n = (int)(r.end() - r.begin());
        lg_ctx* h = mCtx.handle();
        std::lock_guard<std::mutex> lk(mCtx.mutex());
        const size_t cap = mScatter.hard_limit;
        std::vector<float> pts((size_t)n * cap * 3), r2(n);
        std::vector<int32_t> counts(n);
        check(lg_scatter_points(h, &mScatter, first, n, pts.data(), counts.data(), r2.data()), h,
              "lg_scatter_points");
        // the iterations' points back to back, one graph each
        std::vector<int64_t> offsets(n + 1, 0);
        for (int i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + counts[i];
        std::vector<float> packed((size_t)offsets[n] * 3);
        for (int i = 0; i < n; ++i)
            for (int64_t k = 0; k < 3 * (int64_t)counts[i]; ++k)
                packed[(size_t)(3 * offsets[i] + k)] = pts[(size_t)i * cap * 3 + (size_t)k];
        check(lg_build_graphs(h, n, packed.data(), offsets.data(), r2.data(), (int)mMaxConnect, nullptr, nullptr),
              h, "lg_build_graphs");
        std::vector<float> diffuse((size_t)offsets[n] * 3);
        check(lg_solve_graphs(h, diffuse.data()), h, "lg_solve_graphs");
        for (int i = 0; i < n; ++i) {
            std::vector<Vec3R>& pc = mPointCloudGather[first + i];
            std::vector<Vec3R>& dc = mDiffusePointGather[first + i];
            pc.resize(counts[i]);
            dc.resize(counts[i]);
            for (int32_t p = 0; p < counts[i]; ++p)
                for (int c = 0; c < 3; ++c) {
                    pc[p][c] = packed[(size_t)(3 * (offsets[i] + p) + c)];
                    dc[p][c] = diffuse[(size_t)(3 * (offsets[i] + p) + c)];
                }
        }
    }

    /* points::computeVoxelSize(positions, pointsPerVoxel) as buildVdbPointGrid
     * calls it (src/LightGraph.h:713-714): the voxel size of the point index
     * the splat uses. */
    static double computeVoxelSize(const std::vector<Vec3R>& points, int pointsPerVoxel = 8) {
        std::vector<float> p(points.size() * 3);
        for (size_t i = 0; i < points.size(); ++i)
            for (int c = 0; c < 3; ++c) p[3 * i + c] = (float)points[i][c];
        return lg_point_voxel_size((int64_t)points.size(), p.data(), pointsPerVoxel);
    }

private:
    Context& mCtx;
    lg_scatter_opts mScatter;
    uint32_t mMaxConnect;
    std::vector<std::vector<Vec3R>>& mPointCloudGather;
    std::vector<std::vector<Vec3R>>& mDiffusePointGather;
};

/* ScatterGrid (src/ScatterGrid.h:20-144): buildScatterGrid makes the coarse
 * grid's topology (the density's active voxels at scatterGridResFactor,
 * dilated by one) and the splat fills it with every solved vertex of the
 * last LightGraph call, as tools::foreach(ScatterGrid) does
 * (src/main.cc:571-586). pointVoxelSize <= 0 takes computeVoxelSize of those
 * vertices. */
class ScatterGrid {
public:
    struct Values {
        int32_t dims[3] = {0, 0, 0};    // the coarse dense box
        int32_t origin[3] = {0, 0, 0};  // its first coarse voxel (index space)
        std::vector<float> rgb;         // dims[0]*dims[1]*dims[2] x RGB, x fastest (0 = inactive)
    };

    static void buildScatterGrid(Context& ctx, double pointVoxelSize = 0.0) {
        std::lock_guard<std::mutex> lk(ctx.mutex());
        check(lg_splat(ctx.handle(), pointVoxelSize), ctx.handle(), "lg_splat");
    }

    static Values values(Context& ctx) {
        std::lock_guard<std::mutex> lk(ctx.mutex());
        Values v;
        check(lg_get_scatter_grid(ctx.handle(), v.dims, v.origin, nullptr), ctx.handle(), "lg_get_scatter_grid");
        v.rgb.resize((size_t)v.dims[0] * v.dims[1] * v.dims[2] * 3);
        check(lg_get_scatter_grid(ctx.handle(), v.dims, v.origin, v.rgb.data()), ctx.handle(),
              "lg_get_scatter_grid");
        return v;
    }
};

/* Film (src/Renderer.h:68-121): width x height RGBA floats, row-major. */
struct Film {
    int width = 0, height = 0;
    std::vector<float> pixels;
};

/* VolumeRender (src/Renderer.h:403-693): render() marches every pixel and
 * antialiasing sample through the density, shading with the scatter grid,
 * the temperature ramp and the lights, into the beauty film and the direct,
 * scatter and emission AOVs (src/main.cc:80-134). The `threaded` flag is
 * kept for the reference's signature; the GPU always runs every pixel in
 * parallel. */
class VolumeRender {
public:
    VolumeRender(Context& ctx, const lg_camera& camera) : mCtx(ctx), mCamera(camera) {}

    void render(bool threaded = true) {
        (void)threaded;
        const size_t n = (size_t)mCamera.width * (size_t)mCamera.height * 4;
        for (Film* f : {&mRgba, &mDirect, &mScatter, &mEmission}) {
            f->width = mCamera.width;
            f->height = mCamera.height;
            f->pixels.assign(n, 0.f);
        }
        std::lock_guard<std::mutex> lk(mCtx.mutex());
        check(lg_render(mCtx.handle(), &mCamera, mRgba.pixels.data(), mDirect.pixels.data(),
                        mScatter.pixels.data(), mEmission.pixels.data()),
              mCtx.handle(), "lg_render");
    }

    const Film& rgba() const { return mRgba; }
    const Film& direct() const { return mDirect; }
    const Film& scatter() const { return mScatter; }
    const Film& emission() const { return mEmission; }

private:
    Context& mCtx;
    lg_camera mCamera;
    Film mRgba, mDirect, mScatter, mEmission;
};

}  // namespace lightgraph

#endif  // LIGHTGRAPH_HPP_
