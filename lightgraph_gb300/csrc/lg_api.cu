// C ABI of the LightGraph path (include/lightgraph_c.h): context, grid upload,
// scene state and the stage entry points that replace the reference's
// LightGraph / ScatterGrid / VolumeRender member functions.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "lg_ctx.h"
#include "lg_mt.h"

namespace lg {
std::atomic<uint64_t> g_launch_counter{0};
std::atomic<uint64_t> g_alloc_epoch{0};
}

using namespace lg;

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

lg_status Ctx::fail(lg_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return s;
}

lg_status Ctx::cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LG_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(LG_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(LG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                                         \
    do {                                                       \
        const lg_status _s = ctx->cuda((expr), (what));        \
        if (_s != LG_OK) return _s;                            \
    } while (0)

#define GUARD(ctx)                                             \
    if (!(ctx)) return LG_ERR_INVALID;                         \
    std::lock_guard<std::mutex> _lock((ctx)->mu);              \
    {                                                          \
        const cudaError_t _e = cudaSetDevice((ctx)->device);   \
        if (_e != cudaSuccess) return (ctx)->cuda(_e, "cudaSetDevice"); \
    }

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

static int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

// Optical depth where sum_c exp(-2 a_c tau) first drops below cutoff (the
// reference's sTrans.lengthSqr() < cutoff, src/LightGraph.h:396).
static float dropout_depth(const double a[3], double cutoff) {
    auto f = [&](double t) {
        double s = 0;
        for (int c = 0; c < 3; ++c) s += std::exp(-2.0 * a[c] * t);
        return s;
    };
    if (f(0.0) < cutoff) return -1.f;  // drops at the first contributing sample
    int zero = 0;
    for (int c = 0; c < 3; ++c) zero += (a[c] == 0.0);
    if ((double)zero >= cutoff) return INFINITY;  // never drops
    double lo = 0.0, hi = 1.0;
    while (f(hi) >= cutoff) hi *= 2.0;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (f(mid) < cutoff) hi = mid; else lo = mid;
    }
    return (float)lo;
}

// math::rotation<Mat4d>(axis, angle), 3x3 part (row-vector convention).
static void rotation(int axis, double ang, double R[3][3]) {
    const double c = std::cos(ang), s = std::sin(ang);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = (i == j) ? 1.0 : 0.0;
    if (axis == 0) { R[1][1] = c; R[1][2] = s; R[2][1] = -s; R[2][2] = c; }
    else if (axis == 1) { R[0][0] = c; R[0][2] = -s; R[2][0] = s; R[2][2] = c; }
    else { R[0][0] = c; R[0][1] = s; R[1][0] = -s; R[1][1] = c; }
}

static void matmul3(const double A[3][3], const double B[3][3], double C[3][3]) {
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
    std::memcpy(C, T, sizeof T);
}

// AffineMap::accumPostRotation -> Mat4::postRotate, which rotates clockwise:
// M <- M * rotation(axis, -angle).
static void post_rotate(double M[3][3], int axis, double ang) {
    double R[3][3];
    rotation(axis, -ang, R);
    matmul3(M, R, M);
}

// PerspectiveCamera as main.cc:96-102 builds it (src/Renderer.h:148-171,232-239).
// Shadow-ray ordering keys of every light of the scene (see RayBin): about
// 4 x 4 voxel (u, v) bins for distant lights (at most 256^2), a cube map of
// about 4 voxels per
// bin at the far side of the leaf bbox (at most 128^2 per face) for point
// lights, and depth bins of about 4 voxels (at most 128): the lanes of a warp
// then start their rays at nearly the same depth and sample neighbouring
// cells at the same time.
static RayBins ray_bins(const DevScene& sc, int64_t cap) {
    RayBins rb{};
    rb.n = sc.n_lights;
    const DevGrid& G = sc.dens;
    double corner[8][3];
    for (int c = 0; c < 8; ++c)
        for (int a = 0; a < 3; ++a) corner[c][a] = ((c >> a) & 1) ? G.bbmax[a] : G.bbmin[a];
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    auto depth_bins = [](RayBin& b, double lo, double hi) {
        const double range = std::max(hi - lo, 1e-3);
        b.nd = (int)std::min(128.0, std::max(1.0, std::ceil(range / 4.0)));
        b.d0 = (float)lo;
        b.inv_ds = (float)(b.nd / range);
    };
    int64_t off = 0;
    for (int k = 0; k < sc.n_lights; ++k) {
        RayBin& b = rb.b[k];
        const DevLight& L = sc.lights[k];
        if (L.type == 0) {
            b.kind = 0;
            double D[3] = {-(double)L.dir[0], -(double)L.dir[1], -(double)L.dir[2]};
            const double nD = std::sqrt(dot(D, D));
            for (double& x : D) x /= nD > 0 ? nD : 1.0;
            int m = 0;
            for (int a = 1; a < 3; ++a)
                if (std::fabs(D[a]) < std::fabs(D[m])) m = a;
            double e[3] = {0, 0, 0};
            e[m] = 1.0;
            double U[3] = {D[1] * e[2] - D[2] * e[1], D[2] * e[0] - D[0] * e[2], D[0] * e[1] - D[1] * e[0]};
            const double nU = std::sqrt(dot(U, U));
            for (double& x : U) x /= nU;
            const double V[3] = {D[1] * U[2] - D[2] * U[1], D[2] * U[0] - D[0] * U[2], D[0] * U[1] - D[1] * U[0]};
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (int c = 0; c < 8; ++c) {
                const double q[3] = {dot(corner[c], U), dot(corner[c], V), dot(corner[c], D)};
                for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], q[a]); hi[a] = std::max(hi[a], q[a]); }
            }
            const double range = std::max({hi[0] - lo[0], hi[1] - lo[1], 1e-3});
            b.ns = 1;
            while (b.ns < 256 && b.ns * 4.0 < range) b.ns *= 2;
            b.inv_bs = (float)(b.ns / range);
            b.u0 = (float)lo[0];
            b.v0 = (float)lo[1];
            for (int a = 0; a < 3; ++a) { b.U[a] = (float)U[a]; b.V[a] = (float)V[a]; b.D[a] = (float)D[a]; }
            depth_bins(b, lo[2], hi[2]);
            b.nkeys = (int64_t)b.ns * b.ns * b.nd;
        } else if (L.type == 1) {
            b.kind = 1;
            double O[3];
            for (int a = 0; a < 3; ++a) O[a] = ((double)L.pos[a] - G.wo[a]) * G.inv_h;
            double dmax = 0.0;
            for (int c = 0; c < 8; ++c) {
                const double w[3] = {corner[c][0] - O[0], corner[c][1] - O[1], corner[c][2] - O[2]};
                dmax = std::max(dmax, std::sqrt(dot(w, w)));
            }
            b.ns = 4;
            while (b.ns < 128 && b.ns * 4.0 < dmax) b.ns *= 2;
            for (int a = 0; a < 3; ++a) b.O[a] = (float)O[a];
            depth_bins(b, 0.0, dmax);
            b.nkeys = 6 * (int64_t)b.ns * b.ns * b.nd;
        } else {
            b.kind = 2;
            b.shift = 0;
            while ((cap >> b.shift) > 65536) ++b.shift;
            b.nkeys = (cap >> b.shift) + 1;
        }
        b.key_off = off;
        off += b.nkeys;
    }
    return rb;
}

static DevCamera make_camera(const lg_camera& c) {
    const double d2r = 3.14159265358979323846 / 180.0;
    double M[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    post_rotate(M, 0, c.rotate[0] * d2r);
    post_rotate(M, 1, (c.rotate[1] + c.y_rotate) * d2r);
    post_rotate(M, 2, c.rotate[2] * d2r);
    double Ry[3][3];
    rotation(1, c.y_rotate * d2r, Ry);  // yRotXform (src/main.cc:68-70)
    double t[3];
    for (int j = 0; j < 3; ++j)
        t[j] = c.translate[0] * Ry[0][j] + c.translate[1] * Ry[1][j] + c.translate[2] * Ry[2][j];
    DevCamera cam{};
    for (int j = 0; j < 3; ++j) {
        cam.eye[j] = (float)t[j];
        cam.cdir[j] = (float)(-M[2][j]);
        for (int i = 0; i < 3; ++i) cam.m[i * 3 + j] = (float)M[i][j];
    }
    const double sw = 0.5 * c.aperture / c.focal;
    cam.sw = (float)sw;
    cam.sh = (float)(sw * (double)c.height / (double)c.width);
    cam.znear = (float)c.znear;
    cam.zfar = (float)c.zfar;
    cam.width = c.width;
    cam.height = c.height;
    cam.spp = c.samples;
    return cam;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

extern "C" lg_status lg_create(int device, lg_ctx** out) {
    if (!out) return LG_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return LG_ERR_NODEVICE;
    }
    if (device < 0 || device >= n) return LG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    Ctx* ctx = new Ctx();
    ctx->device = device;
    // the main stream at the highest priority, the side stream (the render's
    // early count pass) at the lowest: freed SMs go to the main stream first
    int prio_least = 0, prio_greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest) != cudaSuccess) prio_least = prio_greatest = 0;
    if (cudaStreamCreateWithPriority(&ctx->st, cudaStreamNonBlocking, prio_greatest) != cudaSuccess) {
        delete ctx;
        return LG_ERR_CUDA;
    }
    if (cudaStreamCreateWithPriority(&ctx->st2, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_count, cudaEventDisableTiming) != cudaSuccess) {
        if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
        if (ctx->st2) cudaStreamDestroy(ctx->st2);
        cudaStreamDestroy(ctx->st);
        delete ctx;
        return LG_ERR_CUDA;
    }
    // defaults: Shader() and SceneSettings() of the reference
    lg_shader& s = ctx->shader;
    std::memset(&s, 0, sizeof s);
    s.density_scale = 1.0;
    s.density_max = 100.0;
    s.shadow_density_scale = 1.0;
    s.scatter_density_scale = 0.35;
    s.scatter_density_min = 0.025;
    for (int c = 0; c < 3; ++c) {
        s.scattering[c] = 1.5;
        s.albedo[c] = 1.5 / 1.6;
        s.extinction[c] = -1.6;
    }
    s.emission_scale = 0.0;
    s.scatter_scale = 4.0;
    s.scatter_density_mask_power = 0.25;
    s.ramp_in = 0.0;
    s.ramp_out = 1.0;
    lg_settings& o = ctx->settings;
    std::memset(&o, 0, sizeof o);
    o.cutoff = 0.005;
    o.step[0] = 1.0;
    o.step[1] = 3.0;
    o.iter = 1;
    o.scatter_grid_res_factor = 4;
    o.pts_per_kernel = 3;
    o.seed = 0;
    *out = reinterpret_cast<lg_ctx*>(ctx);
    return LG_OK;
}

extern "C" lg_status lg_destroy(lg_ctx* handle) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    if (!ctx) return LG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->st);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    for (int k = 0; k <= Ctx::kStages; ++k)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    for (int k = 0; k <= Ctx::kWaves; ++k)
        if (ctx->wev[k]) cudaEventDestroy(ctx->wev[k]);
    if (ctx->wev_shade) cudaEventDestroy(ctx->wev_shade);
    cudaStreamSynchronize(ctx->st2);
    cudaEventDestroy(ctx->ev_fork);
    cudaEventDestroy(ctx->ev_count);
    cudaStreamDestroy(ctx->st2);
    cudaStreamDestroy(ctx->st);
    delete ctx;
    return LG_OK;
}

extern "C" const char* lg_last_error(const lg_ctx* handle) {
    const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
    return ctx ? ctx->err.c_str() : "null context";
}

extern "C" void* lg_stream(lg_ctx* handle) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    return ctx ? (void*)ctx->st : nullptr;
}

extern "C" const char* lg_version(void) { return "lightgraph_gb300 1.0 (sm_103a)"; }

extern "C" uint64_t lg_kernel_launches(const lg_ctx*) { return g_launch_counter; }

// ---------------------------------------------------------------------------
// grids
// ---------------------------------------------------------------------------

lg_status Ctx::upload_grid(int which, const lg_grid_desc* desc, const float* values, int dtype) {
    Ctx* ctx = this;
    if (!desc || !values) return fail(LG_ERR_INVALID, "null grid descriptor or values");
    if (which != LG_GRID_DENSITY && which != LG_GRID_TEMPERATURE) return fail(LG_ERR_INVALID, "bad grid kind %d", which);
    if (dtype < 0 || dtype > 2) return fail(LG_ERR_INVALID, "bad storage dtype %d", dtype);
    for (int a = 0; a < 3; ++a) {
        if (desc->dims[a] <= 0 || desc->dims[a] > (1 << 20)) return fail(LG_ERR_INVALID, "bad grid dims");
        if (desc->origin[a] % 8 != 0) return fail(LG_ERR_INVALID, "grid origin must be a multiple of 8");
    }
    if (!(desc->voxel_size > 0.0)) return fail(LG_ERR_INVALID, "voxel size must be > 0");
    GridStore& gs = which == LG_GRID_DENSITY ? dens : temp;
    gs.valid = false;
    DevGrid g;
    g.dtype = dtype;
    int nleaf[3];
    for (int a = 0; a < 3; ++a) {
        nleaf[a] = (desc->dims[a] + 7) / 8;
        g.blo[a] = floor_div(desc->origin[a], 8) - 1;
        g.nb[a] = nleaf[a] + 2;
        g.wo[a] = (float)desc->world_origin[a];
    }
    g.h = (float)desc->voxel_size;
    g.inv_h = (float)(1.0 / desc->voxel_size);
    // the samplers address cell records with 32-bit indices
    if ((uint64_t)g.nb[0] * g.nb[1] * g.nb[2] * 512ull >= (1ull << 32))
        return fail(LG_ERR_INVALID, "grid too large: the padded brick box must hold fewer than 2^32 voxels");
    // the marches take floors of index-space coordinates from float bits
    // (floor_bits), exact for |p| < 2^22: the padded box must lie inside that
    for (int a = 0; a < 3; ++a)
        if ((int64_t)g.blo[a] * 8 < -(int64_t)(1 << 22) + 64 || ((int64_t)g.blo[a] + g.nb[a]) * 8 > (1 << 22) - 64)
            return fail(LG_ERR_INVALID, "grid index box must lie within +-2^22 voxels of the origin");
    for (int a = 0; a < 3; ++a) {
        g.vlo[a] = g.blo[a] * 8;
        g.vn[a] = (uint32_t)g.nb[a] * 8u;
    }
    g.sy = (uint32_t)g.nb[0] * 512u;
    g.sz = (uint32_t)g.nb[0] * (uint32_t)g.nb[1] * 512u;
    g.rec_last = g.sz * (uint32_t)g.nb[2] - 1u;
    g.ky = g.sy - 64u;
    g.kz = g.sz - 512u;
    {
        // span_cell's axis terms carry the floor bits' bias 0x4B400000 as
        // 512 * (0x4B400000 / 8) per brick coordinate; rec_off removes it and
        // the box's first brick (arithmetic mod 2^32)
        const uint32_t b8 = 0x4B400000u >> 3;
        g.rec_off = 0u - ((uint32_t)g.blo[0] + b8 + ((uint32_t)g.blo[1] + b8) * (uint32_t)g.nb[0] +
                          ((uint32_t)g.blo[2] + b8) * (uint32_t)g.nb[0] * (uint32_t)g.nb[1]) *
                             512u;
    }
    const int64_t nvox = (int64_t)desc->dims[0] * desc->dims[1] * desc->dims[2];
    const int64_t nbt = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
    const size_t rec = (size_t)cell_record_bytes(dtype);
    CK(staging.reserve(sizeof(float) * nvox), "grid staging alloc");
    CK(cudaMemcpyAsync(staging.p, values, sizeof(float) * nvox, cudaMemcpyHostToDevice, st), "grid upload");
    CK(gs.bricks.reserve(rec * nbt * 512), "brick alloc");
    g.lbx = g.nb[0] + 2;
    g.lby = g.nb[1] + 2;
    g.lbxy = g.lbx * g.lby;
    g.nbits = (uint32_t)((int64_t)g.lbx * g.lby * (g.nb[2] + 2));
    const size_t bit_words = (size_t)g.nbits / 32 + 1;
    CK(gs.bits.reserve(sizeof(uint32_t) * bit_words), "leaf bitmap alloc");
    CK(cudaMemsetAsync(gs.bits.p, 0, sizeof(uint32_t) * bit_words, st), "leaf bitmap clear");
    const uint8_t* d_mask = nullptr;
    if (desc->leaf_mask) {
        const int64_t nl = (int64_t)nleaf[0] * nleaf[1] * nleaf[2];
        CK(mask_staging.reserve(nl), "leaf mask alloc");
        CK(cudaMemcpyAsync(mask_staging.p, desc->leaf_mask, nl, cudaMemcpyHostToDevice, st), "leaf mask upload");
        d_mask = mask_staging.as<uint8_t>();
    }
    int bbox_init[12] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN,
                         INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
    CK(small.reserve(64), "small alloc");
    CK(cudaMemcpyAsync(small.p, bbox_init, sizeof bbox_init, cudaMemcpyHostToDevice, st), "bbox init");
    g.data = gs.bricks.p;
    g.leafbits = gs.bits.as<uint32_t>();
    CK(launch_pack_bricks(staging.as<float>(), desc->dims, desc->origin, g, gs.bricks.p, st), "pack bricks");
    CK(launch_leaf_bits(staging.as<float>(), desc->dims, desc->origin, d_mask, g, gs.bits.as<uint32_t>(),
                        small.as<int>(), st), "leaf bitmap");
    CK(launch_voxel_bbox(staging.as<float>(), desc->dims, small.as<int>() + 6, st), "active voxel bbox");
    int bbox[12];
    CK(cudaMemcpyAsync(bbox, small.p, sizeof bbox, cudaMemcpyDeviceToHost, st), "bbox download");
    CK(cudaStreamSynchronize(st), "grid upload sync");
    staging.release();
    g.has_leaves = bbox[0] <= bbox[3];
    for (int a = 0; a < 3; ++a) {
        g.bbmin[a] = g.has_leaves ? (float)(bbox[a] * 8) : 0.f;
        g.bbmax[a] = g.has_leaves ? (float)(bbox[3 + a] * 8 + 8) : 0.f;
    }
    gs.has_active = bbox[6] <= bbox[9];
    for (int a = 0; a < 3; ++a) {
        gs.vbbox[a] = gs.has_active ? bbox[6 + a] + desc->origin[a] : 0;
        gs.vbbox[3 + a] = gs.has_active ? bbox[9 + a] + desc->origin[a] : 0;
    }
    gs.g = g;
    gs.desc = *desc;
    gs.desc.leaf_mask = nullptr;
    gs.valid = true;
    graph_valid = false;
    ++gs.version;
    return LG_OK;
}

extern "C" lg_status lg_upload_grid(lg_ctx* handle, int which, const lg_grid_desc* desc,
                                    const float* values, int storage_dtype) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    return ctx->upload_grid(which, desc, values, storage_dtype);
}

extern "C" lg_status lg_clear_temperature(lg_ctx* handle) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    ctx->temp.valid = false;
    ctx->graph_valid = false;
    return LG_OK;
}

// ---------------------------------------------------------------------------
// scene state
// ---------------------------------------------------------------------------

extern "C" lg_status lg_set_shader(lg_ctx* handle, const lg_shader* s) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!s) return ctx->fail(LG_ERR_INVALID, "null shader");
    if (s->ramp_n < 0 || s->ramp_n > LG_MAX_RAMP_KEYS) return ctx->fail(LG_ERR_INVALID, "ramp_n out of range");
    for (int c = 0; c < 3; ++c)
        if (!(s->extinction[c] <= 0.0))
            return ctx->fail(LG_ERR_INVALID, "extinction must be <= 0 per channel (got %g)", s->extinction[c]);
    ctx->shader = *s;
    ctx->graph_valid = false;
    return LG_OK;
}

extern "C" lg_status lg_set_settings(lg_ctx* handle, const lg_settings* o) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!o) return ctx->fail(LG_ERR_INVALID, "null settings");
    if (!(o->step[0] > 0.0) || !(o->step[1] > 0.0)) return ctx->fail(LG_ERR_INVALID, "steps must be > 0");
    if (o->scatter_grid_res_factor < 1) return ctx->fail(LG_ERR_INVALID, "scatterGridResFactor must be >= 1");
    if (o->iter < 1) return ctx->fail(LG_ERR_INVALID, "iter must be >= 1");
    ctx->settings = *o;
    ctx->graph_valid = false;
    return LG_OK;
}

lg_status Ctx::set_lights(const lg_light* ls, int n, const float* env_rgb, int env_w, int env_h) {
    Ctx* ctx = this;
    if (n < 0 || n > LG_MAX_LIGHTS) return fail(LG_ERR_INVALID, "at most %d lights", LG_MAX_LIGHTS);
    if (n > 0 && !ls) return fail(LG_ERR_INVALID, "null lights");
    bool need_env = false;
    for (int k = 0; k < n; ++k) {
        if (ls[k].type < 0 || ls[k].type > 2) return fail(LG_ERR_INVALID, "bad light type");
        if (ls[k].samples < 1) return fail(LG_ERR_INVALID, "light samples must be >= 1");
        need_env |= ls[k].type == LG_LIGHT_ENV;
    }
    if (need_env && (!env_rgb || env_w < 2 || env_h < 2))
        return fail(LG_ERR_INVALID, "environment light needs an env map of at least 2x2");
    lights.assign(ls, ls + n);
    graph_valid = false;
    env_valid = false;
    if (env_rgb && env_w > 1 && env_h > 1) {
        const int64_t w = env_w, h = env_h;
        CK(env_rgb_d.reserve(sizeof(float) * w * h * 3), "env alloc");
        CK(env_cond_func.reserve(sizeof(float) * w * h), "env alloc");
        CK(env_cond_cdf.reserve(sizeof(float) * (w + 1) * h), "env alloc");
        CK(env_cond_int.reserve(sizeof(float) * h), "env alloc");
        CK(env_marg_func.reserve(sizeof(float) * h), "env alloc");
        CK(env_marg_cdf.reserve(sizeof(float) * (h + 1)), "env alloc");
        CK(env_marg_int.reserve(sizeof(float) * 4), "env alloc");
        CK(env_cond_guide.reserve(sizeof(int) * (kEnvGuide + 1) * h), "env alloc");
        CK(env_marg_guide.reserve(sizeof(int) * (kEnvGuide + 1)), "env alloc");
        CK(cudaMemcpyAsync(env_rgb_d.p, env_rgb, sizeof(float) * w * h * 3, cudaMemcpyHostToDevice, st), "env upload");
        CK(launch_env_cdf(env_rgb_d.as<float>(), env_w, env_h, env_cond_func.as<float>(), env_cond_cdf.as<float>(),
                          env_cond_int.as<float>(), env_marg_func.as<float>(), env_marg_cdf.as<float>(),
                          env_marg_int.as<float>(), env_cond_guide.as<int>(), env_marg_guide.as<int>(), st),
           "env cdf");
        float mi = 0.f;
        CK(cudaMemcpyAsync(&mi, env_marg_int.p, sizeof(float), cudaMemcpyDeviceToHost, st), "env int");
        CK(cudaStreamSynchronize(st), "env sync");
        env_marg_int_h = mi;
        env_w_ = env_w;
        env_h_ = env_h;
        env_valid = true;
    }
    return LG_OK;
}

extern "C" lg_status lg_set_lights(lg_ctx* handle, const lg_light* ls, int n, const float* env_rgb,
                                   int env_w, int env_h) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    return ctx->set_lights(ls, n, env_rgb, env_w, env_h);
}

DevScene Ctx::scene() const {
    DevScene sc;
    std::memset(&sc, 0, sizeof sc);
    sc.dens = D().g;
    sc.temp = T().g;
    sc.has_temp = T().valid ? 1 : 0;
    const lg_shader& s = shader;
    DevShader& d = sc.sh;
    d.dS = (float)s.density_scale;
    d.dMax = (float)s.density_max;
    d.shadowDS = (float)s.shadow_density_scale;
    d.scatterDS = (float)s.scatter_density_scale;
    d.scatterDMin = (float)s.scatter_density_min;
    double a[3];
    for (int c = 0; c < 3; ++c) {
        a[c] = -s.extinction[c];
        d.a[c] = (float)a[c];
        d.albedo[c] = (float)s.albedo[c];
        d.inv_scatter[c] = (float)(1.0 / s.scattering[c]);
    }
    d.emission_scale = (float)s.emission_scale;
    d.scatter_scale = (float)s.scatter_scale;
    d.mask_power = (float)s.scatter_density_mask_power;
    d.tau_drop = dropout_depth(a, settings.cutoff);
    d.ramp_n = s.ramp_n;
    for (int k = 0; k < s.ramp_n && k < kMaxRamp; ++k) {
        d.ramp_pos[k] = (float)s.ramp_pos[k];
        for (int c = 0; c < 3; ++c) d.ramp_col[k][c] = (float)s.ramp_color[k][c];
    }
    d.ramp_in = (float)s.ramp_in;
    d.ramp_out = (float)s.ramp_out;
    {
        const int n = std::min(s.ramp_n, kMaxRamp);
        for (int k = 0; k < n; ++k) {
            const float gap = k + 1 < n ? d.ramp_pos[k + 1] - d.ramp_pos[k] : d.ramp_pos[0] - d.ramp_pos[k];
            d.ramp_inv[k] = 1.0f / gap;
        }
    }
    sc.n_lights = (int)lights.size();
    for (size_t k = 0; k < lights.size(); ++k) {
        const lg_light& L = lights[k];
        DevLight& o = sc.lights[k];
        o.type = L.type;
        o.samples = L.samples;
        for (int c = 0; c < 3; ++c) {
            o.I[c] = (float)(L.color[c] * (double)(float)L.intensity);
            o.dir[c] = (float)L.dir[c];
            o.pos[c] = (float)L.pos[c];
        }
        for (int e = 0; e < 9; ++e) o.rot[e] = (float)L.rot[e];
    }
    if (env_valid) {
        sc.env.rgb = env_rgb_d.as<float>();
        sc.env.cond_cdf = env_cond_cdf.as<float>();
        sc.env.cond_guide = env_cond_guide.as<int>();
        sc.env.marg_guide = env_marg_guide.as<int>();
        sc.env.cond_func = env_cond_func.as<float>();
        sc.env.cond_int = env_cond_int.as<float>();
        sc.env.marg_cdf = env_marg_cdf.as<float>();
        sc.env.marg_func = env_marg_func.as<float>();
        sc.env.marg_int = env_marg_int_h;
        sc.env.w = env_w_;
        sc.env.h = env_h_;
    }
    sc.cutoff = (float)settings.cutoff;
    sc.step0 = (float)settings.step[0];
    sc.step1 = (float)settings.step[1];
    sc.seed = settings.seed;
    {
        ShadowMarch& m = sc.smarch;
        m.scale = d.dS * d.shadowDS;
        m.unit = m.scale > 0.f && std::isfinite(m.scale) ? 1 : 0;
        m.dmax = m.unit ? d.dMax / m.scale : d.dMax;
        m.cut = m.unit ? sc.cutoff / m.scale : sc.cutoff;
        m.drop = m.unit ? d.tau_drop / m.scale : d.tau_drop;
    }
    return sc;
}

// ---------------------------------------------------------------------------
// stage 1: graphs
// ---------------------------------------------------------------------------

lg_status Ctx::load_graphs(int n_graphs, const float* points, const int64_t* offsets,
                           const float* radius_sq, int max_connect) {
    Ctx* ctx = this;
    // graph-indexed kernels put the graph in gridDim.y (at most 65535)
    if (n_graphs < 1 || n_graphs > 65535) return fail(LG_ERR_INVALID, "n_graphs must be in [1, 65535]");
    if (!offsets || !radius_sq) return fail(LG_ERR_INVALID, "null offsets or radius");
    if (max_connect < 0 || max_connect > 255) return fail(LG_ERR_INVALID, "max_connect must be in [0, 255]");
    if (offsets[0] != 0) return fail(LG_ERR_INVALID, "offsets[0] must be 0");
    for (int g = 0; g < n_graphs; ++g) {
        const int64_t n = offsets[g + 1] - offsets[g];
        if (n < 0 || n > 65535) return fail(LG_ERR_INVALID, "graph %d has %lld points (0..65535)", g, (long long)n);
    }
    const int64_t P = offsets[n_graphs];
    if (P > 0 && !points) return fail(LG_ERR_INVALID, "null points");
    h_graphs.resize(n_graphs);
    int64_t s_off = 0, e_off = 0;
    max_n = 0;
    max_edges = 0;
    for (int g = 0; g < n_graphs; ++g) {
        GraphInfo& gi = h_graphs[g];
        gi.pt_off = offsets[g];
        gi.n = (int32_t)(offsets[g + 1] - offsets[g]);
        gi.ld = round_up(std::max(gi.n, 1), 128);
        gi.s_off = s_off;
        s_off += (int64_t)gi.ld * gi.ld;
        gi.max_edges = (int32_t)(((int64_t)gi.n * max_connect) / 2);
        gi.e_off = e_off;
        e_off += gi.max_edges;
        gi.r2 = radius_sq[g];
        max_n = std::max(max_n, gi.n);
        max_edges = std::max(max_edges, gi.max_edges);
    }
    this->n_graphs = n_graphs;
    n_points = P;
    s_floats = s_off;
    edge_slots = e_off;
    this->max_connect = max_connect;
    h_pts.assign(points, points + 3 * P);
    std::vector<int32_t> pg(P);
    for (int g = 0; g < n_graphs; ++g)
        for (int64_t i = offsets[g]; i < offsets[g + 1]; ++i) pg[i] = g;
    CK(d_pts.reserve(sizeof(float) * 3 * std::max<int64_t>(P, 1)), "points alloc");
    CK(d_graphs.reserve(sizeof(GraphInfo) * n_graphs), "graphs alloc");
    CK(d_pt_graph.reserve(sizeof(int32_t) * std::max<int64_t>(P, 1)), "point graph alloc");
    CK(d_cand.reserve(sizeof(uint16_t) * kCandCap * std::max<int64_t>(P, 1)), "candidate alloc");
    CK(d_cand_cnt.reserve(sizeof(int32_t) * std::max<int64_t>(P, 1)), "candidate count alloc");
    CK(d_edges.reserve(sizeof(int2) * std::max<int64_t>(e_off, 1)), "edge alloc");
    CK(d_edge_cnt.reserve(sizeof(int32_t) * n_graphs), "edge count alloc");
    if (P > 0) {
        CK(cudaMemcpyAsync(d_pts.p, points, sizeof(float) * 3 * P, cudaMemcpyHostToDevice, st), "points upload");
        CK(cudaMemcpyAsync(d_pt_graph.p, pg.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st), "graph ids upload");
    }
    CK(cudaMemcpyAsync(d_graphs.p, h_graphs.data(), sizeof(GraphInfo) * n_graphs, cudaMemcpyHostToDevice, st),
       "graph info upload");
    // the host copies above read pageable memory; finish them before the
    // caller's buffers can change
    CK(cudaStreamSynchronize(st), "graph upload sync");
    point_voxel_size_cache = -1.0;
    graph_valid = false;
    fw_choice = fw_pinned;
    if (fw_pinned < 0)
        for (auto& kv : fw_tuned)
            if (kv.first == std::make_pair(n_graphs, max_n)) fw_choice = kv.second;
    graphs_built = false;
    return LG_OK;
}

lg_status Ctx::build_edges() {
    Ctx* ctx = this;
    CK(launch_candidates(d_pts.as<float>(), d_graphs.as<GraphInfo>(), d_pt_graph.as<int32_t>(), n_points,
                         d_cand.as<uint16_t>(), d_cand_cnt.as<int32_t>(), st), "edge candidates");
    CK(launch_greedy(d_pts.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_n, d_cand.as<uint16_t>(),
                     d_cand_cnt.as<int32_t>(), max_connect, d_edges.as<int2>(), d_edge_cnt.as<int32_t>(), st),
       "greedy connect");
    graphs_built = true;
    return LG_OK;
}

// ---------------------------------------------------------------------------
// dart throwing (LightGraph::scatterPoints)
// ---------------------------------------------------------------------------

extern "C" lg_status lg_scatter_opts_default(lg_scatter_opts* o) {
    if (!o) return LG_ERR_INVALID;
    *o = lg_scatter_opts{};
    o->scatter_count = 1000000;  // PC_SCATTER_COUNT (src/main.cc:61)
    o->target_size = 750;        // TARGET_PC_SIZE (src/LightGraph.h:25)
    o->n_estimates = 100;        // PC_GROWTH_NUMBER_OF_ESTIMATE (src/LightGraph.h:26)
    o->hard_limit = 1000;        // PC_SIZE_HARD_LIMIT (src/LightGraph.h:22)
    o->growth_power = 0.17f;     // PC_GROWTH_FUNC_POWER (src/LightGraph.h:27)
    o->density_cutoff = 0.001f;  // PC_DENSITY_CUTOFF (src/LightGraph.h:24)
    o->min_dist_mult = 0.13f;    // MIN_DIST_MULT (src/main.cc:60)
    o->connect_mult = 1.7f;      // CONNECT_SEARCH_RADIUS_MULT (src/LightGraph.h:23)
    o->seed_base = 854123;       // RandGen engines (src/RandGen.h:28-30)
    return LG_OK;
}

extern "C" lg_status lg_randgen_draws(uint32_t seed, int64_t n, float* out, uint32_t* raw) {
    if (n < 0) return LG_ERR_INVALID;
    Mt19937 mt(seed);
    for (int64_t k = 0; k < n; ++k) {
        const uint32_t x = mt.next();
        if (raw) raw[k] = x;
        if (out) out[k] = mt_canonical_float(x);
    }
    return LG_OK;
}

lg_status Ctx::scatter_points(const lg_scatter_opts& o, int first_iter, int n_iter) {
    Ctx* ctx = this;
    const GridStore& gs = D();
    if (!gs.valid) return fail(LG_ERR_STATE, "no density grid uploaded");
    if (n_iter < 1 || first_iter < 0) return fail(LG_ERR_INVALID, "bad iteration range");
    if (o.n_estimates < 1 || o.scatter_count < o.n_estimates)
        return fail(LG_ERR_INVALID, "scatter_count must be >= n_estimates >= 1");
    if (o.hard_limit < 1 || o.hard_limit > 4096 || o.target_size >= o.hard_limit)
        return fail(LG_ERR_INVALID, "need target_size < hard_limit <= 4096");
    if (!gs.has_active) return fail(LG_ERR_STATE, "the density grid has no active voxel");
    // world bbox of the active voxels (Transform::indexToWorld of
    // evalActiveVoxelBoundingBox, src/main.cc:512) and the starting minimum
    // distance (src/main.cc:514-518), in the reference's float / double types
    double bbmin[3], bbmax[3];
    float bbsize[3];
    for (int a = 0; a < 3; ++a) {
        bbmin[a] = gs.desc.world_origin[a] + (double)gs.vbbox[a] * gs.desc.voxel_size;
        bbmax[a] = gs.desc.world_origin[a] + (double)gs.vbbox[3 + a] * gs.desc.voxel_size;
        bbsize[a] = (float)(bbmax[a] - bbmin[a]);
    }
    const float avg = (bbsize[0] + bbsize[1] + bbsize[2]) / 3.0f;
    const float min_dist = o.min_dist_mult * avg;
    // expected sizes at the radius updates (n + 1) % batch == 0
    // (src/LightGraph.h:220-222, 240-245), with the C library's pow
    const uint32_t batch = o.scatter_count / o.n_estimates;
    const uint32_t n_upd = o.scatter_count / batch;
    std::vector<uint32_t> expected(n_upd + 1);
    for (uint32_t k = 0; k < n_upd; ++k) {
        const uint64_t n = (uint64_t)(k + 1) * batch - 1;
        expected[k] = (uint32_t)(o.target_size * std::pow((double)n / (double)o.scatter_count, (double)o.growth_power));
    }
    DartParams prm{};
    prm.scatter_count = o.scatter_count;
    prm.target = o.target_size;
    prm.batch = batch;
    prm.hard_limit = o.hard_limit;
    prm.cutoff = o.density_cutoff;
    prm.min_dist_sq0 = min_dist * min_dist;
    prm.seed_base = o.seed_base;
    prm.first_iter = first_iter;
    for (int a = 0; a < 3; ++a) {
        prm.bbmin[a] = bbmin[a];
        prm.bbsize[a] = bbsize[a];
        prm.wo[a] = gs.desc.world_origin[a];
    }
    prm.h = gs.desc.voxel_size;
    // FP32 fast path of the density test: index = (p - wo) * (1 / h). Its
    // error in voxels: the rounding of wo (|wo - wo_f| / h) plus three
    // roundings of at most 2^-24 relative (the subtraction, 1 / h, the
    // product) on indices below max_index, doubled for margin
    double max_index = 0.0, wo_err = 0.0;
    for (int a = 0; a < 3; ++a) {
        prm.wo_f[a] = (float)gs.desc.world_origin[a];
        for (double e : {bbmin[a], bbmax[a]})
            max_index = std::max(max_index, std::fabs((e - gs.desc.world_origin[a]) / gs.desc.voxel_size) + 2.0);
        wo_err = std::max(wo_err, std::fabs(gs.desc.world_origin[a] - (double)prm.wo_f[a]) / gs.desc.voxel_size);
    }
    prm.inv_h_f = (float)(1.0 / gs.desc.voxel_size);
    prm.index_err = (float)(2.0 * (wo_err + 3.0 * max_index * 5.9604644775390625e-8) + 1e-7);
    const size_t npts = (size_t)n_iter * o.hard_limit * 3;
    CK(d_dart_pts.reserve(sizeof(float) * npts), "dart alloc");
    CK(d_dart_cnt.reserve(sizeof(int32_t) * n_iter), "dart alloc");
    CK(d_dart_m2.reserve(sizeof(float) * n_iter), "dart alloc");
    CK(d_dart_expected.reserve(sizeof(uint32_t) * expected.size()), "dart alloc");
    CK(cudaMemcpyAsync(d_dart_expected.p, expected.data(), sizeof(uint32_t) * expected.size(), cudaMemcpyHostToDevice,
                       st), "dart upload");
    CK(launch_dart(gs.g, prm, n_iter, d_dart_expected.as<uint32_t>(), d_dart_pts.as<float>(), d_dart_cnt.as<int32_t>(),
                   d_dart_m2.as<float>(), st), "dart throwing");
    h_dart_pts.resize(npts);
    h_dart_cnt.resize(n_iter);
    h_dart_m2.resize(n_iter);
    CK(cudaMemcpyAsync(h_dart_pts.data(), d_dart_pts.p, sizeof(float) * npts, cudaMemcpyDeviceToHost, st),
       "dart download");
    CK(cudaMemcpyAsync(h_dart_cnt.data(), d_dart_cnt.p, sizeof(int32_t) * n_iter, cudaMemcpyDeviceToHost, st),
       "dart download");
    CK(cudaMemcpyAsync(h_dart_m2.data(), d_dart_m2.p, sizeof(float) * n_iter, cudaMemcpyDeviceToHost, st),
       "dart download");
    CK(cudaStreamSynchronize(st), "dart sync");
    return LG_OK;
}

// searchRadiusConnectSquared of an iteration from its last accepted squared
// minimum distance (src/LightGraph.h:170-171, 268-269), in float.
static float connect_radius_sq(float last_m2, float connect_mult) {
    const float min_dist = std::sqrt(last_m2);
    const float r = min_dist * connect_mult;
    return r * r;
}

extern "C" lg_status lg_scatter_points(lg_ctx* handle, const lg_scatter_opts* opts, int first_iter, int n_iter,
                                       float* points, int32_t* counts, float* radius_sq) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!opts) return ctx->fail(LG_ERR_INVALID, "null options");
    lg_status s = ctx->scatter_points(*opts, first_iter, n_iter);
    if (s != LG_OK) return s;
    if (points) std::memcpy(points, ctx->h_dart_pts.data(), sizeof(float) * ctx->h_dart_pts.size());
    if (counts) std::memcpy(counts, ctx->h_dart_cnt.data(), sizeof(int32_t) * n_iter);
    if (radius_sq)
        for (int i = 0; i < n_iter; ++i) radius_sq[i] = connect_radius_sq(ctx->h_dart_m2[i], opts->connect_mult);
    return LG_OK;
}

extern "C" lg_status lg_scatter_graphs(lg_ctx* handle, const lg_scatter_opts* opts, int first_iter, int n_iter,
                                       int max_connect, int32_t* counts) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!opts) return ctx->fail(LG_ERR_INVALID, "null options");
    lg_status s = ctx->scatter_points(*opts, first_iter, n_iter);
    if (s != LG_OK) return s;
    std::vector<int64_t> offs(n_iter + 1, 0);
    std::vector<float> r2(n_iter);
    for (int i = 0; i < n_iter; ++i) {
        offs[i + 1] = offs[i] + ctx->h_dart_cnt[i];
        r2[i] = connect_radius_sq(ctx->h_dart_m2[i], opts->connect_mult);
    }
    std::vector<float> pts((size_t)offs[n_iter] * 3);
    for (int i = 0; i < n_iter; ++i)
        std::memcpy(pts.data() + 3 * offs[i], ctx->h_dart_pts.data() + (size_t)i * opts->hard_limit * 3,
                    sizeof(float) * 3 * ctx->h_dart_cnt[i]);
    if (counts) std::memcpy(counts, ctx->h_dart_cnt.data(), sizeof(int32_t) * n_iter);
    s = ctx->load_graphs(n_iter, pts.data(), offs.data(), r2.data(), max_connect);
    if (s != LG_OK) return s;
    return ctx->build_edges();
}

extern "C" lg_status lg_build_graphs(lg_ctx* handle, int n_graphs, const float* points,
                                     const int64_t* offsets, const float* radius_sq, int max_connect,
                                     uint8_t* adj_out, int64_t* n_edges_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    lg_status s = ctx->load_graphs(n_graphs, points, offsets, radius_sq, max_connect);
    if (s != LG_OK) return s;
    s = ctx->build_edges();
    if (s != LG_OK) return s;
    if (adj_out) {
        int64_t total = 0;
        std::vector<int64_t> aoff(n_graphs);
        for (int g = 0; g < n_graphs; ++g) {
            aoff[g] = total;
            total += (int64_t)ctx->h_graphs[g].n * ctx->h_graphs[g].n;
        }
        CK(ctx->d_adj.reserve(std::max<int64_t>(total, 1)), "adjacency alloc");
        CK(ctx->d_adj_off.reserve(sizeof(int64_t) * n_graphs), "adjacency offsets alloc");
        CK(cudaMemcpyAsync(ctx->d_adj_off.p, aoff.data(), sizeof(int64_t) * n_graphs, cudaMemcpyHostToDevice,
                           ctx->st), "adjacency offsets upload");
        CK(cudaMemsetAsync(ctx->d_adj.p, 0, std::max<int64_t>(total, 1), ctx->st), "adjacency clear");
        CK(launch_adjacency(ctx->d_graphs.as<GraphInfo>(), n_graphs, ctx->max_edges, ctx->d_edges.as<int2>(),
                            ctx->d_edge_cnt.as<int32_t>(), ctx->d_adj.as<uint8_t>(), ctx->d_adj_off.as<int64_t>(),
                            ctx->st), "adjacency");
        if (total > 0)
            CK(cudaMemcpyAsync(adj_out, ctx->d_adj.p, total, cudaMemcpyDeviceToHost, ctx->st), "adjacency download");
    }
    if (n_edges_out) {
        std::vector<int32_t> ec(n_graphs);
        CK(cudaMemcpyAsync(ec.data(), ctx->d_edge_cnt.p, sizeof(int32_t) * n_graphs, cudaMemcpyDeviceToHost,
                           ctx->st), "edge count download");
        CK(cudaStreamSynchronize(ctx->st), "sync");
        for (int g = 0; g < n_graphs; ++g) n_edges_out[g] = ec[g];
    }
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return LG_OK;
}

lg_status Ctx::copy_matrix_out(float* out) {
    Ctx* ctx = this;
    int64_t o = 0;
    for (const GraphInfo& g : h_graphs) {
        if (g.n > 0)
            CK(cudaMemcpy2DAsync(out + o, sizeof(float) * g.n, d_S.as<float>() + g.s_off, sizeof(float) * g.ld,
                                 sizeof(float) * g.n, g.n, cudaMemcpyDeviceToHost, st), "matrix download");
        o += (int64_t)g.n * g.n;
    }
    CK(cudaStreamSynchronize(st), "sync");
    return fw_wait_status();
}

// The error word of this context's last persistent Floyd-Warshall launch,
// which a bounded dependency wait raises when it gives up (the launch then
// ends early and its matrices are incomplete): LG_ERR_TIMEOUT if raised. Read
// where a call has synchronised the stream to hand results back.
lg_status Ctx::fw_wait_status() {
    Ctx* ctx = this;
    if (!fw_flag_pending || d_fw_sync.bytes < 2 * sizeof(uint32_t)) return LG_OK;
    fw_flag_pending = false;
    uint32_t flags[2] = {0, 0};
    CK(cudaMemcpyAsync(flags, d_fw_sync.p, sizeof flags, cudaMemcpyDeviceToHost, st), "fw flag read");
    CK(cudaStreamSynchronize(st), "sync");
    if (flags[1] != 0) return fail(LG_ERR_TIMEOUT, "batched floyd-warshall: a dependency wait timed out");
    return LG_OK;
}

lg_status Ctx::march_edges() {
    Ctx* ctx = this;
    if (!D().valid) return fail(LG_ERR_STATE, "no density grid uploaded");
    if (!graphs_built) return fail(LG_ERR_STATE, "no graphs built");
    CK(d_S.reserve(sizeof(float) * std::max<int64_t>(s_floats, 1)), "S alloc");
    CK(launch_fill(d_S.as<float>(), s_floats, INFINITY, st), "S fill");
    CK(launch_edge_march(scene(), d_pts.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_edges,
                         d_edges.as<int2>(), d_edge_cnt.as<int32_t>(), d_S.as<float>(), st), "edge march");
    return LG_OK;
}

// Schedules of the path solve: 0 = two launches per round per graph
// (fw_solve); 1, 2 = one persistent launch for all graphs with 1 or 2 CTAs per
// SM; 3, 4 = the symmetric persistent solve (the tiles on and above the
// diagonal, then a mirror pass) with 1 or 2 CTAs per SM; 5 = schedule 4 with
// the update tiles' operands staged by TMA bulk copies. The graph matrices
// are symmetric by construction (k_march.cu stores every edge both ways).
static lg_status run_fw_schedule(Ctx* ctx, float* base, int choice) {
    if (choice == 0) {
        for (const GraphInfo& g : ctx->h_graphs) {
            if (g.n == 0) continue;
            CK(fw_solve(base + g.s_off, g.ld, g.ld, ctx->st), "floyd-warshall");
        }
        return LG_OK;
    }
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "device query");
    ctx->fw_flag_pending = true;
    if (choice >= 3) {
        CK(fw_solve_batched_sym(base, ctx->d_fwg.as<FwGraph>(), ctx->n_graphs, ctx->fw_max_nt,
                                ctx->d_fw_items_sym.as<int4>(), ctx->fw_items_sym_n, ctx->d_fw_sync.as<uint32_t>(),
                                ctx->fw_sync_n, ctx->d_fw_panels.as<float2>(), (choice == 3 ? 1 : 2) * sms,
                                choice == 5, ctx->st),
           "symmetric batched floyd-warshall");
        return LG_OK;
    }
    CK(fw_solve_batched(base, ctx->d_fwg.as<FwGraph>(), ctx->d_fw_items.as<int4>(), ctx->fw_items_n,
                        ctx->d_fw_sync.as<uint32_t>(), ctx->fw_sync_n, choice * sms, ctx->st),
       "batched floyd-warshall");
    return LG_OK;
}

lg_status Ctx::solve_paths_batched(int choice) {
    Ctx* ctx = this;
    // the queues depend only on where each matrix lives and its padded size:
    // a new point set of the same sizes (every frame of lg_render_frame)
    // keeps them
    std::vector<int64_t> key;
    key.reserve(2 * n_graphs + 1);
    key.push_back(n_graphs);
    for (const GraphInfo& gi : h_graphs) {
        key.push_back(gi.s_off);
        key.push_back(gi.n == 0 ? -1 : gi.ld);
    }
    if (fw_queue_valid && key != fw_queue_key) fw_queue_valid = false;
    if (!fw_queue_valid) {
        // graph descriptors, sync words and panel slots (both solves)
        fw_queue_key = key;
        std::vector<FwGraph> fg(n_graphs);
        int64_t vofs = 0, pofs = 0;
        fw_max_nt = 0;
        for (int g = 0; g < n_graphs; ++g) {
            const GraphInfo& gi = h_graphs[g];
            fg[g].off = gi.s_off;
            fg[g].n = gi.ld;  // the padded matrix: every tile is full
            fg[g].ld = gi.ld;
            fg[g].nt = gi.n == 0 ? 0 : gi.ld / 64;
            fg[g].nu = gi.n == 0 ? 0 : gi.ld / 128;
            fg[g].vofs = vofs;
            fg[g].pofs = pofs;
            vofs += (int64_t)fg[g].nt * fg[g].nt + fg[g].nt;
            pofs += (int64_t)fw_panel_words(fg[g]);
            fw_max_nt = std::max(fw_max_nt, fg[g].nt);
        }
        fw_sync_n = fw_sync_words(fg.data(), n_graphs);
        CK(d_fwg.reserve(sizeof(FwGraph) * n_graphs), "fw queue alloc");
        CK(d_fw_sync.reserve(sizeof(uint32_t) * fw_sync_n), "fw queue alloc");
        CK(d_fw_panels.reserve(sizeof(float2) * std::max<int64_t>(pofs, 1)), "fw panel alloc");
        CK(cudaMemcpyAsync(d_fwg.p, fg.data(), sizeof(FwGraph) * n_graphs, cudaMemcpyHostToDevice, st), "fw queue upload");
        CK(cudaStreamSynchronize(st), "fw queue sync");
        h_fwg = std::move(fg);
        fw_queue_valid = true;
        fw_general_built = false;
        fw_sym_built = false;
    }
    if ((choice == 1 || choice == 2) && !fw_general_built) {
        const size_t n_items = fw_batched_items(h_fwg.data(), n_graphs, nullptr);
        std::vector<int4> items(std::max<size_t>(n_items, 1));
        fw_batched_items(h_fwg.data(), n_graphs, items.data());
        CK(d_fw_items.reserve(sizeof(int4) * items.size()), "fw queue alloc");
        CK(cudaMemcpyAsync(d_fw_items.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, st),
           "fw queue upload");
        CK(cudaStreamSynchronize(st), "fw queue sync");
        fw_items_n = (int)n_items;
        fw_general_built = true;
    }
    if (choice >= 3 && !fw_sym_built) {
        const size_t n_items_sym = fw_batched_items(h_fwg.data(), n_graphs, nullptr, true);
        h_fw_items_sym.assign(std::max<size_t>(n_items_sym, 1), make_int4(0, 0, 0, 0));
        fw_batched_items(h_fwg.data(), n_graphs, h_fw_items_sym.data(), true);
        CK(d_fw_items_sym.reserve(sizeof(int4) * h_fw_items_sym.size()), "fw queue alloc");
        CK(cudaMemcpyAsync(d_fw_items_sym.p, h_fw_items_sym.data(), sizeof(int4) * h_fw_items_sym.size(),
                           cudaMemcpyHostToDevice, st), "fw queue upload");
        CK(cudaStreamSynchronize(st), "fw queue sync");
        fw_items_sym_n = (int)n_items_sym;
        fw_sym_built = true;
        fw_queue_uses = 0;
        fw_sym_ordered = false;
    } else if (choice >= 3 && n_graphs == 1 && !fw_sym_ordered && !capturing &&
               (fw_order_next || ++fw_queue_uses >= 2)) {
        // one graph solved again with the same size (frames of a fixed
        // scene), or a frame about to be captured for replay: the
        // list-scheduled order of the symmetric queue pays for its host time
        // (tens of ms at 4096 points) there, so it is computed now rather
        // than for every one-off size. Batches of many graphs keep the
        // structural order, which interleaves the graphs round by round (the
        // simulated order measured 2.8x slower on 64 graphs of 257-3805
        // points: 53 ms against 18.9 ms)
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device query");
        fw_order_sym(h_fwg.data(), n_graphs, h_fw_items_sym.data(), (size_t)fw_items_sym_n, 2 * sms);
        CK(cudaMemcpyAsync(d_fw_items_sym.p, h_fw_items_sym.data(), sizeof(int4) * fw_items_sym_n,
                           cudaMemcpyHostToDevice, st), "fw queue upload");
        CK(cudaStreamSynchronize(st), "fw queue sync");
        fw_sym_ordered = true;
    }
    return LG_OK;
}

// Autotuner: times every candidate schedule once on a scratch copy of the
// batch and keeps the fastest for this (graph count, largest graph) key.
lg_status Ctx::tune_fw() {
    Ctx* ctx = this;
    const std::pair<int, int> key(n_graphs, max_n);
    for (auto& kv : fw_tuned)
        if (kv.first == key) { fw_choice = kv.second; return LG_OK; }
    lg_status s = solve_paths_batched(2);
    if (s == LG_OK) s = solve_paths_batched(4);
    if (s != LG_OK) return s;
    // schedule 0 and the persistent solves at the highest residency (the
    // 1-CTA/SM ones only where 2 do not fit: they never win otherwise)
    std::vector<int> cands = {0};
    cands.push_back(fw_persistent_ctas_per_sm() >= 2 ? 2 : 1);
    cands.push_back(fw_persistent_sym_ctas_per_sm() >= 2 ? 4 : 3);
    if (cands.back() == 4) cands.push_back(5);
    CK(d_fw_tune.reserve(sizeof(float) * std::max<int64_t>(s_floats, 1)), "fw tune alloc");
    // the trial events, destroyed on every way out
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    CK(cudaEventCreate(&ev.a), "event");
    CK(cudaEventCreate(&ev.b), "event");
    const cudaEvent_t e0 = ev.a, e1 = ev.b;
    int best = 0;
    float best_ms = 1e30f;
    for (double& t : fw_tune_ms) t = 0.0;
    // one trial each, then a second trial of the two fastest (the first launch
    // of a kernel can carry one-time costs: module load, a profiler's setup)
    std::vector<int> trials = cands;
    for (size_t c = 0; c < trials.size() && s == LG_OK; ++c) {
        if (c == cands.size()) {
            std::vector<int> order = cands;
            std::sort(order.begin(), order.end(), [&](int a, int b) { return fw_tune_ms[a] < fw_tune_ms[b]; });
            trials.push_back(order[0]);
            trials.push_back(order[1]);
        }
        const int cand = trials[c];
        CK(cudaMemcpyAsync(d_fw_tune.p, d_S.p, sizeof(float) * s_floats, cudaMemcpyDeviceToDevice, st), "fw tune copy");
        CK(cudaEventRecord(e0, st), "event");
        s = run_fw_schedule(this, d_fw_tune.as<float>(), cand);
        if (s != LG_OK) break;
        CK(cudaEventRecord(e1, st), "event");
        CK(cudaEventSynchronize(e1), "event sync");
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1), "event time");
        if (cand > 0) {
            // a persistent launch reports a stalled queue through its error flag
            uint32_t flags[2] = {0, 0};
            CK(cudaMemcpy(flags, d_fw_sync.p, sizeof flags, cudaMemcpyDeviceToHost), "fw flag read");
            if (flags[1] != 0) {
                s = fail(LG_ERR_TIMEOUT, "batched floyd-warshall: a dependency wait timed out");
                break;
            }
        }
        if (fw_tune_ms[cand] == 0.0 || ms < fw_tune_ms[cand]) fw_tune_ms[cand] = ms;
        if (ms < best_ms) { best_ms = ms; best = cand; }
    }
    if (s != LG_OK) return s;
    fw_tuned.push_back({key, best});
    fw_choice = best;
    return LG_OK;
}

lg_status Ctx::solve_paths() {
    Ctx* ctx = this;
    if (fw_choice < 0) {
        lg_status s = tune_fw();
        if (s != LG_OK) return s;
    }
    if (fw_choice > 0) {
        lg_status s = solve_paths_batched(fw_choice);
        if (s != LG_OK) return s;
    }
    lg_status s = run_fw_schedule(this, d_S.as<float>(), fw_choice);
    if (s != LG_OK) return s;
    CK(launch_set_diag(d_S.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_n, st), "diagonal");
    return LG_OK;
}

lg_status Ctx::fw_solve_on(float* base, int choice) {
    if (choice < 3 || choice > 5) return fail(LG_ERR_INVALID, "batched path solves use a symmetric schedule");
    lg_status s = solve_paths_batched(choice);
    if (s != LG_OK) return s;
    return run_fw_schedule(this, base, choice);
}

lg_status Ctx::solve_rest() {
    Ctx* ctx = this;
    CK(launch_set_diag(d_S.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_n, st), "diagonal");
    paths_solved = true;
    lg_status s = vertex_light();
    if (s != LG_OK) return s;
    light_done = true;
    s = diffuse();
    if (s != LG_OK) return s;
    diffuse_done = true;
    return LG_OK;
}

lg_status Ctx::vertex_light() {
    Ctx* ctx = this;
    if (!D().valid) return fail(LG_ERR_STATE, "no density grid uploaded");
    CK(d_L.reserve(sizeof(float) * 3 * std::max<int64_t>(n_points, 1)), "L alloc");
    CK(launch_vertex_light(scene(), d_pts.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_n, d_L.as<float>(),
                           st), "vertex light");
    return LG_OK;
}

lg_status Ctx::diffuse() {
    Ctx* ctx = this;
    const int64_t P = std::max<int64_t>(n_points, 1);
    CK(d_D.reserve(sizeof(float) * 3 * P), "D alloc");
    CK(d_part.reserve(sizeof(float) * 3 * kRowChunks * P), "diffuse scratch alloc");
    CK(d_colw.reserve(sizeof(float) * 3 * P), "diffuse scratch alloc");
    CK(launch_diffuse(scene().sh, d_S.as<float>(), d_graphs.as<GraphInfo>(), n_graphs, max_n, d_L.as<float>(),
                      d_part.as<float>(), d_colw.as<float>(), d_D.as<float>(), st), "diffuse");
    return LG_OK;
}

extern "C" lg_status lg_march_edges(lg_ctx* handle, float* S_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    lg_status s = ctx->march_edges();
    if (s != LG_OK) return s;
    ctx->paths_solved = false;
    if (S_out) return ctx->copy_matrix_out(S_out);
    return LG_OK;
}

extern "C" lg_status lg_solve_paths(lg_ctx* handle, float* dist_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->graphs_built || ctx->d_S.bytes == 0) return ctx->fail(LG_ERR_STATE, "edges not marched");
    lg_status s = ctx->solve_paths();
    if (s != LG_OK) return s;
    ctx->paths_solved = true;
    if (dist_out) return ctx->copy_matrix_out(dist_out);
    return LG_OK;
}

extern "C" lg_status lg_vertex_light(lg_ctx* handle, float* light_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->graphs_built) return ctx->fail(LG_ERR_STATE, "no graphs loaded");
    lg_status s = ctx->vertex_light();
    if (s != LG_OK) return s;
    ctx->light_done = true;
    if (light_out && ctx->n_points > 0) {
        CK(cudaMemcpyAsync(light_out, ctx->d_L.p, sizeof(float) * 3 * ctx->n_points, cudaMemcpyDeviceToHost,
                           ctx->st), "L download");
        CK(cudaStreamSynchronize(ctx->st), "sync");
    }
    return LG_OK;
}

extern "C" lg_status lg_diffuse(lg_ctx* handle, float* diffuse_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->paths_solved || !ctx->light_done)
        return ctx->fail(LG_ERR_STATE, "diffuse needs solved paths and vertex light");
    lg_status s = ctx->diffuse();
    if (s != LG_OK) return s;
    ctx->diffuse_done = true;
    if (diffuse_out && ctx->n_points > 0) {
        CK(cudaMemcpyAsync(diffuse_out, ctx->d_D.p, sizeof(float) * 3 * ctx->n_points, cudaMemcpyDeviceToHost,
                           ctx->st), "D download");
        CK(cudaStreamSynchronize(ctx->st), "sync");
        return ctx->fw_wait_status();
    }
    return LG_OK;
}

lg_status Ctx::solve_all() {
    lg_status s = march_edges();
    if (s != LG_OK) return s;
    s = solve_paths();
    if (s != LG_OK) return s;
    paths_solved = true;
    s = vertex_light();
    if (s != LG_OK) return s;
    light_done = true;
    s = diffuse();
    if (s != LG_OK) return s;
    diffuse_done = true;
    return LG_OK;
}

extern "C" lg_status lg_solve_graphs(lg_ctx* handle, float* diffuse_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->graphs_built) return ctx->fail(LG_ERR_STATE, "no graphs built");
    lg_status s = ctx->solve_all();
    if (s != LG_OK) return s;
    if (diffuse_out && ctx->n_points > 0) {
        CK(cudaMemcpyAsync(diffuse_out, ctx->d_D.p, sizeof(float) * 3 * ctx->n_points, cudaMemcpyDeviceToHost,
                           ctx->st), "D download");
    }
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return ctx->fw_wait_status();
}

extern "C" lg_status lg_get_vertex_data(lg_ctx* handle, float* light_out, float* diffuse_out) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (light_out) {
        if (!ctx->light_done) return ctx->fail(LG_ERR_STATE, "vertex light not computed");
        CK(cudaMemcpyAsync(light_out, ctx->d_L.p, sizeof(float) * 3 * ctx->n_points, cudaMemcpyDeviceToHost,
                           ctx->st), "L download");
    }
    if (diffuse_out) {
        if (!ctx->diffuse_done) return ctx->fail(LG_ERR_STATE, "diffusion not computed");
        CK(cudaMemcpyAsync(diffuse_out, ctx->d_D.p, sizeof(float) * 3 * ctx->n_points, cudaMemcpyDeviceToHost,
                           ctx->st), "D download");
    }
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return ctx->fw_wait_status();
}

// ---------------------------------------------------------------------------
// geometry dump (LightGraph::outputDebugGeo, src/LightGraph.h:604-696)
// ---------------------------------------------------------------------------

extern "C" lg_status lg_geo_dump(lg_ctx* handle, const char* dir, const char* stem, int first_iter) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!dir || !stem || first_iter < 0) return ctx->fail(LG_ERR_INVALID, "null directory or stem");
    if (!ctx->paths_solved || !ctx->light_done || !ctx->diffuse_done)
        return ctx->fail(LG_ERR_STATE, "the graphs are not solved (lg_solve_graphs first)");
    const int G = ctx->n_graphs;
    const int64_t P = ctx->n_points;
    std::vector<float> L(3 * std::max<int64_t>(P, 1)), D(3 * std::max<int64_t>(P, 1));
    std::vector<float> S((size_t)std::max<int64_t>(ctx->s_floats, 1));
    std::vector<int2> edges((size_t)std::max<int64_t>(ctx->edge_slots, 1));
    std::vector<int32_t> ecnt(G);
    CK(cudaMemcpyAsync(L.data(), ctx->d_L.p, sizeof(float) * 3 * P, cudaMemcpyDeviceToHost, ctx->st), "L download");
    CK(cudaMemcpyAsync(D.data(), ctx->d_D.p, sizeof(float) * 3 * P, cudaMemcpyDeviceToHost, ctx->st), "D download");
    CK(cudaMemcpyAsync(S.data(), ctx->d_S.p, sizeof(float) * ctx->s_floats, cudaMemcpyDeviceToHost, ctx->st),
       "S download");
    CK(cudaMemcpyAsync(edges.data(), ctx->d_edges.p, sizeof(int2) * ctx->edge_slots, cudaMemcpyDeviceToHost, ctx->st),
       "edge download");
    CK(cudaMemcpyAsync(ecnt.data(), ctx->d_edge_cnt.p, sizeof(int32_t) * G, cudaMemcpyDeviceToHost, ctx->st),
       "edge count download");
    CK(cudaStreamSynchronize(ctx->st), "sync");
    // create the directory if it does not exist (boost::filesystem::create_directory)
    ::mkdir(dir, 0755);
    const double* ext = ctx->shader.extinction;
    char name[4096];
    auto open = [&](const char* kind, int it) -> FILE* {
        std::snprintf(name, sizeof name, "%s/%s_%s_%04i.txt", dir, stem, kind, it);
        return std::fopen(name, "w");
    };
    // ostream's default formatting of a double: 6 significant digits
    auto v3 = [](FILE* f, double a, double b, double c) { std::fprintf(f, "%.6g,%.6g,%.6g\n", a, b, c); };
    for (int g = 0; g < G; ++g) {
        const GraphInfo& gi = ctx->h_graphs[g];
        const int n = gi.n, it = first_iter + g;
        const float* pts = ctx->h_pts.data() + 3 * gi.pt_off;
        FILE* f = open("pc", it);
        if (!f) return ctx->fail(LG_ERR_INVALID, "cannot write %s", name);
        for (int i = 0; i < n; ++i) v3(f, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        std::fclose(f);
        // the graph's edges in (i, j) row-major order
        std::vector<std::pair<int, int>> e;
        for (int k = 0; k < ecnt[g]; ++k) {
            const int2 p = edges[gi.e_off + k];
            e.push_back({std::min(p.x, p.y), std::max(p.x, p.y)});
        }
        std::sort(e.begin(), e.end());
        if (!(f = open("edge", it))) return ctx->fail(LG_ERR_INVALID, "cannot write %s", name);
        for (auto& p : e) std::fprintf(f, "%d,%d\n", p.first, p.second);
        std::fclose(f);
        // the path matrix as diffuseLight leaves it: T_c = exp(ext_c * S) after
        // the solve (diagonal 1), each column divided by max(column sum, 1)
        const float* Sg = S.data() + gi.s_off;
        std::vector<double> colsum(3 * (size_t)n, 0.0);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double sij = Sg[(size_t)i * gi.ld + j];
                for (int c = 0; c < 3; ++c) colsum[3 * (size_t)j + c] += std::exp(ext[c] * sij);
            }
        if (!(f = open("marching", it))) return ctx->fail(LG_ERR_INVALID, "cannot write %s", name);
        for (auto& p : e) {
            const double sij = Sg[(size_t)p.first * gi.ld + p.second];
            double t[3];
            for (int c = 0; c < 3; ++c) t[c] = std::exp(ext[c] * sij) / std::max(colsum[3 * (size_t)p.second + c], 1.0);
            v3(f, t[0], t[1], t[2]);
        }
        std::fclose(f);
        if (!(f = open("light", it))) return ctx->fail(LG_ERR_INVALID, "cannot write %s", name);
        for (int i = 0; i < n; ++i) {
            const float* l = L.data() + 3 * (gi.pt_off + i);
            v3(f, l[0], l[1], l[2]);
        }
        std::fclose(f);
        if (!(f = open("diffuse", it))) return ctx->fail(LG_ERR_INVALID, "cannot write %s", name);
        for (int i = 0; i < n; ++i) {
            const float* d = D.data() + 3 * (gi.pt_off + i);
            v3(f, d[0], d[1], d[2]);
        }
        std::fclose(f);
    }
    return LG_OK;
}

// ---------------------------------------------------------------------------
// stage 2: scatter grid
// ---------------------------------------------------------------------------

// points::computeVoxelSize(positions, 8) as LightGraph::buildVdbPointGrid
// calls it (src/LightGraph.h:713-714): OpenVDB's procedure with its defaults
// (identity transform, five decimal places). It starts from the points'
// bounding box, voxel = float(pow(volume / target, 1/3)) with target =
// max(1, n / points_per_voxel), then refines on the occupancy: the points
// fall into `count` distinct cell-centred voxels round(p / voxel), volume =
// float(voxel^3) * count, and the voxel is recomputed from that volume until
// the volume stops shrinking, the count stops growing or the voxel shrinks by
// less than 10%. The result is rounded to five decimal places (more if that
// gives 0). Occupancy is counted in a byte map over the points' cell box
// (a sort of the cell keys when that box is large).
namespace {
bool voxel_from_volume(double volume, size_t target, float& voxel) {
    const double fmax = (double)std::numeric_limits<float>::max();
    double vv = volume / (double)target;
    bool ok = true;
    if (vv < 3e-15) {
        vv = 3e-15;
        ok = false;
    } else if (vv > fmax * fmax * fmax) {
        vv = fmax * fmax * fmax;
        ok = false;
    }
    voxel = (float)std::pow(vv, 1.0 / 3.0);
    return ok;
}

int64_t occupied_voxels(int64_t n, const float* pts, const double lo[3], const double hi[3], float voxel) {
    const double inv = 1.0 / (double)voxel;
    int64_t c0[3], dim[3];
    int64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        // round(p * inv) is monotonic in p: the box of the cells is the cells of the box
        c0[a] = (int64_t)std::floor(lo[a] * inv + 0.5);
        dim[a] = (int64_t)std::floor(hi[a] * inv + 0.5) - c0[a] + 1;
        cells = (cells > (int64_t)1 << 40) ? cells : cells * dim[a];
    }
    if (cells <= ((int64_t)1 << 25)) {  // a byte map of at most 32 MB, else a sort of the keys
        std::vector<uint8_t> seen((size_t)cells, 0);
        int64_t count = 0;
        for (int64_t i = 0; i < n; ++i) {
            int64_t k = 0;
            for (int a = 2; a >= 0; --a)
                k = k * dim[a] + ((int64_t)std::floor((double)pts[3 * i + a] * inv + 0.5) - c0[a]);
            count += seen[(size_t)k] == 0;
            seen[(size_t)k] = 1;
        }
        return count;
    }
    std::vector<std::array<int64_t, 3>> keys((size_t)n);
    for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) keys[(size_t)i][a] = (int64_t)std::floor((double)pts[3 * i + a] * inv + 0.5);
    std::sort(keys.begin(), keys.end());
    return (int64_t)(std::unique(keys.begin(), keys.end()) - keys.begin());
}
}  // namespace

extern "C" double lg_point_voxel_size(int64_t n, const float* pts, int points_per_voxel) {
    float voxel = 0.1f;  // OpenVDB's default, kept for fewer than two or coincident points
    if (n <= 1 || !pts || points_per_voxel <= 0) return voxel;
    size_t target = (size_t)n / (size_t)points_per_voxel;
    if (target == 0) target = 1;
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = (double)pts[a];
    for (int64_t i = 1; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            const double v = (double)pts[3 * i + a];
            lo[a] = v < lo[a] ? v : lo[a];
            hi[a] = v > hi[a] ? v : hi[a];
        }
    if (lo[0] == hi[0] && lo[1] == hi[1] && lo[2] == hi[2]) return voxel;
    double ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    double volume = ext[0] * ext[1] * ext[2];
    if (std::fabs(volume) <= 1e-15) {  // coplanar: largest x next^2; collinear: largest^3
        std::sort(ext, ext + 3);
        volume = std::fabs(ext[1]) <= 1e-15 ? ext[2] * ext[2] * ext[2] : ext[2] * ext[1] * ext[1];
    }
    double prev_volume = volume;
    if (!voxel_from_volume(volume, target, voxel)) return voxel;
    int64_t prev_count = 0, count = 1;
    while (count > prev_count) {
        prev_count = count;
        count = occupied_voxels(n, pts, lo, hi, voxel);
        volume = (double)((voxel * voxel * voxel) * (float)count);
        if (volume >= prev_volume) break;
        prev_volume = volume;
        const float prev_voxel = voxel;
        if (!voxel_from_volume(volume, target, voxel)) {
            voxel = prev_voxel;
            break;
        }
        if (voxel / prev_voxel > 0.9f) break;
    }
    float out = voxel;
    double tenth = 1e5;
    for (int d = 5; d < 11; ++d, tenth *= 10.0) {
        out = (float)(std::floor((double)voxel * tenth + 0.5) / tenth);
        if (out != 0.0f) break;
    }
    return (double)out;
}

lg_status Ctx::splat(double point_voxel_size) {
    Ctx* ctx = this;
    if (!D().valid) return fail(LG_ERR_STATE, "no density grid uploaded");
    if (!diffuse_done) return fail(LG_ERR_STATE, "graphs not solved");
    const int f = settings.scatter_grid_res_factor;
    const lg_grid_desc& dd = D().desc;
    CoarseGrid cg;
    for (int a = 0; a < 3; ++a) {
        const int lo = floor_div(dd.origin[a], f) - 1;
        const int hi = floor_div(dd.origin[a] + dd.dims[a] - 1, f) + 1;
        cg.lo[a] = lo;
        cg.dims[a] = hi - lo + 1;
    }
    cg.H = (float)(dd.voxel_size * f);
    const int64_t ncoarse = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (topo_store != &D() || topo_version != D().version || topo_factor != f) {
        CK(d_act0.reserve(ncoarse), "coarse mask alloc");
        CK(d_act.reserve(ncoarse), "coarse mask alloc");
        CK(launch_coarse_topology(D().g, f, cg, d_act0.as<uint8_t>(), d_act.as<uint8_t>(), st), "coarse topology");
        topo_store = &D();
        topo_version = D().version;
        topo_factor = f;
    }
    double hp = point_voxel_size;
    if (!(hp > 0)) {
        if (point_voxel_size_cache < 0) point_voxel_size_cache = lg_point_voxel_size(n_points, h_pts.data(), 8);
        hp = point_voxel_size_cache;
    }
    // ScatterGrid::operator() kernel size (src/ScatterGrid.h:69-75), with
    // K = ptsPerKernel * iter (src/main.cc:586)
    const double K = (double)settings.pts_per_kernel * (double)settings.iter;
    const double hp3 = hp * hp * hp;
    const double radius = std::pow((3.0 * K * hp3) / (32.0 * 3.14159265358979323846), 1.0 / 3.0);
    const double sigma2 = -(radius * radius) / (2.0 * std::log(0.1));
    const float inv2s2 = (float)(1.0 / (2.0 * sigma2));
    // point bins
    PointBins pb{};
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (n_points > 0) {
        for (int a = 0; a < 3; ++a) { lo[a] = 1e300; hi[a] = -1e300; }
        for (int64_t i = 0; i < n_points; ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], (double)h_pts[3 * i + a]);
                hi[a] = std::max(hi[a], (double)h_pts[3 * i + a]);
            }
    }
    double cell = std::max(radius, 1e-12);
    double ext = 0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
    if (ext / cell > 159.0) cell = ext / 159.0;  // at most 160^3 cells (16 MB of bins)
    pb.cell = (float)cell;
    pb.n_cells = 1;
    for (int a = 0; a < 3; ++a) {
        pb.lo[a] = (float)lo[a];
        pb.dims[a] = (int)std::floor((hi[a] - lo[a]) / cell) + 1;
        pb.n_cells *= pb.dims[a];
    }
    const int64_t P = std::max<int64_t>(n_points, 1);
    CK(d_cell_count.reserve(sizeof(int32_t) * pb.n_cells), "bins alloc");
    CK(d_cell_start.reserve(sizeof(int32_t) * pb.n_cells), "bins alloc");
    CK(d_cursor.reserve(sizeof(int32_t) * pb.n_cells), "bins alloc");
    CK(d_scan_tmp.reserve(sizeof(int32_t) * ((pb.n_cells + 1023) / 1024 + 1)), "bins alloc");
    CK(d_sorted.reserve(sizeof(int32_t) * P), "bins alloc");
    CK(launch_bin_points(d_pts.as<float>(), n_points, pb, d_cell_count.as<int32_t>(), d_cell_start.as<int32_t>(),
                         d_cursor.as<int32_t>(), d_sorted.as<int32_t>(), d_scan_tmp.as<int32_t>(), st), "bin points");
    CK(d_sg.reserve(sizeof(float4) * ncoarse), "scatter grid alloc");
    CK(launch_splat(cg, d_act.as<uint8_t>(), d_pts.as<float>(), d_D.as<float>(), pb, d_cell_start.as<int32_t>(),
                    d_cell_count.as<int32_t>(), d_sorted.as<int32_t>(), (float)radius, inv2s2, d_sg.as<float4>(), st),
       "splat");
    coarse = cg;
    splat_done = true;
    splat_radius = radius;
    return LG_OK;
}

extern "C" lg_status lg_splat(lg_ctx* handle, double point_voxel_size) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    lg_status s = ctx->splat(point_voxel_size);
    if (s != LG_OK) return s;
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return LG_OK;
}

extern "C" lg_status lg_get_scatter_grid(lg_ctx* handle, int32_t dims[3], int32_t origin[3], float* values) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->splat_done) return ctx->fail(LG_ERR_STATE, "no scatter grid");
    for (int a = 0; a < 3; ++a) {
        if (dims) dims[a] = ctx->coarse.dims[a];
        if (origin) origin[a] = ctx->coarse.lo[a];
    }
    if (values) {
        const int64_t n = (int64_t)ctx->coarse.dims[0] * ctx->coarse.dims[1] * ctx->coarse.dims[2];
        std::vector<float4> tmp(n);
        CK(cudaMemcpyAsync(tmp.data(), ctx->d_sg.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->st),
           "scatter grid download");
        CK(cudaStreamSynchronize(ctx->st), "sync");
        for (int64_t i = 0; i < n; ++i) {
            values[3 * i] = tmp[i].x;
            values[3 * i + 1] = tmp[i].y;
            values[3 * i + 2] = tmp[i].z;
        }
    }
    return LG_OK;
}

// ---------------------------------------------------------------------------
// stage 3: render
// ---------------------------------------------------------------------------

lg_status Ctx::render_count(const lg_camera* c, cudaStream_t s) {
    Ctx* ctx = this;
    if (!c) return fail(LG_ERR_INVALID, "null camera");
    if (c->width <= 0 || c->height <= 0 || c->samples < 0) return fail(LG_ERR_INVALID, "bad image size or samples");
    if (!(c->focal > 0) || !(c->aperture > 0)) return fail(LG_ERR_INVALID, "bad focal length or aperture");
    if (!(c->znear > 0) || !(c->zfar > c->znear)) return fail(LG_ERR_INVALID, "need 0 < znear < zfar");
    if (!D().valid) return fail(LG_ERR_STATE, "no density grid uploaded");
    const int64_t np = (int64_t)c->width * c->height;
    const int64_t n_ps = np * c->samples;
    if (n_ps > INT32_MAX) return fail(LG_ERR_INVALID, "too many pixel samples");
    for (DevBuf* b : {&d_rgba, &d_direct, &d_scatter, &d_emission}) CK(b->reserve(sizeof(float4) * np), "film alloc");
    // primary samples, shadow samples, and the claim counters of the shadow
    // wave, the count pass and the shading pass
    CK(d_counters.reserve(5 * sizeof(unsigned long long)), "counter alloc");
    CK(cudaMemsetAsync(d_counters.p, 0, 5 * sizeof(unsigned long long), s), "counter clear");
    const int64_t nps1 = std::max<int64_t>(n_ps, 1);
    CK(d_ps_count.reserve(sizeof(int32_t) * nps1), "render alloc");
    CK(d_ps_offset.reserve(sizeof(int32_t) * nps1), "render alloc");
    CK(d_ps_scan.reserve(sizeof(int32_t) * (nps1 / 1024 + 2)), "render alloc");
    CK(d_ps_total.reserve(sizeof(int32_t) * 2), "render alloc");
    CK(d_ps_data.reserve(pixel_sample_bytes() * nps1), "render alloc");
    const DevScene sc = scene();
    const DevCamera cam = make_camera(*c);
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device query");
    wmark(0, s);
    // (the count pass reads no scatter grid); beside the graph stages (the
    // side stream, of the lowest priority) as short CTAs, so that the
    // stages' kernels take the SMs as they free up
    CK(launch_render_count(sc, cam, DevScatterGrid{}, d_ps_count.as<int32_t>(), d_counters.as<unsigned long long>() + 3,
                           sms, s, s != st),
       "render count");
    CK(launch_exclusive_scan(d_ps_count.as<int32_t>(), n_ps, d_ps_offset.as<int32_t>(), d_ps_scan.as<int32_t>(),
                             d_ps_total.as<int32_t>(), s), "render scan");
    wmark(1, s);
    return LG_OK;
}

lg_status Ctx::render_count_early(const lg_camera* c) {
    Ctx* ctx = this;
    CK(cudaEventRecord(ev_fork, st), "fork");
    CK(cudaStreamWaitEvent(st2, ev_fork, 0), "fork");
    const lg_status r = render_count(c, st2);
    CK(cudaEventRecord(ev_count, st2), "join");
    if (r != LG_OK) {
        // keep st2 joined to st (a capture must end with it joined)
        CK(cudaStreamWaitEvent(st, ev_count, 0), "join");
        return r;
    }
    count_early = true;
    count_cam = *c;
    return LG_OK;
}

lg_status Ctx::render(const lg_camera* c) {
    Ctx* ctx = this;
    if (!c) return fail(LG_ERR_INVALID, "null camera");
    const bool early = count_early && std::memcmp(&count_cam, c, sizeof(lg_camera)) == 0;
    if (count_early) {
        // the early count ends before anything that follows on st
        CK(cudaStreamWaitEvent(st, ev_count, 0), "join");
        count_early = false;
    }
    if (!early) {
        const lg_status r = render_count(c, st);
        if (r != LG_OK) return r;
    }
    waves_recorded = false;
    wave_split = early;
    DevScatterGrid sg{};
    if (splat_done) {
        sg.v = d_sg.as<float4>();
        for (int a = 0; a < 3; ++a) {
            sg.lo[a] = coarse.lo[a];
            sg.dims[a] = coarse.dims[a];
        }
        sg.inv_H = 1.f / coarse.H;
    } else {
        // no multiple scattering estimate yet: an empty grid reads 0
        sg.v = nullptr;
        sg.inv_H = 1.f;
    }
    film_w = c->width;
    film_h = c->height;
    const DevScene sc = scene();
    const DevCamera cam = make_camera(*c);
    const int64_t n_lights = std::max(sc.n_lights, 1);
    if (!capturing) {
        // size the shadow-task buffers from this frame's count (a captured
        // replay reuses the capacity of the run it was captured after); an
        // early count is read on its own stream, so the host does not wait
        // for the graph stages
        int32_t total = 0;
        cudaStream_t rs = early ? st2 : st;
        CK(cudaMemcpyAsync(&total, d_ps_total.p, sizeof total, cudaMemcpyDeviceToHost, rs), "render total");
        CK(cudaStreamSynchronize(rs), "render total sync");
        if (total < 0) return fail(LG_ERR_INVALID, "more than 2^31 shading samples in one frame");
        if ((int64_t)total * n_lights > INT32_MAX)
            return fail(LG_ERR_INVALID, "more than 2^31 shadow-ray groups in one frame");
        CK(d_tasks.reserve(sizeof(ShadowTask) * std::max<int64_t>(total, 1)), "shadow task alloc");
    }
    const int64_t cap = std::min<int64_t>((int64_t)(d_tasks.bytes / sizeof(ShadowTask)), INT32_MAX / n_lights);
    RayOrder ro{};
    ro.rb = ray_bins(sc, cap);
    ro.n_keys = 0;
    for (int k = 0; k < ro.rb.n; ++k) ro.n_keys += ro.rb.b[k].nkeys;
    if (ro.n_keys >= INT32_MAX) return fail(LG_ERR_INVALID, "more than 2^31 shadow-ray order keys");
    const size_t order_bytes = sizeof(int32_t) * (size_t)(n_lights * ((cap + kRayUnit - 1) / kRayUnit));
    const size_t direct_bytes = sizeof(float4) * (size_t)(n_lights * cap);
    const size_t key_bytes = sizeof(int32_t) * (size_t)std::max<int64_t>(ro.n_keys, 1);
    const size_t scan_bytes = sizeof(int32_t) * (size_t)(std::max<int64_t>(ro.n_keys, 1) / 1024 + 2);
    if (!capturing) {
        CK(d_task_direct.reserve(direct_bytes), "shadow task alloc");
        CK(d_ray_order.reserve(order_bytes), "ray order alloc");
        CK(d_ray_keys.reserve(order_bytes), "ray order alloc");
        CK(d_ray_counts.reserve(key_bytes), "ray order alloc");
        CK(d_ray_offsets.reserve(key_bytes), "ray order alloc");
        CK(d_ray_scan.reserve(scan_bytes), "ray order alloc");
        CK(d_ray_total.reserve(sizeof(int32_t) * 2), "ray order alloc");
    } else if (d_task_direct.bytes < direct_bytes || d_ray_order.bytes < order_bytes || d_ray_keys.bytes < order_bytes ||
               d_ray_counts.bytes < key_bytes || d_ray_offsets.bytes < key_bytes || d_ray_scan.bytes < scan_bytes ||
               d_ray_total.bytes < sizeof(int32_t) * 2) {
        return fail(LG_ERR_STATE, "render buffers changed size during graph capture");
    }
    // occupancy bounds of the distant and point lights' bins (rebuilt every
    // render: one short kernel over the leaf bitmap)
    {
        int64_t entries = 0;
        for (int k = 0; k < ro.rb.n; ++k) entries += bound_entries(ro.rb.b[k]);
        if (!capturing) CK(d_ray_bounds.reserve(sizeof(float) * (size_t)std::max<int64_t>(entries, 1)), "ray bound alloc");
        else if (d_ray_bounds.bytes < sizeof(float) * (size_t)std::max<int64_t>(entries, 1))
            return fail(LG_ERR_STATE, "render buffers changed size during graph capture");
        int64_t off = 0;
        for (int k = 0; k < ro.rb.n; ++k) {
            RayBin& b = ro.rb.b[k];
            const int64_t ne = bound_entries(b);
            if (ne == 0) continue;
            b.bound = d_ray_bounds.as<float>() + off;
            off += ne;
            if (b.kind == 0) CK(cudaMemsetAsync(b.bound, 0, sizeof(float) * (size_t)ne, st), "ray bound clear");
            else CK(launch_fill(b.bound, ne, kInf, st), "ray bound clear");
        }
        if (off > 0) CK(launch_ray_bounds(sc.dens, ro.rb, st), "ray bounds");
    }
    ro.key_counts = d_ray_counts.as<int32_t>();
    ro.key_offsets = d_ray_offsets.as<int32_t>();
    ro.key_scan = d_ray_scan.as<int32_t>();
    ro.key_total = d_ray_total.as<int32_t>();
    ro.order = d_ray_order.as<int32_t>();
    ro.keys = d_ray_keys.as<uint32_t>();
    ro.unit_cap = (cap + kRayUnit - 1) / kRayUnit;
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device query");
    if (early && profiling && wev_shade) cudaEventRecord(wev_shade, st);
    CK(launch_render_shade(sc, cam, sg, d_ps_count.as<int32_t>(), d_ps_offset.as<int32_t>(), d_ps_total.as<int32_t>(),
                           d_tasks.as<ShadowTask>(), cap, d_ps_data.p, ro, d_task_direct.as<float4>(),
                           d_rgba.as<float4>(), d_direct.as<float4>(), d_scatter.as<float4>(),
                           d_emission.as<float4>(), d_counters.as<unsigned long long>(), sms, st,
                           profiling ? wev + 2 : nullptr),
       "render");
    waves_recorded = profiling;
    return LG_OK;
}

lg_status Ctx::download_films(float* rgba, float* direct, float* scatter, float* emission) {
    Ctx* ctx = this;
    const int64_t np = (int64_t)film_w * film_h;
    const void* src[4] = {d_rgba.p, d_direct.p, d_scatter.p, d_emission.p};
    float* dst[4] = {rgba, direct, scatter, emission};
    for (int k = 0; k < 4; ++k)
        if (dst[k]) CK(cudaMemcpyAsync(dst[k], src[k], sizeof(float4) * np, cudaMemcpyDeviceToHost, st), "film download");
    CK(cudaStreamSynchronize(st), "sync");
    return fw_wait_status();
}

extern "C" lg_status lg_render(lg_ctx* handle, const lg_camera* camera, float* rgba, float* direct,
                               float* scatter, float* emission) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    lg_status s = ctx->render(camera);
    if (s != LG_OK) return s;
    return ctx->download_films(rgba, direct, scatter, emission);
}

extern "C" lg_status lg_get_films(lg_ctx* handle, float* rgba, float* direct, float* scatter, float* emission) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (ctx->film_w == 0) return ctx->fail(LG_ERR_STATE, "nothing rendered yet");
    return ctx->download_films(rgba, direct, scatter, emission);
}

extern "C" lg_status lg_render_stats(lg_ctx* handle, uint64_t* primary, uint64_t* shadow, uint64_t* shading) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    unsigned long long c[2] = {0, 0};
    int32_t tasks = 0;
    if (ctx->d_counters.bytes >= sizeof c) {
        CK(cudaMemcpyAsync(c, ctx->d_counters.p, sizeof c, cudaMemcpyDeviceToHost, ctx->st), "counter download");
        if (ctx->d_ps_total.bytes >= sizeof tasks)
            CK(cudaMemcpyAsync(&tasks, ctx->d_ps_total.p, sizeof tasks, cudaMemcpyDeviceToHost, ctx->st), "task count");
        CK(cudaStreamSynchronize(ctx->st), "sync");
    }
    if (primary) *primary = c[0];
    if (shadow) *shadow = c[1];
    if (shading) *shading = (uint64_t)tasks;
    return LG_OK;
}

extern "C" lg_status lg_render_frame(lg_ctx* handle, int n_graphs, const float* points,
                                     const int64_t* offsets, const float* radius_sq, int max_connect,
                                     double point_voxel_size, const lg_camera* camera, float* rgba,
                                     float* direct, float* scatter, float* emission) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    lg_status s = ctx->load_graphs(n_graphs, points, offsets, radius_sq, max_connect);
    // the render's count pass runs beside the graph stages (side stream)
    if (s == LG_OK) s = ctx->render_count_early(camera);
    if (s == LG_OK) s = ctx->build_edges();
    if (s == LG_OK) s = ctx->solve_all();
    if (s == LG_OK) s = ctx->splat(point_voxel_size);
    if (s == LG_OK) s = ctx->render(camera);
    if (s == LG_OK) s = ctx->download_films(rgba, direct, scatter, emission);
    if (s != LG_OK && ctx->count_early) {
        // a stage failed before render(): join the side stream again
        cudaStreamWaitEvent(ctx->st, ctx->ev_count, 0);
        ctx->count_early = false;
    }
    return s;
}

extern "C" lg_status lg_frame_device(lg_ctx* handle, int max_connect, double point_voxel_size,
                                     const lg_camera* camera) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (ctx->n_graphs == 0) return ctx->fail(LG_ERR_STATE, "no graphs loaded");
    if (max_connect < 0 || max_connect > 255) return ctx->fail(LG_ERR_INVALID, "bad max_connect");
    if (max_connect != ctx->max_connect) return ctx->fail(LG_ERR_INVALID, "max_connect differs from the loaded graphs");
    if (!camera) return ctx->fail(LG_ERR_INVALID, "null camera");
    if (!ctx->graph_mode) return ctx->frame_enqueue(point_voxel_size, camera);
    if (ctx->graph_valid && ctx->graph_epoch == g_alloc_epoch && ctx->graph_pvs == point_voxel_size &&
        std::memcmp(&ctx->graph_cam, camera, sizeof(lg_camera)) == 0) {
        CK(cudaGraphLaunch(ctx->graph_exec, ctx->st), "frame graph launch");
        ++g_launch_counter;
        ctx->ev_recorded = ctx->profiling;
        ctx->waves_recorded = ctx->profiling;
        return LG_OK;
    }
    // run the frame once (this also tunes and allocates), then capture the
    // same launch sequence for replay
    ctx->fw_order_next = true;
    lg_status s = ctx->frame_enqueue(point_voxel_size, camera);
    ctx->fw_order_next = false;
    if (s != LG_OK) return s;
    CK(cudaStreamSynchronize(ctx->st), "sync");
    if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
    if (ctx->graph) { cudaGraphDestroy(ctx->graph); ctx->graph = nullptr; }
    const uint64_t launches = g_launch_counter;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    ctx->capturing = true;
    s = ctx->frame_enqueue(point_voxel_size, camera);
    ctx->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->st, &graph);
    const uint64_t captured = g_launch_counter - launches;
    g_launch_counter -= captured;  // captured, not launched
    if (s != LG_OK) { if (graph) cudaGraphDestroy(graph); return s; }
    CK(ce, "end capture");
    ctx->graph = graph;
    CK(cudaGraphInstantiate(&ctx->graph_exec, graph, 0), "graph instantiate");
    ctx->graph_valid = true;
    ctx->graph_epoch = g_alloc_epoch;
    ctx->graph_cam = *camera;
    ctx->graph_pvs = point_voxel_size;
    ctx->frame_launches = captured;
    return LG_OK;
}

lg_status Ctx::frame_enqueue(double point_voxel_size, const lg_camera* camera) {
    frame_launch_base = g_launch_counter;
    mark(0);
    // the render's count pass runs beside the graph stages (side stream)
    lg_status s = render_count_early(camera);
    if (s == LG_OK) s = build_edges();
    mark(1);
    if (s == LG_OK) s = march_edges();
    mark(2);
    if (s == LG_OK) { s = solve_paths(); paths_solved = s == LG_OK; }
    mark(3);
    if (s == LG_OK) { s = vertex_light(); light_done = s == LG_OK; }
    mark(4);
    if (s == LG_OK) { s = diffuse(); diffuse_done = s == LG_OK; }
    mark(5);
    if (s == LG_OK) s = splat(point_voxel_size);
    mark(6);
    if (s == LG_OK) s = render(camera);
    if (s != LG_OK && count_early) {
        // a stage failed before render(): join the side stream again
        cudaStreamWaitEvent(st, ev_count, 0);
        count_early = false;
    }
    mark(7);
    ev_recorded = profiling && s == LG_OK;
    return s;
}

extern "C" lg_status lg_render_wave_times(lg_ctx* handle, double ms[5]) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->waves_recorded || !ctx->wev[Ctx::kWaves]) return ctx->fail(LG_ERR_STATE, "no profiled render");
    if (!ms) return ctx->fail(LG_ERR_INVALID, "null output");
    CK(cudaEventSynchronize(ctx->wev[Ctx::kWaves]), "event sync");
    for (int k = 0; k < Ctx::kWaves; ++k) {
        float t = 0.f;
        // after an early count (on the side stream) the shading wave starts
        // at its own mark
        const cudaEvent_t from = k == 1 && ctx->wave_split ? ctx->wev_shade : ctx->wev[k];
        CK(cudaEventElapsedTime(&t, from, ctx->wev[k + 1]), "event time");
        ms[k] = t;
    }
    return LG_OK;
}

extern "C" lg_status lg_set_graph_mode(lg_ctx* handle, int on) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    ctx->graph_mode = on != 0;
    ctx->graph_valid = false;
    return LG_OK;
}

extern "C" lg_status lg_set_fw_schedule(lg_ctx* handle, int schedule) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (schedule < -1 || schedule > 5) return ctx->fail(LG_ERR_INVALID, "schedule must be -1, 0, 1, 2, 3, 4 or 5");
    ctx->fw_pinned = schedule;
    if (schedule == -1) {
        ctx->fw_choice = -1;
        for (auto& kv : ctx->fw_tuned)
            if (kv.first == std::make_pair(ctx->n_graphs, ctx->max_n)) ctx->fw_choice = kv.second;
    } else {
        ctx->fw_choice = schedule;
    }
    ctx->graph_valid = false;
    return LG_OK;
}

extern "C" lg_status lg_fw_schedule(lg_ctx* handle, int* schedule, double* tuned_ms, int n) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (schedule) *schedule = ctx->fw_choice;
    for (int k = 0; tuned_ms && k < n && k < kFwSchedules; ++k) tuned_ms[k] = ctx->fw_tune_ms[k];
    if (ctx->fw_choice > 0 && ctx->d_fw_sync.bytes >= 8) {
        uint32_t flags[2] = {0, 0};
        CK(cudaMemcpyAsync(flags, ctx->d_fw_sync.p, sizeof flags, cudaMemcpyDeviceToHost, ctx->st), "flag read");
        CK(cudaStreamSynchronize(ctx->st), "sync");
        if (flags[1] != 0) return ctx->fail(LG_ERR_TIMEOUT, "batched floyd-warshall: a dependency wait timed out");
    }
    return LG_OK;
}

extern "C" lg_status lg_fw_inner_loop_rate(lg_ctx* handle, double* tflops, float* sums) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!tflops) return ctx->fail(LG_ERR_INVALID, "tflops is null");
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "device query");
    DevBuf scratch;
    CK(scratch.reserve(sizeof(float) * 2 * sms * 256), "scratch alloc");
    CK(fw_inner_loop_rate(scratch.as<float>(), sms, tflops, ctx->st), "inner loop rate");
    if (sums) CK(cudaMemcpy(sums, scratch.p, sizeof(float) * 256, cudaMemcpyDeviceToHost), "inner loop sums");
    return LG_OK;
}

extern "C" lg_status lg_expm1_check(lg_ctx* handle, const float* x, float* approx, float* ref, int32_t n) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (n < 0 || (n > 0 && (!x || !approx || !ref))) return ctx->fail(LG_ERR_INVALID, "bad expm1 check arguments");
    if (n == 0) return LG_OK;
    DevBuf buf;
    CK(buf.reserve(sizeof(float) * 3 * (size_t)n), "expm1 check alloc");
    float* dx = buf.as<float>();
    CK(cudaMemcpyAsync(dx, x, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->st), "expm1 check upload");
    CK(launch_expm1_check(dx, dx + n, dx + 2 * (size_t)n, n, ctx->st), "expm1 check");
    CK(cudaMemcpyAsync(approx, dx + n, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->st), "expm1 check read");
    CK(cudaMemcpyAsync(ref, dx + 2 * (size_t)n, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->st), "expm1 check read");
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return LG_OK;
}

extern "C" lg_status lg_wait_timeout_check(lg_ctx* handle, uint32_t polls) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (polls < 1 || polls > (1u << 24)) return ctx->fail(LG_ERR_INVALID, "polls must be in [1, 2^24]");
    CK(ctx->small.reserve(64), "small alloc");
    CK(cudaMemsetAsync(ctx->small.p, 0, 4 * sizeof(uint32_t), ctx->st), "probe clear");
    CK(wait_probe(ctx->small.as<uint32_t>(), polls, ctx->st), "wait probe");
    uint32_t w[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(w, ctx->small.p, sizeof w, cudaMemcpyDeviceToHost, ctx->st), "probe read");
    CK(cudaStreamSynchronize(ctx->st), "sync");
    if (w[2] == 1u && w[1] != 0u) return ctx->fail(LG_ERR_TIMEOUT, "the bounded wait gave up after %u polls", polls);
    return ctx->fail(LG_ERR_STATE, "the bounded wait did not give up (error word %u, outcome %u)", w[1], w[2]);
}

extern "C" lg_status lg_fw_queue_check(int n_graphs, const int32_t* sizes, int sym, int64_t* n_items) {
    if (n_graphs < 0 || (n_graphs > 0 && !sizes)) return LG_ERR_INVALID;
    std::vector<FwGraph> fg(n_graphs);
    int64_t vofs = 0, pofs = 0;
    for (int g = 0; g < n_graphs; ++g) {
        if (sizes[g] < 0) return LG_ERR_INVALID;
        const int ld = (sizes[g] + 127) / 128 * 128;
        fg[g].off = 0;
        fg[g].n = ld;
        fg[g].ld = ld;
        fg[g].nt = sizes[g] == 0 ? 0 : ld / 64;
        fg[g].nu = sizes[g] == 0 ? 0 : ld / 128;
        fg[g].vofs = vofs;
        fg[g].pofs = pofs;
        vofs += (int64_t)fg[g].nt * fg[g].nt + fg[g].nt;
        pofs += (int64_t)fw_panel_words(fg[g]);
    }
    const size_t n = fw_batched_items(fg.data(), n_graphs, nullptr, sym != 0);
    std::vector<int4> items(std::max<size_t>(n, 1));
    fw_batched_items(fg.data(), n_graphs, items.data(), sym != 0);
    if (n_items) *n_items = (int64_t)n;
    if (fw_queue_replay(fg.data(), n_graphs, items.data(), n, sym != 0) != 0) return LG_ERR_STATE;
    if (sym) {
        // the list-scheduled order the solve runs, for 152 and 304 CTAs
        for (int workers : {152, 304}) {
            std::vector<int4> ordered = items;
            fw_order_sym(fg.data(), n_graphs, ordered.data(), n, workers);
            if (fw_queue_replay(fg.data(), n_graphs, ordered.data(), n, true) != 0) return LG_ERR_STATE;
        }
    }
    return LG_OK;
}

extern "C" uint64_t lg_frame_launches(const lg_ctx* handle) {
    const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
    return ctx ? ctx->frame_launches : 0;
}

extern "C" lg_status lg_set_profiling(lg_ctx* handle, int on) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (on && !ctx->ev[0]) {
        for (int k = 0; k <= Ctx::kStages; ++k) CK(cudaEventCreate(&ctx->ev[k]), "event create");
        for (int k = 0; k <= Ctx::kWaves; ++k) CK(cudaEventCreate(&ctx->wev[k]), "event create");
        CK(cudaEventCreate(&ctx->wev_shade), "event create");
    }
    ctx->profiling = on != 0;
    ctx->graph_valid = false;
    ctx->ev_recorded = false;
    return LG_OK;
}

extern "C" lg_status lg_stage_times(lg_ctx* handle, double* ms, int n) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (!ctx->ev_recorded) return ctx->fail(LG_ERR_STATE, "no profiled frame");
    if (!ms || n < 1) return ctx->fail(LG_ERR_INVALID, "bad output");
    CK(cudaEventSynchronize(ctx->ev[Ctx::kStages]), "event sync");
    for (int k = 0; k < n && k < Ctx::kStages; ++k) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, ctx->ev[k], ctx->ev[k + 1]), "event time");
        ms[k] = t;
    }
    return LG_OK;
}

// ---------------------------------------------------------------------------
// kernel-level entry points
// ---------------------------------------------------------------------------

extern "C" lg_status lg_fw_device(float* dist, int n, int ld, void* stream) {
    if (n < 0 || ld < n || (n > 0 && !dist)) return LG_ERR_INVALID;
    if (ld % 4 != 0 || (reinterpret_cast<uintptr_t>(dist) & 15) != 0) return LG_ERR_INVALID;
    const cudaError_t e = fw_solve(dist, n, ld, (cudaStream_t)stream);
    return e == cudaSuccess ? LG_OK : LG_ERR_CUDA;
}

extern "C" lg_status lg_fw_host(lg_ctx* handle, float* dist, int n) {
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    GUARD(ctx);
    if (n < 0 || (n > 0 && !dist)) return ctx->fail(LG_ERR_INVALID, "bad matrix");
    if (n == 0) return LG_OK;
    const int ld = round_up(n, 4);
    CK(ctx->d_fw.reserve(sizeof(float) * (size_t)n * ld), "fw alloc");
    CK(cudaMemcpy2DAsync(ctx->d_fw.p, sizeof(float) * ld, dist, sizeof(float) * n, sizeof(float) * n, n,
                         cudaMemcpyHostToDevice, ctx->st), "fw upload");
    CK(fw_solve(ctx->d_fw.as<float>(), n, ld, ctx->st), "floyd-warshall");
    CK(cudaMemcpy2DAsync(dist, sizeof(float) * n, ctx->d_fw.p, sizeof(float) * ld, sizeof(float) * n, n,
                         cudaMemcpyDeviceToHost, ctx->st), "fw download");
    CK(cudaStreamSynchronize(ctx->st), "sync");
    return LG_OK;
}

