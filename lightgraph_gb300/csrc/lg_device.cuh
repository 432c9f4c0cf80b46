// Device-side building blocks of the LightGraph path: the brick-tiled grid and
// its trilinear sampler, the leaf-level span march that stands in for
// OpenVDB's VolumeRayIntersector/VolumeHDDA, shading, lights and the
// environment-map sampler. All kernels include this header.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "lg_rng.h"

namespace lg {

constexpr float kInf = __builtin_huge_valf();
constexpr int kMaxLights = 8;
constexpr int kMaxRamp = 16;
// OpenVDB math::Delta<double>::value(): default ray start time and the
// minimum length of a valid span (src/Renderer.h:347,368).
constexpr float kDelta = 1e-9f;

// ---------------------------------------------------------------------------
// Grid: voxels stored as 8^3 bricks (x fastest inside a brick), bricks in a
// dense box (x fastest) with one brick of zero padding on every side. A voxel
// outside the box reads the background value 0.
// ---------------------------------------------------------------------------
struct DevGrid {
    const void* data = nullptr;
    const uint32_t* leafbits = nullptr;  // one bit per brick of the box: leaf exists
    int dtype = 0;                       // 0 f32, 1 f16, 2 bf16
    int blo[3] = {0, 0, 0};              // brick coordinate of box brick 0
    int nb[3] = {0, 0, 0};               // bricks per axis
    float inv_h = 1.f;                   // 1 / voxel size
    float h = 1.f;                       // voxel size
    float wo[3] = {0.f, 0.f, 0.f};       // world origin
    float bbmin[3] = {0.f, 0.f, 0.f};    // leaf bbox in index space (origin of min leaf)
    float bbmax[3] = {0.f, 0.f, 0.f};    // ... max leaf origin + 8
    int has_leaves = 0;
    uint32_t sy = 0, sz = 0;             // element strides of one brick step in y and z
};

template <int DT>
__device__ __forceinline__ float ldv(const void* data, uint32_t off) {
    if (DT == 0) return __ldg(reinterpret_cast<const float*>(data) + off);
    if (DT == 1) return __half2float(__ldg(reinterpret_cast<const __half*>(data) + off));
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(data) + off));
}

// Trilinear sample for storage type DT without branches: per axis, the brick
// and in-brick offsets of the two taps are computed once, the eight offsets
// are sums of them, and taps outside the brick box read 0 through a
// predicated load. Offsets are 32-bit (the upload rejects grids whose brick
// box has 2^32 or more elements). Same taps and interpolation order as
// sample_index.
template <int DT>
__device__ __forceinline__ float sample_index_t(const DevGrid& g, float px, float py, float pz) {
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float wx = px - fx, wy = py - fy, wz = pz - fz;
    const int bx0 = (ix >> 3) - g.blo[0], bx1 = ((ix + 1) >> 3) - g.blo[0];
    const int by0 = (iy >> 3) - g.blo[1], by1 = ((iy + 1) >> 3) - g.blo[1];
    const int bz0 = (iz >> 3) - g.blo[2], bz1 = ((iz + 1) >> 3) - g.blo[2];
    const bool vx0 = (unsigned)bx0 < (unsigned)g.nb[0], vx1 = (unsigned)bx1 < (unsigned)g.nb[0];
    const bool vy0 = (unsigned)by0 < (unsigned)g.nb[1], vy1 = (unsigned)by1 < (unsigned)g.nb[1];
    const bool vz0 = (unsigned)bz0 < (unsigned)g.nb[2], vz1 = (unsigned)bz1 < (unsigned)g.nb[2];
    const uint32_t ox0 = (uint32_t)bx0 * 512u + (uint32_t)(ix & 7);
    const uint32_t ox1 = (uint32_t)bx1 * 512u + (uint32_t)((ix + 1) & 7);
    const uint32_t oy0 = (uint32_t)by0 * g.sy + (uint32_t)(iy & 7) * 8u;
    const uint32_t oy1 = (uint32_t)by1 * g.sy + (uint32_t)((iy + 1) & 7) * 8u;
    const uint32_t oz0 = (uint32_t)bz0 * g.sz + (uint32_t)(iz & 7) * 64u;
    const uint32_t oz1 = (uint32_t)bz1 * g.sz + (uint32_t)((iz + 1) & 7) * 64u;
    const uint32_t o00 = oy0 + oz0, o10 = oy1 + oz0, o01 = oy0 + oz1, o11 = oy1 + oz1;
    const bool v00 = vy0 && vz0, v10 = vy1 && vz0, v01 = vy0 && vz1, v11 = vy1 && vz1;
    const void* D = g.data;
    // v[x][y][z]
    const float v000 = (vx0 && v00) ? ldv<DT>(D, ox0 + o00) : 0.f;
    const float v100 = (vx1 && v00) ? ldv<DT>(D, ox1 + o00) : 0.f;
    const float v010 = (vx0 && v10) ? ldv<DT>(D, ox0 + o10) : 0.f;
    const float v110 = (vx1 && v10) ? ldv<DT>(D, ox1 + o10) : 0.f;
    const float v001 = (vx0 && v01) ? ldv<DT>(D, ox0 + o01) : 0.f;
    const float v101 = (vx1 && v01) ? ldv<DT>(D, ox1 + o01) : 0.f;
    const float v011 = (vx0 && v11) ? ldv<DT>(D, ox0 + o11) : 0.f;
    const float v111 = (vx1 && v11) ? ldv<DT>(D, ox1 + o11) : 0.f;
    const float y00 = fmaf(v001 - v000, wz, v000), y01 = fmaf(v011 - v010, wz, v010);
    const float y10 = fmaf(v101 - v100, wz, v100), y11 = fmaf(v111 - v110, wz, v110);
    const float x0 = fmaf(y01 - y00, wy, y00), x1 = fmaf(y11 - y10, wy, y10);
    return fmaf(x1 - x0, wx, x0);
}

__device__ __forceinline__ float load_voxel(const DevGrid& g, int64_t off) {
    if (g.dtype == 0) return __ldg(reinterpret_cast<const float*>(g.data) + off);
    if (g.dtype == 1) return __half2float(__ldg(reinterpret_cast<const __half*>(g.data) + off));
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(g.data) + off));
}

// Linear offset of voxel (x, y, z), or -1 when outside the brick box.
__device__ __forceinline__ int64_t voxel_offset(const DevGrid& g, int x, int y, int z) {
    const int bx = (x >> 3) - g.blo[0], by = (y >> 3) - g.blo[1], bz = (z >> 3) - g.blo[2];
    if ((unsigned)bx >= (unsigned)g.nb[0] || (unsigned)by >= (unsigned)g.nb[1] ||
        (unsigned)bz >= (unsigned)g.nb[2])
        return -1;
    const int64_t b = ((int64_t)bz * g.nb[1] + by) * g.nb[0] + bx;
    return b * 512 + (((z & 7) * 8 + (y & 7)) * 8 + (x & 7));
}

__device__ __forceinline__ float voxel(const DevGrid& g, int x, int y, int z) {
    const int64_t off = voxel_offset(g, x, y, z);
    return off < 0 ? 0.f : load_voxel(g, off);
}

__device__ __forceinline__ float lerpf(float a, float b, float w) { return fmaf(b - a, w, a); }

// Trilinear sample at an index-space position: the eight voxels around
// floor(p), interpolated along z, then y, then x (the order of OpenVDB's
// BoxSampler::trilinearInterpolation).
__device__ __forceinline__ float sample_index(const DevGrid& g, float px, float py, float pz) {
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float wx = px - fx, wy = py - fy, wz = pz - fz;
    float v000, v001, v010, v011, v100, v101, v110, v111;  // v[x][y][z]
    const int64_t o = voxel_offset(g, ix, iy, iz);
    if (o >= 0 && (ix & 7) != 7 && (iy & 7) != 7 && (iz & 7) != 7) {
        // all eight taps inside one brick
        v000 = load_voxel(g, o);
        v100 = load_voxel(g, o + 1);
        v010 = load_voxel(g, o + 8);
        v110 = load_voxel(g, o + 9);
        v001 = load_voxel(g, o + 64);
        v101 = load_voxel(g, o + 65);
        v011 = load_voxel(g, o + 72);
        v111 = load_voxel(g, o + 73);
    } else {
        v000 = voxel(g, ix, iy, iz);
        v100 = voxel(g, ix + 1, iy, iz);
        v010 = voxel(g, ix, iy + 1, iz);
        v110 = voxel(g, ix + 1, iy + 1, iz);
        v001 = voxel(g, ix, iy, iz + 1);
        v101 = voxel(g, ix + 1, iy, iz + 1);
        v011 = voxel(g, ix, iy + 1, iz + 1);
        v111 = voxel(g, ix + 1, iy + 1, iz + 1);
    }
    const float y00 = lerpf(v000, v001, wz), y01 = lerpf(v010, v011, wz);
    const float y10 = lerpf(v100, v101, wz), y11 = lerpf(v110, v111, wz);
    return lerpf(lerpf(y00, y01, wy), lerpf(y10, y11, wy), wx);
}

__device__ __forceinline__ float sample_world(const DevGrid& g, float wx, float wy, float wz) {
    return sample_index(g, (wx - g.wo[0]) * g.inv_h, (wy - g.wo[1]) * g.inv_h,
                        (wz - g.wo[2]) * g.inv_h);
}

__device__ __forceinline__ bool is_leaf(const DevGrid& g, int cx, int cy, int cz) {
    const int bx = cx - g.blo[0], by = cy - g.blo[1], bz = cz - g.blo[2];
    if ((unsigned)bx >= (unsigned)g.nb[0] || (unsigned)by >= (unsigned)g.nb[1] ||
        (unsigned)bz >= (unsigned)g.nb[2])
        return false;
    const int64_t b = ((int64_t)bz * g.nb[1] + by) * g.nb[0] + bx;
    return (__ldg(g.leafbits + (b >> 5)) >> (b & 31)) & 1u;
}

// ---------------------------------------------------------------------------
// Index ray and the leaf-span march.
// The reference marches a ray through maximal runs of existing leaf nodes
// (VolumeRayIntersector::march, src/Renderer.h:345-369, over OpenVDB's
// VolumeHDDA at leaf granularity), after clipping it to the active leaf bbox
// padded by one voxel (src/Renderer.h:295-297,323-327). This is a single-level
// 3D DDA over 8^3 leaf cells that yields the same spans.
// ---------------------------------------------------------------------------
struct IRay {
    float e[3];  // eye, index space
    float d[3];  // unit direction
    float inv[3];
    float t0, t1;
};

__device__ __forceinline__ void make_iray(IRay& r, float ex, float ey, float ez, float dx, float dy,
                                          float dz, float t0, float t1) {
    r.e[0] = ex; r.e[1] = ey; r.e[2] = ez;
    r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
    r.inv[0] = 1.f / dx; r.inv[1] = 1.f / dy; r.inv[2] = 1.f / dz;
    r.t0 = t0; r.t1 = t1;
}

// Ray::clip against the leaf bbox (slab test in x, y, z order).
__device__ __forceinline__ bool clip_to_bbox(const DevGrid& g, IRay& r) {
    if (!g.has_leaves) return false;
    float t0 = r.t0, t1 = r.t1;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float a = (g.bbmin[i] - r.e[i]) * r.inv[i];
        float b = (g.bbmax[i] - r.e[i]) * r.inv[i];
        if (a > b) { const float t = a; a = b; b = t; }
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (t0 > t1) return false;
    }
    r.t0 = t0;
    r.t1 = t1;
    return true;
}

// Per-axis state is kept in scalars (no runtime-indexed arrays), so the
// walker lives in registers.
struct LeafDDA {
    float t, tmax;
    float nx, ny, nz;   // next crossing time per axis
    float dx, dy, dz;   // crossing interval per axis
    int cx, cy, cz;     // current leaf cell
    int sx, sy, sz;     // cell step per axis
    bool open;          // a span has started
    float start;        // its start time
    bool done;
};

__device__ __forceinline__ void dda_axis(float e, float d, float inv, float t0, int& c, int& step, float& next,
                                         float& delta) {
    const float p = e + t0 * d;
    c = ((int)floorf(p)) >> 3;
    if (d == 0.f) {
        step = 0;
        next = kInf;
        delta = kInf;
    } else if (inv > 0.f) {
        step = 1;
        next = t0 + ((float)(c * 8 + 8) - p) * inv;
        delta = 8.f * inv;
    } else {
        step = -1;
        next = t0 + ((float)(c * 8) - p) * inv;
        delta = -8.f * inv;
    }
}

__device__ __forceinline__ void dda_init(LeafDDA& s, const IRay& r) {
    s.t = r.t0;
    s.tmax = r.t1;
    s.open = false;
    s.start = 0.f;
    s.done = false;
    dda_axis(r.e[0], r.d[0], r.inv[0], r.t0, s.cx, s.sx, s.nx, s.dx);
    dda_axis(r.e[1], r.d[1], r.inv[1], r.t0, s.cy, s.sy, s.ny, s.dy);
    dda_axis(r.e[2], r.d[2], r.inv[2], r.t0, s.cz, s.sz, s.nz, s.dz);
}

// Next span [ta, tb] of consecutive leaf cells with tb - ta > kDelta.
__device__ __forceinline__ bool next_span(const DevGrid& g, LeafDDA& s, float& ta, float& tb) {
    while (!s.done) {
        const bool leaf = is_leaf(g, s.cx, s.cy, s.cz);
        if (leaf) {
            if (!s.open) { s.open = true; s.start = s.t; }
        } else if (s.open) {
            s.open = false;
            if (s.t - s.start > kDelta) { ta = s.start; tb = s.t; return true; }
        }
        // step to the next cell (math::MinIndex tie order: x if strictly
        // smallest, else y if below z, else z)
        const bool ax = (s.nx < s.ny) && (s.nx < s.nz);
        const bool ay = !(s.nx < s.ny) && (s.ny < s.nz);
        const bool az = !ax && !ay;
        s.t = ax ? s.nx : (ay ? s.ny : s.nz);
        if (ax) { s.nx += s.dx; s.cx += s.sx; }
        if (ay) { s.ny += s.dy; s.cy += s.sy; }
        if (az) { s.nz += s.dz; s.cz += s.sz; }
        if (!(s.t <= s.tmax)) {
            s.done = true;
            if (s.open && s.tmax - s.start > kDelta) { ta = s.start; tb = s.tmax; return true; }
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Shading, lights and the environment map
// ---------------------------------------------------------------------------
struct DevShader {
    float dS, dMax, shadowDS, scatterDS, scatterDMin;
    float a[3];            // -extinction per channel (>= 0)
    float albedo[3];
    float inv_scatter[3];  // 1 / scattering
    float emission_scale, scatter_scale, mask_power;
    float tau_drop;        // optical depth where |T|^2 first drops below cutoff
    int ramp_n;
    float ramp_pos[kMaxRamp];
    float ramp_col[kMaxRamp][3];
    float ramp_in, ramp_out;
};

struct DevLight {
    int type, samples;
    float I[3];            // color * intensity
    float dir[3];          // distant: DistantLight::mDir
    float pos[3];          // point: PointLight::mPos
    float rot[9];          // env: row-vector rotation
};

struct DevEnv {
    const float* rgb = nullptr;        // h x w x 3
    const float* cond_cdf = nullptr;   // h x (w + 1)
    const float* cond_func = nullptr;  // h x w
    const float* cond_int = nullptr;   // h
    const float* marg_cdf = nullptr;   // h + 1
    const float* marg_func = nullptr;  // h
    float marg_int = 0.f;
    int w = 0, h = 0;
};

struct DevScene {
    DevGrid dens, temp;
    int has_temp;
    DevShader sh;
    DevLight lights[kMaxLights];
    int n_lights;
    DevEnv env;
    float cutoff, step0, step1;
    uint64_t seed;
};

// ColorRamp::getColor (src/Shader.h:63-92), including its edge behaviour.
__device__ __forceinline__ void ramp_color(const DevShader& sh, float temp, float out[3]) {
    if (sh.ramp_n == 0) { out[0] = out[1] = out[2] = 0.f; return; }
    float x = (temp - sh.ramp_in) / (sh.ramp_out - sh.ramp_in);
    x = fminf(fmaxf(x, 0.f), 1.f);
    if (sh.ramp_n == 1) {
        out[0] = sh.ramp_col[0][0]; out[1] = sh.ramp_col[0][1]; out[2] = sh.ramp_col[0][2];
        return;
    }
    int prev = 0, next = 0;
    for (int i = 0; i < sh.ramp_n; ++i) {
        if (sh.ramp_pos[i] <= x) prev = i;
        else { next = i; break; }
    }
    const float range = sh.ramp_pos[next] - sh.ramp_pos[prev];
    const float blend = (x - sh.ramp_pos[prev]) / range;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[c] = sh.ramp_col[prev][c] * (1.f - blend) + sh.ramp_col[next][c] * blend;
}

// Distribution1D::SampleContinuous (src/Sampling.h:102-119) over a CDF of n+1
// entries; FindInterval (src/Sampling.h:59-72) is the same bisection.
__device__ __forceinline__ float sample_1d(const float* cdf, int n, float u, int* off_out) {
    int first = 0, len = n + 1;
    while (len > 0) {
        const int half = len >> 1, middle = first + half;
        if (__ldg(cdf + middle) <= u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    int off = first - 1;
    off = off < 0 ? 0 : (off > n - 1 ? n - 1 : off);
    float du = u - __ldg(cdf + off);
    const float span = __ldg(cdf + off + 1) - __ldg(cdf + off);
    if (span > 0.f) du /= span;
    if (off_out) *off_out = off;
    return ((float)off + du) / (float)n;
}

// EnvLight::illuminate (src/Light.h:185-233) for random numbers (u, v).
// The reference reads col_hi = ceil(x * w) and row_hi = ceil(y * h), which can
// index one past the map; here the column wraps around and the row clamps.
__device__ __forceinline__ void env_illuminate(const DevEnv& env, const DevLight& L, float u,
                                               float v, float dir_out[3], float I_out[3]) {
    int row;
    const float d1 = sample_1d(env.marg_cdf, env.h, v, &row);
    const float d0 = sample_1d(env.cond_cdf + (int64_t)row * (env.w + 1), env.w, u, nullptr);
    const float xs = d0 * (float)env.w, ys = d1 * (float)env.h;
    int col_lo = (int)floorf(xs), row_lo = (int)floorf(ys);
    int col_hi = (int)ceilf(xs), row_hi = (int)ceilf(ys);
    const float col_ratio = xs - (float)col_lo, row_ratio = ys - (float)row_lo;
    // a sample at exactly 1.0 would index one past the map on both sides
    if (col_lo >= env.w) col_lo = env.w - 1;
    if (row_lo >= env.h) row_lo = env.h - 1;
    if (col_hi >= env.w) col_hi -= env.w;
    if (col_hi >= env.w) col_hi = env.w - 1;
    if (row_hi >= env.h) row_hi = env.h - 1;
    const float theta = d0 * 3.14159265358979323846f * 2.0f;
    const float phi = d1 * 3.14159265358979323846f;
    const float sphi = sinf(phi);
    float sd[3] = {cosf(theta) * sphi, cosf(phi), sinf(theta) * sphi};
    // mXform.transform(sampleDir).unit()
    float t[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = sd[0] * L.rot[0 * 3 + c] + sd[1] * L.rot[1 * 3 + c] + sd[2] * L.rot[2 * 3 + c];
    const float invl = rsqrtf(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const float* m = env.rgb;
    const int w = env.w;
    const float wLL = (1.f - row_ratio) * (1.f - col_ratio), wLH = (1.f - row_ratio) * col_ratio;
    const float wHL = row_ratio * (1.f - col_ratio), wHH = row_ratio * col_ratio;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float img = wLL * __ldg(m + ((int64_t)row_lo * w + col_lo) * 3 + c) +
                          wLH * __ldg(m + ((int64_t)row_lo * w + col_hi) * 3 + c) +
                          wHL * __ldg(m + ((int64_t)row_hi * w + col_lo) * 3 + c) +
                          wHH * __ldg(m + ((int64_t)row_hi * w + col_hi) * 3 + c);
        dir_out[c] = -t[c] * invl;  // lightDir = -sampleDir
        I_out[c] = img * L.I[c];
    }
}

// Light::illuminate for distant and point lights (src/Light.h:79-89,118-126).
// Returns the light direction (from light towards the point), the intensity
// and the distance to the light (kInf for distant and env lights).
__device__ __forceinline__ void illuminate(const DevLight& L, const float p[3], float dir[3],
                                           float I[3], float& dist) {
    if (L.type == 1) {
        float d[3] = {p[0] - L.pos[0], p[1] - L.pos[1], p[2] - L.pos[2]};
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        dist = sqrtf(r2);
        const float fall = 1.f / (1.f + 4.f * 3.14159265358979323846f * r2);
#pragma unroll
        for (int c = 0; c < 3; ++c) { dir[c] = d[c] / dist; I[c] = L.I[c] * fall; }
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) { dir[c] = L.dir[c]; I[c] = L.I[c]; }
        dist = kInf;
    }
}

// ---------------------------------------------------------------------------
// Fixed-step shadow march (no jitter) in scalar optical depth:
//   tau = sum over samples of contrib(rho) * step,
// where rho = min(sample * scale, densityMax) and contrib() is given by the
// caller. Returns false if the ray misses the leaf bbox. Sets dropped when
// tau crosses sh.tau_drop (the reference's |T|^2 < cutoff test).
// ---------------------------------------------------------------------------
template <int DT, class Contrib>
__device__ __forceinline__ bool march_fixed(const DevGrid& g, IRay r, float step, float scale,
                                            float dmax, float tau_drop, Contrib contrib,
                                            float& tau, bool& dropped, uint32_t& nsamples) {
    tau = 0.f;
    dropped = false;
    if (!clip_to_bbox(g, r)) return false;
    LeafDDA s;
    dda_init(s, r);
    float ta, tb;
    while (next_span(g, s, ta, tb)) {
        for (float t = step * ceilf(ta / step); t <= tb && t + step > t; t += step) {
            const float rho = fminf(
                sample_index_t<DT>(g, r.e[0] + t * r.d[0], r.e[1] + t * r.d[1], r.e[2] + t * r.d[2]) * scale,
                dmax);
            ++nsamples;
            float c;
            if (!contrib(rho, c)) continue;
            tau += c * step;
            if (tau > tau_drop) { dropped = true; return true; }
        }
    }
    return true;
}

}  // namespace lg
