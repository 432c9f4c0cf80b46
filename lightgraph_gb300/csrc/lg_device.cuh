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
// Grid: one record per voxel cell (x, y, z) of a dense box that is tiled into
// 8^3 bricks (x fastest inside a brick, bricks x fastest in the box) with one
// brick of zero padding on every side. A cell's record holds the eight voxel
// values of its trilinear footprint, v(x + a, y + b, z + c) at index
// a + 2b + 4c (FP16/BF16), or the eight coefficients of its trilinear
// polynomial (FP32, cell_coefs), so one sample is one aligned 32-byte (FP32)
// or 16-byte (FP16/BF16) load instead of eight gathers. A brick's 512 records are one
// contiguous 16 KB block, so a ray crossing a brick in any direction stays in
// one block (rays that run along z would otherwise touch a new page at every
// voxel). Voxels outside the box read the background value 0. The box's first
// and last cells lie in padding corner bricks, so their eight values are 0;
// the checked sampler redirects cells outside the box to the first one.
// Records cost 8x the voxel storage, which HBM holds easily (a 512^3 box is
// 4.6 GB in FP32); what matters for the marches is one L1 request per sample.
// ---------------------------------------------------------------------------
struct DevGrid {
    const void* data = nullptr;
    const uint32_t* leafbits = nullptr;  // one bit per brick of the box: leaf exists
    int dtype = 0;                       // 0 f32, 1 f16, 2 bf16
    int blo[3] = {0, 0, 0};              // brick coordinate of box brick 0
    int nb[3] = {0, 0, 0};               // bricks per axis
    int vlo[3] = {0, 0, 0};              // voxel coordinate of the box's first cell (8 * blo)
    uint32_t vn[3] = {0, 0, 0};          // cells per axis (8 * nb)
    float inv_h = 1.f;                   // 1 / voxel size
    float h = 1.f;                       // voxel size
    float wo[3] = {0.f, 0.f, 0.f};       // world origin
    float bbmin[3] = {0.f, 0.f, 0.f};    // leaf bbox in index space (origin of min leaf)
    float bbmax[3] = {0.f, 0.f, 0.f};    // ... max leaf origin + 8
    int has_leaves = 0;
    uint32_t sy = 0, sz = 0;             // record strides of one brick step in y and z
    uint32_t ky = 0, kz = 0;             // sy - 64 and sz - 512 (span_cell)
    uint32_t rec_off = 0;                // span_cell's record index offset (mod 2^32)
    uint32_t rec_last = 0;               // last record (a padding cell)
    // The leaf bitmap covers the brick box plus a margin of one brick on
    // every side (bits 0), so a walker one cell off the box reads "no leaf"
    // without per-axis bounds checks: bit ((z + 1) * lby + y + 1) * lbx + x + 1
    // for box brick (x, y, z).
    int lbx = 0, lby = 0;                // bitmap cells per row and per column (nb + 2)
    int lbxy = 0;                        // lbx * lby
    uint32_t nbits = 0;                  // bitmap cells
};

// Bytes of one cell record for storage type dtype.
__host__ __device__ constexpr int cell_record_bytes(int dtype) { return dtype == 0 ? 32 : 16; }

// Coefficients of a cell's trilinear polynomial from its eight voxel values
// v[a + 2b + 4c] = v(x + a, y + b, z + c), in the FP32 record order
//   c[0..7] = {k0, kx, kz, kxz, ky, kxy, kyz, kxyz}
// where v(wx, wy, wz) = (k0 + kz wz) + (ky + kyz wz) wy
//                     + ((kx + kxz wz) + (kxy + kxyz wz) wy) wx.
// k0 is the voxel v(x, y, z) itself; the others are nested FP32 differences
// of the voxels (error at most 54 * 2^-24 of the largest |v| in all, which
// the dart test's bound covers).
__host__ __device__ inline void cell_coefs(const float v[8], float c[8]) {
    const float dx = v[1] - v[0];    // v100 - v000
    const float dy = v[2] - v[0];    // v010 - v000
    const float dz = v[4] - v[0];    // v001 - v000
    const float dxz = v[5] - v[1];   // v101 - v100
    const float dxy = v[3] - v[1];   // v110 - v100
    const float dyz = v[6] - v[2];   // v011 - v010
    const float dxyz = v[7] - v[3];  // v111 - v110
    c[0] = v[0];
    c[1] = dx;
    c[2] = dz;
    c[3] = dxz - dz;
    c[4] = dy;
    c[5] = dxy - dy;
    c[6] = dyz - dz;
    c[7] = (dxyz - dxz) - (dyz - dz);
}

// The raw eight values of record rec, decoded to FP32 (FP16/BF16: voxel
// values in a + 2b + 4c order; FP32: cell_coefs).
template <int DT>
__device__ __forceinline__ void ld_cell(const void* data, uint32_t rec, float v[8]) {
    if (DT == 0) {
        const float* p = reinterpret_cast<const float*>(data) + (size_t)rec * 8;
        asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
            : "l"(p));
    } else {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(data) + rec);
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float2 f;
            if (DT == 1) f = __half22float2(*reinterpret_cast<const __half2*>(&w[i]));
            else f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[i]));
            v[2 * i] = f.x;
            v[2 * i + 1] = f.y;
        }
    }
}

// Record index of cell (ix, iy, iz), or 0 (the all-zero padding cell) when
// the cell lies outside the box. 32-bit: the upload rejects boxes with 2^32
// or more cells.
__device__ __forceinline__ uint32_t cell_record(const DevGrid& g, int ix, int iy, int iz) {
    const uint32_t rx = (uint32_t)(ix - g.vlo[0]), ry = (uint32_t)(iy - g.vlo[1]), rz = (uint32_t)(iz - g.vlo[2]);
    const bool in = rx < g.vn[0] && ry < g.vn[1] && rz < g.vn[2];
    const uint32_t rec = (rx >> 3) * 512u + (ry >> 3) * g.sy + (rz >> 3) * g.sz +
                         (((rz & 7u) << 6) | ((ry & 7u) << 3) | (rx & 7u));
    return in ? rec : 0u;
}

// Floor of an index-space coordinate (|p| < 2^22) without a float-to-int
// conversion: adding 1.5 * 2^23 rounding down leaves floor(p) in the low
// mantissa bits. Returns those bits (floor(p) + 0x4B400000) and floor(p) as
// a float.
__device__ __forceinline__ uint32_t floor_bits(float p, float& fl) {
    const float r = __fadd_rd(p, 12582912.0f);
    fl = __fsub_rn(r, 12582912.0f);
    return __float_as_uint(r);
}

// Trilinear weights and record of the cell under an index-space position
// inside a leaf span of g. Leaves lie inside the box with a brick of padding
// around them, so such a cell is always inside the box and needs no per-axis
// test; the index is clamped to the last (all-zero) record all the same, so
// no position can address memory outside the records.
__device__ __forceinline__ uint32_t span_cell(const DevGrid& g, float px, float py, float pz, float& wx,
                                              float& wy, float& wz) {
    float fx, fy, fz;
    const uint32_t bx = floor_bits(px, fx), by = floor_bits(py, fy), bz = floor_bits(pz, fz);
    wx = px - fx;
    wy = py - fy;
    wz = pz - fz;
    // Record of cell (x, y, z): brick (x >> 3, y >> 3, z >> 3) times 512 plus
    // the offset (z & 7) * 64 + (y & 7) * 8 + (x & 7) inside it. With
    // x & 7 = x - 8 (x >> 3) it is linear per axis:
    //   x + 504 (x >> 3) + 8 y + (sy - 64) (y >> 3) + 64 z + (sz - 512) (z >> 3)
    // The bits carry the bias B = 0x4B400000, a multiple of 8, so bits >> 3
    // carry B / 8 and the terms carry (512 + sy + sz) B / 8 in all; rec_off
    // removes that and moves the box's first brick to record 0 (mod 2^32).
    const uint32_t rec = bx + 504u * (bx >> 3) + 8u * by + g.ky * (by >> 3) + 64u * bz + g.kz * (bz >> 3) + g.rec_off;
    return min(rec, g.rec_last);
}

// The interpolation of a cell record's eight values (a + 2b + 4c order) at
// weights (wx, wy, wz): along z, then y, then x (the order of OpenVDB's
// BoxSampler::trilinearInterpolation), each step fmaf(b - a, w, a). The z and
// y steps run two lanes at a time in packed FP32 (same rounding per lane as
// the scalar form).
__device__ __forceinline__ float trilinear8(const float v[8], float wx, float wy, float wz) {
    const float2 wz2 = make_float2(wz, wz), wy2 = make_float2(wy, wy);
    // lanes (x0, x1) at y0 and at y1, interpolated along z
    const float2 a0 = make_float2(v[0], v[1]), b0 = make_float2(v[4], v[5]);
    const float2 a1 = make_float2(v[2], v[3]), b1 = make_float2(v[6], v[7]);
    const float2 z0 = __ffma2_rn(__fadd2_rn(b0, make_float2(-a0.x, -a0.y)), wz2, a0);
    const float2 z1 = __ffma2_rn(__fadd2_rn(b1, make_float2(-a1.x, -a1.y)), wz2, a1);
    // lanes (x0, x1) interpolated along y
    const float2 y = __ffma2_rn(__fadd2_rn(z1, make_float2(-z0.x, -z0.y)), wy2, z0);
    return fmaf(y.y - y.x, wx, y.x);
}

// The trilinear polynomial of an FP32 record (cell_coefs) at weights (wx,
// wy, wz): the z terms of both wx halves as one packed pair, then y, then x.
__device__ __forceinline__ float trilinear_coefs(const float c[8], float wx, float wy, float wz) {
    const float2 wz2 = make_float2(wz, wz), wy2 = make_float2(wy, wy);
    // lanes (without wx, with wx)
    const float2 a = __ffma2_rn(make_float2(c[2], c[3]), wz2, make_float2(c[0], c[1]));  // (k0, kx) + (kz, kxz) wz
    const float2 b = __ffma2_rn(make_float2(c[6], c[7]), wz2, make_float2(c[4], c[5]));  // (ky, kxy) + (kyz, kxyz) wz
    const float2 y = __ffma2_rn(b, wy2, a);
    return fmaf(y.y, wx, y.x);
}

// The interpolation of record values for storage type DT.
template <int DT>
__device__ __forceinline__ float record_sample(const float v[8], float wx, float wy, float wz) {
    return DT == 0 ? trilinear_coefs(v, wx, wy, wz) : trilinear8(v, wx, wy, wz);
}

// Trilinear sample at an index-space position for storage type DT: the cell
// record at floor(p) (the eight voxels around it, or their polynomial).
template <int DT>
__device__ __forceinline__ float sample_index_t(const DevGrid& g, float px, float py, float pz) {
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    float v[8];
    ld_cell<DT>(g.data, cell_record(g, (int)fx, (int)fy, (int)fz), v);
    return record_sample<DT>(v, px - fx, py - fy, pz - fz);
}

// sample_index_t for a position inside a leaf span of g (span_cell): the same
// record and the same interpolation, without the box test.
template <int DT>
__device__ __forceinline__ float sample_span_t(const DevGrid& g, float px, float py, float pz) {
    float wx, wy, wz;
    float v[8];
    ld_cell<DT>(g.data, span_cell(g, px, py, pz, wx, wy, wz), v);
    return record_sample<DT>(v, wx, wy, wz);
}

// Value of voxel (x, y, z): the first entry of its cell's record (the voxel
// itself in both record forms; 0 outside the box).
__device__ __forceinline__ float voxel(const DevGrid& g, int x, int y, int z) {
    const size_t off = (size_t)cell_record(g, x, y, z) * 8;
    if (g.dtype == 0) return __ldg(reinterpret_cast<const float*>(g.data) + off);
    if (g.dtype == 1) return __half2float(__ldg(reinterpret_cast<const __half*>(g.data) + off));
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(g.data) + off));
}

__device__ __forceinline__ float lerpf(float a, float b, float w) { return fmaf(b - a, w, a); }

// Trilinear sample for a storage type known only at run time.
__device__ __forceinline__ float sample_index(const DevGrid& g, float px, float py, float pz) {
    if (g.dtype == 1) return sample_index_t<1>(g, px, py, pz);
    if (g.dtype == 2) return sample_index_t<2>(g, px, py, pz);
    return sample_index_t<0>(g, px, py, pz);
}

__device__ __forceinline__ float sample_world(const DevGrid& g, float wx, float wy, float wz) {
    return sample_index(g, (wx - g.wo[0]) * g.inv_h, (wy - g.wo[1]) * g.inv_h,
                        (wz - g.wo[2]) * g.inv_h);
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
// walker lives in registers. The current cell is its bitmap index lin; a step
// along an axis adds that axis's increment (+-1, +-lbx, +-lbx * lby).
struct LeafDDA {
    float t, tmax;
    float nx, ny, nz;   // next crossing time per axis
    float dx, dy, dz;   // crossing interval per axis
    int lin;            // current leaf cell (bitmap index)
    int ix, iy, iz;     // bitmap increment of one step per axis
    bool open;          // next_span_flat: a span has started
    float start;        // next_span_flat: its start time
    bool done;
};

// Cell coordinate of the ray start along one axis (bitmap coordinates), the
// step direction, the first crossing time and the crossing interval.
__device__ __forceinline__ int dda_axis(float e, float d, float inv, float t0, int blo, int& step, float& next,
                                        float& delta) {
    // fused multiply-adds written out, so every kernel that walks a ray (the
    // two primary passes above all) finds the same cells and crossings
    const float p = __fmaf_rn(t0, d, e);
    const int ca = ((int)floorf(p)) >> 3;
    if (d == 0.f) {
        step = 0;
        next = kInf;
        delta = kInf;
    } else if (inv > 0.f) {
        step = 1;
        next = __fmaf_rn((float)(ca * 8 + 8) - p, inv, t0);
        delta = 8.f * inv;
    } else {
        step = -1;
        next = __fmaf_rn((float)(ca * 8) - p, inv, t0);
        delta = -8.f * inv;
    }
    return ca - blo + 1;
}

__device__ __forceinline__ void dda_init(LeafDDA& s, const IRay& r, const DevGrid& g) {
    s.t = r.t0;
    s.tmax = r.t1;
    s.done = false;
    s.open = false;
    s.start = 0.f;
    int sx, sy, sz;
    const int cx = dda_axis(r.e[0], r.d[0], r.inv[0], r.t0, g.blo[0], sx, s.nx, s.dx);
    const int cy = dda_axis(r.e[1], r.d[1], r.inv[1], r.t0, g.blo[1], sy, s.ny, s.dy);
    const int cz = dda_axis(r.e[2], r.d[2], r.inv[2], r.t0, g.blo[2], sz, s.nz, s.dz);
    const bool in = (unsigned)cx < (unsigned)g.lbx && (unsigned)cy < (unsigned)g.lby &&
                    (unsigned)cz < (unsigned)(g.nb[2] + 2);
    // a start cell off the bitmap (not reached by rays clipped to the leaf
    // bbox) is mapped past its end, where every cell reads "no leaf"
    s.lin = in ? (cz * g.lby + cy) * g.lbx + cx : (int)g.nbits;
    s.ix = sx;
    s.iy = sy * g.lbx;
    s.iz = sz * g.lbx * g.lby;
}

// Leaf test for a walker cell: the index is clamped to nbits (a zero bit: the
// bitmap's last word has room for it), so no branch guards the load.
__device__ __forceinline__ bool walker_leaf(const DevGrid& g, int lin) {
    const uint32_t c = min((uint32_t)lin, g.nbits);
    return (__ldg(g.leafbits + (c >> 5)) >> (c & 31u)) & 1u;
}

// One DDA step to the next cell (math::MinIndex tie order: x if strictly
// smallest, else y if below z, else z); returns false once the crossing
// lies past tmax.
__device__ __forceinline__ bool walker_step(LeafDDA& s) {
    // x strictly first: nx < min(ny, nz); else y if ny < nz (then nx >= ny);
    // else z. The crossing taken is the smallest of the three either way.
    const float myz = fminf(s.ny, s.nz);
    const bool ax = s.nx < myz;
    const bool ay = !ax && (s.ny < s.nz);
    const bool az = !ax && !ay;
    s.t = fminf(s.nx, myz);
    if (ax) { s.nx += s.dx; s.lin += s.ix; }
    if (ay) { s.ny += s.dy; s.lin += s.iy; }
    if (az) { s.nz += s.dz; s.lin += s.iz; }
    return s.t <= s.tmax;
}

// Next span [ta, tb] of consecutive leaf cells with tb - ta > kDelta: first
// the cells up to the next leaf, then the run of leaves; a run cut by tmax
// ends there.
__device__ __forceinline__ bool next_span(const DevGrid& g, LeafDDA& s, float& ta, float& tb) {
    while (!s.done) {
        while (!walker_leaf(g, s.lin)) {
            if (!walker_step(s)) { s.done = true; return false; }
        }
        const float start = s.t;
        bool inside;
        do {
            inside = walker_step(s);
        } while (inside && walker_leaf(g, s.lin));
        if (!inside) {
            s.done = true;
            if (s.tmax - start > kDelta) { ta = start; tb = s.tmax; return true; }
            return false;
        }
        if (s.t - start > kDelta) { ta = start; tb = s.t; return true; }
    }
    return false;
}

// next_span in one loop that examines a cell and steps on every pass (the
// same spans). Marches whose lanes run unrelated rays (graph edges, vertex
// shadow rays) stay converged better with it than with next_span's two inner
// loops, which the render's ordered, neighbouring rays favour.
__device__ __forceinline__ bool next_span_flat(const DevGrid& g, LeafDDA& s, float& ta, float& tb) {
    while (!s.done) {
        // the bounds test skips the bitmap load for cells off the bitmap
        // (measured: the clamped load of walker_leaf makes these marches
        // several times slower)
        const bool leaf = (unsigned)s.lin < g.nbits &&
                          ((__ldg(g.leafbits + ((unsigned)s.lin >> 5)) >> ((unsigned)s.lin & 31u)) & 1u);
        if (leaf) {
            if (!s.open) { s.open = true; s.start = s.t; }
        } else if (s.open) {
            s.open = false;
            if (s.t - s.start > kDelta) { ta = s.start; tb = s.t; return true; }
        }
        if (!walker_step(s)) {
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
    // per knot i the reciprocal of the interval to the next knot (the last
    // knot: to the first, ColorRamp's wrap)
    float ramp_inv[kMaxRamp];
    float ramp_in, ramp_out;
};

struct DevLight {
    int type, samples;
    float I[3];            // color * intensity
    float dir[3];          // distant: DistantLight::mDir
    float pos[3];          // point: PointLight::mPos
    float rot[9];          // env: row-vector rotation
};

// Guide tables of the environment CDFs: entry g of a table is the first
// index i with cdf[i] > g / kEnvGuide (std::upper_bound), so the interval of
// a draw u lies between entries floor(u kEnvGuide) and the next one.
constexpr int kEnvGuide = 256;  // a power of two: u * kEnvGuide is exact

struct DevEnv {
    const float* rgb = nullptr;        // h x w x 3
    const int* cond_guide = nullptr;   // h x (kEnvGuide + 1)
    const int* marg_guide = nullptr;   // kEnvGuide + 1
    const float* cond_cdf = nullptr;   // h x (w + 1)
    const float* cond_func = nullptr;  // h x w
    const float* cond_int = nullptr;   // h
    const float* marg_cdf = nullptr;   // h + 1
    const float* marg_func = nullptr;  // h
    float marg_int = 0.f;
    int w = 0, h = 0;
};

// Constants of the shadow-ray march (k_shadow). A sample's density is
// min(raw * scale, dMax), scale = dS * shadowDS; it counts when at or above
// the cutoff, and the ray drops once tau passes tau_drop. With unit set
// (scale positive and finite) the march accumulates raw density x step
// against dmax, cut and drop divided by scale and multiplies tau by scale
// once per ray; otherwise dmax, cut and drop are the plain values.
struct ShadowMarch {
    int unit;
    float scale, dmax, cut, drop;
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
    ShadowMarch smarch;
};

// ColorRamp::getColor (src/Shader.h:63-92), including its edge behaviour.
// The remap to [0, 1] is a division, so a temperature that maps exactly onto
// a knot lands on it as the reference's does (a product with a reciprocal of
// the range can land a rounding below the first knot, in the empty interval
// whose quotient is 0/0); the blend inside an interval is a product with the
// interval's reciprocal made on the host (within an ulp of the quotient, and
// exactly 0 on a knot; a temperature below the first knot still gives the
// quotient by zero).
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
    // next is prev + 1, or 0 when x lies past the last knot (prev = n - 1,
    // the wrap interval) or before the first (prev = 0, an empty interval)
    const float inv = next > 0 ? sh.ramp_inv[prev] : prev > 0 ? sh.ramp_inv[prev] : kInf;
    const float blend = (x - sh.ramp_pos[prev]) * inv;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[c] = sh.ramp_col[prev][c] * (1.f - blend) + sh.ramp_col[next][c] * blend;
}

// Distribution1D::SampleContinuous (src/Sampling.h:102-119) over a CDF of n+1
// entries; FindInterval (src/Sampling.h:59-72) is the same bisection.
__device__ __forceinline__ float sample_1d(const float* cdf, const int* guide, int n, float u, int* off_out) {
    // the upper bound of u among cdf[0..n], searched only between the guide
    // entries around u (the same index a search of the whole array finds)
    const int g = min(max((int)(u * (float)kEnvGuide), 0), kEnvGuide - 1);
    int first = __ldg(guide + g), len = __ldg(guide + g + 1) - first;
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
    const float d1 = sample_1d(env.marg_cdf, env.marg_guide, env.h, v, &row);
    const float d0 = sample_1d(env.cond_cdf + (int64_t)row * (env.w + 1), env.cond_guide + (int64_t)row * (kEnvGuide + 1),
                               env.w, u, nullptr);
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
    dda_init(s, r, g);
    float ta, tb;
    while (next_span_flat(g, s, ta, tb)) {
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
