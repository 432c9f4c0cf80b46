// Grid upload into the device brick layout, and the environment-map CDFs.
//
// Grids: a dense box of voxels (what a FloatGrid's active region looks like
// once copied to a dense array) is re-tiled into 8^3 bricks with one brick of
// zero padding on every side; every cell of the bricks stores the eight
// values of its trilinear footprint as one record, in FP32, FP16 or BF16.
// The leaf bitmap marks the bricks that are leaves of the VDB tree: given
// explicitly, or "any voxel non-zero" (a dense grid converted to a VDB keeps
// exactly those).
//
// Environment map: EnvLight's constructor (src/Light.h:150-177) weights each
// texel's luminance by sin(theta) and builds a Distribution2D
// (src/Sampling.h:128-167): per-row Distribution1D CDFs and a marginal CDF
// over the rows' integrals (src/Sampling.h:76-93). The prefix sums run in
// FP64 on the device (the reference uses FP32) and are stored as FP32.
#include <climits>

#include "lg_kernels.h"

namespace lg {

// One thread per cell record: gathers the cell's eight voxel values from the
// dense staging array (0 outside it) and writes them as one record.
__global__ void k_pack_bricks(const float* __restrict__ dense, int dx, int dy, int dz, int ox, int oy,
                              int oz, DevGrid g, void* __restrict__ bricks) {
    const int64_t total = (int64_t)g.nb[0] * g.nb[1] * g.nb[2] * 512;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t b = t >> 9;
    const int l = (int)(t & 511);
    const int bx = (int)(b % g.nb[0]), by = (int)((b / g.nb[0]) % g.nb[1]),
              bz = (int)(b / ((int64_t)g.nb[0] * g.nb[1]));
    const int x = (g.blo[0] + bx) * 8 + (l & 7) - ox;
    const int y = (g.blo[1] + by) * 8 + ((l >> 3) & 7) - oy;
    const int z = (g.blo[2] + bz) * 8 + (l >> 6) - oz;
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int xa = x + (c & 1), ya = y + ((c >> 1) & 1), za = z + (c >> 2);
        v[c] = ((unsigned)xa < (unsigned)dx && (unsigned)ya < (unsigned)dy && (unsigned)za < (unsigned)dz)
                   ? dense[((int64_t)za * dy + ya) * dx + xa]
                   : 0.f;
    }
    if (g.dtype == 0) {
        // FP32 records hold the cell's trilinear polynomial (cell_coefs)
        float c[8];
        cell_coefs(v, c);
        float4* o = reinterpret_cast<float4*>(bricks) + 2 * t;
        o[0] = make_float4(c[0], c[1], c[2], c[3]);
        o[1] = make_float4(c[4], c[5], c[6], c[7]);
    } else {
        uint32_t w[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (g.dtype == 1) {
                const __half2 h = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
                w[i] = *reinterpret_cast<const uint32_t*>(&h);
            } else {
                const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                w[i] = *reinterpret_cast<const uint32_t*>(&h);
            }
        }
        reinterpret_cast<uint4*>(bricks)[t] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

cudaError_t launch_pack_bricks(const float* dense, const int dims[3], const int origin[3],
                               const DevGrid& g, void* bricks, cudaStream_t st) {
    const int64_t total = (int64_t)g.nb[0] * g.nb[1] * g.nb[2] * 512;
    k_pack_bricks<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        dense, dims[0], dims[1], dims[2], origin[0], origin[1], origin[2], g, bricks);
    ++g_launch_counter;
    return cudaGetLastError();
}

// One thread per brick of the box; leaf bricks set their bit of the bitmap
// (which has a one-brick margin, cleared beforehand) with an atomic OR.
// bbox (6 ints: min xyz, max xyz brick coordinates) is reduced with atomics.
__global__ void k_leaf_bits(const float* __restrict__ dense, int dx, int dy, int dz, int ox, int oy,
                            int oz, const uint8_t* __restrict__ leaf_mask, DevGrid g,
                            uint32_t* __restrict__ bits, int* __restrict__ bbox) {
    const int64_t nbt = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool leaf = false;
    int cx = 0, cy = 0, cz = 0;
    if (b < nbt) {
        const int bx = (int)(b % g.nb[0]), by = (int)((b / g.nb[0]) % g.nb[1]),
                  bz = (int)(b / ((int64_t)g.nb[0] * g.nb[1]));
        cx = g.blo[0] + bx;
        cy = g.blo[1] + by;
        cz = g.blo[2] + bz;
        // leaf coordinates relative to the dense box (origin is leaf aligned)
        const int lx = cx - (ox >> 3), ly = cy - (oy >> 3), lz = cz - (oz >> 3);
        const int lnx = (dx + 7) >> 3, lny = (dy + 7) >> 3, lnz = (dz + 7) >> 3;
        if ((unsigned)lx < (unsigned)lnx && (unsigned)ly < (unsigned)lny && (unsigned)lz < (unsigned)lnz) {
            if (leaf_mask) {
                leaf = leaf_mask[((int64_t)lz * lny + ly) * lnx + lx] != 0;
            } else {
                for (int z = 0; z < 8 && !leaf; ++z) {
                    const int vz = lz * 8 + z;
                    if (vz >= dz) break;
                    for (int y = 0; y < 8 && !leaf; ++y) {
                        const int vy = ly * 8 + y;
                        if (vy >= dy) break;
                        const float* row = dense + ((int64_t)vz * dy + vy) * dx;
                        for (int x = 0; x < 8; ++x) {
                            const int vx = lx * 8 + x;
                            if (vx >= dx) break;
                            if (row[vx] != 0.f) { leaf = true; break; }
                        }
                    }
                }
            }
        }
    }
    if (leaf) {
        const uint32_t lin = ((uint32_t)(cz - g.blo[2] + 1) * (uint32_t)g.lby + (uint32_t)(cy - g.blo[1] + 1)) *
                                 (uint32_t)g.lbx +
                             (uint32_t)(cx - g.blo[0] + 1);
        atomicOr(bits + (lin >> 5), 1u << (lin & 31u));
        atomicMin(bbox + 0, cx);
        atomicMin(bbox + 1, cy);
        atomicMin(bbox + 2, cz);
        atomicMax(bbox + 3, cx);
        atomicMax(bbox + 4, cy);
        atomicMax(bbox + 5, cz);
    }
}

cudaError_t launch_leaf_bits(const float* dense, const int dims[3], const int origin[3],
                             const uint8_t* leaf_mask, const DevGrid& g, uint32_t* bits, int* bbox,
                             cudaStream_t st) {
    const int64_t nbt = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
    const unsigned blocks = (unsigned)((nbt + 255) / 256);
    k_leaf_bits<<<blocks, 256, 0, st>>>(dense, dims[0], dims[1], dims[2], origin[0], origin[1], origin[2],
                                        leaf_mask, g, bits, bbox);
    ++g_launch_counter;
    return cudaGetLastError();
}

// Bounding box of the non-zero voxels of the dense staging array (the active
// voxels of a dense grid converted to a VDB), in the array's own coordinates:
// bbox = {min x, y, z, max x, y, z}, pre-set to +/-INT_MAX. One thread per
// voxel; warp reductions, then one atomic per warp and bound.
__global__ void k_voxel_bbox(const float* __restrict__ dense, int dx, int dy, int dz, int* __restrict__ bbox) {
    const int64_t n = (int64_t)dx * dy * dz;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = i < n && dense[i] != 0.f;
    int x = INT_MAX, y = INT_MAX, z = INT_MAX;
    if (on) {
        x = (int)(i % dx);
        y = (int)((i / dx) % dy);
        z = (int)(i / ((int64_t)dx * dy));
    }
    const int mnx = __reduce_min_sync(0xffffffffu, x), mny = __reduce_min_sync(0xffffffffu, y),
              mnz = __reduce_min_sync(0xffffffffu, z);
    const int mxx = __reduce_max_sync(0xffffffffu, on ? x : INT_MIN),
              mxy = __reduce_max_sync(0xffffffffu, on ? y : INT_MIN),
              mxz = __reduce_max_sync(0xffffffffu, on ? z : INT_MIN);
    if ((threadIdx.x & 31) == 0 && mnx != INT_MAX) {
        atomicMin(bbox + 0, mnx);
        atomicMin(bbox + 1, mny);
        atomicMin(bbox + 2, mnz);
        atomicMax(bbox + 3, mxx);
        atomicMax(bbox + 4, mxy);
        atomicMax(bbox + 5, mxz);
    }
}

cudaError_t launch_voxel_bbox(const float* dense, const int dims[3], int* bbox, cudaStream_t st) {
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    if (n == 0) return cudaSuccess;
    k_voxel_bbox<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dense, dims[0], dims[1], dims[2], bbox);
    ++g_launch_counter;
    return cudaGetLastError();
}

// --- environment map -------------------------------------------------------

__device__ void dist1d_build(const float* f, int n, float* cdf_out, float* int_out) {
    double acc = 0.0;
    cdf_out[0] = 0.f;
    // unnormalised prefix of f/n, then divide by the total (src/Sampling.h:83-92)
    for (int i = 1; i <= n; ++i) acc += (double)f[i - 1] / (double)n;
    const double total = acc;
    if (total == 0.0) {
        for (int i = 1; i <= n; ++i) cdf_out[i] = (float)((double)i / (double)n);
    } else {
        double run = 0.0;
        for (int i = 1; i <= n; ++i) {
            run += (double)f[i - 1] / (double)n;
            cdf_out[i] = (float)(run / total);
        }
    }
    *int_out = (float)total;
}

// One thread per row: the sin(theta)-weighted luminance and the row's CDF.
__global__ void k_env_rows(const float* __restrict__ rgb, int w, int h, float* __restrict__ cond_func,
                           float* __restrict__ cond_cdf, float* __restrict__ cond_int) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= h) return;
    const float sin_theta = (float)sin(3.14159265358979323846 * (double)((float)r / (float)(h - 1)));
    float* f = cond_func + (int64_t)r * w;
    for (int c = 0; c < w; ++c) {
        const float* p = rgb + ((int64_t)r * w + c) * 3;
        const float y = (float)(0.2126 * (double)p[0] + 0.7152 * (double)p[1] + 0.0722 * (double)p[2]);
        f[c] = y * sin_theta;
    }
    dist1d_build(f, w, cond_cdf + (int64_t)r * (w + 1), cond_int + r);
}

__global__ void k_env_marginal(const float* __restrict__ cond_int, int h, float* __restrict__ marg_func,
                               float* __restrict__ marg_cdf, float* __restrict__ marg_int) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int r = 0; r < h; ++r) marg_func[r] = cond_int[r];
    dist1d_build(marg_func, h, marg_cdf, marg_int);
}

// Guide table entry g of each of `rows` CDFs of n + 1 values (row stride
// n + 1): the first index with cdf > g / kEnvGuide, by binary search.
__global__ void k_env_guide(const float* __restrict__ cdf, int n, int rows, int* __restrict__ guide) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)rows * (kEnvGuide + 1)) return;
    const int r = (int)(e / (kEnvGuide + 1)), g = (int)(e % (kEnvGuide + 1));
    const float x = (float)g / (float)kEnvGuide;  // exact
    const float* c = cdf + (int64_t)r * (n + 1);
    int first = 0, len = n + 1;
    while (len > 0) {
        const int half = len >> 1, middle = first + half;
        if (c[middle] <= x) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    guide[e] = first;
}

cudaError_t launch_env_cdf(const float* rgb, int w, int h, float* cond_func, float* cond_cdf,
                           float* cond_int, float* marg_func, float* marg_cdf, float* marg_int,
                           int* cond_guide, int* marg_guide, cudaStream_t st) {
    k_env_rows<<<(h + 63) / 64, 64, 0, st>>>(rgb, w, h, cond_func, cond_cdf, cond_int);
    k_env_marginal<<<1, 32, 0, st>>>(cond_int, h, marg_func, marg_cdf, marg_int);
    const int64_t ne = (int64_t)h * (kEnvGuide + 1);
    k_env_guide<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(cond_cdf, w, h, cond_guide);
    k_env_guide<<<(kEnvGuide + 1 + 255) / 256, 256, 0, st>>>(marg_cdf, h, 1, marg_guide);
    g_launch_counter += 4;
    return cudaGetLastError();
}

}  // namespace lg
