// ScatterGrid: topology (ScatterGrid::buildScatterGrid, src/ScatterGrid.h:105-144),
// point index (LightGraph::buildVdbPointGrid, src/LightGraph.h:706-755) and the
// truncated-Gaussian splat (ScatterGrid::operator(), src/ScatterGrid.h:61-98).
//
// Topology: the reference copies the density topology, resamples it to a
// voxel `factor` times larger with trilinear GridTransformer (a coarse voxel
// becomes active when an active fine voxel falls in its footprint), then
// dilates it by one voxel in the 26-neighbourhood. Here: coarse voxel c is
// active when a non-zero density voxel v has floor(v / factor) == c, and the
// mask is dilated by one.
//
// Point index: a uniform grid of cells at least one splat radius wide,
// filled by a counting sort. Each cell's points are then ordered by index so
// every sum below runs in a fixed order (deterministic output).
//
// Splat: per active coarse voxel at world x, the weighted mean of the solved
// radiances D_p of points within the radius, w = exp(-|x - p|^2 / (2 sigma^2))
// with the kernel truncated at w = TRUNCATED_GAUSSIAN_TAIL (0.1); 0 if none.
#include "lg_kernels.h"

namespace lg {

__global__ void k_coarse_active0(DevGrid fine, int factor, CoarseGrid cg, uint8_t* __restrict__ act0) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (idx >= total) return;
    const int cx = (int)(idx % cg.dims[0]);
    const int cy = (int)((idx / cg.dims[0]) % cg.dims[1]);
    const int cz = (int)(idx / ((int64_t)cg.dims[0] * cg.dims[1]));
    const int fx0 = (cg.lo[0] + cx) * factor, fy0 = (cg.lo[1] + cy) * factor,
              fz0 = (cg.lo[2] + cz) * factor;
    uint8_t a = 0;
    for (int z = 0; z < factor && !a; ++z)
        for (int y = 0; y < factor && !a; ++y)
            for (int x = 0; x < factor; ++x)
                if (voxel(fine, fx0 + x, fy0 + y, fz0 + z) != 0.f) { a = 1; break; }
    act0[idx] = a;
}

__global__ void k_dilate(CoarseGrid cg, const uint8_t* __restrict__ act0, uint8_t* __restrict__ act) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (idx >= total) return;
    const int cx = (int)(idx % cg.dims[0]);
    const int cy = (int)((idx / cg.dims[0]) % cg.dims[1]);
    const int cz = (int)(idx / ((int64_t)cg.dims[0] * cg.dims[1]));
    uint8_t a = 0;
    for (int dz = -1; dz <= 1 && !a; ++dz)
        for (int dy = -1; dy <= 1 && !a; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = cx + dx, y = cy + dy, z = cz + dz;
                if (x < 0 || y < 0 || z < 0 || x >= cg.dims[0] || y >= cg.dims[1] || z >= cg.dims[2]) continue;
                if (act0[((int64_t)z * cg.dims[1] + y) * cg.dims[0] + x]) { a = 1; break; }
            }
    act[idx] = a;
}

cudaError_t launch_coarse_topology(const DevGrid& fine, int factor, const CoarseGrid& cg,
                                   uint8_t* act0, uint8_t* act, cudaStream_t st) {
    const int64_t total = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (total == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    k_coarse_active0<<<blocks, 256, 0, st>>>(fine, factor, cg, act0);
    k_dilate<<<blocks, 256, 0, st>>>(cg, act0, act);
    g_launch_counter += 2;
    return cudaGetLastError();
}

__device__ __forceinline__ int64_t point_cell(const PointBins& pb, float x, float y, float z) {
    int cx = (int)floorf((x - pb.lo[0]) / pb.cell);
    int cy = (int)floorf((y - pb.lo[1]) / pb.cell);
    int cz = (int)floorf((z - pb.lo[2]) / pb.cell);
    cx = min(max(cx, 0), pb.dims[0] - 1);
    cy = min(max(cy, 0), pb.dims[1] - 1);
    cz = min(max(cz, 0), pb.dims[2] - 1);
    return ((int64_t)cz * pb.dims[1] + cy) * pb.dims[0] + cx;
}

__global__ void k_bin_count(const float* __restrict__ pts, int64_t n, PointBins pb,
                            int32_t* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(count + point_cell(pb, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), 1);
}

// Exclusive scan in blocks of 1024 elements; block totals to `sums`.
__global__ void __launch_bounds__(1024) k_scan_block(const int32_t* __restrict__ in, int64_t n,
                                                     int32_t* __restrict__ out, int32_t* __restrict__ sums) {
    __shared__ int32_t warp_tot[32];
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t v = i < n ? in[i] : 0;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int32_t excl = x - v + (wid > 0 ? warp_tot[wid - 1] : 0);
    if (i < n) out[i] = excl;
    if (threadIdx.x == 1023) sums[blockIdx.x] = excl + v;
}

// Exclusive scan of the block totals by one block, in chunks of 1024.
__global__ void __launch_bounds__(1024) k_scan_sums(int32_t* __restrict__ sums, int64_t nb) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t base = 0; base < nb; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int32_t v = i < nb ? sums[i] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int32_t t = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int32_t excl = x - v + (wid > 0 ? warp_tot[wid - 1] : 0) + carry;
        if (i < nb) sums[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_scan_add(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ sums,
                           int32_t* __restrict__ cursor) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t v = out[i] + sums[i / 1024];
    out[i] = v;
    cursor[i] = v;
}

__global__ void k_scan_add_total(int32_t* __restrict__ out, const int32_t* __restrict__ in, int64_t n,
                                 const int32_t* __restrict__ sums, int32_t* __restrict__ total) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t v = out[i] + sums[i / 1024];
    out[i] = v;
    if (i == n - 1 && total) *total = v + in[i];
}

cudaError_t launch_exclusive_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* block_sums, int32_t* total,
                                  cudaStream_t st) {
    if (n <= 0) return total ? cudaMemsetAsync(total, 0, sizeof(int32_t), st) : cudaSuccess;
    const int64_t nb = (n + 1023) / 1024;
    k_scan_block<<<(unsigned)nb, 1024, 0, st>>>(in, n, out, block_sums);
    k_scan_sums<<<1, 1024, 0, st>>>(block_sums, nb);
    k_scan_add_total<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, in, n, block_sums, total);
    g_launch_counter += 3;
    return cudaGetLastError();
}

__global__ void k_bin_scatter(const float* __restrict__ pts, int64_t n, PointBins pb,
                              int32_t* __restrict__ cursor, int32_t* __restrict__ sorted) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t c = point_cell(pb, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    sorted[atomicAdd(cursor + c, 1)] = (int32_t)i;
}

// Orders each cell's points by index (insertion sort; cells hold few points).
__global__ void k_bin_order(int64_t n_cells, const int32_t* __restrict__ start,
                            const int32_t* __restrict__ count, int32_t* __restrict__ sorted) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    int32_t* s = sorted + start[c];
    const int m = count[c];
    for (int a = 1; a < m; ++a) {
        const int32_t key = s[a];
        int b = a - 1;
        while (b >= 0 && s[b] > key) { s[b + 1] = s[b]; --b; }
        s[b + 1] = key;
    }
}

cudaError_t launch_bin_points(const float* pts, int64_t n, const PointBins& pb, int32_t* cell_count,
                              int32_t* cell_start, int32_t* cursor, int32_t* sorted,
                              int32_t* scan_tmp, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(cell_count, 0, sizeof(int32_t) * pb.n_cells, st);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        k_bin_count<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pts, n, pb, cell_count);
        ++g_launch_counter;
    }
    const int64_t nb = (pb.n_cells + 1023) / 1024;
    k_scan_block<<<(unsigned)nb, 1024, 0, st>>>(cell_count, pb.n_cells, cell_start, scan_tmp);
    k_scan_sums<<<1, 1024, 0, st>>>(scan_tmp, nb);
    k_scan_add<<<(unsigned)((pb.n_cells + 255) / 256), 256, 0, st>>>(cell_start, pb.n_cells, scan_tmp, cursor);
    g_launch_counter += 3;
    if (n > 0) {
        k_bin_scatter<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pts, n, pb, cursor, sorted);
        ++g_launch_counter;
    }
    k_bin_order<<<(unsigned)((pb.n_cells + 255) / 256), 256, 0, st>>>(pb.n_cells, cell_start, cell_count, sorted);
    ++g_launch_counter;
    return cudaGetLastError();
}

__global__ void __launch_bounds__(128) k_splat(CoarseGrid cg, const uint8_t* __restrict__ act,
                                               const float* __restrict__ pts, const float* __restrict__ D,
                                               PointBins pb, const int32_t* __restrict__ start,
                                               const int32_t* __restrict__ count,
                                               const int32_t* __restrict__ sorted, float r2,
                                               float inv2s2, float4* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (idx >= total) return;
    if (!act[idx]) { out[idx] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    const int cx = (int)(idx % cg.dims[0]);
    const int cy = (int)((idx / cg.dims[0]) % cg.dims[1]);
    const int cz = (int)(idx / ((int64_t)cg.dims[0] * cg.dims[1]));
    // coarse voxel centre in world space (transform: world = index * H)
    const float x = (float)(cg.lo[0] + cx) * cg.H, y = (float)(cg.lo[1] + cy) * cg.H,
                z = (float)(cg.lo[2] + cz) * cg.H;
    const int qx = (int)floorf((x - pb.lo[0]) / pb.cell), qy = (int)floorf((y - pb.lo[1]) / pb.cell),
              qz = (int)floorf((z - pb.lo[2]) / pb.cell);
    float wsum = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int dz = -1; dz <= 1; ++dz) {
        const int z3 = qz + dz;
        if (z3 < 0 || z3 >= pb.dims[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y3 = qy + dy;
            if (y3 < 0 || y3 >= pb.dims[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x3 = qx + dx;
                if (x3 < 0 || x3 >= pb.dims[0]) continue;
                const int64_t c = ((int64_t)z3 * pb.dims[1] + y3) * pb.dims[0] + x3;
                const int32_t b = start[c], m = count[c];
                for (int k = 0; k < m; ++k) {
                    const int32_t p = sorted[b + k];
                    const float ex = x - pts[3 * p], ey = y - pts[3 * p + 1], ez = z - pts[3 * p + 2];
                    const float d2 = ex * ex + ey * ey + ez * ez;
                    if (!(d2 < r2)) continue;
                    const float w = expf(-inv2s2 * d2);
                    wsum += w;
                    s0 += D[3 * p] * w;
                    s1 += D[3 * p + 1] * w;
                    s2 += D[3 * p + 2] * w;
                }
            }
        }
    }
    if (wsum > 0.f) { s0 /= wsum; s1 /= wsum; s2 /= wsum; }
    out[idx] = make_float4(s0, s1, s2, 0.f);
}

cudaError_t launch_splat(const CoarseGrid& cg, const uint8_t* act, const float* pts,
                         const float* D, const PointBins& pb, const int32_t* cell_start,
                         const int32_t* cell_count, const int32_t* sorted, float radius,
                         float inv2s2, float4* out, cudaStream_t st) {
    const int64_t total = (int64_t)cg.dims[0] * cg.dims[1] * cg.dims[2];
    if (total == 0) return cudaSuccess;
    k_splat<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(cg, act, pts, D, pb, cell_start, cell_count,
                                                             sorted, radius * radius, inv2s2, out);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg
