// Host-side launchers of the LightGraph kernels (one .cu file per stage).
// All launchers enqueue on `stream` and return the cudaError_t of the launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lg_device.cuh"

namespace lg {

// Per-graph bookkeeping on the device.
struct GraphInfo {
    int64_t pt_off;   // first point (row of the points array)
    int64_t s_off;    // first float of the graph's S / distance matrix
    int64_t e_off;    // first edge slot
    int32_t n;        // points
    int32_t ld;       // leading dimension of S (multiple of 128, >= n)
    int32_t max_edges;
    float r2;         // searchRadiusConnectSquared
};

constexpr int kCandCap = 96;  // stored candidate partners per row

cudaError_t launch_candidates(const float* pts, const GraphInfo* graphs, const int32_t* pt_graph,
                              int64_t n_points, uint16_t* cand, int32_t* cand_cnt,
                              cudaStream_t st);
cudaError_t launch_greedy(const float* pts, const GraphInfo* graphs, int n_graphs, int max_n,
                          const uint16_t* cand, const int32_t* cand_cnt, int max_connect,
                          int2* edges, int32_t* edge_cnt, cudaStream_t st);
cudaError_t launch_adjacency(const GraphInfo* graphs, int n_graphs, int max_edges,
                             const int2* edges, const int32_t* edge_cnt, uint8_t* adj,
                             const int64_t* adj_off, cudaStream_t st);
cudaError_t launch_fill(float* p, int64_t n, float v, cudaStream_t st);

cudaError_t launch_edge_march(const DevScene& sc, const float* pts, const GraphInfo* graphs,
                              int n_graphs, int max_edges, const int2* edges,
                              const int32_t* edge_cnt, float* S, cudaStream_t st);
cudaError_t launch_vertex_light(const DevScene& sc, const float* pts, const GraphInfo* graphs,
                                int n_graphs, int max_n, float* L, cudaStream_t st);

// Floyd-Warshall on one matrix (general, any n, ld % 4 == 0).
cudaError_t fw_solve(float* d, int n, int ld, cudaStream_t st);
// Batched: every graph's matrix in one set of launches.
cudaError_t fw_solve_batched(float* base, const int64_t* offs, const int32_t* ns,
                             const int32_t* lds, int n_graphs, int max_n, cudaStream_t st);
cudaError_t launch_set_diag(float* S, const GraphInfo* graphs, int n_graphs, int max_n,
                            cudaStream_t st);

constexpr int kRowChunks = 16;  // row chunks of the diffusion column sums
// part: kRowChunks * 3 floats per point; colw: 3 floats per point.
cudaError_t launch_diffuse(const DevShader& sh, const float* S, const GraphInfo* graphs,
                           int n_graphs, int max_n, const float* L, float* part, float* colw,
                           float* D, cudaStream_t st);

// ScatterGrid
struct CoarseGrid {
    int lo[3];      // index of coarse voxel (0,0,0)
    int dims[3];
    float H;        // coarse voxel size
};
cudaError_t launch_coarse_topology(const DevGrid& fine, int factor, const CoarseGrid& cg,
                                   uint8_t* act0, uint8_t* act, cudaStream_t st);
struct PointBins {
    float cell;           // cell edge (>= splat radius)
    float lo[3];          // world position of cell (0,0,0)
    int dims[3];
    int64_t n_cells;
};
cudaError_t launch_bin_points(const float* pts, int64_t n, const PointBins& pb, int32_t* cell_count,
                              int32_t* cell_start, int32_t* cursor, int32_t* sorted,
                              int32_t* scan_tmp, cudaStream_t st);
cudaError_t launch_splat(const CoarseGrid& cg, const uint8_t* act, const float* pts,
                         const float* D, const PointBins& pb, const int32_t* cell_start,
                         const int32_t* cell_count, const int32_t* sorted, float radius,
                         float inv2s2, float4* out, cudaStream_t st);

// Render
struct DevCamera {
    float eye[3];
    float m[9];          // row-vector 3x3 (screen -> world directions)
    float cdir[3];       // central ray direction
    float sw, sh;        // mScaleWidth, mScaleHeight
    float znear, zfar;
    int width, height, spp;
};
struct DevScatterGrid {
    const float4* v;
    int lo[3], dims[3];
    float inv_H;
};
cudaError_t launch_render(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                          float4* rgba, float4* direct, float4* scatter, float4* emission,
                          unsigned long long* counters, cudaStream_t st);

// Environment map CDFs (FP64 prefix sums)
cudaError_t launch_env_cdf(const float* rgb, int w, int h, float* cond_func, float* cond_cdf,
                           float* cond_int, float* marg_func, float* marg_cdf, float* marg_int,
                           cudaStream_t st);

// Grid upload helpers
cudaError_t launch_pack_bricks(const float* dense, const int dims[3], const int origin[3],
                               const DevGrid& g, void* bricks, cudaStream_t st);
// bbox: 6 ints (min xyz, max xyz leaf coordinates), pre-set to +/-INT_MAX.
cudaError_t launch_leaf_bits(const float* dense, const int dims[3], const int origin[3],
                             const uint8_t* leaf_mask, const DevGrid& g, uint32_t* bits, int* bbox,
                             cudaStream_t st);

extern uint64_t g_launch_counter;  // kernel launches issued (all contexts)

}  // namespace lg
