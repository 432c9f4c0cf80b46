// Host-side launchers of the LightGraph kernels (one .cu file per stage).
// All launchers enqueue on `stream` and return the cudaError_t of the launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

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

// Path-solve schedules (lg_set_fw_schedule): 0 .. kFwSchedules - 1.
constexpr int kFwSchedules = 6;

// Batched: many matrices in one persistent launch.
struct FwGraph {
    int64_t off;   // first float of the matrix
    int32_t n, ld;
    int32_t nt;    // k-blocks of 64
    int32_t nu;    // update tiles of 128 per side
    int64_t vofs;  // first of the graph's nt^2 block version counters and nt round counters
    int64_t pofs;  // first float2 of the graph's column-panel slots (symmetric solve)
};
// Writes the work queue (if items != null) and returns its length. sym: the
// queue of the symmetric solve (tiles on and above the diagonal only).
size_t fw_batched_items(const FwGraph* graphs, int n_graphs, int4* items, bool sym = false);
// Reorders a symmetric queue (fw_batched_items with sym) by list scheduling
// its dependency graph on `workers` simulated CTAs; the result is still a
// dependency order.
void fw_order_sym(const FwGraph* graphs, int n_graphs, int4* items, size_t n_items, int workers);
// Host replay of a queue with the kernels' waits and version updates in
// queue order: 0 if it cannot deadlock and writes every block once per round,
// else the 1-based index of the first offending item (n_items + 1: a block
// missed a round).
size_t fw_queue_replay(const FwGraph* graphs, int n_graphs, const int4* items, size_t n_items, bool sym);
// uint32 words of the batched solve's sync buffer: 2 + sum of nt^2 + nt.
size_t fw_sync_words(const FwGraph* graphs, int n_graphs);
// float2 words of one graph's column-panel slots (symmetric solve).
size_t fw_panel_words(const FwGraph& g);
// sync: fw_sync_words uint32 (cleared here). ctas: persistent CTAs.
cudaError_t fw_solve_batched(float* base, const FwGraph* graphs, const int4* items, int n_items, uint32_t* sync,
                             size_t sync_words, int ctas, cudaStream_t st);
// The same solve for symmetric matrices (every S_ij == S_ji, as LightGraph's
// path matrices are): computes the tiles on and above the diagonal and then
// mirrors them below it. panels: sum of fw_panel_words float2. tma: the update
// tiles stage their operands with TMA bulk copies instead of through registers
// (the same results bit for bit).
cudaError_t fw_solve_batched_sym(float* base, const FwGraph* graphs, int n_graphs, int max_nt, const int4* items,
                                 int n_items, uint32_t* sync, size_t sync_words, float2* panels, int ctas, bool tma,
                                 cudaStream_t st);
int fw_persistent_ctas_per_sm();
// FP32 ops/s (an add and a min per update) of the update tiles' inner loop
// alone on shared-memory operands, 2 CTAs per SM. scratch: 2 * sms * 256 floats.
cudaError_t fw_inner_loop_rate(float* scratch, int sms, double* tflops, cudaStream_t st);
// The persistent solves' bounded dependency wait run alone on a flag that
// nothing sets (words: 4 zeroed words; words[1] = error word, words[2] = 1
// when the wait gave up).
cudaError_t wait_probe(uint32_t* words, uint32_t limit, cudaStream_t st);
int fw_persistent_sym_ctas_per_sm();
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
// One shading sample of a primary ray: where its shadow rays start and the
// weight pTrans * (1 - dT) of their contribution.
struct ShadowTask {
    float p[3];    // index-space position
    float w[3];    // pTrans * (1 - dT) per channel
    uint32_t sa;   // the pixel-sample stream's first word and the primary
    uint32_t iw;   // iteration's word: they key the shadow random streams
};
static_assert(sizeof(ShadowTask) == 32, "ShadowTask is two 16-byte words");
size_t pixel_sample_bytes();
// Ordering of the shadow rays of one light: tasks are counting-sorted by a
// key that groups rays which cross the same part of the volume, so the rays
// in flight share cache lines and the lanes of a warp walk similar paths.
//   kind 0 (distant light, parallel rays): (u, v) bin of the start point
//          projected on the plane normal to the ray direction D, in Morton
//          order, then the depth bin along D;
//   kind 1 (point light, rays through O): cube-map face and (s, t) bin of the
//          direction from O to the start point, then the distance bin;
//   kind 2 (environment light, random directions): task order in buckets of
//          2^shift tasks.
struct RayBin {
    int kind, ns, nd, shift;  // ns: (u, v) or (s, t) bins per side (power of two), nd: depth bins
    float U[3], V[3], D[3];   // kind 0: orthonormal basis, D the ray direction
    float O[3];               // kind 1: light position (index space)
    float u0, v0, inv_bs;     // kind 0: projected origin, 1 / bin size
    float d0, inv_ds;         // depth origin, 1 / depth bin size
    int64_t key_off, nkeys;   // this light's keys in the combined histogram
    // Occupancy bound per light-space bin (kinds 0 and 1; null: none). A
    // distant light's shadow ray stays in its (u, v) column and a point
    // light's in its cube-map cone, so no leaf lies on the ray past the
    // column's largest leaf depth - d0 (kind 0, ns x ns, v major) or closer to
    // the light than the cone's smallest leaf distance (kind 1, 6 x ns x ns,
    // face major). k_shadow ends its walk there, past every leaf it can meet.
    float* bound;
};
struct RayBins {
    RayBin b[kMaxLights];
    int n;
};
constexpr int kRayUnit = 2;  // consecutive tasks ordered as one unit
// Scatter pass of the shadow-ray order over all lights: offsets holds the
// exclusive scan of the per-key unit counts; order[offsets[key]++] = unit,
// the keys read from keys (n_lights rows of unit_cap).
cudaError_t launch_ray_scatter(const uint32_t* keys, int64_t unit_cap, int n_lights, const int32_t* total,
                               int64_t task_cap, int32_t* offsets, int32_t* order, int sms, cudaStream_t st);
// Fills the occupancy bounds of every light of rb with a bound table (kind 0:
// rb.b[k].ns^2 floats, kind 1: 6 * ns^2, zeroed or set to +inf first by the
// caller as bound_init gives): one thread per leaf-bitmap cell.
cudaError_t launch_ray_bounds(const DevGrid& g, const RayBins& rb, cudaStream_t st);
// expm1_approx (the primary wave's e^x - 1) and expm1f at n points, for the
// accuracy check behind lg_expm1_check.
cudaError_t launch_expm1_check(const float* x, float* approx, float* ref, int n, cudaStream_t st);
// Initial value of a light's bound table entries (bits of a non-negative float).
inline uint32_t bound_init(const RayBin& b) { return b.kind == 0 ? 0u : 0x7F800000u; }
inline int64_t bound_entries(const RayBin& b) {
    return b.kind == 0 ? (int64_t)b.ns * b.ns : b.kind == 1 ? 6 * (int64_t)b.ns * b.ns : 0;
}
// Wave 1: counts[ps] = shading samples of each pixel-sample.
// claim: a zeroed counter the persistent grid's warps claim pixel samples
// from.
cudaError_t launch_render_count(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg, int32_t* counts,
                                unsigned long long* claim, int sms, cudaStream_t st,
                                bool short_ctas = false);
// Shadow-ray ordering buffers: key_counts and key_offsets hold rb's keys,
// key_scan the scan's block sums (keys / 1024 + 2), order n_lights * units
// (units of kRayUnit tasks).
struct RayOrder {
    RayBins rb;
    int64_t n_keys;
    int32_t *key_counts, *key_offsets, *key_scan, *key_total, *order;
    // the order key of every unit and light (light k's keys from
    // k * unit_cap), written by the primary shading pass with the counts
    uint32_t* keys;
    int64_t unit_cap;
};
// Waves 2-5 given the exclusive scan of the counts (offsets, device total):
// primary shading, shadow-ray ordering, shadow rays, resolve. direct holds
// n_lights * task_cap per-light contributions. marks (4 events, optional)
// are recorded after each wave.
cudaError_t launch_render_shade(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                                const int32_t* counts, const int32_t* offsets, const int32_t* total,
                                ShadowTask* tasks, int64_t task_cap, void* pixel_samples, const RayOrder& ro,
                                float4* direct, float4* rgba, float4* dfilm, float4* sfilm, float4* efilm,
                                unsigned long long* counters, int sms, cudaStream_t st,
                                cudaEvent_t* marks = nullptr);
// Exclusive scan of n int32 (block_sums: n/1024 + 1 ints); *total = sum.
cudaError_t launch_exclusive_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* block_sums, int32_t* total,
                                  cudaStream_t st);

// Bounding box of the non-zero voxels of a dense array (array coordinates;
// bbox pre-set to +/-INT_MAX).
cudaError_t launch_voxel_bbox(const float* dense, const int dims[3], int* bbox, cudaStream_t st);

// Dart throwing (LightGraph::scatterPoints), one CTA per iteration.
struct DartParams {
    uint32_t scatter_count, target, batch, hard_limit;
    float cutoff, min_dist_sq0;
    uint32_t seed_base;
    int first_iter;
    double bbmin[3];  // active-voxel bbox, world space
    float bbsize[3];
    double wo[3], h;  // the grid's world origin and voxel size
    float wo_f[3], inv_h_f;  // the same in FP32 (fast path)
    float index_err;         // bound of the FP32 index-position error (voxels)
};
// expected: the expected sizes at the scatter_count / batch radius updates;
// out_pts: n_iter x hard_limit x 3 floats; out_last_m2: the squared minimum
// distance of each iteration's last accepted point.
cudaError_t launch_dart(const DevGrid& g, const DartParams& prm, int n_iter, const uint32_t* expected, float* out_pts,
                        int32_t* out_count, float* out_last_m2, cudaStream_t st);

// Environment map CDFs (FP64 prefix sums)
cudaError_t launch_env_cdf(const float* rgb, int w, int h, float* cond_func, float* cond_cdf,
                           float* cond_int, float* marg_func, float* marg_cdf, float* marg_int,
                           int* cond_guide, int* marg_guide,
                           cudaStream_t st);

// Grid upload helpers
cudaError_t launch_pack_bricks(const float* dense, const int dims[3], const int origin[3],
                               const DevGrid& g, void* bricks, cudaStream_t st);
// bbox: 6 ints (min xyz, max xyz leaf coordinates), pre-set to +/-INT_MAX.
cudaError_t launch_leaf_bits(const float* dense, const int dims[3], const int origin[3],
                             const uint8_t* leaf_mask, const DevGrid& g, uint32_t* bits, int* bbox,
                             cudaStream_t st);

extern std::atomic<uint64_t> g_launch_counter;  // kernel launches issued (all contexts, all host threads)
// Raises a kernel's dynamic shared-memory limit on the current device, once
// per (device, kernel), to all the device allows next to the kernel's static
// shared memory. The limit is one setting per kernel and device shared by
// every host thread, so a launcher that set it to its own launch's size could
// lower it under another thread's larger launch (the server's slots launch
// concurrently); it is set once, to the maximum.
cudaError_t raise_smem_limit(const void* func);

}  // namespace lg
