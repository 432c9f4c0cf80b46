/*
 * lg_oracle.h -- CPU oracle of the LightGraph multiple-scattering path.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load this library, and only to produce the results the GPU
 * path is compared with or as the timed CPU baseline: the product
 * (lightgraph_gb300) never links, calls or falls back to it.
 *
 * It restates, in FP64 C++ and in the loop order of the reference
 * (asiroisvigneux/LightGraph), the functions of the hot path:
 *   LightGraph::scatterPoints      src/LightGraph.h:206-274   lgo_scatter_points
 *   LightGraph::buildGraph         src/LightGraph.h:287-318   lgo_build_graph
 *   LightGraph::raymarchConnection src/LightGraph.h:347-418   lgo_march_edges
 *   LightGraph::floydAlgo          src/LightGraph.h:512-542   lgo_fw_maxtimes
 *   LightGraph::computeLighting    src/LightGraph.h:427-505   lgo_vertex_light
 *   LightGraph::diffuseLight       src/LightGraph.h:554-587   lgo_diffuse
 *   LightGraph::buildVdbPointGrid  src/LightGraph.h:706-755   lgo_point_voxel_size
 *   ScatterGrid::buildScatterGrid  src/ScatterGrid.h:105-144  lgo_splat
 *   ScatterGrid::operator()        src/ScatterGrid.h:61-98    lgo_splat
 *   VolumeRender::operator()       src/Renderer.h:505-693     lgo_render
 * plus FP32 and FP64 min-plus Floyd-Warshall (lgo_fw_minplus_f32/_f64), the
 * forms the GPU path is checked against bit-for-bit / within tolerance.
 *
 * PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors,
 * and cannot be built here (it needs OpenVDB, TBB, OpenEXR 2.x and Boost).
 * This restatement is pinned instead by known-answer tests (tests/test_oracle.py)
 * and by the golden fixtures it generates (tests/golden/). Its random
 * sequence alone is pinned to the reference's code: src/RandGen.h, which
 * needs none of those libraries, is compiled from the reference tree
 * (oracle/build_ref.py) and compared draw for draw (tests/test_ref_randgen.py).
 *
 * OpenVDB behaviour the reference leans on is restated from its documented
 * semantics (OpenVDB 7/8 era; the reference pins no version):
 *   BoxSampler trilinear (z, then y, then x; float values, double weights),
 *   Ray::worldToIndex (unit index direction, times scaled by 1/voxel),
 *   Ray::clip to the active leaf bbox padded by one voxel,
 *   VolumeHDDA spans = maximal runs of leaf nodes along the index ray,
 *   GridTransformer + dilateActiveValues topology of the scatter grid,
 *   PointIndexGrid radial search (points with |x - p| < r),
 *   points::computeVoxelSize (bbox estimate refined on voxel occupancy).
 */
#ifndef LG_ORACLE_H_
#define LG_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Data layouts shared with the C ABI (plain structs only). */
#include "../include/lightgraph_c.h"

typedef struct lgo_grid {
    lg_grid_desc desc;
    const float* values;
} lgo_grid;

typedef struct lgo_env {
    const float* rgb; /* h x w x 3 */
    int32_t w, h;
} lgo_env;

/* buildGraph: adj (n*n bytes) gets 1 for connected pairs; returns the
 * number of edges (connectCount). */
int64_t lgo_build_graph(int n, const float* pts, float radius_sq, int max_connect, uint8_t* adj);

/* raymarchConnection. T (n*n*3, optional): the reference's RGB transmittance
 * (0 where no edge). S (n*n, optional): scalar optical depth sum(x*step)
 * (+inf where no edge or dropout). */
void lgo_march_edges(const lgo_grid* dens, const lg_shader* sh, const lg_settings* st, int n,
                     const float* pts, const uint8_t* adj, double* T, double* S);

/* floydAlgo on the RGB matrix (max-times, skip zero), then diagonal = 1. */
void lgo_fw_maxtimes(int n, double* T);
/* Rounds k0 <= k < k1 of floydAlgo's outer loop only (no diagonal reset):
 * a bounded sample of its cost for the CPU baseline. */
void lgo_fw_maxtimes_rounds(int n, double* T, int k0, int k1);

/* Min-plus FW in the reference's (k, i, j) order, no diagonal reset. */
void lgo_fw_minplus_f32(int n, float* S);
void lgo_fw_minplus_f64(int n, double* S);

/* computeLighting for graph `graph_id` (selects its random streams). */
void lgo_vertex_light(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh, const lg_settings* st,
                      const lg_light* lights, int n_lights, const lgo_env* env, int n, const float* pts,
                      int graph_id, double* L);

/* diffuseLight on the RGB path matrix after FW (diagonal 1): P_ij /= max(colsum_j, 1),
 * D_i = sum_j L_j * P_ij. */
void lgo_diffuse(int n, const double* T, const double* L, double* D);

/* points::computeVoxelSize(positions, points_per_voxel) with OpenVDB's
 * defaults (identity transform, five decimal places), as
 * LightGraph::buildVdbPointGrid calls it (src/LightGraph.h:713-714): the
 * point index grid's voxel size, which sets the splat radius. */
double lgo_point_voxel_size(int64_t n, const float* pts, int points_per_voxel);

/* Scatter-grid topology + splat. Output box: lo = floor(origin/f) - 1, dims
 * from that to floor((origin+dims-1)/f) + 1 (same box as the GPU).
 * out: dims product x 3 doubles. Returns the splat radius. */
double lgo_splat(const lgo_grid* dens, int factor, int64_t n_points, const float* pts, const double* D,
                 double point_voxel_size, double kernel_points, int32_t out_lo[3], int32_t out_dims[3],
                 double* out);

/* Render rows [row0, row1) of the image (films width x height x 4 floats,
 * only those rows written). scatter: coarse grid box (lo, dims, 3 floats per
 * voxel, voxel size sg_h) or null. */
void lgo_render(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh, const lg_settings* st,
                const lg_light* lights, int n_lights, const lgo_env* env, const lg_camera* cam,
                const int32_t sg_lo[3], const int32_t sg_dims[3], double sg_h, const float* sg_values,
                int row0, int row1, float* rgba, float* direct, float* scatter, float* emission,
                uint64_t* counters);

/* lgo_render over a list of image rows (any order), in parallel over their
 * pixels: the bounded sample of a frame that the CPU baseline times. */
void lgo_render_rows(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh, const lg_settings* st,
                     const lg_light* lights, int n_lights, const lgo_env* env, const lg_camera* cam,
                     const int32_t sg_lo[3], const int32_t sg_dims[3], double sg_h, const float* sg_values,
                     const int32_t* rows, int n_rows, float* rgba, float* direct, float* scatter, float* emission,
                     uint64_t* counters);

/* Rounds k0 <= k < k1 of FP32 min-plus FW (rows with S_ik = +inf skipped).
 * It reaches the same sparsity pattern as floydAlgo after the same rounds, so
 * the CPU baseline uses it to bring the matrix to a sampled round cheaply. */
void lgo_fw_minplus_f32_rounds(int n, float* S, int k0, int k1);

/* T[e][c] = exp(ext[c] * S[e]) (0 where S is +inf): the RGB transmittance of
 * an optical-depth matrix, as floydAlgo holds it. */
void lgo_transmittance_of(int64_t count, const double* S, const double ext[3], double* T);

/* The env map's importance-sampling CDFs as EnvLight builds them (FP64 prefix
 * sums stored as FP32): cond_func h*w, cond_cdf h*(w+1), cond_int h,
 * marg_func h, marg_cdf h+1, marg_int 1. */
void lgo_env_cdf(const lgo_env* env, float* cond_func, float* cond_cdf, float* cond_int, float* marg_func,
                 float* marg_cdf, float* marg_int);

/* scatterPoints for iterations first_iter .. first_iter + n_iter - 1: points
 * (n_iter x hard_limit x 3; iteration i's counts[i] points at
 * i * hard_limit * 3) and the squared minimum distance of each iteration's
 * last accepted point. Uses the host C++ library's std::mt19937 and
 * std::uniform_real_distribution<float>, as the reference's RandGen does. */
void lgo_scatter_points(const lgo_grid* dens, const lg_scatter_opts* o, int first_iter, int n_iter,
                        float* points, int32_t* counts, float* last_min_dist_sq);

/* n draws of std::mt19937(seed): through std::uniform_real_distribution<float>
 * (0, 1) (out) and raw (raw); either may be NULL. */
void lgo_randgen_draws(uint32_t seed, int64_t n, float* out, uint32_t* raw);

/* Number of OpenMP threads the oracle uses. */
int lgo_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* LG_ORACLE_H_ */
