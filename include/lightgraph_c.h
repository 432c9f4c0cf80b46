/*
 * lightgraph_c.h -- C ABI of the GB300-native LightGraph multiple-scattering path.
 *
 * The reference (asiroisvigneux/LightGraph) exposes its hot path as three C++
 * classes compiled into one executable: LightGraph (src/LightGraph.h:32-153),
 * ScatterGrid (src/ScatterGrid.h:20-56) and VolumeRender (src/Renderer.h:403-448).
 * Every entry point below replaces one of their member functions; the comment on
 * each names the reference function (file:line) it stands in for.
 *
 * Conventions
 *  - Every call returns an lg_status (LG_OK == 0). On failure lg_last_error()
 *    returns a NUL-terminated description owned by the context.
 *  - Plain pointers and sizes only. Unless a name ends in _device, pointers are
 *    HOST memory owned by the caller; the library copies in/out.
 *  - A context owns one CUDA stream on one device. Calls on one context are
 *    serialised by an internal mutex; use one context per host thread for
 *    concurrency (the serving entry points overlap requests internally).
 *  - All work is deterministic: the same inputs give bit-identical outputs,
 *    independent of how many other requests share the GPU.
 *  - World/index convention (OpenVDB linear transform, uniform voxels):
 *      world = index * voxel_size + world_origin
 *    Voxel centres sit at integer index coordinates. Leaves are the aligned
 *    8^3 bricks of index space (index >> 3).
 */
#ifndef LIGHTGRAPH_C_H_
#define LIGHTGRAPH_C_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int lg_status;
#define LG_OK            0
#define LG_ERR_INVALID   1  /* bad argument (null pointer, size, range)        */
#define LG_ERR_CUDA      2  /* CUDA runtime failure                            */
#define LG_ERR_NOMEM     3  /* device allocation failed or HBM budget exceeded */
#define LG_ERR_STATE     4  /* call order (e.g. render before a grid upload)   */
#define LG_ERR_TIMEOUT   5  /* a bounded device-side wait expired              */
#define LG_ERR_NODEVICE  6  /* no CUDA device / extension built without GPU    */
#define LG_ERR_BUSY      7  /* serving queue full                              */

typedef struct lg_ctx lg_ctx;

/* ------------------------------------------------------------------------- */
/* Grids                                                                     */
/* ------------------------------------------------------------------------- */

#define LG_GRID_DENSITY      0
#define LG_GRID_TEMPERATURE  1

#define LG_DTYPE_F32   0
#define LG_DTYPE_F16   1
#define LG_DTYPE_BF16  2

/* A FloatGrid handed over as a dense box of voxels.
 * values[(z*dims[1] + y)*dims[0] + x] is the voxel at index
 * (origin[0]+x, origin[1]+y, origin[2]+z). Voxels outside the box are the
 * background value 0, as in a sparse VDB. origin must be a multiple of 8 so the
 * box is made of whole leaves.
 * leaf_mask (optional) marks which 8^3 leaves exist, one byte per leaf over
 * ceil(dims/8), x fastest; NULL means "a leaf exists iff one of its voxels is
 * non-zero", which is what converting a dense grid to a VDB produces. */
typedef struct lg_grid_desc {
    int32_t dims[3];
    int32_t origin[3];
    double  voxel_size;
    double  world_origin[3];
    const uint8_t* leaf_mask;
} lg_grid_desc;

/* Uploads a grid once into the device brick layout (8^3 bricks, one padding
 * brick on every side, stored as storage_dtype; FP32 math on read). Replaces
 * the openvdb::io::File::readGrid + GridSampler set-up at src/main.cc:486-502.
 * Re-uploading replaces the previous grid of that kind. The padded box must
 * lie within +-(2^22 - 64) voxels of index 0 on every axis (the marches work
 * in FP32 index space) and hold fewer than 2^32 voxels; LG_ERR_INVALID
 * otherwise. */
lg_status lg_upload_grid(lg_ctx* ctx, int which, const lg_grid_desc* desc,
                         const float* values, int storage_dtype);

/* Drops the temperature grid (samples then read 0, like the empty grid the
 * reference creates at src/main.cc:500). */
lg_status lg_clear_temperature(lg_ctx* ctx);

/* ------------------------------------------------------------------------- */
/* Scene description                                                         */
/* ------------------------------------------------------------------------- */

#define LG_MAX_RAMP_KEYS 16
#define LG_MAX_LIGHTS    8

/* Shader (src/Shader.h:100-274). albedo and extinction are the derived values
 * (Shader::recomputeAlbedo/recomputeExtinction, src/Shader.h:205-211); the
 * caller computes them, exactly as the reference setters do. */
typedef struct lg_shader {
    double density_scale;
    double density_max;
    double shadow_density_scale;
    double scatter_density_scale;
    double scatter_density_min;
    double scattering[3];
    double albedo[3];
    double extinction[3];          /* <= 0 per channel: -(scattering+absorption) */
    double emission_scale;
    double scatter_scale;
    double scatter_density_mask_power;
    int32_t ramp_n;                /* 0: ColorRamp with no keys (black)          */
    int32_t _pad0;
    double ramp_pos[LG_MAX_RAMP_KEYS];
    double ramp_color[LG_MAX_RAMP_KEYS][3];
    double ramp_in;
    double ramp_out;
} lg_shader;

#define LG_LIGHT_DISTANT 0
#define LG_LIGHT_POINT   1
#define LG_LIGHT_ENV     2

/* One light (src/Light.h:26-235) with its transform already applied:
 *  DISTANT: dir = normalised xform.transform(0,0,-1) (DistantLight::mDir)
 *  POINT:   pos = xform.transform(pos)               (PointLight::mPos)
 *  ENV:     rot = 3x3 row-vector rotation applied to sampled directions
 *           (EnvLight::mXform); the map comes from lg_set_lights. */
typedef struct lg_light {
    int32_t type;
    int32_t samples;               /* Light::mSamples (1 for distant/point)      */
    double  color[3];
    double  intensity;             /* Light::mIntensity (a float in the reference) */
    double  dir[3];
    double  pos[3];
    double  rot[9];
} lg_light;

/* Sets the lights. env_rgb (optional, env_h rows x env_w cols x RGB, row 0 at
 * phi = 0) is the environment map shared by ENV lights; its importance-sampling
 * CDFs (src/Sampling.h:76-167, src/Light.h:150-177) are built on the device
 * with FP64 prefix sums. */
lg_status lg_set_lights(lg_ctx* ctx, const lg_light* lights, int n_lights,
                        const float* env_rgb, int env_w, int env_h);

lg_status lg_set_shader(lg_ctx* ctx, const lg_shader* shader);

/* SceneSettings fields the hot path reads (src/SceneSettings.h:21-63), plus
 * the seed of the counter-based random streams that replace RandGen. */
typedef struct lg_settings {
    double   cutoff;
    double   step[2];              /* primary, shadow step in voxels             */
    int32_t  iter;                 /* number of LightGraphs (splat kernel size)  */
    int32_t  scatter_grid_res_factor;
    int32_t  pts_per_kernel;
    int32_t  _pad0;
    uint64_t seed;
} lg_settings;

lg_status lg_set_settings(lg_ctx* ctx, const lg_settings* settings);

/* PerspectiveCamera (src/Renderer.h:129-248) as main.cc:96-102 builds it. */
typedef struct lg_camera {
    double  rotate[3];             /* degrees, X then Y then Z (camRotate)       */
    double  translate[3];          /* camTranslate                               */
    double  y_rotate;              /* camYRotate (turntable, degrees)            */
    double  focal;                 /* mm                                         */
    double  aperture;              /* mm                                         */
    double  znear;
    double  zfar;
    int32_t width;
    int32_t height;
    int32_t samples;               /* antialiasing samples per pixel            */
    int32_t _pad0;
} lg_camera;

/* ------------------------------------------------------------------------- */
/* Context                                                                   */
/* ------------------------------------------------------------------------- */

lg_status lg_create(int device, lg_ctx** out);
lg_status lg_destroy(lg_ctx* ctx);
const char* lg_last_error(const lg_ctx* ctx);
/* The context's cudaStream_t, for callers that time with CUDA events. */
void* lg_stream(lg_ctx* ctx);
/* Library version string and the number of kernel launches issued so far. */
const char* lg_version(void);
uint64_t lg_kernel_launches(const lg_ctx* ctx);

/* ------------------------------------------------------------------------- */
/* Stage 1: LightGraph solve (LightGraph::operator(), src/LightGraph.h:158-196) */
/* ------------------------------------------------------------------------- */

/* Dart throwing of the LightGraph points: the constants of
 * LightGraph::scatterPoints (src/LightGraph.h:22-28, src/main.cc:60-61) and
 * RandGen's seeds (src/RandGen.h:28-30). */
typedef struct lg_scatter_opts {
    uint32_t scatter_count;  /* candidates per iteration, PC_SCATTER_COUNT 1000000       */
    uint32_t target_size;    /* stop once more are accepted, TARGET_PC_SIZE 750          */
    uint32_t n_estimates;    /* radius updates per iteration, PC_GROWTH_NUMBER_OF_ESTIMATE 100 */
    uint32_t hard_limit;     /* point capacity per iteration, PC_SIZE_HARD_LIMIT 1000    */
    float growth_power;      /* PC_GROWTH_FUNC_POWER 0.17                                */
    float density_cutoff;    /* PC_DENSITY_CUTOFF 0.001                                  */
    float min_dist_mult;     /* MIN_DIST_MULT 0.13 (x mean active-bbox edge)             */
    float connect_mult;      /* CONNECT_SEARCH_RADIUS_MULT 1.7                            */
    uint32_t seed_base;      /* iteration i's mt19937 is seeded with seed_base + i, 854123 */
    uint32_t _pad0;
} lg_scatter_opts;
lg_status lg_scatter_opts_default(lg_scatter_opts* out);

/* RandGen::operator() (src/RandGen.h:37-39) on the host: n draws of the
 * mt19937 seeded with seed, as the uniform floats the reference reads (out)
 * and as raw 32-bit outputs (raw); either may be NULL. */
lg_status lg_randgen_draws(uint32_t seed, int64_t n, float* out, uint32_t* raw);

/* LightGraph::scatterPoints (src/LightGraph.h:206-274) for iterations
 * first_iter .. first_iter + n_iter - 1, on the density grid uploaded in ctx
 * (sampled as the reference's BoxSampler, inside its active-voxel bbox):
 * the same mt19937 streams, candidate order, adaptive minimum distance and
 * early stop, so the accepted points are the reference's.
 *   points   : n_iter x hard_limit x 3 floats (optional); iteration i's
 *              counts[i] points start at i * hard_limit * 3
 *   counts   : n_iter accepted-point counts (optional)
 *   radius_sq: n_iter values (minDist * connect_mult)^2, the graph build's
 *              searchRadiusConnectSquared (src/LightGraph.h:170-171) (optional) */
lg_status lg_scatter_points(lg_ctx* ctx, const lg_scatter_opts* opts, int first_iter, int n_iter, float* points,
                            int32_t* counts, float* radius_sq);

/* lg_scatter_points followed by lg_build_graphs on its output: the loop of
 * LightGraph::operator() up to buildGraph (src/LightGraph.h:158-177) for
 * n_iter iterations at once, each iteration one graph.
 *   counts: n_iter point counts (optional) */
lg_status lg_scatter_graphs(lg_ctx* ctx, const lg_scatter_opts* opts, int first_iter, int n_iter, int max_connect,
                            int32_t* counts);

/* Loads n_graphs point sets (the output of LightGraph::scatterPoints,
 * src/LightGraph.h:206-274, injected by the caller) and connects each with the
 * reference's greedy rule: pairs closer than sqrt(radius_sq[g]) in FP64, at
 * most max_connect edges per point, decided in (i, j) order.
 * Replaces LightGraph::buildGraph (src/LightGraph.h:287-318).
 *   n_graphs: 1..65535 graphs of 0..65535 points each (LG_ERR_INVALID otherwise)
 *   points  : sum(N_g) x 3 floats, graph g occupies rows offsets[g]..offsets[g+1]
 *   radius_sq: per graph, the FP32 value searchRadiusConnectSquared
 *   adj_out : optional, sum(N_g^2) bytes, graph g row-major at sum_{h<g} N_h^2
 *   n_edges_out: optional, per graph edge count (connectCount) */
lg_status lg_build_graphs(lg_ctx* ctx, int n_graphs, const float* points,
                          const int64_t* offsets, const float* radius_sq,
                          int max_connect, uint8_t* adj_out, int64_t* n_edges_out);

/* Ray-marches every edge of the loaded graphs into a scalar optical depth
 * S_ij = sum over samples of max(rho, densityMin) * step (voxel units), so the
 * reference's RGB edge transmittance is T_c = exp(extinction_c * S_ij); no edge,
 * a bbox miss or a dropout gives +inf (T = 0).
 * Replaces LightGraph::raymarchConnection (src/LightGraph.h:347-418).
 *   S_out: optional, sum(N_g^2) floats (graph-major, row-major). */
lg_status lg_march_edges(lg_ctx* ctx, float* S_out);

/* All-pairs most-transmissive paths: min-plus Floyd-Warshall over S on the
 * device (equal to the reference's per-channel max-times FW on T because every
 * channel is exp(-a_c * S)), then the diagonal is set to 0 (T = 1).
 * Replaces LightGraph::floydAlgo (src/LightGraph.h:512-542).
 *   dist_out: optional, sum(N_g^2) floats. */
lg_status lg_solve_paths(lg_ctx* ctx, float* dist_out);

/* Direct lighting plus emission per vertex.
 * Replaces LightGraph::computeLighting (src/LightGraph.h:427-505).
 *   light_out: optional, sum(N_g) x 3 floats. */
lg_status lg_vertex_light(lg_ctx* ctx, float* light_out);

/* Column-normalised diffusion of vertex radiance through the path matrix.
 * Replaces LightGraph::diffuseLight (src/LightGraph.h:554-587).
 *   diffuse_out: optional, sum(N_g) x 3 floats (mDiffusePointGather). */
lg_status lg_diffuse(lg_ctx* ctx, float* diffuse_out);

/* Runs lg_march_edges, lg_solve_paths, lg_vertex_light and lg_diffuse. */
lg_status lg_solve_graphs(lg_ctx* ctx, float* diffuse_out);

/* ------------------------------------------------------------------------- */
/* Stage 2: ScatterGrid (src/ScatterGrid.h:61-144, src/LightGraph.h:706-755)  */
/* ------------------------------------------------------------------------- */

/* Builds the coarse scatter grid (voxel = density voxel * res_factor, topology
 * = coarse voxels covering an active density voxel, dilated by one) and splats
 * every solved vertex into it with the truncated Gaussian of ScatterGrid.
 *   point_voxel_size: voxel size of the point index (computeVoxelSize at
 *   src/LightGraph.h:714); <= 0 selects lg_point_voxel_size() of the points. */
lg_status lg_splat(lg_ctx* ctx, double point_voxel_size);

/* The point index's voxel size that lg_splat uses when it gets
 * point_voxel_size <= 0: points::computeVoxelSize(positions, 8) as
 * LightGraph::buildVdbPointGrid calls it (src/LightGraph.h:713-714) -- a
 * bounding-box estimate refined on the voxels the points occupy, rounded to
 * five decimal places; 0.1 for fewer than two or coincident points. Host
 * only (no device work). */
double lg_point_voxel_size(int64_t n_points, const float* points, int points_per_voxel);

/* Copies out the scatter grid: dims/origin of the coarse dense box and, if
 * values is non-null, dims[0]*dims[1]*dims[2]*3 floats (0 = inactive). */
lg_status lg_get_scatter_grid(lg_ctx* ctx, int32_t dims[3], int32_t origin[3],
                              float* values);

/* Vertex light / diffuse radiance of all loaded points (sum(N_g) x 3). */
lg_status lg_get_vertex_data(lg_ctx* ctx, float* light_out, float* diffuse_out);

/* LightGraph::outputDebugGeo (src/LightGraph.h:604-696), the -geoDump flag:
 * for every loaded graph g writes dir/stem_{pc,edge,marching,light,diffuse}_NNNN.txt
 * with NNNN = first_iter + g: point positions, edges (i < j, row-major order),
 * the solved and column-normalised RGB path weights of those edges, and the
 * direct and diffused vertex radiance, one comma-separated line each
 * (6 significant digits). Needs lg_solve_graphs first; creates dir. */
lg_status lg_geo_dump(lg_ctx* ctx, const char* dir, const char* stem, int first_iter);

/* ------------------------------------------------------------------------- */
/* Stage 3: render (VolumeRender::render / operator(), src/Renderer.h:496-693) */
/* ------------------------------------------------------------------------- */

/* Renders the four films of the reference (Film::RGBA, width x height x 4
 * floats each): beauty RGBA, and the direct, scatter and emission AOVs with
 * alpha 0. Any output pointer may be null. */
lg_status lg_render(lg_ctx* ctx, const lg_camera* camera, float* rgba,
                    float* direct, float* scatter, float* emission);

/* One whole frame: lg_build_graphs + lg_solve_graphs + lg_splat + lg_render. */
lg_status lg_render_frame(lg_ctx* ctx, int n_graphs, const float* points,
                          const int64_t* offsets, const float* radius_sq,
                          int max_connect, double point_voxel_size,
                          const lg_camera* camera, float* rgba, float* direct,
                          float* scatter, float* emission);

/* Device-resident variant of lg_render_frame for timing: points already on the
 * device (loaded by a previous lg_build_graphs), outputs stay in device memory.
 * Enqueues the whole frame on the context stream and returns without waiting. */
lg_status lg_frame_device(lg_ctx* ctx, int max_connect, double point_voxel_size,
                          const lg_camera* camera);

/* Copies the films of the last render (lg_render, lg_frame_device) to host
 * memory, waiting for it; width x height x 4 floats each, any may be null. */
lg_status lg_get_films(lg_ctx* ctx, float* rgba, float* direct, float* scatter,
                       float* emission);

/* Statistics of the last render on this context (waits for it): density
 * samples taken by primary and shadow rays, and primary samples that shaded
 * (each casts the shadow rays of every light sample). Any pointer may be null. */
lg_status lg_render_stats(lg_ctx* ctx, uint64_t* primary_samples,
                          uint64_t* shadow_samples, uint64_t* shading_samples);

/* Stage timing of lg_frame_device, the equivalent of the reference's
 * tbb::tick_count prints (src/main.cc:553,589,125, src/LightGraph.h:268-585):
 * when on, CUDA events are recorded on the context stream around each stage.
 * lg_stage_times waits for the last profiled frame and writes up to n stage
 * durations in ms: build graph, edge march, Floyd-Warshall, vertex light,
 * diffusion, splat, render. */
lg_status lg_set_profiling(lg_ctx* ctx, int on);
lg_status lg_stage_times(lg_ctx* ctx, double* ms, int n);
/* The last render made with profiling on (inside a frame or by lg_render)
 * split into its waves (ms): primary count + scan, primary shading,
 * shadow-ray ordering, shadow rays, resolve. LG_ERR_STATE if there is none. */
lg_status lg_render_wave_times(lg_ctx* ctx, double ms[5]);

/* Frame replay: when on, lg_frame_device runs the frame once, captures the
 * same launch sequence in a CUDA graph and replays it on later calls with the
 * same camera while no scene state or buffer changed. */
lg_status lg_set_graph_mode(lg_ctx* ctx, int on);
/* Kernels in one captured frame (0 before the first capture). */
uint64_t lg_frame_launches(const lg_ctx* ctx);

/* Schedule of the path solve over all loaded graphs. -1 (default): chosen by
 * the autotuner, which times every candidate once per (graph count, largest
 * graph) on a scratch copy and keeps the fastest; 0: two launches per round
 * per graph; 1 or 2: one persistent launch for every graph with 1 or 2 CTAs
 * per SM (a work queue with per-graph dependency counters); 3 or 4: the
 * symmetric persistent solve (for the symmetric matrices the graph stage
 * builds) with 1 or 2 CTAs per SM; 5: schedule 4 with the update tiles'
 * operands staged into shared memory by TMA bulk copies (cp.async.bulk on an
 * mbarrier) instead of through registers. All schedules give the same
 * distances bit for bit. A schedule set here stays in force for later graph
 * builds until -1 is set again. */
lg_status lg_set_fw_schedule(lg_ctx* ctx, int schedule);
/* The schedule in use and the autotuner's timings (ms) of schedules 0..5
 * (0 for a schedule it did not time).
 * Returns LG_ERR_TIMEOUT if a persistent solve reported a stalled queue. */
lg_status lg_fw_schedule(lg_ctx* ctx, int* schedule, double* tuned_ms, int n);
/* The ceiling of the Floyd-Warshall update tiles on this GPU: FP32 ops/s
 * (one add and one min per update, as the roofline counts them) of their
 * inner loop alone, with its operands held in shared memory (no staging, no
 * dependency waits, no stores), 2 CTAs per SM. Enqueued on the context's
 * stream and waited for. sums (optional, 256 floats) receives each thread's
 * sum of its final 8 x 8 tile in the first CTA (every CTA computes the same
 * values), so that the loop's arithmetic (packed adds, 3-input mins over
 * fixed operand patterns) can be checked. */
lg_status lg_fw_inner_loop_rate(lg_ctx* ctx, double* tflops, float* sums);
/* Accuracy check of the primary wave's e^x - 1 (a Taylor series below
 * |x| = 1/16, __expf(x) - 1 above): approx[i] is its value at x[i] and ref[i]
 * the CUDA library's expm1f there, both computed on the device (host
 * buffers, n entries). Enqueued on the context's stream and waited for. */
lg_status lg_expm1_check(lg_ctx* ctx, const float* x, float* approx, float* ref, int32_t n);
/* Host-only check of the persistent schedules' work queue for graphs of the
 * given point counts (no device work). Builds the queue the solve would use
 * (sym != 0: the symmetric solve of schedules 3 to 5, in its structural
 * and its list-scheduled order for 152 and 304 CTAs) and replays it in
 * order with the kernels' dependency waits and version updates. LG_OK when
 * every item's waits are met by earlier items (the launch cannot deadlock)
 * and every block is written exactly once per round; LG_ERR_STATE otherwise.
 * *n_items (optional) receives the queue length. */
lg_status lg_fw_queue_check(int n_graphs, const int32_t* sizes, int sym, int64_t* n_items);
/* Device-side check of the bounded dependency wait the persistent solves use
 * (no counterpart in the reference): one thread waits for a flag that
 * nothing sets, for at most `polls` polls (1 to 2^24), and then raises the
 * error word as a stalled solve does. Returns LG_ERR_TIMEOUT when the wait
 * gave up as designed (the context stays usable), LG_ERR_STATE if it did not.
 * The calls that hand results back (lg_solve_paths, lg_solve_graphs,
 * lg_diffuse, lg_render_frame, ...) return LG_ERR_TIMEOUT the same way when
 * a persistent solve of theirs raised its error word. */
lg_status lg_wait_timeout_check(lg_ctx* ctx, uint32_t polls);

/* ------------------------------------------------------------------------- */
/* Image files without the OpenEXR library                                   */
/* ------------------------------------------------------------------------- */

/* Writes an uncompressed scanline OpenEXR file of n_channels FLOAT channels
 * (names[k], planes[k] = w*h floats, row 0 at the top), as the renderer's
 * saveEXR writes its AOV layers (src/Image.h:47-62). */
lg_status lg_write_exr(const char* path, int w, int h, int n_channels, const char* const* names,
                       const float* const* planes);

/* Reads an environment map the way readExr does through Imf::RgbaInputFile
 * (src/Sampling.h:175-189): the data window's R, G, B, A as half-precision
 * values (missing colours 0, missing alpha 1), row 0 at the top, into
 * rgba (w*h*4 floats; NULL queries the size). Only uncompressed scanline
 * files are readable here (LG_ERR_INVALID otherwise). */
lg_status lg_read_exr_rgba(const char* path, int32_t* width, int32_t* height, float* rgba);

/* ------------------------------------------------------------------------- */
/* Kernel-level entry points (device pointers, caller's stream)              */
/* ------------------------------------------------------------------------- */

/* In-place min-plus Floyd-Warshall of one n x n FP32 matrix with leading
 * dimension ld (floats) in device memory, enqueued on `stream`
 * (a cudaStream_t; NULL = legacy default stream). No allocation.
 * Replaces LightGraph::floydAlgo (src/LightGraph.h:516-528) without the final
 * diagonal reset. */
lg_status lg_fw_device(float* dist, int n, int ld, void* stream);

/* Host-memory convenience wrapper of lg_fw_device (copies in and out). */
lg_status lg_fw_host(lg_ctx* ctx, float* dist, int n);

/* Radiance diffusion that allocates nothing. This entry point has no
 * counterpart in the reference. It exists for callers that cannot call
 * cudaMalloc: processes whose device memory belongs to another allocator or a
 * fixed arena, or plugins that must not change the device's memory footprint.
 * The caller owns every input and output, in device memory:
 *   dist_device    n x n optical depths after the path solve (leading
 *                  dimension ld, diagonal 0, +inf = unreachable)
 *   light_device   n x 3 vertex radiance (lg_vertex_light)
 *   diffuse_device n x 3 result, the same as lg_diffuse's
 *   extinction     the shader's extinction (<= 0 per channel)
 * enqueued on `stream` (a cudaStream_t; NULL = legacy default stream).
 * Scratch space is a fixed __device__ array inside the library sized for
 * n <= LG_NOALLOC_MAX_POINTS (larger n returns LG_ERR_INVALID). Every GPU
 * that loads the library keeps that array (about 1.7 MB) until the process
 * exits. All calls share it, so calls whose work overlaps on the GPU race.
 * The work is asynchronous: a host mutex around the calls does not order it.
 * Order the calls on the device instead: issue them on one stream, or put an
 * event wait or a synchronisation between calls on different streams. The
 * first call on each device looks up the array's device address, so make that
 * first call before any stream capture on the device. */
#define LG_NOALLOC_MAX_POINTS 8192
lg_status lg_diffuse_noalloc(const float* dist_device, int n, int ld,
                             const float* light_device, float* diffuse_device,
                             const double extinction[3], void* stream);

/* ------------------------------------------------------------------------- */
/* Serving (no counterpart in the reference, which renders one frame per run) */
/* ------------------------------------------------------------------------- */

typedef struct lg_server lg_server;

typedef struct lg_server_opts {
    int32_t device;
    int32_t max_inflight;          /* requests on the device at once (slots)    */
    int32_t queue_capacity;        /* waiting requests before LG_ERR_BUSY        */
    int32_t solo_paths;            /* 0: the Floyd-Warshall solves of requests in
                                      flight share persistent launches; 1: each
                                      request solves its own graphs alone       */
    uint64_t hbm_budget_bytes;     /* device bytes admitted at once (0: 64 GiB)  */
} lg_server_opts;

/* A render request against a resident volume: one frame of the three stages
 * with its own graphs, lights, shader, settings (settings.seed keys its random
 * streams) and camera. An environment light (LG_LIGHT_ENV) needs the
 * request's env map (env_rgb, env_h rows x env_w columns x RGB, at least
 * 2 x 2). Arrays are copied at submit time. */
typedef struct lg_request {
    int32_t volume;                /* id from lg_server_add_volume                */
    int32_t n_graphs;
    const float* points;
    const int64_t* offsets;
    const float* radius_sq;
    int32_t max_connect;
    int32_t n_lights;
    const lg_light* lights;
    lg_shader shader;
    lg_settings settings;
    lg_camera camera;
    double point_voxel_size;
    const float* env_rgb;          /* env map of the request's env lights, or NULL */
    int32_t env_w, env_h;
} lg_request;

/* Creates a server with max_inflight slots (one context, stream and worker
 * thread each). Admission is FIFO: the head request is admitted when a slot is
 * free and its lg_request_bytes fit in hbm_budget_bytes next to the requests
 * in flight; admitted requests run concurrently. Unless solo_paths is set,
 * the requests whose edges are marched at about the same time (within a
 * fraction of a millisecond of each other) have their all-pairs path solves
 * batched into one persistent Floyd-Warshall launch; every result is the
 * same, bit for bit, as the request's alone. */
lg_status lg_server_create(const lg_server_opts* opts, lg_server** out);
lg_status lg_server_destroy(lg_server* srv);
/* The description of the last failed server call made by the calling thread
 * (each thread reads its own; valid until that thread's next server call). */
const char* lg_server_last_error(const lg_server* srv);
/* Uploads a volume (density and optional temperature) that stays resident for
 * the server's lifetime; *volume_id names it in requests. */
lg_status lg_server_add_volume(lg_server* srv, const lg_grid_desc* density,
                               const float* density_values,
                               const lg_grid_desc* temperature,
                               const float* temperature_values,
                               int storage_dtype, int32_t* volume_id);
/* Enqueues a request and returns at once; *ticket identifies it.
 * LG_ERR_INVALID: a malformed request (the graph layout lg_build_graphs
 * accepts, known volume, lights and env map), checked before anything is
 * copied; LG_ERR_BUSY: queue full; LG_ERR_NOMEM: larger than the whole
 * budget. */
lg_status lg_server_submit(lg_server* srv, const lg_request* req, int64_t* ticket);
/* Non-blocking: *done = 1 once the request has finished (its result waits
 * for lg_server_wait, which this call does not consume), else 0.
 * LG_ERR_INVALID for an unknown (or already waited-for) ticket. */
lg_status lg_server_poll(lg_server* srv, int64_t ticket, int* done);
/* Waits for a request (timeout_ms < 0: no limit; LG_ERR_TIMEOUT otherwise)
 * and copies its beauty film (width x height x 4 floats) into rgba if
 * non-null. queue_us: submit -> admit, latency_us: submit -> done (host
 * microseconds). A ticket can be waited for once. */
lg_status lg_server_wait(lg_server* srv, int64_t ticket, int timeout_ms,
                         float* rgba, double* queue_us, double* latency_us);
/* Device bytes a request is charged against the HBM budget. */
uint64_t lg_request_bytes(const lg_request* req);
/* Floyd-Warshall launches the server has made for its requests and the
 * graphs they solved (more graphs than launches: requests shared a launch).
 * No counterpart in the reference. */
lg_status lg_server_stats(lg_server* srv, uint64_t* path_launches, uint64_t* path_graphs);

/* ------------------------------------------------------------------------- */
/* Host helpers: the reference's scene description (no device work)          */
/* ------------------------------------------------------------------------- */
/* These, lg_write_exr and lg_read_exr_rgba live in liblightgraph_host.so, a
 * host-only library with no CUDA code (link it beside liblightgraph_gb300.so);
 * every other function of this header is in liblightgraph_gb300.so. */

/* Shader() defaults (src/Shader.h:123-138). */
void lg_shader_default(lg_shader* shader);
/* setAbsorption/setScattering/setVolumeColor (src/Shader.h:165-211): stores
 * scattering and recomputes albedo = color*scattering/(scattering+absorption)
 * and extinction = -(scattering+absorption). */
void lg_shader_set_coefficients(lg_shader* shader, const double absorption[3],
                                const double scattering[3], const double volume_color[3]);
/* SceneSettings() defaults (src/SceneSettings.h:40-61) with seed 0. */
void lg_settings_default(lg_settings* settings);
/* PerspectiveCamera/SceneSettings camera defaults (50 mm, 36 mm aperture,
 * znear 1e-3, zfar FLT_MAX, 960x540, 1 sample). */
void lg_camera_default(lg_camera* camera);
/* parseLight (src/main.cc:234-274): "dir:yRot:r,g,b:intensity:rx,ry,rz" and
 * "env:yRot:r,g,b:intensity:samples:file" (the map itself is passed to
 * lg_set_lights), plus "point:yRot:r,g,b:intensity:x,y,z" for the reference's
 * PointLight, which has no command-line syntax there. */
lg_status lg_parse_light(const char* spec, lg_light* out);
/* parseColorRamp (src/main.cc:280-319): "p0,p1,../r,g,b:r,g,b:../in/out". */
lg_status lg_parse_color_ramp(const char* spec, lg_shader* shader);

#ifdef __cplusplus
}
#endif

#endif /* LIGHTGRAPH_C_H_ */
