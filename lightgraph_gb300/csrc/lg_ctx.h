// Context object behind the opaque lg_ctx handle: one device, one stream,
// the resident grids and the device buffers of each stage (grow-only).
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "lg_kernels.h"
#include "lightgraph_c.h"

namespace lg {

// Bumped whenever any DevBuf is reallocated: a captured frame graph is only
// replayed while its buffers are the ones it was captured with.
extern std::atomic<uint64_t> g_alloc_epoch;

// Grow-only device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    cudaError_t reserve(size_t b) {
        if (b <= bytes) return cudaSuccess;
        release();
        ++g_alloc_epoch;
        const cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = b;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

struct GridStore {
    DevBuf bricks, bits;
    DevGrid g;
    lg_grid_desc desc{};
    bool valid = false;
    int version = 0;
    // bounding box of the non-zero (active) voxels, index coordinates
    // {min x, y, z, max x, y, z}; has_active false when every voxel is 0
    int vbbox[6] = {0, 0, 0, 0, 0, 0};
    bool has_active = false;
};

struct Ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    std::mutex mu;
    std::string err;
    cudaGraphExec_t graph_exec = nullptr;

    // grids: owned (uploaded through this context) or bound to a resident
    // volume shared by several contexts (the serving slots)
    GridStore dens, temp;
    const GridStore* dens_ext = nullptr;
    const GridStore* temp_ext = nullptr;
    bool temp_ext_set = false;
    const GridStore& D() const { return dens_ext ? *dens_ext : dens; }
    const GridStore& T() const { return temp_ext_set ? *temp_ext : temp; }
    DevBuf staging, mask_staging, small;

    // scene
    lg_shader shader{};
    lg_settings settings{};
    std::vector<lg_light> lights;
    DevBuf env_rgb_d, env_cond_func, env_cond_cdf, env_cond_int, env_marg_func, env_marg_cdf, env_marg_int;
    DevBuf env_cond_guide, env_marg_guide;  // guide tables of the CDFs (DevEnv)
    float env_marg_int_h = 0.f;
    int env_w_ = 0, env_h_ = 0;
    bool env_valid = false;

    // graphs
    int n_graphs = 0;
    int64_t n_points = 0;
    int max_n = 0, max_edges = 0, max_connect = 12;
    int64_t s_floats = 0, edge_slots = 0;
    std::vector<GraphInfo> h_graphs;
    std::vector<float> h_pts;
    double point_voxel_size_cache = -1.0;
    bool graphs_built = false, paths_solved = false, light_done = false, diffuse_done = false;
    DevBuf d_pts, d_graphs, d_pt_graph, d_cand, d_cand_cnt, d_edges, d_edge_cnt, d_adj, d_adj_off;
    DevBuf d_S, d_L, d_D, d_part, d_colw, d_fw;

    // batched Floyd-Warshall: work queue, counters and the autotuned schedule
    DevBuf d_fwg, d_fw_items, d_fw_sync, d_fw_tune;
    DevBuf d_fw_items_sym, d_fw_panels;  // symmetric solve: its queue and column-panel slots
    int fw_items_n = 0;
    int fw_items_sym_n = 0;
    int fw_max_nt = 0;
    size_t fw_sync_n = 2;  // uint32 words of d_fw_sync
    bool fw_queue_valid = false;
    // a persistent solve ran since the last look at its error word (d_fw_sync)
    bool fw_flag_pending = false;
    std::vector<int64_t> fw_queue_key;  // (graph count, then offset and padded size per graph)
    bool fw_general_built = false;      // d_fw_items holds the general queue
    bool fw_sym_built = false;          // d_fw_items_sym holds the symmetric queue
    int fw_queue_uses = 0;              // solves since the symmetric queue was built
    bool fw_sym_ordered = false;        // the symmetric queue is in list-scheduled order
    bool fw_order_next = false;         // order it at the next solve (a frame about to be captured)
    std::vector<FwGraph> h_fwg;         // host copies for the deferred ordering
    std::vector<int4> h_fw_items_sym;
    // schedule per (graph count, largest n): 0 = per-graph launches,
    // k > 0 = persistent with k CTAs per SM
    std::vector<std::pair<std::pair<int, int>, int>> fw_tuned;
    int fw_choice = -1;
    int fw_pinned = -1;  // lg_set_fw_schedule's choice, kept across graph builds (-1: autotuned)
    double fw_tune_ms[kFwSchedules] = {};

    // frame replay through a captured CUDA graph
    bool graph_mode = false;
    bool graph_valid = false;
    cudaGraph_t graph = nullptr;
    lg_camera graph_cam{};
    double graph_pvs = 0.0;
    uint64_t graph_epoch = 0;
    uint64_t frame_launch_base = 0, frame_launches = 0;  // kernels in one frame
    void invalidate_graph() { graph_valid = false; }
    lg_status frame_enqueue(double point_voxel_size, const lg_camera* camera);
    lg_status solve_paths_batched(int choice);
    lg_status tune_fw();

    // scatter grid
    CoarseGrid coarse{};
    int topo_version = -1, topo_factor = -1;
    const GridStore* topo_store = nullptr;
    bool splat_done = false;
    double splat_radius = 0.0;
    DevBuf d_act0, d_act, d_sg, d_cell_count, d_cell_start, d_cursor, d_sorted, d_scan_tmp;

    // films and the render waves' buffers
    int film_w = 0, film_h = 0;
    DevBuf d_rgba, d_direct, d_scatter, d_emission, d_counters;
    DevBuf d_ps_count, d_ps_offset, d_ps_scan, d_ps_total, d_ps_data, d_tasks, d_task_direct;
    // shadow-ray ordering: key histogram, its scan, the ordered task indices
    DevBuf d_ray_counts, d_ray_offsets, d_ray_scan, d_ray_total, d_ray_order, d_ray_keys;
    DevBuf d_ray_bounds;  // occupancy bound tables of the lights' bins
    bool capturing = false;  // inside a CUDA graph capture: no host syncs

    // stage timing: events recorded on the stream around each stage of a frame
    static constexpr int kStages = 7;  // build, march, fw, light, diffuse, splat, render
    bool profiling = false;
    cudaEvent_t ev[kStages + 1] = {};
    bool ev_recorded = false;     // a whole profiled frame (stage events)
    bool waves_recorded = false;  // a profiled render (wave events), frame or lg_render
    void mark(int k) {
        if (profiling && ev[k]) cudaEventRecord(ev[k], st);
    }
    // render waves: count + scan, primary, ray ordering, shadow, resolve
    static constexpr int kWaves = 5;
    cudaEvent_t wev[kWaves + 1] = {};
    void wmark(int k, cudaStream_t s) {
        if (profiling && wev[k]) cudaEventRecord(wev[k], s);
    }
    // The render's count pass needs only the grids, the scene and the camera,
    // so a frame runs it (and its scan) on the side stream st2 from the start,
    // beside the graph stages: st2 waits for ev_fork (recorded on st) and
    // render() waits for ev_count (recorded on st2). wev_shade then marks
    // the start of the shading wave on st (wave 1 starts there, not at
    // wev[1]).
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_count = nullptr, wev_shade = nullptr;
    bool count_early = false;  // a count for count_cam was enqueued on st2
    bool wave_split = false;   // the last profiled render used wev_shade
    lg_camera count_cam{};

    lg_status fail(lg_status s, const char* fmt, ...);
    lg_status cuda(cudaError_t e, const char* what);

    lg_status upload_grid(int which, const lg_grid_desc* desc, const float* values, int dtype);
    lg_status set_lights(const lg_light* ls, int n, const float* env_rgb, int env_w, int env_h);
    DevScene scene() const;
    lg_status load_graphs(int n_graphs, const float* points, const int64_t* offsets, const float* radius_sq,
                          int max_connect);
    lg_status build_edges();
    // LightGraph::scatterPoints for n_iter iterations into h_dart_* (host)
    lg_status scatter_points(const lg_scatter_opts& o, int first_iter, int n_iter);
    DevBuf d_dart_pts, d_dart_cnt, d_dart_m2, d_dart_expected;
    std::vector<float> h_dart_pts, h_dart_m2;
    std::vector<int32_t> h_dart_cnt;
    lg_status march_edges();
    lg_status solve_paths();
    lg_status vertex_light();
    lg_status diffuse();
    lg_status solve_all();
    // The path solve split for a caller that batches several contexts'
    // matrices into one launch: fw_solve_on runs this context's queue (its
    // h_graphs' s_off relative to base) on its own stream; solve_rest is
    // what follows the solve (diagonal, vertex light, diffusion).
    lg_status fw_solve_on(float* base, int choice);
    lg_status solve_rest();
    lg_status splat(double point_voxel_size);
    // The count pass and scan of a render of camera c on stream s (films and
    // per-sample buffers sized, counters cleared).
    lg_status render_count(const lg_camera* c, cudaStream_t s);
    // render_count on st2, forked from st, for the render() that follows.
    lg_status render_count_early(const lg_camera* c);
    lg_status render(const lg_camera* c);
    lg_status download_films(float* rgba, float* direct, float* scatter, float* emission);
    lg_status copy_matrix_out(float* out);
    lg_status fw_wait_status();
};

}  // namespace lg
