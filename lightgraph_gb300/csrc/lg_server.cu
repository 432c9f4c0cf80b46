// Serving: a request loop over resident volumes with continuous batching.
//
// The reference renders one frame per process run (src/main.cc:343-611). A
// server keeps several volumes resident in HBM and renders requests of
// different volume, graph and image sizes as they arrive:
//   - admission is FIFO and bounded by an HBM budget: a request is admitted
//     when a slot is free and its estimated device bytes fit next to the
//     requests in flight (the head waits; nothing behind it overtakes it);
//   - each slot is a context with its own stream and worker thread, bound to
//     the volume's resident grids, so the kernels of admitted requests
//     overlap on the device; a slot is taken again as soon as it finishes;
//   - the all-pairs path solves of requests in flight are batched: a slot
//     that has marched its edges hands its matrices to a path batcher, and
//     the slots that arrive within a fraction of a millisecond of each other
//     share one persistent Floyd-Warshall launch over all their graphs (the
//     batched solve's queue interleaves the graphs round by round; each
//     matrix stays in its slot's buffers and the launch addresses them from
//     the lowest of them). CUDA events order the launch after every member's
//     edge march and each member's later kernels after the launch;
//   - every kernel is deterministic and every random number is keyed by the
//     request's own seed, so a request's films are the same alone or in the
//     mix, batched or not.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lg_ctx.h"

using namespace lg;

namespace {

double now_us() {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Volume {
    GridStore dens, temp;
    bool has_temp = false;
    Ctx* owner = nullptr;  // context that uploaded the grids
};

// Every device buffer a DevGrid points into (cell records, leaf bitmap)
// passes from the upload context to the volume, whose copy of the DevGrid
// keeps pointing at them.
void take_buffers(GridStore& to, GridStore& from) {
    DevBuf* const pairs[2][2] = {{&to.bricks, &from.bricks}, {&to.bits, &from.bits}};
    for (auto& pr : pairs) {
        std::swap(pr[0]->p, pr[1]->p);
        std::swap(pr[0]->bytes, pr[1]->bytes);
    }
}

struct Request {
    int64_t ticket = 0;
    lg_request r{};
    std::vector<float> pts;
    std::vector<int64_t> offs;
    std::vector<float> r2;
    std::vector<lg_light> lights;
    std::vector<float> env;  // env map (h x w x 3) of the request's env lights
    uint64_t bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    bool done = false;
    lg_status status = LG_OK;
    std::string err;
    std::vector<float> rgba;  // result (beauty film)
};

struct Slot {
    std::unique_ptr<Ctx> ctx;
    std::thread th;
    Request* cur = nullptr;
    float* pinned = nullptr;
    size_t pinned_bytes = 0;
    cudaEvent_t marched = nullptr;  // the slot's edge march is done
    cudaEvent_t solved = nullptr;   // the batched path solve holding its graphs is done
};

// One slot's matrices waiting for, or in, a batched path solve.
struct PathJob {
    Slot* slot = nullptr;
    lg_status status = LG_OK;
    std::string err;
    bool finished = false;
};

// Batches the path solves of the slots in flight (see the file comment).
struct PathBatcher {
    std::mutex mu;
    std::condition_variable cv;
    std::vector<PathJob*> pending;
    bool leading = false;     // a slot thread is forming or running a batch
    int marching = 0;         // slots admitted that have not handed over their matrices yet
    std::unique_ptr<Ctx> ctx; // the batch's queue buffers and stream
    uint64_t launches = 0, graphs = 0;
};

// How long a batch waits for slots still marching their edges.
constexpr double kPathWaitUs = 300.0;

// The description of the last failed server call made by this thread (the
// server's calls come from many threads: each reads its own).
thread_local std::string t_server_err;

}  // namespace

struct lg_server {
    lg_server_opts opts{};
    std::vector<std::unique_ptr<Volume>> volumes;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> queue;
    std::map<int64_t, std::unique_ptr<Request>> requests;
    uint64_t inflight_bytes = 0;
    int64_t next_ticket = 1;
    bool stop = false;
    std::unique_ptr<Ctx> upload_ctx;
    PathBatcher paths;

    void admit_locked();
    void slot_loop(Slot* s);
    void run(Slot* s, Request* q);
    lg_status solve_paths_shared(Slot* s);
    void run_path_batch(std::vector<PathJob*>& batch);
};

extern "C" uint64_t lg_request_bytes(const lg_request* q) {
    if (!q || q->n_graphs < 1 || !q->offsets) return 0;
    uint64_t b = 0, P = (uint64_t)q->offsets[q->n_graphs];
    for (int g = 0; g < q->n_graphs; ++g) {
        const uint64_t n = (uint64_t)(q->offsets[g + 1] - q->offsets[g]);
        const uint64_t ld = (std::max<uint64_t>(n, 1) + 127) / 128 * 128;
        b += ld * ld * 4;                              // S / distances
        b += n * (uint64_t)q->max_connect / 2 * 8;     // edges
    }
    b += P * (12 + 96 * 2 + 4 + 4);                    // points, candidates, graph ids
    b += P * 4 * (3 + 3 + 3 + 3 * kRowChunks);         // L, D, weights, partial sums
    b += (uint64_t)q->camera.width * q->camera.height * 64;  // four films
    // per pixel sample: shading count, offset and primary results (the shadow
    // tasks, their order keys and per-light results depend on the volume and
    // are not counted)
    b += (uint64_t)q->camera.width * q->camera.height * (uint64_t)std::max(q->camera.samples, 1) * 44;
    b += 160ull * 160 * 160 * 12;                      // point bins (upper bound)
    if (q->env_rgb && q->env_w > 1 && q->env_h > 1)  // env map and its CDFs
        b += (uint64_t)q->env_w * q->env_h * 4 * 5 + (uint64_t)q->env_h * 4 * 262;
    return b;
}

void lg_server::admit_locked() {
    while (!queue.empty()) {
        Request* q = queue.front();
        Slot* free_slot = nullptr;
        for (auto& s : slots)
            if (!s->cur) { free_slot = s.get(); break; }
        if (!free_slot) return;
        if (inflight_bytes > 0 && inflight_bytes + q->bytes > opts.hbm_budget_bytes) return;
        queue.pop_front();
        inflight_bytes += q->bytes;
        q->t_admit = now_us();
        free_slot->cur = q;
        cv.notify_all();
    }
}

// One persistent launch over the graphs of every job of the batch, on the
// batcher's stream: it waits for each member's edge march and each member's
// stream waits for it.
void lg_server::run_path_batch(std::vector<PathJob*>& batch) {
    Ctx& b = *paths.ctx;
    lg_status st = LG_OK;
    // the lowest of the members' matrix buffers; each member's offset from
    // it in floats (cudaMalloc aligns every buffer to 256 bytes)
    uintptr_t lowest = UINTPTR_MAX;
    for (PathJob* j : batch) lowest = std::min(lowest, reinterpret_cast<uintptr_t>(j->slot->ctx->d_S.p));
    float* base = reinterpret_cast<float*>(lowest);
    b.h_graphs.clear();
    b.max_n = 0;
    for (PathJob* j : batch) {
        const Ctx& c = *j->slot->ctx;
        const int64_t shift = (int64_t)((reinterpret_cast<uintptr_t>(c.d_S.p) - lowest) / sizeof(float));
        for (GraphInfo g : c.h_graphs) {
            g.s_off += shift;
            b.h_graphs.push_back(g);
            b.max_n = std::max(b.max_n, g.n);
        }
        if (cudaStreamWaitEvent(b.st, j->slot->marched, 0) != cudaSuccess) st = b.fail(LG_ERR_CUDA, "path batch wait");
    }
    b.n_graphs = (int)b.h_graphs.size();
    if (st == LG_OK) st = b.fw_solve_on(base, 4);
    for (PathJob* j : batch) {
        if (st == LG_OK && cudaEventRecord(j->slot->solved, b.st) != cudaSuccess)
            st = b.fail(LG_ERR_CUDA, "path batch record");
    }
    for (PathJob* j : batch) {
        j->status = st;
        if (st != LG_OK) j->err = b.err;
    }
    paths.launches += 1;
    paths.graphs += (uint64_t)b.n_graphs;
}

// Hands the slot's marched matrices to the batcher and returns once a batched
// launch holding them is enqueued (the slot's stream then waits for it). The
// first slot to find no batch forming leads the next one: it waits up to
// kPathWaitUs for the slots still marching, takes every job waiting and runs
// the launch; later arrivals wait for the next leader.
lg_status lg_server::solve_paths_shared(Slot* s) {
    Ctx& c = *s->ctx;
    PathJob job;
    job.slot = s;
    if (cudaEventRecord(s->marched, c.st) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(paths.mu);
        --paths.marching;
        paths.cv.notify_all();
        return c.fail(LG_ERR_CUDA, "edge march event");
    }
    std::unique_lock<std::mutex> lk(paths.mu);
    --paths.marching;
    paths.pending.push_back(&job);
    paths.cv.notify_all();
    while (!job.finished) {
        if (!paths.leading) {
            paths.leading = true;
            const double t0 = now_us();
            while (paths.marching > 0 && now_us() - t0 < kPathWaitUs)
                paths.cv.wait_for(lk, std::chrono::microseconds(50));
            std::vector<PathJob*> batch;
            batch.swap(paths.pending);
            lk.unlock();
            run_path_batch(batch);
            lk.lock();
            for (PathJob* j : batch) j->finished = true;
            paths.leading = false;
            paths.cv.notify_all();
            continue;
        }
        paths.cv.wait(lk);
    }
    lk.unlock();
    if (job.status != LG_OK) return c.fail(job.status, "%s", job.err.c_str());
    if (cudaStreamWaitEvent(c.st, s->solved, 0) != cudaSuccess) return c.fail(LG_ERR_CUDA, "path solve wait");
    return LG_OK;
}

void lg_server::run(Slot* s, Request* q) {
    Ctx& c = *s->ctx;
    const lg_request& r = q->r;
    auto fail = [&](lg_status st) {
        q->status = st;
        q->err = c.err;
    };
    if (!opts.solo_paths) {
        // counted until the slot hands its matrices to the path batcher, so
        // a forming batch can wait for it
        std::lock_guard<std::mutex> lk(paths.mu);
        ++paths.marching;
    }
    const Volume* v = volumes[r.volume].get();
    c.dens_ext = &v->dens;
    c.temp_ext = &v->temp;
    c.temp_ext_set = true;
    c.shader = r.shader;
    c.settings = r.settings;
    lg_status st = c.set_lights(q->lights.data(), (int)q->lights.size(), q->env.empty() ? nullptr : q->env.data(),
                                r.env_w, r.env_h);
    if (st == LG_OK) st = c.load_graphs(r.n_graphs, q->pts.data(), q->offs.data(), q->r2.data(), r.max_connect);
    // the render's count pass runs beside the graph stages (the slot's side
    // stream)
    if (st == LG_OK) st = c.render_count_early(&r.camera);
    // the symmetric persistent solve at 2 CTAs per SM (correct whatever the
    // residency, so the slots' solves may share the SMs; measured 11% more
    // renders/s than 1 CTA per SM on the mixed stream), its queue in
    // structural order (one-off sizes do not pay for the list scheduling)
    if (st == LG_OK) c.fw_choice = 4;
    if (st == LG_OK) st = c.build_edges();
    if (opts.solo_paths) {
        if (st == LG_OK) st = c.solve_all();
    } else {
        if (st == LG_OK) st = c.march_edges();
        if (st == LG_OK) {
            st = solve_paths_shared(s);  // leaves the marching count
        } else {
            std::lock_guard<std::mutex> lk(paths.mu);
            --paths.marching;
            paths.cv.notify_all();
        }
        if (st == LG_OK) st = c.solve_rest();
    }
    if (st == LG_OK) st = c.splat(r.point_voxel_size);
    if (st == LG_OK) st = c.render(&r.camera);
    if (st != LG_OK && c.count_early) {
        // a stage failed before render(): join the side stream again
        cudaStreamWaitEvent(c.st, c.ev_count, 0);
        c.count_early = false;
    }
    if (st == LG_OK) {
        const size_t bytes = sizeof(float) * 4 * (size_t)r.camera.width * r.camera.height;
        if (s->pinned_bytes < bytes) {
            if (s->pinned) cudaFreeHost(s->pinned);
            s->pinned = nullptr;
            s->pinned_bytes = 0;
            if (cudaMallocHost(&s->pinned, bytes) == cudaSuccess) s->pinned_bytes = bytes;
        }
        if (!s->pinned) {
            st = c.fail(LG_ERR_NOMEM, "pinned result buffer");
        } else {
            cudaError_t e = cudaMemcpyAsync(s->pinned, c.d_rgba.p, bytes, cudaMemcpyDeviceToHost, c.st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c.st);
            if (e != cudaSuccess) st = c.cuda(e, "result download");
            else q->rgba.assign(s->pinned, s->pinned + bytes / sizeof(float));
        }
    }
    if (st != LG_OK) fail(st);
}

void lg_server::slot_loop(Slot* s) {
    cudaSetDevice(opts.device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv.wait(lk, [&] { return stop || s->cur != nullptr; });
        if (stop) return;
        Request* q = s->cur;
        lk.unlock();
        run(s, q);
        lk.lock();
        q->t_done = now_us();
        q->done = true;
        inflight_bytes -= q->bytes;
        s->cur = nullptr;
        admit_locked();
        cv.notify_all();
    }
}

extern "C" lg_status lg_server_create(const lg_server_opts* opts, lg_server** out) {
    if (!opts || !out) return LG_ERR_INVALID;
    *out = nullptr;
    if (opts->max_inflight < 1 || opts->max_inflight > 64 || opts->queue_capacity < 1) return LG_ERR_INVALID;
    auto srv = std::make_unique<lg_server>();
    srv->opts = *opts;
    if (srv->opts.hbm_budget_bytes == 0) srv->opts.hbm_budget_bytes = 64ull << 30;
    for (int k = 0; k <= opts->max_inflight + 1; ++k) {
        lg_ctx* h = nullptr;
        const lg_status st = lg_create(opts->device, &h);
        if (st != LG_OK) {
            // what was made so far goes the way lg_server_destroy takes it
            // (no worker thread has started yet)
            lg_server_destroy(srv.release());
            return st;
        }
        std::unique_ptr<Ctx> c(reinterpret_cast<Ctx*>(h));
        if (k == 0) {
            srv->upload_ctx = std::move(c);
        } else if (k == 1) {
            srv->paths.ctx = std::move(c);
        } else {
            srv->slots.push_back(std::make_unique<Slot>());
            Slot& s = *srv->slots.back();
            s.ctx = std::move(c);
            cudaSetDevice(opts->device);
            if (cudaEventCreateWithFlags(&s.marched, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&s.solved, cudaEventDisableTiming) != cudaSuccess) {
                lg_server_destroy(srv.release());
                return LG_ERR_CUDA;
            }
        }
    }
    lg_server* p = srv.release();
    for (auto& s : p->slots) {
        Slot* sp = s.get();
        sp->th = std::thread([p, sp] { p->slot_loop(sp); });
    }
    *out = p;
    return LG_OK;
}

extern "C" lg_status lg_server_destroy(lg_server* srv) {
    if (!srv) return LG_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
        srv->cv.notify_all();
    }
    for (auto& s : srv->slots) {
        if (s->th.joinable()) s->th.join();
        if (s->pinned) cudaFreeHost(s->pinned);
        if (s->marched) cudaEventDestroy(s->marched);
        if (s->solved) cudaEventDestroy(s->solved);
        // the slot contexts are destroyed through the C ABI (stream, events)
        lg_destroy(reinterpret_cast<lg_ctx*>(s->ctx.release()));
    }
    if (srv->paths.ctx) lg_destroy(reinterpret_cast<lg_ctx*>(srv->paths.ctx.release()));
    if (srv->upload_ctx) lg_destroy(reinterpret_cast<lg_ctx*>(srv->upload_ctx.release()));
    delete srv;
    return LG_OK;
}

extern "C" lg_status lg_server_stats(lg_server* srv, uint64_t* path_launches, uint64_t* path_graphs) {
    if (!srv) return LG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(srv->paths.mu);
    if (path_launches) *path_launches = srv->paths.launches;
    if (path_graphs) *path_graphs = srv->paths.graphs;
    return LG_OK;
}

extern "C" const char* lg_server_last_error(const lg_server* srv) { return srv ? t_server_err.c_str() : "null server"; }

extern "C" lg_status lg_server_add_volume(lg_server* srv, const lg_grid_desc* density, const float* density_values,
                                          const lg_grid_desc* temperature, const float* temperature_values,
                                          int storage_dtype, int32_t* volume_id) {
    if (!srv || !density || !density_values) return LG_ERR_INVALID;
    Ctx& c = *srv->upload_ctx;
    std::lock_guard<std::mutex> lk(c.mu);
    cudaSetDevice(c.device);
    auto v = std::make_unique<Volume>();
    lg_status st = c.upload_grid(LG_GRID_DENSITY, density, density_values, storage_dtype);
    if (st != LG_OK) { t_server_err = c.err; return st; }
    // move the uploaded stores into the volume (the buffers change owner)
    take_buffers(v->dens, c.dens);
    v->dens.g = c.dens.g;
    v->dens.desc = c.dens.desc;
    std::copy(c.dens.vbbox, c.dens.vbbox + 6, v->dens.vbbox);
    v->dens.has_active = c.dens.has_active;
    v->dens.valid = true;
    v->dens.version = 1;
    c.dens.valid = false;
    if (temperature && temperature_values) {
        st = c.upload_grid(LG_GRID_TEMPERATURE, temperature, temperature_values, storage_dtype);
        if (st != LG_OK) { t_server_err = c.err; return st; }
        take_buffers(v->temp, c.temp);
        v->temp.g = c.temp.g;
        v->temp.desc = c.temp.desc;
        v->temp.valid = true;
        v->temp.version = 1;
        c.temp.valid = false;
        v->has_temp = true;
    }
    std::lock_guard<std::mutex> lk2(srv->mu);
    srv->volumes.push_back(std::move(v));
    if (volume_id) *volume_id = (int32_t)srv->volumes.size() - 1;
    return LG_OK;
}

extern "C" lg_status lg_server_submit(lg_server* srv, const lg_request* req, int64_t* ticket) {
    if (!srv || !req) return LG_ERR_INVALID;
    if (req->n_graphs < 1 || req->n_graphs > 65535 || !req->offsets || !req->radius_sq || req->n_lights < 0 ||
        req->n_lights > LG_MAX_LIGHTS || (req->n_lights > 0 && !req->lights))
        return LG_ERR_INVALID;
    // the point layout is checked here, before the request's arrays are
    // copied (the same rules as lg_build_graphs)
    auto refuse = [&](const char* why) {
        t_server_err = why;
        return LG_ERR_INVALID;
    };
    if (req->offsets[0] != 0) return refuse("offsets[0] must be 0");
    if (req->max_connect < 0 || req->max_connect > 255) return refuse("max_connect must be in [0, 255]");
    for (int g = 0; g < req->n_graphs; ++g) {
        const int64_t n = req->offsets[g + 1] - req->offsets[g];
        if (n < 0 || n > 65535) return refuse("every graph needs 0..65535 points");
    }
    if (req->offsets[req->n_graphs] > 0 && !req->points) return refuse("null points");
    for (int k = 0; k < req->n_lights; ++k)
        if (req->lights[k].type == LG_LIGHT_ENV && (!req->env_rgb || req->env_w < 2 || req->env_h < 2))
            return refuse("an environment light needs the request's env map (at least 2 x 2)");
    auto q = std::make_unique<Request>();
    q->r = *req;
    const int64_t P = req->offsets[req->n_graphs];
    q->pts.assign(req->points, req->points + 3 * P);
    q->offs.assign(req->offsets, req->offsets + req->n_graphs + 1);
    q->r2.assign(req->radius_sq, req->radius_sq + req->n_graphs);
    q->lights.assign(req->lights, req->lights + req->n_lights);
    if (req->env_rgb && req->env_w > 1 && req->env_h > 1)
        q->env.assign(req->env_rgb, req->env_rgb + (size_t)3 * req->env_w * req->env_h);
    q->r.env_rgb = nullptr;
    q->r.points = nullptr;
    q->r.offsets = nullptr;
    q->r.radius_sq = nullptr;
    q->r.lights = nullptr;
    q->bytes = lg_request_bytes(req);
    std::lock_guard<std::mutex> lk(srv->mu);
    if (req->volume < 0 || req->volume >= (int)srv->volumes.size()) {
        t_server_err = "unknown volume";
        return LG_ERR_INVALID;
    }
    if ((int)srv->queue.size() >= srv->opts.queue_capacity) {
        t_server_err = "queue full";
        return LG_ERR_BUSY;
    }
    if (q->bytes > srv->opts.hbm_budget_bytes) {
        t_server_err = "request exceeds the HBM budget";
        return LG_ERR_NOMEM;
    }
    q->ticket = srv->next_ticket++;
    q->t_submit = now_us();
    Request* raw = q.get();
    srv->requests[q->ticket] = std::move(q);
    srv->queue.push_back(raw);
    srv->admit_locked();
    if (ticket) *ticket = raw->ticket;
    return LG_OK;
}

extern "C" lg_status lg_server_poll(lg_server* srv, int64_t ticket, int* done) {
    if (!srv || !done) return LG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->requests.find(ticket);
    if (it == srv->requests.end()) {
        t_server_err = "unknown ticket";
        return LG_ERR_INVALID;
    }
    *done = it->second->done ? 1 : 0;
    return LG_OK;
}

extern "C" lg_status lg_server_wait(lg_server* srv, int64_t ticket, int timeout_ms, float* rgba, double* queue_us,
                                    double* latency_us) {
    if (!srv) return LG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->requests.find(ticket);
    if (it == srv->requests.end()) {
        t_server_err = "unknown ticket";
        return LG_ERR_INVALID;
    }
    Request* q = it->second.get();
    auto ready = [&] { return q->done; };
    if (timeout_ms < 0) srv->cv.wait(lk, ready);
    else if (!srv->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return LG_ERR_TIMEOUT;
    const lg_status st = q->status;
    if (st != LG_OK) t_server_err = q->err;
    if (st == LG_OK && rgba) std::memcpy(rgba, q->rgba.data(), sizeof(float) * q->rgba.size());
    if (queue_us) *queue_us = q->t_admit - q->t_submit;
    if (latency_us) *latency_us = q->t_done - q->t_submit;
    srv->requests.erase(it);
    return st;
}
