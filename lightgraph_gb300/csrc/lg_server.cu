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
//   - every kernel is deterministic and every random number is keyed by the
//     request's own seed, so a request's films are the same alone or in the
//     mix.
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
};

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
    std::string err;
    std::unique_ptr<Ctx> upload_ctx;

    void admit_locked();
    void slot_loop(Slot* s);
    void run(Slot* s, Request* q);
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
    // tasks depend on the volume and are not counted)
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

void lg_server::run(Slot* s, Request* q) {
    Ctx& c = *s->ctx;
    const lg_request& r = q->r;
    auto fail = [&](lg_status st) {
        q->status = st;
        q->err = c.err;
    };
    const Volume* v = volumes[r.volume].get();
    c.dens_ext = &v->dens;
    c.temp_ext = &v->temp;
    c.temp_ext_set = true;
    c.shader = r.shader;
    c.settings = r.settings;
    lg_status st = c.set_lights(q->lights.data(), (int)q->lights.size(), q->env.empty() ? nullptr : q->env.data(),
                                r.env_w, r.env_h);
    if (st == LG_OK) st = c.load_graphs(r.n_graphs, q->pts.data(), q->offs.data(), q->r2.data(), r.max_connect);
    // the symmetric persistent solve at 2 CTAs per SM (correct whatever the
    // residency, so the slots' solves may share the SMs; measured 11% more
    // renders/s than 1 CTA per SM on the mixed stream), its queue in
    // structural order (one-off sizes do not pay for the list scheduling)
    if (st == LG_OK) c.fw_choice = 4;
    if (st == LG_OK) st = c.build_edges();
    if (st == LG_OK) st = c.solve_all();
    if (st == LG_OK) st = c.splat(r.point_voxel_size);
    if (st == LG_OK) st = c.render(&r.camera);
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
    for (int k = 0; k <= opts->max_inflight; ++k) {
        lg_ctx* h = nullptr;
        const lg_status st = lg_create(opts->device, &h);
        if (st != LG_OK) return st;
        std::unique_ptr<Ctx> c(reinterpret_cast<Ctx*>(h));
        if (k == 0) {
            srv->upload_ctx = std::move(c);
        } else {
            auto s = std::make_unique<Slot>();
            s->ctx = std::move(c);
            srv->slots.push_back(std::move(s));
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
        // the slot contexts are destroyed through the C ABI (stream, events)
        lg_destroy(reinterpret_cast<lg_ctx*>(s->ctx.release()));
    }
    lg_destroy(reinterpret_cast<lg_ctx*>(srv->upload_ctx.release()));
    delete srv;
    return LG_OK;
}

extern "C" const char* lg_server_last_error(const lg_server* srv) { return srv ? srv->err.c_str() : "null server"; }

extern "C" lg_status lg_server_add_volume(lg_server* srv, const lg_grid_desc* density, const float* density_values,
                                          const lg_grid_desc* temperature, const float* temperature_values,
                                          int storage_dtype, int32_t* volume_id) {
    if (!srv || !density || !density_values) return LG_ERR_INVALID;
    Ctx& c = *srv->upload_ctx;
    std::lock_guard<std::mutex> lk(c.mu);
    cudaSetDevice(c.device);
    auto v = std::make_unique<Volume>();
    lg_status st = c.upload_grid(LG_GRID_DENSITY, density, density_values, storage_dtype);
    if (st != LG_OK) { srv->err = c.err; return st; }
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
        if (st != LG_OK) { srv->err = c.err; return st; }
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
    if (req->n_graphs < 1 || !req->offsets || !req->radius_sq || req->n_lights < 0 ||
        req->n_lights > LG_MAX_LIGHTS || (req->n_lights > 0 && !req->lights))
        return LG_ERR_INVALID;
    for (int k = 0; k < req->n_lights; ++k)
        if (req->lights[k].type == LG_LIGHT_ENV && (!req->env_rgb || req->env_w < 2 || req->env_h < 2)) {
            srv->err = "an environment light needs the request's env map (at least 2 x 2)";
            return LG_ERR_INVALID;
        }
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
        srv->err = "unknown volume";
        return LG_ERR_INVALID;
    }
    if ((int)srv->queue.size() >= srv->opts.queue_capacity) {
        srv->err = "queue full";
        return LG_ERR_BUSY;
    }
    if (q->bytes > srv->opts.hbm_budget_bytes) {
        srv->err = "request exceeds the HBM budget";
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
        srv->err = "unknown ticket";
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
        srv->err = "unknown ticket";
        return LG_ERR_INVALID;
    }
    Request* q = it->second.get();
    auto ready = [&] { return q->done; };
    if (timeout_ms < 0) srv->cv.wait(lk, ready);
    else if (!srv->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return LG_ERR_TIMEOUT;
    const lg_status st = q->status;
    if (st != LG_OK) srv->err = q->err;
    if (st == LG_OK && rgba) std::memcpy(rgba, q->rgba.data(), sizeof(float) * q->rgba.size());
    if (queue_us) *queue_us = q->t_admit - q->t_submit;
    if (latency_us) *latency_us = q->t_done - q->t_submit;
    srv->requests.erase(it);
    return st;
}
