// Native serving loop: continuous batching of extraction requests on one GPU.
//
// A request is a cubic grid (n points per axis over [-1, 1]^3) given as a union
// of spheres and boxes, and an extraction (marching cubes or dual contouring).
// The server keeps `slots` worker threads, each with its own CUDA stream and,
// per (kind, n, method, level), device buffers and a CUDA graph of
// iso_sdf_union_grid + iso_mc_dense / iso_dc_dense captured once.  Requests are
// admitted first come, first served when a worker is free and the running
// requests' worst-case bytes plus the new one's fit the budget; requests on
// different slots overlap on the GPU.  A request per call costs one 904-byte
// H2D copy, one graph launch, a 64-byte D2H of the sizes and the mesh's D2H
// through the slot's pinned staging buffer.  A mesh larger than the slot's
// buffers reruns with exact capacities.  No counterpart in isoext.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "isoext_gb300.h"

namespace iso {
void set_last_error(const char* msg);
}

namespace {

constexpr int MAX_PRIMS = 32;
constexpr int PRIM_FLOATS = 1 + 7 * MAX_PRIMS;
constexpr float DC_REG = 1e-2f, DC_SVD_TOL = 1e-6f;  // dual_contouring's defaults (isoext)
const float LO[3] = {-1.0f, -1.0f, -1.0f}, HI[3] = {1.0f, 1.0f, 1.0f};

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Caps {
    long long v, f;
};

// Faces of a closed surface inside the box stay below twice the grid's face
// area in cells; the output check catches the rest.
Caps caps_for(int n) {
    const long long f = 4ll * 6 * (n - 1) * (n - 1) + 4096;
    return {f / 2 + 4096, f};
}

size_t ws_bytes(int kind, int n, Caps c) {
    return kind == 0 ? iso_mc_dense_workspace_size(n, n, n, c.v, c.f) : iso_dc_dense_workspace_size(n, n, n, c.v, c.f);
}

size_t request_bytes(int kind, int n) {
    const Caps c = caps_for(n);
    return size_t(4) * n * n * n + ws_bytes(kind, n, c) + size_t(12) * (c.v + c.f) + 4096;
}

struct Job {
    long long ticket;
    IsoServeRequest req;
    float prims[PRIM_FLOATS];
    double t_submit;
    size_t need;
};

struct Done {
    IsoServeResult r;
};

// One slot's buffers for one (kind, n, method, level), and its graph.
struct GraphBuf {
    int kind = 0, n = 0, method = 0;
    float level = 0.0f;
    Caps cap{0, 0};
    float* values = nullptr;
    float* vout = nullptr;
    int* fout = nullptr;
    void* ws = nullptr;
    size_t wsb = 0;
    long long* small = nullptr;  // counts, status (MC at [2], DC at [6])
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct Slot {
    cudaStream_t stream = nullptr;
    float* prims_dev = nullptr;
    float* prims_host = nullptr;    // pinned
    long long* small_host = nullptr;  // pinned [8]
    uint8_t* out_host = nullptr;    // pinned staging of the largest mesh
    size_t out_bytes = 0;
    std::vector<GraphBuf*> bufs;
};

int queue_extraction(const GraphBuf& b, const float* prims_dev, float* values, float* vout, long long capv, int* fout,
                     long long capf, void* ws, size_t wsb, long long* small, cudaStream_t st) {
    if (cudaMemsetAsync(small, 0, 64, st) != cudaSuccess) return ISO_ERR_CUDA;
    int rc = iso_sdf_union_grid(prims_dev, b.n, b.n, b.n, LO, HI, values, st);
    if (rc) return rc;
    if (b.kind == 0)
        return iso_mc_dense(values, b.n, b.n, b.n, LO, HI, b.level, b.method, vout, capv, fout, capf, ws, wsb, small,
                            reinterpret_cast<int*>(small + 2), st);
    return iso_dc_dense(values, b.n, b.n, b.n, LO, HI, b.level, DC_REG, DC_SVD_TOL, vout, capv, fout, capf, ws, wsb,
                        small, reinterpret_cast<int*>(small + 6), st);
}

}  // namespace

struct IsoServer {
    int device = 0;
    long long budget = 0;
    std::vector<Slot> slots;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::mutex build_mu;  // graph captures, one at a time
    std::deque<Job*> queue;
    std::map<long long, Done> done;
    long long next_ticket = 0;
    long long reserved = 0, max_reserved = 0;
    int running = 0, max_running = 0;
    long long completed = 0;
    bool closing = false;
    double cap_scale = 1.0;  // capacities of buffers built from now on (tests shrink them)

    GraphBuf* buffers(Slot& s, int kind, int n, int method, float level, int* err);
    void worker(int index);
    void run(Slot& s, Job& job, IsoServeResult& r);
};

namespace {

void free_buf(GraphBuf* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->values);
    cudaFree(b->vout);
    cudaFree(b->fout);
    cudaFree(b->ws);
    cudaFree(b->small);
    delete b;
}

}  // namespace

// The slot's buffers and graph for a key, built on first use (under build_mu:
// captures are one at a time; each worker captures on its own stream).
GraphBuf* IsoServer::buffers(Slot& s, int kind, int n, int method, float level, int* err) {
    if (kind != 0) method = 0;  // dual contouring has no method
    for (GraphBuf* b : s.bufs)
        if (b->kind == kind && b->n == n && b->method == method && b->level == level) return b;
    std::lock_guard<std::mutex> lk(build_mu);
    auto* b = new GraphBuf;
    b->kind = kind;
    b->n = n;
    b->method = method;
    b->level = level;
    b->cap = caps_for(n);
    b->cap.v = std::max<long long>(1, (long long)(b->cap.v * cap_scale));
    b->cap.f = std::max<long long>(1, (long long)(b->cap.f * cap_scale));
    b->wsb = ws_bytes(kind, n, b->cap);
    bool ok = cudaMalloc(&b->values, size_t(4) * n * n * n) == cudaSuccess &&
              cudaMalloc(&b->vout, size_t(12) * b->cap.v) == cudaSuccess &&
              cudaMalloc(&b->fout, size_t(12) * b->cap.f) == cudaSuccess &&
              cudaMalloc(&b->ws, std::max<size_t>(b->wsb, 256)) == cudaSuccess &&
              cudaMalloc(&b->small, 64) == cudaSuccess;
    // once outside a graph (first-use set-up of the kernels), then the capture
    ok = ok && queue_extraction(*b, s.prims_dev, b->values, b->vout, b->cap.v, b->fout, b->cap.f, b->ws, b->wsb,
                                b->small, s.stream) == 0;
    ok = ok && cudaStreamSynchronize(s.stream) == cudaSuccess;
    ok = ok && cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        const int rc = queue_extraction(*b, s.prims_dev, b->values, b->vout, b->cap.v, b->fout, b->cap.f, b->ws,
                                        b->wsb, b->small, s.stream);
        const bool ended = cudaStreamEndCapture(s.stream, &b->graph) == cudaSuccess;
        ok = rc == 0 && ended && cudaGraphInstantiate(&b->exec, b->graph, 0) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        free_buf(b);
        *err = ISO_ERR_CUDA;
        return nullptr;
    }
    s.bufs.push_back(b);
    return b;
}

void IsoServer::run(Slot& s, Job& job, IsoServeResult& r) {
    const IsoServeRequest& q = job.req;
    int err = 0;
    GraphBuf* b = buffers(s, q.kind, q.n, q.method, q.level, &err);
    if (!b) {
        r.status = err;
        return;
    }
    std::memcpy(s.prims_host, job.prims, sizeof(job.prims));
    cudaStream_t st = s.stream;
    bool ok = cudaMemcpyAsync(s.prims_dev, s.prims_host, sizeof(job.prims), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaGraphLaunch(b->exec, st) == cudaSuccess &&
              cudaMemcpyAsync(s.small_host, b->small, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        r.status = ISO_ERR_CUDA;
        return;
    }
    long long V = s.small_host[0], F = s.small_host[1];
    int status = int(s.small_host[b->kind == 0 ? 2 : 6] & 0xffffffffll);
    const float* vsrc = b->vout;
    const int* fsrc = b->fout;
    float* tv = nullptr;
    int* tf = nullptr;
    void* tws = nullptr;
    long long* tsmall = nullptr;
    float* tvals = nullptr;
    if (status == ISO_ERR_OVERFLOW) {
        // larger than the slot's buffers: once more with exact capacities
        const Caps c = b->kind == 0 ? Caps{V + 1024, F + 1024}
                                    : Caps{s.small_host[2] + 1024, 2 * s.small_host[4] + 1024};
        const size_t wsb = ws_bytes(b->kind, b->n, c);
        ok = cudaMalloc(&tv, size_t(12) * c.v) == cudaSuccess && cudaMalloc(&tf, size_t(12) * c.f) == cudaSuccess &&
             cudaMalloc(&tws, std::max<size_t>(wsb, 256)) == cudaSuccess && cudaMalloc(&tsmall, 64) == cudaSuccess &&
             cudaMalloc(&tvals, size_t(4) * b->n * b->n * b->n) == cudaSuccess;
        ok = ok && queue_extraction(*b, s.prims_dev, tvals, tv, c.v, tf, c.f, tws, wsb, tsmall, st) == 0 &&
             cudaMemcpyAsync(s.small_host, tsmall, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
        if (ok) {
            V = s.small_host[0];
            F = s.small_host[1];
            status = int(s.small_host[b->kind == 0 ? 2 : 6] & 0xffffffffll);
            vsrc = tv;
            fsrc = tf;
        } else {
            status = ISO_ERR_CUDA;
        }
    }
    if (status == 0 && V > 0 && F > 0) {
        r.vertices = static_cast<float*>(std::malloc(size_t(12) * V));
        r.faces = static_cast<int*>(std::malloc(size_t(12) * F));
        const size_t vb = size_t(12) * V, fb = size_t(12) * F;
        if (!r.vertices || !r.faces) {
            status = ISO_ERR_ARG;
        } else if (vb + fb <= s.out_bytes) {
            ok = cudaMemcpyAsync(s.out_host, vsrc, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaMemcpyAsync(s.out_host + vb, fsrc, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaStreamSynchronize(st) == cudaSuccess;
            if (ok) {
                std::memcpy(r.vertices, s.out_host, vb);
                std::memcpy(r.faces, s.out_host + vb, fb);
            }
        } else {
            ok = cudaMemcpyAsync(r.vertices, vsrc, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaMemcpyAsync(r.faces, fsrc, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaStreamSynchronize(st) == cudaSuccess;
        }
        if (!ok) status = ISO_ERR_CUDA;
        r.num_vertices = V;
        r.num_faces = F;
    }
    if (tv) cudaFree(tv);
    if (tf) cudaFree(tf);
    if (tws) cudaFree(tws);
    if (tsmall) cudaFree(tsmall);
    if (tvals) cudaFree(tvals);
    r.status = status;
}

void IsoServer::worker(int index) {
    cudaSetDevice(device);
    Slot& s = slots[index];
    while (true) {
        Job* job = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] {
                return (!queue.empty() && reserved + (long long)queue.front()->need <= budget) ||
                       (closing && queue.empty());
            });
            if (queue.empty()) return;  // closing
            job = queue.front();
            queue.pop_front();
            reserved += (long long)job->need;
            max_reserved = std::max(max_reserved, reserved);
            ++running;
            max_running = std::max(max_running, running);
        }
        IsoServeResult r{};
        r.ticket = job->ticket;
        r.slot = index;
        r.t_submit = job->t_submit;
        r.t_start = now_s();
        run(s, *job, r);
        r.t_done = now_s();
        {
            std::lock_guard<std::mutex> lk(mu);
            reserved -= (long long)job->need;
            --running;
            ++completed;
            done[job->ticket] = Done{r};
        }
        delete job;
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

int iso_serve_create(int slots, long long budget_bytes, const int* warm_sizes, int num_warm_sizes, IsoServer** out) {
    if (!out || slots < 1 || slots > 256 || budget_bytes <= 0 || num_warm_sizes < 0) return ISO_ERR_ARG;
    *out = nullptr;
    auto* srv = new IsoServer;
    cudaGetDevice(&srv->device);
    srv->budget = budget_bytes;
    srv->slots.resize(slots);
    int nmax = 2;
    for (int i = 0; i < num_warm_sizes; ++i) nmax = std::max(nmax, warm_sizes[i]);
    const Caps cmax = caps_for(nmax);
    bool ok = true;
    for (Slot& s : srv->slots) {
        s.out_bytes = size_t(12) * (cmax.v + cmax.f);
        ok = ok && cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaMalloc(&s.prims_dev, sizeof(float) * PRIM_FLOATS) == cudaSuccess &&
             cudaMallocHost(&s.prims_host, sizeof(float) * PRIM_FLOATS) == cudaSuccess &&
             cudaMallocHost(&s.small_host, 64) == cudaSuccess && cudaMallocHost(&s.out_host, s.out_bytes) == cudaSuccess;
        if (ok) {
            std::memset(s.prims_host, 0, sizeof(float) * PRIM_FLOATS);
            s.prims_host[0] = 1.0f;  // a sphere of radius 0 until the first request
            ok = cudaMemcpy(s.prims_dev, s.prims_host, sizeof(float) * PRIM_FLOATS, cudaMemcpyHostToDevice) == cudaSuccess;
        }
    }
    // buffers and graphs for the warm-up sizes, both kinds, nagae at level 0
    for (int i = 0; ok && i < num_warm_sizes; ++i) {
        if (warm_sizes[i] < 2 || warm_sizes[i] > 1290) ok = false;
        for (Slot& s : srv->slots)
            for (int kind = 0; ok && kind < 2; ++kind) {
                int err = 0;
                ok = srv->buffers(s, kind, warm_sizes[i], 0, 0.0f, &err) != nullptr;
            }
    }
    if (!ok) {
        cudaGetLastError();
        iso_serve_destroy(srv);
        iso::set_last_error("iso_serve_create: device set-up failed (memory or sizes)");
        return ISO_ERR_CUDA;
    }
    for (int i = 0; i < slots; ++i) srv->threads.emplace_back([srv, i] { srv->worker(i); });
    *out = srv;
    return ISO_OK;
}

long long iso_serve_submit(IsoServer* srv, const IsoServeRequest* req) {
    if (!srv || !req) return -ISO_ERR_ARG;
    if ((req->kind != 0 && req->kind != 1) || req->n < 2 || req->n > 1290 || req->num_prims < 1 ||
        req->num_prims > MAX_PRIMS || !req->prims || (req->kind == 0 && req->method != 0 && req->method != 1))
        return -ISO_ERR_ARG;
    auto* job = new Job;
    job->req = *req;
    std::memset(job->prims, 0, sizeof(job->prims));
    job->prims[0] = float(req->num_prims);
    std::memcpy(job->prims + 1, req->prims, sizeof(float) * 7 * req->num_prims);
    job->req.prims = nullptr;
    job->need = request_bytes(req->kind, req->n);
    job->t_submit = now_s();
    if ((long long)job->need > srv->budget) {
        delete job;
        return -ISO_ERR_WORKSPACE;
    }
    long long ticket;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->closing) {
            delete job;
            return -ISO_ERR_ARG;
        }
        ticket = job->ticket = srv->next_ticket++;
        srv->queue.push_back(job);  // a worker owns (and frees) the job from here
    }
    srv->cv_work.notify_all();
    return ticket;
}

int iso_serve_wait(IsoServer* srv, long long ticket, double timeout_s, IsoServeResult* out) {
    if (!srv || !out || ticket < 0) {
        iso::set_last_error("iso_serve_wait: null server or result, or a negative ticket");
        return ISO_ERR_ARG;
    }
    std::unique_lock<std::mutex> lk(srv->mu);
    if (ticket >= srv->next_ticket) {
        iso::set_last_error("iso_serve_wait: no such ticket");
        return ISO_ERR_ARG;
    }
    const auto ready = [&] { return srv->done.count(ticket) > 0; };
    if (timeout_s < 0) {
        srv->cv_done.wait(lk, ready);
    } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
        return ISO_ERR_TIMEOUT;
    }
    auto it = srv->done.find(ticket);
    *out = it->second.r;
    srv->done.erase(it);
    return ISO_OK;
}

void iso_serve_free_result(IsoServeResult* r) {
    if (!r) return;
    std::free(r->vertices);
    std::free(r->faces);
    r->vertices = nullptr;
    r->faces = nullptr;
}

int iso_serve_stats(IsoServer* srv, long long* stats) {
    if (!srv || !stats) return ISO_ERR_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    stats[0] = srv->completed;
    stats[1] = srv->max_running;
    stats[2] = srv->max_reserved;
    stats[3] = (long long)srv->queue.size();
    return ISO_OK;
}

int iso_serve_destroy(IsoServer* srv) {
    if (!srv) return ISO_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->closing = true;
    }
    srv->cv_work.notify_all();
    for (auto& t : srv->threads) t.join();
    for (auto& kv : srv->done) iso_serve_free_result(&kv.second.r);
    for (Slot& s : srv->slots) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        for (GraphBuf* b : s.bufs) free_buf(b);
        cudaFree(s.prims_dev);
        cudaFreeHost(s.prims_host);
        cudaFreeHost(s.small_host);
        cudaFreeHost(s.out_host);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    delete srv;
    return ISO_OK;
}

// Scale of the capacities of buffers built after the call (1 = the bound on a
// closed surface's mesh).  For tests of the exact-size rerun.
int iso_serve_set_capacity_scale(IsoServer* srv, double scale) {
    if (!srv || !(scale > 0.0) || scale > 1.0) return ISO_ERR_ARG;
    srv->cap_scale = scale;
    return ISO_OK;
}

}  // extern "C"
