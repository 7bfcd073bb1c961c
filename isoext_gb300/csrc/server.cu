// Native serving loop: continuous batching of extraction requests on one GPU.
//
// A request is a cubic grid (n points per axis over [-1, 1]^3) given as a union
// of spheres and boxes, and an extraction (marching cubes or dual contouring).
// The server keeps `slots` worker threads, each with its own CUDA stream and a
// cache of entries: per (kind, n, method, level), device buffers and a CUDA
// graph of iso_sdf_union_grid + iso_mc_dense / iso_dc_dense captured once.
// Requests are taken first come, first served by free workers; requests on
// different slots overlap on the GPU.  A request costs one 904-byte H2D copy,
// one graph launch, a 64-byte D2H of the sizes and the mesh's D2H through the
// slot's pinned staging buffer.
//
// Device memory is bounded by the budget.  Every byte the server allocates
// (per-slot buffers and every cached entry) is counted while it is held, and
// an allocation that would take the count above the budget first evicts the
// least recently used entries that no request is using, or waits for running
// requests to release theirs.  A new entry is sized from a count pass on the
// request that needs it: the extraction with minimal output capacities, which
// reports the mesh's exact sizes.  A later mesh larger than its entry's buffers
// grows the entry from the exact sizes it reported, and the graph runs again.
// Allocations come from a private stream-ordered pool, so freeing an entry does
// not synchronise the device.  No counterpart in isoext.
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
constexpr double HEADROOM = 1.25;  // capacity over the counted sizes (other unions of the same key)
constexpr long long SLACK = 1024;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Caps {
    long long v, f;
};

// Output capacities of a warm-up entry, built before any request: faces of a
// closed surface inside the box stay below twice the grid's face area in cells.
Caps warm_caps(int n) {
    const long long f = 4ll * 6 * (n - 1) * (n - 1) + 4096;
    return {f / 2 + 4096, f};
}

size_t ws_bytes(int kind, int n, Caps c) {
    return kind == 0 ? iso_mc_dense_workspace_size(n, n, n, c.v, c.f) : iso_dc_dense_workspace_size(n, n, n, c.v, c.f);
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

// Device bytes of an entry's values, outputs and workspace.
size_t entry_bytes(int kind, int n, Caps c) {
    return al(size_t(4) * n * n * n) + al(size_t(12) * c.v) + al(size_t(12) * c.f) + al(ws_bytes(kind, n, c)) + 256;
}

// The smallest footprint of a request: its count pass.
size_t count_pass_bytes(int kind, int n) { return entry_bytes(kind, n, Caps{1, 1}); }

// Capacities for a mesh whose sizes a pass counted: MC counts vertices and
// faces, DC active cells (its vertices at most) and quads (two faces each).
Caps caps_from_counts(int kind, const long long* small, double scale) {
    const long long v = kind == 0 ? small[0] : small[2];
    const long long f = kind == 0 ? small[1] : 2 * small[4];
    return {std::max<long long>(1, (long long)(scale * (HEADROOM * v + SLACK))),
            std::max<long long>(1, (long long)(scale * (HEADROOM * f + SLACK)))};
}

struct Job {
    long long ticket;
    IsoServeRequest req;
    float prims[PRIM_FLOATS];
    double t_submit;
};

struct Done {
    IsoServeResult r;
};

// A cache entry: one slot's buffers for one (kind, n, method, level), and its graph.
struct Entry {
    int kind = 0, n = 0, method = 0;
    float level = 0.0f;
    int slot = 0;
    Caps cap{0, 0};
    size_t bytes = 0;  // counted against the budget
    float* values = nullptr;
    float* vout = nullptr;
    int* fout = nullptr;
    void* ws = nullptr;
    size_t wsb = 0;
    long long* small = nullptr;  // counts, status (MC at [2], DC at [6])
    cudaGraphExec_t exec = nullptr;
    bool in_use = false;
    long long last_use = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    float* prims_dev = nullptr;
    float* prims_host = nullptr;      // pinned
    long long* small_host = nullptr;  // pinned [8]
    uint8_t* out_host = nullptr;      // pinned staging of the largest mesh
    size_t out_bytes = 0;
    std::vector<Entry*> entries;      // guarded by the server's mutex
};

int queue_extraction(const Entry& b, const float* prims_dev, cudaStream_t st) {
    if (cudaMemsetAsync(b.small, 0, 64, st) != cudaSuccess) return ISO_ERR_CUDA;
    int rc = iso_sdf_union_grid(prims_dev, b.n, b.n, b.n, LO, HI, b.values, st);
    if (rc) return rc;
    if (b.kind == 0)
        return iso_mc_dense(b.values, b.n, b.n, b.n, LO, HI, b.level, b.method, b.vout, b.cap.v, b.fout, b.cap.f, b.ws,
                            b.wsb, b.small, reinterpret_cast<int*>(b.small + 2), st);
    return iso_dc_dense(b.values, b.n, b.n, b.n, LO, HI, b.level, DC_REG, DC_SVD_TOL, b.vout, b.cap.v, b.fout, b.cap.f,
                        b.ws, b.wsb, b.small, reinterpret_cast<int*>(b.small + 6), st);
}

}  // namespace

struct IsoServer {
    int device = 0;
    long long budget = 0;
    cudaMemPool_t pool = nullptr;
    cudaStream_t free_stream = nullptr;  // frees of evicted entries (a slot's stream may be capturing)
    std::vector<Slot> slots;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_mem;
    std::deque<Job*> queue;
    std::map<long long, Done> done;
    long long next_ticket = 0;
    long long held = 0, max_held = 0;  // device bytes the server holds
    long long evictions = 0, count_passes = 0, grows = 0, clock = 0;
    int running = 0, max_running = 0;
    int waiting = 0;  // running requests blocked in acquire
    long long completed = 0;
    bool closing = false;
    double cap_scale = 1.0;  // capacities of entries built or grown from now on (tests shrink them)

    bool acquire(long long bytes);
    void release(long long bytes);
    void free_entry(Entry* e);
    void* alloc(size_t bytes, cudaStream_t st);
    Entry* entry_for(int slot, const Job& job, int* err);
    Entry* build(int slot, int kind, int n, int method, float level, const float* prims_host, bool warm, int* err);
    int size_entry(Entry* e, Caps c);
    void worker(int index);
    void run(int slot, Job& job, IsoServeResult& r);
};

// Counts `bytes` against the budget, evicting idle entries (least recently
// used first) while they do not fit; waits while running requests hold what is
// missing.  False when nothing can make room.
bool IsoServer::acquire(long long bytes) {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        if (held + bytes <= budget) {
            held += bytes;
            max_held = std::max(max_held, held);
            return true;
        }
        Entry* victim = nullptr;
        for (Slot& s : slots)
            for (Entry* e : s.entries)
                if (!e->in_use && (!victim || e->last_use < victim->last_use)) victim = e;
        if (victim) {
            auto& v = slots[victim->slot].entries;
            v.erase(std::find(v.begin(), v.end(), victim));
            ++evictions;
            lk.unlock();
            free_entry(victim);  // releases its bytes
            lk.lock();
            continue;
        }
        // every other running request waits for memory too: nothing can free
        // any, so this request gives up (its result reports ISO_ERR_WORKSPACE)
        if (waiting + 1 >= running) return false;
        ++waiting;
        cv_mem.wait(lk);
        --waiting;
    }
}

void IsoServer::release(long long bytes) {
    {
        std::lock_guard<std::mutex> lk(mu);
        held -= bytes;
    }
    cv_mem.notify_all();
}

void* IsoServer::alloc(size_t bytes, cudaStream_t st) {
    void* p = nullptr;
    return cudaMallocFromPoolAsync(&p, std::max<size_t>(bytes, 256), pool, st) == cudaSuccess ? p : nullptr;
}

// Frees an entry that no request uses.  Its slot's last work on it has
// completed (a request ends with a synchronisation of the slot's stream), and
// that stream may be capturing another entry's graph right now, so the frees
// go to the server's own stream.
void IsoServer::free_entry(Entry* e) {
    cudaStream_t st = free_stream;
    if (e->exec) cudaGraphExecDestroy(e->exec);
    for (void* p : {(void*)e->values, (void*)e->vout, (void*)e->fout, e->ws, (void*)e->small})
        if (p) cudaFreeAsync(p, st);
    release((long long)e->bytes);
    delete e;
}

// (Re)sizes an entry's outputs and workspace to capacities c and captures its
// graph.  The values and sizes buffers stay.  The entry is its slot's alone.
int IsoServer::size_entry(Entry* e, Caps c) {
    cudaStream_t st = slots[e->slot].stream;
    const size_t old_var = e->bytes - (al(size_t(4) * e->n * e->n * e->n) + 256);
    if (e->exec) {
        cudaGraphExecDestroy(e->exec);
        e->exec = nullptr;
    }
    for (void* p : {(void*)e->vout, (void*)e->fout, e->ws})
        if (p) cudaFreeAsync(p, st);
    e->vout = nullptr;
    e->fout = nullptr;
    e->ws = nullptr;
    e->bytes -= old_var;
    release((long long)old_var);
    const size_t wsb = ws_bytes(e->kind, e->n, c);
    const size_t var = al(size_t(12) * c.v) + al(size_t(12) * c.f) + al(wsb);
    if (!acquire((long long)var)) return ISO_ERR_WORKSPACE;
    e->bytes += var;
    e->cap = c;
    e->wsb = wsb;
    e->vout = static_cast<float*>(alloc(size_t(12) * c.v, st));
    e->fout = static_cast<int*>(alloc(size_t(12) * c.f, st));
    e->ws = alloc(wsb, st);
    if (!e->vout || !e->fout || !e->ws) return ISO_ERR_CUDA;
    // once outside a graph (first-use set-up of the kernels), then the capture
    if (queue_extraction(*e, slots[e->slot].prims_dev, st) != 0 || cudaStreamSynchronize(st) != cudaSuccess)
        return ISO_ERR_CUDA;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return ISO_ERR_CUDA;
    const int rc = queue_extraction(*e, slots[e->slot].prims_dev, st);
    const bool ended = cudaStreamEndCapture(st, &graph) == cudaSuccess;
    const bool ok = rc == 0 && ended && cudaGraphInstantiate(&e->exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    return ok ? ISO_OK : ISO_ERR_CUDA;
}

// A new entry for `slot`.  Warm entries (built before any request) take the
// closed-surface bound; others run a count pass on the request's own union
// (prims_host) and take its exact sizes plus headroom.
Entry* IsoServer::build(int slot, int kind, int n, int method, float level, const float* prims_host, bool warm,
                        int* err) {
    Slot& s = slots[slot];
    cudaStream_t st = s.stream;
    auto* e = new Entry;
    e->kind = kind;
    e->n = n;
    e->method = method;
    e->level = level;
    e->slot = slot;
    e->cap = Caps{1, 1};
    e->wsb = ws_bytes(kind, n, e->cap);
    const size_t b0 = count_pass_bytes(kind, n);
    if (!acquire((long long)b0)) {
        delete e;
        *err = ISO_ERR_WORKSPACE;
        return nullptr;
    }
    e->bytes = b0;
    e->values = static_cast<float*>(alloc(size_t(4) * n * n * n, st));
    e->vout = static_cast<float*>(alloc(12, st));
    e->fout = static_cast<int*>(alloc(12, st));
    e->ws = alloc(e->wsb, st);
    e->small = static_cast<long long*>(alloc(64, st));
    int rc = (e->values && e->vout && e->fout && e->ws && e->small) ? ISO_OK : ISO_ERR_CUDA;
    Caps c = warm_caps(n);
    if (rc == ISO_OK && !warm) {
        // the count pass: the extraction with capacity 1 reports the exact sizes
        std::memcpy(s.prims_host, prims_host, sizeof(float) * PRIM_FLOATS);
        rc = cudaMemcpyAsync(s.prims_dev, s.prims_host, sizeof(float) * PRIM_FLOATS, cudaMemcpyHostToDevice, st) ==
                         cudaSuccess && queue_extraction(*e, s.prims_dev, st) == 0 &&
                     cudaMemcpyAsync(s.small_host, e->small, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                     cudaStreamSynchronize(st) == cudaSuccess
                 ? ISO_OK
                 : ISO_ERR_CUDA;
        c = caps_from_counts(kind, s.small_host, 1.0);
        std::lock_guard<std::mutex> lk(mu);
        ++count_passes;
    }
    if (rc == ISO_OK) {
        c.v = std::max<long long>(1, (long long)(c.v * cap_scale));
        c.f = std::max<long long>(1, (long long)(c.f * cap_scale));
        rc = size_entry(e, c);
    }
    if (rc != ISO_OK) {
        cudaGetLastError();
        free_entry(e);
        *err = rc;
        return nullptr;
    }
    return e;
}

// The job's entry on `slot`, marked in use: cached, or built now.
Entry* IsoServer::entry_for(int slot, const Job& job, int* err) {
    const IsoServeRequest& q = job.req;
    const int method = q.kind == 0 ? q.method : 0;  // dual contouring has no method
    {
        std::lock_guard<std::mutex> lk(mu);
        for (Entry* e : slots[slot].entries)
            if (e->kind == q.kind && e->n == q.n && e->method == method && e->level == q.level) {
                e->in_use = true;
                e->last_use = ++clock;
                return e;
            }
    }
    Entry* e = build(slot, q.kind, q.n, method, q.level, job.prims, false, err);
    if (!e) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    e->in_use = true;
    e->last_use = ++clock;
    slots[slot].entries.push_back(e);
    return e;
}

void IsoServer::run(int slot, Job& job, IsoServeResult& r) {
    Slot& s = slots[slot];
    int err = 0;
    Entry* b = entry_for(slot, job, &err);
    if (!b) {
        r.status = err;
        return;
    }
    std::memcpy(s.prims_host, job.prims, sizeof(job.prims));
    cudaStream_t st = s.stream;
    const int at = b->kind == 0 ? 2 : 6;
    bool ok = cudaMemcpyAsync(s.prims_dev, s.prims_host, sizeof(job.prims), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaGraphLaunch(b->exec, st) == cudaSuccess &&
              cudaMemcpyAsync(s.small_host, b->small, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaStreamSynchronize(st) == cudaSuccess;
    int status = ok ? int(s.small_host[at] & 0xffffffffll) : ISO_ERR_CUDA;
    if (status == ISO_ERR_OVERFLOW) {
        // larger than the entry's buffers: grow it from the exact sizes this run
        // counted, and run again
        {
            std::lock_guard<std::mutex> lk(mu);
            ++grows;
        }
        const int rc = size_entry(b, caps_from_counts(b->kind, s.small_host, 1.0));
        ok = rc == ISO_OK && cudaGraphLaunch(b->exec, st) == cudaSuccess &&
             cudaMemcpyAsync(s.small_host, b->small, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
        status = ok ? int(s.small_host[at] & 0xffffffffll) : (rc ? rc : ISO_ERR_CUDA);
    }
    const long long V = s.small_host[0], F = s.small_host[1];
    if (status == 0 && V > 0 && F > 0) {
        r.vertices = static_cast<float*>(std::malloc(size_t(12) * V));
        r.faces = static_cast<int*>(std::malloc(size_t(12) * F));
        const size_t vb = size_t(12) * V, fb = size_t(12) * F;
        if (!r.vertices || !r.faces) {
            status = ISO_ERR_ARG;
        } else if (vb + fb <= s.out_bytes) {
            ok = cudaMemcpyAsync(s.out_host, b->vout, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaMemcpyAsync(s.out_host + vb, b->fout, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaStreamSynchronize(st) == cudaSuccess;
            if (ok) {
                std::memcpy(r.vertices, s.out_host, vb);
                std::memcpy(r.faces, s.out_host + vb, fb);
            }
        } else {
            ok = cudaMemcpyAsync(r.vertices, b->vout, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaMemcpyAsync(r.faces, b->fout, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                 cudaStreamSynchronize(st) == cudaSuccess;
        }
        if (!ok) status = ISO_ERR_CUDA;
        r.num_vertices = V;
        r.num_faces = F;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        b->in_use = false;
    }
    cv_mem.notify_all();
    r.status = status;
}

void IsoServer::worker(int index) {
    cudaSetDevice(device);
    while (true) {
        Job* job = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return !queue.empty() || closing; });
            if (queue.empty()) return;  // closing
            job = queue.front();
            queue.pop_front();
            ++running;
            max_running = std::max(max_running, running);
        }
        IsoServeResult r{};
        r.ticket = job->ticket;
        r.slot = index;
        r.t_submit = job->t_submit;
        r.t_start = now_s();
        run(index, *job, r);
        r.t_done = now_s();
        {
            std::lock_guard<std::mutex> lk(mu);
            --running;
            ++completed;
            done[job->ticket] = Done{r};
        }
        delete job;
        cv_done.notify_all();
        cv_mem.notify_all();
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
    const Caps cmax = warm_caps(nmax);
    // a private stream-ordered pool: freeing an entry does not synchronise the device
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = srv->device;
    bool ok = cudaMemPoolCreate(&srv->pool, &props) == cudaSuccess &&
              cudaStreamCreateWithFlags(&srv->free_stream, cudaStreamNonBlocking) == cudaSuccess;
    for (Slot& s : srv->slots) {
        s.out_bytes = size_t(12) * (cmax.v + cmax.f);
        ok = ok && cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) == cudaSuccess &&
             srv->acquire(al(sizeof(float) * PRIM_FLOATS)) &&
             (s.prims_dev = static_cast<float*>(srv->alloc(sizeof(float) * PRIM_FLOATS, s.stream))) != nullptr &&
             cudaMallocHost(&s.prims_host, sizeof(float) * PRIM_FLOATS) == cudaSuccess &&
             cudaMallocHost(&s.small_host, 64) == cudaSuccess && cudaMallocHost(&s.out_host, s.out_bytes) == cudaSuccess;
        if (ok) {
            std::memset(s.prims_host, 0, sizeof(float) * PRIM_FLOATS);
            s.prims_host[0] = 1.0f;  // a sphere of radius 0 until the first request
            ok = cudaMemcpyAsync(s.prims_dev, s.prims_host, sizeof(float) * PRIM_FLOATS, cudaMemcpyHostToDevice,
                                 s.stream) == cudaSuccess &&
                 cudaStreamSynchronize(s.stream) == cudaSuccess;
        }
    }
    // entries for the warm-up sizes, both kinds, nagae at level 0
    for (int i = 0; ok && i < num_warm_sizes; ++i) {
        if (warm_sizes[i] < 2 || warm_sizes[i] > 1290) ok = false;
        for (int si = 0; ok && si < slots; ++si)
            for (int kind = 0; ok && kind < 2; ++kind) {
                int err = 0;
                Entry* e = srv->build(si, kind, warm_sizes[i], 0, 0.0f, nullptr, true, &err);
                ok = e != nullptr;
                if (ok) {
                    std::lock_guard<std::mutex> lk(srv->mu);
                    e->last_use = ++srv->clock;
                    srv->slots[si].entries.push_back(e);
                }
            }
    }
    if (!ok) {
        cudaGetLastError();
        iso_serve_destroy(srv);
        iso::set_last_error("iso_serve_create: device set-up failed (memory, budget or sizes)");
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
    // the count pass alone (values and the workspace at capacity 1) must fit
    // beside the slots' own buffers
    const long long fixed = (long long)srv->slots.size() * (long long)al(sizeof(float) * PRIM_FLOATS);
    if ((long long)count_pass_bytes(req->kind, req->n) + fixed > srv->budget) return -ISO_ERR_WORKSPACE;
    auto* job = new Job;
    job->req = *req;
    std::memset(job->prims, 0, sizeof(job->prims));
    job->prims[0] = float(req->num_prims);
    std::memcpy(job->prims + 1, req->prims, sizeof(float) * 7 * req->num_prims);
    job->req.prims = nullptr;
    job->t_submit = now_s();
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

int iso_serve_stats_ex(IsoServer* srv, long long* stats, int count) {
    if (!srv || !stats || count < 0) return ISO_ERR_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    long long entries = 0;
    for (const Slot& s : srv->slots) entries += (long long)s.entries.size();
    const long long all[10] = {srv->completed, srv->max_running, srv->max_held, (long long)srv->queue.size(),
                               srv->held, srv->evictions, entries, srv->count_passes, srv->grows, srv->budget};
    for (int i = 0; i < std::min(count, 10); ++i) stats[i] = all[i];
    return ISO_OK;
}

int iso_serve_stats(IsoServer* srv, long long* stats) { return iso_serve_stats_ex(srv, stats, 4); }

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
        for (Entry* e : s.entries) srv->free_entry(e);
        s.entries.clear();
        if (s.prims_dev) cudaFreeAsync(s.prims_dev, s.stream);
        if (s.stream) cudaStreamSynchronize(s.stream);
        cudaFreeHost(s.prims_host);
        cudaFreeHost(s.small_host);
        cudaFreeHost(s.out_host);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    if (srv->free_stream) {
        cudaStreamSynchronize(srv->free_stream);
        cudaStreamDestroy(srv->free_stream);
    }
    if (srv->pool) cudaMemPoolDestroy(srv->pool);
    delete srv;
    return ISO_OK;
}

// Scale of the capacities of entries built or grown after the call (tests of
// the growth path; 1 = the counted sizes plus headroom).
int iso_serve_set_capacity_scale(IsoServer* srv, double scale) {
    if (!srv || !(scale > 0.0) || scale > 1.0) return ISO_ERR_ARG;
    srv->cap_scale = scale;
    return ISO_OK;
}

}  // extern "C"
