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
//
// Length buckets (iso_serve_set_bucket): a worker takes, with the request at
// the head of the queue, up to B - 1 queued requests of the same kind, grid
// size, method and level, and runs them with one launch of a graph that holds
// B parallel branches (fork / join over the slot's helper streams), one per
// request, on an entry with B sets of buffers.  B is a power of two; with
// fewer matching requests the next smaller bucket runs.
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

// Device bytes of an entry of B requests: values and sizes (kept across
// resizes), and outputs and workspaces (resized).
size_t entry_fixed_bytes(int B, int n) { return size_t(B) * al(size_t(4) * n * n * n) + al(size_t(64) * B) + 256; }
size_t entry_var_bytes(int B, int kind, int n, Caps c) {
    return size_t(B) * (al(size_t(12) * c.v) + al(size_t(12) * c.f) + al(ws_bytes(kind, n, c)));
}

// The smallest footprint of a request: its count pass.
size_t count_pass_bytes(int kind, int n) { return entry_fixed_bytes(1, n) + entry_var_bytes(1, kind, n, Caps{1, 1}); }

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

constexpr int BUCKET_MAX = 8;  // requests of one launch at most

// One request's buffers in an entry.
struct Part {
    float* values = nullptr;
    float* vout = nullptr;
    int* fout = nullptr;
    void* ws = nullptr;
    long long* small = nullptr;  // counts, status (MC at [2], DC at [6]); 8 words in the entry's block
};

// A cache entry: one slot's buffers for B requests of one (kind, n, method,
// level), and its graph (B parallel branches).
struct Entry {
    int kind = 0, n = 0, method = 0;
    float level = 0.0f;
    int slot = 0;
    int B = 1;
    Caps cap{0, 0};
    size_t bytes = 0;  // counted against the budget
    size_t wsb = 0;
    Part part[BUCKET_MAX];
    long long* small = nullptr;  // B blocks of 8 words, one copy to the host
    cudaGraphExec_t exec = nullptr;
    bool in_use = false;
    long long last_use = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaStream_t fork[BUCKET_MAX - 1] = {};  // the branches of bucket graphs
    cudaEvent_t ev_fork = nullptr, ev_join[BUCKET_MAX - 1] = {};
    float* prims_dev = nullptr;       // BUCKET_MAX unions
    float* prims_host = nullptr;      // pinned, BUCKET_MAX unions
    long long* small_host = nullptr;  // pinned, BUCKET_MAX blocks of 8 words
    uint8_t* out_host = nullptr;      // pinned staging of the largest mesh
    size_t out_bytes = 0;
    std::vector<Entry*> entries;      // guarded by the server's mutex
};

// Request `i` of entry `e`: its grid from the union at prims_dev, then its
// extraction.
int queue_extraction(const Entry& e, int i, const float* prims_dev, cudaStream_t st) {
    const Part& p = e.part[i];
    if (cudaMemsetAsync(p.small, 0, 64, st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    int rc = iso_sdf_union_grid(prims_dev, e.n, e.n, e.n, LO, HI, p.values, st);
    if (rc) return rc;
    if (e.kind == 0)
        return iso_mc_dense(p.values, e.n, e.n, e.n, LO, HI, e.level, e.method, p.vout, e.cap.v, p.fout, e.cap.f, p.ws,
                            e.wsb, p.small, reinterpret_cast<int*>(p.small + 2), st);
    return iso_dc_dense(p.values, e.n, e.n, e.n, LO, HI, e.level, DC_REG, DC_SVD_TOL, p.vout, e.cap.v, p.fout,
                        e.cap.f, p.ws, e.wsb, p.small, reinterpret_cast<int*>(p.small + 6), st);
}

// Every request of entry e; with B > 1 each on its own branch (fork and join
// over the slot's helper streams, which a capture of `st` takes in).
int queue_entry(const Entry& e, Slot& s, cudaStream_t st) {
    if (e.B == 1) return queue_extraction(e, 0, s.prims_dev, st);
    if (cudaEventRecord(s.ev_fork, st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    for (int i = 1; i < e.B; ++i)
        if (cudaStreamWaitEvent(s.fork[i - 1], s.ev_fork, 0) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    for (int i = 0; i < e.B; ++i) {
        const int rc = queue_extraction(e, i, s.prims_dev + size_t(i) * PRIM_FLOATS, i ? s.fork[i - 1] : st);
        if (rc) return rc;
    }
    for (int i = 1; i < e.B; ++i)
        if (cudaEventRecord(s.ev_join[i - 1], s.fork[i - 1]) != cudaSuccess ||
            cudaStreamWaitEvent(st, s.ev_join[i - 1], 0) != cudaSuccess)
            return iso::fail_code(ISO_ERR_CUDA);
    return ISO_OK;
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
    long long buckets = 0, bucketed = 0;  // launches of more than one request, and their requests
    int running = 0, max_running = 0;     // workers with requests in hand
    int waiting = 0;                      // of them, blocked in acquire
    long long completed = 0;
    bool closing = false;
    double cap_scale = 1.0;  // capacities of entries built or grown from now on (tests shrink them)
    int bucket_max = 1;      // requests per launch at most (a power of two)

    bool acquire(long long bytes);
    void release(long long bytes);
    void free_entry(Entry* e);
    void* alloc(size_t bytes, cudaStream_t st);
    Entry* entry_for(int slot, const Job& job, int B, int* err);
    Entry* build(int slot, int kind, int n, int method, float level, const float* prims_host, bool warm, int B,
                 int* err);
    int size_entry(Entry* e, Caps c);
    void worker(int index);
    void run(int slot, const std::vector<Job*>& jobs, std::vector<IsoServeResult>& res);
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
        // every other running worker waits for memory too: nothing can free
        // any, so this one gives up (its results report ISO_ERR_WORKSPACE)
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
    for (int i = 0; i < e->B; ++i)
        for (void* p : {(void*)e->part[i].values, (void*)e->part[i].vout, (void*)e->part[i].fout, e->part[i].ws})
            if (p) cudaFreeAsync(p, st);
    if (e->small) cudaFreeAsync(e->small, st);
    release((long long)e->bytes);
    delete e;
}

// (Re)sizes an entry's outputs and workspaces to capacities c and captures its
// graph.  The values and sizes buffers stay.  The entry is its slot's alone.
int IsoServer::size_entry(Entry* e, Caps c) {
    Slot& s = slots[e->slot];
    cudaStream_t st = s.stream;
    const size_t old_var = e->bytes - entry_fixed_bytes(e->B, e->n);
    if (e->exec) {
        cudaGraphExecDestroy(e->exec);
        e->exec = nullptr;
    }
    for (int i = 0; i < e->B; ++i) {
        Part& p = e->part[i];
        for (void* q : {(void*)p.vout, (void*)p.fout, p.ws})
            if (q) cudaFreeAsync(q, st);
        p.vout = nullptr;
        p.fout = nullptr;
        p.ws = nullptr;
    }
    e->bytes -= old_var;
    release((long long)old_var);
    const size_t var = entry_var_bytes(e->B, e->kind, e->n, c);
    if (!acquire((long long)var)) return iso::fail_code(ISO_ERR_WORKSPACE);
    e->bytes += var;
    e->cap = c;
    e->wsb = ws_bytes(e->kind, e->n, c);
    for (int i = 0; i < e->B; ++i) {
        Part& p = e->part[i];
        p.vout = static_cast<float*>(alloc(size_t(12) * c.v, st));
        p.fout = static_cast<int*>(alloc(size_t(12) * c.f, st));
        p.ws = alloc(e->wsb, st);
        if (!p.vout || !p.fout || !p.ws) return iso::fail_code(ISO_ERR_CUDA);
    }
    // once outside a graph (first-use set-up of the kernels), then the capture
    for (int i = 0; i < e->B; ++i)
        if (queue_extraction(*e, i, s.prims_dev + size_t(i) * PRIM_FLOATS, st) != 0) return iso::fail_code(ISO_ERR_CUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    const int rc = queue_entry(*e, s, st);
    const bool ended = cudaStreamEndCapture(st, &graph) == cudaSuccess;
    const bool ok = rc == 0 && ended && cudaGraphInstantiate(&e->exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    return ok ? ISO_OK : iso::fail_code(ISO_ERR_CUDA);
}

// A new entry of B requests for `slot`.  Warm entries (built before any
// request) take the closed-surface bound; others run a count pass on the
// request's own union (prims_host) and take its exact sizes plus headroom.
Entry* IsoServer::build(int slot, int kind, int n, int method, float level, const float* prims_host, bool warm,
                        int B, int* err) {
    Slot& s = slots[slot];
    cudaStream_t st = s.stream;
    auto* e = new Entry;
    e->kind = kind;
    e->n = n;
    e->method = method;
    e->level = level;
    e->slot = slot;
    e->B = B;
    e->cap = Caps{1, 1};
    e->wsb = ws_bytes(kind, n, e->cap);
    const size_t b0 = entry_fixed_bytes(B, n) + entry_var_bytes(B, kind, n, e->cap);
    if (!acquire((long long)b0)) {
        delete e;
        *err = ISO_ERR_WORKSPACE;
        return nullptr;
    }
    e->bytes = b0;
    e->small = static_cast<long long*>(alloc(size_t(64) * B, st));
    bool have = e->small != nullptr;
    for (int i = 0; i < B; ++i) {
        Part& p = e->part[i];
        p.values = static_cast<float*>(alloc(size_t(4) * n * n * n, st));
        p.vout = static_cast<float*>(alloc(12, st));
        p.fout = static_cast<int*>(alloc(12, st));
        p.ws = alloc(e->wsb, st);
        p.small = e->small ? e->small + 8 * i : nullptr;
        have = have && p.values && p.vout && p.fout && p.ws;
    }
    int rc = have ? ISO_OK : ISO_ERR_CUDA;
    Caps c = warm_caps(n);
    if (rc == ISO_OK && !warm) {
        // the count pass: the extraction with capacity 1 reports the exact sizes
        std::memcpy(s.prims_host, prims_host, sizeof(float) * PRIM_FLOATS);
        rc = cudaMemcpyAsync(s.prims_dev, s.prims_host, sizeof(float) * PRIM_FLOATS, cudaMemcpyHostToDevice, st) ==
                         cudaSuccess && queue_extraction(*e, 0, s.prims_dev, st) == 0 &&
                     cudaMemcpyAsync(s.small_host, e->part[0].small, 64, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
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

// The entry of B requests like `job` on `slot`, marked in use: cached, or built now.
Entry* IsoServer::entry_for(int slot, const Job& job, int B, int* err) {
    const IsoServeRequest& q = job.req;
    const int method = q.kind == 0 ? q.method : 0;  // dual contouring has no method
    {
        std::lock_guard<std::mutex> lk(mu);
        for (Entry* e : slots[slot].entries)
            if (e->kind == q.kind && e->n == q.n && e->method == method && e->level == q.level && e->B == B) {
                e->in_use = true;
                e->last_use = ++clock;
                return e;
            }
    }
    Entry* e = build(slot, q.kind, q.n, method, q.level, job.prims, false, B, err);
    if (!e) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    e->in_use = true;
    e->last_use = ++clock;
    slots[slot].entries.push_back(e);
    return e;
}

// Requests of one kind, size, method and level (the same entry and graph).
bool same_key(const Job& a, const Job& b) {
    return a.req.kind == b.req.kind && a.req.n == b.req.n && a.req.level == b.req.level &&
           (a.req.kind != 0 || a.req.method == b.req.method);
}

void IsoServer::run(int slot, const std::vector<Job*>& jobs, std::vector<IsoServeResult>& res) {
    Slot& s = slots[slot];
    const int B = int(jobs.size());
    int err = 0;
    Entry* b = entry_for(slot, *jobs[0], B, &err);
    if (!b) {
        for (IsoServeResult& r : res) r.status = err;
        return;
    }
    for (int i = 0; i < B; ++i) std::memcpy(s.prims_host + size_t(i) * PRIM_FLOATS, jobs[i]->prims, sizeof(jobs[i]->prims));
    cudaStream_t st = s.stream;
    const int at = b->kind == 0 ? 2 : 6;
    const size_t pbytes = sizeof(float) * PRIM_FLOATS * B;
    bool ok = cudaMemcpyAsync(s.prims_dev, s.prims_host, pbytes, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaGraphLaunch(b->exec, st) == cudaSuccess &&
              cudaMemcpyAsync(s.small_host, b->small, size_t(64) * B, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaStreamSynchronize(st) == cudaSuccess;
    bool over = false;
    for (int i = 0; ok && i < B; ++i) over = over || int(s.small_host[8 * i + at] & 0xffffffffll) == ISO_ERR_OVERFLOW;
    int rc = ISO_OK;
    if (ok && over) {
        // a mesh larger than the entry's buffers: grow every request's buffers
        // to the largest sizes this run counted, and run again
        {
            std::lock_guard<std::mutex> lk(mu);
            ++grows;
        }
        Caps c{1, 1};
        for (int i = 0; i < B; ++i) {
            const Caps ci = caps_from_counts(b->kind, s.small_host + 8 * i, 1.0);
            c.v = std::max(c.v, ci.v);
            c.f = std::max(c.f, ci.f);
        }
        rc = size_entry(b, c);
        ok = rc == ISO_OK && cudaGraphLaunch(b->exec, st) == cudaSuccess &&
             cudaMemcpyAsync(s.small_host, b->small, size_t(64) * B, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
    }
    for (int i = 0; i < B; ++i) {
        IsoServeResult& r = res[i];
        const long long* sm = s.small_host + 8 * i;
        int status = ok ? int(sm[at] & 0xffffffffll) : (rc ? rc : ISO_ERR_CUDA);
        const long long V = sm[0], F = sm[1];
        if (status == 0 && V > 0 && F > 0) {
            const Part& p = b->part[i];
            r.vertices = static_cast<float*>(std::malloc(size_t(12) * V));
            r.faces = static_cast<int*>(std::malloc(size_t(12) * F));
            const size_t vb = size_t(12) * V, fb = size_t(12) * F;
            bool got = false;
            if (!r.vertices || !r.faces) {
                status = ISO_ERR_ARG;
            } else if (vb + fb <= s.out_bytes) {
                got = cudaMemcpyAsync(s.out_host, p.vout, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                      cudaMemcpyAsync(s.out_host + vb, p.fout, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                      cudaStreamSynchronize(st) == cudaSuccess;
                if (got) {
                    std::memcpy(r.vertices, s.out_host, vb);
                    std::memcpy(r.faces, s.out_host + vb, fb);
                }
            } else {
                got = cudaMemcpyAsync(r.vertices, p.vout, vb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                      cudaMemcpyAsync(r.faces, p.fout, fb, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                      cudaStreamSynchronize(st) == cudaSuccess;
            }
            if (status == 0 && !got) status = ISO_ERR_CUDA;
            r.num_vertices = V;
            r.num_faces = F;
        }
        r.status = status;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        b->in_use = false;
    }
    cv_mem.notify_all();
}

void IsoServer::worker(int index) {
    cudaSetDevice(device);
    while (true) {
        std::vector<Job*> jobs;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return !queue.empty() || closing; });
            if (queue.empty()) return;  // closing
            jobs.push_back(queue.front());
            queue.pop_front();
            if (bucket_max > 1) {
                // the head's bucket: queued requests with its key, in queue order
                for (auto it = queue.begin(); it != queue.end() && int(jobs.size()) < bucket_max;) {
                    if (same_key(**it, *jobs[0])) {
                        jobs.push_back(*it);
                        it = queue.erase(it);
                    } else {
                        ++it;
                    }
                }
                int B = 1;
                while (2 * B <= int(jobs.size())) B *= 2;
                for (int i = int(jobs.size()) - 1; i >= B; --i) queue.push_front(jobs[i]);  // back, in order
                jobs.resize(B);
                if (B > 1) {
                    ++buckets;
                    bucketed += B;
                }
            }
            ++running;
            max_running = std::max(max_running, running);
        }
        std::vector<IsoServeResult> res(jobs.size());
        const double t0 = now_s();
        for (size_t i = 0; i < jobs.size(); ++i) {
            res[i].ticket = jobs[i]->ticket;
            res[i].slot = index;
            res[i].t_submit = jobs[i]->t_submit;
            res[i].t_start = t0;
        }
        run(index, jobs, res);
        const double t1 = now_s();
        {
            std::lock_guard<std::mutex> lk(mu);
            --running;
            for (size_t i = 0; i < jobs.size(); ++i) {
                res[i].t_done = t1;
                ++completed;
                done[jobs[i]->ticket] = Done{res[i]};
            }
        }
        for (Job* j : jobs) delete j;
        cv_done.notify_all();
        cv_mem.notify_all();
    }
}

extern "C" {

int iso_serve_create(int slots, long long budget_bytes, const int* warm_sizes, int num_warm_sizes, IsoServer** out) {
    if (!out || slots < 1 || slots > 256 || budget_bytes <= 0 || num_warm_sizes < 0) return iso::fail_code(ISO_ERR_ARG);
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
    const size_t pbytes = sizeof(float) * PRIM_FLOATS * BUCKET_MAX;
    for (Slot& s : srv->slots) {
        s.out_bytes = size_t(12) * (cmax.v + cmax.f);
        ok = ok && cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&s.ev_fork, cudaEventDisableTiming) == cudaSuccess &&
             srv->acquire(al(pbytes)) &&
             (s.prims_dev = static_cast<float*>(srv->alloc(pbytes, s.stream))) != nullptr &&
             cudaMallocHost(&s.prims_host, pbytes) == cudaSuccess &&
             cudaMallocHost(&s.small_host, size_t(64) * BUCKET_MAX) == cudaSuccess &&
             cudaMallocHost(&s.out_host, s.out_bytes) == cudaSuccess;
        for (int i = 0; ok && i < BUCKET_MAX - 1; ++i)
            ok = cudaStreamCreateWithFlags(&s.fork[i], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&s.ev_join[i], cudaEventDisableTiming) == cudaSuccess;
        if (ok) {
            std::memset(s.prims_host, 0, pbytes);
            for (int i = 0; i < BUCKET_MAX; ++i)
                s.prims_host[size_t(i) * PRIM_FLOATS] = 1.0f;  // a sphere of radius 0 until a request comes
            ok = cudaMemcpyAsync(s.prims_dev, s.prims_host, pbytes, cudaMemcpyHostToDevice, s.stream) == cudaSuccess &&
                 cudaStreamSynchronize(s.stream) == cudaSuccess;
        }
    }
    // entries for the warm-up sizes, both kinds, nagae at level 0
    for (int i = 0; ok && i < num_warm_sizes; ++i) {
        if (warm_sizes[i] < 2 || warm_sizes[i] > 1290) ok = false;
        for (int si = 0; ok && si < slots; ++si)
            for (int kind = 0; ok && kind < 2; ++kind) {
                int err = 0;
                Entry* e = srv->build(si, kind, warm_sizes[i], 0, 0.0f, nullptr, true, 1, &err);
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
    if (!srv || !req) return -iso::fail_code(ISO_ERR_ARG);
    if ((req->kind != 0 && req->kind != 1) || req->n < 2 || req->n > 1290 || req->num_prims < 1 ||
        req->num_prims > MAX_PRIMS || !req->prims || (req->kind == 0 && req->method != 0 && req->method != 1))
        return -iso::fail_code(ISO_ERR_ARG);
    // the count pass alone (values and the workspace at capacity 1) must fit
    // beside the slots' own buffers
    const long long fixed = (long long)srv->slots.size() * (long long)al(sizeof(float) * PRIM_FLOATS * BUCKET_MAX);
    if ((long long)count_pass_bytes(req->kind, req->n) + fixed > srv->budget) return -iso::fail_code(ISO_ERR_WORKSPACE);
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
            return -iso::fail_code(ISO_ERR_ARG);
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
        return iso::fail_code(ISO_ERR_TIMEOUT);
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
    if (!srv || !stats || count < 0) return iso::fail_code(ISO_ERR_ARG);
    std::lock_guard<std::mutex> lk(srv->mu);
    long long entries = 0;
    for (const Slot& s : srv->slots) entries += (long long)s.entries.size();
    const long long all[12] = {srv->completed, srv->max_running, srv->max_held, (long long)srv->queue.size(),
                               srv->held, srv->evictions, entries, srv->count_passes, srv->grows, srv->budget,
                               srv->buckets, srv->bucketed};
    for (int i = 0; i < std::min(count, 12); ++i) stats[i] = all[i];
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
        for (int i = 0; i < BUCKET_MAX - 1; ++i) {
            if (s.fork[i]) cudaStreamDestroy(s.fork[i]);
            if (s.ev_join[i]) cudaEventDestroy(s.ev_join[i]);
        }
        if (s.ev_fork) cudaEventDestroy(s.ev_fork);
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

// Requests per launch at most (1, 2, 4 or 8; 1: each request its own launch).
int iso_serve_set_bucket(IsoServer* srv, int max_requests) {
    if (!srv || max_requests < 1 || max_requests > BUCKET_MAX || (max_requests & (max_requests - 1))) return iso::fail_code(ISO_ERR_ARG);
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->bucket_max = max_requests;
    return ISO_OK;
}

// Scale of the capacities of entries built or grown after the call (tests of
// the growth path; 1 = the counted sizes plus headroom).
int iso_serve_set_capacity_scale(IsoServer* srv, double scale) {
    if (!srv || !(scale > 0.0) || scale > 1.0) return iso::fail_code(ISO_ERR_ARG);
    srv->cap_scale = scale;
    return ISO_OK;
}

}  // extern "C"
