// sod_server.cu -- request loop with continuous batching for CQBEM objects on one GPU.
//
// Two request types arrive at any time from any host thread:
//   * assembly: a new object (mesh, material, BDF order, dt, N) -> the CQ precompute of its time
//     weights G_k, H_k (all Laplace frequencies assembled and transformed on the device) packed into
//     a device-resident FP32 history bank; the object stays resident until evicted;
//   * step: one time step of a resident object -> push (p_n, u_n) into its history ring and return
//     b = sum_k G_k p_{n-k} - H_k u_{n-k} (the per-step work of src/elastodynamics_cqbem_object.cpp:44-48).
//
// Threads and streams:
//   * a scheduler thread admits work and polls completion events; it never blocks on device work;
//   * `slots` assembly threads, each with its own context and stream, run admitted assemblies
//     concurrently with each other and with the steps;
//   * one step stream (the scheduler's context) runs the steps of all objects in arrival order per
//     object: each dispatch groups one pending step of every ready object (up to HIST_GROUP_MAX) into
//     one host-to-device copy, three launches (push, convolution tiles of every bank, finish) and one
//     device-to-host copy, through a ring of pinned host / device staging slots;
//   * a janitor thread frees evicted objects (cudaFree may wait for the device).
// Admission: an assembly is admitted while a slot is free and the bytes of resident banks plus
// in-flight assembly buffers stay under the HBM cap; least recently used idle objects are evicted
// to make room.  Latency = completion (event observed) - submission, per request.
// Results are independent of the mix: every kernel is deterministic and per-object work is ordered.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sod_internal.h"

using namespace sod;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    int64_t id = 0;
    int type = 0;  // 0 assembly, 1 step
    Clock::time_point t_submit;
    // assembly
    std::vector<double> V;
    std::vector<int> F;
    double E = 0, nu = 0, rho = 0, dt = 0;
    int bdf = 2, N = 0, order = 5, subdiv = 1, nV = 0, nF = 0;
    // step
    int64_t object = -1;
    std::vector<double> p, u, b;
    int status = SOD_OK;
};

struct Object {
    int64_t id = 0;
    int n = 0;  // 3 nV
    sod_history *bank = nullptr;
    int64_t bytes = 0;
    bool ready = false;
    int pending = 0;  // steps queued or in flight
    Clock::time_point last_use;
    std::deque<Request *> steps;
};

// One group of time steps in flight: at most one step per object, all run by three launches
// (history_step_group).  Pinned and device buffers hold the members' [p | u] back to back, then their b.
struct StepSlot {
    double *hbuf = nullptr;  // pinned
    double *dbuf = nullptr;  // device
    cudaEvent_t ev = nullptr;
    std::vector<Request *> reqs;
    std::vector<Object *> objs;
    std::vector<size_t> boff;  // offset of each member's b
};

struct AsmDone {
    Request *req;
    int status;
    sod_history *bank;
    int64_t bytes;
    cudaEvent_t packed;
};

}  // namespace

struct sod_server {
    int device = 0;
    int64_t cap = 0, committed = 0;  // bytes: resident banks + in-flight assembly buffers
    int vmax_n = 0;
    std::atomic<int64_t> next_id{1};
    std::atomic<bool> stop{false};
    // inbox (any thread) -> scheduler
    std::mutex in_mu;
    std::condition_variable in_cv;
    std::deque<Request *> inbox;
    int64_t submitted = 0, completed_count = 0;
    // completions (scheduler) -> poll / result
    std::mutex out_mu;
    std::condition_variable out_cv;
    struct Done {
        int64_t id;
        int status;
        int64_t ns;
    };
    std::deque<Done> done;
    std::unordered_map<int64_t, std::vector<double>> results;
    // scheduler state
    std::deque<Request *> pending_asm;
    std::unordered_map<int64_t, std::unique_ptr<Object>> objects;
    // steps naming an object whose assembly has not finished yet
    std::unordered_map<int64_t, std::deque<Request *>> early;
    std::unordered_map<int64_t, int> assembling;  // ids of assemblies not yet finished
    sod_context *step_ctx = nullptr;
    std::vector<StepSlot> ring;
    std::deque<int> free_ring;
    // assembly slots
    struct Slot {
        sod_context *ctx = nullptr;
        std::thread th;
        std::mutex mu;
        std::condition_variable cv;
        Request *job = nullptr;
        int64_t job_bytes = 0;
        bool busy = false;
    };
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex asm_mu;
    std::vector<AsmDone> asm_done;
    std::vector<std::pair<AsmDone, Request *>> packing;  // waiting for the pack event
    // janitor
    std::mutex jan_mu;
    std::condition_variable jan_cv;
    std::deque<std::pair<sod_history *, int64_t>> trash;
    std::thread scheduler, janitor;
};

namespace {

int64_t bank_bytes(int n, int K) { return 4LL * K * 2 * n * (int64_t)((n + 7) / 8 * 8) + 4LL * K * 2 * ((n + 7) / 8 * 8); }
int64_t asm_temp_bytes(int n, int N) { return 4LL * 2 * (N + 1) * (int64_t)n * n; }

void complete(sod_server *s, Request *r, int status) {
    const int64_t ns = std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - r->t_submit).count();
    {
        std::lock_guard<std::mutex> g(s->out_mu);
        s->done.push_back({r->id, status, ns});
        if (r->type == 1 && status == SOD_OK) s->results[r->id] = std::move(r->b);
        s->completed_count++;
    }
    s->out_cv.notify_all();
    delete r;
}

// ---- assembly slot thread ------------------------------------------------------------------
void slot_main(sod_server *s, sod_server::Slot *sl) {
    cudaSetDevice(s->device);
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> g(sl->mu);
            sl->cv.wait(g, [&] { return sl->job != nullptr || s->stop.load(); });
            if (sl->job == nullptr) return;
            r = sl->job;
        }
        AsmDone d{r, SOD_OK, nullptr, 0, nullptr};
        sod_mesh *mesh = nullptr;
        float *tmp = nullptr;
        int rc = sod_mesh_create(sl->ctx, r->V.data(), r->nV, r->F.data(), r->nF, nullptr, nullptr, &mesh);
        const int n = 3 * r->nV, L = r->N + 1;
        const size_t nn = (size_t)n * n;
        const double mu = r->E / (2.0 * (1.0 + r->nu)), lam = 2.0 * r->nu * mu / (1.0 - 2.0 * r->nu);
        const double c1 = std::sqrt((lam + 2.0 * mu) / r->rho), c2 = std::sqrt(mu / r->rho);
        const double cm[3] = {0, 0, 0};
        if (rc == SOD_OK && cudaMallocAsync(reinterpret_cast<void **>(&tmp), sizeof(float) * 2 * L * nn,
                                            sl->ctx->stream) != cudaSuccess) {
            rc = SOD_ERR_OOM;
            tmp = nullptr;
        }
        if (rc == SOD_OK)
            rc = sod_cqbem_precompute(sl->ctx, mesh, SOD_COLLOCATION, c1, c2, r->rho, r->nu, r->bdf, r->dt, r->N,
                                      r->order, r->subdiv, std::min(r->order, 5), r->subdiv, cm, tmp, tmp + L * nn,
                                      nullptr, nullptr, nullptr, SOD_F32);
        if (rc == SOD_OK && cudaStreamSynchronize(sl->ctx->stream) != cudaSuccess) rc = SOD_ERR_CUDA;
        if (rc == SOD_OK) rc = take_device_error(sl->ctx);
        if (rc == SOD_OK) rc = sod_history_create(s->step_ctx, n, n, r->N, 1, SOD_F32, &d.bank);
        for (int k = 1; rc == SOD_OK && k <= r->N; k++)
            rc = sod_history_set_weights(d.bank, k, tmp + k * nn, tmp + (L + k) * nn, SOD_F32);
        if (rc == SOD_OK) {
            cudaEventCreateWithFlags(&d.packed, cudaEventDisableTiming);
            cudaEventRecord(d.packed, s->step_ctx->stream);
        }
        // once a bank exists its weight copies (on the step stream) read tmp, also when a later copy
        // failed: free it behind them; otherwise behind the precompute on the slot's stream
        if (tmp) cudaFreeAsync(tmp, d.bank ? s->step_ctx->stream : sl->ctx->stream);
        if (mesh) sod_mesh_destroy(mesh);
        if (rc != SOD_OK && d.bank) {
            sod_history_destroy(d.bank);
            d.bank = nullptr;
        }
        d.status = rc;
        d.bytes = rc == SOD_OK ? bank_bytes(n, r->N) : 0;
        {
            std::lock_guard<std::mutex> g(sl->mu);
            sl->job = nullptr;
        }
        {
            std::lock_guard<std::mutex> g(s->asm_mu);
            s->asm_done.push_back(d);
        }
        s->in_cv.notify_all();
    }
}

// ---- janitor thread: frees evicted banks -------------------------------------------------------
void janitor_main(sod_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::pair<sod_history *, int64_t> t;
        {
            std::unique_lock<std::mutex> g(s->jan_mu);
            s->jan_cv.wait(g, [&] { return !s->trash.empty() || s->stop.load(); });
            if (s->trash.empty()) return;
            t = s->trash.front();
            s->trash.pop_front();
        }
        sod_history_destroy(t.first);
        {
            std::lock_guard<std::mutex> g(s->in_mu);
            s->committed -= t.second;
        }
        s->in_cv.notify_all();
    }
}

// ---- scheduler -------------------------------------------------------------------------------------
bool evict_one(sod_server *s) {
    Object *victim = nullptr;
    for (auto &kv : s->objects) {
        Object *o = kv.second.get();
        if (!o->ready || o->pending > 0) continue;
        if (!victim || o->last_use < victim->last_use) victim = o;
    }
    if (!victim) return false;
    {
        std::lock_guard<std::mutex> g(s->jan_mu);
        s->trash.push_back({victim->bank, victim->bytes});
    }
    s->jan_cv.notify_one();
    s->objects.erase(victim->id);
    return true;
}

void scheduler_main(sod_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        bool progress = false;
        std::deque<Request *> arrivals;
        {
            std::unique_lock<std::mutex> g(s->in_mu);
            if (s->inbox.empty() && !s->stop.load())
                s->in_cv.wait_for(g, std::chrono::microseconds(50));
            arrivals.swap(s->inbox);
            if (s->stop.load() && arrivals.empty()) {
                bool idle = s->pending_asm.empty() && s->packing.empty() && s->early.empty() &&
                            s->free_ring.size() == s->ring.size();
                for (auto &sl : s->slots) idle = idle && !sl->busy;
                for (auto &kv : s->objects) idle = idle && kv.second->steps.empty();
                if (idle) return;
            }
        }
        for (Request *r : arrivals) {
            progress = true;
            if (r->type == 0) {
                s->assembling[r->id] = 1;
                s->pending_asm.push_back(r);
            } else {
                auto it = s->objects.find(r->object);
                if (it != s->objects.end()) {
                    if ((int)r->p.size() != it->second->n) {
                        complete(s, r, SOD_ERR_INVALID_ARG);  // p, u must have the object's 3V entries
                        continue;
                    }
                    it->second->steps.push_back(r);
                    it->second->pending++;
                } else if (s->assembling.count(r->object)) {
                    s->early[r->object].push_back(r);
                } else {
                    complete(s, r, SOD_ERR_INVALID_ARG);  // unknown or evicted object
                }
            }
        }
        // finished assemblies: object known (steps may queue), ready once its bank is packed
        std::vector<AsmDone> fin;
        {
            std::lock_guard<std::mutex> g(s->asm_mu);
            fin.swap(s->asm_done);
        }
        for (auto &d : fin) {
            progress = true;
            Request *r = d.req;
            if (d.status != SOD_OK) {
                {
                    std::lock_guard<std::mutex> g(s->in_mu);
                    s->committed -= asm_temp_bytes(3 * r->nV, r->N) + bank_bytes(3 * r->nV, r->N);
                }
                s->assembling.erase(r->id);
                auto e = s->early.find(r->id);
                if (e != s->early.end()) {
                    for (Request *q : e->second) complete(s, q, d.status);
                    s->early.erase(e);
                }
                complete(s, r, d.status);
                continue;
            }
            auto o = std::make_unique<Object>();
            o->id = r->id;
            o->n = 3 * r->nV;
            o->bank = d.bank;
            o->bytes = d.bytes;
            o->last_use = Clock::now();
            auto e = s->early.find(r->id);
            if (e != s->early.end()) {
                for (Request *q : e->second) {
                    if ((int)q->p.size() == o->n)
                        o->steps.push_back(q);
                    else
                        complete(s, q, SOD_ERR_INVALID_ARG);  // length other than the object's 3V
                }
                o->pending = (int)o->steps.size();
                s->early.erase(e);
            }
            s->objects[o->id] = std::move(o);
            s->packing.push_back({d, r});
        }
        for (auto &sl : s->slots) {
            std::lock_guard<std::mutex> g(sl->mu);
            if (sl->busy && sl->job == nullptr) sl->busy = false;
        }
        // packed banks: assembly requests complete, objects become ready
        for (size_t k = 0; k < s->packing.size();) {
            auto &pk = s->packing[k];
            if (cudaEventQuery(pk.first.packed) == cudaSuccess) {
                cudaEventDestroy(pk.first.packed);
                Request *r = pk.second;
                auto it = s->objects.find(r->id);
                if (it != s->objects.end()) it->second->ready = true;
                s->assembling.erase(r->id);
                {
                    std::lock_guard<std::mutex> g(s->in_mu);
                    s->committed -= asm_temp_bytes(3 * r->nV, r->N);  // the bank stays committed
                }
                complete(s, r, SOD_OK);
                s->packing.erase(s->packing.begin() + k);
                progress = true;
            } else {
                k++;
            }
        }
        // finished steps
        for (size_t k = 0; k < s->ring.size(); k++) {
            StepSlot &st = s->ring[k];
            if (st.reqs.empty() || cudaEventQuery(st.ev) != cudaSuccess) continue;
            for (size_t g = 0; g < st.reqs.size(); g++) {
                Object *o = st.objs[g];
                st.reqs[g]->b.assign(st.hbuf + st.boff[g], st.hbuf + st.boff[g] + o->n);
                o->pending--;
                o->last_use = Clock::now();
                complete(s, st.reqs[g], SOD_OK);
            }
            st.reqs.clear();
            st.objs.clear();
            s->free_ring.push_back((int)k);
            progress = true;
        }
        // admission of assemblies: a free slot and room under the cap (evicting idle objects)
        while (!s->pending_asm.empty()) {
            sod_server::Slot *free_slot = nullptr;
            for (auto &sl : s->slots)
                if (!sl->busy) {
                    free_slot = sl.get();
                    break;
                }
            if (!free_slot) break;
            Request *r = s->pending_asm.front();
            const int64_t need = asm_temp_bytes(3 * r->nV, r->N) + bank_bytes(3 * r->nV, r->N);
            bool fits;
            for (;;) {
                {
                    std::lock_guard<std::mutex> g(s->in_mu);
                    fits = s->committed + need <= s->cap;
                }
                if (fits || !evict_one(s)) break;
            }
            if (!fits) {
                if (need > s->cap) {  // can never fit
                    s->pending_asm.pop_front();
                    complete(s, r, SOD_ERR_CAPACITY);
                    progress = true;
                    continue;
                }
                break;  // wait for memory
            }
            {
                std::lock_guard<std::mutex> g(s->in_mu);
                s->committed += need;
            }
            s->pending_asm.pop_front();
            {
                std::lock_guard<std::mutex> g(free_slot->mu);
                free_slot->busy = true;
                free_slot->job = r;
                free_slot->job_bytes = need;
            }
            free_slot->cv.notify_one();
            progress = true;
        }
        // dispatch steps of ready objects in groups: one step of each object with work per group (an
        // object's steps stay in arrival order: later groups run after earlier ones on the step stream)
        while (!s->free_ring.empty()) {
            std::vector<Object *> members;
            for (auto &kv : s->objects) {
                Object *o = kv.second.get();
                if (o->ready && !o->steps.empty()) members.push_back(o);
                if ((int)members.size() == HIST_GROUP_MAX) break;
            }
            if (members.empty()) break;
            const int k = s->free_ring.front();
            s->free_ring.pop_front();
            StepSlot &st = s->ring[k];
            size_t in = 0;
            for (Object *o : members) in += 2 * (size_t)o->n;
            std::vector<const double *> dp, du;
            std::vector<double *> db;
            std::vector<sod_history *> banks;
            size_t off = 0, bo = in;
            for (Object *o : members) {
                Request *r = o->steps.front();
                o->steps.pop_front();
                std::memcpy(st.hbuf + off, r->p.data(), sizeof(double) * o->n);
                std::memcpy(st.hbuf + off + o->n, r->u.data(), sizeof(double) * o->n);
                dp.push_back(st.dbuf + off);
                du.push_back(st.dbuf + off + o->n);
                db.push_back(st.dbuf + bo);
                banks.push_back(o->bank);
                st.reqs.push_back(r);
                st.objs.push_back(o);
                st.boff.resize(st.reqs.size());
                st.boff.back() = bo;
                off += 2 * (size_t)o->n;
                bo += o->n;
            }
            cudaStream_t ss = s->step_ctx->stream;
            int rc = cudaMemcpyAsync(st.dbuf, st.hbuf, sizeof(double) * in, cudaMemcpyHostToDevice, ss) == cudaSuccess
                         ? SOD_OK
                         : SOD_ERR_CUDA;
            if (rc == SOD_OK)
                rc = history_step_group(s->step_ctx, banks.data(), (int)banks.size(), dp.data(), du.data(), db.data());
            if (rc == SOD_OK && cudaMemcpyAsync(st.hbuf + in, st.dbuf + in, sizeof(double) * (bo - in),
                                                cudaMemcpyDeviceToHost, ss) != cudaSuccess)
                rc = SOD_ERR_CUDA;
            if (rc == SOD_OK && cudaEventRecord(st.ev, ss) != cudaSuccess) rc = SOD_ERR_CUDA;
            if (rc != SOD_OK) {
                for (size_t g = 0; g < st.reqs.size(); g++) {
                    st.objs[g]->pending--;
                    complete(s, st.reqs[g], rc);
                }
                st.reqs.clear();
                st.objs.clear();
                s->free_ring.push_back(k);
                continue;
            }
            progress = true;
        }
        if (!progress) std::this_thread::yield();
    }
}

}  // namespace

extern "C" {

// The server's device resources: the step context on the highest-priority stream, the staging
// ring and one context per assembly slot.  On failure the caller tears down what was made.
static int server_alloc(sod_server *s, int device, int slots) {
    SOD_TRY(sod_context_create(device, &s->step_ctx));
    {
        // time steps run on the device's highest-priority stream: the block scheduler hands them SMs
        // as soon as CTAs of the assembly kernels (regular grids, short CTAs) retire, instead of
        // queueing them behind whole assemblies
        int lo = 0, hi = 0;
        SOD_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        cudaStream_t hs = nullptr;
        SOD_CHECK_CUDA(cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, hi));
        const cudaError_t e = cudaStreamDestroy(s->step_ctx->own_stream);
        s->step_ctx->own_stream = s->step_ctx->stream = hs;
        SOD_CHECK_CUDA(e);
    }
    constexpr int RING = 6;  // groups in flight
    s->ring.resize(RING);
    const size_t gbytes = sizeof(double) * 3 * (size_t)s->vmax_n * HIST_GROUP_MAX;
    for (int k = 0; k < RING; k++) {
        StepSlot &st = s->ring[k];
        SOD_CHECK_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&st.hbuf), gbytes, cudaHostAllocDefault));
        SOD_CHECK_CUDA(cudaMalloc(reinterpret_cast<void **>(&st.dbuf), gbytes));
        SOD_CHECK_CUDA(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming));
        s->free_ring.push_back(k);
    }
    for (int k = 0; k < slots; k++) {
        s->slots.push_back(std::make_unique<sod_server::Slot>());
        SOD_TRY(sod_context_create(device, &s->slots.back()->ctx));
    }
    return SOD_OK;
}

int sod_server_create(int device, int64_t hbm_cap_bytes, int slots, int max_vertices, sod_server **out) {
    SOD_REQUIRE(out, "null output pointer");
    SOD_REQUIRE(hbm_cap_bytes > 0 && slots >= 1 && slots <= 8 && max_vertices >= 3,
                "need a positive HBM cap, 1..8 assembly slots and max_vertices >= 3");
    auto s = std::make_unique<sod_server>();
    s->device = device;
    s->cap = hbm_cap_bytes;
    s->vmax_n = 3 * max_vertices;
    const int rc = server_alloc(s.get(), device, slots);
    if (rc != SOD_OK) {  // no thread runs yet: the teardown frees whatever was made
        sod_server_destroy(s.release());
        return rc;
    }
    sod_server *raw = s.release();
    for (auto &sl : raw->slots) sl->th = std::thread(slot_main, raw, sl.get());
    raw->janitor = std::thread(janitor_main, raw);
    raw->scheduler = std::thread(scheduler_main, raw);
    *out = raw;
    return SOD_OK;
}

int sod_server_submit_assembly(sod_server *s, const double *V, int nV, const int *F, int nF, double E, double nu,
                               double rho, int bdf, double dt, int N, int order, int subdiv, int64_t *request_id) {
    SOD_REQUIRE(s && V && F && request_id, "null argument");
    SOD_REQUIRE(nV >= 3 && nV <= s->vmax_n / 3 && nF >= 1, "mesh size outside the server's limits");
    SOD_REQUIRE(E > 0 && rho > 0 && nu > -1.0 && nu < 0.5 && dt > 0 && N >= 1 && (bdf == 1 || bdf == 2),
                "bad material or time-stepping parameters");
    auto *r = new Request();
    r->id = s->next_id++;
    r->type = 0;
    r->V.assign(V, V + 3 * (size_t)nV);
    r->F.assign(F, F + 3 * (size_t)nF);
    r->nV = nV, r->nF = nF, r->E = E, r->nu = nu, r->rho = rho, r->bdf = bdf, r->dt = dt, r->N = N;
    r->order = order, r->subdiv = subdiv;
    *request_id = r->id;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->in_mu);
        s->inbox.push_back(r);
        s->submitted++;
    }
    s->in_cv.notify_all();
    return SOD_OK;
}

int sod_server_submit_step(sod_server *s, int64_t object_id, const double *p, const double *u, int n,
                           int64_t *request_id) {
    SOD_REQUIRE(s && p && u && request_id, "null argument");
    SOD_REQUIRE(n >= 9 && n <= s->vmax_n, "vector length outside the server's limits");
    auto *r = new Request();
    r->id = s->next_id++;
    r->type = 1;
    r->object = object_id;
    r->p.assign(p, p + n);
    r->u.assign(u, u + n);
    *request_id = r->id;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->in_mu);
        s->inbox.push_back(r);
        s->submitted++;
    }
    s->in_cv.notify_all();
    return SOD_OK;
}

int sod_server_poll(sod_server *s, int64_t *ids, int *status, int64_t *latency_ns, int cap, int *n) {
    SOD_REQUIRE(s && n && (cap == 0 || (ids && status && latency_ns)), "null argument");
    std::lock_guard<std::mutex> g(s->out_mu);
    int k = 0;
    while (k < cap && !s->done.empty()) {
        const auto d = s->done.front();
        s->done.pop_front();
        ids[k] = d.id, status[k] = d.status, latency_ns[k] = d.ns;
        k++;
    }
    *n = k;
    return SOD_OK;
}

int sod_server_result(sod_server *s, int64_t request_id, double *b, int n) {
    SOD_REQUIRE(s && b, "null argument");
    std::lock_guard<std::mutex> g(s->out_mu);
    auto it = s->results.find(request_id);
    SOD_REQUIRE(it != s->results.end(), "no result for this request (not a completed step)");
    SOD_REQUIRE((int)it->second.size() == n, "result length mismatch");
    std::memcpy(b, it->second.data(), sizeof(double) * n);
    s->results.erase(it);
    return SOD_OK;
}

int sod_server_drain(sod_server *s, double timeout_s) {
    SOD_REQUIRE(s, "null server");
    std::unique_lock<std::mutex> g(s->out_mu);
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
    for (;;) {
        int64_t sub;
        {
            std::lock_guard<std::mutex> gi(s->in_mu);
            sub = s->submitted;
        }
        if (s->completed_count >= sub) return SOD_OK;
        if (s->out_cv.wait_until(g, deadline) == std::cv_status::timeout) {
            set_error("server drain timed out");
            return SOD_ERR_TIMEOUT;
        }
    }
}

int sod_server_stats(sod_server *s, int64_t *committed_bytes, int *resident_objects) {
    SOD_REQUIRE(s, "null server");
    {
        std::lock_guard<std::mutex> g(s->in_mu);
        if (committed_bytes) *committed_bytes = s->committed;
    }
    if (resident_objects) *resident_objects = -1;  // owned by the scheduler thread; not sampled here
    return SOD_OK;
}

int sod_server_destroy(sod_server *s) {
    if (!s) return SOD_OK;
    s->stop = true;
    s->in_cv.notify_all();
    if (s->scheduler.joinable()) s->scheduler.join();
    for (auto &sl : s->slots) {
        sl->cv.notify_all();
        if (sl->th.joinable()) sl->th.join();
    }
    // remaining objects go to the janitor, then it exits
    {
        std::lock_guard<std::mutex> g(s->jan_mu);
        for (auto &kv : s->objects) s->trash.push_back({kv.second->bank, kv.second->bytes});
        s->objects.clear();
    }
    s->jan_cv.notify_all();
    if (s->janitor.joinable()) s->janitor.join();
    cudaSetDevice(s->device);
    if (s->step_ctx) cudaStreamSynchronize(s->step_ctx->stream);
    for (auto &st : s->ring) {  // also a partly made server (sod_server_create's failure path)
        if (st.hbuf) cudaFreeHost(st.hbuf);
        if (st.dbuf) cudaFree(st.dbuf);
        if (st.ev) cudaEventDestroy(st.ev);
    }
    for (auto &sl : s->slots) sod_context_destroy(sl->ctx);
    sod_context_destroy(s->step_ctx);
    delete s;
    return SOD_OK;
}

}  // extern "C"
