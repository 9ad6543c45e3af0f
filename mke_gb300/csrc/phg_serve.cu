// phg_serve.cu -- request loop with continuous batching over the sphere
// operators (host code; no reference counterpart: the reference has no
// serving layer, its drivers call the classes directly).
//
// Requests are Laplace solves and short barotropic integrations on
// icosahedral meshes of mixed levels.  Each (kind, level) gets a lane: its own
// operator handles, CUDA stream and host thread, and `cap` member slots whose
// device memory is reserved when the lane opens and counted against the HBM
// budget.  Requests join a lane as slots free up: a barotropic member enters
// between two time steps and leaves after its last one, while the others keep
// stepping; Laplace solves go into the lane's next batched solve.  Lanes run
// concurrently on their streams, so work of different levels overlaps on the
// device.  A lane that cannot get memory evicts idle lanes; a request whose
// lane can never fit in the budget completes with PHG_ERR_BUDGET.
//
// The solver runs as persistent cooperative launches whose blocks must all be
// resident at once.  Lanes therefore take SMs from a shared pool for each
// launch sequence (one time step, one batched solve): a lane alone gets what
// its work can fill, lanes running together get equal shares, and the SMs of
// concurrent launches never add up to more than the GPU has.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/phelm_gb300.h"
#include "phg_api.hpp"

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
    phg_request r;
    double t_submit = 0.0, t_admit = 0.0;
    int steps_left = 0;
};

struct Server;

// One mesh level of a packed Laplace lane: its handle and member slots.
struct Sub {
    int level = 0;
    phg_ops ops = nullptr;
    int V = 0, os = 0, osb = 1, cap = 0;
    long long bytes = 0;     // budget held for this level
    double last_used = 0;    // server time of its last turn
    double *dU = nullptr, *dOut = nullptr, *dB = nullptr;
    double *hIn = nullptr, *hOut = nullptr, *hB = nullptr;
};

struct Lane {
    Server *srv = nullptr;
    int kind = 0, level = 0;
    // packed Laplace lane: the solves of every level up to Server::pack_level
    // go into one multi-level launch per turn (level = 0, one Sub per level met)
    bool packed = false;
    std::vector<std::unique_ptr<Sub>> subs;
    std::vector<int> want;        // levels to open ahead of traffic (under Server::mu)
    std::vector<int> opened;      // levels whose Sub is ready (under Server::mu)
    // device resources, owned by the lane thread
    phg_ops ops = nullptr;
    phg_barvortex bv = nullptr;
    cudaStream_t stream = nullptr;
    int V = 0, os = 0, osb = 1, cap = 0;
    double *dU = nullptr, *dOut = nullptr, *dB = nullptr, *dBw = nullptr;
    double *hIn = nullptr, *hOut = nullptr, *hB = nullptr;
    long long bytes = 0;   // reserved against the budget
    double step_ms = 0.0;  // barotropic lanes: wall time of the last call, per step
    // shared state, under Server::mu
    std::deque<Pending *> queue;
    std::vector<Pending *> act;   // members in flight, act[k] owns slot k (lane thread only)
    bool ready = false, failed = false, stop = false, closing = false, closed = false;
    int fail_status = PHG_OK;
    std::string fail_msg;
    int active = 0;
    double last_busy = 0.0;
    std::condition_variable cv;
    std::thread th;
};

struct Server {
    phg_serve_conf conf{};
    int dev = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable done_cv, mem_cv, ready_cv;
    std::map<std::pair<int, int>, Lane *> lanes;   // current lane per (kind, level)
    std::vector<std::unique_ptr<Lane>> all;        // every lane ever opened (joined at destroy)
    std::deque<phg_completion> done;
    long long budget = 0, in_use = 0, ndone = 0;
    bool shutting = false;
    int sm_total = 0, sm_free = 0, sm_users = 0;   // SM pool (under mu)
    std::condition_variable sm_cv;
    std::mutex mesh_mu;
    std::map<int, phg_mesh> meshes;
    int pack_level = 0;   // Laplace requests of levels <= this share one lane and one launch per turn
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

// under S->mu; the message is the calling thread's last library error
void push_done(Server *S, Pending *p, int status, int batch, const char *msg = nullptr) {
    phg_completion c;
    memset(&c, 0, sizeof(c));
    if (status != PHG_OK) {
        const char *m = msg ? msg : phg_last_error();
        strncpy(c.error, m ? m : "", sizeof(c.error) - 1);
    }
    c.tag = p->r.tag;
    c.status = status;
    c.kind = p->r.kind;
    c.level = p->r.level;
    c.t_submit = p->t_submit;
    c.t_admit = p->t_admit;
    c.t_done = S->now();
    c.batch = batch;
    S->done.push_back(c);
    S->ndone++;
    delete p;
    S->done_cv.notify_all();
}

int get_mesh(Server *S, int level, phg_mesh *out) {
    std::lock_guard<std::mutex> lk(S->mesh_mu);
    auto it = S->meshes.find(level);
    if (it != S->meshes.end()) { *out = it->second; return PHG_OK; }
    phg_mesh m = nullptr;
    int r = phg_mesh_generate(level, &m);
    if (r) return r;
    S->meshes[level] = m;
    *out = m;
    return PHG_OK;
}

long long thread_bytes() {
    long long t = 0;
    phg_device_bytes(nullptr, &t);
    return t;
}

// SMs the lane's launches can fill: the largest solve of one call has
// rows x right-hand sides work items, two blocks of 256 rows per SM
int natural_sms(const Lane *L, int nv) {
    const long long rows = (long long)(L->V - L->os) * nv * (L->kind == PHG_REQ_BARVORTEX ? 8 : 1);
    return (int)std::max(1LL, std::min<long long>(L->srv->sm_total, (rows + 511) / 512));
}

// take SMs from the pool: at most the fair share of the lanes now using it
int sm_acquire(Server *S, int want) {
    std::unique_lock<std::mutex> lk(S->mu);
    S->sm_users++;
    int grant = 0;
    for (;;) {
        const int fair = std::max(1, S->sm_total / S->sm_users);
        grant = std::min(want, fair);
        if (S->sm_free >= grant) break;
        S->sm_cv.wait(lk);
    }
    S->sm_free -= grant;
    return grant;
}

void sm_release(Server *S, int grant) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->sm_free += grant;
    S->sm_users--;
    S->sm_cv.notify_all();
}

// one call of the lane's kernel work on members [0, nv) of the slot buffers
int lane_run(Lane *L, int nv) {
    Server *S = L->srv;
    const int grant = sm_acquire(S, natural_sms(L, nv));
    int r = phg_ops_set_sms(L->ops, grant);
    if (r == PHG_OK) {
        if (L->kind == PHG_REQ_LAPLACE_SOLVE)
            r = phg_laplace_solve_batch(L->ops, nv, L->dOut, L->dU, L->os ? L->dB : nullptr, L->stream);
        else
            r = phg_barvortex_calc_batch(L->bv, nv, L->dU, L->dU, L->os ? L->dB : nullptr,
                                         L->os ? L->dBw : nullptr, nullptr, L->stream);
    }
    int r2 = phg_ops_check(L->ops, L->stream);   // waits for the launches
    sm_release(S, grant);
    return r ? r : r2;
}

// `steps` time steps of the barotropic members [0, nv) in one call: the step
// captured as a CUDA graph (one per member count, kept by the handle) and
// replayed, then one synchronisation that checks every step's solves
int lane_steps(Lane *L, int nv, int steps) {
    Server *S = L->srv;
    const int grant = sm_acquire(S, natural_sms(L, nv));
    int r = phg_ops_set_sms(L->ops, grant);
    if (r == PHG_OK)
        r = phg_barvortex_run(L->bv, nv, steps, L->dU, L->os ? L->dB : nullptr, L->os ? L->dBw : nullptr, nullptr,
                              L->stream);
    int r2 = phg_barvortex_last_stats(L->bv, nullptr, nullptr, nullptr, nullptr, nullptr);   // waits, checks
    sm_release(S, grant);
    return r ? r : r2;
}

void free_slots(Lane *L) {
    cudaFree(L->dU); cudaFree(L->dOut); cudaFree(L->dB); cudaFree(L->dBw);
    cudaFreeHost(L->hIn); cudaFreeHost(L->hOut); cudaFreeHost(L->hB);
    L->dU = L->dOut = L->dB = L->dBw = nullptr;
    L->hIn = L->hOut = L->hB = nullptr;
}

int alloc_slots(Lane *L, int n) {
    const size_t v = (size_t)L->V * n * 8, b = (size_t)L->osb * n * 8;
    if (cudaMalloc(&L->dU, v) || cudaMalloc(&L->dB, b) || cudaMalloc(&L->dBw, b) ||
        (L->kind == PHG_REQ_LAPLACE_SOLVE && cudaMalloc(&L->dOut, v)) ||
        cudaHostAlloc(&L->hIn, v, cudaHostAllocDefault) || cudaHostAlloc(&L->hOut, v, cudaHostAllocDefault) ||
        cudaHostAlloc(&L->hB, b, cudaHostAllocDefault)) {
        cudaGetLastError();
        free_slots(L);
        return PHG_ERR_CUDA;
    }
    cudaMemset(L->dU, 0, v);
    cudaMemset(L->dB, 0, b);
    cudaMemset(L->dBw, 0, b);
    return PHG_OK;
}

long long slot_bytes(const Lane *L) {
    return (long long)L->V * 8 * (L->kind == PHG_REQ_LAPLACE_SOLVE ? 2 : 1) + (long long)L->osb * 8 * 2;
}

// Reserve base + cap x per bytes of the HBM budget for a lane (cap lowered to
// what fits), evicting idle lanes and waiting for their memory when needed;
// held receives the reservation.
int reserve(Lane *L, long long base, long long per, int &cap, long long &held) {
    Server *S = L->srv;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        for (;;) {
            const long long freeb = S->budget - S->in_use;
            const long long fit = per > 0 ? (freeb - base) / per : cap;
            if (fit >= 1) {
                cap = (int)std::min<long long>(cap, fit);
                break;
            }
            if (base + per > S->budget) return PHG_ERR_BUDGET;   // never fits
            // evict idle lanes, then wait for their memory
            bool any = false;
            for (auto &kv : S->lanes) {
                Lane *o = kv.second;
                if (o != L && o->ready && !o->stop && o->active == 0 && o->queue.empty()) {
                    o->stop = true;
                    o->cv.notify_all();
                    any = true;
                }
            }
            bool busy = false;
            for (auto &kv : S->lanes) busy |= kv.second != L && !kv.second->closed;
            if (!any && !busy) return PHG_ERR_BUDGET;
            if (S->shutting) return PHG_ERR_BUDGET;
            S->mem_cv.wait_for(lk, std::chrono::milliseconds(50));
        }
        held = base + (long long)cap * per;
        S->in_use += held;
    }
    return PHG_OK;
}

// Build the handles, size the slots from two probe calls, reserve the budget
// and allocate everything the lane will use.
int lane_open(Lane *L) {
    Server *S = L->srv;
    const phg_serve_conf &c = S->conf;
    if (L->packed) {   // the per-level handles open with their first requests
        if (cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess) return PHG_ERR_CUDA;
        return PHG_OK;
    }
    phg_mesh m = nullptr;
    int r = get_mesh(S, L->level, &m);
    if (r) return r;
    int T = 0, rs = 0;
    if ((r = phg_mesh_info(m, &L->V, &T, &rs, &L->os))) return r;
    L->osb = std::max(L->os, 1);
    const long long b0 = thread_bytes();
    if ((r = phg_ops_create(m, c.precision, &L->ops))) return r;
    const double tol = L->kind == PHG_REQ_LAPLACE_SOLVE ? c.solve_tol : c.step_tol;
    if ((r = phg_ops_set_solver(L->ops, 30, tol, 20000))) return r;
    if (cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess) return PHG_ERR_CUDA;
    if (L->kind == PHG_REQ_BARVORTEX) {
        // l + h = sin(latitude) in the zone-0 chart (2 Omega = 1, no orography)
        std::vector<double> uv((size_t)L->V * 8), lh(L->V);
        if ((r = phg_mesh_arrays(m, nullptr, uv.data(), nullptr, nullptr, nullptr))) return r;
        for (int p = 0; p < L->V; ++p) lh[p] = std::sin(uv[(size_t)p * 8]);
        if ((r = phg_barvortex_create(L->ops, &c.bv, lh.data(), &L->bv))) return r;
    }
    // probes: device bytes of the handles at 1 and 2 members
    if ((r = alloc_slots(L, 2))) return r;
    if ((r = lane_run(L, 1))) return r;
    const long long b1 = thread_bytes() - b0;
    if ((r = lane_run(L, 2))) return r;
    const long long b2 = thread_bytes() - b0;
    free_slots(L);
    const long long per = std::max(0LL, b2 - b1) + slot_bytes(L);
    const long long base = b1 - (b2 - b1);
    int cap = c.max_slots > 0 ? c.max_slots : 64;
    long long held = 0;
    if ((r = reserve(L, base, per, cap, held))) return r;
    L->bytes += held;
    L->cap = cap;
    if ((r = alloc_slots(L, cap))) return r;
    if ((r = lane_run(L, cap))) return r;   // allocate every workspace now
    // keep the reservation honest: what the handles really hold
    const long long actual = thread_bytes() - b0 + (long long)cap * slot_bytes(L);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->in_use += actual - L->bytes;
        L->bytes = actual;
    }
    return PHG_OK;
}

void sub_free(Sub *u) {
    cudaFree(u->dU); cudaFree(u->dOut); cudaFree(u->dB);
    cudaFreeHost(u->hIn); cudaFreeHost(u->hOut); cudaFreeHost(u->hB);
    u->dU = u->dOut = u->dB = nullptr;
    u->hIn = u->hOut = u->hB = nullptr;
}

int sub_alloc(Sub *u, int n) {
    const size_t v = (size_t)u->V * n * 8, b = (size_t)u->osb * n * 8;
    if (cudaMalloc(&u->dU, v) || cudaMalloc(&u->dOut, v) || cudaMalloc(&u->dB, b) ||
        cudaHostAlloc(&u->hIn, v, cudaHostAllocDefault) || cudaHostAlloc(&u->hOut, v, cudaHostAllocDefault) ||
        cudaHostAlloc(&u->hB, b, cudaHostAllocDefault)) {
        cudaGetLastError();
        sub_free(u);
        return PHG_ERR_CUDA;
    }
    cudaMemset(u->dB, 0, b);
    return PHG_OK;
}

// one batched solve of n members of a packed lane's level alone (the
// probes that size its memory)
int sub_probe(Lane *L, Sub *u, int n) {
    int r = phg_laplace_solve_batch(u->ops, n, u->dOut, u->dU, u->os ? u->dB : nullptr, L->stream);
    int r2 = phg_ops_check(u->ops, L->stream);
    return r ? r : r2;
}

int sub_open_(Lane *L, int level, Sub **out, const std::vector<Sub *> &busy);

// close a level of a packed lane and give its budget back
void sub_close(Lane *L, size_t i) {
    Server *S = L->srv;
    Sub *u = L->subs[i].get();
    if (L->stream) cudaStreamSynchronize(L->stream);
    if (u->ops) phg_ops_destroy(u->ops);
    sub_free(u);
    cudaGetLastError();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->in_use -= u->bytes;
        L->bytes -= u->bytes;
        S->mem_cv.notify_all();
    }
    L->subs.erase(L->subs.begin() + (long)i);
}

// open a level of a packed Laplace lane: handle, probes, budget, slots; a
// level that fails to open leaves no Sub behind (its reservation stays with
// the lane until it closes)
int sub_open(Lane *L, int level, Sub **out, const std::vector<Sub *> &busy) {
    const size_t n0 = L->subs.size();
    const int r = sub_open_(L, level, out, busy);
    if (r && L->subs.size() > n0) sub_close(L, L->subs.size() - 1);
    return r;
}

int sub_open_(Lane *L, int level, Sub **out, const std::vector<Sub *> &busy) {
    Server *S = L->srv;
    const phg_serve_conf &c = S->conf;
    auto u = std::make_unique<Sub>();
    u->level = level;
    phg_mesh m = nullptr;
    int r = get_mesh(S, level, &m);
    if (r) return r;
    int T = 0, rs = 0;
    if ((r = phg_mesh_info(m, &u->V, &T, &rs, &u->os))) return r;
    u->osb = std::max(u->os, 1);
    const long long b0 = thread_bytes();
    if ((r = phg_ops_create(m, c.precision, &u->ops))) return r;
    Sub *raw = u.get();
    L->subs.push_back(std::move(u));   // closed with the lane from here on
    if ((r = phg_ops_set_solver(raw->ops, 30, c.solve_tol, 20000))) return r;
    if ((r = sub_alloc(raw, 2))) return r;
    cudaMemset(raw->dU, 0, (size_t)raw->V * 2 * 8);
    if ((r = sub_probe(L, raw, 1))) return r;
    const long long b1 = thread_bytes() - b0;
    if ((r = sub_probe(L, raw, 2))) return r;
    const long long b2 = thread_bytes() - b0;
    sub_free(raw);
    const long long slot = (long long)raw->V * 16 + (long long)raw->osb * 8;
    const long long per = std::max(0LL, b2 - b1) + slot;
    const long long base = b1 - (b2 - b1);
    int cap = c.max_slots > 0 ? c.max_slots : 64;
    long long held = 0;
    // when the budget is short, the lane's idle levels (least recently used
    // first) make room before other lanes are waited for
    while ((r = reserve(L, base, per, cap, held)) == PHG_ERR_BUDGET) {
        size_t victim = L->subs.size();
        for (size_t i = 0; i < L->subs.size(); ++i) {
            Sub *x = L->subs[i].get();
            if (x == raw || std::find(busy.begin(), busy.end(), x) != busy.end()) continue;
            if (victim == L->subs.size() || x->last_used < L->subs[victim]->last_used) victim = i;
        }
        if (victim == L->subs.size()) return r;
        sub_close(L, victim);
    }
    if (r) return r;
    L->bytes += held;
    raw->bytes = held;
    raw->cap = cap;
    if ((r = sub_alloc(raw, cap))) return r;
    cudaMemset(raw->dU, 0, (size_t)raw->V * cap * 8);
    if ((r = sub_probe(L, raw, cap))) return r;
    const long long actual = thread_bytes() - b0 + (long long)cap * slot;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->in_use += actual - held;
        L->bytes += actual - held;
        raw->bytes = actual;
    }
    *out = raw;
    return PHG_OK;
}

void lane_close(Lane *L) {
    Server *S = L->srv;
    if (L->stream) cudaStreamSynchronize(L->stream);
    for (auto &u : L->subs) {
        if (u->ops) phg_ops_destroy(u->ops);
        u->ops = nullptr;
        sub_free(u.get());
    }
    L->subs.clear();
    if (L->bv) phg_barvortex_destroy(L->bv);
    if (L->ops) phg_ops_destroy(L->ops);
    L->bv = nullptr;
    L->ops = nullptr;
    free_slots(L);
    if (L->stream) cudaStreamDestroy(L->stream);
    L->stream = nullptr;
    std::lock_guard<std::mutex> lk(S->mu);
    S->in_use -= L->bytes;
    L->bytes = 0;
    L->closed = true;
    // requests that raced with the close go to a fresh lane on next submit;
    // any left here are failed rather than lost
    while (!L->queue.empty()) {
        push_done(S, L->queue.front(), L->failed ? L->fail_status : PHG_ERR_BUDGET, 0,
                  L->failed ? L->fail_msg.c_str() : "lane closed");
        L->queue.pop_front();
    }
    S->mem_cv.notify_all();
    S->ready_cv.notify_all();
}

void laplace_loop(Lane *L) {
    Server *S = L->srv;
    const int V = L->V, os = L->os;
    std::vector<Pending *> &batch = L->act;
    for (;;) {
        batch.clear();
        {
            std::unique_lock<std::mutex> lk(S->mu);
            L->cv.wait(lk, [&] { return L->stop || !L->queue.empty(); });
            if (L->queue.empty()) { L->closing = true; return; }
            while (!L->queue.empty() && (int)batch.size() < L->cap) {
                batch.push_back(L->queue.front());
                L->queue.pop_front();
            }
            L->active = (int)batch.size();
        }
        const int n = (int)batch.size();
        const double ta = S->now();
        for (int k = 0; k < n; ++k) {
            Pending *p = batch[k];
            p->t_admit = ta;
            memcpy(L->hIn + (size_t)k * V, p->r.input, 8 * (size_t)V);
            if (os) {
                if (p->r.bnd) memcpy(L->hB + (size_t)k * os, p->r.bnd, 8 * (size_t)os);
                else memset(L->hB + (size_t)k * os, 0, 8 * (size_t)os);
            }
        }
        int st = PHG_OK;
        if (cudaMemcpyAsync(L->dU, L->hIn, 8 * (size_t)V * n, cudaMemcpyHostToDevice, L->stream) ||
            (os && cudaMemcpyAsync(L->dB, L->hB, 8 * (size_t)os * n, cudaMemcpyHostToDevice, L->stream)))
            st = PHG_ERR_CUDA;
        if (!st) st = lane_run(L, n);
        if (!st && (cudaMemcpyAsync(L->hOut, L->dOut, 8 * (size_t)V * n, cudaMemcpyDeviceToHost, L->stream) ||
                    cudaStreamSynchronize(L->stream)))
            st = PHG_ERR_CUDA;
        for (int k = 0; k < n; ++k)
            if (!st) memcpy(batch[k]->r.output, L->hOut + (size_t)k * V, 8 * (size_t)V);
        std::lock_guard<std::mutex> lk(S->mu);
        for (int k = 0; k < n; ++k) push_done(S, batch[k], st, n);
        batch.clear();
        L->active = 0;
        L->last_busy = S->now();
    }
}

// A packed Laplace lane: every turn takes the queued requests of all its
// levels (up to each level's slots) and solves them in ONE multi-level
// persistent launch (phg_laplace_solve_levels): groups of blocks take
// right-hand sides of any level, so small meshes share the GPU instead of
// each holding a launch.
void packed_loop(Lane *L) {
    Server *S = L->srv;
    const int maxs = S->conf.max_slots > 0 ? S->conf.max_slots : 64;
    std::vector<Pending *> batch;
    for (;;) {
        batch.clear();
        std::vector<int> open_now;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            L->cv.wait(lk, [&] { return L->stop || !L->queue.empty() || !L->want.empty(); });
            open_now.swap(L->want);
        }
        for (int lv : open_now) {   // levels preloaded ahead of traffic
            bool have = false;
            for (auto &u : L->subs) have |= u->level == lv;
            Sub *u = nullptr;
            const int r = have ? PHG_OK : sub_open(L, lv, &u, {});
            std::lock_guard<std::mutex> lk(S->mu);
            L->opened.push_back(r ? -lv : lv);   // -lv: the level failed to open
            S->ready_cv.notify_all();
        }
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (L->queue.empty()) {
                if (L->stop) { L->closing = true; return; }
                continue;
            }
            std::map<int, int> per;
            std::deque<Pending *> keep;
            while (!L->queue.empty()) {
                Pending *p = L->queue.front();
                L->queue.pop_front();
                int cap = maxs;
                for (auto &u : L->subs)
                    if (u->level == p->r.level) cap = u->cap;
                if (per[p->r.level] < cap) { per[p->r.level]++; batch.push_back(p); }
                else keep.push_back(p);
            }
            L->queue.swap(keep);
            L->active = (int)batch.size();
        }
        const double ta = S->now();
        // the levels of this turn, opened on first use
        std::vector<Sub *> used;
        std::vector<std::vector<Pending *>> mem;
        std::vector<Pending *> later;   // beyond the slots of a level opened this turn
        int st = PHG_OK;
        for (Pending *p : batch) {
            p->t_admit = ta;
            size_t k = 0;
            while (k < used.size() && used[k]->level != p->r.level) ++k;
            if (k == used.size()) {
                Sub *u = nullptr;
                for (auto &x : L->subs)
                    if (x->level == p->r.level) u = x.get();
                if (!u) {
                    const int r = sub_open(L, p->r.level, &u, used);
                    if (r) { std::lock_guard<std::mutex> lk(S->mu); push_done(S, p, r, 0); continue; }
                }
                used.push_back(u);
                mem.emplace_back();
            }
            if ((int)mem[k].size() < used[k]->cap) mem[k].push_back(p);
            else later.push_back(p);
        }
        if (!later.empty()) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (auto it = later.rbegin(); it != later.rend(); ++it) L->queue.push_front(*it);
            L->active -= (int)later.size();
        }
        const int nseg = (int)used.size();
        std::vector<phg_ops> ops(nseg);
        std::vector<int> nv(nseg);
        std::vector<double *> ans(nseg), bnd(nseg);
        std::vector<const double *> F(nseg);
        long long rows = 0;
        for (int k = 0; k < nseg && !st; ++k) {
            Sub *u = used[k];
            const int n = (int)mem[k].size();
            for (int j = 0; j < n; ++j) {
                Pending *p = mem[k][j];
                memcpy(u->hIn + (size_t)j * u->V, p->r.input, 8 * (size_t)u->V);
                if (u->os) {
                    if (p->r.bnd) memcpy(u->hB + (size_t)j * u->os, p->r.bnd, 8 * (size_t)u->os);
                    else memset(u->hB + (size_t)j * u->os, 0, 8 * (size_t)u->os);
                }
            }
            if (cudaMemcpyAsync(u->dU, u->hIn, 8 * (size_t)u->V * n, cudaMemcpyHostToDevice, L->stream) ||
                (u->os && cudaMemcpyAsync(u->dB, u->hB, 8 * (size_t)u->os * n, cudaMemcpyHostToDevice, L->stream)))
                st = PHG_ERR_CUDA;
            ops[k] = u->ops; nv[k] = n; ans[k] = u->dOut; F[k] = u->dU; bnd[k] = u->os ? u->dB : nullptr;
            rows += (long long)(u->V - u->os) * n;
        }
        if (!st && nseg > 0) {
            const int want = (int)std::max(1LL, std::min<long long>(S->sm_total, (rows + 511) / 512));
            const int grant = sm_acquire(S, want);
            const long long b0 = thread_bytes();
            st = phg_ops_set_sms(ops[0], grant);
            if (!st) st = phg_laplace_solve_levels(nseg, ops.data(), nv.data(), ans.data(), F.data(), bnd.data(),
                                                   L->stream);
            const int r2 = phg_ops_check(ops[0], L->stream);
            sm_release(S, grant);
            if (!st) st = r2;
            const long long grown = thread_bytes() - b0;   // the multi-level workspace, first of its size
            if (grown > 0) {   // held by the first level's handle
                std::lock_guard<std::mutex> lk(S->mu);
                S->in_use += grown;
                L->bytes += grown;
                used[0]->bytes += grown;
            }
            for (Sub *u : used) u->last_used = S->now();
        }
        for (int k = 0; k < nseg && !st; ++k)
            if (cudaMemcpyAsync(used[k]->hOut, used[k]->dOut, 8 * (size_t)used[k]->V * nv[k], cudaMemcpyDeviceToHost,
                                L->stream))
                st = PHG_ERR_CUDA;
        if (!st && cudaStreamSynchronize(L->stream)) st = PHG_ERR_CUDA;
        int total = 0;
        for (int k = 0; k < nseg; ++k) total += nv[k];
        std::lock_guard<std::mutex> lk(S->mu);
        for (int k = 0; k < nseg; ++k)
            for (int j = 0; j < nv[k]; ++j) {
                Pending *p = mem[k][j];
                if (!st) memcpy(p->r.output, used[k]->hOut + (size_t)j * used[k]->V, 8 * (size_t)used[k]->V);
                push_done(S, p, st, total);
            }
        L->active = 0;
        L->last_busy = S->now();
    }
}

void bv_loop(Lane *L) {
    Server *S = L->srv;
    const int V = L->V, os = L->os;
    std::vector<Pending *> &act = L->act;
    std::vector<int> fin;
    for (;;) {
        int n0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (act.empty()) {
                L->cv.wait(lk, [&] { return L->stop || !L->queue.empty(); });
                if (L->queue.empty()) { L->closing = true; return; }
            }
            n0 = (int)act.size();
            while (!L->queue.empty() && (int)act.size() < L->cap) {
                act.push_back(L->queue.front());
                L->queue.pop_front();
            }
            L->active = (int)act.size();
        }
        const int n = (int)act.size();
        const double ta = S->now();
        int st = PHG_OK;
        for (int k = n0; k < n && !st; ++k) {
            Pending *p = act[k];
            p->t_admit = ta;
            p->steps_left = p->r.steps;
            memcpy(L->hIn + (size_t)k * V, p->r.input, 8 * (size_t)V);
            if (cudaMemcpyAsync(L->dU + (size_t)k * V, L->hIn + (size_t)k * V, 8 * (size_t)V, cudaMemcpyHostToDevice,
                                L->stream))
                st = PHG_ERR_CUDA;
            if (os) {
                if (p->r.bnd) memcpy(L->hB + (size_t)k * os, p->r.bnd, 8 * (size_t)os);
                else memset(L->hB + (size_t)k * os, 0, 8 * (size_t)os);
                if (cudaMemcpyAsync(L->dB + (size_t)k * os, L->hB + (size_t)k * os, 8 * (size_t)os,
                                    cudaMemcpyHostToDevice, L->stream))
                    st = PHG_ERR_CUDA;
            }
        }
        // A full lane (no request could join before a member leaves) runs up
        // to the nearest finish in one call, from the captured step graph; a
        // lane with free slots steps once, so that requests arriving meanwhile
        // join at the next step.  A call keeps its SM grant until it returns,
        // so runs are capped at RUN_MS: a long run on a share granted while
        // other lanes were busy would leave the SMs they free idle.
        constexpr double RUN_MS = 20.0;
        int ksteps = 1;
        if (n >= L->cap && L->step_ms > 0.0) {
            ksteps = act[0]->steps_left;
            for (int k = 1; k < n; ++k) ksteps = std::min(ksteps, act[k]->steps_left);
            ksteps = std::max(1, std::min(ksteps, (int)(RUN_MS / L->step_ms)));
        }
        const auto t_run = Clock::now();
        if (!st) st = ksteps > 1 ? lane_steps(L, n, ksteps) : lane_run(L, n);
        L->step_ms = std::chrono::duration<double, std::milli>(Clock::now() - t_run).count() / ksteps;
        if (st) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (Pending *p : act) push_done(S, p, st, n);
            act.clear();
            L->active = 0;
            continue;
        }
        fin.clear();
        for (int k = n - 1; k >= 0; --k)
            if ((act[k]->steps_left -= std::max(1, ksteps)) <= 0) {
                fin.push_back(k);
                if (cudaMemcpyAsync(L->hOut + (size_t)k * V, L->dU + (size_t)k * V, 8 * (size_t)V,
                                    cudaMemcpyDeviceToHost, L->stream))
                    st = PHG_ERR_CUDA;
            }
        if (fin.empty()) continue;
        if (cudaStreamSynchronize(L->stream)) st = PHG_ERR_CUDA;
        std::vector<std::pair<Pending *, int>> out;
        for (int k : fin) {   // descending: slots above k are live members
            Pending *p = act[k];
            if (!st) memcpy(p->r.output, L->hOut + (size_t)k * V, 8 * (size_t)V);
            out.push_back({p, st});
            const int last = (int)act.size() - 1;
            if (k != last) {
                cudaMemcpyAsync(L->dU + (size_t)k * V, L->dU + (size_t)last * V, 8 * (size_t)V,
                                cudaMemcpyDeviceToDevice, L->stream);
                if (os)
                    cudaMemcpyAsync(L->dB + (size_t)k * os, L->dB + (size_t)last * os, 8 * (size_t)os,
                                    cudaMemcpyDeviceToDevice, L->stream);
                act[k] = act[last];
            }
            act.pop_back();
        }
        std::lock_guard<std::mutex> lk(S->mu);
        for (auto &x : out) push_done(S, x.first, x.second, n);
        L->active = (int)act.size();
        L->last_busy = S->now();
    }
}

// A C++ exception inside a lane (host memory exhausted) fails the lane and the
// requests it holds instead of ending the process; queued ones fail at close.
void lane_abort(Lane *L) {
    Server *S = L->srv;
    phg::api_exception();
    std::lock_guard<std::mutex> lk(S->mu);
    L->failed = true;
    L->fail_status = PHG_ERR_HOST;
    L->fail_msg = phg_last_error();
    L->closing = true;
    for (Pending *p : L->act) push_done(S, p, PHG_ERR_HOST, 0, L->fail_msg.c_str());
    L->act.clear();
    L->active = 0;
    S->ready_cv.notify_all();
}

void lane_body(Lane *L) {
    Server *S = L->srv;
    cudaSetDevice(S->dev);
    int st = lane_open(L);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (st) {
            L->failed = true;
            L->fail_status = st;
            L->fail_msg = st == PHG_ERR_BUDGET ? "the lane does not fit in the HBM budget" : phg_last_error();
            L->closing = true;
        } else {
            L->ready = true;
        }
        S->ready_cv.notify_all();
    }
    if (!st) {
        if (L->kind == PHG_REQ_LAPLACE_SOLVE) {
            if (L->packed) packed_loop(L);
            else laplace_loop(L);
        } else {
            bv_loop(L);
        }
    }
}

void lane_main(Lane *L) {
    try {
        lane_body(L);
    } catch (...) {
        lane_abort(L);
    }
    lane_close(L);
}

// under S->mu: the lane that takes new requests for (kind, level)
Lane *lane_for(Server *S, int kind, int level) {
    const bool packed = kind == PHG_REQ_LAPLACE_SOLVE && level <= S->pack_level;
    auto key = std::make_pair(kind, packed ? 0 : level);
    auto it = S->lanes.find(key);
    if (it != S->lanes.end() && !it->second->closing && !it->second->closed) return it->second;
    auto L = std::make_unique<Lane>();
    L->srv = S;
    L->kind = kind;
    L->level = packed ? 0 : level;
    L->packed = packed;
    Lane *raw = L.get();
    S->lanes[key] = raw;
    S->all.push_back(std::move(L));
    raw->th = std::thread(lane_main, raw);
    return raw;
}

}  // namespace

struct phg_serve_s : Server {};

extern "C" int phg_serve_create(const phg_serve_conf *conf, phg_serve *out) {
    PHG_API_BEGIN
    if (!conf || !out) return PHG_ERR_ARG;
    if (!(conf->hbm_budget_bytes > 0) || (conf->precision != PHG_FP64 && conf->precision != PHG_MIXED) ||
        !(conf->solve_tol > 0) || !(conf->step_tol > 0) || conf->max_slots < 0)
        return PHG_ERR_ARG;
    auto s = std::make_unique<phg_serve_s>();
    s->conf = *conf;
    s->budget = (long long)conf->hbm_budget_bytes;
    if (cudaGetDevice(&s->dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&s->sm_total, cudaDevAttrMultiProcessorCount, s->dev) != cudaSuccess)
        return PHG_ERR_CUDA;
    s->sm_free = s->sm_total;
    s->t0 = Clock::now();
    {   // Laplace requests of levels <= pack_level share one lane and one launch per
        // turn; off by default (measured: a packed turn makes the small levels wait
        // for the largest one, p50 77 -> 435 ms on the mixed 2,000-request trace)
        const char *e = getenv("PHG_SERVE_PACK");
        s->pack_level = std::max(0, std::min(6, e ? atoi(e) : 0));
    }
    *out = s.release();
    return PHG_OK;
    PHG_API_END
}

extern "C" double phg_serve_clock(phg_serve s) { return s ? s->now() : 0.0; }

extern "C" int phg_serve_preload(phg_serve s, int kind, int level) {
    PHG_API_BEGIN
    if (!s || (kind != PHG_REQ_LAPLACE_SOLVE && kind != PHG_REQ_BARVORTEX) || level < 1 || level > 9)
        return PHG_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    Lane *L = lane_for(s, kind, level);
    s->ready_cv.wait(lk, [&] { return L->ready || L->failed || L->closed; });
    if (L->failed) return L->fail_status;
    if (L->packed && !L->closed) {   // open this level's handle in the packed lane
        L->want.push_back(level);
        L->cv.notify_all();
        auto done = [&] {
            for (int x : L->opened)
                if (x == level || x == -level) return true;
            return L->failed || L->closed;
        };
        s->ready_cv.wait(lk, done);
        for (int x : L->opened)
            if (x == -level) return PHG_ERR_BUDGET;
        return L->failed ? L->fail_status : PHG_OK;
    }
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_serve_submit(phg_serve s, const phg_request *req) {
    PHG_API_BEGIN
    if (!s || !req) return PHG_ERR_ARG;
    auto p = new Pending();
    p->r = *req;
    p->t_submit = s->now();
    const bool ok = (req->kind == PHG_REQ_LAPLACE_SOLVE || (req->kind == PHG_REQ_BARVORTEX && req->steps >= 1)) &&
                    req->level >= 1 && req->level <= 9 && req->input && req->output;
    std::lock_guard<std::mutex> lk(s->mu);
    if (!ok || s->shutting) {
        push_done(s, p, PHG_ERR_ARG, 0, s->shutting ? "server is shutting down" : "bad request");
        return PHG_OK;
    }
    Lane *L = lane_for(s, req->kind, req->level);
    if (L->failed) {
        push_done(s, p, L->fail_status, 0, L->fail_msg.c_str());
        return PHG_OK;
    }
    L->queue.push_back(p);
    L->cv.notify_all();
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_serve_poll(phg_serve s, phg_completion *out, int max, double wait_s, int *n) {
    PHG_API_BEGIN
    if (!s || !n || (max > 0 && !out)) return PHG_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_s > 0)
        s->done_cv.wait_for(lk, std::chrono::duration<double>(wait_s), [&] { return !s->done.empty(); });
    int k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n = k;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_serve_stats(phg_serve s, double *bytes_in_use, int *lanes_open, long long *completed) {
    PHG_API_BEGIN
    if (!s) return PHG_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    int open = 0;
    for (auto &kv : s->lanes) open += !kv.second->closed;
    if (bytes_in_use) *bytes_in_use = (double)s->in_use;
    if (lanes_open) *lanes_open = open;
    if (completed) *completed = s->ndone;
    return PHG_OK;
    PHG_API_END
}

extern "C" void phg_serve_destroy(phg_serve s) {
    PHG_API_BEGIN
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->shutting = true;
        for (auto &L : s->all) {
            L->stop = true;
            L->cv.notify_all();
        }
        s->mem_cv.notify_all();
    }
    for (auto &L : s->all)
        if (L->th.joinable()) L->th.join();
    for (auto &kv : s->meshes) phg_mesh_destroy(kv.second);
    delete s;
    PHG_API_END_VOID
}
