// kb_server.cpp -- the continuous-batching request server (kb_server_* of
// include/krabgpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kb_field_impl.h"

// A continuous-batching request loop.  Requests (each a whole Flockers
// simulation) are admitted while a slot is free and their device state fits
// the HBM budget; all admitted requests advance together in one batched
// field, one persistent launch per epoch.  An epoch runs until the next
// request finishes, at most `quantum` steps; between epochs finished
// requests are copied out (their latency ends when the result is on the
// host) and queued ones join: the batch is repacked on the device (running
// replicas copied in canonical order, new ones generated in place) and one
// stable sort rebuilds the bag offsets.  Each request keeps its own step
// numbering (Rep::origin), so its result equals a run of it alone.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

namespace {

using Clock = std::chrono::steady_clock;

struct SrvReq {
    uint64_t ticket = 0;
    kb_request r{};
    Rep geom{};
    uint64_t bytes = 0;
    Clock::time_point t_arrive, t_admit, t_done;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    uint32_t remaining = 0;
    uint32_t boid_off = 0;  // in the current packing
    bool fresh = true;
    std::vector<uint32_t> ids;
    std::vector<float> st;
    std::string error;
};

uint64_t request_bytes(const Rep& R, uint32_t n) {
    // read buffer + two write lists + sort scratch per boid; offsets per bag
    return (uint64_t)n * (16 + 4) * 6 + (uint64_t)R.ncells * 4 * 4;
}

}  // namespace

struct kb_server {
    kb_server_desc desc{};
    kb_field* f = nullptr;
    kb_flock_params common{};
    std::thread loop;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    bool stop = false;
    std::deque<SrvReq*> queue;
    std::vector<SrvReq*> active;
    std::map<uint64_t, SrvReq*> all;
    uint64_t next_ticket = 1;
    uint64_t used_bytes = 0;
    uint64_t global_step = 0;
    DevBuf<PackEntry> plan;
    // stats
    std::vector<double> latencies;
    double updates = 0.0;
    uint64_t launches = 0, repacks = 0, max_active = 0, completed = 0, failed = 0;
    Clock::time_point t_first, t_last;
    bool any = false;
    double busy_s = 0.0;
};

namespace {

kb_status srv_repack(kb_server* S, std::vector<SrvReq*>& act) {
    kb_field* f = S->f;
    kb_status st = materialize(f);
    if (st) return st;
    std::vector<Rep> reps;
    std::vector<PackEntry> plan;
    uint64_t cells = 0, boids = 0;
    for (SrvReq* q : act) {
        Rep R = q->geom;
        R.cell_off = (uint32_t)cells;
        R.boid_off = (uint32_t)boids;
        R.nboids = q->r.nboids;
        if (q->fresh) {
            R.origin_lo = (uint32_t)S->global_step;
            R.origin_hi = (uint32_t)(S->global_step >> 32);
        }
        PackEntry e{};
        e.dst_off = (uint32_t)boids;
        e.n = q->r.nboids;
        e.rep = (uint32_t)reps.size();
        e.src_off = q->boid_off;
        e.kind = q->fresh ? 1u : 0u;
        e.seed_lo = (uint32_t)q->r.init_seed;
        e.seed_hi = (uint32_t)(q->r.init_seed >> 32);
        e.heading_scale = q->r.heading_scale;
        plan.push_back(e);
        q->geom = R;
        q->boid_off = (uint32_t)boids;
        cells += R.ncells;
        boids += q->r.nboids;
        reps.push_back(R);
    }
    if (boids > f->cap) return fail(KB_ERR_OOM, "server boid capacity exceeded");
    if (plan.size() > S->plan.n) {
        cudaError_t e = S->plan.alloc(std::max<size_t>(plan.size(), 2 * S->plan.n + 16));
        if (e) return cuda_fail(e, "repack plan");
    }
    KB_CUDA(cudaMemcpyAsync(S->plan.p, plan.data(), sizeof(PackEntry) * plan.size(), cudaMemcpyHostToDevice, f->stream));
    // the old read buffer (rst) is the copy source; the write list the target
    if ((st = field_set_reps(f, reps))) return st;  // synchronises the stream (plan copied)
    KB_CUDA(launch_repack(S->plan.p, (int32_t)plan.size(), (uint32_t)boids, f->d_rep.p, f->rst.p, f->rid.p,
                          f->wst.p, f->wid.p, f->wkey.p, f->wdead.p, f->err.p, f->stream));
    f->wn = (uint32_t)boids;
    f->w_from_compute = false;
    f->w_has_dead = false;
    f->virt = false;
    if ((st = general_rebuild(f, false))) return st;
    f->rn = (uint32_t)boids;
    set_ids_unique(f, true);  // every request's boids are ids 0..n-1
    f->wn = 0;
    f->layout_is_positions = true;
    for (SrvReq* q : act) q->fresh = false;
    S->repacks++;
    return KB_OK;
}

void srv_fail_all(kb_server* S, std::vector<SrvReq*>& act, const std::string& why) {
    std::lock_guard<std::mutex> lk(S->mu);
    for (SrvReq* q : act) {
        q->state = 3;
        try {
            q->error = why;
        } catch (...) {
            q->error.clear();
        }
        q->t_done = Clock::now();
        S->used_bytes -= q->bytes;
        S->failed++;
    }
    act.clear();
    S->active.clear();  // the snapshot wait_idle reads: nothing runs until the next admission
    S->cv_done.notify_all();
}

// One pass of the request loop: admit what fits, run one epoch, copy out the
// finished requests.  Returns false once the server is stopping.
bool srv_epoch(kb_server* S, std::vector<SrvReq*>& act, bool& changed) {
    kb_field* f = S->f;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        while (!S->stop && S->queue.empty() && act.empty()) S->cv.wait(lk);
        if (S->stop) return false;
        while (!S->queue.empty() && act.size() < S->desc.max_slots &&
               S->used_bytes + S->queue.front()->bytes <= S->desc.hbm_budget_bytes) {
            SrvReq* q = S->queue.front();
            S->queue.pop_front();
            q->state = 1;
            q->t_admit = Clock::now();
            q->fresh = true;
            S->used_bytes += q->bytes;
            act.push_back(q);
            changed = true;
        }
        S->active = act;
        S->max_active = std::max<uint64_t>(S->max_active, act.size());
    }
    if (act.empty()) return true;
    const auto t0 = Clock::now();
    kb_status st = KB_OK;
    if (changed) st = srv_repack(S, act);
    changed = false;
    uint32_t K = S->desc.quantum_steps ? S->desc.quantum_steps : 100;
    for (SrvReq* q : act) K = std::min(K, q->remaining);
    if (!st) {
        st = launch_set_u64(f->dstep.p, S->global_step, f->stream) ? fail(KB_ERR_CUDA, "step") : KB_OK;
        f->dstep_host = ~0ull;
    }
    if (!st && K > 0) {
        if (fused_eligible(f, &S->common)) {
            st = tiled_steps(f, &S->common, K);
        } else {
            if (!(st = materialize(f))) st = enqueue_steps(f, &S->common, K, all_fast_rebin_ok(f));
        }
        S->launches++;
    }
    if (st) {
        srv_fail_all(S, act, g_last_error);
        changed = true;
        return true;
    }
    S->global_step += K;
    double upd = 0.0;
    for (SrvReq* q : act) {
        q->remaining -= K;
        upd += (double)q->r.nboids * K;
    }
    // copy out the finished requests
    bool any_done = false;
    for (SrvReq* q : act) any_done |= (q->remaining == 0);
    if (any_done) {
        if (!(st = materialize(f))) {
            std::vector<uint32_t> lohi(2 * act.size());
            for (size_t i = 0; i < act.size(); ++i) {
                if (act[i]->remaining) continue;
                const Rep& R = act[i]->geom;
                cudaMemcpyAsync(&lohi[2 * i], f->start[f->cur].p + R.cell_off, 4, cudaMemcpyDeviceToHost, f->stream);
                cudaMemcpyAsync(&lohi[2 * i + 1], f->start[f->cur].p + R.cell_off + R.ncells, 4, cudaMemcpyDeviceToHost, f->stream);
            }
            if (cudaStreamSynchronize(f->stream) != cudaSuccess) st = fail(KB_ERR_CUDA, "copy-out");
            for (size_t i = 0; i < act.size() && !st; ++i) {
                SrvReq* q = act[i];
                if (q->remaining) continue;
                const uint32_t lo = lohi[2 * i], n = lohi[2 * i + 1] - lohi[2 * i];
                q->ids.resize(n);
                q->st.resize((size_t)n * 4);
                if (n) {
                    cudaMemcpyAsync(q->ids.data(), f->rid.p + lo, 4ull * n, cudaMemcpyDeviceToHost, f->stream);
                    cudaMemcpyAsync(q->st.data(), f->rst.p + lo, 16ull * n, cudaMemcpyDeviceToHost, f->stream);
                }
            }
            if (!st && cudaStreamSynchronize(f->stream) != cudaSuccess) st = fail(KB_ERR_CUDA, "copy-out");
            uint32_t flags = 0;
            if (!st) {
                cudaMemcpy(&flags, f->err.p, 4, cudaMemcpyDeviceToHost);
                if (flags) {
                    st = fail(KB_ERR_DEVICE_FLAG, "device error word set during serving");
                    // the word belongs to the failed batch: later requests start clean
                    cudaMemsetAsync(f->err.p, 0, sizeof(uint32_t), f->stream);
                }
            }
        }
        if (st) {
            srv_fail_all(S, act, g_last_error);
            changed = true;
            return true;
        }
    }
    const auto t1 = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->busy_s += std::chrono::duration<double>(t1 - t0).count();
        S->updates += upd;
        std::vector<SrvReq*> keep;
        for (SrvReq* q : act) {
            if (q->remaining == 0) {
                q->state = 2;
                q->t_done = t1;
                S->used_bytes -= q->bytes;
                S->latencies.push_back(std::chrono::duration<double>(q->t_done - q->t_arrive).count());
                S->completed++;
                S->t_last = t1;
                changed = true;
            } else {
                keep.push_back(q);
            }
        }
        act.swap(keep);
        S->active = act;
        if (changed) S->cv_done.notify_all();
    }
    return true;
}

void srv_loop(kb_server* S) {
    cudaSetDevice(S->desc.device);
    std::vector<SrvReq*> act;
    try {
        act.reserve(S->desc.max_slots);  // admission then never reallocates
    } catch (...) {
    }
    bool changed = false;
    for (;;) {
        try {
            if (!srv_epoch(S, act, changed)) break;
        } catch (...) {
            // a host exception (an allocation) fails the running requests as a CUDA error does
            exception_status();
            srv_fail_all(S, act, g_last_error);
            changed = true;
        }
    }
}

}  // namespace

extern "C" {

kb_status kb_server_create(const kb_server_desc* desc, kb_server** out) try {
    if (!desc || !out) return fail(KB_ERR_ARG, "null argument");
    if (desc->max_slots == 0 || desc->max_request_boids == 0)
        return fail(KB_ERR_ARG, "max_slots and max_request_boids must be positive");
    *out = nullptr;
    kb_flock_params p{};
    p.query_mode = desc->query_mode;
    p.arith = desc->arith;
    p.jump = 0.5f;
    p.neighbor_radius = 1.0f;
    std::string why;
    if (!params_ok(&p, &why)) return fail(KB_ERR_ARG, why);
    const uint64_t cap = (uint64_t)desc->max_slots * desc->max_request_boids;
    const uint64_t cells = (uint64_t)desc->max_slots * desc->max_request_cells;
    if (cap > 0xF0000000ull || cells > 0xF0000000ull) return fail(KB_ERR_ARG, "capacity too large");
    Rep R;
    if (!make_rep_geometry(16.0f, 16.0f, 4.0f, 1, &R, &why)) return fail(KB_ERR_ARG, why);
    kb_field* f = nullptr;
    kb_status st = field_new(desc->device, std::vector<Rep>{R}, true, (uint32_t)cap, &f,
                             (uint32_t)std::max<uint64_t>(cells, R.ncells));
    if (st) return st;
    kb_server* S = new kb_server();
    S->desc = *desc;
    S->f = f;
    S->common = p;
    S->loop = std::thread(srv_loop, S);
    *out = S;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_destroy(kb_server* S) try {
    if (!S) return KB_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->loop.joinable()) S->loop.join();
    {
        DeviceGuard g(S->f->device);
        cudaStreamSynchronize(S->f->stream);
        delete S->f;
    }
    for (auto& kv : S->all) delete kv.second;
    delete S;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_submit(kb_server* S, const kb_request* r, uint64_t* ticket) try {
    if (!S || !r || !ticket) return fail(KB_ERR_ARG, "null argument");
    std::string why;
    if (!params_ok(&r->params, &why)) return fail(KB_ERR_ARG, why);
    if (r->params.query_mode != S->desc.query_mode || r->params.arith != S->desc.arith)
        return fail(KB_ERR_ARG, "request query_mode/arith differ from the server's");
    if (r->nboids == 0 || r->nboids > S->desc.max_request_boids || r->steps == 0)
        return fail(KB_ERR_ARG, "request size out of range");
    SrvReq* q = new SrvReq();
    q->r = *r;
    if (!make_rep_geometry(r->side, r->side, r->discretization, 1, &q->geom, &why)) {
        delete q;
        return fail(KB_ERR_ARG, why);
    }
    if (q->geom.ncells > S->desc.max_request_cells) {
        delete q;
        return fail(KB_ERR_ARG, "request bag matrix above max_request_cells");
    }
    set_rep_params(&q->geom, &r->params);
    q->bytes = request_bytes(q->geom, r->nboids);
    if (q->bytes > S->desc.hbm_budget_bytes) {
        delete q;
        return fail(KB_ERR_BUSY, "request larger than the whole HBM budget");
    }
    q->remaining = r->steps;
    q->t_arrive = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        q->ticket = S->next_ticket++;
        S->all[q->ticket] = q;
        S->queue.push_back(q);
        if (!S->any) {
            S->any = true;
            S->t_first = q->t_arrive;
        }
    }
    S->cv.notify_all();
    *ticket = q->ticket;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_poll(kb_server* S, uint64_t ticket, int32_t* state, double* latency_s) try {
    if (!S || !state) return fail(KB_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return fail(KB_ERR_ARG, "unknown ticket");
    *state = it->second->state;
    if (latency_s)
        *latency_s = it->second->state >= 2
                         ? std::chrono::duration<double>(it->second->t_done - it->second->t_arrive).count()
                         : 0.0;
    if (it->second->state == 3) return fail(KB_ERR_STATE, it->second->error);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_result(kb_server* S, uint64_t ticket, uint32_t* ids, float* states, size_t cap,
                           size_t* n) try {
    if (!S || !n) return fail(KB_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return fail(KB_ERR_ARG, "unknown ticket");
    SrvReq* q = it->second;
    if (q->state != 2) return fail(KB_ERR_STATE, q->state == 3 ? q->error : "request not finished");
    *n = q->ids.size();
    const size_t take = std::min(cap, q->ids.size());
    if (ids && take) std::memcpy(ids, q->ids.data(), 4 * take);
    if (states && take) std::memcpy(states, q->st.data(), 16 * take);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_release(kb_server* S, uint64_t ticket) try {
    if (!S) return fail(KB_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return fail(KB_ERR_ARG, "unknown ticket");
    if (it->second->state < 2) return fail(KB_ERR_STATE, "request still queued or running");
    delete it->second;
    S->all.erase(it);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_wait_idle(kb_server* S, double timeout_s) try {
    if (!S) return fail(KB_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    const auto until = Clock::now() + std::chrono::duration<double>(timeout_s);
    while (!(S->queue.empty() && S->active.empty())) {
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout &&
            !(S->queue.empty() && S->active.empty()))
            return fail(KB_ERR_TIMEOUT, "requests still pending");
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_server_stats(kb_server* S, kb_server_report* out) try {
    if (!S || !out) return fail(KB_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    std::vector<double> v = S->latencies;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        if (v.empty()) return 0.0;
        const size_t i = (size_t)std::min<double>(v.size() - 1, std::ceil(p * v.size()) - 1);
        return v[i];
    };
    std::memset(out, 0, sizeof(*out));
    out->completed = S->completed;
    out->failed = S->failed;
    out->queued = S->queue.size();
    out->running = S->active.size();
    out->p50_s = pct(0.50);
    out->p99_s = pct(0.99);
    out->max_s = v.empty() ? 0.0 : v.back();
    out->boid_updates = S->updates;
    out->wall_s = S->any && S->completed ? std::chrono::duration<double>(S->t_last - S->t_first).count() : 0.0;
    out->busy_s = S->busy_s;
    out->launches = S->launches;
    out->repacks = S->repacks;
    out->max_active = S->max_active;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

}  // extern "C"

