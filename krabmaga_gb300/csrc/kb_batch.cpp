// kb_batch.cpp -- batches of replicas (kb_batch_* of include/krabgpu.h):
// many independent Flockers simulations packed into one field, stepped by
// the same launches, plus replicas that join or leave a running batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kb_field_impl.h"

struct kb_batch {
    kb_field* f = nullptr;
    kb_flock_params common{};  // query mode and arithmetic shared by the replicas
    std::vector<uint8_t> have;  // replica initialised
    struct GKey {
        uint32_t launches, spl;  // spl 0: separate-kernel steps (launches = steps)
        int cur, a_last, virt;
        uint64_t sig;  // separate kernels: the launch shapes the capture baked in
        bool operator<(const GKey& o) const {
            if (launches != o.launches) return launches < o.launches;
            if (spl != o.spl) return spl < o.spl;
            if (cur != o.cur) return cur < o.cur;
            if (a_last != o.a_last) return a_last < o.a_last;
            if (virt != o.virt) return virt < o.virt;
            return sig < o.sig;
        }
    };
    struct GVal {
        cudaGraphExec_t exec;
        int cur, a_last;
    };
    std::map<GKey, GVal> graphs;
    uint64_t graph_epoch = 0;  // the field's graph_epoch when `graphs` were captured
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }
    ~kb_batch() {
        drop_graphs();
        if (f) {
            cudaStreamSynchronize(f->stream);
            delete f;
        }
    }
};

extern "C" {

kb_status kb_batch_create(int32_t device, uint32_t nrep, const kb_replica_desc* reps,
                          kb_batch** out) try {
    if (!reps || !out || nrep == 0) return fail(KB_ERR_ARG, "null argument or no replicas");
    *out = nullptr;
    std::vector<Rep> table(nrep);
    uint64_t cells = 0, boids = 0;
    std::string why;
    for (uint32_t r = 0; r < nrep; ++r) {
        const kb_replica_desc& d = reps[r];
        if (!make_rep_geometry(d.width, d.height, d.discretization, d.toroidal, &table[r], &why,
                               d.cell_wrap))
            return fail(KB_ERR_ARG, "replica " + std::to_string(r) + ": " + why);
        if (!params_ok(&d.params, &why)) return fail(KB_ERR_ARG, "replica " + std::to_string(r) + ": " + why);
        if (d.params.query_mode != reps[0].params.query_mode || d.params.arith != reps[0].params.arith)
            return fail(KB_ERR_ARG, "all replicas of a batch share query_mode and arith");
        set_rep_params(&table[r], &d.params);
        table[r].cell_off = (uint32_t)cells;
        table[r].boid_off = (uint32_t)boids;
        table[r].nboids = d.nboids;
        cells += table[r].ncells;
        boids += d.nboids;
        if (cells > 0xF0000000ull || boids > 0xF0000000ull) return fail(KB_ERR_ARG, "batch too large");
    }
    kb_field* f = nullptr;
    kb_status st = field_new(device, table, true, (uint32_t)boids, &f);
    if (st) return st;
    kb_batch* b = new kb_batch();
    b->f = f;
    b->common = reps[0].params;
    b->have.assign(nrep, 0);
    *out = b;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_destroy(kb_batch* b) try {
    if (!b) return KB_OK;
    DeviceGuard g(b->f->device);
    delete b;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_set_replica(kb_batch* b, uint32_t r, size_t n, const uint32_t* ids,
                               const float* xy, const float* dxy) try {
    if (!b || (n && (!ids || !xy || !dxy))) return fail(KB_ERR_ARG, "null argument");
    kb_field* f = b->f;
    if (r >= f->reps.size()) return fail(KB_ERR_ARG, "replica index out of range");
    if (b->have[r]) return fail(KB_ERR_STATE, "replica already set (create a new batch to reset)");
    if (n != f->reps[r].nboids) return fail(KB_ERR_ARG, "boid count differs from the replica's nboids");
    const Rep& R = f->reps[r];
    const size_t old = f->p_id.size();
    for (size_t i = 0; i < n; ++i) {
        if (!(std::isfinite(xy[2 * i]) && std::isfinite(xy[2 * i + 1]) && std::isfinite(dxy[2 * i]) &&
              std::isfinite(dxy[2 * i + 1]))) {
            f->p_st.resize(old); f->p_id.resize(old); f->p_key.resize(old);
            return fail(KB_ERR_ARG, "non-finite position or heading");
        }
        const int64_t idx = host_bag_index(R, xy[2 * i], xy[2 * i + 1]);
        if (idx < 0) {
            f->p_st.resize(old); f->p_id.resize(old); f->p_key.resize(old);
            return fail(KB_ERR_RANGE, "location outside the replica's bag matrix");
        }
        f->p_st.push_back(make_float4(xy[2 * i], xy[2 * i + 1], dxy[2 * i], dxy[2 * i + 1]));
        f->p_id.push_back(ids[i]);
        f->p_key.push_back(R.cell_off + (uint32_t)idx);
    }
    b->have[r] = 1;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

// Build the packed read buffer (every replica must be set).
kb_status kb_batch_commit(kb_batch* b) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    for (size_t r = 0; r < b->have.size(); ++r)
        if (!b->have[r]) return fail(KB_ERR_STATE, "replica " + std::to_string(r) + " not set");
    kb_field* f = b->f;
    DeviceGuard g(f->device);
    kb_status st = field_lazy_update(f);
    if (st) return st;
    uint64_t expect = 0;
    for (const Rep& R : f->reps) expect += R.nboids;
    if (f->rn != expect) return fail(KB_ERR_STATE, "packed boid count mismatch");
    return upload_rep(f);
} catch (...) {
    return kb::exception_status();
}

// nsteps steps of every replica, each replica with its own parameters.
// steps_per_launch (0 = all) persistent steps per kernel launch; with
// graph_launches > 1 that many launches are captured into one CUDA graph
// and replayed.
kb_status kb_batch_step(kb_batch* b, uint64_t first_step, uint32_t nsteps, uint32_t steps_per_launch,
                        uint32_t graph_launches) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    kb_field* f = b->f;
    if (f->wn || !f->p_id.empty()) return fail(KB_ERR_STATE, "batch not committed");
    if (nsteps == 0) return KB_OK;
    DeviceGuard g(f->device);
    const kb_flock_params* p = &b->common;
    kb_status st;
    KB_CUDA(launch_set_u64(f->dstep.p, first_step, f->stream));
    f->dstep_host = ~0ull;
    if (!fused_eligible(f, p)) {
        if ((st = materialize(f))) return st;
        if ((st = grow(f, f->rn))) return st;
        const bool fast = all_fast_rebin_ok(f) && f->layout_is_positions;
        if (graph_launches <= 1 || !fast) return enqueue_steps(f, p, nsteps, fast);
        // separate-kernel steps replayed from CUDA graphs of up to graph_launches
        // steps (the kernels read the step number from device memory, so one
        // capture serves every step range)
        if (b->graph_epoch != f->graph_epoch) {
            b->drop_graphs();
            b->graph_epoch = f->graph_epoch;
        }
        uint32_t done = 0;
        while (done < nsteps) {
            const uint32_t k = std::min(graph_launches, nsteps - done);
            if (k < 4) {
                if ((st = enqueue_steps(f, p, k, fast))) return st;
                done += k;
                continue;
            }
            const uint64_t sig = ((uint64_t)f->force_block << 48) ^ ((uint64_t)f->nblk_force << 24) ^
                                 (uint64_t)f->nblk_seg ^ ((uint64_t)f->rn << 8) ^
                                 (f->ids_unique ? (1ull << 63) : 0ull);
            kb_batch::GKey key{k, 0u, f->cur, 0, 0, sig};
            auto it = b->graphs.find(key);
            const int cur0 = f->cur;
            if (it == b->graphs.end()) {
                cudaGraph_t graph = nullptr;
                KB_CUDA(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
                st = enqueue_steps(f, p, k, fast);
                cudaError_t ce = cudaStreamEndCapture(f->stream, &graph);
                f->cur = cur0;  // the capture recorded the swaps; the replay performs them
                if (st) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                if (ce) return cuda_fail(ce, "cudaStreamEndCapture");
                cudaGraphExec_t exec = nullptr;
                ce = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ce) return cuda_fail(ce, "cudaGraphInstantiate");
                if (b->graphs.size() > 16) b->drop_graphs();
                it = b->graphs.emplace(key, kb_batch::GVal{exec, (k & 1u) ? 1 - cur0 : cur0, 0}).first;
            }
            KB_CUDA(cudaGraphLaunch(it->second.exec, f->stream));
            f->cur = it->second.cur;
            done += k;
        }
        return KB_OK;
    }
    if ((st = grow(f, f->rn))) return st;
    if ((st = fused_prepare(f, p))) return st;
    if (b->graph_epoch != f->graph_epoch) {  // captured over buffers or a tile shape since replaced
        b->drop_graphs();
        b->graph_epoch = f->graph_epoch;
    }
    if (f->fused_mode == 2)  // split: two launches per step, graphs of graph_launches steps
        return split_steps_graphed(f, p, nsteps, graph_launches > 1 ? graph_launches : 100);
    const uint32_t spl = steps_per_launch == 0 ? nsteps : std::min(steps_per_launch, nsteps);
    uint32_t done = 0;
    while (done < nsteps) {
        const uint32_t left = nsteps - done;
        const uint32_t full = left / spl;
        if (graph_launches > 1 && full >= 2) {
            const uint32_t L = std::min(graph_launches, full);
            kb_batch::GKey key{L, spl, f->cur, f->a_last, f->virt ? 1 : 0};
            auto it = b->graphs.find(key);
            if (it == b->graphs.end()) {
                const int cur0 = f->cur, al0 = f->a_last;
                const bool v0 = f->virt;
                cudaGraph_t graph = nullptr;
                KB_CUDA(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
                st = KB_OK;
                for (uint32_t k = 0; k < L && !st; ++k) st = fused_steps(f, p, spl);
                cudaError_t ce = cudaStreamEndCapture(f->stream, &graph);
                if (st) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                if (ce) return cuda_fail(ce, "cudaStreamEndCapture");
                cudaGraphExec_t exec = nullptr;
                ce = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ce) return cuda_fail(ce, "cudaGraphInstantiate");
                it = b->graphs.emplace(key, kb_batch::GVal{exec, f->cur, f->a_last}).first;
                f->cur = cur0;
                f->a_last = al0;
                f->virt = v0;
            }
            KB_CUDA(cudaGraphLaunch(it->second.exec, f->stream));
            f->cur = it->second.cur;
            f->a_last = it->second.a_last;
            f->virt = true;
            done += L * spl;
        } else {
            const uint32_t k = std::min(spl, left);
            if ((st = fused_steps(f, p, k))) return st;
            done += k;
        }
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}


static kb_status run_batch_steps(void* ctx, uint64_t first, uint32_t n) {
    return kb_batch_step((kb_batch*)ctx, first, n, 0, 0);
}

kb_status kb_batch_autotune(kb_batch* b, uint64_t first_step, uint32_t steps_per_trial,
                            const int32_t* candidates, int32_t ncand, int32_t best[3],
                            float* ms_per_step) try {
    if (!b || steps_per_trial == 0) return fail(KB_ERR_ARG, "null argument or zero steps");
    DeviceGuard g(b->f->device);
    if (b->f->fused_mode == 1 || b->f->fused_mode == 2) {
        if (!fused_eligible(b->f, &b->common))
            return fail(KB_ERR_STATE, "batch not eligible for the fused step");
        return autotune_tiles(b->f, &b->common, first_step, steps_per_trial, candidates, ncand,
                              best, ms_per_step, run_batch_steps, b);
    }
    // the separate kernels: the force pass's block size over the packed replicas
    return autotune_force_block(b->f, first_step, steps_per_trial, candidates, ncand, best,
                                ms_per_step, run_batch_steps, b);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_get_replica(kb_batch* b, uint32_t r, uint32_t* ids, float* states, size_t cap,
                               size_t* n) try {
    if (!b || !n) return fail(KB_ERR_ARG, "null argument");
    kb_field* f = b->f;
    if (r >= f->reps.size()) return fail(KB_ERR_ARG, "replica index out of range");
    DeviceGuard g(f->device);
    kb_status st = materialize(f);
    if (st) return st;
    const Rep& R = f->reps[r];
    uint32_t lo = 0, hi = 0;
    KB_CUDA(cudaMemcpyAsync(&lo, f->start[f->cur].p + R.cell_off, sizeof(uint32_t), cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaMemcpyAsync(&hi, f->start[f->cur].p + R.cell_off + R.ncells, sizeof(uint32_t), cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    *n = hi - lo;
    const size_t take = std::min<size_t>(hi - lo, cap);
    if (take) {
        if (ids) KB_CUDA(cudaMemcpyAsync(ids, f->rid.p + lo, sizeof(uint32_t) * take, cudaMemcpyDeviceToHost, f->stream));
        if (states) KB_CUDA(cudaMemcpyAsync(states, f->rst.p + lo, sizeof(float4) * take, cudaMemcpyDeviceToHost, f->stream));
    }
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return check_flags(f);
} catch (...) {
    return kb::exception_status();
}

// Moments of every replica's headings, reduced on the device.
static kb_status field_moments(kb_field* f, double* out) {
    DeviceGuard g(f->device);
    kb_status st = materialize(f);
    if (st) return st;
    if ((st = upload_rep(f))) return st;
    const uint32_t nr = (uint32_t)f->reps.size();
    DevBuf<double> d;
    cudaError_t e = d.alloc(4 * (size_t)nr);
    if (e) return cuda_fail(e, "moments");
    KB_CUDA(launch_moments(f->d_rep.p, nr, f->start[f->cur].p, f->rst.p, d.p, f->stream));
    KB_CUDA(cudaMemcpyAsync(out, d.p, sizeof(double) * 4 * nr, cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return check_flags(f);
}

kb_status kb_batch_moments(kb_batch* b, double* out) try {
    if (!b || !out) return fail(KB_ERR_ARG, "null argument");
    return field_moments(b->f, out);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_moments(kb_field* f, double out4[4]) try {
    if (!f || !out4) return fail(KB_ERR_ARG, "null argument");
    if (f->is_batch) return fail(KB_ERR_ARG, "a batch field: use kb_batch_moments");
    return field_moments(f, out4);
} catch (...) {
    return kb::exception_status();
}

// Rebuild a committed batch with a new replica table: slot i of `reps`
// takes the canonical records of old replica src[i] (src[i] >= 0) or, for
// src[i] < 0, the n host objects given (a new replica's initial state).
static kb_status batch_repack(kb_batch* b, std::vector<Rep> reps, const std::vector<int64_t>& src,
                              size_t n_new, const uint32_t* ids, const float* xy, const float* dxy) {
    kb_field* f = b->f;
    DeviceGuard g(f->device);
    kb_status st = materialize(f);
    if (st) return st;
    const std::vector<Rep> old = f->reps;
    std::vector<PackEntry> plan;
    uint64_t cells = 0, boids = 0, host_off = 0;
    bool have_host = false;
    for (size_t i = 0; i < reps.size(); ++i) {
        Rep& R = reps[i];
        R.cell_off = (uint32_t)cells;
        R.boid_off = (uint32_t)boids;
        if (src[i] >= 0) {
            PackEntry e{};
            e.dst_off = (uint32_t)boids;
            e.n = R.nboids;
            e.rep = (uint32_t)i;
            e.src_off = old[(size_t)src[i]].boid_off;
            e.kind = 0u;
            if (e.n) plan.push_back(e);
        } else {
            have_host = true;
            host_off = boids;
        }
        cells += R.ncells;
        boids += R.nboids;
    }
    if (cells > 0xF0000000ull || boids > 0xF0000000ull) return fail(KB_ERR_ARG, "batch too large");
    if ((st = grow(f, (uint32_t)std::max<uint64_t>(boids, 1)))) return st;
    if ((st = grow_cells(f, cells))) return st;
    DevBuf<PackEntry> dplan;
    if (!plan.empty()) {
        cudaError_t e = dplan.alloc(plan.size());
        if (e) return cuda_fail(e, "repack plan");
        KB_CUDA(cudaMemcpyAsync(dplan.p, plan.data(), sizeof(PackEntry) * plan.size(), cudaMemcpyHostToDevice, f->stream));
    }
    // the read buffer (rst) is the copy source; the write list the target
    if ((st = field_set_reps(f, reps))) return st;
    if (!plan.empty())
        KB_CUDA(launch_repack(dplan.p, (int32_t)plan.size(), (uint32_t)boids, f->d_rep.p, f->rst.p,
                              f->rid.p, f->wst.p, f->wid.p, f->wkey.p, f->wdead.p, f->err.p, f->stream));
    if (have_host && n_new) {
        const Rep& R = f->reps[std::find(src.begin(), src.end(), (int64_t)-1) - src.begin()];
        const uint32_t m = (uint32_t)n_new, at = (uint32_t)host_off;
        float2* sxy = reinterpret_cast<float2*>(f->tst.p);
        KB_CUDA(cudaMemcpyAsync(sxy, xy, sizeof(float2) * m, cudaMemcpyHostToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(sxy + m, dxy, sizeof(float2) * m, cudaMemcpyHostToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(f->wid.p + at, ids, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, f->stream));
        KB_CUDA(cudaMemsetAsync(f->small.p, 0xFF, sizeof(uint32_t), f->stream));
        KB_CUDA(launch_pack_locations(R, sxy, sxy + m, m, f->wst.p + at, f->wkey.p + at, f->wdead.p + at,
                                      f->small.p, f->stream));
        uint32_t bad = 0;
        if ((st = read_u32(f, f->small.p, &bad))) return st;
        if (bad != 0xFFFFFFFFu)
            return fail(KB_ERR_RANGE, "new replica: object " + std::to_string(bad) +
                                          " outside its bag matrix on the device");
    }
    f->wn = (uint32_t)boids;
    f->w_from_compute = false;
    f->w_has_dead = false;
    f->virt = false;
    f->p_st.clear(); f->p_id.clear(); f->p_key.clear();
    if ((st = general_rebuild(f, false))) return st;
    f->rn = (uint32_t)boids;
    f->wn = 0;
    f->layout_is_positions = true;
    if ((st = check_unique_ids(f))) return st;
    b->have.assign(reps.size(), 1);
    b->drop_graphs();
    return check_flags(f);
}

kb_status kb_batch_remove_replica(kb_batch* b, uint32_t r) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    kb_field* f = b->f;
    if (r >= f->reps.size()) return fail(KB_ERR_ARG, "replica index out of range");
    if (f->reps.size() < 2) return fail(KB_ERR_STATE, "a batch keeps at least one replica");
    if (f->wn || !f->p_id.empty() || std::find(b->have.begin(), b->have.end(), 0) != b->have.end())
        return fail(KB_ERR_STATE, "batch not committed");
    std::vector<Rep> reps;
    std::vector<int64_t> src;
    for (uint32_t i = 0; i < f->reps.size(); ++i)
        if (i != r) {
            reps.push_back(f->reps[i]);
            src.push_back(i);
        }
    return batch_repack(b, reps, src, 0, nullptr, nullptr, nullptr);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_add_replica(kb_batch* b, const kb_replica_desc* d, const uint32_t* ids,
                               const float* xy, const float* dxy, uint64_t origin_step,
                               uint32_t* index) try {
    if (!b || !d || !index || (d->nboids && (!ids || !xy || !dxy))) return fail(KB_ERR_ARG, "null argument");
    kb_field* f = b->f;
    if (f->wn || !f->p_id.empty() || std::find(b->have.begin(), b->have.end(), 0) != b->have.end())
        return fail(KB_ERR_STATE, "batch not committed");
    Rep R;
    std::string why;
    if (!make_rep_geometry(d->width, d->height, d->discretization, d->toroidal, &R, &why, d->cell_wrap))
        return fail(KB_ERR_ARG, why);
    if (!params_ok(&d->params, &why)) return fail(KB_ERR_ARG, why);
    if (d->params.query_mode != b->common.query_mode || d->params.arith != b->common.arith)
        return fail(KB_ERR_ARG, "all replicas of a batch share query_mode and arith");
    set_rep_params(&R, &d->params);
    R.nboids = d->nboids;
    // checked here so that a refused replica leaves the batch as it was
    for (uint32_t i = 0; i < d->nboids; ++i) {
        if (!(std::isfinite(xy[2 * i]) && std::isfinite(xy[2 * i + 1]) && std::isfinite(dxy[2 * i]) &&
              std::isfinite(dxy[2 * i + 1])))
            return fail(KB_ERR_ARG, "object " + std::to_string(i) + ": non-finite position or heading");
        if (host_bag_index(R, xy[2 * i], xy[2 * i + 1]) < 0)
            return fail(KB_ERR_RANGE, "object " + std::to_string(i) + ": location outside the replica's bag matrix");
    }
    R.origin_lo = (uint32_t)origin_step;
    R.origin_hi = (uint32_t)(origin_step >> 32);
    std::vector<Rep> reps = f->reps;
    std::vector<int64_t> src;
    for (uint32_t i = 0; i < reps.size(); ++i) src.push_back(i);
    reps.push_back(R);
    src.push_back(-1);
    kb_status st = batch_repack(b, reps, src, d->nboids, ids, xy, dxy);
    if (st) return st;
    *index = (uint32_t)(reps.size() - 1);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_synchronize(kb_batch* b) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    return kb_field_synchronize(b->f);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_cuda_stream(kb_batch* b, void** stream) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    return kb_field_cuda_stream(b->f, stream);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_set_step_options(kb_batch* b, int32_t fused, int32_t tile_tx, int32_t tile_ty) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    return kb_field_set_step_options(b->f, fused, tile_tx, tile_ty);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_step_stats(kb_batch* b, uint32_t out4[4]) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    return kb_field_step_stats(b->f, out4);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_batch_device_flags(kb_batch* b, uint32_t* flags, int32_t clear) try {
    if (!b) return fail(KB_ERR_ARG, "null argument");
    return kb_field_device_flags(b->f, flags, clear);
} catch (...) {
    return kb::exception_status();
}

}  // extern "C"

