// kb_api.cpp -- host runtime behind include/krabgpu.h: field handles, the
// write-buffer bookkeeping of Field2D, step orchestration with CUDA-graph
// replay, and the Field2D query entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "kb_field_impl.h"

namespace kb {

thread_local std::string g_last_error;

std::atomic<unsigned long long> g_dev_allocs{0}, g_dev_frees{0};
std::atomic<long long> g_fail_allocs{0};

kb_status fail(kb_status code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
// Set the message without letting an allocation failure escape.
static void note_error(const char* head, const char* what) noexcept {
    try {
        g_last_error = std::string(head) + what;
    } catch (...) {
        g_last_error.clear();
    }
}
kb_status exception_status() noexcept {
    try {
        throw;
    } catch (const std::bad_alloc&) {
        note_error("host allocation failed", "");
        return KB_ERR_OOM;
    } catch (const std::length_error& e) {
        note_error("host allocation too large: ", e.what());
        return KB_ERR_OOM;
    } catch (const std::exception& e) {
        note_error("host exception: ", e.what());
        return KB_ERR_STATE;
    } catch (...) {
        note_error("unknown host exception", "");
        return KB_ERR_STATE;
    }
}
kb_status cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(KB_ERR_OOM, m);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return fail(KB_ERR_NO_DEVICE, m);
    return fail(KB_ERR_CUDA, m);
}

// Host copy of discretize + bag index (field_2d.rs:328-339, 840-841) for
// argument checks on API writes; the same IEEE f32 operations as the device.
int64_t host_bag_index(const Rep& R, float x, float y) {
    int32_t cx = as_i32(std::floor(x / R.d));
    int32_t cy = as_i32(std::floor(y / R.d));
    int32_t idx = (int32_t)((uint32_t)cx * (uint32_t)R.dh + (uint32_t)cy);
    if (idx < 0 || (uint32_t)idx >= R.ncells) return -1;
    return idx;
}

bool make_rep_geometry(float w, float h, float d, int toroidal, Rep* R, std::string* why,
                       int cell_wrap) {
    if (!(std::isfinite(w) && std::isfinite(h) && std::isfinite(d)) || w <= 0.f || h <= 0.f ||
        d <= 0.f) {
        *why = "width, height and discretization must be finite and positive";
        return false;
    }
    std::memset(R, 0, sizeof(*R));
    R->w = w;
    R->h = h;
    R->d = d;
    R->toroidal = toroidal ? 1 : 0;
    if (cell_wrap != KB_CELL_WRAP_CLAMP && cell_wrap != KB_CELL_WRAP_TORUS) {
        *why = "cell_wrap must be KB_CELL_WRAP_CLAMP or KB_CELL_WRAP_TORUS";
        return false;
    }
    R->cell_wrap = (toroidal && cell_wrap == KB_CELL_WRAP_TORUS) ? 1 : 0;
    const float cw = std::ceil(w / d), ch = std::ceil(h / d);
    if (cw > 1.0e8f || ch > 1.0e8f || (double)(cw + 1.0f) * (double)(ch + 1.0f) > 2.0e9) {
        *why = "bag matrix too large (more than 2e9 bags)";
        return false;
    }
    R->max_x = as_i32(cw);
    R->max_y = as_i32(ch);
    R->dw = R->max_x + 1;
    R->dh = R->max_y + 1;
    R->ncells = (uint32_t)R->dw * (uint32_t)R->dh;
    R->inv_d = 1.0f / d;
    R->dh_magic = (~0ull / (unsigned long long)R->dh) + 1ull;
    return true;
}

void set_rep_params(Rep* R, const kb_flock_params* p) {
    R->coh = p->cohesion;
    R->avo = p->avoidance;
    R->con = p->consistency;
    R->rnd = p->randomness;
    R->mom = p->momentum;
    R->jump = p->jump;
    R->radius = p->neighbor_radius;
    R->dd = (p->neighbor_radius <= 0.0f) ? -1 : as_i32(std::floor(p->neighbor_radius / R->d));
    R->qmode = p->query_mode;
    R->seed_lo = (uint32_t)p->seed;
    R->seed_hi = (uint32_t)(p->seed >> 32);
    // With the clamped (toroidal) cell range every candidate lies within
    // (dd+1)*d of the boid, so toroidal_distance's |a-b| <= dim/2 test holds
    // whenever (dd+1)*d stays clear of half the side.
    const double reach = ((double)std::max(R->dd, 0) + 1.0) * (double)R->d;
    R->nowrap = (R->toroidal && !R->cell_wrap &&
                 reach * 1.01 + 1e-3 < 0.5 * (double)std::min(R->w, R->h)) ? 1 : 0;
    // A move of at most |jump| wraps to line 0 only from x > w - |jump|, i.e.
    // from lines >= floor((w - |jump|)/d); one line lower covers the f32
    // rounding of x/d.  A narrow last column can put that two or three lines
    // below max_x.
    const double lo = std::floor(((double)R->w - 1.01 * std::fabs((double)p->jump)) / (double)R->d) - 1.0;
    R->seam = (int32_t)std::max(0.0, std::min(lo, (double)R->max_x));
}

bool params_ok(const kb_flock_params* p, std::string* why) {
    const float v[7] = {p->cohesion, p->avoidance, p->consistency, p->randomness,
                        p->momentum, p->jump,      p->neighbor_radius};
    for (float x : v)
        if (!std::isfinite(x)) {
            *why = "flock parameters must be finite";
            return false;
        }
    if (p->query_mode != KB_QUERY_RELAX && p->query_mode != KB_QUERY_EXACT) {
        *why = "query_mode must be KB_QUERY_RELAX or KB_QUERY_EXACT";
        return false;
    }
    if (p->arith != KB_ARITH_STRICT && p->arith != KB_ARITH_FAST) {
        *why = "arith must be KB_ARITH_STRICT or KB_ARITH_FAST";
        return false;
    }
    return true;
}

// The stencil-gather rebin needs every boid to land within one bag of where
// it was (or across the seam): a move shorter than a bag, and y wrapped by
// the same length as x (bird.rs:147 wraps y with the width).
bool fast_rebin_ok(const Rep& R) {
    return R.w == R.h && R.max_x == R.max_y && std::fabs(R.jump) * 1.001f < R.d && R.max_x >= 4 &&
           R.seam >= 2 && R.max_x - R.seam <= 4;
}

}  // namespace kb


// ========================================================================




kb_status grow(kb_field* f, uint32_t need) {
    if (need <= f->cap) return KB_OK;
    if (f->virt) {
        kb_status st = materialize(f);
        if (st) return st;
    }
    uint64_t nc = std::max<uint64_t>(need, (uint64_t)f->cap * 2);
    if (nc < 1024) nc = 1024;
    if (nc > 0xFFFFFFF0ull) nc = 0xFFFFFFF0ull;
    if (need > nc) return fail(KB_ERR_ARG, "object count exceeds 2^32-16");
    const uint32_t c = (uint32_t)nc;
    DevBuf<float4> rst, wst, tst;
    DevBuf<uint32_t> rid, wid, wkey, tid, tsrc, rkey, tkey;
    DevBuf<uint8_t> wdead;
    cudaError_t e;
    if ((e = rst.alloc(c)) || (e = wst.alloc(c)) || (e = tst.alloc(c)) || (e = rid.alloc(c)) ||
        (e = wid.alloc(c)) || (e = wkey.alloc(c)) || (e = tid.alloc(c)) || (e = tsrc.alloc(c)) ||
        (e = wdead.alloc(c)) || (e = rkey.alloc(c)) || (e = tkey.alloc(c)))
        return cuda_fail(e, "growing object storage");
    // no removal marks outside the live write list (they are cleared as consumed)
    KB_CUDA(cudaMemsetAsync(wdead.p, 0, c, f->stream));
    if (f->rn) {
        KB_CUDA(cudaMemcpyAsync(rst.p, f->rst.p, sizeof(float4) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(rid.p, f->rid.p, sizeof(uint32_t) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
    }
    if (f->wn) {
        KB_CUDA(cudaMemcpyAsync(wst.p, f->wst.p, sizeof(float4) * f->wn, cudaMemcpyDeviceToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(wid.p, f->wid.p, sizeof(uint32_t) * f->wn, cudaMemcpyDeviceToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(wkey.p, f->wkey.p, sizeof(uint32_t) * f->wn, cudaMemcpyDeviceToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(wdead.p, f->wdead.p, f->wn, cudaMemcpyDeviceToDevice, f->stream));
    }
    KB_CUDA(cudaStreamSynchronize(f->stream));
    f->rst.swap(rst); f->wst.swap(wst); f->tst.swap(tst);
    f->rid.swap(rid); f->wid.swap(wid); f->wkey.swap(wkey);
    f->tid.swap(tid); f->tsrc.swap(tsrc); f->wdead.swap(wdead);
    f->rkey.swap(rkey); f->tkey.swap(tkey);
    f->cap = c;
    f->drop_graphs();
    return KB_OK;
}

// First segment of each replica (Rep::seg_off), before any table upload.
// Packed replicas take the packed segment height (Rep::seg_rows); a plain
// field keeps the default (or the dense one, chosen per step).
void assign_segments(std::vector<Rep>& reps) {
    uint32_t g = 0;
    for (Rep& R : reps) {
        R.seg_rows = reps.size() > 1 ? PACKED_SEG_ROWS : 0;
        R.seg_off = g;
        g += rep_segments(R);
    }
}

// The per-replica block tables of a packed field (see kb_field::blk_force).
kb_status build_rep_blocks(kb_field* f) {
    f->nblk_force = f->nblk_seg = 0;
    if (f->reps.size() < 2) return KB_OK;
    auto& bf = f->blk_force_h;
    auto& bs = f->blk_seg_h;
    bf.clear();
    bs.clear();
    for (uint32_t r = 0; r < (uint32_t)f->reps.size(); ++r) {
        const Rep& R = f->reps[r];
        for (uint64_t i = 0; i < R.nboids; i += f->force_block) bf.push_back(make_uint2(r, R.boid_off + (uint32_t)i));
        const uint32_t ns = rep_segments(R);
        for (uint32_t g = 0; g < ns; g += REBIN_SEG_WARPS) bs.push_back(make_uint2(r, R.seg_off + g));
    }
    if (bf.size() > f->blk_force.n || bs.size() > f->blk_seg.n)
        f->drop_graphs();  // captured over the tables about to be replaced
    if (bf.size() > f->blk_force.n) {
        cudaError_t e = f->blk_force.alloc(std::max<size_t>(bf.size(), 2 * f->blk_force.n));
        if (e) return cuda_fail(e, "replica block table");
    }
    if (bs.size() > f->blk_seg.n) {
        cudaError_t e = f->blk_seg.alloc(std::max<size_t>(bs.size(), 2 * f->blk_seg.n));
        if (e) return cuda_fail(e, "replica block table");
    }
    if (!bf.empty())
        KB_CUDA(cudaMemcpyAsync(f->blk_force.p, bf.data(), sizeof(uint2) * bf.size(), cudaMemcpyHostToDevice, f->stream));
    if (!bs.empty())
        KB_CUDA(cudaMemcpyAsync(f->blk_seg.p, bs.data(), sizeof(uint2) * bs.size(), cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    f->nblk_force = (uint32_t)bf.size();
    f->nblk_seg = (uint32_t)bs.size();
    return KB_OK;
}

// Segments of the segment rebin over all replicas.
uint32_t total_segments(const kb_field* f) {
    uint64_t t = 0;
    for (const Rep& R : f->reps) t += rep_segments(R);
    return t > 0xFFFFFFF0ull ? 0u : (uint32_t)t;
}

// ------------------------------------------------------------ dense flocks
constexpr uint64_t DENSE_MIN_CANDIDATES = 48;  // estimated mean list length that switches
constexpr uint64_t DENSE_REFRESH = 64;          // steps between two measurements

bool dense_from(unsigned long long occ2, uint32_t n) {
    return n > 0 && 9ull * occ2 >= DENSE_MIN_CANDIDATES * (unsigned long long)n;
}

void set_dense(kb_field* f, bool d) {
    if (f->dense_mode == KB_DENSE_ON) d = true;
    if (f->dense_mode == KB_DENSE_OFF || f->reps.size() != 1) d = false;
    f->dense = d;
}

// Enqueue a measurement of the read buffer into the pinned word (no wait).
kb_status occ_enqueue(kb_field* f) {
    if (f->reps.size() != 1 || f->virt) return KB_OK;
    if (!f->occ_host) {
        if (cudaMallocHost(&f->occ_host, sizeof(unsigned long long)) != cudaSuccess) {
            cudaGetLastError();
            f->occ_host = nullptr;
            return KB_OK;  // no measurement: the flag stays as it is
        }
        cudaError_t e = f->occ_dev.alloc(1);
        if (!e) e = cudaEventCreateWithFlags(&f->occ_ev, cudaEventDisableTiming);
        if (e) return cuda_fail(e, "occupancy measurement");
    }
    KB_CUDA(cudaMemsetAsync(f->occ_dev.p, 0, sizeof(unsigned long long), f->stream));
    KB_CUDA(launch_occupancy_sq(f->start[f->cur].p, f->ncells_total, f->occ_dev.p, f->stream));
    KB_CUDA(cudaMemcpyAsync(f->occ_host, f->occ_dev.p, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaEventRecord(f->occ_ev, f->stream));
    f->occ_pending = true;
    f->occ_n = f->rn;
    f->steps_since_occ = 0;
    return KB_OK;
}

// Take a finished measurement, if any (never waits).
void occ_poll(kb_field* f) {
    if (!f->occ_pending) return;
    const cudaError_t e = cudaEventQuery(f->occ_ev);
    if (e == cudaErrorNotReady) return;
    if (e != cudaSuccess) {
        cudaGetLastError();
        f->occ_pending = false;
        return;
    }
    f->occ_pending = false;
    set_dense(f, dense_from(*f->occ_host, f->occ_n));
}

// Whole steps in one thread block (kb_small.cu): a plain field small enough
// for shared memory, on the default step path.
bool small_eligible(const kb_field* f) {
    return !f->is_batch && f->reps.size() == 1 && f->fused_mode == 0 && !f->virt && f->rn > 0 &&
           f->rn <= SMALL_MAX_BOIDS && f->reps[0].ncells <= SMALL_MAX_CELLS &&
           f->reps[0].cell_off == 0;
}

// Bag rows and segment count of the segment rebin.
void rebin_geometry(const kb_field* f, RebinArgs* a) {
    if (f->dense && f->reps.size() == 1) {
        a->seg_rows = DENSE_SEG_ROWS;
        a->nsegs = rep_segments(f->reps[0], DENSE_SEG_ROWS);
    } else {
        a->seg_rows = 0;
        a->nsegs = total_segments(f);
    }
}

kb_status upload_rep(kb_field* f) {
    assign_segments(f->reps);
    f->rep.seg_off = f->reps[0].seg_off;
    if (!f->is_batch) {
        f->reps[0] = f->rep;
        if (f->rep_valid && std::memcmp(&f->rep_uploaded, &f->rep, sizeof(Rep)) == 0) return KB_OK;
        KB_CUDA(launch_set_rep(f->d_rep.p, f->rep, f->stream));
        f->rep_uploaded = f->rep;
        f->rep_valid = true;
    } else {
        KB_CUDA(cudaMemcpyAsync(f->d_rep.p, f->reps.data(), sizeof(Rep) * f->reps.size(), cudaMemcpyHostToDevice, f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
        if (kb_status st = build_rep_blocks(f)) return st;
    }
    return KB_OK;
}

int32_t nrep(const kb_field* f) { return (int32_t)f->reps.size(); }

bool all_fast_rebin_ok(const kb_field* f) {
    for (const Rep& R : f->reps)
        if (!fast_rebin_ok(R)) return false;
    return true;
}

// Append the host-side pending writes to the device write list.
kb_status flush_pending(kb_field* f) {
    const size_t np = f->p_id.size();
    if (np == 0) return KB_OK;
    if ((uint64_t)f->wn + np > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "too many objects");
    kb_status st = grow(f, f->wn + (uint32_t)np);
    if (st) return st;
    KB_CUDA(cudaMemcpyAsync(f->wst.p + f->wn, f->p_st.data(), sizeof(float4) * np, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(f->wid.p + f->wn, f->p_id.data(), sizeof(uint32_t) * np, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(f->wkey.p + f->wn, f->p_key.data(), sizeof(uint32_t) * np, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemsetAsync(f->wdead.p + f->wn, 0, np, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));  // the pending vectors are reused
    f->wn += (uint32_t)np;
    if (f->p_loc_differs) f->layout_is_positions = false;
    f->p_st.clear(); f->p_id.clear(); f->p_key.clear();
    f->p_loc_differs = false;
    f->w_from_compute = false;
    return KB_OK;
}

kb_status read_u32(kb_field* f, const uint32_t* dptr, uint32_t* out) {
    KB_CUDA(cudaMemcpyAsync(out, dptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return KB_OK;
}

kb_status check_flags(kb_field* f) {
    uint32_t flags = 0;
    kb_status st = read_u32(f, f->err.p, &flags);
    if (st) return st;
    if (flags) {
        char buf[160];
        std::snprintf(buf, sizeof buf,
                      "device error word 0x%x (1 key out of range, 2 rebin miss, 4 spin "
                      "timeout, 8 non-finite)",
                      flags);
        return fail(KB_ERR_DEVICE_FLAG, buf);
    }
    return KB_OK;
}

kb_status ensure_aux_scan(kb_field* f, uint32_t n) {
    const uint32_t t = scan_state_words(n);
    if (t <= f->aux_tiles) return KB_OK;
    DevBuf<unsigned long long> ts;
    cudaError_t e = ts.alloc(t);
    if (e) return cuda_fail(e, "scan workspace");
    KB_CUDA(cudaMemsetAsync(ts.p, 0, sizeof(unsigned long long) * t, f->stream));
    f->aux_tstate.swap(ts);
    f->aux_tiles = t;
    return KB_OK;
}

// Bounded-wait settings of the field's kernels (kb_field_set_wait_test).
WaitCfg scan_wait(const kb_field* f) {
    return WaitCfg{f->wait_spins, f->withhold_kind == KB_WITHHOLD_SCAN_PUBLISH ? f->withhold_index : ~0u};
}
WaitCfg fused_wait(const kb_field* f) {
    return WaitCfg{f->wait_spins, f->withhold_kind == KB_WITHHOLD_GRID_ARRIVAL ? f->withhold_index : ~0u};
}

// After a bounded wait gave up, the control words of the waiting kernels can
// be left mid-protocol (a grid barrier's arrival count, a tile counter, look-
// back words): reset them all, with the epochs restarting at zero.  The step
// that gave up left the read buffer invalid: a plain field is emptied (its
// state is set anew), a batch's replicas are set anew by the caller.
kb_status reset_wait_state(kb_field* f) {
    cudaStream_t s = f->stream;
    if (f->scan_ctl.p) KB_CUDA(cudaMemsetAsync(f->scan_ctl.p, 0, sizeof(ScanCtl) * f->scan_ctl.n, s));
    if (f->tstate.p) KB_CUDA(cudaMemsetAsync(f->tstate.p, 0, sizeof(unsigned long long) * f->tstate.n, s));
    if (f->aux_ctl.p) KB_CUDA(cudaMemsetAsync(f->aux_ctl.p, 0, sizeof(ScanCtl) * f->aux_ctl.n, s));
    if (f->aux_tstate.p)
        KB_CUDA(cudaMemsetAsync(f->aux_tstate.p, 0, sizeof(unsigned long long) * f->aux_tstate.n, s));
    if (f->hist.p) KB_CUDA(cudaMemsetAsync(f->hist.p, 0, sizeof(uint32_t) * f->hist.n, s));
    f->hist_counted = false;
    auto& F = f->fused;
    if (F.ctl.p) KB_CUDA(cudaMemsetAsync(F.ctl.p, 0, sizeof(uint32_t) * F.ctl.n, s));
    if (F.scan_state.p)
        KB_CUDA(cudaMemsetAsync(F.scan_state.p, 0, sizeof(unsigned long long) * F.scan_state.n, s));
    f->virt = false;
    if (!f->is_batch) {
        f->rn = 0;
        if (f->start[f->cur].p)
            KB_CUDA(cudaMemsetAsync(f->start[f->cur].p, 0, sizeof(uint32_t) * (f->ncells_total + 1), s));
    }
    f->dstep_host = ~0ull;
    KB_CUDA(cudaStreamSynchronize(s));
    return KB_OK;
}

// The general stable sort: write list -> read buffer.  hist already holds
// the key counts when counted == true.
kb_status general_rebuild(kb_field* f, bool counted) {
    cudaStream_t s = f->stream;
    const int nxt = 1 - f->cur;
    if (!counted) {
        // a force pass may have counted the list before it was edited
        if (f->hist_counted)
            KB_CUDA(cudaMemsetAsync(f->hist.p, 0, sizeof(uint32_t) * f->ncells_total, s));
        KB_CUDA(launch_hist_list(f->wkey.p, f->wdead.p, f->wn, f->hist.p, s));
    }
    f->hist_counted = false;  // the scan below zeroes it
    KB_CUDA(launch_scan(f->hist.p, f->start[nxt].p, f->ncells_total, f->scan_ctl.p, f->tstate.p, f->err.p, true, s,
                        scan_wait(f)));
    KB_CUDA(launch_scatter_list(f->wkey.p, f->wdead.p, f->wst.p, f->wid.p, f->wn, f->start[nxt].p, f->cursor.p, f->tst.p, f->tid.p, f->tsrc.p, s));
    KB_CUDA(launch_canon(f->start[nxt].p, f->ncells_total, f->tst.p, f->tid.p, f->tsrc.p, f->cursor.p, f->rst.p, f->rid.p, s));
    f->cur = nxt;
    return KB_OK;
}

kb_status fast_rebuild(kb_field* f, bool bump_step) {
    cudaStream_t s = f->stream;
    const int nxt = 1 - f->cur;
    KB_CUDA(launch_scan(f->hist.p, f->start[nxt].p, f->ncells_total, f->scan_ctl.p, f->tstate.p, f->err.p, true, s,
                        scan_wait(f)));
    f->hist_counted = false;
    if (f->kt_cur >= 0) KB_CUDA(cudaEventRecord(f->kt_pending[f->kt_cur].ev[2], s));
    RebinArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = nrep(f);
    a.rep0 = f->reps[0];
    a.start_cur = f->start[f->cur].p;
    a.start_next = f->start[nxt].p;
    a.key = f->wkey.p;
    a.a_st = f->wst.p;
    a.a_ids = f->wid.p;
    a.ncells = f->ncells_total;
    rebin_geometry(f, &a);
    a.sblk = f->nblk_seg ? f->blk_seg.p : nullptr;
    a.nsblk = f->nblk_seg;
    a.s_st = f->rst.p;
    a.s_ids = f->rid.p;
    a.step = bump_step ? f->dstep.p : nullptr;
    a.err = f->err.p;
    a.n = f->rn;
    KB_CUDA(launch_rebin(a, s));
    f->cur = nxt;
    return KB_OK;
}

kb_status enqueue_force(kb_field* f, const kb_flock_params* p) {
    ForceArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = nrep(f);
    a.rep0 = f->reps[0];
    a.st = f->rst.p;
    a.ids = f->rid.p;
    a.start = f->start[f->cur].p;
    a.n = f->rn;
    a.step = f->dstep.p;
    a.out_st = f->wst.p;
    a.out_ids = f->wid.p;
    a.out_key = f->wkey.p;
    a.hist = f->hist.p;
    a.err = f->err.p;
    // The fast rebin is used only when |jump| * 1.001 < d, so no boid can
    // leave the 3x3 stencil; the rebin's own count check (every bag gathers
    // exactly its counted arrivals) reports any miss.  The per-boid move check
    // only names the cause, at two extra discretisations per boid.
    a.check_moves = 0;
    a.blk = f->nblk_force ? f->blk_force.p : nullptr;
    a.nblk = f->nblk_force;
    a.self_by_slot = f->ids_unique ? 1 : 0;
    a.dense = f->dense ? 1 : 0;
    a.block_threads = f->force_block;
    KB_CUDA(launch_flock_force(a, p->arith == KB_ARITH_STRICT, p->query_mode, f->stream));
    f->hist_counted = true;
    return KB_OK;
}

float4* buf_st(kb_field* f, int i) { return i == 0 ? f->rst.p : (i == 1 ? f->wst.p : f->tst.p); }
uint32_t* buf_ids(kb_field* f, int i) { return i == 0 ? f->rid.p : (i == 1 ? f->wid.p : f->tid.p); }
uint32_t* buf_key(kb_field* f, int i) { return i == 0 ? f->rkey.p : (i == 1 ? f->wkey.p : f->tkey.p); }

// Rebuild the read buffer from a virtual state (the stencil gather of the
// last write list into canonical order).  The read buffer keeps its device
// address (a write list held in rst is gathered into the third buffer and
// copied back), so graphs captured over the field's buffers stay valid and
// the query entry points that materialise drop none.
kb_status materialize(kb_field* f) {
    if (!f->virt) return KB_OK;
    int dst = 0;
    if (f->a_last == 0) dst = 2;  // the write list sits in rst: gather into tst, then copy back
    RebinArgs r{};
    r.reps = f->d_rep.p;
    r.nrep = nrep(f);
    r.rep0 = f->reps[0];
    r.start_cur = f->start[1 - f->cur].p;
    r.start_next = f->start[f->cur].p;
    r.key = f->keys_valid ? buf_key(f, f->a_last) : nullptr;
    r.a_st = buf_st(f, f->a_last);
    r.a_ids = buf_ids(f, f->a_last);
    r.ncells = f->ncells_total;
    rebin_geometry(f, &r);
    r.sblk = f->nblk_seg ? f->blk_seg.p : nullptr;
    r.nsblk = f->nblk_seg;
    r.s_st = buf_st(f, dst);
    r.s_ids = buf_ids(f, dst);
    r.step = nullptr;
    r.err = f->err.p;
    r.n = f->rn;
    KB_CUDA(launch_rebin(r, f->stream));
    if (dst == 2 && f->rn) {
        KB_CUDA(cudaMemcpyAsync(f->rst.p, f->tst.p, sizeof(float4) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
        KB_CUDA(cudaMemcpyAsync(f->rid.p, f->tid.p, sizeof(uint32_t) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
    }
    f->virt = false;
    return KB_OK;
}

// Tile shape and shared-memory capacities for a field of n boids: tiles of
// tx x ty bags; capacities sized from the mean occupancy with room for
// Poisson fluctuations (over-full tiles take the global scratch path).
FusedCfg fused_config(const kb_field* f, int dd) {
    FusedCfg c{};
    c.tx = f->tile_tx > 0 ? f->tile_tx : 16;
    c.ty = f->tile_ty > 0 ? f->tile_ty : 32;
    c.dd = dd;
    // mean bag occupancy of the densest replica: every tile's capacity must hold
    // the densest replica's tiles (replicas of one sweep differ several-fold)
    double rho = (double)f->rn / (double)f->ncells_total;  // a plain field: its mean
    if (f->is_batch)
        for (const Rep& R : f->reps)
            if (R.ncells) rho = std::max(rho, (double)R.nboids / (double)R.ncells);
    const double staged_cells = (double)(c.tx + 2 * dd + 2) * (c.ty + 2 * dd + 2);
    const double sord_cells = (double)(c.tx + 2 * dd) * (c.ty + 2 * dd);
    auto cap = [](double mean) {
        double v = mean * 1.5 + 6.0 * std::sqrt(mean + 1.0) + 64.0;
        if (v > 6144.0) v = 6144.0;
        return (uint32_t)((uint32_t)v + 31u) / 32u * 32u;
    };
    c.stage_cap = cap(rho * staged_cells);
    c.sord_cap = cap(rho * sord_cells);
    return c;
}

bool fused_eligible(const kb_field* f, const kb_flock_params* p) {
    if ((f->fused_mode != 1 && f->fused_mode != 2) || !f->layout_is_positions || f->rn == 0)
        return false;
    if (p->query_mode != KB_QUERY_RELAX && p->query_mode != KB_QUERY_EXACT) return false;
    for (const Rep& R : f->reps)
        if (!R.toroidal || R.cell_wrap || !fast_rebin_ok(R) || R.dd > FUSED_DD_MAX || R.dw > 65535 ||
            R.dh > 65535)
            return false;
    return true;
}

kb_status fused_prepare(kb_field* f, const kb_flock_params* p) {
    auto& F = f->fused;
    const int strict = p->arith == KB_ARITH_STRICT ? 1 : 0;
    int dd = 0;
    for (const Rep& R : f->reps) dd = std::max(dd, R.dd);
    if (F.ready && F.n == f->rn && F.strict == strict && F.qmode == p->query_mode && F.dd == dd)
        return KB_OK;
    F.ready = false;
    FusedCfg cfg = fused_config(f, dd);
    int maxc = 0;
    if (F.occ_valid && std::memcmp(&F.occ_cfg, &cfg, sizeof cfg) == 0 && F.occ_strict == strict &&
        F.occ_qmode == p->query_mode)
        maxc = F.occ_ctas;
    else
        maxc = fused_max_ctas(cfg, strict != 0, p->query_mode, f->device);
    while (maxc <= 0 && (cfg.stage_cap > 256 || cfg.sord_cap > 256)) {
        cfg.stage_cap = std::max(256u, cfg.stage_cap / 2);
        cfg.sord_cap = std::max(256u, cfg.sord_cap / 2);
        maxc = fused_max_ctas(cfg, strict != 0, p->query_mode, f->device);
    }
    if (maxc <= 0) return fail(KB_ERR_CUDA, "fused step: no co-resident CTA fits");
    F.occ_valid = true;
    F.occ_cfg = cfg;
    F.occ_strict = strict;
    F.occ_qmode = p->query_mode;
    F.occ_ctas = maxc;
    // tiles of every replica, largest replicas first (long tiles start early)
    std::vector<uint32_t> order(f->reps.size());
    for (uint32_t r = 0; r < order.size(); ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return f->reps[a].nboids > f->reps[b].nboids;
    });
    std::vector<Tile> tiles;
    for (uint32_t r : order) {
        const Rep& R = f->reps[r];
        for (int x = 0; x < R.dw; x += cfg.tx)
            for (int y = 0; y < R.dh; y += cfg.ty) tiles.push_back(Tile{r, (uint16_t)x, (uint16_t)y});
    }
    // grow-only scratch (a serving loop re-plans on every repack)
    cudaError_t e = cudaSuccess;
    if (F.tiles.n < tiles.size()) e = F.tiles.alloc(std::max<size_t>(tiles.size(), 2 * F.tiles.n));
    if (!e && F.g_st.n < f->cap) e = F.g_st.alloc(f->cap);
    if (!e && F.g_ids.n < f->cap) e = F.g_ids.alloc(f->cap);
    bool fresh_ctl = false;
    if (!e && F.scan_state.n < (size_t)maxc) {
        e = F.scan_state.alloc((size_t)maxc);
        fresh_ctl = true;
    }
    if (!e && F.ctl.n < 8) {
        e = F.ctl.alloc(8);
        fresh_ctl = true;
    }
    if (e) return cuda_fail(e, "fused step buffers");
    KB_CUDA(cudaMemcpyAsync(F.tiles.p, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, f->stream));
    if (fresh_ctl) {
        // a new look-back array starts at epoch 0: restart the epoch counter too
        KB_CUDA(cudaMemsetAsync(F.scan_state.p, 0, sizeof(unsigned long long) * F.scan_state.n, f->stream));
        KB_CUDA(cudaMemsetAsync(F.ctl.p, 0, sizeof(uint32_t) * 8, f->stream));
    }
    KB_CUDA(cudaStreamSynchronize(f->stream));
    F.cfg = cfg;
    F.nctas = (uint32_t)maxc;
    F.ntiles = (uint32_t)tiles.size();
    F.n = f->rn;
    F.strict = strict;
    F.qmode = p->query_mode;
    F.dd = dd;
    F.ready = true;
    f->drop_graphs();
    return KB_OK;
}

// nsteps steps of the persistent kernel.  From a materialised read buffer
// the first step's rebin is the identity (previous offsets := current ones);
// from a virtual state the kernel continues from the last write list.  The
// read buffer is left virtual.
kb_status fused_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps) {
    auto& F = f->fused;
    cudaStream_t s = f->stream;
    const int cur0 = f->cur;
    int in = 0;
    if (!f->virt) {
        const size_t sb = sizeof(uint32_t) * ((size_t)f->ncells_total + 1);
        KB_CUDA(cudaMemcpyAsync(f->start[1 - cur0].p, f->start[cur0].p, sb, cudaMemcpyDeviceToDevice, s));
        in = 0;
    } else {
        in = f->a_last;
    }
    const int o0 = in == 0 ? 1 : 0, o1 = in == 2 ? 1 : 2;  // the two buffers that are not the input
    FusedArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = nrep(f);
    a.tiles = F.tiles.p;
    a.ntiles = F.ntiles;
    a.cfg = F.cfg;
    a.ncells = f->ncells_total;
    a.n = f->rn;
    a.a_in_st = buf_st(f, in);
    a.a_in_ids = buf_ids(f, in);
    a.a_st[0] = buf_st(f, o0);
    a.a_st[1] = buf_st(f, o1);
    a.a_ids[0] = buf_ids(f, o0);
    a.a_ids[1] = buf_ids(f, o1);
    a.start_b[0] = f->start[1 - cur0].p;
    a.start_b[1] = f->start[cur0].p;
    a.hist = f->hist.p;
    a.g_sord_st = F.g_st.p;
    a.g_sord_ids = F.g_ids.p;
    a.step = f->dstep.p;
    a.nsteps = nsteps;
    a.tile_counter = F.ctl.p;
    a.bar = F.ctl.p + 1;
    a.scan_state = F.scan_state.p;
    a.scan_epoch = F.ctl.p + 3;
    a.err = f->err.p;
    a.stats = F.ctl.p + 4;
    a.phase_cycles = nullptr;
    a.wait = fused_wait(f);
    if (F.profile) {
        if (F.phase_cycles.n < (size_t)F.nctas * 16) {
            cudaError_t e = F.phase_cycles.alloc((size_t)F.nctas * 16);
            if (e) return cuda_fail(e, "phase clocks");
            KB_CUDA(cudaMemsetAsync(F.phase_cycles.p, 0, sizeof(unsigned long long) * F.nctas * 16, s));
        }
        a.phase_cycles = F.phase_cycles.p;
    }
    KB_CUDA(launch_fused(a, F.strict != 0, F.qmode, F.nctas, s));
    const int last = (int)((nsteps - 1) & 1u);
    f->a_last = last == 0 ? o0 : o1;
    // the newest offsets are in start_b[last]; the previous ones in the other
    f->cur = (last == 0) ? 1 - cur0 : cur0;
    f->virt = true;
    f->keys_valid = false;  // the persistent kernel does not write keys
    return KB_OK;
}

FusedArgs fused_args(kb_field* f) {
    auto& F = f->fused;
    FusedArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = nrep(f);
    a.tiles = F.tiles.p;
    a.ntiles = F.ntiles;
    a.cfg = F.cfg;
    a.ncells = f->ncells_total;
    a.n = f->rn;
    a.hist = f->hist.p;
    a.g_sord_st = F.g_st.p;
    a.g_sord_ids = F.g_ids.p;
    a.step = f->dstep.p;
    a.err = f->err.p;
    a.stats = F.ctl.p + 4;
    a.phase_cycles = nullptr;
    a.wait = fused_wait(f);
    if (F.profile) {
        if (F.phase_cycles.n < 16) {
            if (F.phase_cycles.alloc(16)) return a;
            cudaMemsetAsync(F.phase_cycles.p, 0, sizeof(unsigned long long) * 16, f->stream);
        }
        a.phase_cycles = F.phase_cycles.p;
    }
    return a;
}

// nsteps steps in the split form: per step one tile launch (stage, rebin,
// force) and one scan launch; the step counter advances at the end.  Same
// buffer discipline as fused_steps; leaves the read buffer virtual.
kb_status split_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps) {
    auto& F = f->fused;
    cudaStream_t s = f->stream;
    int cur = f->cur;
    int in = 0;
    if (!f->virt) {
        const size_t sb = sizeof(uint32_t) * ((size_t)f->ncells_total + 1);
        KB_CUDA(cudaMemcpyAsync(f->start[1 - cur].p, f->start[cur].p, sb, cudaMemcpyDeviceToDevice, s));
        in = 0;
    } else {
        in = f->a_last;
    }
    const FusedArgs a = fused_args(f);
    // keys travel with the write lists; a materialised read buffer has none
    bool in_keys = f->virt && f->keys_valid;
    for (uint32_t k = 0; k < nsteps; ++k) {
        const int out = (in + 1) % 3;
        KB_CUDA(launch_tile_step(a, buf_st(f, in), buf_ids(f, in), in_keys ? buf_key(f, in) : nullptr,
                                 buf_st(f, out), buf_ids(f, out), buf_key(f, out),
                                 f->start[1 - cur].p, f->start[cur].p, k, F.strict != 0, F.qmode, s));
        in_keys = true;
        KB_CUDA(launch_scan(f->hist.p, f->start[1 - cur].p, f->ncells_total, f->scan_ctl.p,
                            f->tstate.p, f->err.p, true, s, scan_wait(f)));
        cur = 1 - cur;
        in = out;
    }
    KB_CUDA(launch_add_u64(f->dstep.p, nsteps, s));
    f->cur = cur;
    f->a_last = in;
    f->virt = true;
    f->keys_valid = true;
    return KB_OK;
}

// split_steps in CUDA-graph chunks of at most `chunk` steps, cached by the
// buffer state they start from.
kb_status split_steps_graphed(kb_field* f, const kb_flock_params* p, uint32_t nsteps, uint32_t chunk) {
    uint32_t done = 0;
    while (done < nsteps) {
        const uint32_t k = std::min(chunk, nsteps - done);
        if (k < 2) {
            kb_status st = split_steps(f, p, k);
            if (st) return st;
            done += k;
            continue;
        }
        std::vector<uint32_t> key = {k, (uint32_t)f->cur, (uint32_t)f->a_last, f->virt ? 1u : 0u,
                                     f->keys_valid ? 1u : 0u, (uint32_t)f->fused.strict,
                                     (uint32_t)f->fused.qmode};
        auto it = f->sgraphs.find(key);
        if (it == f->sgraphs.end()) {
            const int cur0 = f->cur, al0 = f->a_last;
            const bool v0 = f->virt, kv0 = f->keys_valid;
            cudaGraph_t graph = nullptr;
            KB_CUDA(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
            kb_status st = split_steps(f, p, k);
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
            if (f->sgraphs.size() > 24) {
                for (auto& kv : f->sgraphs) cudaGraphExecDestroy(kv.second.exec);
                f->sgraphs.clear();
            }
            it = f->sgraphs.emplace(key, kb_field::SGraph{exec, f->cur, f->a_last}).first;
            f->cur = cur0;
            f->a_last = al0;
            f->virt = v0;
            f->keys_valid = kv0;
        }
        KB_CUDA(cudaGraphLaunch(it->second.exec, f->stream));
        f->cur = it->second.cur;
        f->a_last = it->second.a_last;
        f->virt = true;
        f->keys_valid = true;
        done += k;
    }
    return KB_OK;
}

// Run nsteps through the configured tiled path (split or persistent).
kb_status tiled_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps) {
    kb_status st = fused_prepare(f, p);
    if (st) return st;
    if (f->fused_mode == 1) return fused_steps(f, p, nsteps);
    return split_steps_graphed(f, p, nsteps, 100);
}

// ids_unique changes what the captured force launches do: drop the graphs.
void set_ids_unique(kb_field* f, bool u) {
    if (f->ids_unique != u) f->drop_graphs();
    f->ids_unique = u;
}

// Whether the read buffer's ids are distinct within each replica.
kb_status check_unique_ids(kb_field* f) {
    if (f->rn == 0) {
        set_ids_unique(f, true);
        return KB_OK;
    }
    uint64_t cap = 1024;
    while (cap < 2ull * f->rn) cap <<= 1;
    if (cap > 0x80000000ull) {
        set_ids_unique(f, false);
        return KB_OK;
    }
    if (f->dup_tab.n < cap) {
        cudaError_t e = f->dup_tab.alloc(cap);
        if (e) return cuda_fail(e, "id check table");
    }
    if (kb_status st = upload_rep(f)) return st;
    KB_CUDA(cudaMemsetAsync(f->small.p, 0, sizeof(uint32_t), f->stream));
    KB_CUDA(launch_dup_check(f->d_rep.p, nrep(f), f->rid.p, f->rn, f->dup_tab.p, (uint32_t)cap,
                             f->small.p, f->stream));
    uint32_t dup = 0;
    if (kb_status st = read_u32(f, f->small.p, &dup)) return st;
    set_ids_unique(f, dup == 0);
    return KB_OK;
}

kb_status field_lazy_update(kb_field* f) {
    kb_status st = flush_pending(f);
    if (st) return st;
    f->virt = false;  // the write buffer replaces the read buffer
    // field_2d.rs:905-921: the first swap fixes nagents' density estimate.
    if (!f->density_check) f->density_check = true;
    if (f->w_from_compute && !f->w_has_dead) {
        if (all_fast_rebin_ok(f) && f->layout_is_positions) st = fast_rebuild(f, false);
        else st = general_rebuild(f, true);
        if (st) return st;
        f->rn = f->wn;
        f->layout_is_positions = true;
    } else {
        st = general_rebuild(f, false);
        if (st) return st;
        if ((st = occ_enqueue(f))) return st;  // completes with the read below
        uint32_t total = 0;
        st = read_u32(f, f->start[f->cur].p + f->ncells_total, &total);
        if (st) return st;
        f->rn = total;
        if (f->occ_pending) {
            f->occ_n = total;
            occ_poll(f);
        }
        // the id multiset may have changed
        if ((st = check_unique_ids(f))) return st;
    }
    // the removal marks are consumed: the next write list starts with none
    if (f->w_has_dead && f->wn) KB_CUDA(cudaMemsetAsync(f->wdead.p, 0, f->wn, f->stream));
    f->wn = 0;
    f->w_from_compute = false;
    f->w_has_dead = false;
    return KB_OK;
}


// ====================================================================== C ABI
extern "C" {

const char* kb_last_error(void) { return g_last_error.c_str(); }
const char* kb_version(void) { return "krabgpu 0.1.0 (sm_103a)"; }

int32_t kb_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // extern "C"


// Allocate a field over a replica table (cell_off/boid_off already set).
kb_status field_new(int device, const std::vector<Rep>& reps, bool is_batch, uint32_t capacity,
                    kb_field** out, uint32_t cells_cap) {
    *out = nullptr;
    int ndev = kb_device_count();
    if (ndev <= 0) return fail(KB_ERR_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(KB_ERR_ARG, "bad device ordinal");
    uint64_t total = 0;
    for (const Rep& R : reps) total += R.ncells;
    if (total == 0 || total > 0xF0000000ull) return fail(KB_ERR_ARG, "bag matrix too large");
    const uint32_t ncells = (uint32_t)total;
    const uint32_t nc = std::max(ncells, cells_cap);
    DeviceGuard g(device);
    kb_field* f = new kb_field();
    f->device = device;
    f->reps = reps;
    f->rep = f->reps[0];
    f->ncells_total = ncells;
    f->cells_cap = nc;
    f->is_batch = is_batch;
    assign_segments(f->reps);
    f->rep = f->reps[0];
    cudaError_t e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking);
    const uint32_t nt = scan_state_words(nc);
    if (!e) e = f->d_rep.alloc(reps.size());
    if (!e) e = f->start[0].alloc((size_t)nc + 1);
    if (!e) e = f->start[1].alloc((size_t)nc + 1);
    if (!e) e = f->hist.alloc(nc);
    if (!e) e = f->cursor.alloc(nc);
    if (!e) e = f->scan_ctl.alloc(1);
    if (!e) e = f->aux_ctl.alloc(1);
    if (!e) e = f->tstate.alloc(nt);
    if (!e) e = f->err.alloc(1);
    if (!e) e = f->dstep.alloc(1);
    if (!e) e = f->small.alloc(16);
    if (!e) e = cudaMemsetAsync(f->start[0].p, 0, sizeof(uint32_t) * ((size_t)nc + 1), f->stream);
    if (!e) e = cudaMemsetAsync(f->start[1].p, 0, sizeof(uint32_t) * ((size_t)nc + 1), f->stream);
    if (!e) e = cudaMemsetAsync(f->hist.p, 0, sizeof(uint32_t) * nc, f->stream);
    if (!e) e = cudaMemsetAsync(f->cursor.p, 0, sizeof(uint32_t) * nc, f->stream);
    if (!e) e = cudaMemsetAsync(f->scan_ctl.p, 0, sizeof(ScanCtl), f->stream);
    if (!e) e = cudaMemsetAsync(f->aux_ctl.p, 0, sizeof(ScanCtl), f->stream);
    if (!e) e = cudaMemsetAsync(f->tstate.p, 0, sizeof(unsigned long long) * nt, f->stream);
    if (!e) e = cudaMemsetAsync(f->err.p, 0, sizeof(uint32_t), f->stream);
    if (!e) e = cudaMemsetAsync(f->dstep.p, 0, sizeof(unsigned long long), f->stream);
    if (!e) e = cudaMemcpyAsync(f->d_rep.p, f->reps.data(), sizeof(Rep) * reps.size(), cudaMemcpyHostToDevice, f->stream);
    if (!e) e = cudaStreamSynchronize(f->stream);
    if (e) {
        delete f;
        return cuda_fail(e, "creating field");
    }
    if (kb_status st = build_rep_blocks(f)) {
        delete f;
        return st;
    }
    if (capacity) {
        kb_status st = grow(f, capacity);
        if (st) {
            delete f;
            return st;
        }
    }
    *out = f;
    return KB_OK;
}

// Bag arrays for at least `need` bags (contents are not kept: the caller
// rebuilds the offsets with a general sort).
kb_status grow_cells(kb_field* f, uint64_t need) {
    if (need <= f->cells_cap) return KB_OK;
    if (need > 0xF0000000ull) return fail(KB_ERR_ARG, "bag matrix too large");
    const uint32_t nc = (uint32_t)std::min<uint64_t>(0xF0000000ull, std::max<uint64_t>(need, 2ull * f->cells_cap));
    const uint32_t nt = scan_state_words(nc);
    DevBuf<uint32_t> s0, s1, hist, cursor;
    DevBuf<unsigned long long> ts;
    cudaError_t e;
    if ((e = s0.alloc((size_t)nc + 1)) || (e = s1.alloc((size_t)nc + 1)) || (e = hist.alloc(nc)) ||
        (e = cursor.alloc(nc)) || (e = ts.alloc(nt)))
        return cuda_fail(e, "growing the bag arrays");
    KB_CUDA(cudaMemsetAsync(s0.p, 0, sizeof(uint32_t) * ((size_t)nc + 1), f->stream));
    KB_CUDA(cudaMemsetAsync(s1.p, 0, sizeof(uint32_t) * ((size_t)nc + 1), f->stream));
    KB_CUDA(cudaMemsetAsync(hist.p, 0, sizeof(uint32_t) * nc, f->stream));
    KB_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(uint32_t) * nc, f->stream));
    KB_CUDA(cudaMemsetAsync(ts.p, 0, sizeof(unsigned long long) * nt, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    f->start[0].swap(s0);
    f->start[1].swap(s1);
    f->hist.swap(hist);
    f->cursor.swap(cursor);
    f->tstate.swap(ts);
    f->cells_cap = nc;
    f->hist_counted = false;
    f->fused.ready = false;
    f->drop_graphs();
    return KB_OK;
}

// Replace the replica table of a capacity-sized field (the contents are
// rebuilt by the caller).
kb_status field_set_reps(kb_field* f, const std::vector<Rep>& reps) {
    uint64_t total = 0;
    for (const Rep& R : reps) total += R.ncells;
    if (total == 0 || total > f->cells_cap) return fail(KB_ERR_ARG, "bag capacity exceeded");
    if (reps.size() > f->d_rep.n) {
        cudaError_t e = f->d_rep.alloc(std::max<size_t>(reps.size(), 2 * f->d_rep.n));
        if (e) return cuda_fail(e, "replica table");
    }
    f->reps = reps;
    assign_segments(f->reps);
    f->rep = f->reps[0];
    f->ncells_total = (uint32_t)total;
    f->fused.ready = false;
    f->drop_graphs();
    KB_CUDA(cudaMemcpyAsync(f->d_rep.p, f->reps.data(), sizeof(Rep) * reps.size(), cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return build_rep_blocks(f);
}


namespace kb {
// The field's device and its read buffer as query arguments, for query
// launches made by other translation units (kb_noalloc.cu).  Materialises the
// read buffer; the caller has made the field's device current.
int field_device(const kb_field* f) { return f->device; }
kb_status field_query_view(kb_field* f, int32_t kind, float dist, QueryArgs* a, cudaStream_t* s) {
    if (kb_status st = materialize(f)) return st;
    a->rep = f->rep;
    a->kind = kind;
    a->dist = dist;
    a->start = f->start[f->cur].p;
    a->st = f->rst.p;
    a->ids = f->rid.p;
    *s = f->stream;
    return KB_OK;
}
}  // namespace kb

extern "C" {

kb_status kb_debug_allocation_counts(uint64_t* allocs, uint64_t* frees) try {
    if (!allocs || !frees) return fail(KB_ERR_ARG, "null argument");
    *allocs = g_dev_allocs.load(std::memory_order_relaxed);
    *frees = g_dev_frees.load(std::memory_order_relaxed);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_debug_fail_allocations(uint32_t count) try {
    g_fail_allocs.store((long long)count, std::memory_order_relaxed);
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_create(const kb_field_desc* desc, kb_field** out) try {
    if (!desc || !out) return fail(KB_ERR_ARG, "null argument");
    *out = nullptr;
    Rep R;
    std::string why;
    if (!make_rep_geometry(desc->width, desc->height, desc->discretization, desc->toroidal, &R, &why,
                           desc->cell_wrap))
        return fail(KB_ERR_ARG, why);
    return field_new(desc->device, std::vector<Rep>{R}, false, desc->capacity_hint, out);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_destroy(kb_field* f) try {
    if (!f) return KB_OK;
    DeviceGuard g(f->device);
    cudaStreamSynchronize(f->stream);
    delete f;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_dims(const kb_field* f, int32_t out4[4]) try {
    if (!f || !out4) return fail(KB_ERR_ARG, "null argument");
    out4[0] = f->rep.dw;
    out4[1] = f->rep.dh;
    out4[2] = f->rep.max_x;
    out4[3] = f->rep.max_y;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_cuda_stream(kb_field* f, void** stream) try {
    if (!f || !stream) return fail(KB_ERR_ARG, "null argument");
    *stream = (void*)f->stream;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_object_location(kb_field* f, uint32_t id, const float pos[2],
                                       const float last_d[2], const float loc[2]) try {
    if (!f || !pos || !last_d || !loc) return fail(KB_ERR_ARG, "null argument");
    if (!(std::isfinite(pos[0]) && std::isfinite(pos[1]) && std::isfinite(last_d[0]) &&
          std::isfinite(last_d[1]) && std::isfinite(loc[0]) && std::isfinite(loc[1])))
        return fail(KB_ERR_ARG, "non-finite position or heading");
    int64_t idx = host_bag_index(f->rep, loc[0], loc[1]);
    if (idx < 0) return fail(KB_ERR_RANGE, "location outside the bag matrix (the reference panics)");
    f->p_st.push_back(make_float4(pos[0], pos[1], last_d[0], last_d[1]));
    f->p_id.push_back(id);
    f->p_key.push_back((uint32_t)idx);
    if (host_bag_index(f->rep, pos[0], pos[1]) != idx) f->p_loc_differs = true;
    if (!f->density_check) f->nagents += 1;
    f->w_from_compute = false;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_locations(kb_field* f, size_t n, const uint32_t* ids, const float* xy,
                                 const float* dxy) try {
    if (!f || (n && (!ids || !xy || !dxy))) return fail(KB_ERR_ARG, "null argument");
    if (n == 0) return KB_OK;
    if ((uint64_t)f->wn + f->p_id.size() + n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "too many objects");
    DeviceGuard g(f->device);
    // earlier single writes first (insertion order), then this batch packed
    // on the device straight behind them
    kb_status st = flush_pending(f);
    if (st) return st;
    if (f->virt && (st = materialize(f))) return st;
    if ((st = grow(f, f->wn + (uint32_t)n))) return st;
    const uint32_t m = (uint32_t)n;
    // staging in the scratch records buffer: xy in its first 8n bytes, dxy after
    float2* sxy = reinterpret_cast<float2*>(f->tst.p);
    float2* sdxy = sxy + m;
    KB_CUDA(cudaMemcpyAsync(sxy, xy, sizeof(float2) * m, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(sdxy, dxy, sizeof(float2) * m, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(f->wid.p + f->wn, ids, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemsetAsync(f->small.p, 0xFF, sizeof(uint32_t), f->stream));
    KB_CUDA(launch_pack_locations(f->rep, sxy, sdxy, m, f->wst.p + f->wn, f->wkey.p + f->wn,
                                  f->wdead.p + f->wn, f->small.p, f->stream));
    uint32_t bad = 0;
    if ((st = read_u32(f, f->small.p, &bad))) return st;
    if (bad != 0xFFFFFFFFu) {  // the write list is left as it was
        const size_t i = bad;
        if (!(std::isfinite(xy[2 * i]) && std::isfinite(xy[2 * i + 1]) &&
              std::isfinite(dxy[2 * i]) && std::isfinite(dxy[2 * i + 1])))
            return fail(KB_ERR_ARG, "non-finite position or heading");
        char buf[128];
        std::snprintf(buf, sizeof buf, "object %zu: location outside the bag matrix (the reference panics)", i);
        return fail(KB_ERR_RANGE, buf);
    }
    f->wn += m;
    if (!f->density_check) f->nagents += n;
    f->w_from_compute = false;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_remove_object_location(kb_field* f, uint32_t id, const float loc[2]) try {
    if (!f || !loc) return fail(KB_ERR_ARG, "null argument");
    int64_t idx = host_bag_index(f->rep, loc[0], loc[1]);
    if (idx < 0) return fail(KB_ERR_RANGE, "location outside the bag matrix (the reference panics)");
    DeviceGuard g(f->device);
    kb_status st = flush_pending(f);
    if (st) return st;
    KB_CUDA(cudaMemsetAsync(f->small.p, 0, sizeof(uint32_t), f->stream));
    KB_CUDA(launch_remove(f->wkey.p, f->wdead.p, f->wid.p, f->wn, (uint32_t)idx, id, f->small.p, f->stream));
    uint32_t removed = 0;
    st = read_u32(f, f->small.p, &removed);
    if (st) return st;
    if (removed) {
        f->w_has_dead = true;
        if (!f->density_check) f->nagents -= removed;
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_lazy_update(kb_field* f) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    return field_lazy_update(f);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_num_agents(kb_field* f, size_t* out) try {
    if (!f || !out) return fail(KB_ERR_ARG, "null argument");
    *out = f->nagents;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_num_objects(kb_field* f, size_t* out) try {
    if (!f || !out) return fail(KB_ERR_ARG, "null argument");
    *out = f->rn;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

static kb_status query_points(kb_field* f, int kind, float dist, size_t nq, const float* qxy,
                              uint32_t* counts, uint32_t* digest, uint32_t* ids, float* states,
                              size_t cap, size_t* total) {
    if (nq > 0x7FFFFFFFull) return fail(KB_ERR_ARG, "too many query points");
    DeviceGuard g(f->device);
    if (kb_status st0 = materialize(f)) return st0;
    if (nq == 0) {
        if (total) *total = 0;
        return KB_OK;
    }
    const uint32_t n = (uint32_t)nq;
    DevBuf<float2> dq;
    DevBuf<uint32_t> dcounts, ddig, doff, dids;
    DevBuf<float4> dst;
    cudaError_t e = dq.alloc(n);
    if (!e) e = dcounts.alloc(n);
    if (!e && digest) e = ddig.alloc(n);
    if (e) return cuda_fail(e, "query buffers");
    KB_CUDA(cudaMemcpyAsync(dq.p, qxy, sizeof(float2) * n, cudaMemcpyHostToDevice, f->stream));
    QueryArgs a{};
    a.rep = f->rep;
    a.kind = kind;
    a.dist = dist;
    a.start = f->start[f->cur].p;
    a.st = f->rst.p;
    a.ids = f->rid.p;
    a.nq = n;
    a.q = dq.p;
    a.counts = dcounts.p;
    a.digest = digest ? ddig.p : nullptr;
    a.offsets = nullptr;
    a.out_ids = nullptr;
    a.out_st = nullptr;
    a.cap = 0;
    KB_CUDA(launch_query(a, f->stream));
    if (ids || states || total) {
        kb_status st = ensure_aux_scan(f, n);
        if (st) return st;
        e = doff.alloc((size_t)n + 1);
        if (e) return cuda_fail(e, "query offsets");
        KB_CUDA(launch_scan(dcounts.p, doff.p, n, f->aux_ctl.p, f->aux_tstate.p, f->err.p, false, f->stream));
        uint32_t tot = 0;
        st = read_u32(f, doff.p + n, &tot);
        if (st) return st;
        if (total) *total = tot;
        const uint64_t take = std::min<uint64_t>(tot, cap);
        if ((ids || states) && take > 0) {
            if (!e) e = dids.alloc(take);
            if (!e && states) e = dst.alloc(take);
            if (e) return cuda_fail(e, "query output");
            a.offsets = doff.p;
            a.out_ids = dids.p;
            a.out_st = states ? dst.p : nullptr;
            a.cap = take;
            KB_CUDA(launch_query(a, f->stream));
            if (ids) KB_CUDA(cudaMemcpyAsync(ids, dids.p, sizeof(uint32_t) * take, cudaMemcpyDeviceToHost, f->stream));
            if (states) KB_CUDA(cudaMemcpyAsync(states, dst.p, sizeof(float4) * take, cudaMemcpyDeviceToHost, f->stream));
        }
    }
    if (counts) KB_CUDA(cudaMemcpyAsync(counts, dcounts.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, f->stream));
    if (digest) KB_CUDA(cudaMemcpyAsync(digest, ddig.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return KB_OK;
}

kb_status kb_field_get_neighbors_within_relax_distance(kb_field* f, const float loc[2], float dist,
                                                       uint32_t* ids, float* states, size_t cap,
                                                       size_t* n) try {
    if (!f || !loc || !n) return fail(KB_ERR_ARG, "null argument");
    return query_points(f, KB_QUERY_RELAX, dist, 1, loc, nullptr, nullptr, ids, states, cap, n);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_neighbors_within_distance(kb_field* f, const float loc[2], float dist,
                                                 uint32_t* ids, float* states, size_t cap,
                                                 size_t* n) try {
    if (!f || !loc || !n) return fail(KB_ERR_ARG, "null argument");
    return query_points(f, KB_QUERY_EXACT, dist, 1, loc, nullptr, nullptr, ids, states, cap, n);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_neighbor_lists(kb_field* f, int32_t kind, float dist, size_t nq,
                                  const float* qxy, uint32_t* counts, uint32_t* ids, size_t cap,
                                  size_t* total) try {
    if (!f || (nq && (!qxy || !counts))) return fail(KB_ERR_ARG, "null argument");
    if (kind != KB_QUERY_RELAX && kind != KB_QUERY_EXACT) return fail(KB_ERR_ARG, "bad query kind");
    size_t t = 0;
    kb_status st = query_points(f, kind, dist, nq, qxy, counts, nullptr, ids, nullptr, cap, &t);
    if (total) *total = t;
    return st;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_neighbor_digest(kb_field* f, int32_t kind, float dist, size_t nq,
                                   const float* qxy, uint32_t* counts, uint32_t* digest) try {
    if (!f || (nq && (!qxy || !counts || !digest))) return fail(KB_ERR_ARG, "null argument");
    if (kind != KB_QUERY_RELAX && kind != KB_QUERY_EXACT) return fail(KB_ERR_ARG, "bad query kind");
    return query_points(f, kind, dist, nq, qxy, counts, digest, nullptr, nullptr, 0, nullptr);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_objects(kb_field* f, const float loc[2], uint32_t* ids, float* states,
                               size_t cap, size_t* n) try {
    if (!f || !loc || !n) return fail(KB_ERR_ARG, "null argument");
    int64_t idx = host_bag_index(f->rep, loc[0], loc[1]);
    if (idx < 0) return fail(KB_ERR_RANGE, "location outside the bag matrix (the reference panics)");
    DeviceGuard g(f->device);
    if (cap && (ids || states)) {
        if (kb_status st0 = materialize(f)) return st0;
    }
    uint32_t se[2];
    KB_CUDA(cudaMemcpyAsync(se, f->start[f->cur].p + idx, sizeof(se), cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    const uint32_t cnt = se[1] - se[0];
    *n = cnt;
    const size_t take = std::min<size_t>(cnt, cap);
    if (take) {
        if (ids) KB_CUDA(cudaMemcpyAsync(ids, f->rid.p + se[0], sizeof(uint32_t) * take, cudaMemcpyDeviceToHost, f->stream));
        if (states) KB_CUDA(cudaMemcpyAsync(states, f->rst.p + se[0], sizeof(float4) * take, cudaMemcpyDeviceToHost, f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_objects_unbuffered(kb_field* f, const float loc[2], uint32_t* ids,
                                          float* states, size_t cap, size_t* n) try {
    if (!f || !loc || !n) return fail(KB_ERR_ARG, "null argument");
    int64_t idx = host_bag_index(f->rep, loc[0], loc[1]);
    if (idx < 0) return fail(KB_ERR_RANGE, "location outside the bag matrix (the reference panics)");
    DeviceGuard g(f->device);
    kb_status st = flush_pending(f);
    if (st) return st;
    DevBuf<uint32_t> dids;
    DevBuf<float4> dst;
    const uint64_t take = std::min<uint64_t>(cap, f->wn);
    cudaError_t e = cudaSuccess;
    if (take && ids) e = dids.alloc(take);
    if (!e && take && states) e = dst.alloc(take);
    if (e) return cuda_fail(e, "query output");
    KB_CUDA(launch_filter_key(f->wkey.p, f->wdead.p, f->wst.p, f->wid.p, f->wn, (uint32_t)idx, dids.p, dst.p, take, f->small.p, f->stream));
    uint32_t cnt = 0;
    st = read_u32(f, f->small.p, &cnt);
    if (st) return st;
    *n = cnt;
    const uint64_t got = std::min<uint64_t>(cnt, take);
    if (got) {
        if (ids) KB_CUDA(cudaMemcpyAsync(ids, dids.p, sizeof(uint32_t) * got, cudaMemcpyDeviceToHost, f->stream));
        if (states) KB_CUDA(cudaMemcpyAsync(states, dst.p, sizeof(float4) * got, cudaMemcpyDeviceToHost, f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_num_objects_at_location(kb_field* f, const float loc[2], size_t* n) try {
    return kb_field_get_objects(f, loc, nullptr, nullptr, 0, n);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_empty_bags(kb_field* f, float* xy, size_t cap, size_t* n) try {
    if (!f || !n || (cap && !xy)) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    DevBuf<float2> dxy;
    const uint64_t take = std::min<uint64_t>(cap, f->rep.ncells);
    if (take) {
        cudaError_t e = dxy.alloc(take);
        if (e) return cuda_fail(e, "empty bag output");
    }
    KB_CUDA(launch_empty_bags(f->rep, f->start[f->cur].p, dxy.p, take, f->small.p, f->stream));
    uint32_t cnt = 0;
    kb_status st = read_u32(f, f->small.p, &cnt);
    if (st) return st;
    *n = cnt;
    const uint64_t got = std::min<uint64_t>(cnt, take);
    if (got) {
        KB_CUDA(cudaMemcpyAsync(xy, dxy.p, sizeof(float2) * got, cudaMemcpyDeviceToHost, f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_random_empty_bag(kb_field* f, uint64_t seed, float xy[2], int32_t* found) try {
    if (!f || !xy || !found) return fail(KB_ERR_ARG, "null argument");
    size_t n = 0;
    kb_status st = kb_field_get_empty_bags(f, nullptr, 0, &n);
    if (st) return st;
    if (n == 0) {
        *found = 0;
        return KB_OK;
    }
    std::vector<float> all(2 * n);
    st = kb_field_get_empty_bags(f, all.data(), n, &n);
    if (st) return st;
    U4 o = philox4x32_10(U4{0u, 0u, 0u, 2u}, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t pick = (((uint64_t)o.y << 32) | o.x) % n;
    xy[0] = all[2 * pick];
    xy[1] = all[2 * pick + 1];
    *found = 1;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_iter_objects(kb_field* f, int32_t buffered, float* cell_xy, uint32_t* ids,
                                float* states, size_t cap, size_t* n) try {
    if (!f || !n) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    const float4* src_st;
    const uint32_t* src_id;
    const uint32_t* src_start;
    uint32_t cnt;
    DevBuf<uint32_t> tmp_start, tmp_id, tmp_src, cursor;
    DevBuf<float4> tmp_st, tmp_sorted;
    DevBuf<uint32_t> tmp_sorted_id;
    if (buffered) {
        if (kb_status st0 = materialize(f)) return st0;
        src_st = f->rst.p;
        src_id = f->rid.p;
        src_start = f->start[f->cur].p;
        cnt = f->rn;
    } else {
        // stable sort of the live write list into scratch (write buffer order)
        kb_status st = flush_pending(f);
        if (st) return st;
        const uint32_t nc = f->rep.ncells, w = f->wn > 0 ? f->wn : 1;
        cudaError_t e = tmp_start.alloc((size_t)nc + 1);
        if (!e) e = cursor.alloc(nc);
        if (!e) e = tmp_st.alloc(w);
        if (!e) e = tmp_id.alloc(w);
        if (!e) e = tmp_src.alloc(w);
        if (!e) e = tmp_sorted.alloc(w);
        if (!e) e = tmp_sorted_id.alloc(w);
        if (e) return cuda_fail(e, "iteration scratch");
        KB_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(uint32_t) * nc, f->stream));
        KB_CUDA(launch_hist_list(f->wkey.p, f->wdead.p, f->wn, cursor.p, f->stream));
        st = ensure_aux_scan(f, nc);
        if (st) return st;
        KB_CUDA(launch_scan(cursor.p, tmp_start.p, nc, f->aux_ctl.p, f->aux_tstate.p, f->err.p, true, f->stream));
        KB_CUDA(launch_scatter_list(f->wkey.p, f->wdead.p, f->wst.p, f->wid.p, f->wn, tmp_start.p, cursor.p, tmp_st.p, tmp_id.p, tmp_src.p, f->stream));
        KB_CUDA(launch_canon(tmp_start.p, nc, tmp_st.p, tmp_id.p, tmp_src.p, cursor.p, tmp_sorted.p, tmp_sorted_id.p, f->stream));
        st = read_u32(f, tmp_start.p + nc, &cnt);
        if (st) return st;
        src_st = tmp_sorted.p;
        src_id = tmp_sorted_id.p;
        src_start = tmp_start.p;
    }
    *n = cnt;
    const size_t take = std::min<size_t>(cnt, cap);
    if (take) {
        if (cell_xy) {
            DevBuf<uint32_t> cell_of;
            DevBuf<float2> dxy;
            cudaError_t e = cell_of.alloc(cnt);
            if (!e) e = dxy.alloc(cnt);
            if (e) return cuda_fail(e, "iteration output");
            KB_CUDA(launch_cell_of(src_start, f->rep.ncells, cell_of.p, f->stream));
            KB_CUDA(launch_cell_xy(f->rep, cell_of.p, cnt, dxy.p, f->stream));
            KB_CUDA(cudaMemcpyAsync(cell_xy, dxy.p, sizeof(float2) * take, cudaMemcpyDeviceToHost, f->stream));
            KB_CUDA(cudaStreamSynchronize(f->stream));
        }
        if (ids) KB_CUDA(cudaMemcpyAsync(ids, src_id, sizeof(uint32_t) * take, cudaMemcpyDeviceToHost, f->stream));
        if (states) KB_CUDA(cudaMemcpyAsync(states, src_st, sizeof(float4) * take, cudaMemcpyDeviceToHost, f->stream));
    }
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_state(kb_field* f, uint32_t* ids, float* states, size_t cap, size_t* n) try {
    if (!f || !n) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    if (kb_status st0 = materialize(f)) return st0;
    *n = f->rn;
    const size_t take = std::min<size_t>(f->rn, cap);
    if (take) {
        if (ids) KB_CUDA(cudaMemcpyAsync(ids, f->rid.p, sizeof(uint32_t) * take, cudaMemcpyDeviceToHost, f->stream));
        if (states) KB_CUDA(cudaMemcpyAsync(states, f->rst.p, sizeof(float4) * take, cudaMemcpyDeviceToHost, f->stream));
    }
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return check_flags(f);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_device_flags(kb_field* f, uint32_t* flags, int32_t clear) try {
    if (!f || !flags) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    kb_status st = read_u32(f, f->err.p, flags);
    if (st) return st;
    if (clear) {
        if ((*flags & ERR_SPIN_TIMEOUT) && (st = reset_wait_state(f))) return st;
        KB_CUDA(cudaMemsetAsync(f->err.p, 0, sizeof(uint32_t), f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_wait_test(kb_field* f, uint32_t spin_limit, int32_t withhold, uint32_t index) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    if (withhold != KB_WITHHOLD_NONE && withhold != KB_WITHHOLD_SCAN_PUBLISH &&
        withhold != KB_WITHHOLD_GRID_ARRIVAL)
        return fail(KB_ERR_ARG, "withhold must be one of KB_WITHHOLD_*");
    f->wait_spins = spin_limit;
    f->withhold_kind = withhold;
    f->withhold_index = withhold == KB_WITHHOLD_NONE ? 0u : index;
    f->drop_graphs();  // captured launches hold the previous settings
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_synchronize(kb_field* f) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return check_flags(f);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_step_options(kb_field* f, int32_t fused, int32_t tile_tx, int32_t tile_ty) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    if (tile_tx < 0 || tile_ty < 0 || tile_tx > 64 || tile_ty > 128)
        return fail(KB_ERR_ARG, "tile shape out of range (tx <= 64, ty <= 128)");
    if (fused < 0 || fused > 3) return fail(KB_ERR_ARG, "step mode must be 0, 1, 2 or 3");
    f->fused_mode = fused;
    f->tile_tx = tile_tx;
    f->tile_ty = tile_ty;
    f->fused.ready = false;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_dense_mode(kb_field* f, int32_t mode) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    if (mode != KB_DENSE_AUTO && mode != KB_DENSE_OFF && mode != KB_DENSE_ON)
        return fail(KB_ERR_ARG, "dense mode must be KB_DENSE_AUTO, KB_DENSE_OFF or KB_DENSE_ON");
    if (f->is_batch) return fail(KB_ERR_ARG, "a batch field: the batch path keeps one flat list");
    f->dense_mode = mode;
    set_dense(f, f->dense);
    if (mode == KB_DENSE_AUTO) f->steps_since_occ = DENSE_REFRESH;  // measure at the next step
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_step_path(kb_field* f, int32_t* path) try {
    if (!f || !path) return fail(KB_ERR_ARG, "null argument");
    occ_poll(f);
    kb_flock_params q{};
    q.query_mode = KB_QUERY_RELAX;
    if (fused_eligible(f, &q)) *path = f->fused_mode;
    else if (small_eligible(f)) *path = KB_PATH_SMALL;
    else *path = f->dense ? KB_PATH_DENSE : KB_PATH_SEPARATE;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_dense_active(kb_field* f, int32_t* active) try {
    if (!f || !active) return fail(KB_ERR_ARG, "null argument");
    occ_poll(f);
    *active = f->dense ? 1 : 0;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_phase_clocks(kb_field* f, int32_t enable, unsigned long long* out16) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    f->fused.profile = enable != 0;
    if (out16) {
        for (int k = 0; k < 16; ++k) out16[k] = 0;
        const size_t n = f->fused.phase_cycles.n;
        if (n) {
            std::vector<unsigned long long> h(n);
            KB_CUDA(cudaMemcpyAsync(h.data(), f->fused.phase_cycles.p, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, f->stream));
            KB_CUDA(cudaStreamSynchronize(f->stream));
            for (size_t i = 0; i < n; ++i) out16[i % 16] += h[i];
        }
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

}  // extern "C"

// Time `steps` fused steps under each candidate tile shape (real steps of
// the simulation, numbered from first_step) and keep the fastest shape.
kb_status autotune_force_block(kb_field* f, uint64_t first_step, uint32_t steps,
                               const int32_t* cand, int32_t ncand, int32_t* best_out,
                               float* best_ms_out, kb_status (*run)(void*, uint64_t, uint32_t),
                               void* ctx) {
    static const int32_t defaults[] = {128, 1, 256, 1, 512, 1};
    if (!cand || ncand <= 0) {
        cand = defaults;
        ncand = 3;
    }
    for (int32_t i = 0; i < ncand; ++i) {
        const int32_t t = cand[2 * i];
        if ((t != 128 && t != 256 && t != 512) || cand[2 * i + 1] != 1)
            return fail(KB_ERR_ARG, "candidate " + std::to_string(i) +
                                        ": force blocks of 128, 256 or 512 threads, one replica per block");
    }
    cudaEvent_t e0, e1;
    KB_CUDA(cudaEventCreate(&e0));
    KB_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_i = -1;
    uint64_t step = first_step;
    kb_status st = KB_OK;
    auto use = [&](int32_t t) -> kb_status {
        if (f->force_block == (uint32_t)t) return KB_OK;
        f->force_block = (uint32_t)t;
        f->drop_graphs();  // the block table's length is baked into captured launches
        return build_rep_blocks(f);
    };
    for (int32_t i = 0; i < ncand && !st; ++i) {
        if ((st = use(cand[2 * i]))) break;
        if ((st = run(ctx, step, 1))) break;  // warms up
        step += 1;
        if (cudaEventRecord(e0, f->stream) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        if ((st = run(ctx, step, steps))) break;
        step += steps;
        if (cudaEventRecord(e1, f->stream) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        if (cudaEventSynchronize(e1) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            best_i = i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    if ((st = use(cand[2 * best_i]))) return st;
    if (best_out) {
        best_out[0] = (int32_t)f->force_block;
        best_out[1] = 1;
        best_out[2] = (int32_t)(step - first_step);  // steps consumed
    }
    if (best_ms_out) *best_ms_out = best / (float)steps;
    return KB_OK;
}

kb_status autotune_tiles(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                                uint32_t steps, const int32_t* cand, int32_t ncand,
                                int32_t* best_out, float* best_ms_out,
                                kb_status (*run)(void*, uint64_t, uint32_t), void* ctx) {
    static const int32_t defaults[] = {8, 16, 8, 32, 16, 16, 16, 32, 32, 32, 16, 64, 32, 16};
    if (!cand || ncand <= 0) {
        cand = defaults;
        ncand = (int32_t)(sizeof(defaults) / sizeof(defaults[0]) / 2);
    }
    for (int32_t i = 0; i < ncand; ++i)  // the bounds of kb_field_set_step_options
        if (cand[2 * i] < 0 || cand[2 * i + 1] < 0 || cand[2 * i] > 64 || cand[2 * i + 1] > 128)
            return fail(KB_ERR_ARG, "candidate " + std::to_string(i) +
                                        ": tile shape out of range (tx <= 64, ty <= 128)");
    cudaEvent_t e0, e1;
    KB_CUDA(cudaEventCreate(&e0));
    KB_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_i = -1;
    uint64_t step = first_step;
    kb_status st = KB_OK;
    for (int32_t i = 0; i < ncand && !st; ++i) {
        f->tile_tx = cand[2 * i];
        f->tile_ty = cand[2 * i + 1];
        f->fused.ready = false;
        if ((st = run(ctx, step, 1))) break;  // prepares the layout, warms up
        step += 1;
        if (cudaEventRecord(e0, f->stream) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        if ((st = run(ctx, step, steps))) break;
        step += steps;
        if (cudaEventRecord(e1, f->stream) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        if (cudaEventSynchronize(e1) != cudaSuccess) { st = fail(KB_ERR_CUDA, "event"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            best_i = i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    f->tile_tx = cand[2 * best_i];
    f->tile_ty = cand[2 * best_i + 1];
    f->fused.ready = false;
    if (best_out) {
        best_out[0] = f->tile_tx;
        best_out[1] = f->tile_ty;
        best_out[2] = (int32_t)(step - first_step);  // steps consumed
    }
    if (best_ms_out) *best_ms_out = best / (float)steps;
    return KB_OK;
}

extern "C" {

struct FieldTuneCtx {
    kb_field* f;
    const kb_flock_params* p;
};
static kb_status run_field_steps(void* ctx, uint64_t first, uint32_t n) {
    FieldTuneCtx* c = (FieldTuneCtx*)ctx;
    return kb_flock_step(c->f, c->p, first, n);
}

kb_status kb_field_autotune(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                            uint32_t steps_per_trial, const int32_t* candidates, int32_t ncand,
                            int32_t best[3], float* ms_per_step) try {
    if (!f || !p || steps_per_trial == 0) return fail(KB_ERR_ARG, "null argument or zero steps");
    std::string why;
    if (!params_ok(p, &why)) return fail(KB_ERR_ARG, why);
    DeviceGuard g(f->device);
    set_rep_params(&f->rep, p);
    f->reps[0] = f->rep;
    if (!fused_eligible(f, p)) return fail(KB_ERR_STATE, "field not eligible for the fused step");
    FieldTuneCtx ctx{f, p};
    return autotune_tiles(f, p, first_step, steps_per_trial, candidates, ncand, best, ms_per_step,
                          run_field_steps, &ctx);
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_step_stats(kb_field* f, uint32_t out4[4]) try {
    if (!f || !out4) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    out4[0] = out4[1] = out4[2] = out4[3] = 0;
    if (f->fused.ready) {
        KB_CUDA(cudaMemcpyAsync(out4, f->fused.ctl.p + 4, sizeof(uint32_t), cudaMemcpyDeviceToHost, f->stream));
        KB_CUDA(cudaStreamSynchronize(f->stream));
        out4[1] = f->fused.ntiles;
        out4[2] = f->fused.nctas;
        out4[3] = (uint32_t)f->fused.cfg.tx << 16 | (uint32_t)f->fused.cfg.ty;
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_flock_compute(kb_field* f, const kb_flock_params* p, uint64_t step) try {
    if (!f || !p) return fail(KB_ERR_ARG, "null argument");
    std::string why;
    if (!params_ok(p, &why)) return fail(KB_ERR_ARG, why);
    if (f->wn || !f->p_id.empty())
        return fail(KB_ERR_STATE, "write buffer not empty: call lazy_update first");
    DeviceGuard g(f->device);
    kb_status st = materialize(f);
    if (st) return st;
    if ((st = grow(f, f->rn))) return st;
    set_rep_params(&f->rep, p);
    if ((st = upload_rep(f))) return st;
    KB_CUDA(launch_set_u64(f->dstep.p, step, f->stream));
    f->dstep_host = step;
    if ((st = enqueue_force(f, p))) return st;
    f->wn = f->rn;
    f->w_from_compute = true;
    f->w_has_dead = false;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_flock_compute_agents(kb_field* f, const kb_flock_params* p, uint64_t step, size_t n,
                                  const uint32_t* ids, const float* states) try {
    if (!f || !p || (n && (!ids || !states))) return fail(KB_ERR_ARG, "null argument");
    if (f->is_batch) return fail(KB_ERR_ARG, "a batch field: agents join a batch with kb_batch_add_replica");
    std::string why;
    if (!params_ok(p, &why)) return fail(KB_ERR_ARG, why);
    for (size_t j = 0; j < n; ++j)
        for (int c = 0; c < 4; ++c)
            if (!std::isfinite(states[4 * j + c]))
                return fail(KB_ERR_ARG, "agent " + std::to_string(j) + ": non-finite position or heading");
    if (n == 0) return KB_OK;
    DeviceGuard g(f->device);
    // objects set from the host earlier come first in the write buffer
    kb_status st = flush_pending(f);
    if (st) return st;
    if ((st = materialize(f))) return st;
    if ((uint64_t)f->wn + n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "object count exceeds 2^32-16");
    const uint32_t m = (uint32_t)n;
    if ((st = grow(f, std::max(f->rn, f->wn + m)))) return st;
    set_rep_params(&f->rep, p);
    if ((st = upload_rep(f))) return st;
    KB_CUDA(launch_set_u64(f->dstep.p, step, f->stream));
    f->dstep_host = step;
    // the agents are staged in the sort temporaries (free until lazy_update)
    KB_CUDA(cudaMemcpyAsync(f->tst.p, states, sizeof(float4) * m, cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(f->tid.p, ids, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, f->stream));
    ForceArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = 1;
    a.rep0 = f->reps[0];
    a.st = f->rst.p;
    a.ids = f->rid.p;
    a.start = f->start[f->cur].p;
    a.n = f->rn;
    a.step = f->dstep.p;
    a.out_st = f->wst.p + f->wn;
    a.out_ids = f->wid.p + f->wn;
    a.out_key = f->wkey.p + f->wn;
    a.hist = f->hist.p;
    a.err = f->err.p;
    KB_CUDA(launch_flock_agents(a, f->tst.p, f->tid.p, m, p->arith == KB_ARITH_STRICT, p->query_mode,
                                f->stream));
    f->hist_counted = true;
    f->wn += m;
    f->w_from_compute = false;  // the write list is no longer one pass over the read buffer
    if (!f->density_check) f->nagents += m;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

kb_status kb_field_copy_read_buffer(kb_field* f, float* states_dev, uint32_t* ids_dev, size_t cap,
                                    size_t* n) try {
    if (!f || !n) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    kb_status st = materialize(f);
    if (st) return st;
    *n = f->rn;
    if (cap < f->rn) return fail(KB_ERR_ARG, "output capacity below the read buffer's length");
    if (f->rn == 0) return KB_OK;
    if (!states_dev || !ids_dev) return fail(KB_ERR_ARG, "null argument");
    KB_CUDA(cudaMemcpyAsync(states_dev, f->rst.p, sizeof(float4) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
    KB_CUDA(cudaMemcpyAsync(ids_dev, f->rid.p, sizeof(uint32_t) * f->rn, cudaMemcpyDeviceToDevice, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_set_states_device(kb_field* f, size_t n, const uint32_t* ids_dev,
                                     const float* states_dev) try {
    if (!f || (n && (!ids_dev || !states_dev))) return fail(KB_ERR_ARG, "null argument");
    if (n == 0) return KB_OK;
    if (!aligned16(states_dev)) return fail(KB_ERR_ARG, "states_dev is not 16-byte aligned");
    if ((uint64_t)f->wn + f->p_id.size() + n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "too many objects");
    DeviceGuard g(f->device);
    kb_status st = flush_pending(f);  // earlier single writes first (insertion order)
    if (st) return st;
    if (f->virt && (st = materialize(f))) return st;
    if ((st = grow(f, f->wn + (uint32_t)n))) return st;
    const uint32_t m = (uint32_t)n;
    KB_CUDA(cudaMemcpyAsync(f->wid.p + f->wn, ids_dev, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, f->stream));
    KB_CUDA(cudaMemsetAsync(f->small.p, 0xFF, sizeof(uint32_t), f->stream));
    KB_CUDA(launch_pack_states(f->rep, reinterpret_cast<const float4*>(states_dev), m, f->wst.p + f->wn,
                               f->wkey.p + f->wn, f->wdead.p + f->wn, f->small.p, f->stream));
    uint32_t bad = 0;
    if ((st = read_u32(f, f->small.p, &bad))) return st;
    if (bad != 0xFFFFFFFFu) {  // the write list is left as it was
        char buf[128];
        std::snprintf(buf, sizeof buf, "object %u: non-finite record or location outside the bag matrix", bad);
        return fail(KB_ERR_RANGE, buf);
    }
    f->wn += m;
    if (!f->density_check) f->nagents += n;
    f->w_from_compute = false;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_flock_next_states_device(kb_field* f, const kb_flock_params* p, uint64_t step,
                                      size_t n, const uint32_t* ids_dev, const float* states_dev,
                                      float* out_dev) try {
    if (!f || !p || (n && (!ids_dev || !states_dev || !out_dev))) return fail(KB_ERR_ARG, "null argument");
    if (f->is_batch) return fail(KB_ERR_ARG, "a batch field: agents join a batch with kb_batch_add_replica");
    std::string why;
    if (!params_ok(p, &why)) return fail(KB_ERR_ARG, why);
    if (n == 0) return KB_OK;
    if (!aligned16(states_dev) || !aligned16(out_dev)) return fail(KB_ERR_ARG, "state buffers are not 16-byte aligned");
    if (n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "object count exceeds 2^32-16");
    DeviceGuard g(f->device);
    kb_status st = flush_pending(f);
    if (st) return st;
    if ((st = materialize(f))) return st;
    const uint32_t m = (uint32_t)n;
    if ((st = grow(f, std::max(f->rn, m)))) return st;
    if (f->spare_hist.n < f->cells_cap) {
        cudaError_t e = f->spare_hist.alloc(f->cells_cap);
        if (e) return cuda_fail(e, "arrival counts");
    }
    set_rep_params(&f->rep, p);
    if ((st = upload_rep(f))) return st;
    KB_CUDA(launch_set_u64(f->dstep.p, step, f->stream));
    f->dstep_host = step;
    ForceArgs a{};
    a.reps = f->d_rep.p;
    a.nrep = 1;
    a.rep0 = f->reps[0];
    a.st = f->rst.p;
    a.ids = f->rid.p;
    a.start = f->start[f->cur].p;
    a.n = f->rn;
    a.step = f->dstep.p;
    a.out_st = reinterpret_cast<float4*>(out_dev);
    a.out_ids = f->tid.p;
    a.out_key = f->tkey.p;
    a.hist = f->spare_hist.p;
    a.err = f->err.p;
    KB_CUDA(launch_flock_agents(a, reinterpret_cast<const float4*>(states_dev), ids_dev, m,
                                p->arith == KB_ARITH_STRICT, p->query_mode, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_get_locations(kb_field* f, int32_t buffered, size_t n, const uint32_t* ids,
                                 float* states, int32_t* found) try {
    if (!f || (n && (!ids || !states || !found))) return fail(KB_ERR_ARG, "null argument");
    if (n == 0) return KB_OK;
    if (n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "too many ids");
    DeviceGuard g(f->device);
    kb_status st = buffered ? materialize(f) : flush_pending(f);
    if (st) return st;
    std::vector<uint32_t> sorted(ids, ids + n);
    std::sort(sorted.begin(), sorted.end());
    sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
    const uint32_t m = (uint32_t)sorted.size();
    DevBuf<uint32_t> dq, dfirst;
    DevBuf<float4> dout;
    cudaError_t e;
    if ((e = dq.alloc(m)) || (e = dfirst.alloc(m)) || (e = dout.alloc(m))) return cuda_fail(e, "id lookup");
    KB_CUDA(cudaMemcpyAsync(dq.p, sorted.data(), sizeof(uint32_t) * m, cudaMemcpyHostToDevice, f->stream));
    if (buffered)
        KB_CUDA(launch_find_ids(f->rid.p, nullptr, f->rst.p, f->rn, dq.p, m, dfirst.p, dout.p, f->stream));
    else
        KB_CUDA(launch_find_ids(f->wid.p, f->wdead.p, f->wst.p, f->wn, dq.p, m, dfirst.p, dout.p, f->stream));
    std::vector<uint32_t> first(m);
    std::vector<float4> out(m);
    KB_CUDA(cudaMemcpyAsync(first.data(), dfirst.p, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaMemcpyAsync(out.data(), dout.p, sizeof(float4) * m, cudaMemcpyDeviceToHost, f->stream));
    KB_CUDA(cudaStreamSynchronize(f->stream));
    for (size_t q = 0; q < n; ++q) {
        const size_t j = std::lower_bound(sorted.begin(), sorted.end(), ids[q]) - sorted.begin();
        found[q] = first[j] != 0xFFFFFFFFu ? 1 : 0;
        states[4 * q] = out[j].x;
        states[4 * q + 1] = out[j].y;
        states[4 * q + 2] = out[j].z;
        states[4 * q + 3] = out[j].w;
    }
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_remove_ids(kb_field* f, size_t n, const uint32_t* ids, size_t* removed) try {
    if (!f || (n && !ids)) return fail(KB_ERR_ARG, "null argument");
    if (removed) *removed = 0;
    if (n == 0) return KB_OK;
    if (n > 0xFFFFFFF0ull) return fail(KB_ERR_ARG, "too many ids");
    DeviceGuard g(f->device);
    kb_status st = flush_pending(f);
    if (st) return st;
    if (f->wn == 0) return KB_OK;
    std::vector<uint32_t> sorted(ids, ids + n);
    std::sort(sorted.begin(), sorted.end());
    sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
    DevBuf<uint32_t> d;
    cudaError_t e = d.alloc(sorted.size());
    if (e) return cuda_fail(e, "id list");
    KB_CUDA(cudaMemcpyAsync(d.p, sorted.data(), sizeof(uint32_t) * sorted.size(), cudaMemcpyHostToDevice, f->stream));
    KB_CUDA(cudaMemsetAsync(f->small.p, 0, sizeof(uint32_t), f->stream));
    KB_CUDA(launch_remove_ids(f->wid.p, f->wdead.p, f->wn, d.p, (uint32_t)sorted.size(), f->small.p, f->stream));
    uint32_t cnt = 0;
    if ((st = read_u32(f, f->small.p, &cnt))) return st;  // synchronises: d may be freed
    if (cnt) {
        f->w_has_dead = true;
        if (!f->density_check) f->nagents -= cnt;
    }
    if (removed) *removed = cnt;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

// Enqueue nsteps steps (force + rebuild) directly on the stream.
// Four timing events for one separate-kernel step, or -1 (timing off, the
// general rebuild, or the stream is being captured into a graph).
static int kt_begin(kb_field* f, bool fast) {
    if (!f->ktime || !fast) return -1;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(f->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return -1;
    kb_field::KtStep k;
    for (int i = 0; i < 4; ++i) {
        if (f->kt_pool.empty()) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreate(&e) != cudaSuccess) {
                cudaGetLastError();
                for (int j = 0; j < i; ++j) f->kt_pool.push_back(k.ev[j]);
                return -1;
            }
            f->kt_pool.push_back(e);
        }
        k.ev[i] = f->kt_pool.back();
        f->kt_pool.pop_back();
    }
    f->kt_pending.push_back(k);
    return (int)f->kt_pending.size() - 1;
}

}  // extern "C"

kb_status enqueue_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps, bool fast) {
    for (uint32_t s = 0; s < nsteps; ++s) {
        const int t = kt_begin(f, fast);
        if (t >= 0) KB_CUDA(cudaEventRecord(f->kt_pending[t].ev[0], f->stream));
        kb_status st = enqueue_force(f, p);
        if (st) return st;
        if (t >= 0) KB_CUDA(cudaEventRecord(f->kt_pending[t].ev[1], f->stream));
        f->wn = f->rn;
        f->kt_cur = t;
        st = fast ? fast_rebuild(f, true) : general_rebuild(f, true);
        f->kt_cur = -1;
        if (st) return st;
        if (t >= 0) KB_CUDA(cudaEventRecord(f->kt_pending[t].ev[3], f->stream));
        if (!fast) KB_CUDA(launch_add_u64(f->dstep.p, 1ull, f->stream));
        f->wn = 0;
    }
    return KB_OK;
}

extern "C" {

static kb_status flock_step_impl(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                                 uint32_t nsteps) {
    if (f && f->is_batch) return fail(KB_ERR_ARG, "a batch field: use kb_batch_step");
    if (!f || !p) return fail(KB_ERR_ARG, "null argument");
    std::string why;
    if (!params_ok(p, &why)) return fail(KB_ERR_ARG, why);
    if (f->wn || !f->p_id.empty())
        return fail(KB_ERR_STATE, "write buffer not empty: call lazy_update first");
    if (nsteps == 0) return KB_OK;
    DeviceGuard g(f->device);
    set_rep_params(&f->rep, p);
    kb_status st;
    if (f->virt && !fused_eligible(f, p) && (st = materialize(f))) return st;
    if (!f->virt && (st = grow(f, f->rn))) return st;
    if ((st = upload_rep(f))) return st;
    if (f->dstep_host != first_step) {  // the counter already holds it after consecutive calls
        KB_CUDA(launch_set_u64(f->dstep.p, first_step, f->stream));
        f->dstep_host = first_step;
    }
    uint32_t done = 0;
    if (!f->layout_is_positions) {
        // the first step after arbitrary set_object_location calls re-sorts generally
        if ((st = enqueue_steps(f, p, 1, false))) return st;
        f->layout_is_positions = true;
        done = 1;
    }
    if (done < nsteps && fused_eligible(f, p)) return tiled_steps(f, p, nsteps - done);
    if (f->virt && (st = materialize(f))) return st;
    if (small_eligible(f) && nsteps - done >= 2) {
        // a small field: whole steps in one cluster, up to 1000 per launch
        // (a single step is quicker on the separate kernels: the cluster's
        // launch, load and write-back cost more than it saves there)
        while (done < nsteps) {
            const uint32_t k = std::min<uint32_t>(1000u, nsteps - done);
            SmallArgs a{};
            a.rep = f->reps[0];
            a.st = f->rst.p;
            a.ids = f->rid.p;
            a.start = f->start[f->cur].p;
            a.n = f->rn;
            a.nsteps = k;
            a.step = f->dstep.p;
            a.err = f->err.p;
            a.self_by_slot = f->ids_unique ? 1 : 0;
            KB_CUDA(launch_small_steps(a, p->arith == KB_ARITH_STRICT, p->query_mode, f->stream));
            done += k;
        }
        return KB_OK;
    }
    occ_poll(f);
    if (f->dense_mode == KB_DENSE_AUTO && !f->occ_pending && f->steps_since_occ >= DENSE_REFRESH &&
        (st = occ_enqueue(f)))
        return st;
    const bool use_fast = all_fast_rebin_ok(f);
    // CUDA-graph replay of chunks of up to 100 steps (one graph per chunk
    // length and start parity; the graph reads the step number from device
    // memory, so one capture serves every step range).
    const uint32_t CHUNK = 100;
    while (done < nsteps) {
        const uint32_t k = std::min(CHUNK, nsteps - done);
        if (done) occ_poll(f);
        f->steps_since_occ += k;
        if (k < 4) {
            if ((st = enqueue_steps(f, p, k, use_fast))) return st;
            done += k;
            continue;
        }
        kb_field::GraphKey key;
        key.steps = k;
        key.parity = f->cur;
        key.params.assign((const uint8_t*)f->reps.data(), (const uint8_t*)f->reps.data() + sizeof(Rep) * f->reps.size());
        key.params.push_back((uint8_t)p->arith);
        key.params.push_back((uint8_t)(f->rn & 0xff));
        key.params.push_back((uint8_t)((f->rn >> 8) & 0xff));
        key.params.push_back((uint8_t)((f->rn >> 16) & 0xff));
        key.params.push_back((uint8_t)((f->rn >> 24) & 0xff));
        key.params.push_back((uint8_t)f->dense);
        auto it = f->graphs.find(key);
        const int cur0 = f->cur;
        if (it == f->graphs.end()) {
            cudaGraph_t graph = nullptr;
            KB_CUDA(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
            st = enqueue_steps(f, p, k, use_fast);
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
            if (f->graphs.size() > 16) f->drop_graphs();
            it = f->graphs.emplace(key, exec).first;
            f->cur = cur0;  // capture recorded the swaps; replay performs them
        }
        KB_CUDA(cudaGraphLaunch(it->second, f->stream));
        f->cur = (k & 1u) ? 1 - cur0 : cur0;
        done += k;
    }
    return KB_OK;
}

kb_status kb_field_set_kernel_timing(kb_field* f, int32_t enable) try {
    if (!f) return fail(KB_ERR_ARG, "null argument");
    f->ktime = enable != 0;
    return KB_OK;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_field_kernel_times(kb_field* f, double ms[3], uint64_t* steps) try {
    if (!f || !ms || !steps) return fail(KB_ERR_ARG, "null argument");
    DeviceGuard g(f->device);
    ms[0] = ms[1] = ms[2] = 0.0;
    *steps = 0;
    kb_status st = KB_OK;
    for (auto& k : f->kt_pending) {
        cudaError_t e = cudaEventSynchronize(k.ev[3]);
        float t[3] = {0.f, 0.f, 0.f};
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&t[i], k.ev[i], k.ev[i + 1]);
        if (e != cudaSuccess) {
            if (!st) st = cuda_fail(e, "kernel timing events");
            cudaGetLastError();
        } else {
            for (int i = 0; i < 3; ++i) ms[i] += t[i];
            ++*steps;
        }
        for (cudaEvent_t ev : k.ev) f->kt_pool.push_back(ev);
    }
    f->kt_pending.clear();
    return st;
} catch (...) {
    return kb::exception_status();
}

kb_status kb_flock_step(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                        uint32_t nsteps) try {
    kb_status st = flock_step_impl(f, p, first_step, nsteps);
    if (f) f->dstep_host = st ? ~0ull : first_step + nsteps;  // unknown after a failure
    return st;
} catch (...) {
    return kb::exception_status();
}

}  // extern "C"
