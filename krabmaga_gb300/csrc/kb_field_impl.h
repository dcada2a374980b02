// kb_field_impl.h -- the field handle behind include/krabgpu.h and the host
// runtime functions that kb_api.cpp (fields and steps), kb_batch.cpp
// (replica batches) and kb_server.cpp (serving) share.  Internal: not part
// of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/krabgpu.h"
#include "kb_common.h"
#include "kb_fused.h"
#include "kb_launch.h"
#include "kb_runtime.h"

using namespace kb;

struct kb_field {
    int device = 0;
    cudaStream_t stream = nullptr;
    Rep rep{};                  // replica 0: the plain field's geometry + last parameters
    std::vector<Rep> reps;      // every replica (a plain field holds one, == rep)
    uint32_t ncells_total = 0;  // bags over all replicas
    uint32_t cells_cap = 0;     // bag arrays are sized for this many bags
    Rep rep_uploaded{};         // last replica record written to the device (plain fields)
    bool rep_valid = false;
    unsigned long long dstep_host = 0;  // the device step counter once queued work has run
    bool is_batch = false;
    DevBuf<Rep> d_rep;
    // read buffer
    uint32_t cap = 0;
    DevBuf<float4> rst;
    DevBuf<uint32_t> rid;
    DevBuf<uint32_t> start[2];
    int cur = 0;
    uint32_t rn = 0;
    // write list
    DevBuf<float4> wst;
    DevBuf<uint32_t> wid, wkey;
    DevBuf<uint8_t> wdead;
    uint32_t wn = 0;
    bool w_from_compute = false;   // write list == one flock pass over the read buffer
    bool w_has_dead = false;
    bool layout_is_positions = true;  // every stored bag == discretize(own pos)
    std::vector<float4> p_st;
    std::vector<uint32_t> p_id, p_key;
    bool p_loc_differs = false;
    // step temporaries
    DevBuf<uint32_t> hist, cursor, tid, tsrc, rkey, tkey;
    bool hist_counted = false;  // a force pass has counted arrivals into hist (no scan since)
    // Every replica's ids are distinct in the read buffer (checked on the
    // device after each general rebuild; the step paths keep the id multiset)
    bool ids_unique = false;
    DevBuf<unsigned long long> dup_tab;
    // Several replicas: block tables of the force and segment-rebin kernels
    // ({replica, first boid} / {replica, first segment}), no block spanning
    // two replicas; rebuilt with the replica table.
    DevBuf<uint2> blk_force, blk_seg;
    std::vector<uint2> blk_force_h, blk_seg_h;
    uint32_t nblk_force = 0, nblk_seg = 0;
    uint32_t force_block = FORCE_THREADS;  // threads per force block over packed replicas
    DevBuf<float4> tst;
    // arrival counts of kb_flock_next_states_device's agents (written, never read)
    DevBuf<uint32_t> spare_hist;
    DevBuf<ScanCtl> scan_ctl, aux_ctl;
    DevBuf<unsigned long long> tstate, aux_tstate;
    uint32_t aux_tiles = 0;
    DevBuf<uint32_t> err;
    DevBuf<unsigned long long> dstep;
    DevBuf<uint32_t> small;  // 16 words of scratch for counts
    // Field2D bookkeeping (field_2d.rs:276, 284-287)
    size_t nagents = 0;
    bool density_check = false;
    // graphs: (steps per graph, start parity, params) -> exec
    struct GraphKey {
        uint32_t steps;
        int parity;
        std::vector<uint8_t> params;
        bool operator<(const GraphKey& o) const {
            if (steps != o.steps) return steps < o.steps;
            if (parity != o.parity) return parity < o.parity;
            return params < o.params;
        }
    };
    std::map<GraphKey, cudaGraphExec_t> graphs;
    // split-step graphs: (steps, cur, a_last, virt) -> exec + end state
    struct SGraph {
        cudaGraphExec_t exec;
        int cur, a_last;
    };
    std::map<std::vector<uint32_t>, SGraph> sgraphs;
    // Bumped whenever the graphs above are dropped (buffers reallocated, the
    // fused configuration rebuilt): graphs cached outside the field over its
    // buffers (a batch's) are stale once it moves.
    uint64_t graph_epoch = 0;
    // persistent fused step (kb_fused.cu)
    struct Fused {
        bool ready = false;
        uint32_t n = 0;
        int strict = -1, qmode = -1, dd = -1;
        FusedCfg cfg{};
        uint32_t nctas = 0;
        uint32_t ntiles = 0;
        DevBuf<Tile> tiles;
        DevBuf<float4> g_st;
        DevBuf<uint32_t> g_ids;
        DevBuf<unsigned long long> scan_state;
        DevBuf<uint32_t> ctl;  // [0] tile counter, [1..2] barrier, [3] scan epoch, [4] overflow tiles
        DevBuf<unsigned long long> phase_cycles;  // per-CTA phase clocks when profiling
        bool profile = false;
        bool occ_valid = false;  // cached occupancy of the last configuration
        FusedCfg occ_cfg{};
        int occ_strict = -1, occ_qmode = -1, occ_ctas = 0;
    } fused;
    // 0 separate kernels (small fields: one block, kb_small.cu), 1 persistent
    // fused, 2 split tile step, 3 separate kernels whatever the size
    int fused_mode = 0;
    // Bounded device waits (kb_field_set_wait_test): iterations before a wait
    // gives up (0: each kernel's default), and the test hook that makes one
    // publisher withhold its signal (KB_WITHHOLD_*, at index withhold_index).
    uint32_t wait_spins = 0;
    int32_t withhold_kind = KB_WITHHOLD_NONE;
    uint32_t withhold_index = 0;
    // Per-kernel timing of ungraphed separate-kernel steps: four events per
    // step (force | scan | rebin), read and recycled by kb_field_kernel_times.
    bool ktime = false;
    struct KtStep {
        cudaEvent_t ev[4];
    };
    std::vector<cudaEvent_t> kt_pool;
    std::vector<KtStep> kt_pending;
    int kt_cur = -1;  // step whose scan|rebin boundary fast_rebuild records
    // After fused steps the read buffer can stay virtual: the last write list
    // (in buffer a_last: 0 rst, 1 wst, 2 tst) plus start[1-cur] (its bag
    // offsets) and start[cur] (the read buffer's bag offsets).
    bool virt = false;
    int a_last = 0;
    bool keys_valid = false;  // buf_key(a_last) holds the bag keys of the virtual write list
    int32_t tile_tx = 0, tile_ty = 0;  // 0: automatic
    // Dense flocks (long candidate lists, single replica): the force pass
    // walks each column run with a pointer and the rebin takes 8-bag
    // segments.  Chosen (dense_mode KB_DENSE_AUTO) from the read buffer's sum
    // of squared bag occupancies, about 9 * sum / N candidates per boid,
    // measured after every general rebuild and every DENSE_REFRESH steps
    // (read back without blocking).  Both paths give the same bits.
    int32_t dense_mode = KB_DENSE_AUTO;
    bool dense = false;
    DevBuf<unsigned long long> occ_dev;
    unsigned long long* occ_host = nullptr;  // pinned
    cudaEvent_t occ_ev = nullptr;
    bool occ_pending = false;
    uint32_t occ_n = 0;  // boids when the pending measurement was taken
    uint64_t steps_since_occ = 0;

    ~kb_field() {
        drop_graphs();
        if (stream) cudaStreamSynchronize(stream);
        if (occ_ev) cudaEventDestroy(occ_ev);
        if (occ_host) cudaFreeHost(occ_host);
        for (auto& k : kt_pending)
            for (cudaEvent_t e : k.ev) cudaEventDestroy(e);
        for (cudaEvent_t e : kt_pool) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
    void drop_graphs() {
        graph_epoch++;
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        for (auto& kv : sgraphs) cudaGraphExecDestroy(kv.second.exec);
        sgraphs.clear();
    }
};

// Makes a device current for a scope and restores the previous one.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int now = -1;
        cudaGetDevice(&now);
        if (prev >= 0 && now != prev) cudaSetDevice(prev);
    }
};

#define KB_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// ---- shared host runtime (defined in kb_api.cpp)
namespace kb {
extern thread_local std::string g_last_error;  // kb_last_error()'s message for this thread
// Host copy of discretize + bag index (field_2d.rs:328-339): -1 outside the matrix.
int64_t host_bag_index(const Rep& R, float x, float y);
// Field2D::new geometry (field_2d.rs:304-322) into R; false with *why on bad input.
bool make_rep_geometry(float w, float h, float d, int toroidal, Rep* R, std::string* why,
                       int cell_wrap = KB_CELL_WRAP_CLAMP);
void set_rep_params(Rep* R, const kb_flock_params* p);
bool params_ok(const kb_flock_params* p, std::string* why);
}  // namespace kb

// Allocate a field over a replica table (cell_off / boid_off already set).
kb_status field_new(int device, const std::vector<Rep>& reps, bool is_batch, uint32_t capacity,
                    kb_field** out, uint32_t cells_cap = 0);
// Object storage for at least `need` records / bag arrays for `need` bags.
kb_status grow(kb_field* f, uint32_t need);
kb_status grow_cells(kb_field* f, uint64_t need);
// Replace the replica table (contents rebuilt by the caller) / upload it.
kb_status field_set_reps(kb_field* f, const std::vector<Rep>& reps);
kb_status upload_rep(kb_field* f);
// Rebuild a virtual read buffer (after tiled steps).
kb_status materialize(kb_field* f);
// The general stable sort of the write list into the read buffer.
kb_status general_rebuild(kb_field* f, bool counted);
// Field::lazy_update (field_2d.rs:905-921).
kb_status field_lazy_update(kb_field* f);
// nsteps steps on the separate kernels (fast: the stencil-gather rebin).
kb_status enqueue_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps, bool fast);
bool all_fast_rebin_ok(const kb_field* f);
// The tiled step paths (step modes 1 and 2) and whether a field may take them.
bool fused_eligible(const kb_field* f, const kb_flock_params* p);
kb_status fused_prepare(kb_field* f, const kb_flock_params* p);
kb_status fused_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps);
kb_status tiled_steps(kb_field* f, const kb_flock_params* p, uint32_t nsteps);
kb_status split_steps_graphed(kb_field* f, const kb_flock_params* p, uint32_t nsteps, uint32_t chunk);
// Time steps_per_trial real steps (run(ctx, first, n)) under each candidate
// tile shape of the tiled paths and keep the fastest.
kb_status autotune_tiles(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                         uint32_t steps, const int32_t* cand, int32_t ncand, int32_t* best_out,
                         float* best_ms_out, kb_status (*run)(void*, uint64_t, uint32_t),
                         void* ctx);
// The same over the force pass's block size of packed replicas (separate
// kernels): candidates are pairs {threads, replicas per block}, threads one of
// FORCE_BLOCK_SIZES and one replica per block (nullptr: every block size).
kb_status autotune_force_block(kb_field* f, uint64_t first_step, uint32_t steps,
                               const int32_t* cand, int32_t ncand, int32_t* best_out,
                               float* best_ms_out, kb_status (*run)(void*, uint64_t, uint32_t),
                               void* ctx);
// Whether every replica's ids are distinct (checked on the device) / set it.
kb_status check_unique_ids(kb_field* f);
void set_ids_unique(kb_field* f, bool u);
// Reset the control words of the bounded-wait protocols (after a timeout).
kb_status reset_wait_state(kb_field* f);
// Synchronous reads: one device word; the device error word as a status.
kb_status read_u32(kb_field* f, const uint32_t* dptr, uint32_t* out);
kb_status check_flags(kb_field* f);
