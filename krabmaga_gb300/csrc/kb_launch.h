// kb_launch.h -- host-side launchers of the kernels in kb_kernels.cu.  Every
// launcher enqueues on the given stream and returns the launch error.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kb_common.h"

namespace kb {

// Scan workspace: a tile counter, a finish counter and an epoch that tags
// the per-tile look-back words, so the scan needs no reset between launches
// (and replays correctly inside a CUDA graph).
struct ScanCtl {
    uint32_t tile_counter;
    uint32_t done_counter;
    uint32_t epoch;
    uint32_t _pad;
};
constexpr uint32_t SCAN_TILE = 4096;  // items per CTA (256 threads x 16)
inline uint32_t scan_tiles(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }
// Items per tile of the two-pass scan (inputs of up to SCAN2_MAX_TILES tiles).
#ifndef KB_SCAN2_ITEMS
#define KB_SCAN2_ITEMS 4
#endif
constexpr uint32_t SCAN2_TILE = 256u * KB_SCAN2_ITEMS;
#ifndef KB_SCAN2_MAX
#define KB_SCAN2_MAX 4096
#endif
constexpr uint32_t SCAN2_MAX_TILES = KB_SCAN2_MAX;
// Above SCAN2_MAX_TILES tiles a third launch scans the tile sums (up to
// SCAN3_MAX_TILES tiles, about 268 M bags); beyond it the look-back scan.
#ifndef KB_SCAN3_MAX
#define KB_SCAN3_MAX 262144
#endif
constexpr uint32_t SCAN3_MAX_TILES = KB_SCAN3_MAX;
// 64-bit state words a scan of n items needs (either form).
inline uint32_t scan_state_words(uint32_t n) {
    const uint32_t a = scan_tiles(n), b = (n + SCAN2_TILE - 1) / SCAN2_TILE;
    return (a > b ? a : b) + 1u;
}

// Bounded device waits: the iterations a wait makes before it gives up and
// raises ERR_SPIN_TIMEOUT (0: the kernel's default), and a test hook that
// makes one publisher (a look-back scan tile, a persistent block at its first
// grid barrier) withhold its signal so that a wait runs out on purpose
// (~0u: none).
struct WaitCfg {
    uint32_t spin_limit;
    uint32_t withhold;
};
constexpr WaitCfg WAIT_DEFAULT = {0u, 0xFFFFFFFFu};

// Exclusive scan of in[0..n) into out[0..n]; out[n] = total.  When zero_in,
// in[] is cleared as it is read (the histogram is ready for the next step).
cudaError_t launch_scan(const uint32_t* in, uint32_t* out, uint32_t n, ScanCtl* ctl,
                        unsigned long long* tile_state, uint32_t* err, bool zero_in,
                        cudaStream_t s, WaitCfg wait = WAIT_DEFAULT);

// Flock step agent pass: reads the canonical read buffer (st, ids, start),
// writes next states into the write list in the same order plus each one's
// new bag key, and counts keys into hist.
struct ForceArgs {
    const Rep* reps;
    int32_t nrep;
    Rep rep0;  // the single replica, read from the parameter bank when nrep == 1
    const float4* st;
    const uint32_t* ids;
    const uint32_t* start;
    uint32_t n;
    const unsigned long long* step;
    float4* out_st;
    uint32_t* out_ids;
    uint32_t* out_key;
    uint32_t* hist;
    uint32_t* err;
    int32_t check_moves;  // flag moves the stencil-gather rebin cannot follow
    // several replicas: one block per entry {replica, first boid}; no block
    // spans two replicas (built by the host with the replica table)
    const uint2* blk;
    uint32_t nblk;
    // ids are unique within every replica: a candidate is the boid itself
    // exactly when it is the boid's own slot, so no id is loaded per candidate
    int32_t self_by_slot;
    // long candidate lists (dense flocks, single replica): walk each column
    // run with a plain pointer instead of the flat index formula (the same
    // visiting order, fewer instructions per candidate)
    int32_t dense;
    // several replicas: threads per block of the block table (FORCE_BLOCKS_*;
    // 0: FORCE_THREADS), the launch shape the batch autotuner picks
    uint32_t block_threads;
};
constexpr int FORCE_THREADS = 256;  // the force kernel's block (one replica per block)
// Block sizes of the force pass over packed replicas (one replica per block).
constexpr int FORCE_BLOCK_SIZES[3] = {128, 256, 512};
cudaError_t launch_flock_force(const ForceArgs& a, bool strict, int qmode, cudaStream_t s);
// Whole steps of a small single-replica field in one cluster of SMALL_CTAS
// blocks (kb_small.cu): every block loads the read buffer (st, ids, start
// over rep.ncells bags) into its shared memory, nsteps steps run there, and
// the final read buffer, offsets and step counter (*step += nsteps) are
// written back.
constexpr int SMALL_THREADS = 1024;
constexpr uint32_t SMALL_CTAS = 8;  // a portable cluster size
// Measured on GB300 (uniform flocks, 400-step calls): 4.8 / 7.0 / 9.3 / 13.9 us
// per step at 16 / 1000 / 2048 / 4096 boids, against 13.5 / 14.2 / 14.7 /
// 15.4 us for the separate kernels; the bound is the shared memory.
constexpr uint32_t SMALL_MAX_BOIDS = 4096;
constexpr uint32_t SMALL_MAX_CELLS = 4096;
struct SmallArgs {
    Rep rep;
    float4* st;
    uint32_t* ids;
    uint32_t* start;
    uint32_t n;
    uint32_t nsteps;
    unsigned long long* step;
    uint32_t* err;
    int32_t self_by_slot;
};
size_t small_smem_bytes(uint32_t n, uint32_t ncells);
cudaError_t launch_small_steps(const SmallArgs& a, bool strict, int qmode, cudaStream_t s);

// Bird::step of nin caller-given agents (in_st {x, y, dx, dy}, in_ids) against
// the read buffer of a single replica; agent j's next state, id and bag key
// go to slot j of a.out_st / a.out_ids / a.out_key, its arrival into a.hist.
cudaError_t launch_flock_agents(const ForceArgs& a, const float4* in_st, const uint32_t* in_ids,
                               uint32_t nin, bool strict, int qmode, cudaStream_t s);

// Stencil-gather rebin: builds the canonical read buffer of the next step
// from the write list (in the previous canonical order) and the scanned
// histogram.  Bumps *step when step != nullptr.  With key == nullptr each
// record's bag is recomputed from its position.
struct RebinArgs {
    const Rep* reps;
    int32_t nrep;
    Rep rep0;  // the single replica when nrep == 1
    const uint32_t* start_cur;
    const uint32_t* start_next;
    const uint32_t* key;
    const float4* a_st;
    const uint32_t* a_ids;
    uint32_t ncells;
    uint32_t nsegs;  // column segments over all replicas (0: per-bag kernel only)
    int32_t seg_rows;  // bags per segment of a single replica: 0 (SEG_ROWS) or DENSE_SEG_ROWS
    // several replicas: one block per entry {replica, first segment}, up to
    // REBIN_SEG_WARPS segments of that replica
    const uint2* sblk;
    uint32_t nsblk;
    float4* s_st;
    uint32_t* s_ids;
    unsigned long long* step;
    uint32_t* err;
    uint32_t n;  // records (every slot index is below it)
};
// Bag segments of the segment rebin: SEG_ROWS consecutive bags of one column.
constexpr int SEG_ROWS = 32;
// Shorter segments for dense flocks: a segment's source runs are long there,
// and the warp walks them in order, so fewer rows per warp shorten the tail.
constexpr int DENSE_SEG_ROWS = 8;
constexpr int REBIN_SEG_WARPS = 8;  // segments (warps) per block
// Segments of the replicas of a packed batch: 64 bags (two per lane), half
// as many segments as 32-bag ones (the packed rebin's time follows the
// number of segments; measured on the 512-replica sweep).
constexpr int PACKED_SEG_ROWS = 64;
// rows 0: the replica's own segment height (Rep::seg_rows, else SEG_ROWS).
inline uint32_t rep_segments(const Rep& R, int rows = 0) {
    if (rows == 0) rows = R.seg_rows > 0 ? R.seg_rows : SEG_ROWS;
    return (uint32_t)R.dw * (((uint32_t)R.dh + (uint32_t)rows - 1) / (uint32_t)rows);
}
cudaError_t launch_rebin(const RebinArgs& a, cudaStream_t s);
// *out += sum over bags of (start[c+1] - start[c])^2 (the caller zeroes *out).
cudaError_t launch_occupancy_sq(const uint32_t* start, uint32_t ncells, unsigned long long* out,
                                cudaStream_t s);
// Whether any (replica, id) pair repeats in the read buffer (n boids, nrep
// replicas by boid_off): an open-addressing table of cap (a power of two,
// >= 2n) 64-bit words, cleared here; *dup is set to 1 on a repeat.
cudaError_t launch_dup_check(const Rep* reps, int32_t nrep, const uint32_t* ids, uint32_t n,
                             unsigned long long* table, uint32_t cap, uint32_t* dup,
                             cudaStream_t s);
// out[4r..4r+3] = {boids, sum dx, sum dy, sum |(dx,dy)|} of replica r's read buffer.
cudaError_t launch_moments(const Rep* reps, uint32_t nrep, const uint32_t* start, const float4* st,
                           double* out, cudaStream_t s);

// Bulk set_object_location on the device: n objects at their own positions
// (xy and dxy as float2 arrays) appended to the write list as records, bag
// keys and live marks; *bad takes the smallest index of an object with a
// non-finite value or a location outside the bag matrix (~0u when none).
cudaError_t launch_pack_locations(const Rep& rep, const float2* xy, const float2* dxy, uint32_t n,
                                  float4* out_st, uint32_t* out_key, uint8_t* out_dead,
                                  uint32_t* bad, cudaStream_t s);
// The same for records already packed as float4 {x, y, last_d} on the device.
cudaError_t launch_pack_states(const Rep& rep, const float4* st, uint32_t n, float4* out_st,
                               uint32_t* out_key, uint8_t* out_dead, uint32_t* bad, cudaStream_t s);

// General stable counting sort of the write list by key (insertion order
// kept inside each bag): histogram, scatter, per-bag canonicalisation.
cudaError_t launch_hist_list(const uint32_t* key, const uint8_t* dead, uint32_t n, uint32_t* hist,
                             cudaStream_t s);
cudaError_t launch_scatter_list(const uint32_t* key, const uint8_t* dead, const float4* st,
                                const uint32_t* ids, uint32_t n, const uint32_t* start,
                                uint32_t* cursor, float4* t_st, uint32_t* t_ids, uint32_t* t_src,
                                cudaStream_t s);
cudaError_t launch_canon(const uint32_t* start, uint32_t ncells, const float4* t_st,
                         const uint32_t* t_ids, const uint32_t* t_src, uint32_t* cursor,
                         float4* s_st, uint32_t* s_ids, cudaStream_t s);

// Field2D queries over the read buffer of a single replica.
//   mode 0: counts only (+ digest when digest != nullptr)
//   mode 1: fill ids/states at offsets[q]
struct QueryArgs {
    Rep rep;
    int32_t kind;  // 0 relax, 1 exact
    float dist;
    const uint32_t* start;
    const float4* st;
    const uint32_t* ids;
    uint32_t nq;
    const float2* q;
    uint32_t* counts;
    uint32_t* digest;
    const uint32_t* offsets;
    uint32_t* out_ids;
    float4* out_st;
    uint64_t cap;
};
cudaError_t launch_query(const QueryArgs& a, cudaStream_t s);

// Ordered filter of the write list: entries with key == target and not dead,
// in list order; writes ids/states (up to cap) and the count.
cudaError_t launch_filter_key(const uint32_t* key, const uint8_t* dead, const float4* st,
                              const uint32_t* ids, uint32_t n, uint32_t target, uint32_t* out_ids,
                              float4* out_st, uint64_t cap, uint32_t* out_count, cudaStream_t s);
// Mark write-list entries (key == target, id == id, live) dead; adds the
// number marked to *removed.
cudaError_t launch_remove(const uint32_t* key, uint8_t* dead, const uint32_t* ids, uint32_t n,
                          uint32_t target, uint32_t id, uint32_t* removed, cudaStream_t s);
// For each id sorted[j] (ascending, distinct): first[j] = the first index i
// < n with ids[i] == sorted[j] (skipping dead entries when dead != nullptr),
// ~0u when none, and out[j] = st[first[j]] (zeros when none).
cudaError_t launch_find_ids(const uint32_t* ids, const uint8_t* dead, const float4* st, uint32_t n,
                            const uint32_t* sorted, uint32_t m, uint32_t* first, float4* out,
                            cudaStream_t s);
// Mark live write-list entries whose id is in sorted[0..m) (ascending) dead;
// adds the number marked to *removed.
cudaError_t launch_remove_ids(const uint32_t* ids, uint8_t* dead, uint32_t n, const uint32_t* sorted,
                              uint32_t m, uint32_t* removed, cudaStream_t s);
// Empty bags of the read buffer in index order, as (i*d, j*d).
cudaError_t launch_empty_bags(const Rep& rep, const uint32_t* start, float2* out, uint64_t cap,
                              uint32_t* out_count, cudaStream_t s);
// Bag index of every stored object (read buffer), for iteration.
cudaError_t launch_cell_of(const uint32_t* start, uint32_t ncells, uint32_t* cell_of,
                           cudaStream_t s);
// (i*d, j*d) of the bag of each object.
cudaError_t launch_cell_xy(const Rep& rep, const uint32_t* cell_of, uint32_t n, float2* out,
                           cudaStream_t s);

// Repacking plan for a continuous batch: each entry fills write-list slots
// [dst_off, dst_off+n) for replica `rep`, either copying its canonical
// records from the read buffer (kind 0, from src_off) or generating its
// initial uniform flock (kind 1: kb_gen_uniform's draws, bit for bit).
struct PackEntry {
    uint32_t dst_off, n, rep, src_off;
    uint32_t kind, seed_lo, seed_hi;
    float heading_scale;
};
cudaError_t launch_repack(const PackEntry* plan, int32_t nplan, uint32_t total, const Rep* reps,
                          const float4* src_st, const uint32_t* src_ids, float4* dst_st,
                          uint32_t* dst_ids, uint32_t* dst_key, uint8_t* dst_dead, uint32_t* err,
                          cudaStream_t s);

}  // namespace kb
