// kb_fused.h -- the persistent flock step (kb_fused.cu): configuration,
// shared-memory layout and launcher.
//
// One cooperative launch runs `nsteps` whole steps.  The bag matrix of every
// replica is cut into tiles of tx x ty bags; each step, the CTAs take tiles
// from a counter and for each one
//   1. TMA-stage the previous step's write list (its records sit in the
//      previous canonical order) for the tile's bags plus a two-bag ring and
//      the seam lines,
//   2. rebin those records in shared memory into this step's canonical order
//      (a bag's arrivals gathered in write-list order: the reference's bag
//      insertion order),
//   3. run Bird::step for the tile's own boids from shared memory and write
//      the next states at their canonical slots, counting the new bags in a
//      shared histogram flushed with one atomic per touched bag,
// then a grid barrier, the scan of the histogram into the next bag offsets
// (decoupled look-back across CTAs), and another grid barrier.  Tiles whose
// records exceed the shared-memory capacity run the same steps through a
// global scratch buffer instead.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kb_common.h"
#include "kb_launch.h"

namespace kb {

constexpr int FUSED_THREADS = 256;
constexpr int FUSED_DD_MAX = 2;  // largest query ring (floor(radius/d)) the fused kernel takes

struct Tile {
    uint32_t rep;
    uint16_t x0, y0;
};

struct FusedCfg {
    int32_t tx, ty;      // tile shape in bags
    int32_t dd;          // largest query ring over the replicas (0..FUSED_DD_MAX)
    uint32_t stage_cap;  // staged records per CTA
    uint32_t sord_cap;   // canonical-order records per CTA
};

struct FusedLayout {
    uint32_t off_mbar, off_stage_st, off_sord_st, off_stage_ids, off_stage_key, off_sord_ids;
    uint32_t off_seg, off_cell_lo, off_cell_cnt, off_stt, off_colblk, off_owned, off_hist;
    uint32_t off_srcx, off_nsrcx, off_srcy, off_nsrcy, off_sord_cell;
    uint32_t total;
    int32_t maxlx, maxly, maxqx, maxqy, maxseg, maxhx, maxhy;
};

KB_HD uint32_t fused_align(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

KB_HD FusedLayout fused_layout(const FusedCfg& c) {
    FusedLayout L;
    L.maxqx = c.tx + 2 * c.dd;
    L.maxqy = c.ty + 2 * c.dd;
    L.maxlx = L.maxqx + 2 + 6;  // rebin ring + seam lines (line 0, up to 5 high lines)
    L.maxly = L.maxqy + 2 + 6;
    L.maxseg = L.maxlx * 3;     // per staged column: up to three row runs
    L.maxhx = c.tx + 2;
    L.maxhy = c.ty + 2;
    uint32_t o = 0;
    L.off_mbar = o; o += 16;
    L.off_stage_st = o; o += c.stage_cap * 16u;
    L.off_sord_st = o; o += c.sord_cap * 16u;
    L.off_stage_ids = o; o += c.stage_cap * 4u;
    L.off_stage_key = o; o += c.stage_cap * 4u;
    L.off_sord_ids = o; o += c.sord_cap * 4u;
    o = fused_align(o, 16);
    L.off_seg = o; o += (uint32_t)L.maxseg * 16u;
    L.off_cell_lo = o; o += (uint32_t)(L.maxlx * L.maxly) * 4u;
    L.off_cell_cnt = o; o += (uint32_t)(L.maxlx * L.maxly) * 4u;
    L.off_stt = o; o += (uint32_t)(L.maxqx * (L.maxqy + 1)) * 4u;
    L.off_colblk = o; o += (uint32_t)(L.maxqx + 1) * 4u;
    L.off_owned = o; o += (uint32_t)(c.tx + 1) * 4u;
    L.off_hist = o; o += (uint32_t)(L.maxhx * L.maxhy) * 4u;
    L.off_srcx = o; o += (uint32_t)L.maxqx * 8u;        // staged column indices per column
    L.off_nsrcx = o; o += (uint32_t)L.maxqx;
    o = fused_align(o, 4);
    L.off_srcy = o; o += (uint32_t)L.maxqy * 4u * 2u;   // (first, last) staged row runs per row
    L.off_nsrcy = o; o += (uint32_t)L.maxqy;
    o = fused_align(o, 4);
    L.off_sord_cell = o; o += c.sord_cap * 2u;          // region-local bag per record
    L.total = fused_align(o, 16);
    return L;
}

struct FusedArgs {
    const Rep* reps;
    int32_t nrep;
    const Tile* tiles;
    uint32_t ntiles;
    FusedCfg cfg;
    uint32_t ncells;  // all replicas
    uint32_t n;       // all boids
    // step s reads A_{s-1} (a_in at s = 0, then a_st[(s-1)&1]) and writes a_st[s&1]
    const float4* a_in_st;
    const uint32_t* a_in_ids;
    float4* a_st[2];
    uint32_t* a_ids[2];
    // bag offsets: at step s, previous = start_b[s&1], current = start_b[(s+1)&1];
    // the scan of step s writes the next offsets over the previous ones
    uint32_t* start_b[2];
    uint32_t* hist;
    float4* g_sord_st;  // canonical-order scratch for tiles over capacity (n records)
    uint32_t* g_sord_ids;
    unsigned long long* step;  // first step number; advanced by nsteps
    uint32_t nsteps;
    uint32_t* tile_counter;
    uint32_t* bar;  // [0] arrivals, [1] generation
    unsigned long long* scan_state;  // one look-back word per CTA
    uint32_t* scan_epoch;
    uint32_t* err;
    uint32_t* stats;  // [0] tiles that ran through the global scratch path
    unsigned long long* phase_cycles;  // optional [gridDim][16] cycle counters per phase
    // bounded waits: iterations before a wait gives up (0: the defaults), and
    // the test hook: block `withhold` of the persistent kernel leaves before
    // its first grid barrier (~0u: none)
    WaitCfg wait;
};

// Largest CTA count that can be co-resident for this layout (0 if none).
int fused_max_ctas(const FusedCfg& cfg, bool strict, int qmode, int device);
cudaError_t launch_fused(const FusedArgs& a, bool strict, int qmode, uint32_t nctas,
                         cudaStream_t s);
// One step, one CTA per tile (the split form): reads the previous write list
// (prev_*, its bag keys prev_key or nullptr to recompute them) with its bag
// offsets start_prev, writes the next one (and its keys) at the canonical
// slots of start_cur and counts the new bags into a.hist.  The
// step number is *a.step + step_offset.  The scan of a.hist follows as its
// own launch.
cudaError_t launch_tile_step(const FusedArgs& a, const float4* prev_st, const uint32_t* prev_ids,
                             const uint32_t* prev_key, float4* next_st, uint32_t* next_ids,
                             uint32_t* next_key, const uint32_t* start_prev,
                             const uint32_t* start_cur, uint32_t step_offset, bool strict, int qmode,
                             cudaStream_t s);

}  // namespace kb
