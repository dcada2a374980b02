// kb_fused.cu -- the persistent flock step (see kb_fused.h for the plan).
//
// Index discipline: every shared-memory table is sized by fused_layout() for
// the configured tile shape and ring; every access below is to a region whose
// extent was checked against those maxima (or against stage_cap / sord_cap,
// falling back to the global scratch path when a tile is over capacity).
// Every wait (TMA mbarrier, grid barrier, look-back) is bounded and raises
// ERR_SPIN_TIMEOUT on expiry, after which the kernel returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kb_common.h"
#include "kb_device.cuh"
#include "kb_fused.h"

namespace kb {
namespace {

constexpr int FT = FUSED_THREADS;
constexpr uint32_t BAR_SPINS = 1u << 22;
constexpr uint32_t TMA_SPINS = 1u << 20;
constexpr uint32_t LB_SPINS = 1u << 22;
constexpr unsigned long long LB_AGG = 1ull, LB_INC = 2ull;

struct Seg {
    uint32_t glo, cnt, soff, pad;
};

struct TileCtx {
    int32_t rep, dd;
    int32_t X0, X1, Y0, Y1;          // owned bags [X0,X1) x [Y0,Y1)
    int32_t qx0, qx1, qy0, qy1;      // canonical-order region (inclusive)
    int32_t nqx, nqy;
    // staged lines: up to three disjoint ascending runs of line values
    // [lo, hi] (the low seam line 0, the main run, the high seam run), run r
    // starting at staged index off[r]
    int32_t xlo[3], xhi[3], xoff[3], nxr, nsx;
    int32_t ylo[3], yhi[3], yoff[3], nyr, nsy;
    int32_t hx0, hy0, hnx, hny;      // shared histogram region
    uint32_t nseg, staged, sord, owned;
    int32_t overflow;
};

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t sptr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sptr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sptr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(sptr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         unsigned long long* bar) {
    unsigned long long g;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            sptr(dst)),
        "l"(g), "r"(bytes), "r"(sptr(bar))
        : "memory");
}

// ------------------------------------------------------------ small helpers
// Staged index of line value v (-1 if not staged) / value of staged index i.
__device__ __forceinline__ int run_index(int v, const int32_t* lo, const int32_t* hi,
                                         const int32_t* off, int nr) {
    for (int r = 0; r < nr; ++r)
        if (v >= lo[r] && v <= hi[r]) return off[r] + (v - lo[r]);
    return -1;
}
__device__ __forceinline__ int run_value(int i, const int32_t* lo, const int32_t* hi,
                                         const int32_t* off, int nr, int* run) {
    int r = 0;
    while (r + 1 < nr && i >= off[r + 1]) ++r;
    *run = r;
    return lo[r] + (i - off[r]);
}

// Staged lines for a canonical region [q0, q1] of lines 0..maxv: the rebin
// sources of every line in it (see src_line): the main run [q0-1, q1+1]
// clipped, line 0 when the region reaches the seam line, and the high run
// [seam, maxv] when the region holds line 0.  Disjoint ascending runs.
__device__ void staged_lines(int q0, int q1, int maxv, int seam, int32_t* lo, int32_t* hi,
                             int32_t* off, int32_t* nr, int32_t* n) {
    int a[3], b[3], k = 0;
    if (q1 >= seam) { a[k] = 0; b[k] = 0; ++k; }
    a[k] = max(q0 - 1, 0); b[k] = min(q1 + 1, maxv); ++k;
    if (q0 == 0) { a[k] = seam; b[k] = maxv; ++k; }
    // sort by start (at most three), then merge overlapping or adjacent runs
    for (int i = 1; i < k; ++i)
        for (int j = i; j > 0 && a[j] < a[j - 1]; --j) {
            int t = a[j]; a[j] = a[j - 1]; a[j - 1] = t;
            t = b[j]; b[j] = b[j - 1]; b[j - 1] = t;
        }
    int m = 0;
    for (int i = 0; i < k; ++i) {
        if (m > 0 && a[i] <= hi[m - 1] + 1) {
            hi[m - 1] = max(hi[m - 1], b[i]);
        } else {
            lo[m] = a[i];
            hi[m] = b[i];
            ++m;
        }
    }
    int o = 0;
    for (int r = 0; r < m; ++r) {
        off[r] = o;
        o += hi[r] - lo[r] + 1;
    }
    *nr = m;
    *n = o;
}

__device__ __forceinline__ uint32_t ldcg_u32(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ float4 ldcg_f4(const float4* p) { return __ldcg(p); }

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t* s_warp, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < FT / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < FT / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = v - x + (warp > 0 ? s_warp[warp - 1] : 0u);
    *total = s_warp[FT / 32 - 1];
    __syncthreads();
    return excl;
}

__device__ __forceinline__ uint32_t limit_or(uint32_t runtime, uint32_t dflt) {
    return runtime ? runtime : dflt;
}

// Grid barrier for a cooperative launch; false if the wait expired.
__device__ bool grid_sync(uint32_t* bar, uint32_t* err, uint32_t spin_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_ok = 1;
        volatile uint32_t* gen = bar + 1;
        const uint32_t g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t spins = 0;
            while (*gen == g) {
                if (++spins > limit_or(spin_limit, BAR_SPINS)) {
                    atomicOr(err, ERR_SPIN_TIMEOUT);
                    s_ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (s_ok && (*((volatile uint32_t*)err) & ERR_SPIN_TIMEOUT)) s_ok = 0;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ unsigned long long lb_pack(uint32_t epoch, unsigned long long flag,
                                                      uint32_t v) {
    return ((unsigned long long)(epoch & 0x3FFFFFFFu) << 34) | (flag << 32) | v;
}

// hist[0..ncells) -> start_next[0..ncells] (exclusive), hist cleared.  CTA b
// scans a contiguous chunk; chunk prefixes come from a decoupled look-back in
// CTA order (all CTAs are co-resident).
__device__ void scan_phase(const FusedArgs& a, uint32_t* start_next, uint32_t epoch) {
    __shared__ uint32_t s_warp[FT / 32];
    __shared__ uint32_t s_prefix;
    const uint32_t nb = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
    const uint32_t chunk = (a.ncells + nb - 1) / nb;
    const uint32_t lo = min(b * chunk, a.ncells), hi = min(lo + chunk, a.ncells);
    uint32_t t = 0;
    for (uint32_t i = lo + tid; i < hi; i += FT) t += ldcg_u32(a.hist + i);
    uint32_t total;
    (void)block_excl_scan(t, s_warp, &total);
    if (tid < 32) {
        uint32_t prefix = 0;
        if (b == 0) {
            if (tid == 0) atomicExch(&a.scan_state[0], lb_pack(epoch, LB_INC, total));
        } else {
            if (tid == 0) atomicExch(&a.scan_state[b], lb_pack(epoch, LB_AGG, total));
            int64_t pred = (int64_t)b - 1;
            bool done = false;
            while (!done) {
                const int64_t j = pred - tid;
                unsigned long long w = lb_pack(epoch, LB_INC, 0u);
                if (j >= 0) {
                    uint32_t spins = 0;
                    while (true) {
                        w = *((volatile unsigned long long*)&a.scan_state[j]);
                        if ((uint32_t)(w >> 34) == (epoch & 0x3FFFFFFFu) && ((w >> 32) & 3ull))
                            break;
                        if (++spins > limit_or(a.wait.spin_limit, LB_SPINS)) {
                            atomicOr(a.err, ERR_SPIN_TIMEOUT);
                            w = lb_pack(epoch, LB_INC, 0u);
                            break;
                        }
                        __nanosleep(32);
                    }
                }
                const bool inc = ((w >> 32) & 3ull) == LB_INC;
                const uint32_t m = __ballot_sync(0xffffffffu, inc);
                uint32_t v = (uint32_t)w;
                const int stop = m ? (__ffs(m) - 1) : 32;
                if ((int)tid > stop) v = 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                prefix += v;
                if (m) done = true;
                else pred -= 32;
            }
            if (tid == 0) atomicExch(&a.scan_state[b], lb_pack(epoch, LB_INC, prefix + total));
        }
        if (tid == 0) s_prefix = prefix;
    }
    __syncthreads();
    uint32_t carry = s_prefix;
    for (uint32_t base = lo; base < hi; base += FT * 4) {
        uint32_t v[4], ts = 0;
        const uint32_t i0 = base + tid * 4;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = (i0 + k < hi) ? ldcg_u32(a.hist + i0 + k) : 0u;
            ts += v[k];
        }
        uint32_t rt;
        uint32_t ex = block_excl_scan(ts, s_warp, &rt);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < hi) {
                start_next[i0 + k] = carry + ex;
                a.hist[i0 + k] = 0u;
            }
            ex += v[k];
        }
        carry += rt;
    }
    if (tid == 0 && lo < hi && hi == a.ncells) start_next[a.ncells] = s_prefix + total;
}

// Optional per-phase cycle counters (thread 0 of each CTA), for tuning.
struct PhaseClock {
    unsigned long long* out;
    long long t;
    __device__ void init(unsigned long long* base) {
        out = base ? base + (size_t)blockIdx.x * 16 : nullptr;
        if (out && threadIdx.x == 0) t = clock64();
    }
    __device__ void mark(int k) {
        if (out && threadIdx.x == 0) {
            const long long n = clock64();
            atomicAdd(&out[k], (unsigned long long)(n - t));
            t = n;
        }
    }
};

// ------------------------------------------------------------ one tile
struct Smem {
    unsigned long long* mbar;
    float4* stage_st;
    float4* sord_st;
    uint32_t* stage_ids;
    uint32_t* stage_key;
    uint32_t* sord_ids;
    Seg* seg;
    uint32_t* cell_lo;
    uint32_t* cell_cnt;
    uint32_t* stt;
    uint32_t* colblk;
    uint32_t* owned;
    uint32_t* hist;
    uint8_t* srcx;    // [maxqx][8] staged column indices feeding each canonical column
    uint8_t* nsrcx;
    uint8_t* srcy;    // [maxqy][4][2] staged row runs feeding each canonical row
    uint8_t* nsrcy;
    uint16_t* sord_cell;  // region-local bag (iq * nqy + jq) of each canonical record
    uint32_t* abort;      // set when a bounded wait of this block gave up (beside mbar)
};

struct StepBufs {
    const float4* prev_st;
    const uint32_t* prev_ids;
    const uint32_t* prev_key;  // bag of each previous record (nullptr: recompute)
    float4* next_st;
    uint32_t* next_ids;
    uint32_t* next_key;
    const uint32_t* start_prev;
    const uint32_t* start_cur;
};

// Gather the arrivals of canonical bag (X', Y') in write-list order.
// Shared-memory form: the source bags are the tile's precomputed source
// columns x source row runs, each run contiguous in the staged records.
__device__ __forceinline__ void gather_bag_smem(const FusedArgs& a, const Rep& R, const TileCtx& c,
                                                const Smem& S, int iq, int jq) {
    const uint32_t* stt_col = S.stt + iq * (c.nqy + 1);
    const uint32_t s0 = stt_col[jq], e0 = stt_col[jq + 1];
    if (s0 == e0) return;
    const uint32_t expected = e0 - s0;
    const uint32_t cglob = R.cell_off + (uint32_t)(c.qx0 + iq) * (uint32_t)R.dh + (uint32_t)(c.qy0 + jq);
    const uint32_t sdst = S.colblk[iq] + (s0 - stt_col[0]);
    const uint16_t lcell = (uint16_t)(iq * c.nqy + jq);
    for (uint32_t k = 0; k < expected; ++k) S.sord_cell[sdst + k] = lcell;
    uint32_t m = 0;
    const int ncx = S.nsrcx[iq], nry = S.nsrcy[jq];
    for (int ax = 0; ax < ncx; ++ax) {
        const int rowbase = (int)S.srcx[iq * 8 + ax] * c.nsy;
        for (int r = 0; r < nry; ++r) {
            const int ja = S.srcy[(jq * 4 + r) * 2], jb = S.srcy[(jq * 4 + r) * 2 + 1];
            const uint32_t lo = S.cell_lo[rowbase + ja];
            const uint32_t hi = S.cell_lo[rowbase + jb] + S.cell_cnt[rowbase + jb];
            for (uint32_t e = lo; e < hi; ++e) {
                if (S.stage_key[e] == cglob) {
                    if (m < expected) {
                        S.sord_st[sdst + m] = S.stage_st[e];
                        S.sord_ids[sdst + m] = S.stage_ids[e];
                    }
                    ++m;
                }
            }
        }
    }
    if (m != expected) atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_GATHER);
}

// Global form (tiles over capacity): read the previous write list through L2.
__device__ __forceinline__ void gather_bag_global(const FusedArgs& a, const Rep& R, const TileCtx& c,
                                                  const Smem& S, const StepBufs& B, int Xq, int Yq) {
    const int iq = Xq - c.qx0, jq = Yq - c.qy0;
    const uint32_t* stt_col = S.stt + iq * (c.nqy + 1);
    const uint32_t s0 = stt_col[jq], e0 = stt_col[jq + 1];
    if (s0 == e0) return;
    const uint32_t expected = e0 - s0;
    const uint32_t cglob = R.cell_off + (uint32_t)Xq * (uint32_t)R.dh + (uint32_t)Yq;
    uint32_t m = 0;
    int lastx = -1;
#pragma unroll 1
    for (int kx = 0; kx < SRC_LINES; ++kx) {
        const int sx = src_line(kx, Xq, R.max_x, R.seam);
        if (sx < 0 || sx > R.max_x || sx <= lastx) continue;
        lastx = sx;
        int lasty = -1;
#pragma unroll 1
        for (int ky = 0; ky < SRC_LINES; ++ky) {
            const int sy = src_line(ky, Yq, R.max_y, R.seam);
            if (sy < 0 || sy > R.max_y || sy <= lasty) continue;
            lasty = sy;
            const uint32_t cell = R.cell_off + (uint32_t)sx * (uint32_t)R.dh + (uint32_t)sy;
            const uint32_t gs = ldcg_u32(B.start_prev + cell), ge = ldcg_u32(B.start_prev + cell + 1);
            for (uint32_t q = gs; q < ge; ++q) {
                uint32_t key;
                if (B.prev_key) {
                    key = ldcg_u32(B.prev_key + q);
                } else {
                    const float4 r = ldcg_f4(B.prev_st + q);
                    const int64_t k = bag_index(R, disc(r.x, R), disc(r.y, R));
                    key = k >= 0 ? R.cell_off + (uint32_t)k : 0xFFFFFFFFu;
                }
                if (key == cglob) {
                    if (m < expected) {
                        a.g_sord_st[s0 + m] = ldcg_f4(B.prev_st + q);
                        a.g_sord_ids[s0 + m] = ldcg_u32(B.prev_ids + q);
                    }
                    ++m;
                }
            }
        }
    }
    if (m != expected) atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_GATHER);
}

// Source lists of the tile's canonical lines (thread t < nqx: column qx0+t;
// nqx <= t < nqx+nqy: row qy0+t-nqx), in ascending line value.
__device__ __forceinline__ void build_sources(const Rep& R, const TileCtx& c, const Smem& S, int t) {
    if (t < c.nqx) {
        const int X = c.qx0 + t;
        int n = 0, last = -1;
        for (int k = 0; k < SRC_LINES; ++k) {
            const int v = src_line(k, X, R.max_x, R.seam);
            if (v < 0 || v > R.max_x || v <= last) continue;
            last = v;
            const int i = run_index(v, c.xlo, c.xhi, c.xoff, c.nxr);
            if (i >= 0 && n < 8) S.srcx[t * 8 + n++] = (uint8_t)i;
        }
        S.nsrcx[t] = (uint8_t)n;
    } else if (t < c.nqx + c.nqy) {
        const int jq = t - c.nqx, Y = c.qy0 + jq;
        int n = 0, last = -1, last_run = -1;
        for (int k = 0; k < SRC_LINES; ++k) {
            const int v = src_line(k, Y, R.max_y, R.seam);
            if (v < 0 || v > R.max_y || v <= last) continue;
            const int j = run_index(v, c.ylo, c.yhi, c.yoff, c.nyr);
            if (j < 0) continue;
            int run = 0;
            while (run + 1 < c.nyr && j >= c.yoff[run + 1]) ++run;
            // extend the previous run of rows when contiguous in the staging
            if (n > 0 && last == v - 1 && run == last_run &&
                S.srcy[(jq * 4 + n - 1) * 2 + 1] == j - 1) {
                S.srcy[(jq * 4 + n - 1) * 2 + 1] = (uint8_t)j;
            } else if (n < 4) {
                S.srcy[(jq * 4 + n) * 2] = (uint8_t)j;
                S.srcy[(jq * 4 + n) * 2 + 1] = (uint8_t)j;
                ++n;
            }
            last = v;
            last_run = run;
        }
        S.nsrcy[jq] = (uint8_t)n;
    }
}

// Bird::step for owned boid b of the tile; writes its next state.
template <bool STRICT, int QMODE, bool SM>
__device__ __forceinline__ void force_boid(const FusedArgs& a, const Rep& R, const TileCtx& c,
                                           const Smem& S, const StepBufs& B, uint32_t b,
                                           unsigned long long step) {
    // owned column of b: owned[k] <= b < owned[k+1]
    const int ncol = c.X1 - c.X0;
    int lo = 0, hi = ncol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S.owned[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const int X = c.X0 + lo;
    const uint32_t* sttX = S.stt + (X - c.qx0) * (c.nqy + 1);
    const uint32_t p = sttX[c.Y0 - c.qy0] + (b - S.owned[lo]);  // canonical slot
    float4 me;
    uint32_t my_id;
    if (SM) {
        const uint32_t si = S.colblk[X - c.qx0] + (p - sttX[0]);
        me = S.sord_st[si];
        my_id = S.sord_ids[si];
    } else {
        me = ldcg_f4(a.g_sord_st + p);
        my_id = ldcg_u32(a.g_sord_ids + p);
    }
    // the boid's bag: recorded by the shared-memory gather, else recomputed
    int cx, cy;
    if (SM) {
        const uint32_t lc = S.sord_cell[S.colblk[X - c.qx0] + (p - sttX[0])];
        cx = c.qx0 + (int)(lc / (uint32_t)c.nqy);
        cy = c.qy0 + (int)(lc % (uint32_t)c.nqy);
    } else {
        cx = disc(me.x, R);
        cy = disc(me.y, R);
    }
    const int32_t ocx = cx, ocy = cy;
    Acc<STRICT> acc;
    if (R.dd >= 0) {
        if (cx < c.X0 || cx >= c.X1 || cy < c.Y0 || cy >= c.Y1) {
            atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_OUTSIDE);  // a boid outside its own bag
            cx = min(max(cx, c.X0), c.X1 - 1);
            cy = min(max(cy, c.Y0), c.Y1 - 1);
        }
        const int mi = max(0, cx - R.dd), Mi = min(cx + R.dd, R.max_x - 1);
        const int mj = max(0, cy - R.dd), Mj = min(cy + R.dd, R.max_y - 1);
        if (mj <= Mj) {
            for (int ci = mi; ci <= Mi; ++ci) {
                const uint32_t* sttc = S.stt + (ci - c.qx0) * (c.nqy + 1);
                const int64_t adj = SM ? (int64_t)S.colblk[ci - c.qx0] - (int64_t)sttc[0] : 0;
                const float4* base_st = SM ? S.sord_st : a.g_sord_st;
                const uint32_t* base_id = SM ? S.sord_ids : a.g_sord_ids;
                if (QMODE == 0) {
                    const uint32_t s = sttc[mj - c.qy0], e = sttc[Mj + 1 - c.qy0];
                    acc.vec += e - s;
                    if (R.nowrap) {
                        for (uint32_t q = s; q < e; ++q) {
                            const uint32_t qi = (uint32_t)((int64_t)q + adj);
                            const uint32_t oid = SM ? base_id[qi] : ldcg_u32(base_id + qi);
                            if (oid != my_id)
                                acc.template add<true>(R, me.x, me.y, SM ? base_st[qi] : ldcg_f4(base_st + qi));
                        }
                    } else {
                        for (uint32_t q = s; q < e; ++q) {
                            const uint32_t qi = (uint32_t)((int64_t)q + adj);
                            const uint32_t oid = SM ? base_id[qi] : ldcg_u32(base_id + qi);
                            if (oid != my_id) acc.add(R, me.x, me.y, SM ? base_st[qi] : ldcg_f4(base_st + qi));
                        }
                    }
                } else {
                    for (int cj = mj; cj <= Mj; ++cj) {
                        const uint32_t s = sttc[cj - c.qy0], e = sttc[cj + 1 - c.qy0];
                        if (s == e) continue;
                        const int check = check_circle(ci, cj, R, me.x, me.y, R.radius);
                        if (check == -1) continue;
                        for (uint32_t q = s; q < e; ++q) {
                            const uint32_t qi = (uint32_t)((int64_t)q + adj);
                            const float4 o = SM ? base_st[qi] : ldcg_f4(base_st + qi);
                            if (check == 0 &&
                                !(distance(me.x, me.y, o.x, o.y, R.w, R.h, R.toroidal != 0) <= R.radius))
                                continue;
                            acc.vec += 1;
                            const uint32_t oid = SM ? base_id[qi] : ldcg_u32(base_id + qi);
                            if (oid != my_id) acc.add(R, me.x, me.y, o);
                        }
                    }
                }
            }
        }
    }
    const float4 nxt = finish_bird<STRICT>(R, me, my_id, step, acc);
    B.next_st[p] = nxt;
    B.next_ids[p] = my_id;
    const int32_t ncx = disc(nxt.x, R), ncy = disc(nxt.y, R);
    int64_t idx = bag_index(R, ncx, ncy);
    if (B.next_key) B.next_key[p] = R.cell_off + (uint32_t)(idx < 0 ? 0 : idx);
    uint32_t flags = 0;
    if (idx < 0) {
        flags |= ERR_KEY_RANGE;
        idx = 0;
    }
    if (!isfinite(nxt.x) || !isfinite(nxt.y)) flags |= ERR_NONFINITE;
    const bool okx = move_ok(ocx, ncx, R.seam), oky = move_ok(ocy, ncy, R.seam);
    if (!(okx && oky)) flags |= ERR_REBIN_MISS | ERR_MISS_MOVE;
    if (flags) atomicOr(a.err, flags);
    const int hx = ncx - c.hx0, hy = ncy - c.hy0;
    if (idx >= 0 && hx >= 0 && hx < c.hnx && hy >= 0 && hy < c.hny && flags == 0)
        atomicAdd(&S.hist[hx * c.hny + hy], 1u);
    else
        atomicAdd(&a.hist[R.cell_off + (uint32_t)idx], 1u);
}

template <bool STRICT, int QMODE>
__device__ bool process_tile(const FusedArgs& a, const Tile tile, TileCtx& c, const Smem& S,
                             const StepBufs& B, unsigned long long step, uint32_t* phase,
                             PhaseClock& pc) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const Rep R = a.reps[tile.rep];
    // ---- 1. tile geometry
    if (tid == 0) {
        const int dd = max(R.dd, 0);
        c.rep = tile.rep;
        c.dd = dd;
        c.X0 = tile.x0;
        c.Y0 = tile.y0;
        c.X1 = min((int)tile.x0 + a.cfg.tx, R.dw);
        c.Y1 = min((int)tile.y0 + a.cfg.ty, R.dh);
        c.qx0 = max(c.X0 - dd, 0);
        c.qx1 = min(c.X1 - 1 + dd, R.dw - 1);
        c.qy0 = max(c.Y0 - dd, 0);
        c.qy1 = min(c.Y1 - 1 + dd, R.dh - 1);
        c.nqx = c.qx1 - c.qx0 + 1;
        c.nqy = c.qy1 - c.qy0 + 1;
        staged_lines(c.qx0, c.qx1, R.max_x, R.seam, c.xlo, c.xhi, c.xoff, &c.nxr, &c.nsx);
        staged_lines(c.qy0, c.qy1, R.max_y, R.seam, c.ylo, c.yhi, c.yoff, &c.nyr, &c.nsy);
        c.nseg = (uint32_t)(c.nsx * c.nyr);
        c.hx0 = max(c.X0 - 1, 0);
        c.hy0 = max(c.Y0 - 1, 0);
        c.hnx = min(c.X1 + 1, R.dw) - c.hx0;
        c.hny = min(c.Y1 + 1, R.dh) - c.hy0;
        // a ring wider than the layout was sized for: refuse the tile
        c.overflow = (dd > a.cfg.dd || c.X0 >= c.X1 || c.Y0 >= c.Y1) ? 2 : 0;
        if (c.overflow) atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_TILE);
    }
    __syncthreads();
    pc.mark(0);
    if (c.overflow == 2) return;
    const FusedLayout L = fused_layout(a.cfg);
    // ---- 2. segments (warp 0) and the canonical offsets table (other warps)
    if (warp == 0) {
        uint32_t run = 0;
        for (uint32_t k0 = 0; k0 < c.nseg; k0 += 32) {
            const uint32_t k = k0 + lane;
            uint32_t glo = 0, cnt = 0;
            if (k < c.nseg) {
                const int i = (int)(k / (uint32_t)c.nyr), r = (int)(k % (uint32_t)c.nyr);
                int xr;
                const int vx = run_value(i, c.xlo, c.xhi, c.xoff, c.nxr, &xr);
                const int ra = c.ylo[r], rb = c.yhi[r];
                const uint32_t cb = R.cell_off + (uint32_t)vx * (uint32_t)R.dh;
                glo = ldcg_u32(B.start_prev + cb + ra);
                cnt = ldcg_u32(B.start_prev + cb + rb + 1) - glo;
            }
            uint32_t x = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (k < c.nseg) S.seg[k] = Seg{glo, cnt, run + x - cnt, 0u};
            run += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) c.staged = run;
    } else {
        const int nrow = c.nqy + 1;
        for (int t = tid - 32; t < c.nqx * nrow; t += FT - 32) {
            const int i = t / nrow, j = t % nrow;
            const uint32_t cell = R.cell_off + (uint32_t)(c.qx0 + i) * (uint32_t)R.dh + (uint32_t)(c.qy0 + j);
            S.stt[t] = ldcg_u32(B.start_cur + cell);
        }
    }
    __syncthreads();
    pc.mark(1);
    // ---- 3. column blocks, owned prefix (warp 0), capacity decision, TMA arm
    if (warp == 0) {
        uint32_t run = 0;
        for (int i0 = 0; i0 < c.nqx; i0 += 32) {
            const int i = i0 + lane;
            uint32_t v = 0;
            if (i < c.nqx) {
                const uint32_t* col = S.stt + i * (c.nqy + 1);
                v = col[c.nqy] - col[0];
            }
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (i < c.nqx) S.colblk[i] = run + x - v;
            run += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) S.colblk[c.nqx] = run;
        const uint32_t sord = run;
        run = 0;
        const int ncol = c.X1 - c.X0;
        for (int i0 = 0; i0 < ncol; i0 += 32) {
            const int i = i0 + lane;
            uint32_t v = 0;
            if (i < ncol) {
                const uint32_t* col = S.stt + (c.X0 + i - c.qx0) * (c.nqy + 1);
                v = col[c.Y1 - c.qy0] - col[c.Y0 - c.qy0];
            }
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (i < ncol) S.owned[i] = run + x - v;
            run += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) {
            S.owned[ncol] = run;
            c.owned = run;
            c.sord = sord;
            c.overflow = (c.staged > a.cfg.stage_cap || sord > a.cfg.sord_cap ||
                          c.nsx > L.maxlx || c.nsy > L.maxly) ? 1 : 0;
            if (!c.overflow) {
                fence_proxy_async();
                mbar_arrive_expect_tx(S.mbar, c.staged * 16u);
            } else {
                atomicAdd(&a.stats[0], 1u);
            }
        }
    } else if (tid - 32 < c.nqx + c.nqy) {
        build_sources(R, c, S, tid - 32);
    }
    __syncthreads();
    pc.mark(2);
    const bool sm = !c.overflow;
    if (sm) {
        // ---- 4. staging: records by TMA (warp 0), ids and bag tables by all
        if (warp == 0) {
            for (uint32_t k = lane; k < c.nseg; k += 32) {
                const Seg g = S.seg[k];
                if (g.cnt) bulk_g2s(S.stage_st + g.soff, B.prev_st + g.glo, g.cnt * 16u, S.mbar);
            }
        }
        for (uint32_t k = warp; k < c.nseg; k += FT / 32) {
            const Seg g = S.seg[k];
            for (uint32_t e = lane; e < g.cnt; e += 32) {
                S.stage_ids[g.soff + e] = ldcg_u32(B.prev_ids + g.glo + e);
                if (B.prev_key) S.stage_key[g.soff + e] = ldcg_u32(B.prev_key + g.glo + e);
            }
        }
        for (int t = tid; t < c.nsx * c.nsy; t += FT) {
            const int i = t / c.nsy, j = t % c.nsy;
            int xr, r;
            const int vx = run_value(i, c.xlo, c.xhi, c.xoff, c.nxr, &xr);
            const int vy = run_value(j, c.ylo, c.yhi, c.yoff, c.nyr, &r);
            const Seg g = S.seg[i * c.nyr + r];
            const uint32_t cell = R.cell_off + (uint32_t)vx * (uint32_t)R.dh + (uint32_t)vy;
            const uint32_t s0 = ldcg_u32(B.start_prev + cell), s1 = ldcg_u32(B.start_prev + cell + 1);
            S.cell_lo[t] = g.soff + (s0 - g.glo);
            S.cell_cnt[t] = s1 - s0;
        }
        // one warp waits on the transaction barrier; the rest block at the
        // CTA barrier, then observe the completed phase once
        if (warp == 0) {
            const uint32_t lim = limit_or(a.wait.spin_limit, TMA_SPINS);
            uint32_t spins = 0;
            bool done = true;
            while (!mbar_try_wait(S.mbar, *phase & 1u)) {
                if (++spins > lim) {
                    done = false;
                    break;
                }
            }
            if (!done) {
                // the copies of this phase did not land in time: give them one
                // more bounded wait (they write this block's shared memory), then
                // the whole block stops without reading the staged records
                spins = 0;
                while (!mbar_try_wait(S.mbar, *phase & 1u) && ++spins <= lim) {
                }
                if (lane == 0) {
                    atomicOr(a.err, ERR_SPIN_TIMEOUT);
                    *S.abort = 1u;
                }
            }
        }
        __syncthreads();
        if (*S.abort) return false;
        if (warp != 0) {
            uint32_t spins = 0;
            while (!mbar_try_wait(S.mbar, *phase & 1u) && ++spins < 64u) {
            }
        }
        *phase += 1;
        pc.mark(3);
        for (uint32_t e = tid; e < c.staged; e += FT) {
            const float4 r = S.stage_st[e];
            const int64_t k = bag_index(R, disc(r.x, R), disc(r.y, R));
            S.stage_key[e] = k >= 0 ? R.cell_off + (uint32_t)k : 0xFFFFFFFFu;
        }
        __syncthreads();
        pc.mark(4);
    }
    // ---- 5. rebin: canonical order of the region's bags
    for (int t = tid; t < c.nqx * c.nqy; t += FT) {
        const int iq = t / c.nqy, jq = t % c.nqy;
        if (sm) gather_bag_smem(a, R, c, S, iq, jq);
        else gather_bag_global(a, R, c, S, B, c.qx0 + iq, c.qy0 + jq);
    }
    __syncthreads();
    pc.mark(5);
    // ---- 6. force pass for the owned boids
    for (uint32_t b = tid; b < c.owned; b += FT) {
        if (sm) force_boid<STRICT, QMODE, true>(a, R, c, S, B, b, step);
        else force_boid<STRICT, QMODE, false>(a, R, c, S, B, b, step);
    }
    __syncthreads();
    pc.mark(6);
    // ---- 7. flush the shared histogram
    for (int t = tid; t < c.hnx * c.hny; t += FT) {
        const uint32_t v = S.hist[t];
        if (v) {
            const int i = t / c.hny, j = t % c.hny;
            atomicAdd(&a.hist[R.cell_off + (uint32_t)(c.hx0 + i) * (uint32_t)R.dh + (uint32_t)(c.hy0 + j)], v);
            S.hist[t] = 0u;
        }
    }
    __syncthreads();
    pc.mark(7);
    return true;
}

__device__ __forceinline__ Smem smem_view(unsigned char* smem, const FusedLayout& L) {
    Smem S;
    S.mbar = reinterpret_cast<unsigned long long*>(smem + L.off_mbar);
    S.abort = reinterpret_cast<uint32_t*>(smem + L.off_mbar + 8);
    S.stage_st = reinterpret_cast<float4*>(smem + L.off_stage_st);
    S.sord_st = reinterpret_cast<float4*>(smem + L.off_sord_st);
    S.stage_ids = reinterpret_cast<uint32_t*>(smem + L.off_stage_ids);
    S.stage_key = reinterpret_cast<uint32_t*>(smem + L.off_stage_key);
    S.sord_ids = reinterpret_cast<uint32_t*>(smem + L.off_sord_ids);
    S.seg = reinterpret_cast<Seg*>(smem + L.off_seg);
    S.cell_lo = reinterpret_cast<uint32_t*>(smem + L.off_cell_lo);
    S.cell_cnt = reinterpret_cast<uint32_t*>(smem + L.off_cell_cnt);
    S.stt = reinterpret_cast<uint32_t*>(smem + L.off_stt);
    S.colblk = reinterpret_cast<uint32_t*>(smem + L.off_colblk);
    S.owned = reinterpret_cast<uint32_t*>(smem + L.off_owned);
    S.hist = reinterpret_cast<uint32_t*>(smem + L.off_hist);
    S.srcx = smem + L.off_srcx;
    S.nsrcx = smem + L.off_nsrcx;
    S.srcy = smem + L.off_srcy;
    S.nsrcy = smem + L.off_nsrcy;
    S.sord_cell = reinterpret_cast<uint16_t*>(smem + L.off_sord_cell);
    return S;
}

// One step of one tile per CTA (no grid-wide waits): the split form of the
// step, followed by the histogram scan as its own launch.
template <bool STRICT, int QMODE>
__global__ void __launch_bounds__(FT, 4) k_tile_step(FusedArgs a, StepBufs B, uint32_t step_offset) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ TileCtx ctx;
    const FusedLayout L = fused_layout(a.cfg);
    const Smem S = smem_view(smem, L);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(S.mbar, 1);
        fence_proxy_async();
        *S.abort = 0u;
    }
    for (int t = tid; t < L.maxhx * L.maxhy; t += FT) S.hist[t] = 0u;
    __syncthreads();
    const unsigned long long step = *a.step + step_offset;
    uint32_t phase = 0;
    PhaseClock pc;
    pc.out = a.phase_cycles;  // all CTAs add into one set of counters
    if (pc.out && tid == 0) pc.t = clock64();
    process_tile<STRICT, QMODE>(a, a.tiles[blockIdx.x], ctx, S, B, step, &phase, pc);
}

template <bool STRICT, int QMODE>
__global__ void __launch_bounds__(FT, 2) k_fused(FusedArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ TileCtx ctx;
    __shared__ uint32_t s_tile;
    const FusedLayout L = fused_layout(a.cfg);
    Smem S;
    S.mbar = reinterpret_cast<unsigned long long*>(smem + L.off_mbar);
    S.abort = reinterpret_cast<uint32_t*>(smem + L.off_mbar + 8);
    S.stage_st = reinterpret_cast<float4*>(smem + L.off_stage_st);
    S.sord_st = reinterpret_cast<float4*>(smem + L.off_sord_st);
    S.stage_ids = reinterpret_cast<uint32_t*>(smem + L.off_stage_ids);
    S.stage_key = reinterpret_cast<uint32_t*>(smem + L.off_stage_key);
    S.sord_ids = reinterpret_cast<uint32_t*>(smem + L.off_sord_ids);
    S.seg = reinterpret_cast<Seg*>(smem + L.off_seg);
    S.cell_lo = reinterpret_cast<uint32_t*>(smem + L.off_cell_lo);
    S.cell_cnt = reinterpret_cast<uint32_t*>(smem + L.off_cell_cnt);
    S.stt = reinterpret_cast<uint32_t*>(smem + L.off_stt);
    S.colblk = reinterpret_cast<uint32_t*>(smem + L.off_colblk);
    S.owned = reinterpret_cast<uint32_t*>(smem + L.off_owned);
    S.hist = reinterpret_cast<uint32_t*>(smem + L.off_hist);
    S.srcx = smem + L.off_srcx;
    S.nsrcx = smem + L.off_nsrcx;
    S.srcy = smem + L.off_srcy;
    S.nsrcy = smem + L.off_nsrcy;
    S.sord_cell = reinterpret_cast<uint16_t*>(smem + L.off_sord_cell);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(S.mbar, 1);
        fence_proxy_async();
        *S.abort = 0u;
    }
    for (int t = tid; t < L.maxhx * L.maxhy; t += FT) S.hist[t] = 0u;
    __syncthreads();
    const unsigned long long base_step = *((volatile unsigned long long*)a.step);
    const uint32_t epoch0 = *((volatile uint32_t*)a.scan_epoch);
    uint32_t phase = 0;
    PhaseClock pc;
    pc.init(a.phase_cycles);
    for (uint32_t s = 0; s < a.nsteps; ++s) {
        StepBufs B;
        B.prev_st = s == 0 ? a.a_in_st : a.a_st[(s - 1) & 1];
        B.prev_ids = s == 0 ? a.a_in_ids : a.a_ids[(s - 1) & 1];
        B.prev_key = nullptr;
        B.next_st = a.a_st[s & 1];
        B.next_ids = a.a_ids[s & 1];
        B.next_key = nullptr;
        B.start_prev = a.start_b[s & 1];
        B.start_cur = a.start_b[(s + 1) & 1];
        const unsigned long long step = base_step + s;
        for (;;) {
            if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
            __syncthreads();
            const uint32_t t = s_tile;
            __syncthreads();
            pc.mark(8);
            if (t >= a.ntiles) break;
            if (!process_tile<STRICT, QMODE>(a, a.tiles[t], ctx, S, B, step, &phase, pc)) return;
        }
        // test hook: this block leaves before the barrier, so the others' wait runs out
        if (s == 0 && blockIdx.x == a.wait.withhold) return;
        if (!grid_sync(a.bar, a.err, a.wait.spin_limit)) return;
        pc.mark(9);
        if (blockIdx.x == 0 && tid == 0) atomicExch(a.tile_counter, 0u);
        scan_phase(a, a.start_b[s & 1], epoch0 + s + 1);
        pc.mark(10);
        if (!grid_sync(a.bar, a.err, a.wait.spin_limit)) return;
        pc.mark(11);
    }
    if (blockIdx.x == 0 && tid == 0) {
        *a.step = base_step + a.nsteps;
        *a.scan_epoch = epoch0 + a.nsteps;
    }
}

template <bool STRICT, int QMODE>
void* fused_fn() {
    return reinterpret_cast<void*>(&k_fused<STRICT, QMODE>);
}

void* pick(bool strict, int qmode) {
    if (strict) return qmode == 0 ? fused_fn<true, 0>() : fused_fn<true, 1>();
    return qmode == 0 ? fused_fn<false, 0>() : fused_fn<false, 1>();
}

template <bool STRICT, int QMODE>
void* tile_fn() {
    return reinterpret_cast<void*>(&k_tile_step<STRICT, QMODE>);
}

void* pick_tile(bool strict, int qmode) {
    if (strict) return qmode == 0 ? tile_fn<true, 0>() : tile_fn<true, 1>();
    return qmode == 0 ? tile_fn<false, 0>() : tile_fn<false, 1>();
}

}  // namespace

int fused_max_ctas(const FusedCfg& cfg, bool strict, int qmode, int device) {
    const FusedLayout L = fused_layout(cfg);
    void* fn = pick(strict, qmode);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, FT, L.total) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * sms;
}

cudaError_t launch_tile_step(const FusedArgs& a, const float4* prev_st, const uint32_t* prev_ids,
                             const uint32_t* prev_key, float4* next_st, uint32_t* next_ids,
                             uint32_t* next_key, const uint32_t* start_prev,
                             const uint32_t* start_cur, uint32_t step_offset, bool strict, int qmode,
                             cudaStream_t s) {
    if (a.ntiles == 0) return cudaSuccess;
    const FusedLayout L = fused_layout(a.cfg);
    void* fn = pick_tile(strict, qmode);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return e;
    StepBufs B;
    B.prev_st = prev_st;
    B.prev_ids = prev_ids;
    B.prev_key = prev_key;
    B.next_st = next_st;
    B.next_ids = next_ids;
    B.next_key = next_key;
    B.start_prev = start_prev;
    B.start_cur = start_cur;
    void* args[] = {const_cast<FusedArgs*>(&a), &B, &step_offset};
    return cudaLaunchKernel(fn, dim3(a.ntiles), dim3(FT), args, L.total, s);
}

cudaError_t launch_fused(const FusedArgs& a, bool strict, int qmode, uint32_t nctas,
                         cudaStream_t s) {
    const FusedLayout L = fused_layout(a.cfg);
    void* fn = pick(strict, qmode);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nctas);
    cfg.blockDim = dim3(FT);
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<FusedArgs*>(&a)};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace kb
