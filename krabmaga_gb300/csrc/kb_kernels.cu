// kb_kernels.cu -- sm_103a kernels of the continuous-space agent step.
//
// Data layout in HBM (one field, or many replicas packed back to back):
//   read buffer  st[n] float4 {x, y, last_dx, last_dy}, ids[n] u32, sorted by
//                bag index (cell_off + x*dh + y, field_2d.rs:508), each bag in
//                insertion order; start[ncells+1] u32 bag offsets.
//   write list   the same records in arbitrary order plus a u32 bag key each
//                (the write buffer of field_2d.rs:838-846).
// A flock step is: force pass (read buffer -> write list, key histogram),
// scan of the histogram, stencil-gather rebin (write list -> read buffer).
#include <cuda_runtime.h>
#include <stdint.h>

#include "kb_common.h"
#include "kb_launch.h"
#include "kb_runtime.h"
#include "kb_device.cuh"

namespace kb {
namespace {

// Programmatic dependent launch.  The step's kernels are launched so that
// the next one may be scheduled before the previous one ends; each first
// waits until its predecessor has finished and its writes are visible
// (griddepcontrol.wait, before touching any memory), then lets its own
// successor launch (griddepcontrol.launch_dependents).  Launched without the
// attribute, the wait returns at once.
#ifndef KB_PDL
#define KB_PDL 1
#endif
__device__ __forceinline__ void pdl_enter() {
#if KB_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                       Args... args) {
#if KB_PDL
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
#else
    kernel<<<grid, block, 0, s>>>(static_cast<KArgs>(args)...);
    return cudaGetLastError();
#endif
}

// Accumulate the candidates of one contiguous run [s, e) of the read
// buffer, four at a time so their loads are in flight together.
// Force-kernel launch shape, chosen by timing builds on GB300 (1M boids,
// density 0.025): 2-candidate load groups and 6 resident 256-thread blocks
// per SM (40 registers) beat deeper unrolling at lower occupancy.
#ifndef KB_FORCE_UNROLL
#define KB_FORCE_UNROLL 2
#endif

template <bool STRICT, bool NOWRAP>
__device__ __forceinline__ void accumulate_run_t(const Rep& R, const float4* __restrict__ st,
                                                 const uint32_t* __restrict__ ids, uint32_t s,
                                                 uint32_t e, float4 me, uint32_t my_id,
                                                 Acc<STRICT>& acc) {
    acc.vec += e - s;
    uint32_t q = s;
    constexpr int U = KB_FORCE_UNROLL;  // candidates whose loads are issued together
    for (; q + U <= e; q += U) {
        uint32_t oid[U];
        float4 o[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            oid[u] = __ldg(ids + q + u);
            o[u] = __ldg(st + q + u);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (oid[u] != my_id) acc.template add<NOWRAP>(R, me.x, me.y, o[u]);
    }
    for (; q < e; ++q) {
        const uint32_t oid = __ldg(ids + q);
        const float4 o = __ldg(st + q);
        if (oid != my_id) acc.template add<NOWRAP>(R, me.x, me.y, o);
    }
}
template <bool STRICT>
__device__ __forceinline__ void accumulate_run(const Rep& R, const float4* __restrict__ st,
                                               const uint32_t* __restrict__ ids, uint32_t s,
                                               uint32_t e, float4 me, uint32_t my_id,
                                               Acc<STRICT>& acc) {
    if (R.nowrap) accumulate_run_t<STRICT, true>(R, st, ids, s, e, me, my_id, acc);
    else accumulate_run_t<STRICT, false>(R, st, ids, s, e, me, my_id, acc);
}

// The candidate runs of up to NC columns (one contiguous run of bags per
// column), every run's bounds loaded before any candidate.
template <int NC, bool STRICT>
__device__ __forceinline__ void columns_runs(const ForceArgs& a, const Rep& R, int mi, int Mi,
                                             int mj, int Mj, float4 me, uint32_t my_id,
                                             Acc<STRICT>& acc) {
    uint32_t s[NC], e[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        if (mi + k <= Mi) {
            const uint32_t colbase = R.cell_off + (uint32_t)(mi + k) * (uint32_t)R.dh;
            e[k] = min(__ldg(a.start + colbase + Mj + 1), a.n);
            s[k] = min(__ldg(a.start + colbase + mj), e[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < NC; ++k)
        if (mi + k <= Mi) accumulate_run(R, a.st, a.ids, s[k], e[k], me, my_id, acc);
}
// The three runs of a one-bag ring as one flat list: a warp then iterates
// the longest lane's total instead of the sum of the per-column maxima.
// DENSE: long lists; each run is walked with a plain pointer (one run after
// the other, the same visiting order), which costs fewer instructions per
// candidate once the runs are long enough that the per-run maxima of a warp
// add little.
template <bool STRICT, bool DENSE>
// my_slot: the boid's own read-buffer slot when ids are unique (a candidate
// is the boid itself exactly there), else ~0u and ids are compared.
__device__ __forceinline__ void columns_flat3(const ForceArgs& a, const Rep& R, int mi, int Mi,
                                              int mj, int Mj, float4 me, uint32_t my_id,
                                              Acc<STRICT>& acc, uint32_t my_slot) {
    uint32_t s[3], e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s[k] = e[k] = 0u;
        if (mi + k <= Mi) {
            const uint32_t colbase = R.cell_off + (uint32_t)(mi + k) * (uint32_t)R.dh;
            e[k] = min(__ldg(a.start + colbase + Mj + 1), a.n);
            s[k] = min(__ldg(a.start + colbase + mj), e[k]);
        }
    }
    const uint32_t P1 = e[0] - s[0], P2 = P1 + (e[1] - s[1]), T = P2 + (e[2] - s[2]);
    acc.vec += T;
    const uint32_t d1 = s[1] - P1, d2 = s[2] - P2;  // position = f + d (mod 2^32)
    if (R.nowrap && my_slot != 0xFFFFFFFFu) {
        // every candidate but the boid's own slot counts: no count per candidate
        const bool self_in = (my_slot - s[0] < e[0] - s[0]) || (my_slot - s[1] < e[1] - s[1]) ||
                             (my_slot - s[2] < e[2] - s[2]);
        acc.count = (int)(T - (self_in ? 1u : 0u));
    }
    if (DENSE && R.nowrap && my_slot != 0xFFFFFFFFu) {
#pragma unroll 1
        for (int k = 0; k < 3; ++k) {
            const uint32_t ek = e[k];
            for (uint32_t q = s[k]; q < ek; ++q) {
                const float4 o = __ldg(a.st + q);
                if (q != my_slot) acc.template add<true, false>(R, me.x, me.y, o);
            }
        }
    } else if (R.nowrap && my_slot != 0xFFFFFFFFu) {
        for (uint32_t f = 0; f < T; ++f) {
            const uint32_t p = f < P1 ? s[0] + f : (f < P2 ? f + d1 : f + d2);
            const float4 o = __ldg(a.st + p);
            if (p != my_slot) acc.template add<true, false>(R, me.x, me.y, o);
        }
    } else if (R.nowrap) {
        for (uint32_t f = 0; f < T; ++f) {
            const uint32_t p = f < P1 ? s[0] + f : (f < P2 ? f + d1 : f + d2);
            const uint32_t oid = __ldg(a.ids + p);
            const float4 o = __ldg(a.st + p);
            if (oid != my_id) acc.template add<true>(R, me.x, me.y, o);
        }
    } else {
        for (uint32_t f = 0; f < T; ++f) {
            const uint32_t p = f < P1 ? s[0] + f : (f < P2 ? f + d1 : f + d2);
            const uint32_t oid = __ldg(a.ids + p);
            const float4 o = __ldg(a.st + p);
            if (oid != my_id) acc.template add<false>(R, me.x, me.y, o);
        }
    }
}

// The wider ring out of line, so that it does not set the register budget of
// the common one-ring case.
template <bool STRICT>
__device__ __noinline__ void columns_runs_5(const ForceArgs& a, const Rep& R, int mi, int Mi,
                                            int mj, int Mj, float4 me, uint32_t my_id,
                                            Acc<STRICT>& acc) {
    columns_runs<5>(a, R, mi, Mi, mj, Mj, me, my_id, acc);
}

template <bool STRICT>
__device__ __forceinline__ void force_finish(const ForceArgs& a, const Rep& R, uint32_t i,
                                             float4 me, uint32_t my_id, unsigned long long step,
                                             const Acc<STRICT>& acc);

// The candidate sums of one agent at `me` against the read buffer (the
// query of bird.rs:41 and the loop of bird.rs:48-82).  my_slot: the agent's
// own read-buffer slot when self is recognised by slot, else ~0u.
template <bool STRICT, int QMODE, bool DENSE = false>
__device__ __forceinline__ void gather_candidates(const ForceArgs& a, const Rep& R, float4 me,
                                                  uint32_t my_id, uint32_t my_slot,
                                                  Acc<STRICT>& acc) {
    int mi, Mi, mj, Mj;
    if (cell_range(R, me.x, me.y, R.dd, &mi, &Mi, &mj, &Mj)) {
        const bool clamped = R.toroidal && !R.cell_wrap;  // runs never cross the seam
        if (QMODE == 0 && clamped && Mi - mi < 5) {
            // clamped range: each column's bags mj..Mj are one contiguous
            // run; fetch every run's bounds before touching candidates
            if (mj <= Mj) {
                // a one-bag ring (the common case) as one flat list; the wider
                // two-bag ring out of line
                if (Mi - mi < 3)
                    columns_flat3<STRICT, DENSE>(a, R, mi, Mi, mj, Mj, me, my_id, acc, my_slot);
                else columns_runs_5(a, R, mi, Mi, mj, Mj, me, my_id, acc);
            }
        } else {
            for (int ci = mi; ci <= Mi; ++ci) {
                const int bx = t_transform(ci, R.max_x);
                const uint32_t colbase = R.cell_off + (uint32_t)bx * (uint32_t)R.dh;
                if (QMODE == 0 && clamped) {
                    if (mj > Mj) continue;
                    const uint32_t e = min(__ldg(a.start + colbase + Mj + 1), a.n);
                    accumulate_run(R, a.st, a.ids, min(__ldg(a.start + colbase + mj), e), e, me,
                                   my_id, acc);
                    continue;
                }
                for (int cj = mj; cj <= Mj; ++cj) {
                    const int by = t_transform(cj, R.max_y);
                    const uint32_t c = colbase + (uint32_t)by;
                    const uint32_t e = min(__ldg(a.start + c + 1), a.n);
                    const uint32_t s = min(__ldg(a.start + c), e);
                    if (s == e) continue;
                    if (QMODE == 0) {
                        accumulate_run(R, a.st, a.ids, s, e, me, my_id, acc);
                        continue;
                    }
                    const int check = check_circle(bx, by, R, me.x, me.y, R.radius);
                    if (check == -1) continue;
                    for (uint32_t k = s; k < e; ++k) {
                        const float4 o = __ldg(a.st + k);
                        if (check == 0 &&
                            !(distance(me.x, me.y, o.x, o.y, R.w, R.h, R.toroidal != 0) <= R.radius))
                            continue;
                        acc.vec += 1;
                        if (__ldg(a.ids + k) != my_id) acc.add(R, me.x, me.y, o);
                    }
                }
            }
        }
    }
}

template <bool STRICT, int QMODE, bool DENSE>
__device__ __forceinline__ void force_body(const ForceArgs& a, const Rep& R, uint32_t i) {
    const unsigned long long step = *a.step;
    const float4 me = __ldg(a.st + i);
    const uint32_t my_id = __ldg(a.ids + i);
    Acc<STRICT> acc;
    gather_candidates<STRICT, QMODE, DENSE>(a, R, me, my_id, a.self_by_slot ? i : 0xFFFFFFFFu, acc);
    force_finish<STRICT>(a, R, i, me, my_id, step, acc);
}

// bird.rs:84-153 after the candidate sums: the next state at slot i of the
// write list, its bag key and the arrival count of that bag.
template <bool STRICT>
__device__ __forceinline__ void force_finish(const ForceArgs& a, const Rep& R, uint32_t i,
                                             float4 me, uint32_t my_id, unsigned long long step,
                                             const Acc<STRICT>& acc) {
    const float4 nxt = finish_bird<STRICT>(R, me, my_id, step, acc);
    const float nx = nxt.x, ny = nxt.y;
    a.out_st[i] = nxt;
    a.out_ids[i] = my_id;
    const int32_t ncx = disc(nx, R), ncy = disc(ny, R);
    int64_t idx = bag_index(R, ncx, ncy);
    uint32_t flags = 0;
    if (idx < 0) {
        flags |= ERR_KEY_RANGE;
        idx = 0;
    }
    if (!isfinite(nx) || !isfinite(ny)) flags |= ERR_NONFINITE;
    // the rebin gathers a bag's arrivals from the 3x3 old bags around it
    // (plus the seam columns/rows); anything else must take the general sort
    if (a.check_moves) {
        const int32_t ocx = disc(me.x, R), ocy = disc(me.y, R);
        if (!(move_ok(ocx, ncx, R.seam) && move_ok(ocy, ncy, R.seam)))
            flags |= ERR_REBIN_MISS | ERR_MISS_MOVE;
    }
    if (flags) atomicOr(a.err, flags);
    const uint32_t key = R.cell_off + (uint32_t)idx;
    a.out_key[i] = key;
    atomicAdd(&a.hist[key], 1u);
}

#ifndef KB_FORCE_THREADS
#define KB_FORCE_THREADS 256
#endif
static_assert(KB_FORCE_THREADS == FORCE_THREADS, "the host block tables assume this block size");
#ifndef KB_FORCE_MINB
#define KB_FORCE_MINB 6
#endif
#ifndef KB_FORCE_MINB_MULTI
#define KB_FORCE_MINB_MULTI 6
#endif

// A replica record into shared memory, one word per thread (blockDim >= words).
__device__ __forceinline__ void load_rep_shared(Rep* dst, const Rep* src) {
    constexpr int WORDS = sizeof(Rep) / 4;
    static_assert(sizeof(Rep) % 4 == 0 && WORDS <= 256, "replica record words");
    if (threadIdx.x < WORDS)
        reinterpret_cast<uint32_t*>(dst)[threadIdx.x] = __ldg(reinterpret_cast<const uint32_t*>(src) + threadIdx.x);
}

// BT: threads per block (the packed-replica block table's granularity); the
// same 48 warps per SM at every block size.
template <bool STRICT, int QMODE, bool MULTI, bool DENSE = false, int BT = KB_FORCE_THREADS>
__global__ void __launch_bounds__(BT, (MULTI ? KB_FORCE_MINB_MULTI : KB_FORCE_MINB) * KB_FORCE_THREADS / BT)
    k_flock_force(ForceArgs a) {
    pdl_enter();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (MULTI) {
        // one replica per block: its record is read once into shared memory
        __shared__ Rep sR;
        const uint2 e = a.blk[blockIdx.x];
        load_rep_shared(&sR, a.reps + e.x);
        __syncthreads();
        const uint32_t k = e.y + threadIdx.x;
        if (k >= sR.boid_off + sR.nboids) return;
        force_body<STRICT, QMODE, false>(a, sR, k);
        return;
    }
    if (i >= a.n) return;
    force_body<STRICT, QMODE, DENSE>(a, a.rep0, i);
}

// Bird::step for agents given by the caller rather than read from the read
// buffer (agents that join the schedule, schedule.rs:283-303): agent j reads
// its neighbours from the read buffer, skips candidates with its own id
// (bird.rs:50) and writes its next state to slot j of the outputs.
template <bool STRICT, int QMODE>
__global__ void __launch_bounds__(KB_FORCE_THREADS)
    k_flock_agents(ForceArgs a, const float4* __restrict__ in_st, const uint32_t* __restrict__ in_ids,
                   uint32_t nin) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nin) return;
    const unsigned long long step = *a.step;
    const float4 me = in_st[j];
    const uint32_t my_id = in_ids[j];
    Acc<STRICT> acc;
    gather_candidates<STRICT, QMODE>(a, a.rep0, me, my_id, 0xFFFFFFFFu, acc);
    force_finish<STRICT>(a, a.rep0, j, me, my_id, step, acc);
}

// Mark every live write-list entry whose id is in sorted[0..m) removed.
__global__ void k_remove_ids(const uint32_t* __restrict__ ids, uint8_t* dead, uint32_t n,
                             const uint32_t* __restrict__ sorted, uint32_t m, uint32_t* removed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || dead[i]) return;
    const uint32_t id = ids[i];
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sorted[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    if (lo < m && sorted[lo] == id) {
        dead[i] = 1;
        atomicAdd(removed, 1u);
    }
}

// first[j] = the smallest index i < n with ids[i] == sorted[j] (live entries
// only when dead != nullptr); first[] starts at ~0u.
__global__ void k_find_ids(const uint32_t* __restrict__ ids, const uint8_t* __restrict__ dead,
                           uint32_t n, const uint32_t* __restrict__ sorted, uint32_t m,
                           uint32_t* first) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (dead && dead[i])) return;
    const uint32_t id = ids[i];
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sorted[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    if (lo < m && sorted[lo] == id) atomicMin(&first[lo], i);
}

__global__ void k_gather_found(const float4* __restrict__ st, const uint32_t* __restrict__ first,
                               uint32_t m, float4* __restrict__ out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const uint32_t i = first[j];
    out[j] = i == 0xFFFFFFFFu ? make_float4(0.f, 0.f, 0.f, 0.f) : st[i];
}

// ---------------------------------------------------------- scan
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr unsigned long long FLAG_AGG = 1ull, FLAG_INC = 2ull;
constexpr uint32_t SPIN_LIMIT = 1u << 20;

__device__ __forceinline__ unsigned long long pack_tile(uint32_t epoch, unsigned long long flag,
                                                        uint32_t v) {
    return ((unsigned long long)(epoch & 0x3FFFFFFFu) << 34) | (flag << 32) | v;
}

__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n, ScanCtl* ctl,
           unsigned long long* tstate, uint32_t* err, int zero_in, uint32_t ntiles, WaitCfg wait) {
    pdl_enter();
    const uint32_t spin_limit = wait.spin_limit ? wait.spin_limit : SPIN_LIMIT;
    __shared__ uint32_t s_tile, s_epoch, s_prefix;
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_tile = atomicAdd(&ctl->tile_counter, 1u);
        s_epoch = *((volatile uint32_t*)&ctl->epoch);
    }
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    const uint64_t base = (uint64_t)tile * SCAN_TILE + (uint64_t)tid * SCAN_ITEMS;

    uint32_t v[SCAN_ITEMS];
    if (base + SCAN_ITEMS <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS / 4; ++k) {
            const uint4 w = p[k];
            v[4 * k] = w.x; v[4 * k + 1] = w.y; v[4 * k + 2] = w.z; v[4 * k + 3] = w.w;
        }
        if (zero_in) {
            uint4* q = reinterpret_cast<uint4*>(const_cast<uint32_t*>(in + base));
#pragma unroll
            for (int k = 0; k < SCAN_ITEMS / 4; ++k) q[k] = make_uint4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = (base + k < n) ? in[base + k] : 0u;
            if (zero_in && base + k < n) const_cast<uint32_t*>(in)[base + k] = 0u;
        }
    }
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) tsum += v[k];
    // block exclusive scan of the per-thread sums
    uint32_t x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < SCAN_THREADS / 32) ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) s_warp[lane] = w;  // inclusive warp prefixes
    }
    __syncthreads();
    const uint32_t agg = s_warp[SCAN_THREADS / 32 - 1];
    const uint32_t texcl = x - tsum + (warp > 0 ? s_warp[warp - 1] : 0u);

    // decoupled look-back across tiles, 256 predecessors per round trip
    __shared__ int s_jinc;
    __shared__ uint32_t s_sum[SCAN_THREADS / 32];
    const bool publish = tile != wait.withhold;  // the test hook withholds one tile's words
    if (tile == 0) {
        if (tid == 0) {
            if (publish) atomicExch(&tstate[0], pack_tile(epoch, FLAG_INC, agg));
            s_prefix = 0;
        }
    } else {
        if (tid == 0) {
            if (publish) atomicExch(&tstate[tile], pack_tile(epoch, FLAG_AGG, agg));
            s_jinc = -0x7fffffff;
        }
        __syncthreads();
        uint32_t prefix = 0;
        int64_t pred = (int64_t)tile - 1;
        for (;;) {
            const int64_t j = pred - tid;
            unsigned long long word = pack_tile(epoch, FLAG_INC, 0u);  // below tile 0
            if (j >= 0) {
                uint32_t spins = 0;
                while (true) {
                    word = *((volatile unsigned long long*)&tstate[j]);
                    if ((uint32_t)(word >> 34) == (epoch & 0x3FFFFFFFu) && ((word >> 32) & 3ull) != 0ull)
                        break;
                    if (++spins > spin_limit) {
                        atomicOr(err, ERR_SPIN_TIMEOUT);
                        word = pack_tile(epoch, FLAG_INC, 0u);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            const bool inc = ((word >> 32) & 3ull) == FLAG_INC;
            // the nearest inclusive predecessor in this window: the smallest tid
            if (inc) atomicMax(&s_jinc, -(int)tid);
            __syncthreads();
            const int stop = -s_jinc;  // tid of the nearest inclusive word, or huge
            uint32_t v = ((int)tid <= stop) ? (uint32_t)word : 0u;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) s_sum[warp] = v;
            __syncthreads();
            uint32_t tot = 0;
#pragma unroll
            for (int w = 0; w < SCAN_THREADS / 32; ++w) tot += s_sum[w];
            prefix += tot;
            const bool done = stop < SCAN_THREADS;
            __syncthreads();
            if (done) break;
            if (tid == 0) s_jinc = -0x7fffffff;
            pred -= SCAN_THREADS;
            __syncthreads();
        }
        if (tid == 0) {
            if (publish) atomicExch(&tstate[tile], pack_tile(epoch, FLAG_INC, prefix + agg));
            s_prefix = prefix;
        }
    }
    __syncthreads();
    const uint32_t prefix = s_prefix;
    uint32_t run = prefix + texcl;
    if (base + SCAN_ITEMS <= n) {
        uint32_t o[SCAN_ITEMS];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            o[k] = run;
            run += v[k];
        }
        uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS / 4; ++k)
            p[k] = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (base + k < n) out[base + k] = run;
            run += v[k];
        }
    }
    if (tile == ntiles - 1 && tid == 0) out[n] = prefix + agg;
    // the last CTA to finish re-arms the control block for the next launch
    if (tid == 0) {
        __threadfence();
        const uint32_t d = atomicAdd(&ctl->done_counter, 1u);
        if (d == ntiles - 1) {
            ctl->tile_counter = 0u;
            ctl->done_counter = 0u;
            __threadfence();
            atomicAdd(&ctl->epoch, 1u);
        }
    }
}

// ---------------------------------------------------------- rebin
// The arrivals of bag c in write-list order from the records [s, e).
__device__ __forceinline__ void rebin_run(const RebinArgs& a, const Rep& R, uint32_t c, uint32_t s,
                                          uint32_t e, uint32_t& dst, uint32_t end) {
    for (uint32_t p = s; p < e; ++p) {
        uint32_t k;
        if (a.key) {
            k = __ldg(a.key + p);
        } else {  // key from the record's own position
            const float4 r = __ldg(a.a_st + p);
            const int64_t b = bag_index(R, disc(r.x, R), disc(r.y, R));
            k = b >= 0 ? R.cell_off + (uint32_t)b : 0xFFFFFFFFu;
        }
        if (k == c) {
            if (dst < end) {
                a.s_st[dst] = __ldg(a.a_st + p);
                a.s_ids[dst] = __ldg(a.a_ids + p);
            }
            ++dst;
        }
    }
}

__device__ __forceinline__ void rebin_cell(const RebinArgs& a, const Rep& R, uint32_t c) {
    const uint32_t end = min(__ldg(a.start_next + c + 1), a.n);
    uint32_t dst = min(__ldg(a.start_next + c), end);
    if (dst == end) return;
    const uint32_t local = c - R.cell_off;
    const uint32_t Xu = div_dh(local, R);
    const int X = (int)Xu, Y = (int)(local - Xu * (uint32_t)R.dh);
    if (X > 0 && X < R.seam && Y > 0 && Y < R.seam) {
        // interior bag: three source columns, rows Y-1..Y+1 contiguous in each
        uint32_t s[3], e[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t base = R.cell_off + (uint32_t)(X - 1 + k) * (uint32_t)R.dh + (uint32_t)Y;
            e[k] = min(__ldg(a.start_cur + base + 2), a.n);
            s[k] = min(__ldg(a.start_cur + base - 1), e[k]);
        }
        if (a.key) {
            // the first keys of every run in flight together
            uint32_t kk[3][4];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    kk[k][u] = (s[k] + u < e[k]) ? __ldg(a.key + s[k] + u) : 0xFFFFFFFFu;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (kk[k][u] == c) {
                        if (dst < end) {
                            a.s_st[dst] = __ldg(a.a_st + s[k] + u);
                            a.s_ids[dst] = __ldg(a.a_ids + s[k] + u);
                        }
                        ++dst;
                    }
                }
                if (s[k] + 4 < e[k]) rebin_run(a, R, c, s[k] + 4, e[k], dst, end);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) rebin_run(a, R, c, s[k], e[k], dst, end);
        }
    } else {
        int lastx = -1;
#pragma unroll 1
        for (int kx = 0; kx < SRC_LINES; ++kx) {
            const int sx = src_line(kx, X, R.max_x, R.seam);
            if (sx < 0 || sx > R.max_x || sx <= lastx) continue;
            lastx = sx;
            const uint32_t colbase = R.cell_off + (uint32_t)sx * (uint32_t)R.dh;
            int lasty = -1;
#pragma unroll 1
            for (int ky = 0; ky < SRC_LINES; ++ky) {
                const int sy = src_line(ky, Y, R.max_y, R.seam);
                if (sy < 0 || sy > R.max_y || sy <= lasty) continue;
                lasty = sy;
                const uint32_t re = min(__ldg(a.start_cur + colbase + sy + 1), a.n);
                rebin_run(a, R, c, min(__ldg(a.start_cur + colbase + sy), re), re, dst, end);
            }
        }
    }
    if (dst != end) atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_MATERIALIZE);
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_rebin(RebinArgs a) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0 && a.step != nullptr) *a.step += 1ull;
    if (c >= a.ncells) return;
    if (MULTI) {
        const Rep R = a.reps[rep_of_cell(a.reps, a.nrep, c)];
        rebin_cell(a, R, c);
    } else {
        rebin_cell(a, a.rep0, c);
    }
}

// ---------------------------------------------------------- two-pass scan
// For up to SCAN2_MAX_TILES tiles the offsets are a reduce-then-scan pair of
// launches with no waiting between blocks: per-tile sums, then every tile
// adds the sums before it (at most SCAN2_MAX_TILES / 256 loads a thread),
// scans its items and writes them.  Larger inputs take the single-pass
// look-back kernel above.  The sums go into the look-back state words as
// plain 64-bit values: their flag bits stay zero, so a later look-back
// launch on the same buffer reads them as "not published".
constexpr int S2_ITEMS = KB_SCAN2_ITEMS;

// Exclusive block scan of one value per thread (SCAN_THREADS threads).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t* s_warp, uint32_t* total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t base = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; ++w) {
        const uint32_t v = s_warp[w];
        if (w < warp) base += v;
        tot += v;
    }
    *total = tot;
    return base + incl - x;
}

template <int ITEMS>
__device__ __forceinline__ void load_items(const uint32_t* in, uint32_t n, uint64_t base,
                                           uint32_t (&v)[ITEMS]) {
    if (base + ITEMS <= n) {
        const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int k = 0; k < ITEMS / 4; ++k) {
            const uint4 w = p[k];
            v[4 * k] = w.x; v[4 * k + 1] = w.y; v[4 * k + 2] = w.z; v[4 * k + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) v[k] = (base + k < n) ? in[base + k] : 0u;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
    k_tile_sums(const uint32_t* __restrict__ in, uint32_t n, unsigned long long* __restrict__ sums) {
    pdl_enter();
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN2_TILE + (uint64_t)threadIdx.x * S2_ITEMS;
    uint32_t v[S2_ITEMS];
    load_items<S2_ITEMS>(in, n, base, v);
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < S2_ITEMS; ++k) t += v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < SCAN_THREADS / 32; ++w) s += s_warp[w];
        sums[blockIdx.x] = (unsigned long long)s;
    }
}

// The exclusive scan, in place, of ntiles tile sums (one block; large bag
// matrices: the tiles then take their prefix with one load).
constexpr int SUMS_THREADS = 1024;
constexpr int SUMS_ITEMS = 8;
__global__ void __launch_bounds__(SUMS_THREADS) k_scan_sums(unsigned long long* sums, uint32_t ntiles) {
    pdl_enter();
    __shared__ uint32_t s_warp[SUMS_THREADS / 32];
    __shared__ uint32_t s_carry;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_carry = 0u;
    __syncthreads();
    for (uint64_t chunk = 0; chunk < ntiles; chunk += (uint64_t)SUMS_THREADS * SUMS_ITEMS) {
        const uint64_t base = chunk + (uint64_t)tid * SUMS_ITEMS;
        uint32_t v[SUMS_ITEMS], t = 0;
#pragma unroll
        for (int k = 0; k < SUMS_ITEMS; ++k) {
            v[k] = base + k < ntiles ? (uint32_t)sums[base + k] : 0u;
            t += v[k];
        }
        uint32_t x = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31u) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= (uint32_t)o) w += y;
            }
            s_warp[lane] = w;  // inclusive warp prefixes
        }
        __syncthreads();
        uint32_t run = s_carry + (warp > 0 ? s_warp[warp - 1] : 0u) + x - t;
#pragma unroll
        for (int k = 0; k < SUMS_ITEMS; ++k) {
            if (base + k < ntiles) sums[base + k] = (unsigned long long)run;
            run += v[k];
        }
        __syncthreads();
        if (tid == 0) s_carry += s_warp[SUMS_THREADS / 32 - 1];
        __syncthreads();
    }
}

// PREFIX: sums[] already holds each tile's exclusive prefix (k_scan_sums);
// otherwise the tile adds up the sums of the tiles before it.
template <bool PREFIX>
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_tiles(uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n,
                 const unsigned long long* __restrict__ sums, int zero_in, uint32_t ntiles) {
    pdl_enter();
    __shared__ uint32_t s_warp[SCAN_THREADS / 32], s_red[SCAN_THREADS / 32];
    const uint32_t tile = blockIdx.x, tid = threadIdx.x;
    // this tile's prefix: the sums of the tiles before it
    uint32_t part = 0;
    if (PREFIX) {
        if (tid == 0) part = (uint32_t)sums[tile];
    } else {
        for (uint32_t k = tid; k < tile; k += SCAN_THREADS) part += (uint32_t)sums[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) s_red[tid >> 5] = part;
    const uint64_t base = (uint64_t)tile * SCAN2_TILE + (uint64_t)tid * S2_ITEMS;
    uint32_t v[S2_ITEMS];
    load_items<S2_ITEMS>(in, n, base, v);
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < S2_ITEMS; ++k) tsum += v[k];
    uint32_t total;
    const uint32_t texcl = block_excl_scan(tsum, s_warp, &total);  // syncs s_red too
    uint32_t prefix = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; ++w) prefix += s_red[w];
    uint32_t run = prefix + texcl;
    if (base + S2_ITEMS <= n) {
        uint32_t o[S2_ITEMS];
#pragma unroll
        for (int k = 0; k < S2_ITEMS; ++k) {
            o[k] = run;
            run += v[k];
        }
        uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
        for (int k = 0; k < S2_ITEMS / 4; ++k)
            p[k] = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
        if (zero_in) {
            uint4* q = reinterpret_cast<uint4*>(in + base);
#pragma unroll
            for (int k = 0; k < S2_ITEMS / 4; ++k) q[k] = make_uint4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < S2_ITEMS; ++k) {
            if (base + k < n) {
                out[base + k] = run;
                if (zero_in) in[base + k] = 0u;
            }
            run += v[k];
        }
    }
    if (tile == ntiles - 1 && tid == 0) out[n] = prefix + total;
}

// ---------------------------------------------------------- segment rebin
// One warp per segment of up to 32 consecutive bags of one column (lane l
// owns bag c0 + l).  The arrivals of those bags sit in the write list inside
// the source runs of the neighbouring columns: rows Y0-1..Y1+1 of columns
// X-1..X+1 (plus the seam lines at the field's edges).  The warp streams
// those runs in ascending bag order, 32 entries at a time with coalesced key
// loads; entries whose key falls in the segment take the next slot of their
// bag: __match_any_sync ranks equal keys within a batch in lane (= list)
// order, a per-bag counter in shared memory carries the rank across batches.
// That is the per-bag insertion order of the reference's lazy_update.
constexpr uint32_t FULL_MASK = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t rep_segments_dev(const Rep& R) {
    const uint32_t rows = R.seg_rows > 0 ? (uint32_t)R.seg_rows : (uint32_t)SEG_ROWS;
    return (uint32_t)R.dw * (((uint32_t)R.dh + rows - 1) / rows);
}

__device__ __forceinline__ int rep_of_seg(const Rep* reps, int nrep, uint32_t g) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&reps[mid].seg_off) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Slot of one write-list entry of a batch of 32 (key k per lane, ~0u for
// none) in its bag of the segment, or ~0u when the key is outside the
// segment.  Every lane of the warp calls it.
// Bag offsets of a segment: lane l holds bag l (lo[0], hi[0]) and, with two
// bags per lane (64-bag segments), bag l + 32 (lo[1], hi[1]).
template <int BPL>
struct SegBags {
    uint32_t lo[BPL], hi[BPL];
};

template <int BPL>
__device__ __forceinline__ uint32_t seg_rank(uint32_t k, uint32_t c0, int nb, const SegBags<BPL>& sb,
                                             uint32_t* cnt, uint32_t lane_lt, bool& bad) {
    const uint32_t local = k - c0;
    const bool in = local < (uint32_t)nb;
    if (__ballot_sync(FULL_MASK, in) == 0u) return 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(FULL_MASK, in ? local : 0xFFFFFFFFu);
    const uint32_t rank = __popc(peers & lane_lt);
    const uint32_t src = local & 31u;
    uint32_t blo = __shfl_sync(FULL_MASK, sb.lo[0], src);
    uint32_t bhi = __shfl_sync(FULL_MASK, sb.hi[0], src);
    if (BPL == 2) {
        const uint32_t blo1 = __shfl_sync(FULL_MASK, sb.lo[BPL - 1], src);
        const uint32_t bhi1 = __shfl_sync(FULL_MASK, sb.hi[BPL - 1], src);
        if (local >= 32u) {
            blo = blo1;
            bhi = bhi1;
        }
    }
    const uint32_t slot = BPL == 2 ? local : src;
    const uint32_t base = in ? cnt[slot] : 0u;
    __syncwarp();
    uint32_t dst = 0xFFFFFFFFu;
    if (in) {
        dst = blo + base + rank;
        if (dst >= bhi) {
            bad = true;
            dst = 0xFFFFFFFFu;
        }
        if (rank + 1u == (uint32_t)__popc(peers)) cnt[slot] = base + rank + 1u;
    }
    __syncwarp();
    return dst;
}

// One batch of 32 write-list entries (p, valid per lane): rank and copy.
#ifndef KB_REBIN_BATCHES
#define KB_REBIN_BATCHES 2
#endif

template <int BPL>
__device__ __forceinline__ void seg_batch(const RebinArgs& a, bool valid, uint32_t p, uint32_t c0,
                                          int nb, const SegBags<BPL>& sb, uint32_t* cnt,
                                          uint32_t lane_lt, bool& bad) {
    const uint32_t k = valid ? __ldg(a.key + p) : 0xFFFFFFFFu;
    const uint32_t dst = seg_rank<BPL>(k, c0, nb, sb, cnt, lane_lt, bad);
    if (dst != 0xFFFFFFFFu) {
        a.s_st[dst] = __ldg(a.a_st + p);
        a.s_ids[dst] = __ldg(a.a_ids + p);
    }
}

// ROWS (<= 64) consecutive bags of one column per warp (one or two per lane).
template <int ROWS>
__device__ __forceinline__ void rebin_segment(const RebinArgs& a, const Rep& R, uint32_t g,
                                              uint32_t* cnt) {
    static_assert(ROWS >= 1 && ROWS <= 64, "a segment's bags map to one or two per lane");
    constexpr int BPL = ROWS > 32 ? 2 : 1;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nsy = ((uint32_t)R.dh + ROWS - 1) / ROWS;
    const uint32_t local = g - R.seg_off;
    const uint32_t Xu = local / nsy;
    const int X = (int)Xu;
    const int Y0 = (int)(local - Xu * nsy) * ROWS;
    const int nb = min(ROWS, R.dh - Y0);
    const int Y1 = Y0 + nb - 1;
    const uint32_t c0 = R.cell_off + Xu * (uint32_t)R.dh + (uint32_t)Y0;
    const bool interior = X > 0 && X < R.seam && Y0 > 0 && Y1 < R.seam;
    // this segment's bag offsets and (interior) the bounds of its three
    // source runs, in one round trip
    SegBags<BPL> sb;
    uint32_t b = 0;
#pragma unroll
    for (int h = 0; h < BPL; ++h) {
        sb.lo[h] = sb.hi[h] = 0u;
        const int bag = (int)lane + 32 * h;
        if (bag < nb) {
            sb.hi[h] = min(__ldg(a.start_next + c0 + bag + 1), a.n);
            sb.lo[h] = min(__ldg(a.start_next + c0 + bag), sb.hi[h]);
        }
    }
    if (interior && lane < 6u) {
        const uint32_t cb = R.cell_off + (uint32_t)(X - 1 + (int)(lane % 3u)) * (uint32_t)R.dh;
        b = min(__ldg(a.start_cur + cb + (lane < 3u ? (uint32_t)(Y0 - 1) : (uint32_t)(Y1 + 2))), a.n);
    }
    {
        const uint32_t first = __shfl_sync(FULL_MASK, sb.lo[0], 0);
        uint32_t last = __shfl_sync(FULL_MASK, sb.hi[0], (nb - 1) & 31);
        if (BPL == 2) {
            const uint32_t last1 = __shfl_sync(FULL_MASK, sb.hi[BPL - 1], (nb - 1) & 31);
            if (nb > 32) last = last1;
        }
        if (first == last) return;  // no arrivals
    }
#pragma unroll
    for (int h = 0; h < BPL; ++h) cnt[lane + 32 * h] = 0u;
    __syncwarp();
    const uint32_t lane_lt = (1u << lane) - 1u;
    bool bad = false;
    if (interior) {
        // columns X-1..X+1, rows Y0-1..Y1+1, as one list of three runs
        const uint32_t s0 = __shfl_sync(FULL_MASK, b, 0), s1 = __shfl_sync(FULL_MASK, b, 1);
        const uint32_t s2 = __shfl_sync(FULL_MASK, b, 2), e0 = __shfl_sync(FULL_MASK, b, 3);
        const uint32_t e1 = __shfl_sync(FULL_MASK, b, 4), e2 = __shfl_sync(FULL_MASK, b, 5);
        // run bounds out of order (only after a failed step) read as empty runs
        const uint32_t P1 = e0 - min(s0, e0), P2 = P1 + (e1 - min(s1, e1)), T = P2 + (e2 - min(s2, e2));
        // KB_REBIN_BATCHES batches of 32 list entries per round: every key of
        // the round in flight at once, then the ranks in list order, then every
        // record of the round in flight at once
        for (uint32_t f0 = 0; f0 < T; f0 += 32u * KB_REBIN_BATCHES) {
            uint32_t p[KB_REBIN_BATCHES], dst[KB_REBIN_BATCHES];
#pragma unroll
            for (int b = 0; b < KB_REBIN_BATCHES; ++b) {
                const uint32_t ff = f0 + 32u * b + lane;
                p[b] = ff < P1 ? s0 + ff : (ff < P2 ? s1 + (ff - P1) : s2 + (ff - P2));
                dst[b] = ff < T ? __ldg(a.key + p[b]) : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int b = 0; b < KB_REBIN_BATCHES; ++b)
                dst[b] = seg_rank<BPL>(dst[b], c0, nb, sb, cnt, lane_lt, bad);
            float4 rec[KB_REBIN_BATCHES];
            uint32_t rid[KB_REBIN_BATCHES];
#pragma unroll
            for (int b = 0; b < KB_REBIN_BATCHES; ++b) {
                if (dst[b] != 0xFFFFFFFFu) {
                    rec[b] = __ldg(a.a_st + p[b]);
                    rid[b] = __ldg(a.a_ids + p[b]);
                }
            }
#pragma unroll
            for (int b = 0; b < KB_REBIN_BATCHES; ++b) {
                if (dst[b] != 0xFFFFFFFFu) {
                    a.s_st[dst[b]] = rec[b];
                    a.s_ids[dst[b]] = rid[b];
                }
            }
        }
    } else {
        // a segment at the seam or the field's edge: the source lines of
        // src_line on both axes, run by run in ascending bag order
        const int mlo = max(0, Y0 - 1), mhi = min(R.max_y, Y1 + 1);
        int lastx = -1;
#pragma unroll 1
        for (int kx = 0; kx < SRC_LINES; ++kx) {
            const int sx = src_line(kx, X, R.max_x, R.seam);
            if (sx < 0 || sx > R.max_x || sx <= lastx) continue;
            lastx = sx;
            const uint32_t cb = R.cell_off + (uint32_t)sx * (uint32_t)R.dh;
            int ra[3], rb[3], nr = 0;
            if (Y1 >= R.seam && mlo > 0) { ra[nr] = 0; rb[nr] = 0; ++nr; }   // bags >= seam take row 0
            ra[nr] = mlo; rb[nr] = mhi; ++nr;
            if (Y0 == 0) {  // row 0 takes rows seam..seam+3
                const int l2 = max(R.seam, mhi + 1), h2 = min(R.seam + SRC_LINES - 5, R.max_y);
                if (l2 <= h2) { ra[nr] = l2; rb[nr] = h2; ++nr; }
            }
#pragma unroll 1
            for (int r = 0; r < nr; ++r) {
                const uint32_t e = min(__ldg(a.start_cur + cb + (uint32_t)rb[r] + 1u), a.n);
                const uint32_t s = min(__ldg(a.start_cur + cb + (uint32_t)ra[r]), e);
#pragma unroll 1
                for (uint32_t f = s; f < e; f += 32u)
                    seg_batch<BPL>(a, f + lane < e, f + lane, c0, nb, sb, cnt, lane_lt, bad);
            }
        }
    }
#pragma unroll
    for (int h = 0; h < BPL; ++h) {
        const int bag = (int)lane + 32 * h;
        if (bag < nb && cnt[bag] != sb.hi[h] - sb.lo[h]) bad = true;
    }
    if (__any_sync(FULL_MASK, bad) && lane == 0u) atomicOr(a.err, ERR_REBIN_MISS | ERR_MISS_MATERIALIZE);
}

#ifndef KB_REBIN_MINB
#define KB_REBIN_MINB 6
#endif

#ifndef KB_REBIN_MINB_MULTI
#define KB_REBIN_MINB_MULTI 6
#endif

template <bool MULTI, int ROWS = SEG_ROWS>
__global__ void __launch_bounds__(32 * REBIN_SEG_WARPS, MULTI ? KB_REBIN_MINB_MULTI : KB_REBIN_MINB)
    k_rebin_seg(RebinArgs a) {
    pdl_enter();
    __shared__ uint32_t s_cnt[REBIN_SEG_WARPS][MULTI ? PACKED_SEG_ROWS : 32];
    const uint32_t w = threadIdx.x >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.step != nullptr) *a.step += 1ull;
    if (MULTI) {
        // one replica per block: its record is read once into shared memory
        __shared__ Rep sR;
        const uint2 e = a.sblk[blockIdx.x];
        load_rep_shared(&sR, a.reps + e.x);
        __syncthreads();
        const uint32_t g = e.y + w;
        // packed replicas always carry seg_rows == PACKED_SEG_ROWS (assign_segments)
        if (g >= sR.seg_off + rep_segments_dev(sR)) return;  // whole warps
        rebin_segment<PACKED_SEG_ROWS>(a, sR, g, s_cnt[w]);
        return;
    }
    const uint32_t g = blockIdx.x * REBIN_SEG_WARPS + w;
    if (g >= a.nsegs) return;  // whole warps
    rebin_segment<ROWS>(a, a.rep0, g, s_cnt[w]);
}

// Sum of squared bag occupancies of a read buffer (its offsets), a measure
// of how long the candidate lists are: about 9 * sum / N per boid.
__global__ void k_occupancy_sq(const uint32_t* __restrict__ start, uint32_t ncells,
                               unsigned long long* out) {
    __shared__ unsigned long long s_part[8];
    unsigned long long acc = 0;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        const unsigned long long o = (unsigned long long)(start[c + 1] - start[c]);
        acc += o * o;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(FULL_MASK, acc, d);
    if ((threadIdx.x & 31u) == 0u) s_part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        atomicAdd(out, t);
    }
}

// ---------------------------------------------------------- general sort
__global__ void k_hist_list(const uint32_t* __restrict__ key, const uint8_t* __restrict__ dead,
                            uint32_t n, uint32_t* __restrict__ hist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (dead && dead[i])) return;
    atomicAdd(&hist[key[i]], 1u);
}

__global__ void k_scatter_list(const uint32_t* __restrict__ key, const uint8_t* __restrict__ dead,
                               const float4* __restrict__ st, const uint32_t* __restrict__ ids,
                               uint32_t n, const uint32_t* __restrict__ start,
                               uint32_t* __restrict__ cursor, float4* __restrict__ t_st,
                               uint32_t* __restrict__ t_ids, uint32_t* __restrict__ t_src) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (dead && dead[i])) return;
    const uint32_t k = key[i];
    const uint32_t slot = start[k] + atomicAdd(&cursor[k], 1u);
    t_st[slot] = st[i];
    t_ids[slot] = ids[i];
    t_src[slot] = i;
}

// One thread per bag: order the bag's members by their write-list index
// (the reference's insertion order), then reset the bag's cursor.
__global__ void k_canon(const uint32_t* __restrict__ start, uint32_t ncells,
                        const float4* __restrict__ t_st, const uint32_t* __restrict__ t_ids,
                        const uint32_t* __restrict__ t_src, uint32_t* __restrict__ cursor,
                        float4* __restrict__ s_st, uint32_t* __restrict__ s_ids) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const uint32_t s = start[c], e = start[c + 1];
    if (s == e) return;
    cursor[c] = 0u;
    for (uint32_t m = s; m < e; ++m) {
        const uint32_t src = t_src[m];
        uint32_t rank = 0;
        for (uint32_t m2 = s; m2 < e; ++m2) rank += (t_src[m2] < src) ? 1u : 0u;
        s_st[s + rank] = t_st[m];
        s_ids[s + rank] = t_ids[m];
    }
}

// ---------------------------------------------------------- queries
template <int KIND>
__global__ void k_query(QueryArgs a) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.nq) return;
    const Rep& R = a.rep;
    const float2 p = a.q[q];
    const bool fill = a.offsets != nullptr;
    const uint64_t off = fill ? a.offsets[q] : 0;
    uint32_t cnt = 0, dig = 0;
    int mi, Mi, mj, Mj;
    const int32_t dd = (a.dist <= 0.0f) ? -1 : disc(a.dist, R);
    if (cell_range(R, p.x, p.y, dd, &mi, &Mi, &mj, &Mj)) {
        for (int ci = mi; ci <= Mi; ++ci) {
            const int bx = t_transform(ci, R.max_x);
            for (int cj = mj; cj <= Mj; ++cj) {
                const int by = t_transform(cj, R.max_y);
                const uint32_t c = R.cell_off + (uint32_t)bx * (uint32_t)R.dh + (uint32_t)by;
                const uint32_t s = a.start[c], e = a.start[c + 1];
                if (s == e) continue;
                int check = 1;
                if (KIND == 1) {
                    check = check_circle(bx, by, R, p.x, p.y, a.dist);
                    if (check == -1) continue;
                }
                for (uint32_t k = s; k < e; ++k) {
                    if (KIND == 1 && check == 0) {
                        const float4 o = a.st[k];
                        if (!(distance(p.x, p.y, o.x, o.y, R.w, R.h, R.toroidal != 0) <= a.dist))
                            continue;
                    }
                    const uint32_t id = a.ids[k];
                    if (fill && off + cnt < a.cap) {
                        a.out_ids[off + cnt] = id;
                        if (a.out_st) a.out_st[off + cnt] = a.st[k];
                    }
                    dig += id_mix(id);
                    ++cnt;
                }
            }
        }
    }
    if (!fill) {
        a.counts[q] = cnt;
        if (a.digest) a.digest[q] = dig;
    }
}

// ---------------------------------------------------------- ordered filters
// One block walks the list in chunks, keeping list order (write-buffer
// lookups are API calls, not the per-step path).
constexpr int FILTER_THREADS = 1024;

template <typename Pred, typename Emit>
__device__ void ordered_filter(uint32_t n, Pred pred, Emit emit, uint32_t* out_count) {
    __shared__ uint32_t s_warp[FILTER_THREADS / 32];
    __shared__ uint32_t s_base;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_base = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < n; c0 += FILTER_THREADS) {
        const uint32_t i = c0 + tid;
        const bool f = i < n && pred(i);
        const uint32_t bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int w = 0; w < FILTER_THREADS / 32; ++w) {
            const uint32_t cw = s_warp[w];
            if (w < warp) before += cw;
            total += cw;
        }
        const uint32_t pos = s_base + before + __popc(bal & ((1u << lane) - 1u));
        if (f) emit(i, pos);
        __syncthreads();
        if (tid == 0) s_base += total;
        __syncthreads();
    }
    if (tid == 0) *out_count = s_base;
}

__global__ void __launch_bounds__(FILTER_THREADS)
    k_filter_key(const uint32_t* key, const uint8_t* dead, const float4* st, const uint32_t* ids,
                 uint32_t n, uint32_t target, uint32_t* out_ids, float4* out_st, uint64_t cap,
                 uint32_t* out_count) {
    ordered_filter(
        n, [&](uint32_t i) { return key[i] == target && !(dead && dead[i]); },
        [&](uint32_t i, uint32_t pos) {
            if (pos < cap) {
                if (out_ids) out_ids[pos] = ids[i];
                if (out_st) out_st[pos] = st[i];
            }
        },
        out_count);
}

__global__ void __launch_bounds__(FILTER_THREADS)
    k_empty_bags(Rep R, const uint32_t* start, float2* out, uint64_t cap, uint32_t* out_count) {
    ordered_filter(
        R.ncells, [&](uint32_t c) { return start[c + 1] == start[c]; },
        [&](uint32_t c, uint32_t pos) {
            if (pos < cap) {
                const uint32_t i = c / (uint32_t)R.dh, j = c % (uint32_t)R.dh;
                out[pos] = make_float2(__fmul_rn((float)i, R.d), __fmul_rn((float)j, R.d));
            }
        },
        out_count);
}

__global__ void k_remove(const uint32_t* key, uint8_t* dead, const uint32_t* ids, uint32_t n,
                         uint32_t target, uint32_t id, uint32_t* removed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (key[i] == target && ids[i] == id && !dead[i]) {
        dead[i] = 1;
        atomicAdd(removed, 1u);
    }
}

__global__ void k_cell_of(const uint32_t* start, uint32_t ncells, uint32_t* cell_of) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    for (uint32_t k = start[c]; k < start[c + 1]; ++k) cell_of[k] = c;
}

__global__ void k_cell_xy(Rep R, const uint32_t* cell_of, uint32_t n, float2* out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t c = cell_of[k] - R.cell_off;
    const uint32_t i = c / (uint32_t)R.dh, j = c % (uint32_t)R.dh;
    out[k] = make_float2(__fmul_rn((float)i, R.d), __fmul_rn((float)j, R.d));
}

// Initial uniform flock of one boid: kb_gen_uniform (kb_gen.cpp) with every
// operation rounded once, so host and device draw the same bits.
__device__ void gen_uniform_boid(uint32_t id, uint32_t seed_lo, uint32_t seed_hi, float w, float h,
                                 float scale, float4* out) {
    U4 o = philox4x32_10(U4{id, 0u, 0u, STREAM_INIT}, seed_lo, seed_hi);
    const float x = __fmul_rn(w, unit_f32(o.x));
    const float y = __fmul_rn(h, unit_f32(o.y));
    uint32_t z = o.z, ww = o.w;
    float hx = 0.f, hy = 0.f;
    for (uint32_t attempt = 1; attempt < 1000u; ++attempt) {
        const float a = __fsub_rn(__fmul_rn(unit_f32(z), 2.0f), 1.0f);
        const float b = __fsub_rn(__fmul_rn(unit_f32(ww), 2.0f), 1.0f);
        const float r2 = __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
        if (r2 > 0.0f && r2 <= 1.0f) {
            const float r = __fsqrt_rn(r2);
            hx = __fdiv_rn(a, r);
            hy = __fdiv_rn(b, r);
            break;
        }
        o = philox4x32_10(U4{id, attempt, 0u, STREAM_INIT}, seed_lo, seed_hi);
        z = o.z;
        ww = o.w;
    }
    *out = make_float4(x, y, __fmul_rn(hx, scale), __fmul_rn(hy, scale));
}

__global__ void k_repack(const PackEntry* __restrict__ plan, int32_t nplan, uint32_t total,
                         const Rep* __restrict__ reps, const float4* __restrict__ src_st,
                         const uint32_t* __restrict__ src_ids, float4* __restrict__ dst_st,
                         uint32_t* __restrict__ dst_ids, uint32_t* __restrict__ dst_key,
                         uint8_t* __restrict__ dst_dead, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int lo = 0, hi = nplan - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (plan[mid].dst_off <= i) lo = mid;
        else hi = mid - 1;
    }
    const PackEntry e = plan[lo];
    const uint32_t k = i - e.dst_off;
    if (k >= e.n) return;
    const Rep R = reps[e.rep];
    float4 st;
    uint32_t id;
    if (e.kind == 0) {
        st = src_st[e.src_off + k];
        id = src_ids[e.src_off + k];
    } else {
        id = k;
        gen_uniform_boid(k, e.seed_lo, e.seed_hi, R.w, R.h, e.heading_scale, &st);
    }
    const int64_t b = bag_index(R, disc(st.x, R), disc(st.y, R));
    if (b < 0) atomicOr(err, ERR_KEY_RANGE);
    dst_st[i] = st;
    dst_ids[i] = id;
    dst_key[i] = R.cell_off + (uint32_t)(b < 0 ? 0 : b);
    dst_dead[i] = 0;
}

// Per replica (one block each): {count, sum dx, sum dy, sum |(dx, dy)|} of
// the read buffer, in double.
__global__ void __launch_bounds__(256) k_moments(const Rep* __restrict__ reps,
                                                 const uint32_t* __restrict__ start,
                                                 const float4* __restrict__ st, double* out) {
    __shared__ double s_acc[4][8];
    const Rep& R = reps[blockIdx.x];
    const uint32_t lo = start[R.cell_off], hi = start[R.cell_off + R.ncells];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        const float4 o = st[k];
        const double dx = (double)o.z, dy = (double)o.w;
        a0 += dx;
        a1 += dy;
        a2 += sqrt(dx * dx + dy * dy);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_acc[0][w] = a0;
        s_acc[1][w] = a1;
        s_acc[2][w] = a2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 3; ++k)
            for (int v = 0; v < 8; ++v) t[k] += s_acc[k][v];
        out[4 * blockIdx.x + 0] = (double)(hi - lo);
        out[4 * blockIdx.x + 1] = t[0];
        out[4 * blockIdx.x + 2] = t[1];
        out[4 * blockIdx.x + 3] = t[2];
    }
}

// One thread per read-buffer slot: insert (replica, id) into an open-
// addressing table; a key that is already there is a repeat.
__global__ void k_dup_check(const Rep* __restrict__ reps, int32_t nrep, const uint32_t* __restrict__ ids,
                            uint32_t n, unsigned long long* table, uint32_t cap, uint32_t* dup) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t r = nrep > 1 ? (uint32_t)rep_of_boid(reps, nrep, k) : 0u;
    const unsigned long long key = ((unsigned long long)r << 32) | ids[k];
    uint32_t h = id_mix(ids[k] ^ (r * 0x9E3779B9u)) & (cap - 1u);
    for (uint32_t probe = 0; probe < cap; ++probe) {  // the table is at most half full
        const unsigned long long prev = atomicCAS(table + h, ~0ull, key);
        if (prev == ~0ull) return;
        if (prev == key) {
            *dup = 1u;
            return;
        }
        h = (h + 1u) & (cap - 1u);
    }
    *dup = 1u;  // no free slot found (cannot happen at half occupancy): be conservative
}

__global__ void k_pack_locations(Rep R, const float2* __restrict__ xy, const float2* __restrict__ dxy,
                                 uint32_t n, float4* __restrict__ out_st, uint32_t* __restrict__ out_key,
                                 uint8_t* __restrict__ out_dead, uint32_t* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 p = xy[i], d = dxy[i];
    const int64_t idx = bag_index(R, disc(p.x, R), disc(p.y, R));
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(d.x) && isfinite(d.y)) || idx < 0) {
        atomicMin(bad, i);
        return;
    }
    out_st[i] = make_float4(p.x, p.y, d.x, d.y);
    out_key[i] = R.cell_off + (uint32_t)idx;
    out_dead[i] = 0;
}

// The same for records already packed as {x, y, last_d} (device-resident input).
__global__ void k_pack_states(Rep R, const float4* __restrict__ st, uint32_t n,
                              float4* __restrict__ out_st, uint32_t* __restrict__ out_key,
                              uint8_t* __restrict__ out_dead, uint32_t* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = st[i];
    const int64_t idx = bag_index(R, disc(v.x, R), disc(v.y, R));
    if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w)) || idx < 0) {
        atomicMin(bad, i);
        return;
    }
    out_st[i] = v;
    out_key[i] = R.cell_off + (uint32_t)idx;
    out_dead[i] = 0;
}

__global__ void k_set_rep(Rep* dst, Rep v) { *dst = v; }
__global__ void k_set_u64(unsigned long long* dst, unsigned long long v) { *dst = v; }
__global__ void k_add_u64(unsigned long long* dst, unsigned long long v) { *dst += v; }

inline unsigned grid_for(uint64_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t launch_repack(const PackEntry* plan, int32_t nplan, uint32_t total, const Rep* reps,
                          const float4* src_st, const uint32_t* src_ids, float4* dst_st,
                          uint32_t* dst_ids, uint32_t* dst_key, uint8_t* dst_dead, uint32_t* err,
                          cudaStream_t s) {
    if (total == 0 || nplan <= 0) return cudaSuccess;
    k_repack<<<grid_for(total, 256), 256, 0, s>>>(plan, nplan, total, reps, src_st, src_ids, dst_st,
                                                   dst_ids, dst_key, dst_dead, err);
    return cudaGetLastError();
}

cudaError_t launch_moments(const Rep* reps, uint32_t nrep, const uint32_t* start, const float4* st,
                           double* out, cudaStream_t s) {
    if (nrep == 0) return cudaSuccess;
    k_moments<<<nrep, 256, 0, s>>>(reps, start, st, out);
    return cudaGetLastError();
}

cudaError_t launch_dup_check(const Rep* reps, int32_t nrep, const uint32_t* ids, uint32_t n,
                             unsigned long long* table, uint32_t cap, uint32_t* dup,
                             cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(table, 0xFF, sizeof(unsigned long long) * cap, s);
    if (e != cudaSuccess || n == 0) return e;
    k_dup_check<<<grid_for(n, 256), 256, 0, s>>>(reps, nrep, ids, n, table, cap, dup);
    return cudaGetLastError();
}

cudaError_t launch_pack_locations(const Rep& rep, const float2* xy, const float2* dxy, uint32_t n,
                                  float4* out_st, uint32_t* out_key, uint8_t* out_dead,
                                  uint32_t* bad, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_pack_locations<<<grid_for(n, 256), 256, 0, s>>>(rep, xy, dxy, n, out_st, out_key, out_dead, bad);
    return cudaGetLastError();
}

cudaError_t launch_pack_states(const Rep& rep, const float4* st, uint32_t n, float4* out_st,
                               uint32_t* out_key, uint8_t* out_dead, uint32_t* bad, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_pack_states<<<grid_for(n, 256), 256, 0, s>>>(rep, st, n, out_st, out_key, out_dead, bad);
    return cudaGetLastError();
}

cudaError_t launch_set_rep(Rep* dst, const Rep& v, cudaStream_t s) {
    k_set_rep<<<1, 1, 0, s>>>(dst, v);
    return cudaGetLastError();
}
cudaError_t launch_set_u64(unsigned long long* dst, unsigned long long v, cudaStream_t s) {
    k_set_u64<<<1, 1, 0, s>>>(dst, v);
    return cudaGetLastError();
}
cudaError_t launch_add_u64(unsigned long long* dst, unsigned long long v, cudaStream_t s) {
    k_add_u64<<<1, 1, 0, s>>>(dst, v);
    return cudaGetLastError();
}

// ====================================================================== launchers
cudaError_t launch_scan(const uint32_t* in, uint32_t* out, uint32_t n, ScanCtl* ctl,
                        unsigned long long* tile_state, uint32_t* err, bool zero_in,
                        cudaStream_t s, WaitCfg wait) {
    const uint32_t nt = scan_tiles(n);
    if (nt == 0) {
        return cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
    }
    const uint32_t nt2 = (n + SCAN2_TILE - 1) / SCAN2_TILE;
    // tile_state holds scan_state_words(n) >= nt2 + 1 words: one sum per tile
    if (nt2 <= SCAN2_MAX_TILES) {
        cudaError_t e = launch_pdl(k_tile_sums, nt2, SCAN_THREADS, s, in, n, tile_state);
        if (e != cudaSuccess) return e;
        return launch_pdl(k_scan_tiles<false>, nt2, SCAN_THREADS, s, const_cast<uint32_t*>(in), out, n,
                          tile_state, zero_in ? 1 : 0, nt2);
    }
    // larger matrices: the tile sums scanned by one block in between (no
    // waits); the single-pass look-back scan below serves the largest ones
    // and the bounded-wait test of its look-back (wait.withhold)
    if (nt2 <= SCAN3_MAX_TILES && wait.withhold == ~0u) {
        cudaError_t e = launch_pdl(k_tile_sums, nt2, SCAN_THREADS, s, in, n, tile_state);
        if (e != cudaSuccess) return e;
        e = launch_pdl(k_scan_sums, 1u, (unsigned)SUMS_THREADS, s, tile_state, nt2);
        if (e != cudaSuccess) return e;
        return launch_pdl(k_scan_tiles<true>, nt2, SCAN_THREADS, s, const_cast<uint32_t*>(in), out, n,
                          tile_state, zero_in ? 1 : 0, nt2);
    }
    return launch_pdl(k_scan, nt, SCAN_THREADS, s, in, out, n, ctl, tile_state, err, zero_in ? 1 : 0, nt,
                      wait);
}

cudaError_t launch_flock_force(const ForceArgs& a, bool strict, int qmode, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    const bool multi = a.nrep > 1;
    if (multi && a.blk == nullptr) return cudaErrorInvalidValue;
    const unsigned g = multi ? a.nblk : grid_for(a.n, KB_FORCE_THREADS);
#define KB_FORCE(S, Q, MU)                                                                      \
    do {                                                                                        \
        if constexpr (MU) {                                                                     \
            if (a.block_threads == 128)                                                         \
                return launch_pdl(k_flock_force<S, Q, MU, false, 128>, g, 128, s, a);           \
            if (a.block_threads == 512)                                                         \
                return launch_pdl(k_flock_force<S, Q, MU, false, 512>, g, 512, s, a);           \
        }                                                                                       \
        return launch_pdl(k_flock_force<S, Q, MU>, g, KB_FORCE_THREADS, s, a);                  \
    } while (0)
    if (a.dense && qmode == 0 && !multi) {
        if (strict) return launch_pdl(k_flock_force<true, 0, false, true>, g, KB_FORCE_THREADS, s, a);
        return launch_pdl(k_flock_force<false, 0, false, true>, g, KB_FORCE_THREADS, s, a);
    }
    if (strict) {
        if (qmode == 0) { if (multi) KB_FORCE(true, 0, true); else KB_FORCE(true, 0, false); }
        else { if (multi) KB_FORCE(true, 1, true); else KB_FORCE(true, 1, false); }
    } else {
        if (qmode == 0) { if (multi) KB_FORCE(false, 0, true); else KB_FORCE(false, 0, false); }
        else { if (multi) KB_FORCE(false, 1, true); else KB_FORCE(false, 1, false); }
    }
#undef KB_FORCE
    return cudaGetLastError();
}

cudaError_t launch_flock_agents(const ForceArgs& a, const float4* in_st, const uint32_t* in_ids,
                               uint32_t nin, bool strict, int qmode, cudaStream_t s) {
    if (nin == 0) return cudaSuccess;
    if (a.nrep != 1) return cudaErrorInvalidValue;
    const unsigned g = grid_for(nin, KB_FORCE_THREADS);
    if (strict) {
        if (qmode == 0) k_flock_agents<true, 0><<<g, KB_FORCE_THREADS, 0, s>>>(a, in_st, in_ids, nin);
        else k_flock_agents<true, 1><<<g, KB_FORCE_THREADS, 0, s>>>(a, in_st, in_ids, nin);
    } else {
        if (qmode == 0) k_flock_agents<false, 0><<<g, KB_FORCE_THREADS, 0, s>>>(a, in_st, in_ids, nin);
        else k_flock_agents<false, 1><<<g, KB_FORCE_THREADS, 0, s>>>(a, in_st, in_ids, nin);
    }
    return cudaGetLastError();
}

cudaError_t launch_find_ids(const uint32_t* ids, const uint8_t* dead, const float4* st, uint32_t n,
                            const uint32_t* sorted, uint32_t m, uint32_t* first, float4* out,
                            cudaStream_t s) {
    if (m == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(first, 0xFF, sizeof(uint32_t) * m, s);
    if (e != cudaSuccess) return e;
    if (n) k_find_ids<<<grid_for(n, 256), 256, 0, s>>>(ids, dead, n, sorted, m, first);
    k_gather_found<<<grid_for(m, 256), 256, 0, s>>>(st, first, m, out);
    return cudaGetLastError();
}

cudaError_t launch_remove_ids(const uint32_t* ids, uint8_t* dead, uint32_t n, const uint32_t* sorted,
                              uint32_t m, uint32_t* removed, cudaStream_t s) {
    if (n == 0 || m == 0) return cudaSuccess;
    k_remove_ids<<<grid_for(n, 256), 256, 0, s>>>(ids, dead, n, sorted, m, removed);
    return cudaGetLastError();
}

cudaError_t launch_rebin(const RebinArgs& a, cudaStream_t s) {
    if (a.key != nullptr && a.nsegs > 0 && (a.nrep == 1 || a.sblk != nullptr)) {
        if (a.nrep > 1) return launch_pdl(k_rebin_seg<true>, a.nsblk, 32 * REBIN_SEG_WARPS, s, a);
        const unsigned gs = grid_for(a.nsegs, REBIN_SEG_WARPS);
        if (a.seg_rows == DENSE_SEG_ROWS)
            return launch_pdl(k_rebin_seg<false, DENSE_SEG_ROWS>, gs, 32 * REBIN_SEG_WARPS, s, a);
        if (a.seg_rows != 0 && a.seg_rows != SEG_ROWS) return cudaErrorInvalidValue;
        return launch_pdl(k_rebin_seg<false>, gs, 32 * REBIN_SEG_WARPS, s, a);
    }
    const unsigned g = grid_for(a.ncells > 0 ? a.ncells : 1, 256);
    if (a.nrep > 1) k_rebin<true><<<g, 256, 0, s>>>(a);
    else k_rebin<false><<<g, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_occupancy_sq(const uint32_t* start, uint32_t ncells, unsigned long long* out,
                                cudaStream_t s) {
    if (ncells == 0) return cudaSuccess;
    const unsigned g0 = grid_for(ncells, 256);
    const unsigned g = g0 < 608u ? g0 : 608u;  // grid-stride: four blocks per SM of 152
    k_occupancy_sq<<<g, 256, 0, s>>>(start, ncells, out);
    return cudaGetLastError();
}

cudaError_t launch_hist_list(const uint32_t* key, const uint8_t* dead, uint32_t n, uint32_t* hist,
                             cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_hist_list<<<grid_for(n, 256), 256, 0, s>>>(key, dead, n, hist);
    return cudaGetLastError();
}

cudaError_t launch_scatter_list(const uint32_t* key, const uint8_t* dead, const float4* st,
                                const uint32_t* ids, uint32_t n, const uint32_t* start,
                                uint32_t* cursor, float4* t_st, uint32_t* t_ids, uint32_t* t_src,
                                cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_scatter_list<<<grid_for(n, 256), 256, 0, s>>>(key, dead, st, ids, n, start, cursor, t_st,
                                                     t_ids, t_src);
    return cudaGetLastError();
}

cudaError_t launch_canon(const uint32_t* start, uint32_t ncells, const float4* t_st,
                         const uint32_t* t_ids, const uint32_t* t_src, uint32_t* cursor,
                         float4* s_st, uint32_t* s_ids, cudaStream_t s) {
    if (ncells == 0) return cudaSuccess;
    k_canon<<<grid_for(ncells, 256), 256, 0, s>>>(start, ncells, t_st, t_ids, t_src, cursor, s_st,
                                                  s_ids);
    return cudaGetLastError();
}

cudaError_t launch_query(const QueryArgs& a, cudaStream_t s) {
    if (a.nq == 0) return cudaSuccess;
    const unsigned g = grid_for(a.nq, 128);
    if (a.kind == 1) k_query<1><<<g, 128, 0, s>>>(a);
    else k_query<0><<<g, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_filter_key(const uint32_t* key, const uint8_t* dead, const float4* st,
                              const uint32_t* ids, uint32_t n, uint32_t target, uint32_t* out_ids,
                              float4* out_st, uint64_t cap, uint32_t* out_count, cudaStream_t s) {
    k_filter_key<<<1, FILTER_THREADS, 0, s>>>(key, dead, st, ids, n, target, out_ids, out_st, cap,
                                              out_count);
    return cudaGetLastError();
}

cudaError_t launch_remove(const uint32_t* key, uint8_t* dead, const uint32_t* ids, uint32_t n,
                          uint32_t target, uint32_t id, uint32_t* removed, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_remove<<<grid_for(n, 256), 256, 0, s>>>(key, dead, ids, n, target, id, removed);
    return cudaGetLastError();
}

cudaError_t launch_empty_bags(const Rep& rep, const uint32_t* start, float2* out, uint64_t cap,
                              uint32_t* out_count, cudaStream_t s) {
    k_empty_bags<<<1, FILTER_THREADS, 0, s>>>(rep, start, out, cap, out_count);
    return cudaGetLastError();
}

cudaError_t launch_cell_of(const uint32_t* start, uint32_t ncells, uint32_t* cell_of,
                           cudaStream_t s) {
    if (ncells == 0) return cudaSuccess;
    k_cell_of<<<grid_for(ncells, 256), 256, 0, s>>>(start, ncells, cell_of);
    return cudaGetLastError();
}

cudaError_t launch_cell_xy(const Rep& rep, const uint32_t* cell_of, uint32_t n, float2* out,
                           cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_cell_xy<<<grid_for(n, 256), 256, 0, s>>>(rep, cell_of, n, out);
    return cudaGetLastError();
}

}  // namespace kb
