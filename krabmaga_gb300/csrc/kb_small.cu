// kb_small.cu -- whole steps of a small field in one thread-block cluster.
//
// A field of at most SMALL_MAX_BOIDS boids and SMALL_MAX_CELLS bags (the
// 1,000-boid Flockers case, the reference's own test fields) is launch-bound
// on the separate-kernel path: four launches per step for a few microseconds
// of work.  Here a cluster of SMALL_CTAS blocks runs every step of the call
// in one launch.  Each block holds a full copy of the read buffer and its
// bag offsets in shared memory and owns one contiguous chunk of the boids:
//   1. agent pass: Bird::step for the chunk's boids against the local copy
//      (the same candidate order, accumulator and finish as k_flock_force);
//      next states and ids go to a local write list, and each bag key is
//      written into every block's copy of the list of keys (distributed
//      shared memory);
//   -- cluster barrier --
//   2. lazy_update: every block counts all keys in its own shared memory,
//      scans the counts into the next bag offsets, and places its own chunk:
//      position = offset of the bag + arrivals from lower-ranked blocks
//      (earlier in list order) + rank inside the chunk (one warp walks the
//      chunk in list order, __match_any_sync ranks equal keys, a per-bag
//      cursor carries the rank), which is the reference's insertion order
//      inside a bag; each record is written into every block's copy of the
//      next read buffer;
//   -- cluster barrier --
// and block 0 writes the final read buffer, offsets and step counter back.
// No bound on how far a boid moves is needed.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "kb_common.h"
#include "kb_device.cuh"
#include "kb_launch.h"

namespace cg = cooperative_groups;

namespace kb {
namespace {

constexpr uint32_t SMALL_FULL = 0xFFFFFFFFu;

// One candidate of the relaxed query in list order: self is skipped (by
// slot when ids are unique, else by id).
template <bool STRICT>
__device__ __forceinline__ void take_small(const Rep& R, const uint32_t* ids, uint32_t p, float4 o,
                                           float4 me, uint32_t my_id, uint32_t my_slot,
                                           Acc<STRICT>& acc) {
    const bool self = my_slot != 0xFFFFFFFFu ? p == my_slot : ids[p] == my_id;
    if (!self) acc.add(R, me.x, me.y, o);
}

// Bird::step's candidate sums for `me` against a read buffer in shared
// memory: the query's cells x-outer / y-inner (t_transform wraps the range
// where the field does), each bag in insertion order, the exact query's
// corner rule (check_circle) for QMODE 1.  Self is the slot my_slot when ids
// are unique, else every candidate with the boid's id.  The relaxed query of
// a clamped one-bag ring (the common case) walks its three column runs as one
// flat list, two candidates per iteration, so the loads and reciprocals of
// the next candidate overlap the sums of the current one (the sums are still
// taken in list order: the same bits).
template <bool STRICT, int QMODE>
__device__ __forceinline__ void gather_small(const Rep& R, const float4* st, const uint32_t* ids,
                                             const uint32_t* start, float4 me, uint32_t my_id,
                                             uint32_t my_slot, Acc<STRICT>& acc) {
    int mi, Mi, mj, Mj;
    if (!cell_range(R, me.x, me.y, R.dd, &mi, &Mi, &mj, &Mj)) return;
    if (QMODE == 0 && R.toroidal && !R.cell_wrap && Mi - mi < 3) {
        if (mj > Mj) return;
        uint32_t s[3], e[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            s[k] = e[k] = 0u;
            if (mi + k <= Mi) {
                const uint32_t colbase = (uint32_t)(mi + k) * (uint32_t)R.dh;
                s[k] = start[colbase + (uint32_t)mj];
                e[k] = start[colbase + (uint32_t)Mj + 1u];
            }
        }
        const uint32_t P1 = e[0] - s[0], P2 = P1 + (e[1] - s[1]), T = P2 + (e[2] - s[2]);
        const uint32_t d1 = s[1] - P1, d2 = s[2] - P2;  // position = f + d (mod 2^32)
        acc.vec += T;
        uint32_t f = 0;
        for (; f + 1u < T; f += 2u) {
            const uint32_t g = f + 1u;
            const uint32_t p0 = f < P1 ? s[0] + f : (f < P2 ? f + d1 : f + d2);
            const uint32_t p1 = g < P1 ? s[0] + g : (g < P2 ? g + d1 : g + d2);
            const float4 o0 = st[p0], o1 = st[p1];
            take_small(R, ids, p0, o0, me, my_id, my_slot, acc);
            take_small(R, ids, p1, o1, me, my_id, my_slot, acc);
        }
        if (f < T) {
            const uint32_t p0 = f < P1 ? s[0] + f : (f < P2 ? f + d1 : f + d2);
            take_small(R, ids, p0, st[p0], me, my_id, my_slot, acc);
        }
        return;
    }
    for (int ci = mi; ci <= Mi; ++ci) {
        const int bx = t_transform(ci, R.max_x);
        const uint32_t colbase = (uint32_t)bx * (uint32_t)R.dh;
        for (int cj = mj; cj <= Mj; ++cj) {
            const int by = t_transform(cj, R.max_y);
            const uint32_t c = colbase + (uint32_t)by;
            const uint32_t s = start[c], e = start[c + 1];
            if (s == e) continue;
            int check = 1;
            if (QMODE == 1) {
                check = check_circle(bx, by, R, me.x, me.y, R.radius);
                if (check == -1) continue;
            }
            for (uint32_t k = s; k < e; ++k) {
                const float4 o = st[k];
                if (QMODE == 1 && check == 0 &&
                    !(distance(me.x, me.y, o.x, o.y, R.w, R.h, R.toroidal != 0) <= R.radius))
                    continue;
                acc.vec += 1;
                const bool self = my_slot != 0xFFFFFFFFu ? k == my_slot : ids[k] == my_id;
                if (!self) acc.add(R, me.x, me.y, o);
            }
        }
    }
}

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total) by one block of
// SMALL_THREADS threads, n <= SMALL_THREADS * SMALL_SCAN_ITEMS; in may be out.
constexpr int SMALL_SCAN_ITEMS = (int)SMALL_MAX_CELLS / SMALL_THREADS;
static_assert(SMALL_SCAN_ITEMS * SMALL_THREADS == (int)SMALL_MAX_CELLS, "scan tiling");
__device__ __forceinline__ void block_scan_small(const uint32_t* in, uint32_t* out, uint32_t n,
                                                 uint32_t* warp_sums) {
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    constexpr uint32_t NW = SMALL_THREADS / 32;
    const uint32_t b = t * SMALL_SCAN_ITEMS;
    uint32_t v[SMALL_SCAN_ITEMS], sum = 0;
#pragma unroll
    for (int j = 0; j < SMALL_SCAN_ITEMS; ++j) {
        v[j] = b + j < n ? in[b + j] : 0u;
        sum += v[j];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(SMALL_FULL, incl, d);
        if (lane >= (uint32_t)d) incl += y;
    }
    if (lane == 31u) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t x = lane < NW ? warp_sums[lane] : 0u;
        uint32_t xi = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(SMALL_FULL, xi, d);
            if (lane >= (uint32_t)d) xi += y;
        }
        if (lane < NW) warp_sums[lane] = xi - x;  // exclusive prefix of each warp
        if (lane == 31u) warp_sums[32] = xi;      // total
    }
    __syncthreads();
    uint32_t run = warp_sums[w] + incl - sum;
#pragma unroll
    for (int j = 0; j < SMALL_SCAN_ITEMS; ++j) {
        if (b + j < n) out[b + j] = run;
        run += v[j];
    }
    if (t == 0) out[n] = warp_sums[32];
    __syncthreads();
}

// Shared-memory layout (byte offsets), the same in every block of the cluster.
struct SmallLayout {
    uint32_t rd_st, wr_st, rd_id, wr_id, wr_key, keys, start, nstart, cnt, cur, bytes;
};
__host__ __device__ inline SmallLayout small_layout(uint32_t n, uint32_t ncells, uint32_t chunk) {
    SmallLayout L{};
    uint32_t o = 0;
    L.rd_st = o;  o += n * 16u;
    L.wr_st = o;  o += chunk * 16u;
    L.rd_id = o;  o += n * 4u;
    L.wr_id = o;  o += chunk * 4u;
    L.wr_key = o; o += chunk * 4u;
    L.keys = o;   o += n * 4u;
    L.start = o;  o += (ncells + 1u) * 4u;
    L.nstart = o; o += (ncells + 1u) * 4u;
    L.cnt = o;    o += ncells * 4u;
    L.cur = o;    o += ncells * 4u;
    L.bytes = o;
    return L;
}

template <bool STRICT, int QMODE>
__global__ void __launch_bounds__(SMALL_THREADS, 1) k_small_steps(SmallArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    const Rep& R = a.rep;
    const uint32_t n = a.n, C = R.ncells;
    const uint32_t rank = cl.block_rank();
    const uint32_t chunk = (n + SMALL_CTAS - 1) / SMALL_CTAS;
    const uint32_t lo = min(n, rank * chunk), hi = min(n, lo + chunk);
    const SmallLayout Lo = small_layout(n, C, chunk);
    float4* rd_st = reinterpret_cast<float4*>(smem + Lo.rd_st);
    uint32_t* rd_id = reinterpret_cast<uint32_t*>(smem + Lo.rd_id);
    uint32_t* start = reinterpret_cast<uint32_t*>(smem + Lo.start);
    uint32_t* nstart = reinterpret_cast<uint32_t*>(smem + Lo.nstart);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + Lo.cnt);  // arrivals per bag
    uint32_t* cur = reinterpret_cast<uint32_t*>(smem + Lo.cur);  // lower-ranked arrivals, cursors
    uint32_t* keys = reinterpret_cast<uint32_t*>(smem + Lo.keys);  // every boid's next bag
    float4* wr_st = reinterpret_cast<float4*>(smem + Lo.wr_st);
    uint32_t* wr_id = reinterpret_cast<uint32_t*>(smem + Lo.wr_id);
    uint32_t* wr_key = reinterpret_cast<uint32_t*>(smem + Lo.wr_key);
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t s_err;
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < n; i += blockDim.x) {
        rd_st[i] = a.st[i];
        rd_id[i] = a.ids[i];
    }
    for (uint32_t c = t; c <= C; c += blockDim.x) start[c] = a.start[c];
    if (t == 0) s_err = 0u;
    unsigned long long step = *a.step;
    // every block of the cluster is running (its shared memory may be written
    // through the cluster) and has its whole copy loaded before any thread
    // reads a neighbour
    cl.sync();
    for (uint32_t s = 0; s < a.nsteps; ++s, ++step) {
        // 1. agent pass over the own chunk
        for (uint32_t c = t; c < C; c += blockDim.x) {
            cnt[c] = 0u;
            cur[c] = 0u;
        }
        for (uint32_t i = lo + t; i < hi; i += blockDim.x) {
            const float4 me = rd_st[i];
            const uint32_t my_id = rd_id[i];
            Acc<STRICT> acc;
            gather_small<STRICT, QMODE>(R, rd_st, rd_id, start, me, my_id,
                                        a.self_by_slot ? i : 0xFFFFFFFFu, acc);
            const float4 nx = finish_bird<STRICT>(R, me, my_id, step, acc);
            int64_t idx = bag_index(R, disc(nx.x, R), disc(nx.y, R));
            uint32_t flags = 0;
            if (idx < 0) {
                flags |= ERR_KEY_RANGE;
                idx = 0;
            }
            if (!isfinite(nx.x) || !isfinite(nx.y)) flags |= ERR_NONFINITE;
            if (flags) atomicOr(&s_err, flags);
            wr_st[i - lo] = nx;
            wr_id[i - lo] = my_id;
            wr_key[i - lo] = (uint32_t)idx;
#pragma unroll
            for (uint32_t q = 0; q < SMALL_CTAS; ++q) *cl.map_shared_rank(keys + i, q) = (uint32_t)idx;
        }
        cl.sync();  // every copy of the keys is complete; no block reads rd_* any more
        // 2. next offsets (all arrivals) and this chunk's cursors (arrivals
        //    from lower-ranked blocks, earlier in the list, come first in a bag)
        for (uint32_t i = t; i < n; i += blockDim.x) {
            atomicAdd(&cnt[keys[i]], 1u);
            if (i < lo) atomicAdd(&cur[keys[i]], 1u);
        }
        __syncthreads();
        block_scan_small(cnt, nstart, C, warp_sums);
        for (uint32_t c = t; c < C; c += blockDim.x) cur[c] += nstart[c];
        __syncthreads();
        if (t < 32u) {
            const uint32_t lt = (1u << t) - 1u;
            for (uint32_t base = 0; base < hi - lo; base += 32u) {
                const uint32_t j = base + t;
                const bool valid = j < hi - lo;
                const uint32_t k = valid ? wr_key[j] : 0xFFFFFFFFu;
                const uint32_t peers = __match_any_sync(SMALL_FULL, k);
                const uint32_t r = __popc(peers & lt);
                const uint32_t pos = valid ? cur[k] + r : 0u;
                __syncwarp();
                if (valid) {
                    if (r + 1u == (uint32_t)__popc(peers)) cur[k] = pos + 1u;
                    wr_key[j] = pos;  // the key becomes the destination slot
                }
                __syncwarp();
            }
        }
        __syncthreads();
        // every block's copy of the next read buffer gets this chunk
        for (uint32_t x = t; x < (hi - lo) * SMALL_CTAS; x += blockDim.x) {
            const uint32_t j = x / SMALL_CTAS, q = x % SMALL_CTAS;
            const uint32_t pos = wr_key[j];
            *cl.map_shared_rank(rd_st + pos, q) = wr_st[j];
            *cl.map_shared_rank(rd_id + pos, q) = wr_id[j];
        }
        for (uint32_t c = t; c <= C; c += blockDim.x) start[c] = nstart[c];
        cl.sync();  // every copy of the next read buffer is complete; counters are free
    }
    if (rank == 0) {
        for (uint32_t i = t; i < n; i += blockDim.x) {
            a.st[i] = rd_st[i];
            a.ids[i] = rd_id[i];
        }
        for (uint32_t c = t; c <= C; c += blockDim.x) a.start[c] = start[c];
        if (t == 0) *a.step = step;
    }
    __syncthreads();
    if (t == 0 && s_err) atomicOr(a.err, s_err);
}

}  // namespace

size_t small_smem_bytes(uint32_t n, uint32_t ncells) {
    return small_layout(n, ncells, (n + SMALL_CTAS - 1) / SMALL_CTAS).bytes;
}

cudaError_t launch_small_steps(const SmallArgs& a, bool strict, int qmode, cudaStream_t s) {
    if (a.nsteps == 0) return cudaSuccess;
    if (a.n == 0 || a.n > SMALL_MAX_BOIDS || a.rep.ncells > SMALL_MAX_CELLS || a.rep.cell_off != 0)
        return cudaErrorInvalidValue;
    const size_t bytes = small_smem_bytes(a.n, a.rep.ncells);
    void (*k)(SmallArgs) = strict ? (qmode == 0 ? k_small_steps<true, 0> : k_small_steps<true, 1>)
                                  : (qmode == 0 ? k_small_steps<false, 0> : k_small_steps<false, 1>);
    // the largest layout once per kernel (and device), not per launch
    static thread_local int opted[4] = {-1, -1, -1, -1};
    const int ki = (strict ? 2 : 0) + (qmode == 0 ? 0 : 1);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (opted[ki] != dev) {
        const size_t most = small_smem_bytes(SMALL_MAX_BOIDS, SMALL_MAX_CELLS);
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
        if (e != cudaSuccess) return e;
        opted[ki] = dev;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(SMALL_CTAS, 1, 1);
    cfg.blockDim = dim3(SMALL_THREADS, 1, 1);
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = SMALL_CTAS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, a);
}

}  // namespace kb
