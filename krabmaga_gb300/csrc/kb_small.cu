// kb_small.cu -- whole steps of a small field in one thread block.
//
// A field of at most SMALL_MAX_BOIDS boids and SMALL_MAX_CELLS bags (the
// reference's own test fields) is launch-bound on the separate-kernel path:
// four launches per step for a few microseconds of work.  Here one
// 1024-thread block loads the read buffer and its bag offsets into shared
// memory and runs every step of the call there:
//   1. the agent pass: Bird::step for every boid against the read buffer
//      (the same candidate order, accumulator and finish as k_flock_force),
//      next states into a write list in read order, arrivals counted per bag;
//   2. lazy_update: an exclusive scan of the arrivals into the next bag
//      offsets, then a stable scatter of the write list by bag key by one
//      warp in list order (__match_any_sync ranks equal keys by lane, a
//      per-bag cursor carries the rank across batches), which is the
//      reference's insertion order inside a bag;
// and writes the final read buffer, its offsets and the step counter back.
// The scatter needs no bound on how far a boid moves.  Beyond a few hundred
// boids one SM's issue rate and the one-warp scatter cost more than the
// separate kernels' launches (the bound SMALL_MAX_BOIDS is measured).
#include <cuda_runtime.h>

#include "kb_common.h"
#include "kb_device.cuh"
#include "kb_launch.h"

namespace kb {
namespace {

constexpr uint32_t SMALL_FULL = 0xFFFFFFFFu;

// Bird::step's candidate sums for `me` against a read buffer in shared
// memory: the query's cells x-outer / y-inner (t_transform wraps the range
// where the field does), each bag in insertion order, the exact query's
// corner rule (check_circle) for QMODE 1.  Self is the slot my_slot when ids
// are unique, else every candidate with the boid's id.
template <bool STRICT, int QMODE>
__device__ __forceinline__ void gather_small(const Rep& R, const float4* st, const uint32_t* ids,
                                             const uint32_t* start, float4 me, uint32_t my_id,
                                             uint32_t my_slot, Acc<STRICT>& acc) {
    int mi, Mi, mj, Mj;
    if (!cell_range(R, me.x, me.y, R.dd, &mi, &Mi, &mj, &Mj)) return;
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

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total), n <= 4096, by
// a 1024-thread block; in[] is zeroed as it is read.
__device__ __forceinline__ void block_scan_small(uint32_t* in, uint32_t* out, uint32_t n,
                                                 uint32_t* warp_sums) {
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    const uint32_t b = t * 4u;
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
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
        uint32_t x = warp_sums[lane], xi = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(SMALL_FULL, xi, d);
            if (lane >= (uint32_t)d) xi += y;
        }
        warp_sums[lane] = xi - x;  // exclusive prefix of each warp
        if (lane == 31u) warp_sums[32] = xi;  // total
    }
    __syncthreads();
    uint32_t run = warp_sums[w] + incl - sum;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (b + j < n) {
            out[b + j] = run;
            in[b + j] = 0u;
        }
        run += v[j];
    }
    if (t == 0) out[n] = warp_sums[32];
    __syncthreads();
}

template <bool STRICT, int QMODE>
__global__ void __launch_bounds__(SMALL_THREADS, 1) k_small_steps(SmallArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Rep& R = a.rep;
    const uint32_t n = a.n, C = R.ncells;
    float4* s_rd = reinterpret_cast<float4*>(smem);   // read buffer (canonical)
    float4* s_wr = s_rd + n;                           // write list (read order)
    uint32_t* i_rd = reinterpret_cast<uint32_t*>(s_wr + n);
    uint32_t* i_wr = i_rd + n;
    uint32_t* key = i_wr + n;
    uint32_t* start = key + n;          // offsets of the read buffer (C+1)
    uint32_t* nstart = start + C + 1;   // offsets of the next one (C+1)
    uint32_t* cnt = nstart + C + 1;     // arrivals per bag, then the scatter cursors (C)
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t s_err;
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < n; i += blockDim.x) {
        s_rd[i] = a.st[i];
        i_rd[i] = a.ids[i];
    }
    for (uint32_t c = t; c <= C; c += blockDim.x) start[c] = a.start[c];
    for (uint32_t c = t; c < C; c += blockDim.x) cnt[c] = 0u;
    if (t == 0) s_err = 0u;
    unsigned long long step = *a.step;
    __syncthreads();
    for (uint32_t s = 0; s < a.nsteps; ++s, ++step) {
        // 1. agent pass
        for (uint32_t i = t; i < n; i += blockDim.x) {
            const float4 me = s_rd[i];
            const uint32_t my_id = i_rd[i];
            Acc<STRICT> acc;
            gather_small<STRICT, QMODE>(R, s_rd, i_rd, start, me, my_id,
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
            s_wr[i] = nx;
            i_wr[i] = my_id;
            key[i] = (uint32_t)idx;
            atomicAdd(&cnt[idx], 1u);
        }
        __syncthreads();
        // 2. lazy_update: next offsets, cursors, stable scatter
        block_scan_small(cnt, nstart, C, warp_sums);
        for (uint32_t c = t; c < C; c += blockDim.x) cnt[c] = nstart[c];
        __syncthreads();
        if (t < 32u) {
            const uint32_t lt = (1u << t) - 1u;
            for (uint32_t base = 0; base < n; base += 32u) {
                const uint32_t i = base + t;
                const bool valid = i < n;
                const uint32_t k = valid ? key[i] : 0xFFFFFFFFu;
                const uint32_t peers = __match_any_sync(SMALL_FULL, k);
                const uint32_t rank = __popc(peers & lt);
                const uint32_t pos = valid ? cnt[k] + rank : 0u;
                __syncwarp();
                if (valid) {
                    if (rank + 1u == (uint32_t)__popc(peers)) cnt[k] = pos + 1u;
                    s_rd[pos] = s_wr[i];
                    i_rd[pos] = i_wr[i];
                }
                __syncwarp();
            }
        }
        __syncthreads();
        for (uint32_t c = t; c <= C; c += blockDim.x) {
            start[c] = nstart[c];
            if (c < C) cnt[c] = 0u;
        }
        __syncthreads();
    }
    for (uint32_t i = t; i < n; i += blockDim.x) {
        a.st[i] = s_rd[i];
        a.ids[i] = i_rd[i];
    }
    for (uint32_t c = t; c <= C; c += blockDim.x) a.start[c] = start[c];
    if (t == 0) {
        *a.step = step;
        if (s_err) atomicOr(a.err, s_err);
    }
}

}  // namespace

size_t small_smem_bytes(uint32_t n, uint32_t ncells) {
    return (size_t)n * (2 * sizeof(float4) + 3 * sizeof(uint32_t)) +
           (size_t)(3 * (size_t)ncells + 2) * sizeof(uint32_t);
}

cudaError_t launch_small_steps(const SmallArgs& a, bool strict, int qmode, cudaStream_t s) {
    if (a.nsteps == 0) return cudaSuccess;
    if (a.n > SMALL_MAX_BOIDS || a.rep.ncells > SMALL_MAX_CELLS || a.rep.cell_off != 0)
        return cudaErrorInvalidValue;
    const size_t bytes = small_smem_bytes(a.n, a.rep.ncells);
    void (*k)(SmallArgs) = strict ? (qmode == 0 ? k_small_steps<true, 0> : k_small_steps<true, 1>)
                                  : (qmode == 0 ? k_small_steps<false, 0> : k_small_steps<false, 1>);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    k<<<1, SMALL_THREADS, bytes, s>>>(a);
    return cudaGetLastError();
}

}  // namespace kb
