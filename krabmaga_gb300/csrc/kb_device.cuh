// kb_device.cuh -- device helpers shared by the kernels: the reference's
// f32 helper functions with its rounding points, the query cell range, bag
// indexing, replica lookup and the per-boid force accumulator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kb_common.h"

namespace kb {

// ---------------------------------------------------------- f32 arithmetic
// STRICT: every operation rounds once, as the reference's Rust f32 code does
// (no fused multiply-add, IEEE division and square root).  FAST: the
// compiler may fuse, and divisions use the approximate reciprocal.
template <bool STRICT>
struct F;
template <>
struct F<true> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
};
// Single-instruction approximations (PTX rcp/sqrt/rsqrt .approx.ftz) for
// the fast arithmetic.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The fast arithmetic spells out every rounding too (fused multiply-adds
// only where written as __fmaf_rn), so the compiler cannot contract the same
// expression differently in different kernels: every step path gives the
// same bits in fast mode as well.
template <>
struct F<false> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fmul_rn(a, rcp_approx(b)); }
    static __device__ __forceinline__ float sqrt(float a) { return sqrt_approx(a); }
};

// field_2d.rs:1004-1014
__device__ __forceinline__ float toroidal_transform(float v, float dim) {
    if (v >= 0.0f && v < dim) return v;
    float r = fmodf(v, dim);
    if (r < 0.0f) r = __fadd_rn(r, dim);
    return r;
}

// field_2d.rs:988-1002
__device__ __forceinline__ float toroidal_distance(float a, float b, float dim) {
    float d0 = __fsub_rn(a, b);
    // dim / 2.0 is exact, so it equals dim * 0.5 bit for bit
    if (fabsf(d0) <= __fmul_rn(dim, 0.5f)) return d0;
    float d = __fsub_rn(toroidal_transform(a, dim), toroidal_transform(b, dim));
    float d2 = __fmul_rn(d, 2.0f);
    if (d2 > dim) return __fsub_rn(d, dim);
    if (d2 < -dim) return __fadd_rn(d, dim);
    return d;
}

// field_2d.rs:974-986
__device__ __forceinline__ float distance(float x1, float y1, float x2, float y2, float w, float h,
                                          bool tor) {
    float dx, dy;
    if (tor) {
        dx = toroidal_distance(x1, x2, w);
        dy = toroidal_distance(y1, y2, h);
    } else {
        dx = __fsub_rn(x1, x2);
        dy = __fsub_rn(y1, y2);
    }
    return __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
}

// field_2d.rs:934-972: 1 = whole bag inside, -1 = bag skipped, 0 = filter.
__device__ __forceinline__ int check_circle(int bx, int by, const Rep& R, float lx, float ly,
                                            float dis) {
    float nw_x = __fmul_rn((float)bx, R.d), nw_y = __fmul_rn((float)by, R.d);
    float ne_y = fminf(__fadd_rn(nw_y, R.d), R.h);
    float sw_x = fminf(__fadd_rn(nw_x, R.d), R.w);
    bool tor = R.toroidal != 0;
    float a = distance(nw_x, nw_y, lx, ly, R.w, R.h, tor);
    float b = distance(nw_x, ne_y, lx, ly, R.w, R.h, tor);
    float c = distance(sw_x, nw_y, lx, ly, R.w, R.h, tor);
    float e = distance(sw_x, ne_y, lx, ly, R.w, R.h, tor);
    if (a <= dis && b <= dis && c <= dis && e <= dis) return 1;
    if (a > dis && b > dis && c > dis && e > dis) return -1;
    return 0;
}

// floor(fl(v/d)) as i32 (field_2d.rs:328-339), bit-exact: fl(v * fl(1/d))
// is within ~2 ulp of the IEEE quotient fl(v/d), so their floors can only
// differ when the product lies within 4 ulp of an integer; only then is the
// IEEE quotient formed.  NaN and infinities take the same values as the
// direct form (NaN -> 0, saturation).
__device__ __forceinline__ int32_t disc_d(float v, float d, float inv_d) {
    const float q = v * inv_d;
    float f = floorf(q);
    const float fr = q - f;
    const float tol = fabsf(q) * 4.8e-7f;
    if (fr < tol || fr > 1.0f - tol) f = floorf(__fdiv_rn(v, d));
    return as_i32(f);
}
__device__ __forceinline__ int32_t disc(float v, const Rep& R) { return disc_d(v, R.d, R.inv_d); }
// x / dh and x % dh for a replica's bag index (x < 2^32).
__device__ __forceinline__ uint32_t div_dh(uint32_t x, const Rep& R) {
    return (uint32_t)__umul64hi((unsigned long long)x, R.dh_magic);
}

// The query's cell range (field_2d.rs:398-418 / 484-500).  False: dist <= 0.
__device__ __forceinline__ bool cell_range(const Rep& R, float x, float y, int32_t dd, int* mi,
                                           int* Mi, int* mj, int* Mj) {
    if (dd < 0) return false;
    int cx = disc(x, R), cy = disc(y, R);
    int a = cx - dd, b = cx + dd, c = cy - dd, e = cy + dd;
    if (R.toroidal && !R.cell_wrap) {
        a = max(0, a);
        b = min(b, R.max_x - 1);
        c = max(0, c);
        e = min(e, R.max_y - 1);
    } else if (R.toroidal) {
        // true torus: the range wraps (t_transform); a ring as wide as the
        // field visits every line once, in ascending order
        if (2 * dd + 1 >= R.max_x) { a = 0; b = R.max_x - 1; }
        if (2 * dd + 1 >= R.max_y) { c = 0; e = R.max_y - 1; }
    }
    *mi = a; *Mi = b; *mj = c; *Mj = e;
    return true;
}

// Reference bag index ((x*dh)+y) with i32 wrapping; -1 outside the matrix.
__device__ __forceinline__ int64_t bag_index(const Rep& R, int32_t cx, int32_t cy) {
    int32_t idx = (int32_t)((uint32_t)cx * (uint32_t)R.dh + (uint32_t)cy);
    if (idx < 0 || (uint32_t)idx >= R.ncells) return -1;
    return idx;
}

__device__ __forceinline__ uint32_t id_mix(uint32_t id) {
    uint32_t z = id * 0x9E3779B1u;
    z ^= z >> 15;
    z *= 0x85EBCA77u;
    z ^= z >> 13;
    return z;
}

// Replica owning boid slot i / cell c (tables sorted by offset).
__device__ __forceinline__ int rep_of_boid(const Rep* reps, int nrep, uint32_t i) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&reps[mid].boid_off) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_of_cell(const Rep* reps, int nrep, uint32_t c) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&reps[mid].cell_off) <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------- force pass
// One thread per boid of the read buffer: Bird::step (bird.rs:39-154)
// against the read buffer, next state into the write list at the same slot.
template <bool STRICT>
struct Acc {
    float xa = 0.f, ya = 0.f, xc = 0.f, yc = 0.f, xs = 0.f, ys = 0.f;
    int count = 0;
    uint32_t vec = 0;  // candidates including self (the reference's vec.len())

    // toroidal_distance's first branch is taken for every pair when the
    // replica guarantees it (Rep::nowrap, hoisted out of the loops by the
    // callers): the same bits, no test
    // COUNT = false: the caller sets count itself (a walk that knows how
    // many of its candidates are not the boid itself)
    template <bool NOWRAP = false, bool COUNT = true>
    __device__ __forceinline__ void add(const Rep& R, float sx, float sy, float4 o) {
        using M = F<STRICT>;
        const float dx = NOWRAP ? __fsub_rn(sx, o.x) : toroidal_distance(sx, o.x, R.w);
        const float dy = NOWRAP ? __fsub_rn(sy, o.y) : toroidal_distance(sy, o.y, R.h);
        add_d<COUNT>(dx, dy, o);
    }
    template <bool COUNT = true>
    __device__ __forceinline__ void add_d(float dx, float dy, float4 o) {
        using M = F<STRICT>;
        if (COUNT) count += 1;
        if (STRICT) {
            float sq = M::add(M::mul(dx, dx), M::mul(dy, dy));
            float q = M::add(M::mul(sq, sq), 1.0f);
            xa = M::add(xa, M::div(dx, q));
            ya = M::add(ya, M::div(dy, q));
        } else {
            const float sq = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            const float inv = rcp_approx(__fmaf_rn(sq, sq, 1.0f));
            xa = __fmaf_rn(dx, inv, xa);
            ya = __fmaf_rn(dy, inv, ya);
        }
        xc = M::add(xc, dx);
        yc = M::add(yc, dy);
        xs = M::add(xs, o.z);
        ys = M::add(ys, o.w);
    }
};

// k-th candidate source line of line X (k = 0..7): the lines a bag of line X
// can receive boids from in one step.  X >= seam receives from line 0 (moves
// wrapping past x = w), line 0 from every line >= seam (moves wrapping below
// x = 0), every line from X-1..X+1.  -1 when absent.  With seam >= 2 the
// sequence is non-decreasing, so skipping values <= the last taken (and
// outside 0..maxv) yields the ascending unique set.
__device__ __forceinline__ int src_line(int k, int X, int maxv, int seam) {
    if (k == 0) return X >= seam ? 0 : -1;
    if (k <= 3) return X + (k - 2);
    return X == 0 ? seam + (k - 4) : -1;
}
constexpr int SRC_LINES = 8;

// The one-step move check of the stencil rebin (see src_line).
__device__ __forceinline__ bool move_ok(int o, int n, int seam) {
    return abs(n - o) <= 1 || (n == 0 && o >= seam) || (o == 0 && n >= seam);
}

// bird.rs:84-149: averages, avoidance/cohesion/consistency, Philox jitter
// (only when the candidate list is non-empty), the weighted sum, the JUMP
// normalisation and the toroidal move.  Returns {x, y, dx, dy}.
template <bool STRICT>
__device__ __forceinline__ float4 finish_bird(const Rep& R, float4 me, uint32_t my_id,
                                              unsigned long long step, const Acc<STRICT>& acc) {
    using M = F<STRICT>;
    float avx = 0.f, avy = 0.f, cox = 0.f, coy = 0.f, rax = 0.f, ray = 0.f, csx = 0.f, csy = 0.f;
    if (acc.vec > 0) {
        float xa = acc.xa, ya = acc.ya, xc = acc.xc, yc = acc.yc, xs = acc.xs, ys = acc.ys;
        if (acc.count > 0 && !STRICT) {
            const float ic = rcp_approx((float)acc.count);
            xa = __fmul_rn(xa, ic); ya = __fmul_rn(ya, ic);
            xc = __fmul_rn(xc, ic); yc = __fmul_rn(yc, ic);
            xs = __fmul_rn(xs, ic); ys = __fmul_rn(ys, ic);
            csx = __fmul_rn(xs, ic);  // bird.rs:91-94: a second division by count
            csy = __fmul_rn(ys, ic);
        } else if (acc.count > 0) {
            const float c = (float)acc.count;
            xa = M::div(xa, c); ya = M::div(ya, c);
            xc = M::div(xc, c); yc = M::div(yc, c);
            xs = M::div(xs, c); ys = M::div(ys, c);
            csx = M::div(xs, c);  // bird.rs:91-94: a second division by count
            csy = M::div(ys, c);
        } else {
            csx = xs;
            csy = ys;
        }
        avx = M::mul(400.0f, xa);
        avy = M::mul(400.0f, ya);
        cox = M::div(-xc, 10.0f);
        coy = M::div(-yc, 10.0f);
        // the replica's own step number keys the jitter stream
        const unsigned long long ls =
            step - (((unsigned long long)R.origin_hi << 32) | (unsigned long long)R.origin_lo);
        const U4 o = philox4x32_10(U4{my_id, (uint32_t)ls, (uint32_t)(ls >> 32), STREAM_JITTER},
                                   R.seed_lo, R.seed_hi);
        const float xr = M::sub(M::mul(unit_f32(o.x), 2.0f), 1.0f);
        const float yr = M::sub(M::mul(unit_f32(o.y), 2.0f), 1.0f);
        if (STRICT) {
            const float sq = M::sqrt(M::add(M::mul(xr, xr), M::mul(yr, yr)));
            rax = M::div(M::mul(0.05f, xr), sq);
            ray = M::div(M::mul(0.05f, yr), sq);
        } else {
            const float rs = __fmul_rn(0.05f, rsqrt_approx(__fmaf_rn(xr, xr, __fmul_rn(yr, yr))));
            rax = __fmul_rn(xr, rs);
            ray = __fmul_rn(yr, rs);
        }
    }
    float dx, dy;
    if (STRICT) {
        dx = M::add(M::add(M::add(M::add(M::mul(R.coh, cox), M::mul(R.avo, avx)),
                                  M::mul(R.con, csx)),
                           M::mul(R.rnd, rax)),
                    M::mul(R.mom, me.z));
        dy = M::add(M::add(M::add(M::add(M::mul(R.coh, coy), M::mul(R.avo, avy)),
                                  M::mul(R.con, csy)),
                           M::mul(R.rnd, ray)),
                    M::mul(R.mom, me.w));
    } else {
        dx = __fmaf_rn(R.mom, me.z, __fmaf_rn(R.rnd, rax, __fmaf_rn(R.con, csx,
                       __fmaf_rn(R.avo, avx, __fmul_rn(R.coh, cox)))));
        dy = __fmaf_rn(R.mom, me.w, __fmaf_rn(R.rnd, ray, __fmaf_rn(R.con, csy,
                       __fmaf_rn(R.avo, avy, __fmul_rn(R.coh, coy)))));
    }
    if (STRICT) {
        const float dis = M::sqrt(M::add(M::mul(dx, dx), M::mul(dy, dy)));
        if (dis > 0.0f) {
            dx = M::mul(M::div(dx, dis), R.jump);
            dy = M::mul(M::div(dy, dis), R.jump);
        }
    } else {
        const float d2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
        if (d2 > 0.0f) {
            const float s = __fmul_rn(rsqrt_approx(d2), R.jump);
            dx = __fmul_rn(dx, s);
            dy = __fmul_rn(dy, s);
        }
    }
    const float nx = toroidal_transform(__fadd_rn(me.x, dx), R.w);
    const float ny = toroidal_transform(__fadd_rn(me.y, dy), R.w);  // bird.rs:147: y wraps with w

    return make_float4(nx, ny, dx, dy);
}

}  // namespace kb
