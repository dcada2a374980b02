// kb_common.h -- definitions shared by the host runtime (g++) and the
// kernels (nvcc): replica/geometry records, Philox4x32-10, the reference's
// f32 helper functions, and the error-word bits.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define KB_HD __host__ __device__ __forceinline__
#else
#define KB_HD inline
#endif

namespace kb {

// Device error-word bits (mirrored as KB_FLAG_* in include/krabgpu.h).
enum : uint32_t {
    ERR_KEY_RANGE = 0x1u,
    ERR_REBIN_MISS = 0x2u,
    ERR_SPIN_TIMEOUT = 0x4u,
    ERR_NONFINITE = 0x8u,
    // which check raised a rebin miss (set together with ERR_REBIN_MISS)
    ERR_MISS_GATHER = 0x10u,   // a bag gathered a different count than its offsets say
    ERR_MISS_OUTSIDE = 0x20u,  // a boid sits outside the bag its slot belongs to
    ERR_MISS_MOVE = 0x40u,     // a boid moved further than the neighbouring bag
    ERR_MISS_TILE = 0x80u,     // a tile was refused (ring wider than the layout)
    ERR_MISS_MATERIALIZE = 0x100u,  // the standalone rebin found a different count
};

// One simulation on the device: its Field2D geometry (field_2d.rs:304-322),
// its slice of the packed cell and boid arrays, and its Flockers parameters
// (bird.rs:12-17).  A plain field is a table of one replica; a sweep packs
// many, each with its own geometry and parameters.
struct Rep {
    float w, h, d;          // width, height, discretization
    int32_t toroidal;       // clamp (1) or wrap (0) the query's cell range
    int32_t max_x, max_y;   // ceil(w/d), ceil(h/d)   (field_2d.rs:396-397)
    int32_t dw, dh;         // max_x+1, max_y+1       (field_2d.rs:316-317)
    uint32_t cell_off;      // first cell of this replica in the packed cell index space
    uint32_t ncells;        // dw*dh
    uint32_t boid_off;      // first slot of this replica in the packed boid arrays
    uint32_t nboids;
    // Flockers parameters
    float coh, avo, con, rnd, mom, jump, radius;
    int32_t dd;             // floor(radius/d) (field_2d.rs:488), -1 when radius <= 0
    int32_t qmode;          // 0 relax, 1 exact
    uint32_t seed_lo, seed_hi;
    int32_t nowrap;         // 1: no candidate pair can straddle the seam ((dd+1)*d < min(w,h)/2)
    uint32_t origin_lo, origin_hi;  // global step at which this replica's step 0 ran
    int32_t seam;           // first line from which a one-step move can wrap to line 0
    float inv_d;            // fl(1/d), for the exact fast discretisation
    uint32_t seg_off;       // first 32-bag column segment of this replica (segment rebin)
    unsigned long long dh_magic;  // ceil(2^64 / dh): n / dh == umul64hi(n, dh_magic) for n < 2^32
    int32_t cell_wrap;      // toroidal fields: 0 clamp the query's cell range (the reference), 1 wrap it
    int32_t seg_rows;       // bags per segment of the packed segment rebin (0: the default)
};

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two 32x32
// multiplies with the Weyl key schedule between rounds.
constexpr uint32_t PHILOX_M0 = 0xD2511F53u, PHILOX_M1 = 0xCD9E8D57u;
constexpr uint32_t PHILOX_W0 = 0x9E3779B9u, PHILOX_W1 = 0xBB67AE85u;

KB_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
#ifdef __CUDA_ARCH__
    *hi = __umulhi(a, b);
    *lo = a * b;
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
#endif
}

struct U4 {
    uint32_t x, y, z, w;
};

KB_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(PHILOX_M0, c.x, &hi0, &lo0);
        mulhilo32(PHILOX_M1, c.z, &hi1, &lo1);
        U4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        c = n;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    return c;
}

// The f32 sample rand 0.9 draws from a u32 (top 24 bits scaled by 2^-24).
KB_HD float unit_f32(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// Counter-word 3 separates the streams keyed on the same (seed, id).
constexpr uint32_t STREAM_JITTER = 0u;   // ctr = (id, step lo, step hi, 0)
constexpr uint32_t STREAM_INIT = 1u;     // ctr = (id, attempt, 0, 1)

// ------------------------------------------------------- reference helpers
// Rust `f as i32`: truncation, saturating, NaN -> 0.  On the device that is
// the conversion instruction itself (cvt.rzi.s32.f32 saturates and maps NaN
// to 0); on the host the checks are spelled out.
KB_HD int32_t as_i32(float v) {
#ifdef __CUDA_ARCH__
    return __float2int_rz(v);
#else
    if (!(v == v)) return 0;
    if (v >= 2147483647.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)v;
#endif
}

// field_2d.rs:926-932
KB_HD int32_t t_transform(int32_t n, int32_t size) {
    return n >= 0 ? n % size : (n % size) + size;
}

}  // namespace kb
