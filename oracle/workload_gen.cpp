// workload_gen.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle library).
//
// The seeded synthetic flocks of the benchmark workloads, restated on the
// oracle side so that the CPU arms (the timed reference-equivalent run and
// its baseline) build their inputs without loading the GPU library.  The
// reference initialises birds from an unseeded rand::rng()
// (tests/model/flockers/state.rs:41-56: pos = dim * U[0,1), last_d = 0); the
// workloads draw the same distributions from Philox4x32-10 so that a run is
// reproducible from its seed.  The draws are:
//
//   uniform:   counter (id, 0, 0, 1) -> x = w*u(o0), y = h*u(o1); the unit
//              heading by rejection in the unit disc from (o2, o3), further
//              candidates from counters (id, attempt, 0, 1), attempt = 1, 2, ..
//   clustered: cluster c = id mod K; counter (c, 0, 0, 2) -> centre
//              (w*u(o0), h*u(o1)) and mean angle 2*pi*u(o2); counter
//              (id, 0, 0, 3) -> Box-Muller normals for the offset (sigma) and
//              the angle noise; positions wrapped onto the torus.
//
// Every f32 operation is a plain IEEE operation (built with
// -ffp-contract=off), so x86 and Arm hosts give the same bits, and the
// library's own generator gives the same bits as this one (checked by
// tests/test_workload_gen.py).
#include <cmath>
#include <cstddef>
#include <cstdint>

namespace {

const uint32_t GM0 = 0xD2511F53u, GM1 = 0xCD9E8D57u;
const uint32_t GW0 = 0x9E3779B9u, GW1 = 0xBB67AE85u;

struct Draw {
    uint32_t v[4];
};

// Philox4x32-10 (Salmon et al., SC'11) on counter (a, b, c, d), key = seed.
Draw philox(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint64_t seed) {
    uint32_t x[4] = {a, b, c, d};
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int round = 0; round < 10; ++round) {
        const uint64_t m0 = (uint64_t)GM0 * x[0];
        const uint64_t m1 = (uint64_t)GM1 * x[2];
        const uint32_t y0 = (uint32_t)(m1 >> 32) ^ x[1] ^ k0;
        const uint32_t y1 = (uint32_t)m1;
        const uint32_t y2 = (uint32_t)(m0 >> 32) ^ x[3] ^ k1;
        const uint32_t y3 = (uint32_t)m0;
        x[0] = y0; x[1] = y1; x[2] = y2; x[3] = y3;
        k0 += GW0;
        k1 += GW1;
    }
    return Draw{{x[0], x[1], x[2], x[3]}};
}

// The top 24 bits of a draw scaled into [0, 1) (rand 0.9's f32 sample).
inline float unit(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// Wrap a double onto [0, dim) (field_2d.rs:1004-1014 in double).
double wrap_d(double v, double dim) {
    if (v >= 0.0 && v < dim) return v;
    double r = std::fmod(v, dim);
    if (r < 0.0) r += dim;
    return r;
}

void heading(uint32_t id, uint64_t seed, uint32_t z, uint32_t w, float* hx, float* hy) {
    uint32_t attempt = 0;
    for (;;) {
        const float a = unit(z) * 2.0f - 1.0f;
        const float b = unit(w) * 2.0f - 1.0f;
        const float r2 = a * a + b * b;
        if (r2 > 0.0f && r2 <= 1.0f) {
            const float r = std::sqrt(r2);
            *hx = a / r;
            *hy = b / r;
            return;
        }
        ++attempt;
        const Draw o = philox(id, attempt, 0u, 1u, seed);
        z = o.v[2];
        w = o.v[3];
    }
}

}  // namespace

extern "C" {

// n boids uniform on a w x h torus with unit headings scaled by heading_scale.
int orc_gen_uniform(size_t n, float w, float h, uint64_t seed, float heading_scale, uint32_t* ids,
                    float* xy, float* dxy) {
    if (n > 0xFFFFFFFFull || !(w > 0.0f) || !(h > 0.0f)) return -1;
    for (size_t i = 0; i < n; ++i) {
        const uint32_t id = (uint32_t)i;
        const Draw o = philox(id, 0u, 0u, 1u, seed);
        ids[i] = id;
        xy[2 * i] = w * unit(o.v[0]);
        xy[2 * i + 1] = h * unit(o.v[1]);
        float hx, hy;
        heading(id, seed, o.v[2], o.v[3], &hx, &hy);
        dxy[2 * i] = hx * heading_scale;
        dxy[2 * i + 1] = hy * heading_scale;
    }
    return 0;
}

// n boids in k Gaussian clusters (offset sigma, heading = cluster angle plus
// N(0, angle_sigma)) on a w x h torus.
int orc_gen_clustered(size_t n, float w, float h, uint32_t k, float sigma, float angle_sigma,
                      uint64_t seed, uint32_t* ids, float* xy, float* dxy) {
    if (n > 0xFFFFFFFFull || !(w > 0.0f) || !(h > 0.0f) || k == 0) return -1;
    const double tau = 6.283185307179586;
    const double two24 = 16777216.0;
    for (size_t i = 0; i < n; ++i) {
        const uint32_t id = (uint32_t)i;
        const Draw c = philox(id % k, 0u, 0u, 2u, seed);
        const double cx = (double)w * unit(c.v[0]);
        const double cy = (double)h * unit(c.v[1]);
        const double mean_angle = tau * unit(c.v[2]);
        const Draw g = philox(id, 0u, 0u, 3u, seed);
        // Box-Muller: the radius draws are shifted by half a step off zero
        const double p1 = ((double)(g.v[0] >> 8) + 0.5) / two24;
        const double q1 = (double)(g.v[1] >> 8) / two24;
        const double p2 = ((double)(g.v[2] >> 8) + 0.5) / two24;
        const double q2 = (double)(g.v[3] >> 8) / two24;
        const double rad = std::sqrt(-2.0 * std::log(p1));
        const double nx = rad * std::cos(tau * q1);
        const double ny = rad * std::sin(tau * q1);
        const double na = std::sqrt(-2.0 * std::log(p2)) * std::cos(tau * q2);
        float px = (float)wrap_d(cx + sigma * nx, w);
        float py = (float)wrap_d(cy + sigma * ny, h);
        if (px >= w) px = 0.0f;  // a double just below w can round up to w in f32
        if (py >= h) py = 0.0f;
        const double ang = mean_angle + angle_sigma * na;
        ids[i] = id;
        xy[2 * i] = px;
        xy[2 * i + 1] = py;
        dxy[2 * i] = (float)std::cos(ang);
        dxy[2 * i + 1] = (float)std::sin(ang);
    }
    return 0;
}

}  // extern "C"
