// kb_gen.cpp -- seeded synthetic flocks (host only, no GPU needed).
//
// The reference initialises birds with an unseeded rand::rng()
// (tests/model/flockers/state.rs:41-56: pos = dim * U[0,1), last_d = 0).
// These generators draw the same distributions from Philox4x32-10 so that a
// workload is reproducible from its seed.
#include <cmath>
#include <cstring>

#include "../../include/krabgpu.h"
#include "kb_common.h"
#include "kb_runtime.h"

namespace kb {

// Unit heading from Philox draws by rejection in the unit disc: uniform in
// angle and made of IEEE operations only (no libm), so host and device give
// the same bits.
static void unit_heading(uint32_t id, uint64_t seed, uint32_t first_z, uint32_t first_w, float* hx,
                         float* hy) {
    uint32_t z = first_z, w = first_w;
    for (uint32_t attempt = 1;; ++attempt) {
        const float a = unit_f32(z) * 2.0f - 1.0f;
        const float b = unit_f32(w) * 2.0f - 1.0f;
        const float r2 = a * a + b * b;
        if (r2 > 0.0f && r2 <= 1.0f) {
            const float r = std::sqrt(r2);
            *hx = a / r;
            *hy = b / r;
            return;
        }
        const U4 o = philox4x32_10(U4{id, attempt, 0u, STREAM_INIT}, (uint32_t)seed,
                                   (uint32_t)(seed >> 32));
        z = o.z;
        w = o.w;
    }
}

// field_2d.rs:1004-1014 in double, for wrapping generated positions.
static double wrap(double v, double dim) {
    if (v >= 0.0 && v < dim) return v;
    double r = std::fmod(v, dim);
    if (r < 0.0) r += dim;
    return r;
}

}  // namespace kb

using namespace kb;

extern "C" {

kb_status kb_gen_uniform(size_t n, float w, float h, uint64_t seed, float heading_scale,
                         uint32_t* ids, float* xy, float* dxy) {
    if (n && (!ids || !xy || !dxy)) return fail(KB_ERR_ARG, "null argument");
    if (!(w > 0.0f) || !(h > 0.0f) || n > 0xFFFFFFFFull) return fail(KB_ERR_ARG, "bad size");
    for (size_t i = 0; i < n; ++i) {
        const uint32_t id = (uint32_t)i;
        const U4 o = philox4x32_10(U4{id, 0u, 0u, STREAM_INIT}, (uint32_t)seed, (uint32_t)(seed >> 32));
        ids[i] = id;
        xy[2 * i] = w * unit_f32(o.x);
        xy[2 * i + 1] = h * unit_f32(o.y);
        float hx, hy;
        unit_heading(id, seed, o.z, o.w, &hx, &hy);
        dxy[2 * i] = hx * heading_scale;
        dxy[2 * i + 1] = hy * heading_scale;
    }
    return KB_OK;
}

kb_status kb_gen_clustered(size_t n, float w, float h, uint32_t nclusters, float sigma,
                           float angle_sigma, uint64_t seed, uint32_t* ids, float* xy, float* dxy) {
    if (n && (!ids || !xy || !dxy)) return fail(KB_ERR_ARG, "null argument");
    if (!(w > 0.0f) || !(h > 0.0f) || nclusters == 0 || n > 0xFFFFFFFFull)
        return fail(KB_ERR_ARG, "bad size");
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const double two_pi = 6.283185307179586;
    for (size_t i = 0; i < n; ++i) {
        const uint32_t id = (uint32_t)i;
        const uint32_t c = id % nclusters;
        const U4 oc = philox4x32_10(U4{c, 0u, 0u, 2u}, k0, k1);  // cluster centre + angle
        const double cx = (double)w * unit_f32(oc.x), cy = (double)h * unit_f32(oc.y);
        const double theta = two_pi * unit_f32(oc.z);
        const U4 o = philox4x32_10(U4{id, 0u, 0u, 3u}, k0, k1);  // Box-Muller draws
        const double u1 = ((double)(o.x >> 8) + 0.5) / 16777216.0;
        const double u2 = (double)(o.y >> 8) / 16777216.0;
        const double u3 = ((double)(o.z >> 8) + 0.5) / 16777216.0;
        const double u4 = (double)(o.w >> 8) / 16777216.0;
        const double r = std::sqrt(-2.0 * std::log(u1));
        const double g1 = r * std::cos(two_pi * u2), g2 = r * std::sin(two_pi * u2);
        const double g3 = std::sqrt(-2.0 * std::log(u3)) * std::cos(two_pi * u4);
        float px = (float)wrap(cx + sigma * g1, w);
        float py = (float)wrap(cy + sigma * g2, h);
        if (px >= w) px = 0.0f;  // rounding to f32 can land on the seam
        if (py >= h) py = 0.0f;
        const double ang = theta + angle_sigma * g3;
        ids[i] = id;
        xy[2 * i] = px;
        xy[2 * i + 1] = py;
        dxy[2 * i] = (float)std::cos(ang);
        dxy[2 * i + 1] = (float)std::sin(ang);
    }
    return KB_OK;
}

}  // extern "C"
