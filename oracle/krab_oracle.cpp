// krab_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of krABMaga's sequential continuous-space path, used by the
// parity tests and by the CPU-baseline leg of bench.py.  Nothing in the
// product (krabmaga_gb300/, include/) links or calls this file.
//
// It restates, in f32 with the reference's own rounding points:
//   * Field2D, sequential build  (src/engine/fields/field_2d.rs:267-1014)
//   * Bird::step                  (tests/model/flockers/bird.rs:39-154)
//   * Flocker::init / update      (tests/model/flockers/state.rs:41-60)
//   * Schedule::step              (src/engine/schedule.rs:347-413)
//   * simulate_old! timing        (src/lib.rs:1473-1582)
// plus an FP64 force mode (same f32 neighbour sets, force arithmetic in
// double) for the one-step tolerance check, and an independent restatement of
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11) for the jitter term.  The reference draws its
// jitter from an unseeded `rand::rng()` (bird.rs:113-117); both this oracle
// and the GPU library replace it with Philox keyed on (seed, agent id, step).
//
// Must be compiled with -ffp-contract=off: Rust never fuses a*b+c, so neither
// may the oracle (gcc fuses by default on aarch64).
//
// Schedule order.  The reference pops agents from a PriorityQueue whose order
// for equal priorities is unspecified (schedule.rs:377-393, crate
// priority-queue 2.0.2), and that order decides the order of each write bag.
// The parity mode fixes it: agents run in the read buffer's iteration order
// (cells ascending by index x*dh+y, each bag in insertion order), which is
// exactly what iter_objects (field_2d.rs:619-640) visits.  The timing mode
// keeps a binary-heap schedule like the reference (ties broken by insertion).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- Philox
// Philox4x32-10: 10 rounds, Weyl key schedule between rounds.
const uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
const uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += PH_W0; k1 += PH_W1; }
        uint64_t p0 = (uint64_t)PH_M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)PH_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// rand 0.9's f32 sample from a u32: the top 24 bits scaled by 2^-24 -> [0,1).
inline float u32_to_unit_f32(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// Jitter stream: counter (id, step lo, step hi, 0), key (seed lo, seed hi).
void jitter_pair(uint64_t seed, uint32_t id, uint64_t step, float* r1, float* r2) {
    uint32_t ctr[4] = {id, (uint32_t)step, (uint32_t)(step >> 32), 0u};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    philox4x32_10(ctr, key, o);
    *r1 = u32_to_unit_f32(o[0]);
    *r2 = u32_to_unit_f32(o[1]);
}

// ---------------------------------------------------------------- helpers
// Rust `f as i32`: saturating, NaN -> 0.
inline int32_t as_i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483647.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

// field_2d.rs:926-932
inline int t_transform(int n, int size) { return n >= 0 ? n % size : (n % size) + size; }

// field_2d.rs:1004-1014
inline float toroidal_transform(float val, float dim) {
    if (val >= 0.0f && val < dim) return val;
    float v = std::fmod(val, dim);
    if (v < 0.0f) v += dim;
    return v;
}
inline double toroidal_transform_d(double val, double dim) {
    if (val >= 0.0 && val < dim) return val;
    double v = std::fmod(val, dim);
    if (v < 0.0) v += dim;
    return v;
}

// field_2d.rs:988-1002
inline float toroidal_distance(float a, float b, float dim) {
    if (std::fabs(a - b) <= dim / 2.0f) return a - b;
    float d = toroidal_transform(a, dim) - toroidal_transform(b, dim);
    if (d * 2.0f > dim) return d - dim;
    if (d * 2.0f < -dim) return d + dim;
    return d;
}
inline double toroidal_distance_d(double a, double b, double dim) {
    if (std::fabs(a - b) <= dim / 2.0) return a - b;
    double d = toroidal_transform_d(a, dim) - toroidal_transform_d(b, dim);
    if (d * 2.0 > dim) return d - dim;
    if (d * 2.0 < -dim) return d + dim;
    return d;
}

// field_2d.rs:974-986
inline float distance(float x1, float y1, float x2, float y2, float dim1, float dim2, bool tor) {
    float dx, dy;
    if (tor) {
        dx = toroidal_distance(x1, x2, dim1);
        dy = toroidal_distance(y1, y2, dim2);
    } else {
        dx = x1 - x2;
        dy = y1 - y2;
    }
    return std::sqrt(dx * dx + dy * dy);
}

// field_2d.rs:934-972
int check_circle(int bx, int by, float disc, float width, float height, float lx, float ly,
                 float dis, bool tor) {
    float nw_x = (float)bx * disc, nw_y = (float)by * disc;
    float ne_x = nw_x, ne_y = std::min(nw_y + disc, height);
    float sw_x = std::min(nw_x + disc, width), sw_y = nw_y;
    float se_x = sw_x, se_y = ne_y;
    float a = distance(nw_x, nw_y, lx, ly, width, height, tor);
    float b = distance(ne_x, ne_y, lx, ly, width, height, tor);
    float c = distance(sw_x, sw_y, lx, ly, width, height, tor);
    float e = distance(se_x, se_y, lx, ly, width, height, tor);
    if (a <= dis && b <= dis && c <= dis && e <= dis) return 1;
    if (a > dis && b > dis && c > dis && e > dis) return -1;
    return 0;
}

// bird.rs:20-25 (the unused `flag` is dropped)
struct Bird {
    uint32_t id;
    float x, y;    // pos
    float dx, dy;  // last_d
};

// ---------------------------------------------------------------- Field2D
struct Field2D {
    std::vector<std::vector<Bird>> bags[2];
    int read = 0, write = 1;
    size_t nagents = 0;
    float width, height, disc;
    bool toroidal;
    bool cell_wrap = false;  // toroidal only: wrap the query's cell range instead of clamping it
    int dh, dw;
    size_t density_estimation = 0;
    bool density_check = false;
    size_t nbags;
    bool panicked = false;  // set where the reference would panic (index out of range)

    // field_2d.rs:304-322
    Field2D(float w, float h, float d, bool t) : width(w), height(h), disc(d), toroidal(t) {
        nbags = (size_t)((std::ceil(w / d) + 1.0f) * (std::ceil(h / d) + 1.0f));
        bags[0].assign(nbags, {});
        bags[1].assign(nbags, {});
        dh = as_i32(std::ceil(h / d)) + 1;
        dw = as_i32(std::ceil(w / d)) + 1;
    }
    int max_x() const { return as_i32(std::ceil(width / disc)); }
    int max_y() const { return as_i32(std::ceil(height / disc)); }

    // field_2d.rs:328-339
    void discretize(float x, float y, int* cx, int* cy) const {
        *cx = as_i32(std::floor(x / disc));
        *cy = as_i32(std::floor(y / disc));
    }
    // bag index ((x*dh)+y) as usize; -1 where the reference would index out of range
    int64_t bag_index(int cx, int cy) const {
        int64_t idx = (int64_t)(int32_t)((uint32_t)cx * (uint32_t)dh + (uint32_t)cy);
        if (idx < 0 || (size_t)idx >= nbags) return -1;
        return idx;
    }

    // field_2d.rs:838-846
    bool set_object_location(const Bird& b, float lx, float ly) {
        int cx, cy;
        discretize(lx, ly, &cx, &cy);
        int64_t idx = bag_index(cx, cy);
        if (idx < 0) { panicked = true; return false; }
        bags[write][idx].push_back(b);
        if (!density_check) nagents += 1;
        return true;
    }

    // field_2d.rs:885-898
    bool remove_object_location(const Bird& b, float lx, float ly) {
        int cx, cy;
        discretize(lx, ly, &cx, &cy);
        int64_t idx = bag_index(cx, cy);
        if (idx < 0) { panicked = true; return false; }
        auto& bag = bags[write][idx];
        if (!bag.empty()) {
            size_t before = bag.size();
            bag.erase(std::remove_if(bag.begin(), bag.end(),
                                     [&](const Bird& o) { return o.id == b.id; }),
                      bag.end());
            size_t after = bag.size();
            if (!density_check) nagents -= before - after;
        }
        return true;
    }

    // field_2d.rs:905-921
    void lazy_update() {
        std::swap(read, write);
        if (!density_check) {
            density_estimation = nagents / (size_t)(dw * dh);
            density_check = true;
            bags[write].assign(nbags, {});
            for (auto& b : bags[write]) b.reserve(density_estimation);
        } else {
            for (auto& b : bags[write]) b.clear();
        }
    }

    // Shared cell-range logic of field_2d.rs:398-418 / 484-500.
    bool cell_range(float lx, float ly, float dist, int* mi, int* Mi, int* mj, int* Mj) const {
        if (dist <= 0.0f) return false;
        int dd = as_i32(std::floor(dist / disc));
        int cx, cy;
        discretize(lx, ly, &cx, &cy);
        int mx = max_x(), my = max_y();
        int min_i = cx - dd, max_i = cx + dd, min_j = cy - dd, max_j = cy + dd;
        if (toroidal && !cell_wrap) {
            min_i = std::max(0, min_i);
            max_i = std::min(max_i, mx - 1);
            min_j = std::max(0, min_j);
            max_j = std::min(max_j, my - 1);
        } else if (toroidal) {
            // The true-torus option (not in the reference): the range wraps
            // through t_transform; a ring as wide as the field visits every
            // line once, in ascending order.
            if (2 * dd + 1 >= mx) { min_i = 0; max_i = mx - 1; }
            if (2 * dd + 1 >= my) { min_j = 0; max_j = my - 1; }
        }
        *mi = min_i; *Mi = max_i; *mj = min_j; *Mj = max_j;
        return true;
    }

    // field_2d.rs:472-516
    void neighbors_relax(float lx, float ly, float dist, std::vector<Bird>& out) const {
        int mi, Mi, mj, Mj;
        if (!cell_range(lx, ly, dist, &mi, &Mi, &mj, &Mj)) return;
        int mx = max_x(), my = max_y();
        for (int i = mi; i <= Mi; ++i)
            for (int j = mj; j <= Mj; ++j) {
                int bx = t_transform(i, mx), by = t_transform(j, my);
                size_t idx = (size_t)(bx * dh + by);
                for (const Bird& e : bags[read][idx]) out.push_back(e);
            }
    }

    // field_2d.rs:386-440
    void neighbors_exact(float lx, float ly, float dist, std::vector<Bird>& out) const {
        int mi, Mi, mj, Mj;
        if (!cell_range(lx, ly, dist, &mi, &Mi, &mj, &Mj)) return;
        int mx = max_x(), my = max_y();
        for (int i = mi; i <= Mi; ++i)
            for (int j = mj; j <= Mj; ++j) {
                int bx = t_transform(i, mx), by = t_transform(j, my);
                int check = check_circle(bx, by, disc, width, height, lx, ly, dist, toroidal);
                size_t idx = (size_t)(bx * dh + by);
                for (const Bird& e : bags[read][idx]) {
                    if ((check == 0 &&
                         distance(lx, ly, e.x, e.y, width, height, toroidal) <= dist) ||
                        check == 1)
                        out.push_back(e);
                }
            }
    }
};

struct FlockParams {  // bird.rs:12-17 statics, made per-run parameters
    float cohesion, avoidance, consistency, randomness, momentum, jump;
    float radius;        // bird.rs:41 uses 10.0
    int query_mode;      // 0 = relax (field_2d.rs:472), 1 = exact (field_2d.rs:386)
    uint64_t seed;
};

// bird.rs:39-154 in f32.  `self_b` is the agent's own copy (its read-buffer
// state); returns the bird to write and its new location.
Bird bird_step(const Field2D& f, const FlockParams& p, const Bird& self_b, uint64_t step,
               std::vector<Bird>& vec) {
    vec.clear();
    if (p.query_mode == 0) f.neighbors_relax(self_b.x, self_b.y, p.radius, vec);
    else f.neighbors_exact(self_b.x, self_b.y, p.radius, vec);
    const float width = f.width, height = f.height;

    float avoid_x = 0.f, avoid_y = 0.f, cohe_x = 0.f, cohe_y = 0.f;
    float rand_x = 0.f, rand_y = 0.f, cons_x = 0.f, cons_y = 0.f;

    if (!vec.empty()) {
        float x_avoid = 0.f, y_avoid = 0.f, x_cohe = 0.f, y_cohe = 0.f, x_cons = 0.f, y_cons = 0.f;
        int count = 0;
        for (const Bird& e : vec) {
            if (self_b.id != e.id) {
                float dx = toroidal_distance(self_b.x, e.x, width);
                float dy = toroidal_distance(self_b.y, e.y, height);
                count += 1;
                float square = dx * dx + dy * dy;
                x_avoid += dx / (square * square + 1.0f);
                y_avoid += dy / (square * square + 1.0f);
                x_cohe += dx;
                y_cohe += dy;
                x_cons += e.dx;
                y_cons += e.dy;
            }
        }
        if (count > 0) {
            float c = (float)count;
            x_avoid /= c; y_avoid /= c;
            x_cohe /= c; y_cohe /= c;
            x_cons /= c; y_cons /= c;
            cons_x = x_cons / c;  // bird.rs:91-94 divides by count a second time
            cons_y = y_cons / c;
        } else {
            cons_x = x_cons;
            cons_y = y_cons;
        }
        avoid_x = 400.0f * x_avoid;
        avoid_y = 400.0f * y_avoid;
        cohe_x = -x_cohe / 10.0f;
        cohe_y = -y_cohe / 10.0f;

        float r1, r2;
        jitter_pair(p.seed, self_b.id, step, &r1, &r2);
        float x_rand = r1 * 2.0f - 1.0f;
        float y_rand = r2 * 2.0f - 1.0f;
        float sq = std::sqrt(x_rand * x_rand + y_rand * y_rand);
        rand_x = 0.05f * x_rand / sq;
        rand_y = 0.05f * y_rand / sq;
    }

    float dx = p.cohesion * cohe_x + p.avoidance * avoid_x + p.consistency * cons_x +
               p.randomness * rand_x + p.momentum * self_b.dx;
    float dy = p.cohesion * cohe_y + p.avoidance * avoid_y + p.consistency * cons_y +
               p.randomness * rand_y + p.momentum * self_b.dy;
    float dis = std::sqrt(dx * dx + dy * dy);
    if (dis > 0.0f) {
        dx = dx / dis * p.jump;
        dy = dy / dis * p.jump;
    }
    Bird nb = self_b;
    nb.dx = dx;
    nb.dy = dy;
    nb.x = toroidal_transform(self_b.x + dx, width);
    nb.y = toroidal_transform(self_b.y + dy, width);  // bird.rs:147 wraps y with the width
    return nb;
}

// The same step with the force arithmetic in double (neighbour set from the
// f32 query).  out = {x, y, dx, dy} before any rounding to f32.
void bird_step_fp64(const Field2D& f, const FlockParams& p, const Bird& self_b, uint64_t step,
                    std::vector<Bird>& vec, double out[4]) {
    vec.clear();
    if (p.query_mode == 0) f.neighbors_relax(self_b.x, self_b.y, p.radius, vec);
    else f.neighbors_exact(self_b.x, self_b.y, p.radius, vec);
    const double width = f.width, height = f.height;
    double avoid_x = 0, avoid_y = 0, cohe_x = 0, cohe_y = 0, rand_x = 0, rand_y = 0, cons_x = 0,
           cons_y = 0;
    if (!vec.empty()) {
        double x_avoid = 0, y_avoid = 0, x_cohe = 0, y_cohe = 0, x_cons = 0, y_cons = 0;
        int count = 0;
        for (const Bird& e : vec) {
            if (self_b.id != e.id) {
                double dx = toroidal_distance_d(self_b.x, e.x, width);
                double dy = toroidal_distance_d(self_b.y, e.y, height);
                count += 1;
                double square = dx * dx + dy * dy;
                x_avoid += dx / (square * square + 1.0);
                y_avoid += dy / (square * square + 1.0);
                x_cohe += dx;
                y_cohe += dy;
                x_cons += e.dx;
                y_cons += e.dy;
            }
        }
        if (count > 0) {
            double c = count;
            x_avoid /= c; y_avoid /= c; x_cohe /= c; y_cohe /= c; x_cons /= c; y_cons /= c;
            cons_x = x_cons / c;
            cons_y = y_cons / c;
        } else {
            cons_x = x_cons;
            cons_y = y_cons;
        }
        avoid_x = 400.0 * x_avoid;
        avoid_y = 400.0 * y_avoid;
        cohe_x = -x_cohe / 10.0;
        cohe_y = -y_cohe / 10.0;
        float r1, r2;
        jitter_pair(p.seed, self_b.id, step, &r1, &r2);
        double x_rand = (double)r1 * 2.0 - 1.0, y_rand = (double)r2 * 2.0 - 1.0;
        double sq = std::sqrt(x_rand * x_rand + y_rand * y_rand);
        rand_x = 0.05 * x_rand / sq;
        rand_y = 0.05 * y_rand / sq;
    }
    double dx = (double)p.cohesion * cohe_x + (double)p.avoidance * avoid_x +
                (double)p.consistency * cons_x + (double)p.randomness * rand_x +
                (double)p.momentum * (double)self_b.dx;
    double dy = (double)p.cohesion * cohe_y + (double)p.avoidance * avoid_y +
                (double)p.consistency * cons_y + (double)p.randomness * rand_y +
                (double)p.momentum * (double)self_b.dy;
    double dis = std::sqrt(dx * dx + dy * dy);
    if (dis > 0.0) {
        dx = dx / dis * (double)p.jump;
        dy = dy / dis * (double)p.jump;
    }
    out[0] = toroidal_transform_d((double)self_b.x + dx, width);
    out[1] = toroidal_transform_d((double)self_b.y + dy, width);
    out[2] = dx;
    out[3] = dy;
}

// Agents in the read buffer's iteration order (see the header comment).
void read_order(const Field2D& f, std::vector<Bird>& agents) {
    agents.clear();
    for (size_t c = 0; c < f.nbags; ++c)
        for (const Bird& b : f.bags[f.read][c]) agents.push_back(b);
}

// One Schedule::step for the Flocker model (schedule.rs:347-413): every agent
// steps against the read buffer and writes into the write buffer, then
// State::update -> lazy_update swaps them.  The caller has already done the
// step-0 lazy_update (schedule.rs:349-351).
// The agent pass of one Schedule::step (schedule.rs:395-408): every agent
// of the read buffer, in read order, writes its next state into the write
// buffer.  The field's lazy_update follows separately.
bool flock_compute(Field2D& f, const FlockParams& p, uint64_t step) {
    std::vector<Bird> agents, vec;
    read_order(f, agents);
    for (const Bird& a : agents) {
        Bird nb = bird_step(f, p, a, step, vec);
        if (!f.set_object_location(nb, nb.x, nb.y)) return false;
    }
    return true;
}

bool flock_step(Field2D& f, const FlockParams& p, uint64_t step) {
    if (!flock_compute(f, p, step)) return false;
    f.lazy_update();
    return true;
}

// Priority-queue schedule with the reference's cost structure (one heap
// entry per agent, pop every agent at the current time, re-push at time+1).
struct Event {
    float time;
    int ordering;
    uint64_t seq;
    Bird bird;
};
struct EventLess {
    // std::priority_queue pops the "largest": earliest time, then lowest
    // ordering (priority.rs:21-38), then insertion sequence.
    bool operator()(const Event& a, const Event& b) const {
        if (a.time != b.time) return a.time > b.time;
        if (a.ordering != b.ordering) return a.ordering > b.ordering;
        return a.seq > b.seq;
    }
};

}  // namespace

// ====================================================================== C API
extern "C" {

typedef struct {
    float cohesion, avoidance, consistency, randomness, momentum, jump, radius;
    int32_t query_mode;
    uint64_t seed;
} orc_params;

static FlockParams to_params(const orc_params* p) {
    FlockParams f;
    f.cohesion = p->cohesion; f.avoidance = p->avoidance; f.consistency = p->consistency;
    f.randomness = p->randomness; f.momentum = p->momentum; f.jump = p->jump;
    f.radius = p->radius; f.query_mode = p->query_mode; f.seed = p->seed;
    return f;
}

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    philox4x32_10(ctr, key, out);
}

void orc_jitter_pair(uint64_t seed, uint32_t id, uint64_t step, float* r1, float* r2) {
    jitter_pair(seed, id, step, r1, r2);
}

void* orc_field_new(float w, float h, float d, int toroidal) {
    return new Field2D(w, h, d, toroidal != 0);
}
void orc_field_free(void* f) { delete (Field2D*)f; }
void orc_field_set_cell_wrap(void* f, int wrap) { ((Field2D*)f)->cell_wrap = wrap != 0; }

void orc_field_dims(void* fp, int32_t* out4) {
    Field2D* f = (Field2D*)fp;
    out4[0] = f->dw; out4[1] = f->dh; out4[2] = f->max_x(); out4[3] = f->max_y();
}

size_t orc_field_nagents(void* f) { return ((Field2D*)f)->nagents; }
int orc_field_panicked(void* f) { return ((Field2D*)f)->panicked ? 1 : 0; }

// set_object_location(Bird{id, (x,y), (dx,dy)}, loc=(lx,ly)); 0 ok, -1 reference panic
int orc_field_set(void* fp, uint32_t id, float x, float y, float dx, float dy, float lx, float ly) {
    Bird b{id, x, y, dx, dy};
    return ((Field2D*)fp)->set_object_location(b, lx, ly) ? 0 : -1;
}
// bulk form: loc = the bird's own position (what Bird::step and Flocker::init do)
int orc_field_set_many(void* fp, size_t n, const uint32_t* ids, const float* xy, const float* dxy) {
    Field2D* f = (Field2D*)fp;
    for (size_t i = 0; i < n; ++i) {
        Bird b{ids[i], xy[2 * i], xy[2 * i + 1], dxy[2 * i], dxy[2 * i + 1]};
        if (!f->set_object_location(b, b.x, b.y)) return -1;
    }
    return 0;
}
int orc_field_remove(void* fp, uint32_t id, float lx, float ly) {
    Bird b{id, 0, 0, 0, 0};
    return ((Field2D*)fp)->remove_object_location(b, lx, ly) ? 0 : -1;
}
void orc_field_lazy_update(void* f) { ((Field2D*)f)->lazy_update(); }

// kind: 0 relax query, 1 exact query, 2 get_objects, 3 get_objects_unbuffered.
// Writes up to cap ids (and, if state != NULL, {x,y,dx,dy}); returns the full
// count, or -1 where the reference would panic.
int64_t orc_field_query(void* fp, int kind, float x, float y, float dist, uint32_t* ids,
                        float* state, size_t cap) {
    Field2D* f = (Field2D*)fp;
    std::vector<Bird> v;
    if (kind == 0) f->neighbors_relax(x, y, dist, v);
    else if (kind == 1) f->neighbors_exact(x, y, dist, v);
    else {
        int cx, cy;
        f->discretize(x, y, &cx, &cy);
        int64_t idx = f->bag_index(cx, cy);
        if (idx < 0) return -1;
        v = f->bags[kind == 2 ? f->read : f->write][idx];
    }
    for (size_t i = 0; i < v.size() && i < cap; ++i) {
        if (ids) ids[i] = v[i].id;
        if (state) {
            state[4 * i] = v[i].x; state[4 * i + 1] = v[i].y;
            state[4 * i + 2] = v[i].dx; state[4 * i + 3] = v[i].dy;
        }
    }
    return (int64_t)v.size();
}

// field_2d.rs:803-808 num_objects_at_location
int64_t orc_field_num_at(void* fp, float x, float y) {
    Field2D* f = (Field2D*)fp;
    int cx, cy;
    f->discretize(x, y, &cx, &cy);
    int64_t idx = f->bag_index(cx, cy);
    if (idx < 0) return -1;
    return (int64_t)f->bags[f->read][idx].size();
}

// field_2d.rs:727-739 get_empty_bags: (i*d, j*d) for empty read bags, i outer.
size_t orc_field_empty_bags(void* fp, float* xy, size_t cap) {
    Field2D* f = (Field2D*)fp;
    size_t n = 0;
    for (int i = 0; i < f->dw; ++i)
        for (int j = 0; j < f->dh; ++j) {
            size_t idx = (size_t)(i * f->dh + j);
            if (f->bags[f->read][idx].empty()) {
                if (n < cap) { xy[2 * n] = (float)i * f->disc; xy[2 * n + 1] = (float)j * f->disc; }
                ++n;
            }
        }
    return n;
}

// field_2d.rs:619-640 / 677-698 iteration order; buffered=1 read, 0 write.
// cells[i] = bag index of object i.
size_t orc_field_iter(void* fp, int buffered, uint32_t* ids, float* state, uint32_t* cells,
                      size_t cap) {
    Field2D* f = (Field2D*)fp;
    int buf = buffered ? f->read : f->write;
    size_t n = 0;
    for (size_t c = 0; c < f->nbags; ++c)
        for (const Bird& b : f->bags[buf][c]) {
            if (n < cap) {
                if (ids) ids[n] = b.id;
                if (state) {
                    state[4 * n] = b.x; state[4 * n + 1] = b.y;
                    state[4 * n + 2] = b.dx; state[4 * n + 3] = b.dy;
                }
                if (cells) cells[n] = (uint32_t)c;
            }
            ++n;
        }
    return n;
}

// Candidate lists of many query points against the read buffer, each list in
// the reference's visiting order.  counts[q] = list length; ids are packed.
// Returns the total, or -1 if cap was too small.
int64_t orc_neighbor_lists(void* fp, int kind, float dist, size_t nq, const float* qxy,
                           uint32_t* counts, uint32_t* ids, size_t cap) {
    Field2D* f = (Field2D*)fp;
    std::vector<Bird> v;
    size_t total = 0;
    bool over = false;
    for (size_t q = 0; q < nq; ++q) {
        v.clear();
        if (kind == 0) f->neighbors_relax(qxy[2 * q], qxy[2 * q + 1], dist, v);
        else f->neighbors_exact(qxy[2 * q], qxy[2 * q + 1], dist, v);
        counts[q] = (uint32_t)v.size();
        for (const Bird& b : v) {
            if (total < cap) ids[total] = b.id;
            else over = true;
            ++total;
        }
    }
    return over ? -1 : (int64_t)total;
}

// Per query point: candidate count and an order-independent id digest
// (sum over candidates of a 32-bit mix of the id), for full-size checks.
void orc_neighbor_digest(void* fp, int kind, float dist, size_t nq, const float* qxy,
                         uint32_t* counts, uint32_t* digest) {
    Field2D* f = (Field2D*)fp;
    std::vector<Bird> v;
    for (size_t q = 0; q < nq; ++q) {
        v.clear();
        if (kind == 0) f->neighbors_relax(qxy[2 * q], qxy[2 * q + 1], dist, v);
        else f->neighbors_exact(qxy[2 * q], qxy[2 * q + 1], dist, v);
        uint32_t h = 0;
        for (const Bird& b : v) {
            uint32_t z = b.id * 0x9E3779B1u;
            z ^= z >> 15; z *= 0x85EBCA77u; z ^= z >> 13;
            h += z;
        }
        counts[q] = (uint32_t)v.size();
        digest[q] = h;
    }
}

// `nsteps` Schedule::step calls of the Flocker model on field f, with step
// numbers first_step.. (parity mode: read-buffer iteration order).  The field
// must already hold the agents in its read buffer.  0 ok, -1 reference panic.
int orc_flock_compute(void* fp, const orc_params* pp, uint64_t step) {
    return flock_compute(*(Field2D*)fp, to_params(pp), step) ? 0 : -1;
}

// Bird::step of one agent held by the caller (bird.rs:39-154) against the
// read buffer; out4 = its next {x, y, dx, dy}.  Nothing is written.
void orc_bird_step(void* fp, const orc_params* pp, uint64_t step, uint32_t id, const float* in4,
                   float* out4) {
    std::vector<Bird> vec;
    const Bird b{id, in4[0], in4[1], in4[2], in4[3]};
    const Bird nb = bird_step(*(Field2D*)fp, to_params(pp), b, step, vec);
    out4[0] = nb.x; out4[1] = nb.y; out4[2] = nb.dx; out4[3] = nb.dy;
}

// Agents that the caller holds (ids, states n x 4), stepped in order
// against the read buffer and written into the write buffer.
int orc_flock_compute_agents(void* fp, const orc_params* pp, uint64_t step, size_t n,
                             const uint32_t* ids, const float* states) {
    Field2D* f = (Field2D*)fp;
    const FlockParams p = to_params(pp);
    std::vector<Bird> vec;
    for (size_t j = 0; j < n; ++j) {
        const Bird b{ids[j], states[4 * j], states[4 * j + 1], states[4 * j + 2], states[4 * j + 3]};
        const Bird nb = bird_step(*f, p, b, step, vec);
        if (!f->set_object_location(nb, nb.x, nb.y)) return -1;
    }
    return 0;
}

// Every write-buffer object whose id is in ids[0..n) removed (each one as
// remove_object_location at its write location); returns the count.
size_t orc_field_remove_ids(void* fp, size_t n, const uint32_t* ids) {
    Field2D* f = (Field2D*)fp;
    std::vector<uint32_t> s(ids, ids + n);
    std::sort(s.begin(), s.end());
    size_t removed = 0;
    for (auto& bag : f->bags[f->write]) {
        const size_t before = bag.size();
        bag.erase(std::remove_if(bag.begin(), bag.end(),
                                 [&](const Bird& o) { return std::binary_search(s.begin(), s.end(), o.id); }),
                  bag.end());
        removed += before - bag.size();
    }
    if (!f->density_check) f->nagents -= removed;
    return removed;
}

int orc_flock_run(void* fp, const orc_params* pp, uint64_t first_step, uint32_t nsteps) {
    Field2D* f = (Field2D*)fp;
    FlockParams p = to_params(pp);
    for (uint32_t s = 0; s < nsteps; ++s)
        if (!flock_step(*f, p, first_step + s)) return -1;
    return 0;
}

// One step in FP64 force arithmetic for every agent of the read buffer, in
// read order; out[4*i..] = {x, y, dx, dy} for the i-th agent, ids[i] its id.
size_t orc_flock_step_fp64(void* fp, const orc_params* pp, uint64_t step, uint32_t* ids,
                           double* out, size_t cap) {
    Field2D* f = (Field2D*)fp;
    FlockParams p = to_params(pp);
    std::vector<Bird> agents, vec;
    read_order(*f, agents);
    for (size_t i = 0; i < agents.size() && i < cap; ++i) {
        ids[i] = agents[i].id;
        bird_step_fp64(*f, p, agents[i], step, vec, out + 4 * i);
    }
    return agents.size();
}

// Reference-equivalent timed run (simulate_old!, lib.rs:1473-1582): builds
// the field, inits n birds (Flocker::init order), then runs nsteps
// Schedule::steps through a binary-heap schedule.  Returns the seconds spent
// in the step loop (init excluded, lib.rs:1515-1526); the final read buffer
// is left in *out_field if non-NULL (caller frees).
double orc_simulate_timed_warm(float w, float h, float d, const orc_params* pp, size_t n,
                               const uint32_t* ids, const float* xy, const float* dxy,
                               uint32_t nwarm, uint32_t nsteps, void** out_field);
double orc_simulate_timed_threads_warm(float w, float h, float d, const orc_params* pp, size_t n,
                                       const uint32_t* ids, const float* xy, const float* dxy,
                                       uint32_t nwarm, uint32_t nsteps, uint32_t threads,
                                       void** out_field);

double orc_simulate_timed(float w, float h, float d, const orc_params* pp, size_t n,
                          const uint32_t* ids, const float* xy, const float* dxy,
                          uint32_t nsteps, void** out_field) {
    return orc_simulate_timed_warm(w, h, d, pp, n, ids, xy, dxy, 0, nsteps, out_field);
}

// The same after nwarm untimed steps (steps 0 .. nwarm-1): the seconds of
// steps nwarm .. nwarm+nsteps-1 alone.
double orc_simulate_timed_warm(float w, float h, float d, const orc_params* pp, size_t n,
                               const uint32_t* ids, const float* xy, const float* dxy,
                               uint32_t nwarm, uint32_t nsteps, void** out_field) {
    FlockParams p = to_params(pp);
    Field2D* f = new Field2D(w, h, d, true);
    typedef std::priority_queue<Event, std::vector<Event>, EventLess> PQ;
    PQ pq;
    uint64_t seq = 0;
    for (size_t i = 0; i < n; ++i) {  // state.rs:41-56
        Bird b{ids[i], xy[2 * i], xy[2 * i + 1], dxy[2 * i], dxy[2 * i + 1]};
        f->set_object_location(b, b.x, b.y);
        pq.push(Event{0.0f, 0, seq++, b});
    }
    auto t0 = std::chrono::steady_clock::now();
    std::vector<Event> cevents;
    std::vector<Bird> vec;
    for (uint32_t s = 0; s < nwarm + nsteps; ++s) {
        if (s == nwarm) t0 = std::chrono::steady_clock::now();
        if (s == 0) f->lazy_update();  // schedule.rs:349-351
        if (pq.empty()) break;
        float now = pq.top().time;
        cevents.clear();
        while (!pq.empty() && pq.top().time <= now) {
            cevents.push_back(pq.top());
            pq.pop();
        }
        for (Event& e : cevents) {
            Bird nb = bird_step(*f, p, e.bird, s, vec);
            f->set_object_location(nb, nb.x, nb.y);
            e.bird = nb;
            pq.push(Event{e.time + 1.0f, e.ordering, seq++, nb});
        }
        f->lazy_update();  // schedule.rs:410-412
    }
    auto t1 = std::chrono::steady_clock::now();
    if (out_field) *out_field = f;
    else delete f;
    return std::chrono::duration<double>(t1 - t0).count();
}

// The same run with the agent pass spread over `threads` host threads
// (not the reference: its sequential schedule runs one agent at a time, and
// its parallel build serialises agents on one mutex, schedule.rs:187).  Every
// agent reads the read buffer only, so the threads compute the next states
// of consecutive agent ranges into one array; the insertion into the write
// buffer stays sequential, in agent order, so the result equals the
// sequential run's bit for bit.  Agents run in read-buffer order (the
// oracle's parity order) rather than through the priority queue.
double orc_simulate_timed_threads(float w, float h, float d, const orc_params* pp, size_t n,
                                  const uint32_t* ids, const float* xy, const float* dxy,
                                  uint32_t nsteps, uint32_t threads, void** out_field) {
    return orc_simulate_timed_threads_warm(w, h, d, pp, n, ids, xy, dxy, 0, nsteps, threads, out_field);
}

double orc_simulate_timed_threads_warm(float w, float h, float d, const orc_params* pp, size_t n,
                                       const uint32_t* ids, const float* xy, const float* dxy,
                                       uint32_t nwarm, uint32_t nsteps, uint32_t threads,
                                       void** out_field) {
    FlockParams p = to_params(pp);
    Field2D* f = new Field2D(w, h, d, true);
    for (size_t i = 0; i < n; ++i) {
        Bird b{ids[i], xy[2 * i], xy[2 * i + 1], dxy[2 * i], dxy[2 * i + 1]};
        f->set_object_location(b, b.x, b.y);
    }
    if (threads == 0) threads = 1;
    auto t0 = std::chrono::steady_clock::now();
    f->lazy_update();
    std::vector<Bird> agents, next;
    for (uint32_t s = 0; s < nwarm + nsteps; ++s) {
        if (nwarm && s == nwarm) t0 = std::chrono::steady_clock::now();
        read_order(*f, agents);
        next.resize(agents.size());
        const size_t m = agents.size();
        const size_t chunk = (m + threads - 1) / threads;
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < threads; ++t) {
            const size_t lo = t * chunk, hi = std::min(m, lo + chunk);
            if (lo >= hi) break;
            pool.emplace_back([&, lo, hi]() {
                std::vector<Bird> vec;
                for (size_t k = lo; k < hi; ++k) next[k] = bird_step(*f, p, agents[k], s, vec);
            });
        }
        for (auto& th : pool) th.join();
        for (const Bird& nb : next) f->set_object_location(nb, nb.x, nb.y);
        f->lazy_update();
    }
    auto t1 = std::chrono::steady_clock::now();
    if (out_field) *out_field = f;
    else delete f;
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
