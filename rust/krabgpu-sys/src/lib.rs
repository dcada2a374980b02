//! Raw bindings of `libkrabgpu.so` (the C ABI of `include/krabgpu.h`): the
//! GB300 continuous-space agent step behind krABMaga's `Field2D` /
//! `Schedule::step` / `simulate!` path.  Every struct is `#[repr(C)]` and laid
//! out field for field as in the header; every function returns a
//! `kb_status` (0 = `KB_OK`), with the message of the last failure on this
//! thread from `kb_last_error()`.  Safe wrappers live in the `krabmaga-gpu`
//! crate.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_void};

pub type kb_status = i32;
pub const KB_OK: kb_status = 0;
pub const KB_ERR_ARG: kb_status = 1;
pub const KB_ERR_OOM: kb_status = 2;
pub const KB_ERR_CUDA: kb_status = 3;
pub const KB_ERR_TIMEOUT: kb_status = 4;
pub const KB_ERR_DEVICE_FLAG: kb_status = 5;
pub const KB_ERR_STATE: kb_status = 6;
pub const KB_ERR_RANGE: kb_status = 7;
pub const KB_ERR_NO_DEVICE: kb_status = 8;
pub const KB_ERR_BUSY: kb_status = 9;

pub const KB_FLAG_KEY_RANGE: u32 = 0x1;
pub const KB_FLAG_REBIN_MISS: u32 = 0x2;
pub const KB_FLAG_SPIN_TIMEOUT: u32 = 0x4;
pub const KB_FLAG_NONFINITE: u32 = 0x8;

pub const KB_QUERY_RELAX: i32 = 0; // get_neighbors_within_relax_distance (field_2d.rs:472-516)
pub const KB_QUERY_EXACT: i32 = 1; // get_neighbors_within_distance (field_2d.rs:386-440)
pub const KB_DENSE_AUTO: i32 = 0;
pub const KB_DENSE_OFF: i32 = 1;
pub const KB_DENSE_ON: i32 = 2;
pub const KB_ARITH_STRICT: i32 = 0;
pub const KB_ARITH_FAST: i32 = 1;
pub const KB_CELL_WRAP_CLAMP: i32 = 0; // the reference's clamped query range
pub const KB_CELL_WRAP_TORUS: i32 = 1;
pub const KB_PATH_SEPARATE: i32 = 0;
pub const KB_PATH_FUSED: i32 = 1;
pub const KB_PATH_TILED: i32 = 2;
pub const KB_PATH_SMALL: i32 = 3;
pub const KB_PATH_DENSE: i32 = 4;
pub const KB_NOALLOC_MAX_QUERIES: usize = 65536;
pub const KB_WITHHOLD_NONE: i32 = 0;
pub const KB_WITHHOLD_SCAN_PUBLISH: i32 = 1;
pub const KB_WITHHOLD_GRID_ARRIVAL: i32 = 2;

#[repr(C)]
pub struct kb_field {
    _p: [u8; 0],
}
#[repr(C)]
pub struct kb_batch {
    _p: [u8; 0],
}
#[repr(C)]
pub struct kb_server {
    _p: [u8; 0],
}

/// Field2D::new(w, h, d, toroidal) (field_2d.rs:304-322) plus the device.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct kb_field_desc {
    pub width: f32,
    pub height: f32,
    pub discretization: f32,
    pub toroidal: i32,
    pub device: i32,
    pub capacity_hint: u32,
    pub cell_wrap: i32,
}

/// The Flockers constants (bird.rs:12-17), the query radius (bird.rs:41) and
/// the seed of the jitter stream that replaces rand::rng() (bird.rs:113-117).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct kb_flock_params {
    pub cohesion: f32,
    pub avoidance: f32,
    pub consistency: f32,
    pub randomness: f32,
    pub momentum: f32,
    pub jump: f32,
    pub neighbor_radius: f32,
    pub query_mode: i32,
    pub arith: i32,
    pub _pad: u32,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct kb_replica_desc {
    pub width: f32,
    pub height: f32,
    pub discretization: f32,
    pub toroidal: i32,
    pub nboids: u32,
    pub cell_wrap: i32,
    pub params: kb_flock_params,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct kb_server_desc {
    pub device: i32,
    pub max_slots: u32,
    pub hbm_budget_bytes: u64,
    pub quantum_steps: u32,
    pub max_request_boids: u32,
    pub max_request_cells: u32,
    pub query_mode: i32,
    pub arith: i32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct kb_request {
    pub nboids: u32,
    pub side: f32,
    pub discretization: f32,
    pub steps: u32,
    pub params: kb_flock_params,
    pub init_seed: u64,
    pub heading_scale: f32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct kb_server_report {
    pub completed: u64,
    pub failed: u64,
    pub queued: u64,
    pub running: u64,
    pub p50_s: f64,
    pub p99_s: f64,
    pub max_s: f64,
    pub boid_updates: f64,
    pub wall_s: f64,
    pub busy_s: f64,
    pub launches: u64,
    pub repacks: u64,
    pub max_active: u64,
}

extern "C" {
    pub fn kb_last_error() -> *const c_char;
    pub fn kb_version() -> *const c_char;
    pub fn kb_device_count() -> i32;

    // ---- Field2D (field_2d.rs:267-1014)
    pub fn kb_field_create(desc: *const kb_field_desc, out: *mut *mut kb_field) -> kb_status;
    pub fn kb_field_destroy(f: *mut kb_field) -> kb_status;
    // {dw, dh, max_x, max_y} (field_2d.rs:316-317, 396-397)
    pub fn kb_field_dims(f: *const kb_field, out4: *mut i32) -> kb_status;
    // set_object_location (field_2d.rs:838-846), one or many
    pub fn kb_field_set_object_location(f: *mut kb_field, id: u32, pos: *const f32,
                                        last_d: *const f32, loc: *const f32) -> kb_status;
    pub fn kb_field_set_locations(f: *mut kb_field, n: usize, ids: *const u32, xy: *const f32,
                                  dxy: *const f32) -> kb_status;
    // remove_object_location (field_2d.rs:885-898)
    pub fn kb_field_remove_object_location(f: *mut kb_field, id: u32, loc: *const f32) -> kb_status;
    pub fn kb_field_remove_ids(f: *mut kb_field, n: usize, ids: *const u32,
                               removed: *mut usize) -> kb_status;
    // get / get_location and the _unbuffered forms (parallel build, field_2d.rs:165-217):
    // found[q] = 0 is the reference's None
    pub fn kb_field_get_locations(f: *mut kb_field, buffered: i32, n: usize, ids: *const u32,
                                  states: *mut f32, found: *mut i32) -> kb_status;
    // lazy_update (field_2d.rs:905-921)
    pub fn kb_field_lazy_update(f: *mut kb_field) -> kb_status;
    pub fn kb_field_num_agents(f: *mut kb_field, out: *mut usize) -> kb_status;
    pub fn kb_field_num_objects(f: *mut kb_field, out: *mut usize) -> kb_status;
    // get_neighbors_within_relax_distance (field_2d.rs:472-516)
    pub fn kb_field_get_neighbors_within_relax_distance(
        f: *mut kb_field, loc: *const f32, dist: f32, ids: *mut u32, states: *mut f32,
        cap: usize, n: *mut usize) -> kb_status;
    // get_neighbors_within_distance (field_2d.rs:386-440)
    pub fn kb_field_get_neighbors_within_distance(
        f: *mut kb_field, loc: *const f32, dist: f32, ids: *mut u32, states: *mut f32,
        cap: usize, n: *mut usize) -> kb_status;
    pub fn kb_field_get_objects(f: *mut kb_field, loc: *const f32, ids: *mut u32,
                                states: *mut f32, cap: usize, n: *mut usize) -> kb_status;
    pub fn kb_field_get_objects_unbuffered(f: *mut kb_field, loc: *const f32, ids: *mut u32,
                                           states: *mut f32, cap: usize,
                                           n: *mut usize) -> kb_status;
    pub fn kb_field_num_objects_at_location(f: *mut kb_field, loc: *const f32,
                                            n: *mut usize) -> kb_status;
    pub fn kb_field_get_empty_bags(f: *mut kb_field, xy: *mut f32, cap: usize,
                                   n: *mut usize) -> kb_status;
    // get_random_empty_bag with a seed in place of the unseeded rng (field_2d.rs:764-772)
    pub fn kb_field_get_random_empty_bag(f: *mut kb_field, seed: u64, xy: *mut f32,
                                         found: *mut i32) -> kb_status;
    pub fn kb_field_iter_objects(f: *mut kb_field, buffered: i32, cell_xy: *mut f32,
                                 ids: *mut u32, states: *mut f32, cap: usize,
                                 n: *mut usize) -> kb_status;

    // ---- the Flockers step (bird.rs:39-154) driven by Schedule::step (schedule.rs:347-413)
    pub fn kb_flock_compute(f: *mut kb_field, p: *const kb_flock_params, step: u64) -> kb_status;
    pub fn kb_flock_compute_agents(f: *mut kb_field, p: *const kb_flock_params, step: u64,
                                   n: usize, ids: *const u32, states: *const f32) -> kb_status;

    // ---- device-resident record exchange (device pointers; no reference counterpart)
    pub fn kb_field_copy_read_buffer(f: *mut kb_field, states_dev: *mut f32, ids_dev: *mut u32,
                                     cap: usize, n: *mut usize) -> kb_status;
    pub fn kb_field_set_states_device(f: *mut kb_field, n: usize, ids_dev: *const u32,
                                      states_dev: *const f32) -> kb_status;
    pub fn kb_flock_next_states_device(f: *mut kb_field, p: *const kb_flock_params, step: u64,
                                       n: usize, ids_dev: *const u32, states_dev: *const f32,
                                       out_dev: *mut f32) -> kb_status;
    pub fn kb_flock_step(f: *mut kb_field, p: *const kb_flock_params, first_step: u64,
                         nsteps: u32) -> kb_status;

    // ---- step control and measurement (no reference counterpart)
    pub fn kb_field_set_step_options(f: *mut kb_field, fused: i32, tile_tx: i32,
                                     tile_ty: i32) -> kb_status;
    pub fn kb_field_set_dense_mode(f: *mut kb_field, mode: i32) -> kb_status;
    pub fn kb_field_step_path(f: *mut kb_field, path: *mut i32) -> kb_status;
    pub fn kb_field_dense_active(f: *mut kb_field, active: *mut i32) -> kb_status;
    pub fn kb_field_set_kernel_timing(f: *mut kb_field, enable: i32) -> kb_status;
    pub fn kb_field_kernel_times(f: *mut kb_field, ms: *mut f64, steps: *mut u64) -> kb_status;
    pub fn kb_field_step_stats(f: *mut kb_field, out4: *mut u32) -> kb_status;
    pub fn kb_field_phase_clocks(f: *mut kb_field, enable: i32, out16: *mut u64) -> kb_status;
    pub fn kb_field_autotune(f: *mut kb_field, p: *const kb_flock_params, first_step: u64,
                             steps_per_trial: u32, candidates: *const i32, ncand: i32,
                             best: *mut i32, ms_per_step: *mut f32) -> kb_status;
    pub fn kb_field_get_state(f: *mut kb_field, ids: *mut u32, states: *mut f32, cap: usize,
                              n: *mut usize) -> kb_status;
    pub fn kb_field_device_flags(f: *mut kb_field, flags: *mut u32, clear: i32) -> kb_status;
    // bounded device waits: iteration limit, and the test hook that withholds one signal
    pub fn kb_field_set_wait_test(f: *mut kb_field, spin_limit: u32, withhold: i32,
                                  index: u32) -> kb_status;
    pub fn kb_field_synchronize(f: *mut kb_field) -> kb_status;
    // heading moments {boids, sum dx, sum dy, sum |d|}, reduced on the device
    pub fn kb_field_moments(f: *mut kb_field, out4: *mut f64) -> kb_status;
    pub fn kb_field_cuda_stream(f: *mut kb_field, stream: *mut *mut c_void) -> kb_status;
    // many queries in one call: the id lists, or counts and an order-free digest
    pub fn kb_field_neighbor_lists(f: *mut kb_field, kind: i32, dist: f32, nq: usize,
                                   qxy: *const f32, counts: *mut u32, ids: *mut u32, cap: usize,
                                   total: *mut usize) -> kb_status;
    pub fn kb_field_neighbor_digest(f: *mut kb_field, kind: i32, dist: f32, nq: usize,
                                    qxy: *const f32, counts: *mut u32,
                                    digest: *mut u32) -> kb_status;
    // kb_field_neighbor_digest for hosts that cannot allocate device memory
    // while they query: one fixed staging array per device, at most
    // KB_NOALLOC_MAX_QUERIES points per call, overlapping calls race
    pub fn kb_field_neighbor_digest_noalloc(f: *mut kb_field, kind: i32, dist: f32, nq: usize,
                                            qxy: *const f32, counts: *mut u32,
                                            digest: *mut u32) -> kb_status;
    // device allocations and frees the library has made in this process
    pub fn kb_debug_allocation_counts(allocs: *mut u64, frees: *mut u64) -> kb_status;
    // allocation-failure injection: the next `count` device allocations fail
    pub fn kb_debug_fail_allocations(count: u32) -> kb_status;

    // ---- batched replicas: the runs of explore_parallel! (model_exploration.rs:354-432)
    pub fn kb_batch_create(device: i32, nrep: u32, reps: *const kb_replica_desc,
                           out: *mut *mut kb_batch) -> kb_status;
    pub fn kb_batch_destroy(b: *mut kb_batch) -> kb_status;
    pub fn kb_batch_set_replica(b: *mut kb_batch, r: u32, n: usize, ids: *const u32,
                                xy: *const f32, dxy: *const f32) -> kb_status;
    pub fn kb_batch_commit(b: *mut kb_batch) -> kb_status;
    pub fn kb_batch_step(b: *mut kb_batch, first_step: u64, nsteps: u32, steps_per_launch: u32,
                         graph_launches: u32) -> kb_status;
    pub fn kb_batch_get_replica(b: *mut kb_batch, r: u32, ids: *mut u32, states: *mut f32,
                                cap: usize, n: *mut usize) -> kb_status;
    pub fn kb_batch_moments(b: *mut kb_batch, out: *mut f64) -> kb_status;
    pub fn kb_batch_add_replica(b: *mut kb_batch, d: *const kb_replica_desc, ids: *const u32,
                                xy: *const f32, dxy: *const f32, origin_step: u64,
                                index: *mut u32) -> kb_status;
    pub fn kb_batch_remove_replica(b: *mut kb_batch, r: u32) -> kb_status;
    pub fn kb_batch_synchronize(b: *mut kb_batch) -> kb_status;
    pub fn kb_batch_cuda_stream(b: *mut kb_batch, stream: *mut *mut c_void) -> kb_status;
    pub fn kb_batch_set_step_options(b: *mut kb_batch, fused: i32, tile_tx: i32,
                                     tile_ty: i32) -> kb_status;
    pub fn kb_batch_step_stats(b: *mut kb_batch, out4: *mut u32) -> kb_status;
    pub fn kb_batch_device_flags(b: *mut kb_batch, flags: *mut u32, clear: i32) -> kb_status;
    pub fn kb_batch_autotune(b: *mut kb_batch, first_step: u64, steps_per_trial: u32,
                             candidates: *const i32, ncand: i32, best: *mut i32,
                             ms_per_step: *mut f32) -> kb_status;

    // ---- continuous-batching request server
    pub fn kb_server_create(desc: *const kb_server_desc, out: *mut *mut kb_server) -> kb_status;
    pub fn kb_server_destroy(s: *mut kb_server) -> kb_status;
    pub fn kb_server_submit(s: *mut kb_server, r: *const kb_request, ticket: *mut u64) -> kb_status;
    pub fn kb_server_poll(s: *mut kb_server, ticket: u64, state: *mut i32,
                          latency_s: *mut f64) -> kb_status;
    pub fn kb_server_result(s: *mut kb_server, ticket: u64, ids: *mut u32, states: *mut f32,
                            cap: usize, n: *mut usize) -> kb_status;
    pub fn kb_server_release(s: *mut kb_server, ticket: u64) -> kb_status;
    pub fn kb_server_wait_idle(s: *mut kb_server, timeout_s: f64) -> kb_status;
    pub fn kb_server_stats(s: *mut kb_server, out: *mut kb_server_report) -> kb_status;

    // ---- seeded synthetic flocks (uniform; Gaussian clusters)
    pub fn kb_gen_uniform(n: usize, w: f32, h: f32, seed: u64, heading_scale: f32,
                          ids: *mut u32, xy: *mut f32, dxy: *mut f32) -> kb_status;
    pub fn kb_gen_clustered(n: usize, w: f32, h: f32, nclusters: u32, sigma: f32,
                            angle_sigma: f32, seed: u64, ids: *mut u32, xy: *mut f32,
                            dxy: *mut f32) -> kb_status;
}

/// The library's message for the last failure on this thread.
pub fn last_error() -> String {
    unsafe {
        let p = kb_last_error();
        if p.is_null() {
            return String::new();
        }
        std::ffi::CStr::from_ptr(p).to_string_lossy().into_owned()
    }
}

/// Panics with the library's message, as the reference's Field2D panics on misuse.
pub fn check(st: kb_status) {
    if st != KB_OK {
        panic!("libkrabgpu: {} ({})", last_error(), st);
    }
}
