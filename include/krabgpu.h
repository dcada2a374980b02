/*
 * krabgpu.h -- C ABI of the GB300 continuous-space agent step.
 *
 * The drop-in boundary for krABMaga's Field2D + Flockers path.  Every entry
 * point below names the reference item it replaces (file:line within the
 * krABMaga 0.6.1 tree).  Conventions:
 *   - opaque handles; the library owns all device memory, host arrays are
 *     caller-owned and copied;
 *   - every call returns kb_status (KB_OK = 0); no exception, abort or panic
 *     crosses the ABI; kb_last_error() gives a message for the calling thread;
 *   - one handle per host thread (the reference Field2D is !Sync: RefCell);
 *     calls are ordered on the handle's own CUDA stream and the calls that
 *     return host data synchronise that stream;
 *   - positions are f32 (Real2D, src/engine/location.rs:17-22), ids u32
 *     (Bird::id, tests/model/flockers/bird.rs:21).
 */
#ifndef KRABGPU_H
#define KRABGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t kb_status;
#define KB_OK 0
#define KB_ERR_ARG 1         /* bad argument (null pointer, size, non-finite geometry) */
#define KB_ERR_OOM 2         /* device or pinned allocation failed */
#define KB_ERR_CUDA 3        /* a CUDA runtime call failed */
#define KB_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define KB_ERR_DEVICE_FLAG 5 /* a kernel raised its error word (see kb_field_device_flags) */
#define KB_ERR_STATE 6       /* call not valid in the handle's current state */
#define KB_ERR_RANGE 7       /* a location maps outside the bag matrix: the reference panics */
#define KB_ERR_NO_DEVICE 8   /* no CUDA device / the library cannot run here */
#define KB_ERR_BUSY 9        /* admission refused (serving budget or slot table full) */

/* Device error-word bits (kb_field_device_flags). */
#define KB_FLAG_KEY_RANGE 0x1u     /* a position discretised outside the bag matrix */
#define KB_FLAG_REBIN_MISS 0x2u    /* a boid moved more than one cell in one step */
#define KB_FLAG_SPIN_TIMEOUT 0x4u  /* a bounded spin-wait expired */
#define KB_FLAG_NONFINITE 0x8u     /* a non-finite position was produced */

/* Query kinds: which Field2D neighbour query the flock step uses. */
#define KB_QUERY_RELAX 0 /* get_neighbors_within_relax_distance, field_2d.rs:472-516 */
#define KB_QUERY_EXACT 1 /* get_neighbors_within_distance, field_2d.rs:386-440 (in-tree Bird) */

/* Candidate-list walk of the force pass (kb_field_set_dense_mode). */
#define KB_DENSE_AUTO 0 /* chosen from the bag occupancies (default) */
#define KB_DENSE_OFF 1  /* one flat list over the three column runs */
#define KB_DENSE_ON 2   /* each column run with a pointer; 8-bag rebin segments */

/* Arithmetic of the flock step. */
#define KB_ARITH_STRICT 0 /* IEEE f32 with the reference's rounding points: bit-exact */
#define KB_ARITH_FAST 1   /* approximate division/sqrt; within 1e-5 of domain vs FP64 */

typedef struct kb_field kb_field;

/* Field2D::new(w, h, d, toroidal), field_2d.rs:304-322. */
/* Cell range of the neighbour queries on a toroidal field.  CLAMP is the
 * reference (field_2d.rs:398-418, 484-500: the range is clamped to the bag
 * matrix, so a query does not see across the seam); TORUS wraps the range
 * (t_transform, field_2d.rs:926-932), so it does.  Non-toroidal fields
 * always wrap, as the reference does. */
#define KB_CELL_WRAP_CLAMP 0
#define KB_CELL_WRAP_TORUS 1

typedef struct {
    float width;
    float height;
    float discretization;
    int32_t toroidal;
    int32_t device;         /* CUDA ordinal */
    uint32_t capacity_hint; /* expected object count (storage grows as needed) */
    int32_t cell_wrap;      /* KB_CELL_WRAP_* (0: the reference's clamped range) */
} kb_field_desc;

/* The Flockers constants (bird.rs:12-17) and query radius (bird.rs:41) as a
 * parameter block; seed keys the Philox jitter stream that replaces
 * rand::rng() (bird.rs:113-117). */
typedef struct {
    float cohesion;
    float avoidance;
    float consistency;
    float randomness;
    float momentum;
    float jump;
    float neighbor_radius;
    int32_t query_mode; /* KB_QUERY_* */
    int32_t arith;      /* KB_ARITH_* */
    uint32_t _pad;
    uint64_t seed;
} kb_flock_params;

/* Message of the last failed call on this thread ("" if none). */
const char* kb_last_error(void);
/* Library version string. */
const char* kb_version(void);
/* Number of visible CUDA devices (0 if none); never fails. */
int32_t kb_device_count(void);

/* ------------------------------------------------------------------ Field2D */

/* Field2D::new -- field_2d.rs:304-322 */
kb_status kb_field_create(const kb_field_desc* desc, kb_field** out);
kb_status kb_field_destroy(kb_field* f);
/* dw, dh, max_x = ceil(w/d), max_y = ceil(h/d) -- field_2d.rs:316-317, 396-397 */
kb_status kb_field_dims(const kb_field* f, int32_t out4[4]);

/* set_object_location(object, loc) -- field_2d.rs:838-846.  The object is
 * {id, pos, last_d}; loc picks its bag.  Goes to the write buffer. */
kb_status kb_field_set_object_location(kb_field* f, uint32_t id, const float pos[2],
                                       const float last_d[2], const float loc[2]);
/* Bulk form: n objects, each placed at its own position (what Flocker::init,
 * state.rs:41-56, and Bird::step, bird.rs:151-153, do). xy and dxy are n*2. */
kb_status kb_field_set_locations(kb_field* f, size_t n, const uint32_t* ids, const float* xy,
                                 const float* dxy);
/* remove_object_location(object, loc) -- field_2d.rs:885-898 (write buffer). */
kb_status kb_field_remove_object_location(kb_field* f, uint32_t id, const float loc[2]);
/* Bulk removal by id (no single reference counterpart): every object of the
 * write buffer whose id is in ids[0..n) is removed, wherever its bag; for
 * each such object that is remove_object_location at its write location
 * (field_2d.rs:885-898).  An agent that leaves the schedule after
 * kb_flock_compute wrote it (Schedule::dequeue, schedule.rs:329-343, or
 * Agent::is_stopped, schedule.rs:401) is dropped this way: the reference
 * writes nothing for it.  *removed (may be NULL) = objects removed. */
kb_status kb_field_remove_ids(kb_field* f, size_t n, const uint32_t* ids, size_t* removed);
/* Lookups by object (the parallel build's Field2D::get / get_location,
 * field_2d.rs:165-170, 189-191, and get_unbuffered / get_location_unbuffered,
 * field_2d.rs:194-217): for each ids[q], found[q] = 1 and states[4q..4q+3] =
 * its {x, y, dx, dy} when an object with that id is in the read buffer
 * (buffered != 0) or the write buffer (buffered == 0); the first one in
 * stored order when several share the id; found[q] = 0 (None) otherwise. */
kb_status kb_field_get_locations(kb_field* f, int32_t buffered, size_t n, const uint32_t* ids,
                                 float* states, int32_t* found);
/* Field::lazy_update -- field_2d.rs:905-921: the write buffer becomes the
 * read buffer and a new empty write buffer starts. */
kb_status kb_field_lazy_update(kb_field* f);
/* *nagents (field_2d.rs:276, counted by set_object_location until the first
 * lazy_update). */
kb_status kb_field_num_agents(kb_field* f, size_t* out);
/* Objects in the read buffer. */
kb_status kb_field_num_objects(kb_field* f, size_t* out);

/* Neighbour queries against the read buffer.  ids (and, if non-NULL,
 * states = {x, y, dx, dy} per object) receive up to cap objects in the
 * reference's visiting order; *n receives the full count.
 * get_neighbors_within_relax_distance -- field_2d.rs:472-516 */
kb_status kb_field_get_neighbors_within_relax_distance(kb_field* f, const float loc[2], float dist,
                                                       uint32_t* ids, float* states, size_t cap,
                                                       size_t* n);
/* get_neighbors_within_distance -- field_2d.rs:386-440 */
kb_status kb_field_get_neighbors_within_distance(kb_field* f, const float loc[2], float dist,
                                                 uint32_t* ids, float* states, size_t cap,
                                                 size_t* n);
/* get_objects -- field_2d.rs:544-549 (read buffer bag at loc) */
kb_status kb_field_get_objects(kb_field* f, const float loc[2], uint32_t* ids, float* states,
                               size_t cap, size_t* n);
/* get_objects_unbuffered -- field_2d.rs:577-582 (write buffer bag at loc) */
kb_status kb_field_get_objects_unbuffered(kb_field* f, const float loc[2], uint32_t* ids,
                                          float* states, size_t cap, size_t* n);
/* num_objects_at_location -- field_2d.rs:803-808 */
kb_status kb_field_num_objects_at_location(kb_field* f, const float loc[2], size_t* n);
/* get_empty_bags -- field_2d.rs:727-739: (i*d, j*d) of every empty read bag,
 * i (x) outer. xy holds cap pairs. */
kb_status kb_field_get_empty_bags(kb_field* f, float* xy, size_t cap, size_t* n);
/* get_random_empty_bag -- field_2d.rs:764-772; the reference's unseeded rng
 * becomes Philox(seed).  *found = 0 when no bag is empty (None). */
kb_status kb_field_get_random_empty_bag(kb_field* f, uint64_t seed, float xy[2], int32_t* found);
/* iter_objects / iter_objects_unbuffered -- field_2d.rs:619-640 / 677-698:
 * every object with its bag's real position, bags i-outer, j-inner, each bag
 * in insertion order.  buffered = 1 for the read buffer, 0 for the write one.
 * cell_xy (2 per object), ids, states (4 per object) may be NULL. */
kb_status kb_field_iter_objects(kb_field* f, int32_t buffered, float* cell_xy, uint32_t* ids,
                                float* states, size_t cap, size_t* n);

/* --------------------------------------------------------------- Flockers */

/* One Schedule::step agent pass for the Flockers model (schedule.rs:395-408
 * running Bird::step, bird.rs:39-154, for every bird): reads the read
 * buffer, writes every bird's next state into the (empty) write buffer.
 * `step` keys the jitter stream. */
kb_status kb_flock_compute(kb_field* f, const kb_flock_params* p, uint64_t step);
/* Bird::step (bird.rs:39-154) for n agents that the caller holds rather
 * than the read buffer: agents that join the schedule at this step
 * (schedule_repeating / schedule_once at a later time, schedule.rs:283-303)
 * or skipped earlier steps.  Agent j = {ids[j], states[4j..4j+3] = x, y,
 * last_d.x, last_d.y} reads its neighbours from the read buffer, skips
 * candidates with its own id (bird.rs:50) and is written into the write
 * buffer after what is already there, in the given order (the order in
 * which the schedule pops them).  May follow kb_flock_compute for the same
 * step.  The next lazy_update takes the general rebuild. */
kb_status kb_flock_compute_agents(kb_field* f, const kb_flock_params* p, uint64_t step, size_t n,
                                  const uint32_t* ids, const float* states);
/* Device-resident record exchange (no reference counterpart: the halo and
 * migration messages of the MPI field, kdtree_mpi.rs:705-795, without a
 * host round trip).  Every pointer below is device memory on the field's
 * device; records are {x, y, last_d.x, last_d.y} as four floats.  The
 * caller's writes to input buffers must be complete before the call (e.g.
 * its stream synchronised); the calls return with their own device work
 * finished, so outputs can be read on any stream.
 *
 * kb_field_copy_read_buffer: the read buffer (bags ascending, insertion
 * order inside a bag) into states_dev[4*cap] / ids_dev[cap]; *n = its
 * length.  KB_ERR_ARG (with *n set) when cap < *n. */
kb_status kb_field_copy_read_buffer(kb_field* f, float* states_dev, uint32_t* ids_dev, size_t cap,
                                    size_t* n);
/* kb_field_set_locations for records in device memory: the n records are
 * appended to the write buffer in this order (set_object_location per
 * record, field_2d.rs:838-846).  KB_ERR_RANGE / KB_ERR_ARG as
 * kb_field_set_locations, with the write buffer left as it was. */
kb_status kb_field_set_states_device(kb_field* f, size_t n, const uint32_t* ids_dev,
                                     const float* states_dev);
/* Bird::step (bird.rs:39-154) of n agents held in device memory against the
 * read buffer, as kb_flock_compute_agents, but the next states go to
 * out_dev[4*n] (agent order) and nothing is added to the write buffer. */
kb_status kb_flock_next_states_device(kb_field* f, const kb_flock_params* p, uint64_t step,
                                      size_t n, const uint32_t* ids_dev, const float* states_dev,
                                      float* out_dev);
/* nsteps full steps: compute + lazy_update each (schedule.rs:395-412), with
 * step numbers first_step ... first_step+nsteps-1.  The read buffer must
 * hold the flock and the write buffer must be empty (call lazy_update after
 * initialisation, as Schedule::step does at step 0, schedule.rs:349-351). */
kb_status kb_flock_step(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                        uint32_t nsteps);
/* Step implementation options (no reference counterpart; tuning only).
 * mode (the `fused` argument): 0 (default) the separate force / scan / rebin
 * kernels (a plain field replays runs of 4 steps or more from CUDA graphs),
 * except that a call of 2 steps or more on a plain field of at most 4096
 * boids and 4096 bags runs whole steps in one 8-block thread-block cluster
 * (shared memory, up to 1000 steps per launch);
 * 3 the separate kernels whatever the field's size;
 * for eligible fields (toroidal, square, jump < discretization) 2 the tiled
 * step as two launches per step (stage + rebin + force per tile, then the
 * bag-offset scan) and 1 the same tiles in one persistent cooperative launch.
 * tile_tx x tile_ty bags per tile (0 = automatic).  All modes give the same
 * bits, in both arithmetic modes. */
kb_status kb_field_set_step_options(kb_field* f, int32_t fused, int32_t tile_tx, int32_t tile_ty);
/* Candidate-list walk of the separate-kernel step (no reference counterpart;
 * tuning only): KB_DENSE_AUTO (default) switches to KB_DENSE_ON when the read
 * buffer's estimated mean candidate count per boid (9 * sum of squared bag
 * occupancies / N) is at least 48, measured after each general rebuild and
 * every 64 steps without waiting.  ON walks each column run with a pointer
 * and rebins 8-bag segments (faster for dense flocks); OFF keeps one flat
 * list and 32-bag segments (faster for uniform ones).  Same bits either way.
 * *active (kb_field_dense_active) = the walk the next step uses. */
kb_status kb_field_set_dense_mode(kb_field* f, int32_t mode);
/* The path the next kb_flock_step takes: KB_PATH_* below. */
#define KB_PATH_SEPARATE 0 /* separate kernels, flat candidate list */
#define KB_PATH_FUSED 1    /* persistent fused tiles */
#define KB_PATH_TILED 2    /* split tile step */
#define KB_PATH_SMALL 3    /* whole steps in one cluster (calls of 2 steps or more) */
#define KB_PATH_DENSE 4    /* separate kernels, per-run walk (dense flocks) */
kb_status kb_field_step_path(kb_field* f, int32_t* path);
kb_status kb_field_dense_active(kb_field* f, int32_t* active);
/* Per-kernel timing (no reference counterpart; measurement only).  While
 * enabled, every separate-kernel step that is not replayed from a graph (a
 * kb_flock_step call of fewer than 4 steps) records CUDA events around its
 * launches on the field's stream (force | the offsets scan | rebin; the
 * one-block path of small fields records none).  kb_field_kernel_times waits
 * for them, returns the summed milliseconds of {force, scan, rebin} and the
 * number of steps timed, and starts a new tally. */
kb_status kb_field_set_kernel_timing(kb_field* f, int32_t enable);
kb_status kb_field_kernel_times(kb_field* f, double ms[3], uint64_t* steps);
/* Counters of the fused step: out4 = {tiles that ran through the global
 * scratch path (cumulative), tiles per step, CTAs, tx << 16 | ty}. */
kb_status kb_field_step_stats(kb_field* f, uint32_t out4[4]);
/* Tuning aid (no reference counterpart): enable = 1 makes the fused step
 * accumulate per-phase cycle counts; out16 (may be NULL) receives the sums
 * over CTAs of the 16 phase counters. */
kb_status kb_field_phase_clocks(kb_field* f, int32_t enable, unsigned long long* out16);
/* Tile-shape autotuner (no reference counterpart): runs steps_per_trial + 1
 * real steps (numbered from first_step) under each candidate shape
 * (candidates = ncand pairs tx, ty; NULL for the built-in list), keeps the
 * fastest; best = {tx, ty, steps consumed}, *ms_per_step its time. */
kb_status kb_field_autotune(kb_field* f, const kb_flock_params* p, uint64_t first_step,
                            uint32_t steps_per_trial, const int32_t* candidates, int32_t ncand,
                            int32_t best[3], float* ms_per_step);
/* Read buffer in its stored order (bags ascending, insertion order inside a
 * bag): ids and {x, y, dx, dy} states; either may be NULL. */
kb_status kb_field_get_state(kb_field* f, uint32_t* ids, float* states, size_t cap, size_t* n);
/* Error word raised by this handle's kernels since the last clear (KB_FLAG_*). */
kb_status kb_field_device_flags(kb_field* f, uint32_t* flags, int32_t clear);

/* No counterpart in the reference (it has no device waits; it panics on its
 * errors, src/engine/schedule.rs:374).  Every wait of this library's kernels
 * on another block (the look-back scan of large bag matrices, the grid
 * barrier and TMA waits of the tiled steps) is bounded: after spin_limit
 * iterations (0: each kernel's default) it gives up, raises
 * KB_FLAG_SPIN_TIMEOUT and the kernel returns; the results of that call are
 * invalid, and kb_field_synchronize reports KB_ERR_DEVICE_FLAG.  Clearing the
 * flag (kb_field_device_flags with clear) resets the kernels' control words
 * and empties the field's read buffer, which the failed call left invalid (a
 * batch's replicas are set anew with kb_batch_set_replica); the field is then
 * used again once its state is set anew.  withhold (KB_WITHHOLD_*) is the test
 * hook that makes a wait run out on purpose, without any fault: the
 * look-back scan tile, or the block of the persistent step, numbered `index`
 * does not publish its signal (KB_WITHHOLD_SCAN_PUBLISH also makes the bag
 * offsets of any size go through the look-back scan, which otherwise serves
 * the largest matrices only). */
#define KB_WITHHOLD_NONE 0
#define KB_WITHHOLD_SCAN_PUBLISH 1
#define KB_WITHHOLD_GRID_ARRIVAL 2
kb_status kb_field_set_wait_test(kb_field* f, uint32_t spin_limit, int32_t withhold, uint32_t index);
/* Wait for the handle's stream; returns KB_ERR_DEVICE_FLAG if a kernel
 * raised the error word. */
kb_status kb_field_synchronize(kb_field* f);
/* The same four moments for a plain field (kb_batch_moments). */
kb_status kb_field_moments(kb_field* f, double out4[4]);
/* The handle's CUDA stream (a cudaStream_t), for recording events or
 * ordering other work against the handle's kernels. */
kb_status kb_field_cuda_stream(kb_field* f, void** stream);

/* Parity support.  For nq query points (qxy, 2 per point) against the read
 * buffer: counts[q] = candidate count of the query kind (KB_QUERY_*), and if
 * ids != NULL the candidate ids packed in visiting order (cap entries max;
 * *total = sum of counts). */
kb_status kb_field_neighbor_lists(kb_field* f, int32_t kind, float dist, size_t nq,
                                  const float* qxy, uint32_t* counts, uint32_t* ids, size_t cap,
                                  size_t* total);
/* Per query point: candidate count and an order-independent 32-bit digest of
 * the candidate ids (sum of a 32-bit mix of each id). */
kb_status kb_field_neighbor_digest(kb_field* f, int32_t kind, float dist, size_t nq,
                                   const float* qxy, uint32_t* counts, uint32_t* digest);

/* No counterpart in the reference.  kb_field_neighbor_digest for hosts that
 * cannot allocate device memory when they query: one whose own pools hold the
 * rest of the device's memory, or one that must not stall other streams with
 * the device-wide synchronisation of cudaFree.  It makes no cudaMalloc,
 * cudaFree or other allocating call: query points, counts and digests are
 * staged in one fixed device array of KB_NOALLOC_MAX_QUERIES x 16 bytes
 * (1 MiB) per device, shared by every call on that device.  nq above
 * KB_NOALLOC_MAX_QUERIES returns KB_ERR_ARG.  Calls whose GPU work overlaps
 * (two host threads, fields on the same device) race on that array.  The
 * first call on a device sets the array up for that device
 * (cudaGetSymbolAddress); make it before any stream capture on the device.
 * The array's address is kept for the life of the process: a reset of the
 * device's primary context (cudaDeviceReset) invalidates it, as it
 * invalidates every field on that device. */
#define KB_NOALLOC_MAX_QUERIES 65536
kb_status kb_field_neighbor_digest_noalloc(kb_field* f, int32_t kind, float dist, size_t nq,
                                           const float* qxy, uint32_t* counts, uint32_t* digest);

/* No counterpart in the reference.  Device allocations and frees the library
 * has made so far in this process (all devices), for checking that a call
 * allocates nothing. */
kb_status kb_debug_allocation_counts(uint64_t* allocs, uint64_t* frees);

/* No counterpart in the reference.  Allocation-failure injection for testing
 * failure handling on the host: the next `count` device allocations the
 * library attempts fail as if the device were out of memory (no cudaMalloc
 * is made for them); 0 ends the injection.  Calls that need an allocation
 * then return KB_ERR_OOM, and the request server fails the requests of the
 * epoch that met it and carries on with the next ones. */
kb_status kb_debug_fail_allocations(uint32_t count);

/* ------------------------------------------------------ batched replicas */
/* Many independent Flockers simulations (the model-exploration workload of
 * explore_parallel!, src/explore/model_exploration.rs:354-432: one
 * simulate_explore! per configuration, lines 160-190) packed into one
 * device field, each replica with its own geometry and parameters, and
 * stepped together: by default the force, offsets and rebin kernels run once
 * per step over all replicas (one replica per block); the tiled step paths
 * (kb_batch_set_step_options) group steps into launches and graphs. */
typedef struct kb_batch kb_batch;
typedef struct {
    float width;
    float height;
    float discretization;
    int32_t toroidal;
    uint32_t nboids;   /* boids this replica holds */
    int32_t cell_wrap; /* KB_CELL_WRAP_* */
    kb_flock_params params; /* query_mode and arith must be equal across a batch */
} kb_replica_desc;

kb_status kb_batch_create(int32_t device, uint32_t nrep, const kb_replica_desc* reps,
                          kb_batch** out);
kb_status kb_batch_destroy(kb_batch* b);
/* Initial boids of replica r (n == its nboids; positions in its own frame);
 * the replica's Flocker::init (state.rs:41-56). */
kb_status kb_batch_set_replica(kb_batch* b, uint32_t r, size_t n, const uint32_t* ids,
                               const float* xy, const float* dxy);
/* Pack every replica into the read buffer (the step-0 lazy_update). */
kb_status kb_batch_commit(kb_batch* b);
/* nsteps steps of every replica.  The launch grouping applies to the tiled
 * step paths: steps_per_launch persistent steps per kernel launch (0 = all
 * in one) and graph_launches > 1 launches captured into one CUDA graph and
 * replayed; the default path ignores both (four launches per step). */
kb_status kb_batch_step(kb_batch* b, uint64_t first_step, uint32_t nsteps,
                        uint32_t steps_per_launch, uint32_t graph_launches);
/* Replica r's read buffer (ids, {x,y,dx,dy}) in its stored order. */
kb_status kb_batch_get_replica(kb_batch* b, uint32_t r, uint32_t* ids, float* states, size_t cap,
                               size_t* n);
/* Flock observables for model exploration (no reference counterpart: the
 * reference's explore! macros read user-defined output fields of the State,
 * model_exploration.rs:160-449).  out[4r..4r+3] = {boids, sum dx, sum dy,
 * sum |(dx, dy)|} of replica r's current headings (last_d), reduced on the
 * device in double: the polar order parameter is |(sum dx, sum dy)| / sum |d|,
 * the mean speed sum |d| / boids. */
kb_status kb_batch_moments(kb_batch* b, double* out);
/* Add a replica to a committed batch (no reference counterpart: the
 * reference's sweep runs each configuration as its own simulation,
 * model_exploration.rs:56-151).  The new replica gets the last index
 * (*index); its nboids objects (ids, xy, dxy as in kb_batch_set_replica) are
 * placed like set_object_location + lazy_update (field_2d.rs:905-921), and
 * its step numbering starts at origin_step: a later kb_batch_step with
 * first_step = origin_step + k advances it exactly like step k of a batch of
 * it alone.  The other replicas keep their records in their canonical order,
 * so their next steps are unchanged.  The objects are checked on the host
 * first: a non-finite value (KB_ERR_ARG) or a location outside the new
 * replica's bag matrix (KB_ERR_RANGE) leaves the batch as it was. */
kb_status kb_batch_add_replica(kb_batch* b, const kb_replica_desc* d, const uint32_t* ids,
                               const float* xy, const float* dxy, uint64_t origin_step,
                               uint32_t* index);
/* Remove replica r from a committed batch; replicas after r move down one
 * index.  A batch keeps at least one replica (KB_ERR_STATE). */
kb_status kb_batch_remove_replica(kb_batch* b, uint32_t r);
kb_status kb_batch_synchronize(kb_batch* b);
kb_status kb_batch_cuda_stream(kb_batch* b, void** stream);
kb_status kb_batch_set_step_options(kb_batch* b, int32_t fused, int32_t tile_tx, int32_t tile_ty);
kb_status kb_batch_step_stats(kb_batch* b, uint32_t out4[4]);
kb_status kb_batch_device_flags(kb_batch* b, uint32_t* flags, int32_t clear);
/* The tile-shape autotuner of kb_field_autotune for a batch. */
kb_status kb_batch_autotune(kb_batch* b, uint64_t first_step, uint32_t steps_per_trial,
                            const int32_t* candidates, int32_t ncand, int32_t best[3],
                            float* ms_per_step);

/* --------------------------------------------------------------- serving */
/* A continuous-batching request server (no reference counterpart: the
 * reference runs one simulate! per process).  Requests are whole Flockers
 * simulations; admitted ones share batched persistent launches and join or
 * leave between epochs of at most quantum_steps steps.  Admission needs a
 * free slot and the request's device state within hbm_budget_bytes. */
typedef struct kb_server kb_server;
typedef struct {
    int32_t device;
    uint32_t max_slots;         /* requests running at once */
    uint64_t hbm_budget_bytes;  /* device-state budget for running requests */
    uint32_t quantum_steps;     /* longest epoch between admissions (0 = 100) */
    uint32_t max_request_boids; /* largest request (sizes the device pool) */
    uint32_t max_request_cells; /* largest request bag matrix */
    int32_t query_mode;         /* shared by all requests */
    int32_t arith;
    uint32_t _pad;
} kb_server_desc;
typedef struct {
    uint32_t nboids;      /* ids 0..nboids-1, uniform flock from init_seed */
    float side;           /* square torus */
    float discretization;
    uint32_t steps;
    kb_flock_params params;
    uint64_t init_seed;
    float heading_scale;  /* as kb_gen_uniform */
    uint32_t _pad;
} kb_request;
typedef struct {
    uint64_t completed, failed, queued, running;
    double p50_s, p99_s, max_s; /* arrival -> result on the host */
    double boid_updates;        /* over completed epochs */
    double wall_s;              /* first arrival -> last completion */
    double busy_s;              /* time the loop spent in epochs */
    uint64_t launches, repacks, max_active;
} kb_server_report;

kb_status kb_server_create(const kb_server_desc* desc, kb_server** out);
/* Stops the loop (unfinished requests are dropped) and frees everything. */
kb_status kb_server_destroy(kb_server* s);
/* Thread-safe; the arrival time is taken here. */
kb_status kb_server_submit(kb_server* s, const kb_request* r, uint64_t* ticket);
/* *state: 0 queued, 1 running, 2 done, 3 failed; latency once done. */
kb_status kb_server_poll(kb_server* s, uint64_t ticket, int32_t* state, double* latency_s);
/* Final read buffer of a finished request (ids, {x,y,dx,dy}), stored order. */
kb_status kb_server_result(kb_server* s, uint64_t ticket, uint32_t* ids, float* states, size_t cap,
                           size_t* n);
/* Forget a finished request. */
kb_status kb_server_release(kb_server* s, uint64_t ticket);
kb_status kb_server_wait_idle(kb_server* s, double timeout_s);
kb_status kb_server_stats(kb_server* s, kb_server_report* out);

/* ------------------------------------------------------------ workloads */

/* Uniform flock: ids 0..n-1, pos = (w*u1, h*u2), heading a uniform unit
 * vector scaled by heading_scale (0 gives the reference's last_d = (0,0),
 * state.rs:47), all drawn from Philox(seed).  Host-only; needs no GPU. */
kb_status kb_gen_uniform(size_t n, float w, float h, uint64_t seed, float heading_scale,
                         uint32_t* ids, float* xy, float* dxy);
/* Clustered flock: nclusters isotropic Gaussian clusters (sigma) with
 * uniform centres on a w x h torus, positions wrapped; headings share the
 * cluster's angle plus N(0, angle_sigma) noise.  Host-only. */
kb_status kb_gen_clustered(size_t n, float w, float h, uint32_t nclusters, float sigma,
                           float angle_sigma, uint64_t seed, uint32_t* ids, float* xy, float* dxy);

#ifdef __cplusplus
}
#endif
#endif /* KRABGPU_H */
