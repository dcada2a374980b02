//! krABMaga's Field2D + Flockers step on a GB300, as a drop-in for the
//! reference's own types.
//!
//! * `GpuField2D` keeps the method names and argument meaning of
//!   `engine::fields::field_2d::Field2D` (src/engine/fields/field_2d.rs) for
//!   the Flockers' `Bird` records: `set_object_location`, `lazy_update`,
//!   `get_neighbors_within_relax_distance`, `get_neighbors_within_distance`,
//!   `get_objects`, `num_objects_at_location`, `get_empty_bags`,
//!   `iter_objects`, `remove_object_location`, `get_location`.  It implements
//!   the reference's `Field` trait (src/engine/fields/field.rs:4-9).
//! * `GpuFlocker` implements `State` (src/engine/state.rs:45-63) like the
//!   in-tree `Flocker` (tests/model/flockers/state.rs:11-60), but runs each
//!   whole step (every `Bird::step`, tests/model/flockers/bird.rs:39-154, plus
//!   the field's `lazy_update`) as one `kb_flock_step` from its `update`, so
//!   `Schedule::step` (src/engine/schedule.rs:347-413) and `simulate!`
//!   (src/lib.rs:1158-1175) drive it unchanged.  The schedule holds no
//!   per-bird agents: the step is specialised to the Flockers model.
//!
//! Errors: the reference panics on misuse (`expect`, out-of-range bags); so
//! do these wrappers, with the library's message.  Lookups return `Option`
//! as the reference's do.
use krabgpu_sys as sys;
use krabmaga::engine::fields::field::Field;
use krabmaga::engine::location::Real2D;
use krabmaga::engine::schedule::Schedule;
use krabmaga::engine::state::State;
use std::any::Any;

/// One Flockers bird as the field stores it: id, position and last heading
/// (tests/model/flockers/bird.rs:20-25).
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct GpuBird {
    pub id: u32,
    pub pos: Real2D,
    pub last_d: Real2D,
}

/// Field2D on the device.  One handle per thread, as the reference's
/// Field2D is not Sync.
pub struct GpuField2D {
    raw: *mut sys::kb_field,
    pub width: f32,
    pub height: f32,
    pub discretization: f32,
    pub toroidal: bool,
}

unsafe impl Send for GpuField2D {}

fn loc2(p: Real2D) -> [f32; 2] {
    [p.x, p.y]
}

impl GpuField2D {
    /// Field2D::new (field_2d.rs:304-322) on CUDA device `device`.
    pub fn new(width: f32, height: f32, discretization: f32, toroidal: bool) -> Self {
        Self::on_device(width, height, discretization, toroidal, 0, 0)
    }

    pub fn on_device(width: f32, height: f32, discretization: f32, toroidal: bool, device: i32,
                     capacity_hint: u32) -> Self {
        let desc = sys::kb_field_desc {
            width,
            height,
            discretization,
            toroidal: toroidal as i32,
            device,
            capacity_hint,
            cell_wrap: sys::KB_CELL_WRAP_CLAMP,
        };
        let mut raw = std::ptr::null_mut();
        sys::check(unsafe { sys::kb_field_create(&desc, &mut raw) });
        GpuField2D { raw, width, height, discretization, toroidal }
    }

    pub fn raw(&self) -> *mut sys::kb_field {
        self.raw
    }

    /// set_object_location (field_2d.rs:838-846): into the write buffer.
    pub fn set_object_location(&self, bird: GpuBird, loc: Real2D) {
        let pos = loc2(bird.pos);
        let last = loc2(bird.last_d);
        let at = loc2(loc);
        sys::check(unsafe {
            sys::kb_field_set_object_location(self.raw, bird.id, pos.as_ptr(), last.as_ptr(),
                                              at.as_ptr())
        });
    }

    /// Many birds at their own positions in one copy.
    pub fn set_locations(&self, ids: &[u32], xy: &[f32], dxy: &[f32]) {
        assert!(xy.len() == 2 * ids.len() && dxy.len() == 2 * ids.len());
        sys::check(unsafe {
            sys::kb_field_set_locations(self.raw, ids.len(), ids.as_ptr(), xy.as_ptr(),
                                        dxy.as_ptr())
        });
    }

    /// remove_object_location (field_2d.rs:885-898): from the write buffer.
    pub fn remove_object_location(&self, bird: GpuBird, loc: Real2D) {
        let at = loc2(loc);
        sys::check(unsafe { sys::kb_field_remove_object_location(self.raw, bird.id, at.as_ptr()) });
    }

    fn list(&self, f: unsafe extern "C" fn(*mut sys::kb_field, *const f32, f32, *mut u32,
                                           *mut f32, usize, *mut usize) -> sys::kb_status,
            loc: Real2D, dist: f32) -> Vec<GpuBird> {
        let at = loc2(loc);
        let mut n = 0usize;
        sys::check(unsafe {
            f(self.raw, at.as_ptr(), dist, std::ptr::null_mut(), std::ptr::null_mut(), 0, &mut n)
        });
        let mut ids = vec![0u32; n];
        let mut st = vec![0f32; 4 * n];
        let mut got = 0usize;
        sys::check(unsafe { f(self.raw, at.as_ptr(), dist, ids.as_mut_ptr(), st.as_mut_ptr(), n, &mut got) });
        birds(&ids[..got.min(n)], &st)
    }

    /// get_neighbors_within_relax_distance (field_2d.rs:472-516).
    pub fn get_neighbors_within_relax_distance(&self, loc: Real2D, dist: f32) -> Vec<GpuBird> {
        self.list(sys::kb_field_get_neighbors_within_relax_distance, loc, dist)
    }

    /// get_neighbors_within_distance (field_2d.rs:386-440).
    pub fn get_neighbors_within_distance(&self, loc: Real2D, dist: f32) -> Vec<GpuBird> {
        self.list(sys::kb_field_get_neighbors_within_distance, loc, dist)
    }

    fn bag(&self, f: unsafe extern "C" fn(*mut sys::kb_field, *const f32, *mut u32, *mut f32,
                                          usize, *mut usize) -> sys::kb_status,
           loc: Real2D) -> Vec<GpuBird> {
        let at = loc2(loc);
        let mut n = 0usize;
        sys::check(unsafe {
            f(self.raw, at.as_ptr(), std::ptr::null_mut(), std::ptr::null_mut(), 0, &mut n)
        });
        let mut ids = vec![0u32; n];
        let mut st = vec![0f32; 4 * n];
        let mut got = 0usize;
        sys::check(unsafe { f(self.raw, at.as_ptr(), ids.as_mut_ptr(), st.as_mut_ptr(), n, &mut got) });
        birds(&ids[..got.min(n)], &st)
    }

    /// get_objects (field_2d.rs:544-558): the read buffer's bag at `loc`.
    pub fn get_objects(&self, loc: Real2D) -> Vec<GpuBird> {
        self.bag(sys::kb_field_get_objects, loc)
    }

    /// get_objects_unbuffered (field_2d.rs:577-582): the write buffer's bag.
    pub fn get_objects_unbuffered(&self, loc: Real2D) -> Vec<GpuBird> {
        self.bag(sys::kb_field_get_objects_unbuffered, loc)
    }

    /// num_objects_at_location (field_2d.rs:803-810).
    pub fn num_objects_at_location(&self, loc: Real2D) -> usize {
        let at = loc2(loc);
        let mut n = 0usize;
        sys::check(unsafe { sys::kb_field_num_objects_at_location(self.raw, at.as_ptr(), &mut n) });
        n
    }

    /// get_empty_bags (field_2d.rs:727-739): the corners (i*d, j*d) of the
    /// read buffer's empty bags, in bag order.
    pub fn get_empty_bags(&self) -> Vec<Real2D> {
        let mut n = 0usize;
        sys::check(unsafe { sys::kb_field_get_empty_bags(self.raw, std::ptr::null_mut(), 0, &mut n) });
        let mut xy = vec![0f32; 2 * n];
        let mut got = 0usize;
        sys::check(unsafe { sys::kb_field_get_empty_bags(self.raw, xy.as_mut_ptr(), n, &mut got) });
        xy.chunks(2).take(got).map(|c| Real2D { x: c[0], y: c[1] }).collect()
    }

    /// iter_objects / iter_objects_unbuffered (field_2d.rs:619-640): every
    /// stored bird with its bag corner, in the buffer's order.
    pub fn iter_objects(&self, buffered: bool) -> Vec<(Real2D, GpuBird)> {
        let mut n = 0usize;
        sys::check(unsafe {
            sys::kb_field_iter_objects(self.raw, buffered as i32, std::ptr::null_mut(),
                                       std::ptr::null_mut(), std::ptr::null_mut(), 0, &mut n)
        });
        let (mut cells, mut ids, mut st) = (vec![0f32; 2 * n], vec![0u32; n], vec![0f32; 4 * n]);
        let mut got = 0usize;
        sys::check(unsafe {
            sys::kb_field_iter_objects(self.raw, buffered as i32, cells.as_mut_ptr(), ids.as_mut_ptr(),
                                       st.as_mut_ptr(), n, &mut got)
        });
        let b = birds(&ids[..got.min(n)], &st);
        cells.chunks(2).zip(b).map(|(c, bird)| (Real2D { x: c[0], y: c[1] }, bird)).collect()
    }

    /// get_location (parallel build, field_2d.rs:189-199): None when absent.
    pub fn get_location(&self, bird: GpuBird) -> Option<Real2D> {
        let mut st = [0f32; 4];
        let mut found = 0i32;
        sys::check(unsafe {
            sys::kb_field_get_locations(self.raw, 1, 1, &bird.id, st.as_mut_ptr(), &mut found)
        });
        if found != 0 { Some(Real2D { x: st[0], y: st[1] }) } else { None }
    }

    /// The agents counted by set_object_location until the first lazy_update
    /// (field_2d.rs:276, 843-845).
    pub fn nagents(&self) -> usize {
        let mut n = 0usize;
        sys::check(unsafe { sys::kb_field_num_agents(self.raw, &mut n) });
        n
    }

    /// Every stored bird of the read buffer in bag order.
    pub fn state(&self) -> (Vec<u32>, Vec<f32>) {
        let mut n = 0usize;
        sys::check(unsafe { sys::kb_field_num_objects(self.raw, &mut n) });
        let (mut ids, mut st) = (vec![0u32; n], vec![0f32; 4 * n]);
        let mut got = 0usize;
        sys::check(unsafe { sys::kb_field_get_state(self.raw, ids.as_mut_ptr(), st.as_mut_ptr(), n, &mut got) });
        ids.truncate(got);
        st.truncate(4 * got);
        (ids, st)
    }
}

fn birds(ids: &[u32], st: &[f32]) -> Vec<GpuBird> {
    ids.iter()
        .enumerate()
        .map(|(k, &id)| GpuBird {
            id,
            pos: Real2D { x: st[4 * k], y: st[4 * k + 1] },
            last_d: Real2D { x: st[4 * k + 2], y: st[4 * k + 3] },
        })
        .collect()
}

impl Field for GpuField2D {
    /// field.rs:4-9: swap the buffers (field_2d.rs:905-921).
    fn lazy_update(&mut self) {
        sys::check(unsafe { sys::kb_field_lazy_update(self.raw) });
    }
    fn update(&mut self) {
        self.lazy_update();
    }
}

impl Drop for GpuField2D {
    fn drop(&mut self) {
        if !self.raw.is_null() {
            unsafe { sys::kb_field_destroy(self.raw) };
        }
    }
}

/// The Flockers model's constants (bird.rs:12-17) and the query radius of
/// the step (bird.rs:41) as the device parameter block; `seed` keys the
/// jitter stream that replaces the unseeded rand::rng() (bird.rs:113-117).
pub fn flockers_params(seed: u64, relaxed: bool, fast: bool) -> sys::kb_flock_params {
    sys::kb_flock_params {
        cohesion: 1.0,
        avoidance: 1.0,
        consistency: 1.0,
        randomness: 1.0,
        momentum: 1.0,
        jump: 0.7,
        neighbor_radius: 10.0,
        query_mode: if relaxed { sys::KB_QUERY_RELAX } else { sys::KB_QUERY_EXACT },
        arith: if fast { sys::KB_ARITH_FAST } else { sys::KB_ARITH_STRICT },
        _pad: 0,
        seed,
    }
}

/// tests/model/flockers/state.rs:11-60 with the whole step on the device.
pub struct GpuFlocker {
    pub step: u64,
    pub field1: GpuField2D,
    pub initial_flockers: u32,
    pub dim: (f32, f32),
    pub discretization: f32,
    pub params: sys::kb_flock_params,
    pub init_seed: u64,
}

impl GpuFlocker {
    pub fn new(dim: (f32, f32), initial_flockers: u32, discretization: f32,
               params: sys::kb_flock_params, init_seed: u64) -> Self {
        GpuFlocker {
            step: 0,
            field1: GpuField2D::on_device(dim.0, dim.1, discretization, true, 0, initial_flockers),
            initial_flockers,
            dim,
            discretization,
            params,
            init_seed,
        }
    }
}

impl State for GpuFlocker {
    fn reset(&mut self) {
        self.step = 0;
        self.field1 = GpuField2D::on_device(self.dim.0, self.dim.1, self.discretization, true, 0,
                                            self.initial_flockers);
    }

    /// state.rs:41-56: every bird at dim * U[0,1)^2 with last_d = 0, set into
    /// the field; the positions come from the library's seeded generator.
    fn init(&mut self, _schedule: &mut Schedule) {
        let n = self.initial_flockers as usize;
        let (mut ids, mut xy, mut dxy) = (vec![0u32; n], vec![0f32; 2 * n], vec![0f32; 2 * n]);
        sys::check(unsafe {
            sys::kb_gen_uniform(n, self.dim.0, self.dim.1, self.init_seed, 0.0, ids.as_mut_ptr(),
                                xy.as_mut_ptr(), dxy.as_mut_ptr())
        });
        self.field1.set_locations(&ids, &xy, &dxy);
    }

    /// The schedule calls update(0) once before the first step and update(k)
    /// after step k (schedule.rs:349-351, 410-412): update(0) is the initial
    /// lazy_update, every later call runs one whole step on the device.
    fn update(&mut self, step: u64) {
        if step == 0 {
            self.field1.lazy_update();
        } else {
            sys::check(unsafe { sys::kb_flock_step(self.field1.raw(), &self.params, self.step, 1) });
            self.step += 1;
        }
    }

    fn as_any_mut(&mut self) -> &mut dyn Any {
        self
    }
    fn as_any(&self) -> &dyn Any {
        self
    }
    fn as_state_mut(&mut self) -> &mut dyn State {
        self
    }
    fn as_state(&self) -> &dyn State {
        self
    }
}
