// simulate! over the device Flocker: 1,048,576 boids at density 0.025 for
// 1000 steps, driven by the reference's own Schedule and macro.
use krabmaga::simulate;
use krabmaga_gpu::{flockers_params, GpuFlocker};

fn main() {
    let n: u32 = 1 << 20;
    let side = ((n as f64) / 0.025).sqrt() as f32;
    let state = GpuFlocker::new((side, side), n, 10.0 / 1.5, flockers_params(7, true, true), 7);
    simulate!(state, 1000, 1, false);
}
