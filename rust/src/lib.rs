//! Rust binding of libribo_world.so, the GB300 world-step library.
//!
//! The reference's `World` (src/world/mod.rs) keeps its `params: SimParams`
//! and `settings: WorldSettings` and calls this crate for the GPU half of the
//! world step: buffer ownership (`World::new`, mod.rs:416), the fluid and
//! transport dispatches of `encode_steps` (mod.rs:1406) and the readbacks
//! (`ledger_blocking` mod.rs:1834, `read_cells_blocking` mod.rs:1807,
//! `read_f32_blocking` mod.rs:1802).  The declarations mirror
//! include/ribo_world.h field for field.
//!
//! `SimParams` (src/params.rs:86-487) is `#[repr(C)]` with 116 four-byte
//! fields, the layout of `ribo_sim_params`; the reference passes a pointer to
//! its own struct where these functions take `*mut RiboSimParams`.

use std::ffi::{CStr, CString};
use std::os::raw::{c_char, c_int, c_void};

/// `ribo_sim_params`: 116 four-byte words in `SimParams` order (464 bytes).
#[repr(C)]
#[derive(Clone, Copy)]
pub struct RiboSimParams {
    pub words: [u32; 116],
}
const _: () = assert!(std::mem::size_of::<RiboSimParams>() == 464);

#[repr(C)]
pub struct RiboWorld {
    _p: [u8; 0],
}
#[repr(C)]
pub struct RiboBatch {
    _p: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct RiboWorldCfg {
    pub grid_w: u32,
    pub grid_h: u32,
    pub fluid_w: u32,
    pub fluid_h: u32,
    pub world_units_per_cell: u32,
    pub mg_min_size: u32,
    pub mg_pre: u32,
    pub mg_post: u32,
    pub mg_coarse: u32,
    pub precision_mode: u32,
    pub device: u32,
    pub no_graphs: u32,
    /// CTAs per cluster of the small multigrid levels' V-cycle (0 automatic, 1 none, 8, 16).
    pub mg_cluster: u32,
    pub reserved: [u32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct RiboWorldSettings {
    pub fluid_enabled: u32,
    pub fluid_substep: u32,
    pub multigrid: u32,
    pub mg_cycles: u32,
    pub jacobi_iters: u32,
    pub ledger_each_step: u32,
    pub mg_unfused: u32,
    pub transport_simple: u32,
    pub mixed_tol: f32,
    pub mixed_inner_tol: f32,
    pub mixed_max_outer: u32,
    pub mixed_max_inner: u32,
    pub mixed_alpha: f32,
    pub light_mode: u32,
    pub light_rows_per_step: u32,
    pub light_interval: u32,
    pub terrain_mode: u32,
}
const _: () = assert!(std::mem::size_of::<RiboWorldSettings>() == 68);

/// Fields of `ribo_field` (sizes per include/ribo_world.h).
#[repr(i32)]
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum RiboField {
    Chem = 0,
    Gamma = 1,
    Light = 2,
    Slope = 3,
    Velocity = 4,
    Pressure = 5,
    Temp = 6,
    Redox = 7,
    Heat = 8,
    VelSmooth = 9,
    SolidMask = 10,
    Divergence = 11,
    ForceVectors = 12,
    RedoxEaten = 13,
    NetFlux = 14,
    Shade = 15,
    PressureLo = 16,
}

pub const RIBO_PRECISION_F32: u32 = 0;
pub const RIBO_PRECISION_MIXED: u32 = 1;

extern "C" {
    pub fn ribo_last_error() -> *const c_char;
    pub fn ribo_sim_params_default(out: *mut RiboSimParams);
    pub fn ribo_world_settings_default(out: *mut RiboWorldSettings);
    pub fn ribo_world_create(cfg: *const RiboWorldCfg, out: *mut *mut RiboWorld) -> c_int;
    pub fn ribo_world_destroy(w: *mut RiboWorld);
    pub fn ribo_world_footprint(cfg: *const RiboWorldCfg, bytes: *mut u64) -> c_int;
    pub fn ribo_world_memory(w: *const RiboWorld, bytes: *mut u64) -> c_int;
    pub fn ribo_world_set_settings(w: *mut RiboWorld, s: *const RiboWorldSettings) -> c_int;
    pub fn ribo_world_get_settings(w: *const RiboWorld, out: *mut RiboWorldSettings) -> c_int;
    pub fn ribo_world_upload(w: *mut RiboWorld, field: RiboField, host: *const c_void, bytes: usize) -> c_int;
    pub fn ribo_world_paint_terrain(w: *mut RiboWorld, cx: f32, cy: f32, radius: f32, grains: u32) -> c_int;
    pub fn ribo_world_read(w: *mut RiboWorld, field: RiboField, host: *mut c_void, bytes: usize) -> c_int;
    pub fn ribo_world_device_ptr(w: *mut RiboWorld, field: RiboField, dptr: *mut *mut c_void, bytes: *mut usize)
        -> c_int;
    pub fn ribo_world_step(w: *mut RiboWorld, per_step: *const RiboSimParams, n: u32) -> c_int;
    pub fn ribo_world_encode_steps(w: *mut RiboWorld, params: *mut RiboSimParams, steps: u32) -> c_int;
    pub fn ribo_world_ledger(w: *mut RiboWorld, out: *mut u32) -> c_int;
    pub fn ribo_world_request_ledger(w: *mut RiboWorld) -> c_int;
    pub fn ribo_world_poll_ledger(w: *mut RiboWorld, out: *mut u32, ready: *mut u32) -> c_int;
    pub fn ribo_world_sync(w: *mut RiboWorld) -> c_int;
    pub fn ribo_world_solve_info(w: *mut RiboWorld, outer: *mut u32, inner: *mut u32, rho: *mut f64) -> c_int;
    pub fn ribo_world_save_scene(w: *mut RiboWorld, path: *const c_char, params: *const RiboSimParams) -> c_int;
    pub fn ribo_world_load_scene(w: *mut RiboWorld, path: *const c_char, params: *mut RiboSimParams) -> c_int;
    pub fn ribo_batch_create(device: u32, out: *mut *mut RiboBatch) -> c_int;
    pub fn ribo_batch_destroy(b: *mut RiboBatch);
    pub fn ribo_batch_add(b: *mut RiboBatch, w: *mut RiboWorld) -> c_int;
    pub fn ribo_batch_remove(b: *mut RiboBatch, w: *mut RiboWorld) -> c_int;
    pub fn ribo_batch_encode_steps(b: *mut RiboBatch, params: *mut RiboSimParams, n: u32) -> c_int;
    pub fn ribo_batch_autotune(b: *mut RiboBatch, modes_out: *mut u32) -> c_int;
    pub fn ribo_batch_sync(b: *mut RiboBatch) -> c_int;
}

fn last_error() -> String {
    unsafe {
        let p = ribo_last_error();
        if p.is_null() {
            return String::from("unknown error");
        }
        CStr::from_ptr(p).to_string_lossy().into_owned()
    }
}

fn check(code: c_int, what: &str) -> Result<(), String> {
    if code == 0 {
        Ok(())
    } else {
        Err(format!("{what}: status {code}: {}", last_error()))
    }
}

/// The GPU half of one reference `World`: owns the device buffers of a world
/// and steps it on the GB300.
pub struct GpuWorld {
    h: *mut RiboWorld,
}

impl GpuWorld {
    /// `World::new(&gpu, cfg, seed)` (mod.rs:416): a `grid` x `grid` world
    /// with a `fluid` x `fluid` fluid grid.
    pub fn new(grid: u32, fluid: u32) -> Result<Self, String> {
        let cfg = RiboWorldCfg {
            grid_w: grid,
            grid_h: grid,
            fluid_w: fluid,
            fluid_h: fluid,
            world_units_per_cell: 30,
            ..Default::default()
        };
        Self::with_cfg(&cfg)
    }

    pub fn with_cfg(cfg: &RiboWorldCfg) -> Result<Self, String> {
        let mut h = std::ptr::null_mut();
        check(unsafe { ribo_world_create(cfg, &mut h) }, "ribo_world_create")?;
        Ok(GpuWorld { h })
    }

    pub fn set_settings(&mut self, s: &RiboWorldSettings) -> Result<(), String> {
        check(unsafe { ribo_world_set_settings(self.h, s) }, "ribo_world_set_settings")
    }

    /// Uploads of `seed_matter` (mod.rs:982-983), `upload_heat` and the
    /// frozen light / shade inputs: `bytes` must match the field's size.
    pub fn upload<T: Copy>(&mut self, field: RiboField, data: &[T]) -> Result<(), String> {
        let bytes = std::mem::size_of_val(data);
        check(unsafe { ribo_world_upload(self.h, field, data.as_ptr() as *const c_void, bytes) }, "ribo_world_upload")
    }

    /// `encode_steps(queue, enc, n)` (mod.rs:1406): `n` steps, advancing
    /// `params.epoch` as the reference does.
    pub fn encode_steps(&mut self, params: &mut RiboSimParams, n: u32) -> Result<(), String> {
        check(unsafe { ribo_world_encode_steps(self.h, params, n) }, "ribo_world_encode_steps")
    }

    /// `ledger_blocking` (mod.rs:1834): activated A U G C, spent A U G C, held A U G C.
    pub fn ledger_blocking(&mut self) -> Result<[u32; 12], String> {
        let mut out = [0u32; 12];
        check(unsafe { ribo_world_ledger(self.h, out.as_mut_ptr()) }, "ribo_world_ledger")?;
        Ok(out)
    }

    /// `read_cells_blocking` (mod.rs:1807) and `read_f32_blocking`
    /// (mod.rs:1802): `out` must have the field's size.
    pub fn read<T: Copy>(&mut self, field: RiboField, out: &mut [T]) -> Result<(), String> {
        let bytes = std::mem::size_of_val(out);
        check(unsafe { ribo_world_read(self.h, field, out.as_mut_ptr() as *mut c_void, bytes) }, "ribo_world_read")
    }

    pub fn sync(&mut self) -> Result<(), String> {
        check(unsafe { ribo_world_sync(self.h) }, "ribo_world_sync")
    }

    /// `save_scene` (src/world/snapshot.rs:274), world blocks.
    pub fn save_scene(&mut self, path: &str, params: &RiboSimParams) -> Result<(), String> {
        let p = CString::new(path).map_err(|e| e.to_string())?;
        check(unsafe { ribo_world_save_scene(self.h, p.as_ptr(), params) }, "ribo_world_save_scene")
    }

    /// `Scene::read` + `load_scene` (src/world/snapshot.rs:145,372), world blocks.
    pub fn load_scene(&mut self, path: &str, params: &mut RiboSimParams) -> Result<(), String> {
        let p = CString::new(path).map_err(|e| e.to_string())?;
        check(unsafe { ribo_world_load_scene(self.h, p.as_ptr(), params) }, "ribo_world_load_scene")
    }

    pub fn raw(&mut self) -> *mut RiboWorld {
        self.h
    }
}

impl Drop for GpuWorld {
    fn drop(&mut self) {
        unsafe { ribo_world_destroy(self.h) }
    }
}
