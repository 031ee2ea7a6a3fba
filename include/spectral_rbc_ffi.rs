// Rust declaration of the C ABI of libspectral_rbc (generated from spectral_rbc.h by
// gen_rust_ffi.py; regenerate, do not edit).  rustpde adds it as src/gpu/ffi.rs.
#![allow(non_camel_case_types, dead_code)]
use std::os::raw::{c_char, c_double, c_int, c_long, c_longlong, c_uint, c_void};

pub const RBC_OK: c_int = 0;
pub const RBC_ERR_INVALID: c_int = -1;
pub const RBC_ERR_CUDA: c_int = -2;
pub const RBC_ERR_NUMERIC: c_int = -3;
pub const RBC_ERR_UNSUPPORTED: c_int = -4;
pub const RBC_ERR_NOMEM: c_int = -5;
pub const RBC_ERR_CANCELLED: c_int = -6;
pub const RBC_BOX_ADIABATIC: c_int = 0;
pub const RBC_BOX_CONDUCTING: c_int = 1;
pub const RBC_PERIODIC: c_int = 2;
pub const RBC_PREC_FP64: c_int = 0;
pub const RBC_PREC_MIXED: c_int = 1;
pub const RBC_TEMP: c_int = 0;
pub const RBC_UX: c_int = 1;
pub const RBC_UY: c_int = 2;
pub const RBC_PRES: c_int = 3;
pub const RBC_PSEUDO_PRES: c_int = 4;
pub const RBC_FIELDBC: c_int = 5;
pub const RBC_NU: c_int = 0;
pub const RBC_NUVOL: c_int = 1;
pub const RBC_RE: c_int = 2;
pub const RBC_KE: c_int = 3;
pub const RBC_DIV_NORM: c_int = 4;
pub const FS_CHEBYSHEV: c_int = 0;
pub const FS_CHEB_DIRICHLET: c_int = 1;
pub const FS_CHEB_NEUMANN: c_int = 2;
pub const FS_CHEB_DIRICHLET_BC: c_int = 3;
pub const FS_CHEB_NEUMANN_BC: c_int = 4;
pub const FS_FOURIER_R2C: c_int = 5;
pub const FS_PHYSICAL: c_int = 0;
pub const FS_SPECTRAL: c_int = 1;
pub const FS_ORTHO: c_int = 2;
pub const FS_NOALLOC_SCRATCH_BYTES: usize = 4*1024*1024;
pub const FS_OP_FORWARD: c_int = 0;
pub const FS_OP_BACKWARD: c_int = 1;
pub const FS_OP_TO_ORTHO: c_int = 2;
pub const FS_OP_FROM_ORTHO: c_int = 3;
pub const FS_OP_HHOLTZ: c_int = 4;
pub const SV_HHOLTZ: c_int = 0;
pub const SV_HHOLTZ_ADI: c_int = 1;
pub const SV_POISSON: c_int = 2;
pub const RBC_ADJ_TEMP_RES: c_int = 10;
pub const RBC_ADJ_UX_RES: c_int = 11;
pub const RBC_ADJ_UY_RES: c_int = 12;

#[repr(C)] pub struct RbcCase { _p: [u8; 0] }
#[repr(C)] pub struct RbcBatch { _p: [u8; 0] }
#[repr(C)] pub struct RbcServer { _p: [u8; 0] }
#[repr(C)] pub struct FsSpace { _p: [u8; 0] }
#[repr(C)] pub struct FsLanes { _p: [u8; 0] }
#[repr(C)] pub struct SvSolver { _p: [u8; 0] }
#[repr(C)] pub struct RbcAdjoint { _p: [u8; 0] }
#[repr(C)] pub struct DfCase { _p: [u8; 0] }
#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct RbcParams {
    pub nx: c_int,
    pub ny: c_int,
    pub ra: c_double,
    pub pr: c_double,
    pub dt: c_double,
    pub aspect: c_double,
    pub kind: c_int,
    pub precision: c_int,
}
#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct RbcServerConfig {
    pub hbm_budget_bytes: usize,
    pub max_active: c_int,
    pub chunk_steps: c_int,
    pub setup_threads: c_int,
}
#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct RbcRequestResult {
    pub id: c_longlong,
    pub status: c_int,
    pub steps: c_int,
    pub sim_time: c_double,
    pub t_submit: c_double,
    pub t_admit: c_double,
    pub t_done: c_double,
    pub nu: c_double,
    pub ke: c_double,
    pub grid_points: c_longlong,
}
#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct RbcServerStats {
    pub now: c_double,
    pub pending: c_int,
    pub active: c_int,
    pub completed: c_longlong,
    pub bytes_in_use: usize,
    pub grid_point_steps: c_double,
    pub steps_launched: c_longlong,
    pub rebuilds: c_longlong,
    pub peak_bytes_in_use: usize,
}
pub type RbcCallback = unsafe extern "C" fn(c: *mut RbcCase, time: c_double, user: *mut c_void) -> c_int;

#[link(name = "spectral_rbc")]
extern "C" {
    pub fn rbc_last_error() -> *const c_char;
    pub fn rbc_version() -> *const c_char;
    pub fn rbc_create(params: *const RbcParams, out: *mut *mut RbcCase) -> c_int;
    pub fn rbc_destroy(c: *mut RbcCase) -> c_int;
    pub fn rbc_get_params(c: *const RbcCase, out: *mut c_double) -> c_int;
    pub fn rbc_set_velocity(c: *mut RbcCase, amp: c_double, m: c_double, n: c_double) -> c_int;
    pub fn rbc_set_temperature(c: *mut RbcCase, amp: c_double, m: c_double, n: c_double) -> c_int;
    pub fn rbc_random_disturbance(c: *mut RbcCase, amp: c_double, seed: u64) -> c_int;
    pub fn rbc_set_temperature_noise(c: *mut RbcCase, amp: c_double, seed: u64) -> c_int;
    pub fn rbc_set_solid(c: *mut RbcCase, mask: *const c_double, value: *const c_double, n_doubles: usize) -> c_int;
    pub fn rbc_get_solid(c: *const RbcCase, present: *mut c_int, mask: *mut c_double, value: *mut c_double, n_doubles: usize) -> c_int;
    pub fn rbc_solid_cylinder_inner(x: *const c_double, nx: c_int, y: *const c_double, ny: c_int, x0: c_double, y0: c_double, radius: c_double, mask: *mut c_double, value: *mut c_double) -> c_int;
    pub fn rbc_solid_roughness_sinusoid(x: *const c_double, nx: c_int, y: *const c_double, ny: c_int, height: c_double, wavenumber: c_double, mask: *mut c_double, value: *mut c_double) -> c_int;
    pub fn rbc_solid_porosity(x: *const c_double, nx: c_int, y: *const c_double, ny: c_int, diameter: c_double, porosity: c_double, mask: *mut c_double, value: *mut c_double) -> c_int;
    pub fn rbc_solid_porosity_interpolate(nx: c_int, ny: c_int, diameter: c_double, porosity: c_double, mask: *mut c_double, value: *mut c_double) -> c_int;
    pub fn rbc_step(c: *mut RbcCase, nsteps: c_int) -> c_int;
    pub fn rbc_synchronize(c: *mut RbcCase) -> c_int;
    pub fn rbc_get_time(c: *const RbcCase, t: *mut c_double) -> c_int;
    pub fn rbc_set_time(c: *mut RbcCase, t: c_double) -> c_int;
    pub fn rbc_get_dt(c: *const RbcCase, dt: *mut c_double) -> c_int;
    pub fn rbc_status(c: *mut RbcCase, status: *mut c_int) -> c_int;
    pub fn rbc_exit(c: *mut RbcCase, stop: *mut c_int) -> c_int;
    pub fn rbc_integrate(c: *mut RbcCase, max_time: c_double, save_intervall: c_double, cb: Option<RbcCallback>, user: *mut c_void, steps_done: *mut c_long) -> c_int;
    pub fn rbc_field_shape(c: *const RbcCase, field: c_int, n0: *mut c_int, n1: *mut c_int, is_complex: *mut c_int) -> c_int;
    pub fn rbc_get_state(c: *mut RbcCase, field: c_int, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn rbc_set_state(c: *mut RbcCase, field: c_int, host: *const c_double, n_doubles: usize) -> c_int;
    pub fn rbc_get_physical(c: *mut RbcCase, field: c_int, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn rbc_get_coords(c: *const RbcCase, field: c_int, x: *mut c_double, y: *mut c_double) -> c_int;
    pub fn rbc_eval(c: *mut RbcCase, what: c_int, out: *mut c_double) -> c_int;
    pub fn rbc_get_stream(c: *mut RbcCase, stream: *mut *mut c_void) -> c_int;
    pub fn rbc_device_bytes(c: *const RbcCase, bytes: *mut usize) -> c_int;
    pub fn rbc_profile_step(c: *mut RbcCase, nsteps: c_int, stage_ms: *mut c_double, max_stages: c_int, nstages: *mut c_int) -> c_int;
    pub fn rbc_stage_name(c: *const RbcCase, k: c_int) -> *const c_char;
    pub fn rbc_stage_bytes(c: *const RbcCase, k: c_int, bytes: *mut c_double) -> c_int;
    pub fn rbc_kernel_name(kernel: c_int) -> *const c_char;
    pub fn rbc_batch_create(params: *const RbcParams, ncases: c_int, out: *mut *mut RbcBatch) -> c_int;
    pub fn rbc_batch_destroy(b: *mut RbcBatch) -> c_int;
    pub fn rbc_batch_size(b: *const RbcBatch, ncases: *mut c_int) -> c_int;
    pub fn rbc_batch_case(b: *mut RbcBatch, i: c_int, c: *mut *mut RbcCase) -> c_int;
    pub fn rbc_batch_step(b: *mut RbcBatch, nsteps: c_int) -> c_int;
    pub fn rbc_batch_synchronize(b: *mut RbcBatch) -> c_int;
    pub fn rbc_batch_layout(b: *const RbcBatch, nbuckets: *mut c_int, launches_per_step: *mut c_int) -> c_int;
    pub fn rbc_batch_get_stream(b: *mut RbcBatch, stream: *mut *mut c_void) -> c_int;
    pub fn rbc_batch_profile_step(b: *mut RbcBatch, nsteps: c_int, stage_ms: *mut c_double, stage_bytes: *mut c_double, stage_kernel: *mut c_int, max_stages: c_int, nstages: *mut c_int) -> c_int;
    pub fn rbc_batch_profile_launches(b: *mut RbcBatch, nsteps: c_int, kernel: *mut c_int, bucket: *mut c_int, pass: *mut c_int, ms: *mut c_double, bytes: *mut c_double, max_launches: c_int, nlaunches: *mut c_int) -> c_int;
    pub fn rbc_batch_tuning(b: *const RbcBatch, k: c_int, kernel_cta: *mut c_int, kernel_lanes: *mut c_int, ms_cta: *mut c_double, ms_lanes: *mut c_double, n: *mut c_int) -> c_int;
    pub fn rbc_batch_tuning_forms(b: *const RbcBatch, buf: *mut c_char, len: usize) -> c_int;
    pub fn rbc_batch_state_bytes(b: *const RbcBatch, bytes: *mut usize) -> c_int;
    pub fn rbc_batch_state_offset(b: *const RbcBatch, i: c_int, offset: *mut usize) -> c_int;
    pub fn rbc_batch_get_state_all(b: *mut RbcBatch, host: *mut c_void, bytes: usize) -> c_int;
    pub fn rbc_batch_set_state_all(b: *mut RbcBatch, host: *const c_void, bytes: usize) -> c_int;
    pub fn rbc_batch_step_io(b: *mut RbcBatch, host_in: *const c_void, host_out: *mut c_void, bytes: usize, nsteps: c_int) -> c_int;
    pub fn rbc_write_snapshot(c: *mut RbcCase, path: *const c_char) -> c_int;
    pub fn rbc_read_snapshot(c: *mut RbcCase, path: *const c_char) -> c_int;
    pub fn rbc_stats_reset(c: *mut RbcCase) -> c_int;
    pub fn rbc_stats_update(c: *mut RbcCase) -> c_int;
    pub fn rbc_stats_info(c: *const RbcCase, tot_time: *mut c_double, avg_time: *mut c_double, num_save: *mut c_long) -> c_int;
    pub fn rbc_stats_get(c: *mut RbcCase, which: c_int, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn rbc_stats_write(c: *mut RbcCase, path: *const c_char) -> c_int;
    pub fn rbc_diag_record(c: *mut RbcCase) -> c_int;
    pub fn rbc_diag_series(c: *const RbcCase, time: *mut c_double, nu: *mut c_double, nuvol: *mut c_double, re: *mut c_double, max_entries: c_int, n: *mut c_int) -> c_int;
    pub fn rbc_server_create(cfg: *const RbcServerConfig, out: *mut *mut RbcServer) -> c_int;
    pub fn rbc_server_submit(s: *mut RbcServer, params: *const RbcParams, horizon: c_double, seed: u64, id: *mut c_longlong) -> c_int;
    pub fn rbc_server_cancel(s: *mut RbcServer, id: c_longlong, found: *mut c_int) -> c_int;
    pub fn rbc_server_poll(s: *mut RbcServer, out: *mut RbcRequestResult, max_results: c_int, n: *mut c_int) -> c_int;
    pub fn rbc_server_wait_idle(s: *mut RbcServer, timeout_s: c_double, idle: *mut c_int) -> c_int;
    pub fn rbc_server_stats(s: *mut RbcServer, stats: *mut RbcServerStats) -> c_int;
    pub fn rbc_server_destroy(s: *mut RbcServer) -> c_int;
    pub fn rbc_host_alloc_pinned(ptr: *mut *mut c_void, bytes: usize) -> c_int;
    pub fn rbc_host_free_pinned(ptr: *mut c_void) -> c_int;
    pub fn rbc_dev_alloc(ptr: *mut *mut c_void, bytes: usize) -> c_int;
    pub fn rbc_dev_free(ptr: *mut c_void) -> c_int;
    pub fn rbc_memcpy_h2d(dst: *mut c_void, src: *const c_void, bytes: usize) -> c_int;
    pub fn rbc_memcpy_d2h(dst: *mut c_void, src: *const c_void, bytes: usize) -> c_int;
    pub fn rbc_device_synchronize() -> c_int;
    pub fn rbc_set_device(ordinal: c_int) -> c_int;
    pub fn rbc_get_device(ordinal: *mut c_int) -> c_int;
    pub fn fs_space_create(base0: c_int, n0: c_int, base1: c_int, n1: c_int, out: *mut *mut FsSpace) -> c_int;
    pub fn fs_space_destroy(s: *mut FsSpace) -> c_int;
    pub fn fs_space_shape(s: *const FsSpace, which: c_int, n0: *mut c_int, n1: *mut c_int, is_complex: *mut c_int) -> c_int;
    pub fn fs_forward(s: *mut FsSpace, d_phys: *const c_double, d_spec: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn fs_backward(s: *mut FsSpace, d_spec: *const c_double, d_phys: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn fs_to_ortho(s: *mut FsSpace, d_spec: *const c_double, d_ortho: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn fs_from_ortho(s: *mut FsSpace, d_ortho: *const c_double, d_spec: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn fs_gradient(s: *mut FsSpace, d_spec: *const c_double, d_ortho: *mut c_double, deriv0: c_int, deriv1: c_int, scale: *const c_double, stream: *mut c_void) -> c_int;
    pub fn fs_forward_noalloc(s: *mut FsSpace, d_phys: *const c_double, d_spec: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn fs_lanes_create(base: c_int, n: c_int, precision: c_int, out: *mut *mut FsLanes) -> c_int;
    pub fn fs_lanes_destroy(p: *mut FsLanes) -> c_int;
    pub fn fs_lanes_shape(p: *const FsLanes, n: *mut c_int, m: *mut c_int) -> c_int;
    pub fn fs_lanes_set_hholtz(p: *mut FsLanes, c: c_double) -> c_int;
    pub fn fs_lanes_apply(p: *mut FsLanes, op: c_int, d_in: *const c_double, d_out: *mut c_double, lanes: c_int, stream: *mut c_void) -> c_int;
    pub fn fs_lanes_status(p: *mut FsLanes, stream: *mut c_void, status: *mut c_uint) -> c_int;
    pub fn rbc_set_gemm_wait_limit(polls: c_longlong) -> c_int;
    pub fn sv_create(s: *mut FsSpace, kind: c_int, c: *const c_double, out: *mut *mut SvSolver) -> c_int;
    pub fn sv_destroy(sv: *mut SvSolver) -> c_int;
    pub fn sv_solve(sv: *mut SvSolver, d_in: *const c_double, d_out: *mut c_double, stream: *mut c_void) -> c_int;
    pub fn rbc_adjoint_create(params: *const RbcParams, out: *mut *mut RbcAdjoint) -> c_int;
    pub fn rbc_adjoint_destroy(a: *mut RbcAdjoint) -> c_int;
    pub fn rbc_adjoint_set_velocity(a: *mut RbcAdjoint, amp: c_double, m: c_double, n: c_double) -> c_int;
    pub fn rbc_adjoint_set_temperature(a: *mut RbcAdjoint, amp: c_double, m: c_double, n: c_double) -> c_int;
    pub fn rbc_adjoint_step(a: *mut RbcAdjoint, nsteps: c_int) -> c_int;
    pub fn rbc_adjoint_synchronize(a: *mut RbcAdjoint) -> c_int;
    pub fn rbc_adjoint_get_time(a: *const RbcAdjoint, t: *mut c_double) -> c_int;
    pub fn rbc_adjoint_set_time(a: *mut RbcAdjoint, t: c_double) -> c_int;
    pub fn rbc_adjoint_field_shape(a: *const RbcAdjoint, field: c_int, n0: *mut c_int, n1: *mut c_int, is_complex: *mut c_int) -> c_int;
    pub fn rbc_adjoint_get_state(a: *mut RbcAdjoint, field: c_int, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn rbc_adjoint_set_state(a: *mut RbcAdjoint, field: c_int, host: *const c_double, n_doubles: usize) -> c_int;
    pub fn rbc_adjoint_eval(a: *mut RbcAdjoint, what: c_int, out: *mut c_double) -> c_int;
    pub fn rbc_adjoint_residual(a: *mut RbcAdjoint, out: *mut c_double) -> c_int;
    pub fn rbc_adjoint_exit(a: *mut RbcAdjoint, stop: *mut c_int) -> c_int;
    pub fn rbc_adjoint_get_stream(a: *mut RbcAdjoint, stream: *mut *mut c_void) -> c_int;
    pub fn rbc_adjoint_write_snapshot(a: *mut RbcAdjoint, path: *const c_char) -> c_int;
    pub fn rbc_adjoint_read_snapshot(a: *mut RbcAdjoint, path: *const c_char) -> c_int;
    pub fn df_create(base0: c_int, n0: c_int, base1: c_int, n1: c_int, kappa: c_double, dt: c_double, out: *mut *mut DfCase) -> c_int;
    pub fn df_destroy(d: *mut DfCase) -> c_int;
    pub fn df_shape(d: *const DfCase, which: c_int, n0: *mut c_int, n1: *mut c_int, is_complex: *mut c_int) -> c_int;
    pub fn df_get_state(d: *mut DfCase, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn df_set_state(d: *mut DfCase, host: *const c_double, n_doubles: usize) -> c_int;
    pub fn df_impulse(d: *mut DfCase) -> c_int;
    pub fn df_add_force(d: *mut DfCase, force: *const c_double, n_doubles: usize) -> c_int;
    pub fn df_add_fieldbc(d: *mut DfCase, base0: c_int, base1: c_int, vhat: *const c_double, n_doubles: usize) -> c_int;
    pub fn df_step(d: *mut DfCase, nsteps: c_int) -> c_int;
    pub fn df_synchronize(d: *mut DfCase) -> c_int;
    pub fn df_get_time(d: *const DfCase, t: *mut c_double) -> c_int;
    pub fn df_get_dt(d: *const DfCase, dt: *mut c_double) -> c_int;
    pub fn df_get_physical(d: *mut DfCase, with_bc: c_int, host: *mut c_double, n_doubles: usize) -> c_int;
    pub fn df_get_stream(d: *mut DfCase, stream: *mut *mut c_void) -> c_int;
}
