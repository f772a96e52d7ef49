//! Raw bindings of `include/bacon_gb300.h`.  Every `#[repr(C)]` struct has
//! the header's fields in the header's order, and every function its
//! signature; `tests/test_rust_binding_cpu.py` checks both against the
//! header.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

/// Opaque `bacon_ctx`.
#[repr(C)]
pub struct bacon_ctx {
    _private: [u8; 0],
}

/// Opaque `bacon_builder`.
#[repr(C)]
pub struct bacon_builder {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_problem {
    pub n: i64,
    pub dim: i32,
    pub rhs: i32,
    pub n_params: i32,
    pub dyn_dim: i32,
    pub y0: *const f64,
    pub params: *const f64,
    pub t0: *const f64,
    pub t_end: *const f64,
    pub shared: *const f64,
    pub t0_scalar: f64,
    pub t_end_scalar: f64,
    pub tol: f64,
    pub dt_min: f64,
    pub dt_max: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_rk_options {
    pub method: i32,
    pub layout: i32,
    pub precision: i32,
    pub memory: i32,
    pub max_attempts: i64,
    pub block: i32,
    pub blocks_per_sm: i32,
    pub use_graph: i32,
    pub schedule: i32,
    pub systems_per_warp: i32,
    pub reserved: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_rk_result {
    pub y_final: *mut f64,
    pub t_final: *mut f64,
    pub accepted: *mut i32,
    pub rejected: *mut i32,
    pub status: *mut i32,
    pub traj_t: *mut f64,
    pub traj_y: *mut f64,
    pub traj_cap: i32,
    pub reserved: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_bdf_options {
    pub method: i32,
    pub mode: i32,
    pub memory: i32,
    pub max_iter: i32,
    pub max_steps: i64,
    pub block: i32,
    pub blocks_per_sm: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_adams_options {
    pub order: i32,
    pub memory: i32,
    pub max_attempts: i64,
    pub block: i32,
    pub blocks_per_sm: i32,
    pub systems_per_warp: i32,
    pub reserved: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_ragged_problem {
    pub n: i64,
    pub rhs: i32,
    pub reserved: i32,
    pub y_offsets: *const i64,
    pub p_offsets: *const i64,
    pub y0: *const f64,
    pub params: *const f64,
    pub t0: *const f64,
    pub t_end: *const f64,
    pub t0_scalar: f64,
    pub t_end_scalar: f64,
    pub tol: f64,
    pub dt_min: f64,
    pub dt_max: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_ragged_result {
    pub y_final: *mut f64,
    pub t_final: *mut f64,
    pub accepted: *mut i32,
    pub rejected: *mut i32,
    pub status: *mut i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_rk_kernel_args {
    pub n: i64,
    pub y0: *const f64,
    pub params: *const f64,
    pub t0: *const f64,
    pub t_end: *const f64,
    pub t0_s: f64,
    pub t_end_s: f64,
    pub tol: f64,
    pub dt_min: f64,
    pub dt_max: f64,
    pub max_attempts: i64,
    pub y_out: *mut f64,
    pub t_out: *mut f64,
    pub accepted: *mut i32,
    pub rejected: *mut i32,
    pub status: *mut i32,
    pub traj_t: *mut f64,
    pub traj_y: *mut f64,
    pub traj_cap: i32,
    pub traj_off: *const i64,
    pub queue: *mut u64,
    pub first_fail: *mut u64,
    pub order: *const u32,
    pub dt_log: *mut f64,
    pub ckpt: *mut f64,
    pub ckpt_every: i32,
    pub max_steps: i32,
    pub ckpt_slots: i32,
    pub lanes: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_tune_result {
    pub variant: i32,
    pub max_registers: i32,
    pub systems_per_warp: i32,
    pub block: i32,
    pub blocks_per_sm: i32,
    pub candidates: i32,
    pub best_ms: f64,
    pub default_ms: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_dense_output {
    pub capacity: i64,
    pub t: *mut f64,
    pub y: *mut f64,
    pub offsets: *mut i64,
    pub total: i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_ragged_dense_output {
    pub capacity: i64,
    pub value_capacity: i64,
    pub t: *mut f64,
    pub y: *mut f64,
    pub offsets: *mut i64,
    pub value_offsets: *mut i64,
    pub total: i64,
    pub total_values: i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bacon_adjoint {
    pub target: *const f64,
    pub loss: *mut f64,
    pub dl_dy0: *mut f64,
    pub dl_dp: *mut f64,
    pub checkpoint_every: i32,
    pub max_steps: i32,
}

extern "C" {
    pub fn bacon_ctx_create(device: c_int, out: *mut *mut bacon_ctx) -> c_int;
    pub fn bacon_ctx_destroy(ctx: *mut bacon_ctx) -> c_int;
    pub fn bacon_last_error() -> *const c_char;
    pub fn bacon_ctx_kernel_launches(ctx: *const bacon_ctx) -> i64;
    pub fn bacon_ctx_stream(ctx: *const bacon_ctx, stream: *mut *mut c_void) -> c_int;
    pub fn bacon_ctx_last_kernel_ms(ctx: *const bacon_ctx, ms: *mut f64) -> c_int;
    pub fn bacon_ctx_set_fault_injection(ctx: *mut bacon_ctx, kind: c_int) -> c_int;
    pub fn bacon_rk_solve(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
    ) -> c_int;
    pub fn bacon_rk_autotune(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        best_block: *mut i32,
        best_blocks_per_sm: *mut i32,
    ) -> c_int;
    pub fn bacon_rk_autotune_ex(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        tuned: *mut bacon_tune_result,
    ) -> c_int;
    pub fn bacon_rk_set_tuned(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        tuned: *const bacon_tune_result,
    ) -> c_int;
    pub fn bacon_rk_solve_user(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        launch: bacon_rk_launch_fn,
        user: *mut c_void,
    ) -> c_int;
    pub fn bacon_rk_solve_plain(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
    ) -> c_int;
    pub fn bacon_bdf_solve(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_bdf_options,
        result: *mut bacon_rk_result,
    ) -> c_int;
    pub fn bacon_adams_solve(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_adams_options,
        result: *mut bacon_rk_result,
    ) -> c_int;
    pub fn bacon_euler_solve(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        dt: f64,
        options: *const bacon_adams_options,
        result: *mut bacon_rk_result,
    ) -> c_int;
    pub fn bacon_ragged_validate(problem: *const bacon_ragged_problem) -> c_int;
    pub fn bacon_bdf_solve_mixed(
        ctx: *mut bacon_ctx,
        uniform: *const bacon_problem,
        ragged: *const bacon_ragged_problem,
        options: *const bacon_bdf_options,
        uniform_result: *mut bacon_rk_result,
        ragged_result: *mut bacon_ragged_result,
    ) -> c_int;
    pub fn bacon_rk_solve_adjoint(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        adjoint: *mut bacon_adjoint,
    ) -> c_int;
    pub fn bacon_ctx_last_reverse_ms(ctx: *const bacon_ctx, ms: *mut f64) -> c_int;
    pub fn bacon_rk_solve_dense(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        dense: *mut bacon_dense_output,
    ) -> c_int;
    pub fn bacon_bdf_solve_mixed_dense(
        ctx: *mut bacon_ctx,
        uniform: *const bacon_problem,
        ragged: *const bacon_ragged_problem,
        options: *const bacon_bdf_options,
        uniform_result: *mut bacon_rk_result,
        ragged_result: *mut bacon_ragged_result,
        uniform_dense: *mut bacon_dense_output,
        ragged_dense: *mut bacon_ragged_dense_output,
    ) -> c_int;
    pub fn bacon_bdf_solve_dense(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_bdf_options,
        result: *mut bacon_rk_result,
        dense: *mut bacon_dense_output,
    ) -> c_int;
    pub fn bacon_euler_solve_dense(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        dt: f64,
        options: *const bacon_adams_options,
        result: *mut bacon_rk_result,
        dense: *mut bacon_dense_output,
    ) -> c_int;
    pub fn bacon_adams_solve_dense(
        ctx: *mut bacon_ctx,
        problem: *const bacon_problem,
        options: *const bacon_adams_options,
        result: *mut bacon_rk_result,
        dense: *mut bacon_dense_output,
    ) -> c_int;
    pub fn bacon_rk_solve_noalloc(
        problem: *const bacon_problem,
        options: *const bacon_rk_options,
        result: *mut bacon_rk_result,
        stream: *mut c_void,
    ) -> c_int;
    pub fn bacon_rk_validate(problem: *const bacon_problem) -> c_int;
    pub fn bacon_builder_new(kind: i32, dim: i32, out: *mut *mut bacon_builder) -> c_int;
    pub fn bacon_builder_new_dyn(kind: i32, size: i32, out: *mut *mut bacon_builder) -> c_int;
    pub fn bacon_builder_free(b: *mut bacon_builder);
    pub fn bacon_builder_with_tolerance(b: *mut bacon_builder, tol: f64) -> c_int;
    pub fn bacon_builder_with_maximum_dt(b: *mut bacon_builder, max: f64) -> c_int;
    pub fn bacon_builder_with_minimum_dt(b: *mut bacon_builder, min: f64) -> c_int;
    pub fn bacon_builder_with_initial_time(b: *mut bacon_builder, initial: f64) -> c_int;
    pub fn bacon_builder_with_ending_time(b: *mut bacon_builder, ending: f64) -> c_int;
    pub fn bacon_builder_with_initial_conditions(b: *mut bacon_builder, y0: *const f64, n: i64) -> c_int;
    pub fn bacon_builder_with_derivative(
        b: *mut bacon_builder,
        rhs: i32,
        params: *const f64,
        n_params: i32,
    ) -> c_int;
    pub fn bacon_builder_with_ending_times(b: *mut bacon_builder, t_end: *const f64, n: i64) -> c_int;
    pub fn bacon_builder_problem(b: *const bacon_builder, out: *mut bacon_problem) -> c_int;
    pub fn bacon_measure_fp64_peak(ctx: *mut bacon_ctx, gflops: *mut f64) -> c_int;
}

/// `bacon_rk_launch_fn`: the caller's launcher of its own right-hand side's
/// persistent kernel (see include/bacon_gb300_rhs.cuh).
pub type bacon_rk_launch_fn = Option<
    unsafe extern "C" fn(
        args: *const bacon_rk_kernel_args,
        method: i32,
        layout: i32,
        precision: i32,
        grid: i32,
        block: i32,
        stream: *mut c_void,
        user: *mut c_void,
    ) -> c_int,
>;
