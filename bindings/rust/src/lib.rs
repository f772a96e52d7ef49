//! Rust host side of the bacon_gb300 engine.
//!
//! `ffi` binds every entry point of `include/bacon_gb300.h` one to one.
//! `gpu` puts the builder spelling of bacon-sci 0.16.2's `IVPSolver` trait
//! (`src/ivp.rs:134-190`) and the README's spelling (`with_dt_min`,
//! `with_dt_max`, `with_start`, `with_end`, `build`, `solve_ivp`,
//! `README.md:32-40`) over batched solves, plus the gradient entry point
//! `solve_ivp_adjoint`.
pub mod ffi;
pub mod gpu;

pub use gpu::{
    last_error, solve_mixed, AdjointSolution, BatchSolution, Context, GpuBdf6, GpuError, GpuRungeKutta23,
    GpuRungeKutta45, Layout, Precision, RaggedBatch, RaggedSolution, Rhs,
};
