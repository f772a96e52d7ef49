//! Safe batched solvers over the C ABI, spelled like bacon-sci 0.16.2.
//!
//! A builder here describes `n` independent systems at once.  The methods
//! keep the names, argument meaning and error behaviour of the `IVPSolver`
//! trait (`src/ivp.rs:134-190`) and of its `RungeKutta` / `BDF` impls
//! (`src/ivp/rk.rs:136-247`, `src/ivp/bdf.rs:144-255`); the README's older
//! spelling (`README.md:32-40`) is accepted as aliases.  The one deliberate
//! difference is the derivative: device code cannot call a Rust closure, so
//! `with_derivative` takes a registry right-hand side (`Rhs`) and per-system
//! parameters in place of `FnMut(t, &[N], &mut T)` and its cloned `data: T`.
//! Every error maps back to an `IVPError` variant by its code (1..12 in the
//! declaration order of `src/ivp.rs:50-76`); 13.. are engine extensions.
use std::ffi::CStr;
use std::ptr;

use crate::ffi;

/// The `IVPError` variants (codes 1..12) and the engine's extensions.
#[derive(Clone, Debug, PartialEq)]
pub enum GpuError {
    MissingParameters,
    UserError(String),
    ToleranceOOB,
    TimeDeltaOOB,
    TimeEndOOB,
    TimeStartOOB,
    FromPrimitiveFailure,
    MinimumTimeDeltaExceeded,
    MaximumIterationsExceeded,
    SingularMatrix,
    DynamicOnStatic,
    StaticOnDynamic,
    /// A system reached the attempt cap (the reference loops forever).
    MaxAttemptsExceeded,
    Cuda(String),
    InvalidArgument(String),
    Unsupported(String),
    /// A system took more accepted steps than a fixed buffer holds.
    CapacityExceeded,
}

impl GpuError {
    /// The error of a status code, None for BACON_OK.
    pub fn from_code(code: i32) -> Option<GpuError> {
        Some(match code {
            0 => return None,
            1 => GpuError::MissingParameters,
            2 => GpuError::UserError(last_error()),
            3 => GpuError::ToleranceOOB,
            4 => GpuError::TimeDeltaOOB,
            5 => GpuError::TimeEndOOB,
            6 => GpuError::TimeStartOOB,
            7 => GpuError::FromPrimitiveFailure,
            8 => GpuError::MinimumTimeDeltaExceeded,
            9 => GpuError::MaximumIterationsExceeded,
            10 => GpuError::SingularMatrix,
            11 => GpuError::DynamicOnStatic,
            12 => GpuError::StaticOnDynamic,
            13 => GpuError::MaxAttemptsExceeded,
            14 => GpuError::Cuda(last_error()),
            15 => GpuError::InvalidArgument(last_error()),
            16 => GpuError::Unsupported(last_error()),
            17 => GpuError::CapacityExceeded,
            other => GpuError::UserError(format!("unknown bacon_gb300 status {other}")),
        })
    }
}

impl std::fmt::Display for GpuError {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        write!(f, "{self:?}")
    }
}

impl std::error::Error for GpuError {}

fn check(code: i32) -> Result<(), GpuError> {
    match GpuError::from_code(code) {
        None => Ok(()),
        Some(e) => Err(e),
    }
}

/// Message of the calling thread's last failed call (`bacon_last_error`).
pub fn last_error() -> String {
    unsafe {
        let p = ffi::bacon_last_error();
        if p.is_null() {
            String::new()
        } else {
            CStr::from_ptr(p).to_string_lossy().into_owned()
        }
    }
}

/// The registry right-hand sides (`bacon_rhs`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[repr(i32)]
pub enum Rhs {
    Exp = 0,
    Decay = 1,
    Quadratic = 2,
    Sine = 3,
    Harmonic = 4,
    VanDerPol = 5,
    Lorenz = 6,
    LotkaVolterra = 7,
    Robertson = 8,
    Chain = 9,
    Linear = 10,
}

/// Butcher-matrix variants of the reference tableaux (`bacon_layout`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[repr(i32)]
pub enum Layout {
    AsCompiled = 0,
    AsWritten = 1,
    Fehlberg = 2,
}

/// Arithmetic of the stages (`bacon_precision`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[repr(i32)]
pub enum Precision {
    Fp64Exact = 0,
    Fp64Fma = 1,
    Fp32Comp = 2,
    TcSplit = 3,
}

/// A `bacon_ctx`: one CUDA device, its stream and the engine's caches.
pub struct Context {
    raw: *mut ffi::bacon_ctx,
}

impl Context {
    pub fn new(device: i32) -> Result<Context, GpuError> {
        let mut raw = ptr::null_mut();
        check(unsafe { ffi::bacon_ctx_create(device, &mut raw) })?;
        Ok(Context { raw })
    }

    /// Device time (ms) of the last solve's main kernel.
    pub fn last_kernel_ms(&self) -> Result<f64, GpuError> {
        let mut ms = 0.0;
        check(unsafe { ffi::bacon_ctx_last_kernel_ms(self.raw, &mut ms) })?;
        Ok(ms)
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe {
            ffi::bacon_ctx_destroy(self.raw);
        }
    }
}

/// Per-system outcome of a batched solve, host memory, row-major per system.
#[derive(Clone, Debug)]
pub struct BatchSolution {
    pub n: usize,
    pub dim: usize,
    /// Last yielded state of system i at `y[i*dim .. (i+1)*dim]`.
    pub y: Vec<f64>,
    pub t: Vec<f64>,
    /// Items the reference iterator yields per system.
    pub accepted: Vec<i32>,
    /// `Redo` results per system.
    pub rejected: Vec<i32>,
    /// 0 when the system's iterator ended with `Done`, else its error code.
    pub status: Vec<i32>,
}

impl BatchSolution {
    fn from_soa(n: usize, dim: usize, y_soa: &[f64], t: Vec<f64>, acc: Vec<i32>, rej: Vec<i32>, st: Vec<i32>) -> Self {
        let mut y = vec![0.0; n * dim];
        for i in 0..n {
            for d in 0..dim {
                y[i * dim + d] = y_soa[d * n + i];
            }
        }
        BatchSolution { n, dim, y, t, accepted: acc, rejected: rej, status: st }
    }

    /// System i as the reference's `collect_vec` would end: its last
    /// yielded `(t, y)`, or the error its iterator returned.
    pub fn system(&self, i: usize) -> Result<(f64, &[f64]), GpuError> {
        match GpuError::from_code(self.status[i]) {
            Some(e) => Err(e),
            None => Ok((self.t[i], &self.y[i * self.dim..(i + 1) * self.dim])),
        }
    }
}

/// Gradients of `L_i = ||y_i(T) - target_i||^2` per system.
#[derive(Clone, Debug)]
pub struct AdjointSolution {
    pub forward: BatchSolution,
    pub loss: Vec<f64>,
    /// dL_i / dy0_i at `dl_dy0[i*dim .. (i+1)*dim]`.
    pub dl_dy0: Vec<f64>,
    /// dL_i / dp_i at `dl_dp[i*n_params .. (i+1)*n_params]`.
    pub dl_dp: Vec<f64>,
}

/// Builder state shared by the Runge-Kutta and BDF front ends.
#[derive(Clone, Debug)]
struct Spec {
    dim: usize,
    dynamic: bool,
    tol: Option<f64>,
    dt_min: Option<f64>,
    dt_max: Option<f64>,
    t0: Option<f64>,
    t_end: Option<f64>,
    t_ends: Option<Vec<f64>>,
    n: usize,
    y0_soa: Vec<f64>,
    rhs: Option<Rhs>,
    n_params: usize,
    params_soa: Vec<f64>,
}

impl Spec {
    fn new(dim: usize, dynamic: bool) -> Spec {
        Spec {
            dim,
            dynamic,
            tol: None,
            dt_min: None,
            dt_max: None,
            t0: None,
            t_end: None,
            t_ends: None,
            n: 0,
            y0_soa: Vec::new(),
            rhs: None,
            n_params: 0,
            params_soa: Vec::new(),
        }
    }

    // src/ivp/rk.rs:168-174
    fn tolerance(&mut self, tol: f64) -> Result<(), GpuError> {
        if tol <= 0.0 {
            return Err(GpuError::ToleranceOOB);
        }
        self.tol = Some(tol);
        Ok(())
    }

    // src/ivp/rk.rs:179-192: a larger minimum is lowered to the new maximum
    fn maximum_dt(&mut self, max: f64) -> Result<(), GpuError> {
        if max <= 0.0 {
            return Err(GpuError::TimeDeltaOOB);
        }
        if let Some(min) = self.dt_min {
            if min > max {
                self.dt_min = Some(max);
            }
        }
        self.dt_max = Some(max);
        Ok(())
    }

    // src/ivp/rk.rs:197-210: a smaller maximum is raised to the new minimum
    fn minimum_dt(&mut self, min: f64) -> Result<(), GpuError> {
        if min <= 0.0 {
            return Err(GpuError::TimeDeltaOOB);
        }
        if let Some(max) = self.dt_max {
            if max < min {
                self.dt_max = Some(min);
            }
        }
        self.dt_min = Some(min);
        Ok(())
    }

    // src/ivp/rk.rs:212-221
    fn initial_time(&mut self, initial: f64) -> Result<(), GpuError> {
        if let Some(end) = self.t_end {
            if end <= initial {
                return Err(GpuError::TimeStartOOB);
            }
        }
        self.t0 = Some(initial);
        Ok(())
    }

    // src/ivp/rk.rs:223-234
    fn ending_time(&mut self, ending: f64) -> Result<(), GpuError> {
        if let Some(start) = self.t0 {
            if start >= ending {
                return Err(GpuError::TimeEndOOB);
            }
        }
        self.t_end = Some(ending);
        Ok(())
    }

    /// Row-major `n x dim` initial states, stored SoA (`[dim][n]`).
    fn initial_conditions(&mut self, y0: &[f64], n: usize) -> Result<(), GpuError> {
        if n == 0 || y0.len() != n * self.dim {
            return Err(GpuError::InvalidArgument("initial conditions are not n x dim".into()));
        }
        self.n = n;
        self.y0_soa = vec![0.0; n * self.dim];
        for i in 0..n {
            for d in 0..self.dim {
                self.y0_soa[d * n + i] = y0[i * self.dim + d];
            }
        }
        Ok(())
    }

    /// Row-major `n x n_params` parameters, stored SoA.
    fn derivative(&mut self, rhs: Rhs, params: &[f64], n_params: usize) {
        let n = if n_params == 0 { 0 } else { params.len() / n_params };
        self.rhs = Some(rhs);
        self.n_params = n_params;
        self.params_soa = vec![0.0; params.len()];
        for i in 0..n {
            for k in 0..n_params {
                self.params_soa[k * n + i] = params[i * n_params + k];
            }
        }
    }

    // The MissingParameters checks of solve (src/ivp/rk.rs:250-256).
    fn problem(&self) -> Result<ffi::bacon_problem, GpuError> {
        let (tol, dt_min, dt_max) = match (self.tol, self.dt_min, self.dt_max) {
            (Some(a), Some(b), Some(c)) => (a, b, c),
            _ => return Err(GpuError::MissingParameters),
        };
        let t0 = self.t0.ok_or(GpuError::MissingParameters)?;
        let rhs = self.rhs.ok_or(GpuError::MissingParameters)?;
        if self.n == 0 || (self.t_end.is_none() && self.t_ends.is_none()) {
            return Err(GpuError::MissingParameters);
        }
        if self.n_params > 0 && self.params_soa.len() != self.n * self.n_params {
            return Err(GpuError::InvalidArgument("parameters are not n x n_params".into()));
        }
        Ok(ffi::bacon_problem {
            n: self.n as i64,
            dim: self.dim as i32,
            rhs: rhs as i32,
            n_params: self.n_params as i32,
            dyn_dim: self.dynamic as i32,
            y0: self.y0_soa.as_ptr(),
            params: if self.n_params > 0 { self.params_soa.as_ptr() } else { ptr::null() },
            t0: ptr::null(),
            t_end: match &self.t_ends {
                Some(v) => v.as_ptr(),
                None => ptr::null(),
            },
            shared: ptr::null(),
            t0_scalar: t0,
            t_end_scalar: self.t_end.unwrap_or(0.0),
            tol,
            dt_min,
            dt_max,
        })
    }
}

struct HostOut {
    y: Vec<f64>,
    t: Vec<f64>,
    acc: Vec<i32>,
    rej: Vec<i32>,
    st: Vec<i32>,
}

impl HostOut {
    fn new(n: usize, dim: usize) -> HostOut {
        HostOut { y: vec![0.0; n * dim], t: vec![0.0; n], acc: vec![0; n], rej: vec![0; n], st: vec![0; n] }
    }

    fn result(&mut self) -> ffi::bacon_rk_result {
        ffi::bacon_rk_result {
            y_final: self.y.as_mut_ptr(),
            t_final: self.t.as_mut_ptr(),
            accepted: self.acc.as_mut_ptr(),
            rejected: self.rej.as_mut_ptr(),
            status: self.st.as_mut_ptr(),
            traj_t: ptr::null_mut(),
            traj_y: ptr::null_mut(),
            traj_cap: 0,
            reserved: 0,
        }
    }

    fn solution(self, n: usize, dim: usize) -> BatchSolution {
        BatchSolution::from_soa(n, dim, &self.y, self.t, self.acc, self.rej, self.st)
    }
}

/// Status of a whole batch: per-system failures live in `status`; only
/// argument and CUDA errors fail the call.
fn batch_ok(code: i32) -> Result<(), GpuError> {
    match code {
        14 | 15 | 16 => check(code),
        _ => Ok(()),
    }
}

/// Batched `RungeKutta45` (METHOD 0) / `RungeKutta23` (METHOD 1).
#[derive(Clone, Debug)]
pub struct GpuRungeKutta<const METHOD: i32> {
    spec: Spec,
    layout: Layout,
    precision: Precision,
    max_attempts: i64,
}

pub type GpuRungeKutta45 = GpuRungeKutta<0>;
pub type GpuRungeKutta23 = GpuRungeKutta<1>;

impl<const METHOD: i32> GpuRungeKutta<METHOD> {
    /// `IVPSolver::new` for systems of static dimension `dim`.
    pub fn new(dim: usize) -> Result<Self, GpuError> {
        if dim == 0 {
            return Err(GpuError::StaticOnDynamic);
        }
        Ok(Self { spec: Spec::new(dim, false), layout: Layout::Fehlberg, precision: Precision::Fp64Exact, max_attempts: 0 })
    }

    /// `IVPSolver::new_dyn(size)`: nalgebra `Dyn` states (dynamic norm order).
    pub fn new_dyn(size: usize) -> Result<Self, GpuError> {
        if size == 0 {
            return Err(GpuError::DynamicOnStatic);
        }
        Ok(Self { spec: Spec::new(size, true), layout: Layout::Fehlberg, precision: Precision::Fp64Exact, max_attempts: 0 })
    }

    pub fn dim(&self) -> usize {
        self.spec.dim
    }

    pub fn with_tolerance(mut self, tol: f64) -> Result<Self, GpuError> {
        self.spec.tolerance(tol)?;
        Ok(self)
    }

    pub fn with_maximum_dt(mut self, max: f64) -> Result<Self, GpuError> {
        self.spec.maximum_dt(max)?;
        Ok(self)
    }

    pub fn with_minimum_dt(mut self, min: f64) -> Result<Self, GpuError> {
        self.spec.minimum_dt(min)?;
        Ok(self)
    }

    pub fn with_initial_time(mut self, initial: f64) -> Result<Self, GpuError> {
        self.spec.initial_time(initial)?;
        Ok(self)
    }

    pub fn with_ending_time(mut self, ending: f64) -> Result<Self, GpuError> {
        self.spec.ending_time(ending)?;
        Ok(self)
    }

    /// One system's initial state (`with_initial_conditions_slice`).
    pub fn with_initial_conditions_slice(mut self, start: &[f64]) -> Result<Self, GpuError> {
        self.spec.initial_conditions(start, 1)?;
        Ok(self)
    }

    /// n systems at once, row-major `n x dim`.
    pub fn with_initial_conditions_batch(mut self, start: &[f64], n: usize) -> Result<Self, GpuError> {
        self.spec.initial_conditions(start, n)?;
        Ok(self)
    }

    /// A registry right-hand side and its parameters, row-major
    /// `n x n_params` (empty when the right-hand side has none).
    pub fn with_derivative(mut self, rhs: Rhs, params: &[f64], n_params: usize) -> Self {
        self.spec.derivative(rhs, params, n_params);
        self
    }

    /// Batched extension: one end time per system.
    pub fn with_ending_times(mut self, ends: &[f64]) -> Result<Self, GpuError> {
        if let Some(start) = self.spec.t0 {
            if ends.iter().any(|&e| start >= e) {
                return Err(GpuError::TimeEndOOB);
            }
        }
        self.spec.t_ends = Some(ends.to_vec());
        Ok(self)
    }

    pub fn with_layout(mut self, layout: Layout) -> Self {
        self.layout = layout;
        self
    }

    pub fn with_precision(mut self, precision: Precision) -> Self {
        self.precision = precision;
        self
    }

    pub fn with_max_attempts(mut self, max_attempts: i64) -> Self {
        self.max_attempts = max_attempts;
        self
    }

    // ---- the README's spelling (README.md:32-40) ----
    pub fn with_dt_min(self, min: f64) -> Result<Self, GpuError> {
        self.with_minimum_dt(min)
    }

    pub fn with_dt_max(self, max: f64) -> Result<Self, GpuError> {
        self.with_maximum_dt(max)
    }

    pub fn with_start(self, initial: f64) -> Result<Self, GpuError> {
        self.with_initial_time(initial)
    }

    pub fn with_end(self, ending: f64) -> Result<Self, GpuError> {
        self.with_ending_time(ending)
    }

    /// The README's `with_initial_conditions(&[..])` (one system).
    pub fn with_initial_conditions(self, start: &[f64]) -> Result<Self, GpuError> {
        self.with_initial_conditions_slice(start)
    }

    /// The README's `build()`: the builder is already the solver.
    pub fn build(self) -> Self {
        self
    }

    fn options(&self) -> ffi::bacon_rk_options {
        ffi::bacon_rk_options {
            method: METHOD,
            layout: self.layout as i32,
            precision: self.precision as i32,
            memory: 1, // BACON_MEM_HOST
            max_attempts: self.max_attempts,
            block: 0,
            blocks_per_sm: 0,
            use_graph: 1,
            schedule: 0,
            systems_per_warp: 0,
            reserved: 0,
        }
    }

    /// `solve(data)?.collect_vec()` for every system: the last yielded item,
    /// the counts and the per-system status.
    pub fn solve(&self, ctx: &mut Context) -> Result<BatchSolution, GpuError> {
        let prob = self.spec.problem()?;
        let opts = self.options();
        let (n, dim) = (self.spec.n, self.spec.dim);
        let mut out = HostOut::new(n, dim);
        let mut res = out.result();
        batch_ok(unsafe { ffi::bacon_rk_solve(ctx.raw, &prob, &opts, &mut res) })?;
        Ok(out.solution(n, dim))
    }

    /// The README's `solve_ivp`.
    pub fn solve_ivp(&self, ctx: &mut Context) -> Result<BatchSolution, GpuError> {
        self.solve(ctx)
    }

    /// Batched `solve_ivp_adjoint`: the forward solve plus
    /// `L_i = ||y_i(T) - target_i||^2` and its gradient with respect to each
    /// system's initial state and parameters (discrete adjoint through the
    /// accepted steps, checkpoints every `checkpoint_every` accepted steps).
    /// `target` is row-major `n x dim`.
    pub fn solve_ivp_adjoint(&self, ctx: &mut Context, target: &[f64], checkpoint_every: i32,
                             max_steps: i32) -> Result<AdjointSolution, GpuError> {
        let prob = self.spec.problem()?;
        let opts = self.options();
        let (n, dim, np) = (self.spec.n, self.spec.dim, self.spec.n_params);
        if target.len() != n * dim {
            return Err(GpuError::InvalidArgument("target is not n x dim".into()));
        }
        let mut tgt = vec![0.0; n * dim];
        for i in 0..n {
            for d in 0..dim {
                tgt[d * n + i] = target[i * dim + d];
            }
        }
        let mut loss = vec![0.0; n];
        let mut gy = vec![0.0; n * dim];
        let mut gp = vec![0.0; n * np.max(1)];
        let mut adj = ffi::bacon_adjoint {
            target: tgt.as_ptr(),
            loss: loss.as_mut_ptr(),
            dl_dy0: gy.as_mut_ptr(),
            dl_dp: if np > 0 { gp.as_mut_ptr() } else { ptr::null_mut() },
            checkpoint_every,
            max_steps,
        };
        let mut out = HostOut::new(n, dim);
        let mut res = out.result();
        batch_ok(unsafe { ffi::bacon_rk_solve_adjoint(ctx.raw, &prob, &opts, &mut res, &mut adj) })?;
        let mut dl_dy0 = vec![0.0; n * dim];
        for i in 0..n {
            for d in 0..dim {
                dl_dy0[i * dim + d] = gy[d * n + i];
            }
        }
        let mut dl_dp = vec![0.0; n * np];
        for i in 0..n {
            for k in 0..np {
                dl_dp[i * np + k] = gp[k * n + i];
            }
        }
        Ok(AdjointSolution { forward: out.solution(n, dim), loss, dl_dy0, dl_dp })
    }
}

/// Batched corrected `BDF6` over systems of one right-hand side.
#[derive(Clone, Debug)]
pub struct GpuBdf6 {
    spec: Spec,
    max_steps: i64,
}

impl GpuBdf6 {
    pub fn new(dim: usize) -> Result<Self, GpuError> {
        if dim == 0 {
            return Err(GpuError::StaticOnDynamic);
        }
        Ok(GpuBdf6 { spec: Spec::new(dim, false), max_steps: 0 })
    }

    pub fn with_tolerance(mut self, tol: f64) -> Result<Self, GpuError> {
        self.spec.tolerance(tol)?;
        Ok(self)
    }

    pub fn with_maximum_dt(mut self, max: f64) -> Result<Self, GpuError> {
        self.spec.maximum_dt(max)?;
        Ok(self)
    }

    pub fn with_minimum_dt(mut self, min: f64) -> Result<Self, GpuError> {
        self.spec.minimum_dt(min)?;
        Ok(self)
    }

    pub fn with_initial_time(mut self, initial: f64) -> Result<Self, GpuError> {
        self.spec.initial_time(initial)?;
        Ok(self)
    }

    pub fn with_ending_time(mut self, ending: f64) -> Result<Self, GpuError> {
        self.spec.ending_time(ending)?;
        Ok(self)
    }

    pub fn with_initial_conditions_batch(mut self, start: &[f64], n: usize) -> Result<Self, GpuError> {
        self.spec.initial_conditions(start, n)?;
        Ok(self)
    }

    pub fn with_derivative(mut self, rhs: Rhs, params: &[f64], n_params: usize) -> Self {
        self.spec.derivative(rhs, params, n_params);
        self
    }

    fn options(&self) -> ffi::bacon_bdf_options {
        ffi::bacon_bdf_options { method: 0, mode: 1, memory: 1, max_iter: 0, max_steps: self.max_steps, block: 0, blocks_per_sm: 0 }
    }

    /// `BDF::solve(data)?.collect_vec()` per system (dim <= 8).
    pub fn solve(&self, ctx: &mut Context) -> Result<BatchSolution, GpuError> {
        let prob = self.spec.problem()?;
        let opts = self.options();
        let (n, dim) = (self.spec.n, self.spec.dim);
        let mut out = HostOut::new(n, dim);
        let mut res = out.result();
        batch_ok(unsafe { ffi::bacon_bdf_solve(ctx.raw, &prob, &opts, &mut res) })?;
        Ok(out.solution(n, dim))
    }
}

/// Systems of uneven size: a `Vec<BDF<Dyn>>` packed back to back.
#[derive(Clone, Debug)]
pub struct RaggedBatch {
    pub rhs: Rhs,
    pub y_offsets: Vec<i64>,
    pub p_offsets: Vec<i64>,
    pub y0: Vec<f64>,
    pub params: Vec<f64>,
    pub t0: f64,
    pub t_end: f64,
    pub tol: f64,
    pub dt_min: f64,
    pub dt_max: f64,
}

#[derive(Clone, Debug)]
pub struct RaggedSolution {
    pub y: Vec<f64>,
    pub t: Vec<f64>,
    pub accepted: Vec<i32>,
    pub rejected: Vec<i32>,
    pub status: Vec<i32>,
}

/// One launch of the corrected BDF6 over a uniform batch and a ragged batch
/// (`bacon_bdf_solve_mixed`); either may be None, not both.
pub fn solve_mixed(ctx: &mut Context, uniform: Option<&GpuBdf6>, ragged: Option<&RaggedBatch>)
                   -> Result<(Option<BatchSolution>, Option<RaggedSolution>), GpuError> {
    let uprob = match uniform {
        Some(u) => Some(u.spec.problem()?),
        None => None,
    };
    let rprob = ragged.map(|g| ffi::bacon_ragged_problem {
        n: (g.y_offsets.len() as i64) - 1,
        rhs: g.rhs as i32,
        reserved: 0,
        y_offsets: g.y_offsets.as_ptr(),
        p_offsets: g.p_offsets.as_ptr(),
        y0: g.y0.as_ptr(),
        params: g.params.as_ptr(),
        t0: ptr::null(),
        t_end: ptr::null(),
        t0_scalar: g.t0,
        t_end_scalar: g.t_end,
        tol: g.tol,
        dt_min: g.dt_min,
        dt_max: g.dt_max,
    });
    let opts = ffi::bacon_bdf_options { method: 0, mode: 1, memory: 1, max_iter: 0, max_steps: 0, block: 0, blocks_per_sm: 0 };
    let (un, ud) = uniform.map(|u| (u.spec.n, u.spec.dim)).unwrap_or((0, 0));
    let mut uout = HostOut::new(un, ud);
    let mut ures = uout.result();
    let rn = ragged.map(|g| g.y_offsets.len() - 1).unwrap_or(0);
    let rtotal = ragged.map(|g| g.y0.len()).unwrap_or(0);
    let mut rs = RaggedSolution { y: vec![0.0; rtotal], t: vec![0.0; rn], accepted: vec![0; rn], rejected: vec![0; rn], status: vec![0; rn] };
    let mut rres = ffi::bacon_ragged_result {
        y_final: rs.y.as_mut_ptr(),
        t_final: rs.t.as_mut_ptr(),
        accepted: rs.accepted.as_mut_ptr(),
        rejected: rs.rejected.as_mut_ptr(),
        status: rs.status.as_mut_ptr(),
    };
    let code = unsafe {
        ffi::bacon_bdf_solve_mixed(
            ctx.raw,
            uprob.as_ref().map_or(ptr::null(), |p| p as *const _),
            rprob.as_ref().map_or(ptr::null(), |p| p as *const _),
            &opts,
            if uniform.is_some() { &mut ures as *mut ffi::bacon_rk_result } else { ptr::null_mut() },
            if ragged.is_some() { &mut rres as *mut ffi::bacon_ragged_result } else { ptr::null_mut() },
        )
    };
    batch_ok(code)?;
    Ok((uniform.map(|_| uout.solution(un, ud)), ragged.map(|_| rs)))
}
