//! GPU back end of `sde_sim_rs::sim::simulate` (src/sim/mod.rs:20-92)
//! through libsdegpu's C ABI (include/sdegpu.h).
//!
//! Files a maintainer adds to the reference crate: this module as
//! `src/gpu.rs`, `build.rs` beside `Cargo.toml`, and in `Cargo.toml`
//!
//! ```toml
//! [features]
//! gpu = []
//! ```
//!
//! plus, in `src/lib.rs`, `#[cfg(feature = "gpu")] pub mod gpu;`.  With the
//! feature on, `sim::simulate` starts with
//!
//! ```ignore
//! #[cfg(feature = "gpu")]
//! return crate::gpu::simulate(process_universe, &equations, timesteps,
//!                             initial_values, num_scenarios, scheme, rng_method);
//! ```
//!
//! where `equations` are the strings the universe was parsed from
//! (`parse_equations`, src/proc/util.rs:52-55, would keep them).
//!
//! Written against include/sdegpu.h; not compiled in this repository (no
//! cargo or rustc on the machines it was built on).  The call sequence it
//! makes -- sde_simulate, sde_result_shape, sde_result_copy_long,
//! sde_result_destroy, and sde_last_error on failure -- is exercised through
//! ctypes by tests/test_gpu_rust_shim_sequence.py, and its extern block is
//! checked against the header by tests/test_abi_cpu.py.

use std::collections::HashMap;
use std::ffi::{CStr, CString, c_char, c_int};

use ordered_float::OrderedFloat;
use polars::prelude::*;

use crate::proc::ProcessUniverse;

/// Opaque result handle (`sde_result*`).
#[repr(C)]
pub struct SdeResult {
    _private: [u8; 0],
}

unsafe extern "C" {
    fn sde_simulate(
        equations: *const *const c_char,
        n_equations: i32,
        times: *const f64,
        n_times: i32,
        init_names: *const *const c_char,
        init_values: *const f64,
        n_init: i32,
        n_scenarios: u64,
        scheme: *const c_char,
        rng_method: *const c_char,
        seed: u64,
        has_seed: i32,
        out_result: *mut *mut SdeResult,
    ) -> c_int;
    fn sde_result_shape(
        r: *const SdeResult,
        n_paths: *mut u64,
        n_out_times: *mut i32,
        n_processes: *mut i32,
        n_replicates: *mut i32,
    ) -> c_int;
    fn sde_result_copy_long(
        r: *mut SdeResult,
        scenario: *mut i32,
        time: *mut f64,
        process: *mut i32,
        value: *mut f64,
    ) -> c_int;
    fn sde_result_destroy(r: *mut SdeResult) -> c_int;
    fn sde_last_error(buf: *mut c_char, buf_len: usize) -> c_int;
}

/// The engine's message for the calling thread's last failure.
fn last_error() -> String {
    let mut buf = vec![0 as c_char; 4096];
    unsafe {
        sde_last_error(buf.as_mut_ptr(), buf.len());
        CStr::from_ptr(buf.as_ptr()).to_string_lossy().into_owned()
    }
}

fn check(rc: c_int, what: &str) -> PolarsResult<()> {
    if rc == 0 {
        Ok(())
    } else {
        Err(PolarsError::ComputeError(format!("{what}: {} (status {rc})", last_error()).into()))
    }
}

/// Owns a result handle; destroys it on every path out.
struct ResultGuard(*mut SdeResult);

impl Drop for ResultGuard {
    fn drop(&mut self) {
        if !self.0.is_null() {
            unsafe { sde_result_destroy(self.0) };
        }
    }
}

fn cstrings(items: &[String]) -> PolarsResult<Vec<CString>> {
    items
        .iter()
        .map(|s| CString::new(s.as_str()).map_err(|e| PolarsError::ComputeError(e.to_string().into())))
        .collect()
}

/// `sim::simulate` on the GPU: same arguments, the same long frame
/// (scenario:i32, time:f64, process_name:str, value:f64) in the same row
/// order (src/filtration.rs:81-116 per scenario, concatenated by scenario).
/// The seed is drawn from the OS as the reference draws it
/// (src/sim/mod.rs:28-29); the engine does that when has_seed is 0.
pub fn simulate(
    process_universe: &ProcessUniverse,
    equations: &[String],
    timesteps: Vec<OrderedFloat<f64>>,
    initial_values: HashMap<String, f64>,
    num_scenarios: u64,
    scheme: &str,
    rng_method: &str,
) -> PolarsResult<LazyFrame> {
    let eqs = cstrings(equations)?;
    let eq_ptrs: Vec<*const c_char> = eqs.iter().map(|s| s.as_ptr()).collect();
    let names: Vec<String> = initial_values.keys().cloned().collect();
    let name_cs = cstrings(&names)?;
    let name_ptrs: Vec<*const c_char> = name_cs.iter().map(|s| s.as_ptr()).collect();
    let values: Vec<f64> = names.iter().map(|k| initial_values[k]).collect();
    let times: Vec<f64> = timesteps.iter().map(|t| t.into_inner()).collect();
    let scheme_c = CString::new(scheme).map_err(|e| PolarsError::ComputeError(e.to_string().into()))?;
    let rng_c = CString::new(rng_method).map_err(|e| PolarsError::ComputeError(e.to_string().into()))?;

    let mut raw: *mut SdeResult = std::ptr::null_mut();
    check(
        unsafe {
            sde_simulate(
                eq_ptrs.as_ptr(),
                eq_ptrs.len() as i32,
                times.as_ptr(),
                times.len() as i32,
                name_ptrs.as_ptr(),
                values.as_ptr(),
                values.len() as i32,
                num_scenarios,
                scheme_c.as_ptr(),
                rng_c.as_ptr(),
                0,
                0,
                &mut raw,
            )
        },
        "sde_simulate",
    )?;
    let result = ResultGuard(raw);

    let (mut n_paths, mut n_out, mut n_proc, mut n_rep) = (0u64, 0i32, 0i32, 0i32);
    check(
        unsafe { sde_result_shape(result.0, &mut n_paths, &mut n_out, &mut n_proc, &mut n_rep) },
        "sde_result_shape",
    )?;
    let rows = n_paths as usize * n_out as usize * n_proc as usize * n_rep as usize;
    let mut scenario = vec![0i32; rows];
    let mut time = vec![0f64; rows];
    let mut process = vec![0i32; rows];
    let mut value = vec![0f64; rows];
    check(
        unsafe {
            sde_result_copy_long(
                result.0,
                scenario.as_mut_ptr(),
                time.as_mut_ptr(),
                process.as_mut_ptr(),
                value.as_mut_ptr(),
            )
        },
        "sde_result_copy_long",
    )?;
    drop(result);

    // process index -> ProcessUniverse.processes[i].name() (src/proc/mod.rs:46-59)
    let process_name: Vec<&str> = process
        .iter()
        .map(|&i| process_universe.processes[i as usize].name())
        .collect();
    Ok(df![
        "scenario" => scenario,
        "time" => time,
        "process_name" => process_name,
        "value" => value,
    ]?
    .lazy())
}
