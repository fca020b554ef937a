//! `coupe_gpu::Rcb` and `coupe_gpu::Rib`: coupe's recursive coordinate and
//! inertial bisection on a GB300 GPU, implementing coupe's own
//! `Partition<(points, weights)>` trait (coupe/src/lib.rs:76-91) with the same
//! `iter_count` / `tolerance` fields as `coupe::Rcb` and `coupe::Rib`
//! (coupe/src/algorithms/recursive_bisection.rs:780-812, 902-930).
//!
//! The work is done by libcoupe_gpu.so through its C ABI (include/coupe.h,
//! include/coupe_gpu.h); there is no CPU fallback.  With integer weights the
//! part ids equal coupe's.  The partitioners' error type is `GpuError`:
//! coupe's own errors, plus the library's failures (allocation, CUDA), which
//! are returned rather than panicking.
//!
//! This crate is source only in this repository: the build image has no Rust
//! toolchain.  It is the binding a coupe user would add to switch the path to
//! the GPU.

use coupe::PointND;
use rayon::iter::{IndexedParallelIterator, IntoParallelIterator, ParallelIterator};
use std::ffi::CStr;
use std::fmt;
use std::os::raw::{c_char, c_int, c_void};

#[repr(C)]
struct CoupeData {
    _opaque: [u8; 0],
}

const COUPE_INT: c_int = 0;
const COUPE_INT64: c_int = 1;
const COUPE_DOUBLE: c_int = 2;

const ERR_OK: c_int = 0;
const ERR_ALLOC: c_int = 1;
const ERR_LEN_MISMATCH: c_int = 6;
const ERR_NOT_FOUND: c_int = 7;
const ERR_NEG_VALUES: c_int = 8;

#[link(name = "coupe_gpu")]
unsafe extern "C" {
    fn coupe_data_array(len: usize, type_: c_int, data: *const c_void) -> *mut CoupeData;
    fn coupe_data_free(data: *mut CoupeData);
    fn coupe_gpu_rcb(partition: *mut usize, dimension: usize, points: *const CoupeData,
                     weights: *const CoupeData, iter_count: usize, tolerance: f64, mode: c_int) -> c_int;
    fn coupe_gpu_rib(partition: *mut usize, dimension: usize, points: *const CoupeData,
                     weights: *const CoupeData, iter_count: usize, tolerance: f64, mode: c_int) -> c_int;
    fn coupe_gpu_parts_load(partition: *const usize, num_parts: usize, weights: *const CoupeData,
                            loads: *mut c_void) -> c_int;
    fn coupe_gpu_imbalance(num_parts: usize, partition: *const usize, weights: *const CoupeData,
                           imbalance: *mut f64) -> c_int;
    fn coupe_gpu_grid_rcb(partition: *mut usize, dimension: usize, size: *const usize, weights: *const CoupeData,
                          iter_count: usize, threads: usize) -> c_int;
    fn coupe_gpu_multi_jagged(partition: *mut usize, dimension: usize, points: *const CoupeData,
                              weights: *const CoupeData, part_count: usize, max_iter: usize) -> c_int;
    fn coupe_gpu_last_error() -> *const c_char;
}

/// Errors of the GPU partitioners: the ones coupe's partitioners return, and
/// the library's own (a failed allocation, a CUDA error or a failed device
/// check, with the library's message).  coupe's algorithms would panic on
/// the latter; here they are returned.
#[derive(Debug)]
pub enum GpuError {
    Coupe(coupe::Error),
    Alloc(String),
    Device { code: i32, message: String },
}

impl From<coupe::Error> for GpuError {
    fn from(e: coupe::Error) -> Self {
        GpuError::Coupe(e)
    }
}

impl fmt::Display for GpuError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        match self {
            GpuError::Coupe(e) => write!(f, "{e}"),
            GpuError::Alloc(m) => write!(f, "libcoupe_gpu: allocation failed ({m})"),
            GpuError::Device { code, message } => write!(f, "libcoupe_gpu error {code} ({message})"),
        }
    }
}

impl std::error::Error for GpuError {}

// The library's message for the last call on this thread.
fn last_error() -> String {
    unsafe {
        let p = coupe_gpu_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    }
}

fn check(rc: c_int, expected: usize, actual: usize) -> Result<(), GpuError> {
    match rc {
        ERR_OK => Ok(()),
        ERR_LEN_MISMATCH => Err(coupe::Error::InputLenMismatch { expected, actual }.into()),
        ERR_NOT_FOUND => Err(coupe::Error::NotFound.into()),
        ERR_NEG_VALUES => Err(coupe::Error::NegativeValues.into()),
        ERR_ALLOC => Err(GpuError::Alloc(last_error())),
        code => Err(GpuError::Device { code, message: last_error() }),
    }
}

/// Key precision (enum coupe_gpu_mode).
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub enum Mode {
    /// coupe's f32 arithmetic: ids equal coupe::Rcb's for integer weights.
    #[default]
    Ref32 = 0,
    /// The same algorithm in f64.
    F64 = 1,
    /// f32 keys with f64 decisions in the band of each cut: F64's ids.
    F32KeyF64Band = 2,
}

/// Weight types the library accepts (enum coupe_type).
pub trait GpuWeight: Copy + Send + Sync {
    const TYPE: c_int;
}
impl GpuWeight for i32 {
    const TYPE: c_int = COUPE_INT;
}
impl GpuWeight for i64 {
    const TYPE: c_int = COUPE_INT64;
}
impl GpuWeight for f64 {
    const TYPE: c_int = COUPE_DOUBLE;
}

fn run<const D: usize, W: GpuWeight>(rib: bool, part_ids: &mut [usize], points: &[PointND<D>], weights: &[W],
                                     iter_count: usize, tolerance: f64, mode: Mode) -> Result<(), GpuError> {
    if weights.len() != part_ids.len() {
        return Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: weights.len() }.into());
    }
    if points.len() != part_ids.len() {
        return Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: points.len() }.into());
    }
    // PointND<D> is D contiguous f64 (nalgebra's column storage), the layout
    // coupe_data_array expects for points.
    let rc = unsafe {
        let p = coupe_data_array(points.len(), COUPE_DOUBLE, points.as_ptr() as *const c_void);
        let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
        let f = if rib { coupe_gpu_rib } else { coupe_gpu_rcb };
        let rc = f(part_ids.as_mut_ptr(), D, p, w, iter_count, tolerance, mode as c_int);
        coupe_data_free(p);
        coupe_data_free(w);
        rc
    };
    check(rc, part_ids.len(), points.len())
}

/// Recursive coordinate bisection on the GPU (see `coupe::Rcb`).
#[derive(Clone, Copy, Debug, Default)]
pub struct Rcb {
    pub iter_count: usize,
    pub tolerance: f64,
    pub mode: Mode,
}

impl<const D: usize, P, W> coupe::Partition<(P, W)> for Rcb
where
    P: IntoParallelIterator<Item = PointND<D>>,
    P::Iter: IndexedParallelIterator,
    W: IntoParallelIterator,
    W::Item: GpuWeight,
    W::Iter: IndexedParallelIterator,
{
    type Metadata = ();
    type Error = GpuError;

    fn partition(&mut self, part_ids: &mut [usize], (points, weights): (P, W)) -> Result<(), GpuError> {
        let points: Vec<PointND<D>> = points.into_par_iter().collect();
        let weights: Vec<W::Item> = weights.into_par_iter().collect();
        run(false, part_ids, &points, &weights, self.iter_count, self.tolerance, self.mode)
    }
}

/// Recursive inertial bisection on the GPU (see `coupe::Rib`).
#[derive(Clone, Copy, Debug, Default)]
pub struct Rib {
    pub iter_count: usize,
    pub tolerance: f64,
    pub mode: Mode,
}

impl<'a, const D: usize, W> coupe::Partition<(&'a [PointND<D>], W)> for Rib
where
    W: IntoParallelIterator,
    W::Item: GpuWeight,
    W::Iter: IndexedParallelIterator,
{
    type Metadata = ();
    type Error = GpuError;

    fn partition(&mut self, part_ids: &mut [usize], (points, weights): (&'a [PointND<D>], W))
                 -> Result<(), GpuError> {
        let weights: Vec<W::Item> = weights.into_par_iter().collect();
        run(true, part_ids, points, &weights, self.iter_count, self.tolerance, self.mode)
    }
}

/// MultiJagged on the GPU (see `coupe::MultiJagged`,
/// coupe/src/algorithms/multi_jagged.rs:368-385): part ids numbered as coupe
/// numbers them with one rayon worker.  Weights must be finite and
/// non-negative (`coupe::Error::NegativeValues` otherwise); a scheme that
/// does not exist gives `coupe::Error::NotFound` where coupe's recursion
/// does not end.
#[derive(Clone, Copy, Debug)]
pub struct MultiJagged {
    pub part_count: usize,
    pub max_iter: usize,
}

impl<'a, const D: usize> coupe::Partition<(&'a [PointND<D>], &'a [f64])> for MultiJagged {
    type Metadata = ();
    type Error = GpuError;

    fn partition(&mut self, part_ids: &mut [usize], (points, weights): (&'a [PointND<D>], &'a [f64]))
                 -> Result<(), GpuError> {
        if points.len() != part_ids.len() || weights.len() != part_ids.len() {
            return Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: weights.len() }.into());
        }
        let rc = unsafe {
            let p = coupe_data_array(points.len(), COUPE_DOUBLE, points.as_ptr() as *const c_void);
            let w = coupe_data_array(weights.len(), COUPE_DOUBLE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_multi_jagged(part_ids.as_mut_ptr(), D, p, w, self.part_count, self.max_iter);
            coupe_data_free(p);
            coupe_data_free(w);
            rc
        };
        check(rc, part_ids.len(), points.len())
    }
}

/// coupe::imbalance on the GPU (coupe/src/imbalance.rs:14-77).  Integer
/// loads wrap like coupe's release build; f64 loads are exact sums rounded
/// once.  `compute_parts_load` and `imbalance` keep coupe's signatures and
/// panic where coupe's do (a part id >= num_parts, lengths that differ), with
/// the library's message on a device error; the `try_` forms return every
/// failure as a `GpuError`.
pub mod imbalance {
    use super::*;

    /// The load of each part, or the library's error.
    pub fn try_compute_parts_load<W: GpuWeight + Default>(partition: &[usize], num_parts: usize, weights: &[W])
                                                          -> Result<Vec<W>, GpuError> {
        if partition.len() != weights.len() {
            return Err(coupe::Error::InputLenMismatch { expected: partition.len(), actual: weights.len() }.into());
        }
        let mut loads = vec![W::default(); num_parts];
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_parts_load(partition.as_ptr(), num_parts, w, loads.as_mut_ptr() as *mut c_void);
            coupe_data_free(w);
            rc
        };
        check(rc, partition.len(), weights.len())?;
        Ok(loads)
    }

    /// The imbalance of a partition, or the library's error.
    pub fn try_imbalance<W: GpuWeight>(num_parts: usize, partition: &[usize], weights: &[W])
                                       -> Result<f64, GpuError> {
        if partition.len() != weights.len() {
            return Err(coupe::Error::InputLenMismatch { expected: partition.len(), actual: weights.len() }.into());
        }
        let mut out = 0.0;
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_imbalance(num_parts, partition.as_ptr(), w, &mut out);
            coupe_data_free(w);
            rc
        };
        check(rc, partition.len(), weights.len())?;
        Ok(out)
    }

    /// The load of each part (see `coupe::imbalance::compute_parts_load`).
    pub fn compute_parts_load<W: GpuWeight + Default>(partition: &[usize], num_parts: usize, weights: &[W]) -> Vec<W> {
        try_compute_parts_load(partition, num_parts, weights).unwrap_or_else(|e| panic!("{e}"))
    }

    /// The imbalance of a partition (see `coupe::imbalance::imbalance`).
    pub fn imbalance<W: GpuWeight>(num_parts: usize, partition: &[usize], weights: &[W]) -> f64 {
        try_imbalance(num_parts, partition, weights).unwrap_or_else(|e| panic!("{e}"))
    }
}

/// A cartesian grid whose Rcb runs on the GPU (see `coupe::Grid`,
/// coupe/src/cartesian/mod.rs:130-179).  The weighted median replays the
/// current rayon pool's worker count, so the ids equal coupe's in the same
/// process.
#[derive(Clone, Copy, Debug)]
pub struct Grid<const D: usize> {
    size: [usize; D],
}

impl<const D: usize> Grid<D> {
    /// Rcb on the grid (weights and ids with the first size varying
    /// fastest), or the library's error.
    pub fn try_rcb<W: GpuWeight>(self, partition: &mut [usize], weights: &[W], iter_count: usize)
                                 -> Result<(), GpuError> {
        let cells: usize = self.size.iter().product();
        if partition.len() != cells {
            return Err(coupe::Error::InputLenMismatch { expected: cells, actual: partition.len() }.into());
        }
        if weights.len() != cells {
            return Err(coupe::Error::InputLenMismatch { expected: cells, actual: weights.len() }.into());
        }
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_grid_rcb(partition.as_mut_ptr(), D, self.size.as_ptr(), w, iter_count,
                                        rayon::current_num_threads().max(2));
            coupe_data_free(w);
            rc
        };
        check(rc, cells, weights.len())
    }

    /// Rcb on the grid with coupe's signature (see `coupe::Grid::rcb`,
    /// which cannot fail): a wrong length or a device error panics with the
    /// library's message.
    pub fn rcb<W: GpuWeight>(self, partition: &mut [usize], weights: &[W], iter_count: usize) {
        self.try_rcb(partition, weights, iter_count).unwrap_or_else(|e| panic!("{e}"))
    }
}

impl Grid<2> {
    pub fn new_2d(width: std::num::NonZeroUsize, height: std::num::NonZeroUsize) -> Self {
        Self { size: [width.get(), height.get()] }
    }
}

impl Grid<3> {
    pub fn new_3d(width: std::num::NonZeroUsize, height: std::num::NonZeroUsize,
                  depth: std::num::NonZeroUsize) -> Self {
        Self { size: [width.get(), height.get(), depth.get()] }
    }
}
