//! `coupe_gpu::Rcb` and `coupe_gpu::Rib`: coupe's recursive coordinate and
//! inertial bisection on a GB300 GPU, implementing coupe's own
//! `Partition<(points, weights)>` trait (coupe/src/lib.rs:76-91) with the same
//! `iter_count` / `tolerance` fields as `coupe::Rcb` and `coupe::Rib`
//! (coupe/src/algorithms/recursive_bisection.rs:780-812, 902-930).
//!
//! The work is done by libcoupe_gpu.so through its C ABI (include/coupe.h,
//! include/coupe_gpu.h); there is no CPU fallback.  With integer weights the
//! part ids equal coupe's.
//!
//! This crate is source only in this repository: the build image has no Rust
//! toolchain.  It is the binding a coupe user would add to switch the path to
//! the GPU.

use coupe::PointND;
use rayon::iter::{IndexedParallelIterator, IntoParallelIterator, ParallelIterator};
use std::os::raw::{c_int, c_void};

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

#[link(name = "coupe_gpu")]
unsafe extern "C" {
    fn coupe_data_array(len: usize, type_: c_int, data: *const c_void) -> *mut CoupeData;
    fn coupe_data_free(data: *mut CoupeData);
    fn coupe_gpu_rcb(partition: *mut usize, dimension: usize, points: *const CoupeData,
                     weights: *const CoupeData, iter_count: usize, tolerance: f64, mode: c_int) -> c_int;
    fn coupe_gpu_rib(partition: *mut usize, dimension: usize, points: *const CoupeData,
                     weights: *const CoupeData, iter_count: usize, tolerance: f64, mode: c_int) -> c_int;
}

/// Key precision (enum coupe_gpu_mode).
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub enum Mode {
    /// coupe's f32 arithmetic: ids equal coupe::Rcb's for integer weights.
    #[default]
    Ref32 = 0,
    /// The same algorithm in f64.
    F64 = 1,
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
                                     iter_count: usize, tolerance: f64, mode: Mode) -> Result<(), coupe::Error> {
    if weights.len() != part_ids.len() {
        return Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: weights.len() });
    }
    if points.len() != part_ids.len() {
        return Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: points.len() });
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
    match rc {
        ERR_OK => Ok(()),
        ERR_LEN_MISMATCH => Err(coupe::Error::InputLenMismatch { expected: part_ids.len(), actual: points.len() }),
        ERR_ALLOC => panic!("libcoupe_gpu: allocation failed"),
        other => panic!("libcoupe_gpu error {other}"),
    }
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
    type Error = coupe::Error;

    fn partition(&mut self, part_ids: &mut [usize], (points, weights): (P, W)) -> Result<(), coupe::Error> {
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
    type Error = coupe::Error;

    fn partition(&mut self, part_ids: &mut [usize], (points, weights): (&'a [PointND<D>], W))
                 -> Result<(), coupe::Error> {
        let weights: Vec<W::Item> = weights.into_par_iter().collect();
        run(true, part_ids, points, &weights, self.iter_count, self.tolerance, self.mode)
    }
}
