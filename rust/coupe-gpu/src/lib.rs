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
    fn coupe_gpu_parts_load(partition: *const usize, num_parts: usize, weights: *const CoupeData,
                            loads: *mut c_void) -> c_int;
    fn coupe_gpu_imbalance(num_parts: usize, partition: *const usize, weights: *const CoupeData,
                           imbalance: *mut f64) -> c_int;
    fn coupe_gpu_grid_rcb(partition: *mut usize, dimension: usize, size: *const usize, weights: *const CoupeData,
                          iter_count: usize, threads: usize) -> c_int;
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

/// coupe::imbalance on the GPU (coupe/src/imbalance.rs:14-77).  Integer
/// loads wrap like coupe's release build; f64 loads are exact sums rounded
/// once.  A part id >= num_parts panics, as coupe's indexing does.
pub mod imbalance {
    use super::*;

    /// The load of each part (see `coupe::imbalance::compute_parts_load`).
    pub fn compute_parts_load<W: GpuWeight + Default>(partition: &[usize], num_parts: usize, weights: &[W]) -> Vec<W> {
        assert_eq!(partition.len(), weights.len());
        let mut loads = vec![W::default(); num_parts];
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_parts_load(partition.as_ptr(), num_parts, w, loads.as_mut_ptr() as *mut c_void);
            coupe_data_free(w);
            rc
        };
        assert_eq!(rc, ERR_OK, "libcoupe_gpu error {rc}");
        loads
    }

    /// The imbalance of a partition (see `coupe::imbalance::imbalance`).
    pub fn imbalance<W: GpuWeight>(num_parts: usize, partition: &[usize], weights: &[W]) -> f64 {
        assert_eq!(partition.len(), weights.len());
        let mut out = 0.0;
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_imbalance(num_parts, partition.as_ptr(), w, &mut out);
            coupe_data_free(w);
            rc
        };
        assert_eq!(rc, ERR_OK, "libcoupe_gpu error {rc}");
        out
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
    fn run<W: GpuWeight>(self, partition: &mut [usize], weights: &[W], iter_count: usize) {
        let cells: usize = self.size.iter().product();
        assert_eq!(partition.len(), cells);
        let rc = unsafe {
            let w = coupe_data_array(weights.len(), W::TYPE, weights.as_ptr() as *const c_void);
            let rc = coupe_gpu_grid_rcb(partition.as_mut_ptr(), D, self.size.as_ptr(), w, iter_count,
                                        rayon::current_num_threads().max(2));
            coupe_data_free(w);
            rc
        };
        assert_eq!(rc, ERR_OK, "libcoupe_gpu error {rc}");
    }
}

impl Grid<2> {
    pub fn new_2d(width: std::num::NonZeroUsize, height: std::num::NonZeroUsize) -> Self {
        Self { size: [width.get(), height.get()] }
    }

    /// Rcb on the 2D grid (see `coupe::Grid::<2>::rcb`); weights and ids row major.
    pub fn rcb<W: GpuWeight>(self, partition: &mut [usize], weights: &[W], iter_count: usize) {
        self.run(partition, weights, iter_count)
    }
}

impl Grid<3> {
    pub fn new_3d(width: std::num::NonZeroUsize, height: std::num::NonZeroUsize,
                  depth: std::num::NonZeroUsize) -> Self {
        Self { size: [width.get(), height.get(), depth.get()] }
    }

    /// Rcb on the 3D grid (see `coupe::Grid::<3>::rcb`).
    pub fn rcb<W: GpuWeight>(self, partition: &mut [usize], weights: &[W], iter_count: usize) {
        self.run(partition, weights, iter_count)
    }
}
