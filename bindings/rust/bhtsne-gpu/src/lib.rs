//! `tSNE` on one GB300 GPU with the builder surface of bhtsne 0.7.10
//! (src/lib.rs:149-1249): the same setters, finishers, getters and panic
//! messages, over the C ABI of libbhtsne_gpu.so.
//!
//! Arbitrary metric closures stay on the host, as the C ABI cannot take them:
//! `barnes_hut` / `fit_sne` with a closure compute the neighbour table on the
//! host by brute force ordered by (distance, index), the lists the reference's
//! VP-tree returns (its tests, src/test.rs:888-928, check exactly that), and
//! hand it to the `*_with_neighbors` entry points; `exact` evaluates the
//! closure on the strict upper triangle and passes the matrix. For Euclidean
//! data, `barnes_hut_euclidean` / `fit_sne_euclidean` / `exact_euclidean` run
//! the neighbour search on the device.
//!
//! Not compiled here (no cargo or rustc on either machine).
#![allow(non_camel_case_types)]

use std::ffi::CStr;
use std::marker::PhantomData;
use std::os::raw::{c_int, c_void};

use bhtsne_gpu_sys as sys;

/// The reference's `T`: f32 or f64.
pub trait GpuFloat: Copy + Default + PartialOrd + Into<f64> + 'static {
    const DTYPE: c_int;
    fn from_f64(v: f64) -> Self;
}
impl GpuFloat for f32 {
    const DTYPE: c_int = sys::BHTSNE_F32;
    fn from_f64(v: f64) -> Self {
        v as f32
    }
}
impl GpuFloat for f64 {
    const DTYPE: c_int = sys::BHTSNE_F64;
    fn from_f64(v: f64) -> Self {
        v
    }
}

/// `Neighbor<T>` (src/lib.rs:108-111).
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct Neighbor<T> {
    pub index: usize,
    pub distance: T,
}

/// `SparseAffinities<T>` (src/lib.rs:117-144).
#[derive(Clone)]
pub struct SparseAffinities<T> {
    rows: Vec<usize>,
    columns: Vec<u32>,
    values: Vec<T>,
    perplexity: T,
}

impl<T> SparseAffinities<T> {
    pub fn rows(&self) -> &[usize] {
        &self.rows
    }
    pub fn columns(&self) -> &[u32] {
        &self.columns
    }
    pub fn values(&self) -> &[T] {
        &self.values
    }
    pub fn perplexity(&self) -> &T {
        &self.perplexity
    }
}

/// One CUDA device and stream (`bhtsne_ctx`); a builder borrows one.
pub struct Context {
    raw: *mut sys::bhtsne_ctx,
}

impl Context {
    pub fn new(device: i32) -> Context {
        let mut raw = std::ptr::null_mut();
        let rc = unsafe { sys::bhtsne_ctx_create(device, &mut raw) };
        assert!(rc == 0, "error: bhtsne_ctx_create failed with status {rc} (is a CUDA device visible?)");
        Context { raw }
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe {
            sys::bhtsne_ctx_destroy(self.raw);
        }
    }
}

thread_local! {
    static DEFAULT_CTX: Context = Context::new(0);
}

type Callback<'data, T> = Box<dyn FnMut(usize, &[T]) + 'data>;

/// The builder. `U` is the sample type of the data (for Euclidean data,
/// `&[T]`), `D` the embedding dimension: 2..7 for Barnes-Hut, 1..2 for
/// FIt-SNE, 1..7 for exact.
pub struct tSNE<'data, T: GpuFloat, U, const D: usize = 2> {
    data: &'data [U],
    raw: *mut sys::bhtsne_tsne,
    // the callback and the snapshot length, at a stable address the library holds
    callback: Option<Box<(Callback<'data, T>, usize)>>,
    perplexity: f64,
    _t: PhantomData<T>,
}

unsafe extern "C" fn trampoline<T: GpuFloat>(epoch: i64, y: *const c_void, user: *mut c_void) {
    let (cb, len) = &mut *(user as *mut (Callback<'static, T>, usize));
    let snapshot = std::slice::from_raw_parts(y as *const T, *len);
    cb(epoch as usize, snapshot);
}

impl<'data, T: GpuFloat, U, const D: usize> tSNE<'data, T, U, D> {
    /// `tSNE::new` (src/lib.rs:241-266): the reference's defaults.
    pub fn new(data: &'data [U]) -> Self {
        let mut raw = std::ptr::null_mut();
        let rc = DEFAULT_CTX.with(|c| unsafe { sys::bhtsne_tsne_new(c.raw, T::DTYPE, D as i32, data.len() as i64, &mut raw) });
        assert!(rc == 0, "error: bhtsne_tsne_new failed with status {rc}");
        tSNE { data, raw, callback: None, perplexity: 20.0, _t: PhantomData }
    }

    fn check(&self, rc: c_int) {
        if rc != 0 {
            let msg = unsafe { CStr::from_ptr(sys::bhtsne_tsne_last_error(self.raw)) }.to_string_lossy().into_owned();
            panic!("{msg}");
        }
    }

    pub fn learning_rate(&mut self, learning_rate: T) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_learning_rate(self.raw, learning_rate.into()) });
        self
    }
    pub fn epochs(&mut self, epochs: usize) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_epochs(self.raw, epochs as i64) });
        self
    }
    pub fn momentum(&mut self, momentum: T) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_momentum(self.raw, momentum.into()) });
        self
    }
    pub fn final_momentum(&mut self, final_momentum: T) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_final_momentum(self.raw, final_momentum.into()) });
        self
    }
    pub fn momentum_switch_epoch(&mut self, momentum_switch_epoch: usize) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_momentum_switch_epoch(self.raw, momentum_switch_epoch as i64) });
        self
    }
    pub fn stop_lying_epoch(&mut self, stop_lying_epoch: usize) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_stop_lying_epoch(self.raw, stop_lying_epoch as i64) });
        self
    }
    pub fn early_exaggeration(&mut self, early_exaggeration: T) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_early_exaggeration(self.raw, early_exaggeration.into()) });
        self
    }
    pub fn perplexity(&mut self, perplexity: T) -> &mut Self {
        self.check(unsafe { sys::bhtsne_tsne_perplexity(self.raw, perplexity.into()) });
        self.perplexity = perplexity.into();
        self
    }

    /// `epoch_callback` (src/lib.rs:415-422): called on this thread after
    /// every epoch with a host snapshot of the embedding.
    pub fn epoch_callback<C>(&mut self, callback: C) -> &mut Self
    where
        C: FnMut(usize, &[T]) + 'data,
    {
        let len = self.data.len() * D;
        let mut boxed: Box<(Callback<'data, T>, usize)> = Box::new((Box::new(callback), len));
        let user = &mut *boxed as *mut (Callback<'data, T>, usize) as *mut c_void;
        self.check(unsafe { sys::bhtsne_tsne_epoch_callback(self.raw, Some(trampoline::<T>), user) });
        // replaces (and drops) the previous callback only after the library points at the new one
        self.callback = Some(boxed);
        self
    }

    /// `initial_embedding` (src/lib.rs:431-435).
    pub fn initial_embedding(&mut self, embedding: impl Into<Vec<T>>) -> &mut Self {
        let y: Vec<T> = embedding.into();
        self.check(unsafe { sys::bhtsne_tsne_initial_embedding(self.raw, y.as_ptr().cast(), y.len() as i64) });
        self
    }

    /// `embedding` (src/lib.rs:438-440).
    pub fn embedding(&self) -> Vec<T> {
        let mut out = vec![T::default(); self.data.len() * D];
        self.check(unsafe { sys::bhtsne_tsne_embedding(self.raw, out.as_mut_ptr().cast()) });
        out
    }

    /// `kl_divergence` (src/lib.rs:448-477), in the reference's form (its
    /// sparse cost reads the value array by row, src/tsne/mod.rs:768-770).
    pub fn kl_divergence(&self) -> Option<T> {
        let (mut v, mut has) = (0.0f64, 0i32);
        self.check(unsafe { sys::bhtsne_tsne_kl_divergence(self.raw, 1, &mut v, &mut has) });
        (has != 0).then(|| T::from_f64(v))
    }

    /// `affinities` (src/lib.rs:1019-1037).
    pub fn affinities(&self) -> Option<SparseAffinities<T>> {
        let (mut nnz, mut perp, mut has) = (0i64, 0.0f64, 0i32);
        let null = std::ptr::null_mut();
        self.check(unsafe { sys::bhtsne_tsne_affinities(self.raw, null, null.cast(), null.cast(), &mut nnz, &mut perp, &mut has) });
        if has == 0 {
            return None;
        }
        let mut rows = vec![0u64; self.data.len() + 1];
        let mut columns = vec![0u32; nnz as usize];
        let mut values = vec![T::default(); nnz as usize];
        self.check(unsafe {
            sys::bhtsne_tsne_affinities(self.raw, rows.as_mut_ptr(), columns.as_mut_ptr(), values.as_mut_ptr().cast(),
                                        &mut nnz, &mut perp, &mut has)
        });
        Some(SparseAffinities { rows: rows.into_iter().map(|r| r as usize).collect(), columns, values,
                                perplexity: T::from_f64(perp) })
    }

    /// `with_affinities` (src/lib.rs:1043-1051).
    pub fn with_affinities(&mut self, affinities: SparseAffinities<T>) -> &mut Self {
        let rows: Vec<u64> = affinities.rows.iter().map(|&r| r as u64).collect();
        self.check(unsafe {
            sys::bhtsne_tsne_with_affinities(self.raw, rows.as_ptr(), rows.len() as i64, affinities.columns.as_ptr(),
                                             affinities.values.as_ptr().cast(), affinities.values.len() as i64,
                                             affinities.perplexity.into())
        });
        self
    }

    /// `barnes_hut_with_neighbors` (src/lib.rs:757-772).
    pub fn barnes_hut_with_neighbors(&mut self, theta: T, neighbors: &[Vec<Neighbor<T>>]) -> &mut Self {
        if !(theta.into() > 0.0) {
            // the reference rejects theta before reading the table
            self.check(unsafe { sys::bhtsne_tsne_barnes_hut_with_neighbors(self.raw, theta.into(), std::ptr::null(),
                                                                           std::ptr::null(), 0, 0) });
        }
        let (idx, dist, k) = self.flatten(neighbors);
        self.check(unsafe {
            sys::bhtsne_tsne_barnes_hut_with_neighbors(self.raw, theta.into(), idx.as_ptr(), dist.as_ptr().cast(),
                                                       neighbors.len() as i64, k as i64)
        });
        self
    }

    /// `fit_sne_with_neighbors` (src/lib.rs:884-894).
    pub fn fit_sne_with_neighbors(&mut self, neighbors: &[Vec<Neighbor<T>>]) -> &mut Self {
        let (idx, dist, k) = self.flatten(neighbors);
        self.check(unsafe {
            sys::bhtsne_tsne_fit_sne_with_neighbors(self.raw, idx.as_ptr(), dist.as_ptr().cast(), neighbors.len() as i64,
                                                    k as i64)
        });
        self
    }

    /// `barnes_hut` (src/lib.rs:701-742) with an arbitrary metric.
    pub fn barnes_hut<F>(&mut self, theta: T, metric_f: F) -> &mut Self
    where
        F: Fn(&U, &U) -> T + Send + Sync,
    {
        if self.affinities().is_some() {
            // cached affinities: the metric is not evaluated, as in the reference
            self.check(unsafe { sys::bhtsne_tsne_barnes_hut_euclidean(self.raw, theta.into(), std::ptr::null(), 0) });
            return self;
        }
        let k = self.neighbour_count();
        let table = self.host_neighbours(k, &metric_f);
        self.barnes_hut_with_neighbors(theta, &table)
    }

    /// `fit_sne` (src/lib.rs:835-871) with an arbitrary metric.
    pub fn fit_sne<F>(&mut self, metric_f: F) -> &mut Self
    where
        F: Fn(&U, &U) -> T + Send + Sync,
    {
        if self.affinities().is_some() {
            self.check(unsafe { sys::bhtsne_tsne_fit_sne_euclidean(self.raw, std::ptr::null(), 0) });
            return self;
        }
        let k = self.neighbour_count();
        let table = self.host_neighbours(k, &metric_f);
        self.fit_sne_with_neighbors(&table)
    }

    /// `exact` (src/lib.rs:489-646) with an arbitrary distance: the closure
    /// is evaluated on the strict upper triangle, as the reference does.
    pub fn exact<F: Fn(&U, &U) -> T + Send + Sync>(&mut self, distance_f: F) -> &mut Self {
        let n = self.data.len();
        let mut m = vec![T::default(); n * n];
        for i in 0..n {
            for j in (i + 1)..n {
                m[i * n + j] = distance_f(&self.data[i], &self.data[j]);
            }
        }
        self.check(unsafe { sys::bhtsne_tsne_exact_distances(self.raw, m.as_ptr().cast()) });
        self
    }

    fn neighbour_count(&self) -> usize {
        // k = 3 * perplexity, floored, as the reference sizes its search
        (3.0 * self.perplexity) as usize
    }

    fn host_neighbours<F: Fn(&U, &U) -> T>(&self, k: usize, metric_f: &F) -> Vec<Vec<Neighbor<T>>> {
        let n = self.data.len();
        let k = k.min(n.saturating_sub(1)).max(1);
        (0..n)
            .map(|i| {
                let mut row: Vec<Neighbor<T>> = (0..n)
                    .filter(|&j| j != i)
                    .map(|j| Neighbor { index: j, distance: metric_f(&self.data[i], &self.data[j]) })
                    .collect();
                row.sort_by(|a, b| {
                    a.distance.partial_cmp(&b.distance).unwrap_or(std::cmp::Ordering::Equal).then(a.index.cmp(&b.index))
                });
                row.truncate(k);
                row
            })
            .collect()
    }

    fn flatten(&self, neighbors: &[Vec<Neighbor<T>>]) -> (Vec<u64>, Vec<T>, usize) {
        let k = neighbors.first().map_or(0, Vec::len);
        assert!(k > 0 && neighbors.iter().all(|r| r.len() == k),
                "error: every neighbors row must have the same length, greater than zero.");
        let idx = neighbors.iter().flatten().map(|n| n.index as u64).collect();
        let dist = neighbors.iter().flatten().map(|n| n.distance).collect();
        (idx, dist, k)
    }
}

impl<'data, T: GpuFloat, const D: usize> tSNE<'data, T, &'data [T], D> {
    fn packed(&self) -> (Vec<T>, usize) {
        let dim = self.data.first().map_or(0, |r| r.len());
        let mut x = Vec::with_capacity(self.data.len() * dim);
        for r in self.data {
            assert_eq!(r.len(), dim, "error: every sample must have the same length.");
            x.extend_from_slice(r);
        }
        (x, dim)
    }

    /// `barnes_hut` with the Euclidean metric, its neighbour search on the device.
    pub fn barnes_hut_euclidean(&mut self, theta: T) -> &mut Self {
        let (x, dim) = self.packed();
        self.check(unsafe { sys::bhtsne_tsne_barnes_hut_euclidean(self.raw, theta.into(), x.as_ptr().cast(), dim as i32) });
        self
    }

    /// `fit_sne` with the Euclidean metric, its neighbour search on the device.
    pub fn fit_sne_euclidean(&mut self) -> &mut Self {
        let (x, dim) = self.packed();
        self.check(unsafe { sys::bhtsne_tsne_fit_sne_euclidean(self.raw, x.as_ptr().cast(), dim as i32) });
        self
    }

    /// `exact` with the Euclidean distance (`squared` false) or the squared
    /// Euclidean distance the reference's README passes (`squared` true).
    pub fn exact_euclidean(&mut self, squared: bool) -> &mut Self {
        let (x, dim) = self.packed();
        self.check(unsafe { sys::bhtsne_tsne_exact_euclidean(self.raw, x.as_ptr().cast(), dim as i32, squared as i32) });
        self
    }
}

impl<'data, T: GpuFloat, U, const D: usize> tSNE<'data, T, U, D> {
    /// `write_csv` (src/csv.rs:31-58).
    pub fn write_csv(&mut self, path: &str) -> Result<&mut Self, Box<dyn std::error::Error>> {
        let p = std::ffi::CString::new(path)?;
        let rc = unsafe { sys::bhtsne_tsne_write_csv(self.raw, p.as_ptr()) };
        if rc != 0 {
            let msg = unsafe { CStr::from_ptr(sys::bhtsne_tsne_last_error(self.raw)) }.to_string_lossy().into_owned();
            return Err(msg.into());
        }
        Ok(self)
    }
}

/// `load_csv` (src/csv.rs:61-118) for numeric fields: the reference converts
/// each field with a closure; here fields are parsed as Rust's `str::parse`.
pub fn load_csv<T: GpuFloat>(path: &str, has_headers: bool, skip: Option<&[usize]>)
                             -> Result<Vec<T>, Box<dyn std::error::Error>> {
    let p = std::ffi::CString::new(path)?;
    let skip: Vec<i64> = skip.unwrap_or(&[]).iter().map(|&c| c as i64).collect();
    let (mut count, mut records) = (0i64, 0i64);
    let call = |out: *mut c_void, count: &mut i64, records: &mut i64| unsafe {
        sys::bhtsne_load_csv(p.as_ptr(), has_headers as i32, skip.as_ptr(), skip.len() as i64, T::DTYPE, out, count,
                             records)
    };
    let fail = || -> Box<dyn std::error::Error> {
        unsafe { CStr::from_ptr(sys::bhtsne_io_last_error()) }.to_string_lossy().into_owned().into()
    };
    if call(std::ptr::null_mut(), &mut count, &mut records) != 0 {
        return Err(fail());
    }
    let mut data = vec![T::default(); count as usize];
    if call(data.as_mut_ptr().cast(), &mut count, &mut records) != 0 {
        return Err(fail());
    }
    Ok(data)
}

/// Array `name` of an .npz archive, the input of the reference's example
/// (examples/mnist_pca_tsne.rs:39-44, `NpzArchive::by_name(..).into_vec()`),
/// in C order and converted to `T`, with its shape.
pub fn load_npz<T: GpuFloat>(path: &str, name: &str) -> Result<(Vec<T>, Vec<usize>), Box<dyn std::error::Error>> {
    let p = std::ffi::CString::new(path)?;
    let nm = std::ffi::CString::new(name)?;
    let (mut count, mut ndim) = (0i64, 0i32);
    let mut shape = [0i64; 8];
    let fail = || -> Box<dyn std::error::Error> {
        unsafe { CStr::from_ptr(sys::bhtsne_io_last_error()) }.to_string_lossy().into_owned().into()
    };
    if unsafe {
        sys::bhtsne_load_npz(p.as_ptr(), nm.as_ptr(), T::DTYPE, std::ptr::null_mut(), &mut count, &mut ndim,
                             shape.as_mut_ptr())
    } != 0 {
        return Err(fail());
    }
    let mut data = vec![T::default(); count as usize];
    if unsafe {
        sys::bhtsne_load_npz(p.as_ptr(), nm.as_ptr(), T::DTYPE, data.as_mut_ptr().cast(), &mut count,
                             std::ptr::null_mut(), std::ptr::null_mut())
    } != 0 {
        return Err(fail());
    }
    let dims = shape[..(ndim as usize).min(8)].iter().map(|&v| v as usize).collect();
    Ok((data, dims))
}

impl<'data, T: GpuFloat, U, const D: usize> Drop for tSNE<'data, T, U, D> {
    fn drop(&mut self) {
        unsafe {
            sys::bhtsne_tsne_free(self.raw);
        }
    }
}
