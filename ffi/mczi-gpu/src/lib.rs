//! MC's library entry points and ZI's two seams on libmczi_gpu, with the
//! reference's signatures and `anyhow` errors, so that the bodies of
//!
//! * `count_inputs` (src/lib.rs:278), `count_datasets` (:289),
//! * `count_inputs_to_fasta_path` (:427), `count_datasets_to_fasta_path` (:442),
//! * `count_inputs_to_kff_path` (:457), `count_datasets_to_kff_path` (:509),
//! * `count_inputs_to_kmer_fasta_path` (:306), `count_datasets_to_kmer_fasta_path` (:357),
//! * `build_dictionary` (src/zi.rs:114),
//! * `collect_query_kmers_absent_from_index` (src/zi.rs:152)
//!
//! become calls into this crate and their callers (src/main.rs:88-100,
//! src/zi.rs:85-96) stay unchanged.  `CounterConfig` and `CountedKmer`
//! mirror src/lib.rs:48-66; inside the reference tree they are the crate's
//! own types.  Validation failures carry the reference's `ensure!` messages
//! (the library checks exactly src/lib.rs:110-152 and src/zi.rs:103-107).
//! Inputs may be plain, gzip, xz or zstd files: the library reads them.
//! There is no CPU fallback: without a CUDA device every call fails.
use std::collections::HashSet;
use std::ffi::{CStr, CString};
use std::os::raw::c_char;
use std::os::unix::ffi::OsStrExt;
use std::path::{Path, PathBuf};
use std::sync::{Mutex, OnceLock};

use anyhow::{bail, ensure, Result};
use mczi_gpu_sys as sys;

pub type Count = u64;
pub type EncodedKmer = u128;

#[derive(Clone, Copy, Debug)]
pub struct CounterConfig {
    pub k: usize,
    pub minimizer: usize,
    pub threshold: Count,
    pub partition_count: usize,
}

#[derive(Clone, Debug, Eq, PartialEq)]
pub struct CountedKmer {
    pub encoded: EncodedKmer,
    pub count: Count,
}

/// One library context: a CUDA device, its stream and the buffers the
/// pipeline keeps between calls.  A context serves one host thread at a
/// time, which the `Mutex` around the process-wide one enforces.
pub struct Gpu {
    ctx: *mut sys::mczi_ctx,
}

// the C ABI allows a context to move between threads as long as one thread
// uses it at a time
unsafe impl Send for Gpu {}

impl Gpu {
    pub fn open(device: i32) -> Result<Self> {
        let mut ctx = std::ptr::null_mut();
        let rc = unsafe { sys::mczi_open(device, &mut ctx) };
        ensure!(rc == sys::MCZI_OK && !ctx.is_null(), "no usable CUDA device {device} for libmczi_gpu (status {rc})");
        Ok(Gpu { ctx })
    }

    fn check(&self, rc: i32) -> Result<()> {
        if rc >= 0 {
            return Ok(());
        }
        let msg = unsafe { sys::mczi_last_error(self.ctx) };
        let text = if msg.is_null() {
            String::new()
        } else {
            unsafe { CStr::from_ptr(msg) }.to_string_lossy().into_owned()
        };
        if text.is_empty() {
            bail!("libmczi_gpu failed with status {rc}");
        }
        bail!(text)
    }

    /// The path entry points.  As the reference's (e.g. src/lib.rs:466-480),
    /// a compressed output (.gz, .gzip, .xz, .zst, .zstd) is written plain
    /// first and then compressed (compress_existing_file, src/lib.rs:1397).
    fn count_paths(&self, inputs: &[PathBuf], config: CounterConfig, output: &Path, datasets: bool,
                   kff: bool) -> Result<()> {
        if !output_compressed(output) {
            return self.count_paths_plain(inputs, config, output, datasets, kff);
        }
        let mut tmp = output.as_os_str().to_owned();
        tmp.push(".tmp-plain");
        let tmp = PathBuf::from(tmp);
        let result = self
            .count_paths_plain(inputs, config, &tmp, datasets, kff)
            .and_then(|_| compress_output(&tmp, output));
        let _ = std::fs::remove_file(&tmp);
        result
    }

    fn count_paths_plain(&self, inputs: &[PathBuf], config: CounterConfig, output: &Path, datasets: bool,
                         kff: bool) -> Result<()> {
        let cfg = c_config(&config)?;
        let (_keep, ptrs) = c_paths(inputs)?;
        let out = c_path(output)?;
        let rc = unsafe {
            match (datasets, kff) {
                (false, true) => sys::mczi_count_inputs_to_kff_path(self.ctx, ptrs.as_ptr(), ptrs.len(), &cfg, out.as_ptr()),
                (false, false) => sys::mczi_count_inputs_to_fasta_path(self.ctx, ptrs.as_ptr(), ptrs.len(), &cfg, out.as_ptr()),
                (true, true) => sys::mczi_count_datasets_to_kff_path(self.ctx, ptrs.as_ptr(), ptrs.len(), &cfg, out.as_ptr()),
                (true, false) => sys::mczi_count_datasets_to_fasta_path(self.ctx, ptrs.as_ptr(), ptrs.len(), &cfg, out.as_ptr()),
            }
        };
        self.check(rc)
    }

    /// Counts in-memory inputs (mode 0 abundance, 1 dataset presence) and
    /// returns the kept records sorted by `encoded`, as count_inputs does.
    pub fn count(&self, inputs: &[Vec<u8>], config: CounterConfig, mode: i32) -> Result<Vec<CountedKmer>> {
        let cfg = c_config(&config)?;
        let ins: Vec<sys::mczi_input> =
            inputs.iter().map(|b| sys::mczi_input { data: b.as_ptr(), len: b.len() as u64 }).collect();
        let mut n = 0u64;
        self.check(unsafe { sys::mczi_count(self.ctx, &cfg, mode, ins.as_ptr(), ins.len(), &mut n) })?;
        let len = n as usize;
        let (mut lo, mut hi, mut cnt) = (vec![0u64; len], vec![0u64; len], vec![0u64; len]);
        if len > 0 {
            self.check(unsafe {
                sys::mczi_result_copy(self.ctx, lo.as_mut_ptr(), hi.as_mut_ptr(), cnt.as_mut_ptr(), n, 1)
            })?;
        }
        Ok((0..len)
            .map(|i| CountedKmer { encoded: ((hi[i] as u128) << 64) | lo[i] as u128, count: cnt[i] })
            .collect())
    }
}

impl Drop for Gpu {
    fn drop(&mut self) {
        unsafe {
            sys::mczi_close(self.ctx);
        }
    }
}

fn shared() -> Result<&'static Mutex<Gpu>> {
    static GPU: OnceLock<Mutex<Gpu>> = OnceLock::new();
    if let Some(g) = GPU.get() {
        return Ok(g);
    }
    let g = Gpu::open(0)?;
    Ok(GPU.get_or_init(|| Mutex::new(g)))
}

fn with_gpu<T>(f: impl FnOnce(&Gpu) -> Result<T>) -> Result<T> {
    let g = shared()?;
    let guard = g.lock().map_err(|_| anyhow::anyhow!("libmczi_gpu context poisoned by a panic"))?;
    f(&guard)
}

fn c_config(c: &CounterConfig) -> Result<sys::mczi_counter_config> {
    // values beyond u32 are passed as u32::MAX so that the library's own
    // validation reports them with the reference's messages
    let narrow = |v: usize| u32::try_from(v).unwrap_or(u32::MAX);
    Ok(sys::mczi_counter_config {
        k: narrow(c.k),
        minimizer: narrow(c.minimizer),
        threshold: c.threshold,
        partition_count: narrow(c.partition_count),
    })
}

fn c_path(p: &Path) -> Result<CString> {
    CString::new(p.as_os_str().as_bytes())
        .map_err(|_| anyhow::anyhow!("path {} contains a NUL byte", p.display()))
}

fn c_paths(paths: &[PathBuf]) -> Result<(Vec<CString>, Vec<*const c_char>)> {
    let owned = paths.iter().map(|p| c_path(p)).collect::<Result<Vec<_>>>()?;
    let ptrs = owned.iter().map(|c| c.as_ptr()).collect();
    Ok((owned, ptrs))
}

fn output_compressed(path: &Path) -> bool {
    matches!(
        path.extension().and_then(|e| e.to_str()).map(str::to_ascii_lowercase).as_deref(),
        Some("gz" | "gzip" | "xz" | "zst" | "zstd")
    )
}

fn compress_output(plain: &Path, output: &Path) -> Result<()> {
    let (p, o) = (c_path(plain)?, c_path(output)?);
    let mut err = vec![0 as c_char; 1024];
    let rc = unsafe { sys::mczi_compress_output(p.as_ptr(), o.as_ptr(), err.as_mut_ptr(), err.len() as u64) };
    if rc != sys::MCZI_OK {
        let msg = unsafe { CStr::from_ptr(err.as_ptr()) }.to_string_lossy().into_owned();
        bail!(msg);
    }
    Ok(())
}

fn read_input(path: &Path) -> Result<Vec<u8>> {
    let c = c_path(path)?;
    let mut data = std::ptr::null_mut();
    let mut len = 0u64;
    let mut err = vec![0 as c_char; 1024];
    let rc = unsafe { sys::mczi_read_input_file(c.as_ptr(), &mut data, &mut len, err.as_mut_ptr(), err.len() as u64) };
    if rc != sys::MCZI_OK {
        let msg = unsafe { CStr::from_ptr(err.as_ptr()) }.to_string_lossy().into_owned();
        bail!(msg);
    }
    let out = unsafe { std::slice::from_raw_parts(data, len as usize) }.to_vec();
    unsafe { sys::mczi_free_input(data) };
    Ok(out)
}

pub fn count_inputs(inputs: &[PathBuf], config: CounterConfig) -> Result<Vec<CountedKmer>> {
    ensure!(!inputs.is_empty(), "at least one input file is required");
    let data = inputs.iter().map(|p| read_input(p)).collect::<Result<Vec<_>>>()?;
    with_gpu(|g| g.count(&data, config, sys::MCZI_MODE_ABUNDANCE))
}

pub fn count_datasets(inputs: &[PathBuf], config: CounterConfig) -> Result<Vec<CountedKmer>> {
    ensure!(!inputs.is_empty(), "at least one dataset file is required");
    let data = inputs.iter().map(|p| read_input(p)).collect::<Result<Vec<_>>>()?;
    with_gpu(|g| g.count(&data, config, sys::MCZI_MODE_PRESENCE))
}

pub fn count_inputs_to_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()> {
    with_gpu(|g| g.count_paths(inputs, config, output_path, false, false))
}

pub fn count_datasets_to_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()> {
    with_gpu(|g| g.count_paths(inputs, config, output_path, true, false))
}

pub fn count_inputs_to_kff_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()> {
    with_gpu(|g| g.count_paths(inputs, config, output_path, false, true))
}

pub fn count_datasets_to_kff_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()> {
    with_gpu(|g| g.count_paths(inputs, config, output_path, true, true))
}

/// The selected-k-mer FASTA (src/lib.rs:306-311): every kept k-mer as
/// ">MC_kmer_<i> count=<c>" and its bases, in ascending `encoded` order;
/// returns the number written.  The `_with_stats` / `_silent_stats` forms
/// (:314-425, MCZI's index step at src/mczi.rs:340-344) keep their phase
/// bookkeeping and take `selected_kmers` from here.
pub fn count_inputs_to_kmer_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<u64> {
    write_kmer_fasta(&count_inputs(inputs, config)?, config.k, output_path)
}

/// count_datasets_to_kmer_fasta_path (src/lib.rs:357-363): as above with the
/// number of datasets containing each k-mer as its count.
pub fn count_datasets_to_kmer_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<u64> {
    write_kmer_fasta(&count_datasets(inputs, config)?, config.k, output_path)
}

fn write_kmer_fasta(records: &[CountedKmer], k: usize, output: &Path) -> Result<u64> {
    let out = c_path(output)?;
    let lo: Vec<u64> = records.iter().map(|r| r.encoded as u64).collect();
    let hi: Vec<u64> = records.iter().map(|r| (r.encoded >> 64) as u64).collect();
    let cnt: Vec<u64> = records.iter().map(|r| r.count).collect();
    let mut err = vec![0 as c_char; 1024];
    let rc = unsafe {
        sys::mczi_write_kmer_fasta(out.as_ptr(), lo.as_ptr(), hi.as_ptr(), cnt.as_ptr(), lo.len() as u64,
                                   u32::try_from(k).unwrap_or(u32::MAX), err.as_mut_ptr(), err.len() as u64)
    };
    if rc != sys::MCZI_OK {
        let msg = unsafe { CStr::from_ptr(err.as_ptr()) }.to_string_lossy().into_owned();
        if msg.is_empty() {
            bail!("libmczi_gpu failed with status {rc}");
        }
        bail!(msg);
    }
    Ok(records.len() as u64)
}

/// ZI's dictionary, resident on the device in its own context.
pub struct Dictionary {
    gpu: Mutex<Gpu>,
    k: usize,
}

impl Dictionary {
    pub fn k(&self) -> usize {
        self.k
    }
}

/// build_dictionary (src/zi.rs:114): `threads`, `ram_limit_gib` and
/// `tmp_dir` configure sshash-lib's CPU builder and have no role here; they
/// stay in the signature so the caller does not change.
pub fn build_dictionary(index_path: &Path, k: usize, m: usize, _threads: usize, _ram_limit_gib: usize,
                        _tmp_dir: &Path) -> Result<Dictionary> {
    let gpu = Gpu::open(0)?;
    let p = c_path(index_path)?;
    let narrow = |v: usize| u32::try_from(v).unwrap_or(u32::MAX);
    gpu.check(unsafe { sys::mczi_zi_build_path(gpu.ctx, p.as_ptr(), narrow(k), narrow(m)) })?;
    Ok(Dictionary { gpu: Mutex::new(gpu), k })
}

/// collect_query_kmers_absent_from_index (src/zi.rs:152): the distinct
/// canonical query k-mers absent from the index, MC-encoded.
pub fn collect_query_kmers_absent_from_index(dictionary: &Dictionary, query_inputs: &[PathBuf])
    -> Result<HashSet<EncodedKmer>> {
    let gpu = dictionary.gpu.lock().map_err(|_| anyhow::anyhow!("dictionary context poisoned by a panic"))?;
    let (_keep, ptrs) = c_paths(query_inputs)?;
    let mut n = 0u64;
    gpu.check(unsafe { sys::mczi_zi_query_paths(gpu.ctx, ptrs.as_ptr(), ptrs.len(), &mut n) })?;
    let len = n as usize;
    let (mut lo, mut hi) = (vec![0u64; len], vec![0u64; len]);
    if len > 0 {
        gpu.check(unsafe {
            sys::mczi_result_copy(gpu.ctx, lo.as_mut_ptr(), hi.as_mut_ptr(), std::ptr::null_mut(), n, 0)
        })?;
    }
    Ok((0..len).map(|i| ((hi[i] as u128) << 64) | lo[i] as u128).collect())
}
