//! Raw `extern "C"` bindings of `libmczi_gpu.so`, one item per declaration of
//! `include/mczi_gpu.h` in the same order and with the same types.
//!
//! Every function returns an `i32` status (`MCZI_OK` or a negative code, the
//! message from `mczi_last_error`); no panic or exception crosses the
//! boundary.  The safe wrapper that MC and ZI call is the `mczi-gpu` crate
//! next to this one.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_void};

pub const MCZI_OK: i32 = 0;
pub const MCZI_ERR_INVALID_CONFIG: i32 = -1;
pub const MCZI_ERR_IO: i32 = -2;
pub const MCZI_ERR_OOM: i32 = -3;
pub const MCZI_ERR_DEVICE: i32 = -4;
pub const MCZI_ERR_TIMEOUT: i32 = -5;
pub const MCZI_ERR_STATE: i32 = -6;
pub const MCZI_ERR_TOO_LARGE: i32 = -7;

pub const MCZI_MODE_ABUNDANCE: i32 = 0;
pub const MCZI_MODE_PRESENCE: i32 = 1;

/// `CounterConfig{k, minimizer, threshold, partition_count}` (src/lib.rs:48-53).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct mczi_counter_config {
    pub k: u32,
    pub minimizer: u32,
    pub threshold: u64,
    pub partition_count: u32,
}

/// One FASTA/FASTQ input held in host memory.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct mczi_input {
    pub data: *const u8,
    pub len: u64,
}

/// Opaque library context (one device, one stream, one host thread at a time).
#[repr(C)]
pub struct mczi_ctx {
    _private: [u8; 0],
}

/// Opaque ZI serving loop.
#[repr(C)]
pub struct mczi_server {
    _private: [u8; 0],
}

extern "C" {
    pub fn mczi_open(device: i32, out: *mut *mut mczi_ctx) -> i32;
    pub fn mczi_close(ctx: *mut mczi_ctx) -> i32;
    pub fn mczi_last_error(ctx: *const mczi_ctx) -> *const c_char;
    pub fn mczi_set_stream(ctx: *mut mczi_ctx, cuda_stream: *mut c_void) -> i32;
    pub fn mczi_validate_config(ctx: *mut mczi_ctx, cfg: *const mczi_counter_config, mode: i32) -> i32;

    // ---------------------------------------------------------------- MC
    pub fn mczi_count(ctx: *mut mczi_ctx, cfg: *const mczi_counter_config, mode: i32, inputs: *const mczi_input,
                      n_inputs: usize, n_records: *mut u64) -> i32;
    pub fn mczi_stage(ctx: *mut mczi_ctx, inputs: *const mczi_input, n_inputs: usize) -> i32;
    pub fn mczi_count_staged(ctx: *mut mczi_ctx, cfg: *const mczi_counter_config, mode: i32,
                             n_records: *mut u64) -> i32;
    pub fn mczi_result_copy(ctx: *mut mczi_ctx, key_lo: *mut u64, key_hi: *mut u64, counts: *mut u64, cap: u64,
                            sorted: i32) -> i32;
    pub fn mczi_result_digest(ctx: *mut mczi_ctx, unit_counts: i32, out: *mut u64) -> i32;
    pub fn mczi_result_write_kff(ctx: *mut mczi_ctx, path: *const c_char) -> i32;
    pub fn mczi_result_write_fasta(ctx: *mut mczi_ctx, path: *const c_char) -> i32;
    pub fn mczi_count_inputs_to_kff_path(ctx: *mut mczi_ctx, inputs: *const *const c_char, n_inputs: usize,
                                         cfg: *const mczi_counter_config, output_path: *const c_char) -> i32;
    pub fn mczi_count_inputs_to_fasta_path(ctx: *mut mczi_ctx, inputs: *const *const c_char, n_inputs: usize,
                                           cfg: *const mczi_counter_config, output_path: *const c_char) -> i32;
    pub fn mczi_count_datasets_to_kff_path(ctx: *mut mczi_ctx, inputs: *const *const c_char, n_inputs: usize,
                                           cfg: *const mczi_counter_config, output_path: *const c_char) -> i32;
    pub fn mczi_count_datasets_to_fasta_path(ctx: *mut mczi_ctx, inputs: *const *const c_char, n_inputs: usize,
                                             cfg: *const mczi_counter_config, output_path: *const c_char) -> i32;
    pub fn mczi_route_superkmers(ctx: *mut mczi_ctx, cfg: *const mczi_counter_config, inputs: *const mczi_input,
                                 n_inputs: usize, n_dest: u32, dest_bytes: *mut u64) -> i32;
    pub fn mczi_route_copy(ctx: *mut mczi_ctx, dest: u32, out: *mut u8, cap: u64) -> i32;
    pub fn mczi_phase_times(ctx: *mut mczi_ctx, ms: *mut f32, cap: i32) -> i32;
    pub fn mczi_run_stats(ctx: *mut mczi_ctx, out: *mut u64, cap: i32) -> i32;
    pub fn mczi_set_count_tuning(ctx: *mut mczi_ctx, threads: i32, table_slots: i32, ctas_per_sm: i32) -> i32;
    pub fn mczi_set_count_options(ctx: *mut mczi_ctx, chunk: i32, fill: f32) -> i32;
    pub fn mczi_set_count_filter(ctx: *mut mczi_ctx, mode: i32) -> i32;
    pub fn mczi_set_graph_replay(ctx: *mut mczi_ctx, enable: i32) -> i32;
    pub fn mczi_set_key_range_passes(ctx: *mut mczi_ctx, passes: i32) -> i32;
    pub fn mczi_set_minimizer_precount(ctx: *mut mczi_ctx, enable: i32) -> i32;
    pub fn mczi_set_streamed_staging(ctx: *mut mczi_ctx, enable: i32, segment_bytes: u64) -> i32;
    pub fn mczi_debug_packed(ctx: *mut mczi_ctx, codes: *mut u8, starts: *mut u8, cap: u64,
                             n_bases: *mut u64) -> i32;
    pub fn mczi_debug_set_bucket_window_limit(ctx: *mut mczi_ctx, windows: u64) -> i32;

    // ---------------------------------------------------------------- ZI
    pub fn mczi_zi_build(ctx: *mut mczi_ctx, index_fasta: *const u8, len: u64, k: u32, m: u32) -> i32;
    pub fn mczi_zi_query(ctx: *mut mczi_ctx, queries: *const mczi_input, n: usize, n_absent: *mut u64) -> i32;
    pub fn mczi_zi_build_from_result(ctx: *mut mczi_ctx, m: u32) -> i32;
    pub fn mczi_zi_build_path(ctx: *mut mczi_ctx, index_path: *const c_char, k: u32, m: u32) -> i32;
    pub fn mczi_zi_query_paths(ctx: *mut mczi_ctx, query_paths: *const *const c_char, n: usize,
                               n_absent: *mut u64) -> i32;
    pub fn mczi_zi_query_per_input(ctx: *mut mczi_ctx, queries: *const mczi_input, n: usize,
                                   n_records: *mut u64) -> i32;
    pub fn mczi_zi_input_result(ctx: *mut mczi_ctx, input: i32, key_lo: *mut u64, key_hi: *mut u64, cap: u64,
                                n: *mut u64) -> i32;
    pub fn mczi_zi_result_masks(ctx: *mut mczi_ctx, masks: *mut u64, cap_words: u64,
                                words_per_record: *mut i32) -> i32;
    pub fn mczi_zi_batch_split(ctx: *mut mczi_ctx, key_lo: *mut u64, key_hi: *mut u64, offsets: *mut u64, cap: u64,
                               total: *mut u64) -> i32;
    pub fn mczi_zi_info(ctx: *mut mczi_ctx, out: *mut u64, cap: i32) -> i32;
    pub fn mczi_set_zi_bucket_records(ctx: *mut mczi_ctx, records: u32) -> i32;

    // ------------------------------------------------------------ inputs
    pub fn mczi_read_input_file(path: *const c_char, data: *mut *mut u8, len: *mut u64, err: *mut c_char,
                                err_cap: u64) -> i32;
    pub fn mczi_free_input(data: *mut u8);
    pub fn mczi_compress_output(plain_path: *const c_char, output_path: *const c_char, err: *mut c_char,
                                err_cap: u64) -> i32;
    pub fn mczi_write_kmer_fasta(path: *const c_char, key_lo: *const u64, key_hi: *const u64, counts: *const u64,
                                 n: u64, k: u32, err: *mut c_char, err_cap: u64) -> i32;
    pub fn mczi_inflate_gzip(ctx: *mut mczi_ctx, gz: *const u8, len: u64, out: *mut u8, cap: u64, n_out: *mut u64)
        -> i32;

    // --------------------------------------------------------- ZI serving
    pub fn mczi_serve_open(device: i32, index_fasta: *const u8, len: u64, k: u32, m: u32, workers: i32,
                           max_batch: i32, hbm_budget: u64, out: *mut *mut mczi_server) -> i32;
    pub fn mczi_serve_submit(srv: *mut mczi_server, query_fasta: *const u8, len: u64, request_id: *mut u64) -> i32;
    pub fn mczi_serve_next(srv: *mut mczi_server, timeout_ms: i32, request_id: *mut u64, status: *mut i32,
                           n_kmers: *mut u64, latency_ms: *mut f64, queue_ms: *mut f64) -> i32;
    pub fn mczi_serve_result(srv: *mut mczi_server, request_id: u64, key_lo: *mut u64, key_hi: *mut u64, cap: u64,
                             n: *mut u64) -> i32;
    pub fn mczi_serve_release(srv: *mut mczi_server, request_id: u64) -> i32;
    pub fn mczi_serve_error(srv: *mut mczi_server, request_id: u64) -> *const c_char;
    pub fn mczi_serve_stats(srv: *mut mczi_server, out: *mut f64, cap: i32) -> i32;
    pub fn mczi_serve_close(srv: *mut mczi_server) -> i32;

    // ------------------------------------------ packing without allocation
    pub fn mczi_pack_fastx_noalloc(d_text: *const u8, text_len: u64, fastq: i32, d_packed: *mut u32,
                                   packed_words: u64, d_fbits: *mut u32, fbits_words: u64, n_bases: *mut u64,
                                   stream: *mut c_void) -> i32;
}
