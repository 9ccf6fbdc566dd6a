/*
 * mczi_gpu.h -- C ABI of libmczi_gpu, the GB300 (sm_103a) implementation of
 * the MC / ZI k-mer hot path.
 *
 * Conventions
 *  - Every call returns an int32_t status: MCZI_OK (0) or a negative code; the
 *    message of the last failure is available from mczi_last_error(ctx).  No
 *    C++ exception and no abort crosses this boundary.
 *  - The library owns device memory; the caller owns host buffers.  Results
 *    are kept in the context until the next run and copied out with the
 *    *_copy calls (call with NULL pointers or query the size first).
 *  - One context is bound to one CUDA device, one stream and one host thread
 *    at a time; several contexts may coexist.
 *  - There is no CPU fallback: if the device or the kernels are unavailable
 *    the call fails with MCZI_ERR_DEVICE.
 *
 * Reference interfaces (paths inside the MCZI project) each entry replaces
 * are cited on the declarations.
 */
#ifndef MCZI_GPU_H
#define MCZI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCZI_OK 0
#define MCZI_ERR_INVALID_CONFIG (-1) /* the reference's `ensure!` failures, same messages */
#define MCZI_ERR_IO (-2)             /* file open/read/write failure */
#define MCZI_ERR_OOM (-3)            /* not enough free HBM for the request */
#define MCZI_ERR_DEVICE (-4)         /* CUDA error or kernels unavailable */
#define MCZI_ERR_TIMEOUT (-5)        /* a bounded device-side wait gave up */
#define MCZI_ERR_STATE (-6)          /* call out of order (e.g. no result yet) */
#define MCZI_ERR_TOO_LARGE (-7)      /* input beyond a fixed maximum (mczi_pack_fastx_noalloc) */

#define MCZI_MODE_ABUNDANCE 0 /* count every occurrence */
#define MCZI_MODE_PRESENCE 1  /* fof: count each dataset (input) at most once */

/* CounterConfig{k, minimizer, threshold, partition_count}, src/lib.rs:48-53.
 * partition_count only shapes the reference's temporary files; it is
 * validated (> 0) and otherwise has no effect on results, as in MC. */
typedef struct {
  uint32_t k;
  uint32_t minimizer;
  uint64_t threshold;
  uint32_t partition_count;
} mczi_counter_config;

/* One FASTA/FASTQ input held in host memory.  The entry points that take an
 * array of them (mczi_count, mczi_stage, mczi_route_superkmers, mczi_zi_query,
 * mczi_zi_query_per_input) accept each plain or compressed (gzip, xz, zstd,
 * recognised by their magic bytes): BGZF gzip is decoded on the device, the
 * rest on the host. */
typedef struct {
  const uint8_t* data;
  uint64_t len;
} mczi_input;

typedef struct mczi_ctx mczi_ctx;

/* Opens a context on CUDA device `device`. */
int32_t mczi_open(int32_t device, mczi_ctx** out);
int32_t mczi_close(mczi_ctx* ctx);
const char* mczi_last_error(const mczi_ctx* ctx);
/* Makes the context enqueue its work on `cuda_stream` (a cudaStream_t; NULL
 * restores the context's own stream). */
int32_t mczi_set_stream(mczi_ctx* ctx, void* cuda_stream);

/* Validation exactly as MC: validate_config (src/lib.rs:110-116, shape checks
 * :119-139) for mode 0, validate_dataset_presence_config (:141-152) for mode 1. */
int32_t mczi_validate_config(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode);

/* ---------------------------------------------------------------- MC */

/* count_inputs (src/lib.rs:278) / count_datasets (src/lib.rs:289): counts the
 * canonical k-mers of `inputs` and keeps those with count > threshold.
 * Mode 0 counts occurrences (exact counts); mode 1 counts the inputs
 * (datasets) containing each k-mer (fof, k <= 32).  Inputs may be plain or
 * compressed (gzip, xz, zstd, recognised by their magic bytes): gzip whose
 * members carry their sizes (BGZF) is decoded on the device, the rest on the
 * host.  Inputs that do not start with a FASTA/FASTQ record are skipped with
 * an MC_WARN line, like src/lib.rs:3371-3392.  *n_records receives the number
 * of kept k-mers. */
int32_t mczi_count(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode, const mczi_input* inputs,
                   size_t n_inputs, uint64_t* n_records);

/* Split form of mczi_count for callers that keep the inputs resident:
 * mczi_stage copies the inputs to HBM (host->device), mczi_count_staged runs
 * the device pipeline on the staged bytes. */
int32_t mczi_stage(mczi_ctx* ctx, const mczi_input* inputs, size_t n_inputs);
int32_t mczi_count_staged(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode, uint64_t* n_records);

/* Copies the kept records of the last count.  key_hi may be NULL for k <= 32.
 * sorted != 0 sorts by canonical k-mer (the order of count_inputs). */
int32_t mczi_result_copy(mczi_ctx* ctx, uint64_t* key_lo, uint64_t* key_hi, uint64_t* counts, uint64_t cap,
                         int32_t sorted);

/* Order-independent digest of the last result's records, computed on the
 * device (no reference counterpart: a check for comparing a large result with
 * one computed elsewhere without moving the records).  out[0] = records,
 * out[1] = sum of counts, out[2] = wrapping sum and out[3] = xor over the
 * records of mix(mix(mix(lo) ^ hi) + count), mix = the murmur3 64-bit
 * finaliser, hi = 0 for k <= 32; unit_counts != 0 digests every count as 1
 * (a ZI absent set compared as a set). */
int32_t mczi_result_digest(mczi_ctx* ctx, int32_t unit_counts, uint64_t* out);

/* KFF file of the last count (src/lib.rs:1633-1670, 3071-3121): count bytes 1
 * (mode 0, k <= 32, counts saturated at min(x+1, 255)), 8 (mode 0, k > 32) or
 * 4 (mode 1), as MC's count_inputs_to_kff_path / count_datasets_to_kff_path. */
int32_t mczi_result_write_kff(mczi_ctx* ctx, const char* path);
/* Greedy simplitig FASTA of the last count (src/lib.rs:1469-1533), as
 * count_inputs_to_fasta_path / count_datasets_to_fasta_path. */
int32_t mczi_result_write_fasta(mczi_ctx* ctx, const char* path);

/* Path-based drop-ins for the MC library entry points.  The files are
 * FASTA/FASTQ, plain or gzip / xz / zstd compressed (recognised by their
 * magic bytes, decoded with the system's zlib / liblzma / libzstd loaded at
 * run time, several files on parallel host threads), as MC reads them
 * (src/lib.rs:3127-3143, 3218-3226):
 *   count_inputs_to_kff_path   src/lib.rs:457
 *   count_inputs_to_fasta_path src/lib.rs:427
 *   count_datasets_to_kff_path src/lib.rs:509
 *   count_datasets_to_fasta_path src/lib.rs:442  */
int32_t mczi_count_inputs_to_kff_path(mczi_ctx* ctx, const char* const* inputs, size_t n_inputs,
                                      const mczi_counter_config* cfg, const char* output_path);
int32_t mczi_count_inputs_to_fasta_path(mczi_ctx* ctx, const char* const* inputs, size_t n_inputs,
                                        const mczi_counter_config* cfg, const char* output_path);
int32_t mczi_count_datasets_to_kff_path(mczi_ctx* ctx, const char* const* inputs, size_t n_inputs,
                                        const mczi_counter_config* cfg, const char* output_path);
int32_t mczi_count_datasets_to_fasta_path(mczi_ctx* ctx, const char* const* inputs, size_t n_inputs,
                                          const mczi_counter_config* cfg, const char* output_path);

/* The local step of counting on several GPUs (the reference's counterpart
 * is its partition files: src/lib.rs:4821-4925 writes each superkmer to
 * partition_NNNN.skm by minimizer, src/lib.rs:2803-2845).  Packs and scans
 * this GPU's share of the reads and groups every superkmer by destination
 * GPU d = (minimizer bucket) mod n_dest, n_dest <= 1024, as one-line FASTA
 * records of its windows + k - 1 bases; dest_bytes[d] receives each group's
 * size.  The groups stay in the context until the next routing and are
 * copied out with mczi_route_copy.  Each GPU then counts the records it
 * received (mczi_count): every k-mer occurrence lies in exactly one
 * superkmer and a canonical k-mer's superkmers share one minimizer, so the
 * union of the GPUs' results equals one GPU's result on all the reads. */
int32_t mczi_route_superkmers(mczi_ctx* ctx, const mczi_counter_config* cfg, const mczi_input* inputs,
                              size_t n_inputs, uint32_t n_dest, uint64_t* dest_bytes);
int32_t mczi_route_copy(mczi_ctx* ctx, uint32_t dest, uint8_t* out, uint64_t cap);

/* Per-phase device times (ms) of the last run, measured with CUDA events on
 * the context's stream: [0] pack, [1] minimizer scan, [2] partition,
 * [3] k-mer counting, [4] minimizer pre-count (0 when not run).  After a
 * streamed mczi_count, [0] spans the overlapped staging + pack + scan and
 * [1] only a rescan, if one was needed.  After a ZI query: [0] pack, [1] scan,
 * [2] partition of the absent windows, [3] their deduplication, [4] probe; a
 * query of at least 64 MiB of text is streamed like mczi_count ([0] then
 * spans staging + pack + scan).  [5]: the device gzip decoding of the last
 * call that decoded gzip members on the device (mczi_inflate_gzip, or inputs
 * staged compressed), 0 before any.  Returns the number of phases written. */
int32_t mczi_phase_times(mczi_ctx* ctx, float* ms, int32_t cap);
/* Statistics of the last run: [0] bases, [1] superkmers, [2] counting rounds,
 * [3] round splits, [4] distinct k-mers inserted, [5] kept records,
 * [6] k-mer windows, [7] skipped inputs, [8] kernel launches of the last
 * count, [9] host-to-device input bytes of the last staging.  After a ZI
 * query: [1] absent runs, [2] query superkmers, [6] absent windows. */
int32_t mczi_run_stats(mczi_ctx* ctx, uint64_t* out, int32_t cap);

/* Tuning knobs (results never depend on them): threads per counting CTA,
 * table slots per CTA (0 = largest that fits), CTAs per SM; 0 selects the
 * built-in default for the key width. */
int32_t mczi_set_count_tuning(mczi_ctx* ctx, int32_t threads, int32_t table_slots, int32_t ctas_per_sm);
/* Windows per work item of the counting insert phase (0 = default: 4 for
 * k > 32, else 2) and the target fill of a counting round's table (0 =
 * default: 0.8 for two-pass filtered rounds, 0.6 otherwise; at most 0.85). */
int32_t mczi_set_count_options(mczi_ctx* ctx, int32_t chunk, float fill);

/* Counting rounds for threshold >= 1: 1 uses two passes over a shared-memory
 * bitmap so that k-mers seen once are never stored; 0 uses one claim-or-count
 * pass; -1 (default) picks two passes for k > 32.  Results are identical. */
int32_t mczi_set_count_filter(mczi_ctx* ctx, int32_t mode);

/* CUDA-graph replay of the counting pipeline.  When enabled, a count runs the
 * plain path once and captures its launches; later counts of staged inputs
 * with the same layout and configuration replay the graph (one launch, no
 * host synchronisation between phases) and fall back to the plain path --
 * and recapture -- if the inputs outgrow the captured buffer sizes.  With the
 * graph, mczi_phase_times reports the whole device time as the counting
 * phase.  Off by default; not used with the minimizer pre-count. */
int32_t mczi_set_graph_replay(mczi_ctx* ctx, int32_t enable);

/* Inputs with more superkmers than one pass holds are counted in passes over
 * disjoint ranges of the minimizer key (each pass rescans the packed stream).
 * 0 (default) picks the number from the input size and free HBM; 1..64 forces
 * it.  Results are identical. */
int32_t mczi_set_key_range_passes(mczi_ctx* ctx, int32_t passes);

/* Pass-1 minimizer pre-count (MC's CompactMinimizerTable / DatasetMinimizerTable,
 * src/lib.rs:4171-4370, filter :4625-4629): when enabled, superkmers whose
 * minimizer count (windows, or datasets in fof mode) is <= threshold are dropped
 * before counting.  The filter is conservative, so results are identical with
 * it on or off; it only changes the work done.  Default off. */
int32_t mczi_set_minimizer_precount(mczi_ctx* ctx, int32_t enable);

/* Streamed staging of mczi_count (no reference counterpart: MC reads its
 * inputs from files): the input bytes are copied to the device in segments
 * while earlier segments are packed and scanned.  enable 0 stages everything
 * first; segment_bytes (a multiple of 8192) sets the segment size, 0 =
 * automatic (>= 32 MiB, about 16 segments).  Results are identical either way.
 * Default on.  Batches estimated (from their text length) to need more than
 * two key-range passes, counts with the pre-count, and graph replay always
 * stage first; a streamed batch that overflows one pass is recounted through
 * the staged path. */
int32_t mczi_set_streamed_staging(mczi_ctx* ctx, int32_t enable, uint64_t segment_bytes);

/* Packer parity hook: after mczi_count/mczi_count_staged, copies the 2-bit
 * codes (one byte per base) and fragment-start flags (one byte per base) of
 * the packed stream; *n_bases receives the base count. */
int32_t mczi_debug_packed(mczi_ctx* ctx, uint8_t* codes, uint8_t* starts, uint64_t cap, uint64_t* n_bases);

/* Test hook (no reference counterpart): the counting kernel keeps per-bin
 * occupancies, their prefix and per-k-mer counts in 32-bit counters, each
 * bounded by the k-mer windows of one minimizer bucket; a bucket with more
 * than 2^32 - 1 windows makes the count fail with MCZI_ERR_TOO_LARGE instead
 * of wrapping.  This lowers that limit (0 restores 2^32 - 1) so the error
 * path can be exercised on small inputs. */
int32_t mczi_debug_set_bucket_window_limit(mczi_ctx* ctx, uint64_t windows);

/* ---------------------------------------------------------------- ZI */

/* build_dictionary (src/zi.rs:114-141): indexes the canonical k-mers of the
 * index FASTA (fragments of length >= k) in a device-resident dictionary --
 * the 2-bit index stream, its superkmers bucketed by minimizer, a BBHash-style
 * minimal perfect hash of the minimizers and the bucket offsets -- which
 * stays on the device until the next build or mczi_close.  k odd in [3, 63],
 * 0 < m < k (validate_k, src/zi.rs:103-107). */
int32_t mczi_zi_build(mczi_ctx* ctx, const uint8_t* index_fasta, uint64_t len, uint32_t k, uint32_t m);

/* collect_query_kmers_absent_from_index (src/zi.rs:152-175): the distinct
 * canonical k-mers of the queries (fragments of length >= k) absent from the
 * index.  They become the context's result: mczi_result_copy gives them
 * (counts are the number of absent occurrences), mczi_result_write_fasta
 * writes them as simplitigs like write_novel_simplitigs (src/zi.rs:177-189). */
int32_t mczi_zi_query(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_absent);

/* The dictionary of the last count's kept k-mers, built on the device
 * without leaving it (MCZI's orchestration, src/mczi.rs:340-360, writes MC's
 * k-mers to FASTA, compacts them with GGCAT and indexes the simplitigs; the
 * k-mer set is the same).  Each kept k-mer becomes its own index sequence;
 * k is the count's, odd in [3, 63], and 0 < m < k (validate_k,
 * src/zi.rs:103-107).  The count's result and staged inputs are consumed. */
int32_t mczi_zi_build_from_result(mczi_ctx* ctx, uint32_t m);

/* Path-based forms of the two ZI seams (build_dictionary src/zi.rs:114 and
 * collect_query_kmers_absent_from_index src/zi.rs:152, whose callers pass
 * paths, src/zi.rs:85-96): the files are plain or gzip / xz / zstd
 * compressed FASTA, read as the MC path-based entry points read them. */
int32_t mczi_zi_build_path(mczi_ctx* ctx, const char* index_path, uint32_t k, uint32_t m);
int32_t mczi_zi_query_paths(mczi_ctx* ctx, const char* const* query_paths, size_t n, uint64_t* n_absent);

/* The same for a batch of independent requests (one input each) in one set
 * of launches: each absent k-mer carries the set of inputs it is absent
 * from; mczi_zi_input_result extracts one input's sorted absent set, which is
 * identical to what that input gives when queried alone. */
int32_t mczi_zi_query_per_input(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_records);
int32_t mczi_zi_input_result(mczi_ctx* ctx, int32_t input, uint64_t* key_lo, uint64_t* key_hi, uint64_t cap,
                             uint64_t* n);

/* The per-input masks of the last mczi_zi_query_per_input, in the record order
 * of mczi_result_copy(..., sorted = 0): *words_per_record words per record,
 * bit i set when the k-mer is absent for input i. */
int32_t mczi_zi_result_masks(mczi_ctx* ctx, uint64_t* masks, uint64_t cap_words, int32_t* words_per_record);

/* All inputs' absent sets of the last mczi_zi_query_per_input in one pass:
 * input i's k-mers are key_lo/key_hi[offsets[i] .. offsets[i + 1]) (a set,
 * in no particular order, like ZI's AHashSet).  offsets holds n_inputs + 1
 * entries; call with key_lo == NULL to get *total first. */
int32_t mczi_zi_batch_split(mczi_ctx* ctx, uint64_t* key_lo, uint64_t* key_hi, uint64_t* offsets, uint64_t cap,
                            uint64_t* total);

/* Index description: [0] built, [1] k, [2] m, [3] index bases, [4] superkmers,
 * [5] distinct minimizers (MPHF keys), [6] MPHF levels, [7] build time (us). */
int32_t mczi_zi_info(mczi_ctx* ctx, uint64_t* out, int32_t cap);

/* Records per final bucket of the ZI deduplication (no reference counterpart:
 * a sizing knob of this library).  The absent windows are partitioned by
 * k-mer hash into 2^b <= 131072 buckets of about `records` each, in one level
 * of <= 256 buckets or two; 0 = automatic (half the shared-memory table).
 * Smaller values only add partition work; results are identical. */
int32_t mczi_set_zi_bucket_records(mczi_ctx* ctx, uint32_t records);

/* Reads one FASTA/FASTQ file as the path-based entry points do (plain, or
 * gzip / xz / zstd decoded on the host; no reference counterpart beyond its
 * readers, src/lib.rs:3127-3143): *data receives a buffer of *len bytes
 * allocated by the library, released with mczi_free_input.  On failure
 * (MCZI_ERR_IO: unreadable file, corrupt stream, or the decoding library
 * missing) the message is written to err (err_cap bytes, may be NULL). */
int32_t mczi_read_input_file(const char* path, uint8_t** data, uint64_t* len, char* err, uint64_t err_cap);
void mczi_free_input(uint8_t* data);

/* compress_existing_file (src/lib.rs:1397-1405) with MC's output writer
 * (src/lib.rs:1355-1395): writes the bytes of plain_path to output_path,
 * compressed as output_path's extension says (.gz / .gzip: gzip at level 1;
 * .xz: xz preset 6; .zst / .zstd: zstd level 1; case-insensitive), or as
 * they are for any other extension.  The reference's path entry points write
 * a compressed output this way (a plain file first, then this step, e.g.
 * src/lib.rs:466-480); the ones here write the plain file, so a caller
 * wanting the reference's behaviour adds this step (the Rust crate does).
 * Host only, no context; the codecs are the system's zlib / liblzma /
 * libzstd loaded at run time.  MCZI_ERR_IO with the message in err (err_cap
 * bytes, may be NULL) on an unreadable input, a missing codec or a write
 * failure. */
int32_t mczi_compress_output(const char* plain_path, const char* output_path, char* err, uint64_t err_cap);

/* The selected-k-mer FASTA of count_inputs_to_kmer_fasta_path /
 * count_datasets_to_kmer_fasta_path (src/lib.rs:306-425, records as
 * write_kmer_fasta_record_u128, src/lib.rs:1535-1544; MCZI writes its index
 * set this way, src/mczi.rs:340-344): record i (from 1) is
 * ">MC_kmer_<i> count=<counts[i-1]>" followed by the k-mer's k bases on one
 * line (MSB-first, A0 C1 G2 T3; 1 <= k <= 64).  Host memory only, no
 * context: pass the records copied with mczi_result_copy (sorted = 1 gives
 * ascending encoded order; the reference writes them in its partition
 * order).  key_hi may be NULL for k <= 32.  Returns MCZI_ERR_IO with the
 * message in err (err_cap bytes, may be NULL) when the file cannot be
 * written. */
int32_t mczi_write_kmer_fasta(const char* path, const uint64_t* key_lo, const uint64_t* key_hi,
                              const uint64_t* counts, uint64_t n, uint32_t k, char* err, uint64_t err_cap);

/* Decodes on the device a gzip buffer whose members carry their sizes (BGZF:
 * the "BC" extra subfield), one warp per member, each member checked against
 * its ISIZE and CRC-32, and copies the bytes to out (cap bytes; *n_out gets
 * the decoded length, also when out is too small).  The counting and ZI
 * entry points take such inputs compressed (and the path-based ones keep such
 * files compressed) and decode them this way in HBM; other gzip, xz and zstd
 * inputs are decoded on the host.  The decompression the reference runs in
 * front of its FASTX parser: src/lib.rs:3127-3143.  Errors:
 * MCZI_ERR_INVALID_CONFIG (not such a buffer), MCZI_ERR_TOO_LARGE (out too
 * small), MCZI_ERR_IO (a member is not valid DEFLATE or fails its checks). */
int32_t mczi_inflate_gzip(mczi_ctx* ctx, const uint8_t* gz, uint64_t len, uint8_t* out, uint64_t cap,
                          uint64_t* n_out);

/* ------------------------------------------------------------- ZI serving */

/* A resident ZI dictionary answering subtraction requests with continuous
 * batching (no counterpart in the reference: ZI is a one-shot CLI,
 * src/zi.rs:64-101).  `workers` host threads each own a context (its own
 * stream and buffers) holding the dictionary of `index_fasta`, built at open
 * (src/zi.rs:114-141 semantics).  Whenever a worker is idle it takes every
 * waiting request that fits -- at most `max_batch` requests and at most its
 * share of `hbm_budget` bytes of device memory (0 = 60 % of the free memory
 * at open), estimated at 8 device bytes per query byte; a larger request runs
 * alone -- and answers them with one mczi_zi_query_per_input, so each request
 * gets exactly the absent set it gets alone.  Batches of different workers
 * overlap on the device. */
typedef struct mczi_server mczi_server;

int32_t mczi_serve_open(int32_t device, const uint8_t* index_fasta, uint64_t len, uint32_t k, uint32_t m,
                        int32_t workers, int32_t max_batch, uint64_t hbm_budget, mczi_server** out);

/* Queues one query FASTA.  The bytes are not copied: they must stay valid and
 * unchanged until mczi_serve_next has reported the request. */
int32_t mczi_serve_submit(mczi_server* srv, const uint8_t* query_fasta, uint64_t len, uint64_t* request_id);

/* Waits up to timeout_ms (< 0: no limit) for the next finished request and
 * reports its id, its status (MCZI_OK or the failing call's code), the size of
 * its absent set, its latency (submit to result) and its time in the queue.
 * Returns MCZI_ERR_TIMEOUT when none finished in time. */
int32_t mczi_serve_next(mczi_server* srv, int32_t timeout_ms, uint64_t* request_id, int32_t* status,
                        uint64_t* n_kmers, double* latency_ms, double* queue_ms);

/* Copies a reported request's absent canonical k-mers (a set, in no
 * particular order; key_hi may be NULL for k <= 32) and releases the request.
 * With key_lo == NULL only *n is set and the request is kept.  A failed
 * request returns its status (and is released when key_lo is not NULL);
 * mczi_serve_error gives its message until then. */
int32_t mczi_serve_result(mczi_server* srv, uint64_t request_id, uint64_t* key_lo, uint64_t* key_hi, uint64_t cap,
                          uint64_t* n);
/* Releases a reported request without copying its absent set (a client that
 * needs only the size from mczi_serve_next); returns the request's status. */
int32_t mczi_serve_release(mczi_server* srv, uint64_t request_id);
/* mczi_serve_error(NULL, 0) gives the message of this thread's last failed
 * mczi_serve_open. */
const char* mczi_serve_error(mczi_server* srv, uint64_t request_id);

/* Counters: [0] batches, [1] requests answered, [2] largest batch, [3] seconds
 * in mczi_zi_query_per_input, [4] seconds splitting batch results, [5]
 * requests waiting, [6] admitted query bytes per worker.  Returns the number
 * written. */
int32_t mczi_serve_stats(mczi_server* srv, double* out, int32_t cap);

/* Stops accepting requests, lets the workers finish the queued ones, joins
 * them and frees everything (results not yet copied are dropped).  No other
 * call on the same server may run during or after it: stop the thread that
 * waits in mczi_serve_next first. */
int32_t mczi_serve_close(mczi_server* srv);

/* ------------------------------------------------ packing without allocation */

/* The 2-bit packer of mczi_count's first phase, for callers that cannot
 * allocate device memory where they call it: services that give out device
 * memory only from their own pre-sized arena (an allocation behind the
 * arena's back breaks its accounting and fails once the arena holds the free
 * HBM), or latency-critical paths where a cudaMalloc (and the
 * synchronisation it may cause) is not allowed.  This entry point has no
 * counterpart in the reference; it allocates nothing and calls no allocating
 * routine.
 *
 * Inputs and outputs are the caller's device buffers: `d_text` holds one
 * FASTA (fastq = 0) or four-line FASTQ (fastq = 1) input of `text_len` bytes,
 * padded with '\n' to a multiple of 8192 bytes; at most 512 MiB
 * (65,536 tiles of 8192 bytes) -- larger inputs return MCZI_ERR_TOO_LARGE.
 * `d_packed` (>= text_len/16 + 8 words) receives the bases, 16 per word,
 * MSB-first, A0 C1 G2 T3; `d_fbits` (>= text_len/32 + 8 words) one bit per
 * base, set where a fragment (a maximal A/C/G/T run of one record) starts.
 * Both are cleared by the call.  *n_bases (host) receives the base count: the
 * call copies it from the device and synchronises `stream` before returning.
 *
 * Scratch: an 8 MiB array in device memory, part of this library's CUDA
 * module, reserved on a device when the module loads there (at library load
 * with eager module loading; at the first use on that device, normally the
 * first call, with lazy loading) and held until the process exits.  The first
 * call on a device looks its address up (cudaGetSymbolAddress) with that
 * device current and keeps it for the life of the device's primary context
 * (do not call again on a device after cudaDeviceReset); that first lookup
 * may itself load the module on the device.  Every call shares the array, so calls that
 * overlap on the GPU race: issue them one at a time. */
int32_t mczi_pack_fastx_noalloc(const uint8_t* d_text, uint64_t text_len, int32_t fastq, uint32_t* d_packed,
                                uint64_t packed_words, uint32_t* d_fbits, uint64_t fbits_words, uint64_t* n_bases,
                                void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MCZI_GPU_H */
