/*
 * esperanto_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * ESPERANTO read-alignment inner loop.
 *
 * The entry points mirror the reference's Rust functions one for one (each
 * declaration cites the function it replaces, by path:line within the
 * reference project) so that a thin FFI shim can keep the reference's
 * signatures.  Everything is plain C: pointers, sizes and PODs; no CUDA or
 * PyTorch types cross the boundary.  Streams are passed as `void *`
 * (a cudaStream_t, NULL = the handle's own stream).
 *
 * Conventions
 *   - Return value: ESP_OK (0) or a negative ESP_E* status.  The reference's
 *     functions are infallible; a nonzero status here means a CUDA error, a
 *     full output buffer, or an argument outside the supported domain.
 *   - Sequences at the per-call entry points are ASCII bytes exactly as the
 *     reference receives them (`&[u8]`); bases are folded by the reference's
 *     base_code (A/a=0 C/c=1 G/g=2 T/t=3, anything else 4).
 *   - CIGAR ops are u32 `(len << 4) | code` with code M=0 I=1 D=2 N=3 S=4.
 *   - Handles are not thread-safe; use one handle per host thread (the
 *     reference keeps one ExtendBuffer per rayon worker).
 */
#ifndef ESPERANTO_GB300_H
#define ESPERANTO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ESP_OK 0
#define ESP_EINVAL (-1)   /* bad argument                                    */
#define ESP_ECUDA (-2)    /* CUDA runtime error (see esp_last_error)         */
#define ESP_ECAP (-3)     /* CIGAR output buffer too small                   */
#define ESP_EDOMAIN (-4)  /* parameters outside the device kernels' domain   */
#define ESP_ENOMEM (-5)   /* device or host allocation failed                */
#define ESP_EBUSY (-6)    /* admission refused (serve loop over budget)      */
#define ESP_ETIMEOUT (-7) /* bounded wait expired                            */
#define ESP_ECLOSED (-8)  /* queue closed                                    */
#define ESP_ESCRATCH (-9) /* work too large for the fixed no-allocation scratch */
#define ESP_EFORMAT (-10) /* malformed index file (AlignError::IndexFormat)  */
#define ESP_EVERSION (-11) /* unsupported index version (AlignError::IndexVersion) */

#define ESP_OP_M 0
#define ESP_OP_I 1
#define ESP_OP_D 2
#define ESP_OP_N 3
#define ESP_OP_S 4

#define ESP_EDIT_OFF 0 /* EditDir::Off */
#define ESP_EDIT_AG 1  /* EditDir::Ag  */
#define ESP_EDIT_TC 2  /* EditDir::Tc  */

typedef struct esp_handle esp_handle;

/* crates/map/src/extend.rs:97-122 ExtendParams */
typedef struct {
    int32_t match_score; /* reward, e.g. 2                 */
    int32_t mismatch;    /* stored negative, e.g. -4        */
    int32_t gap_open;    /* stored positive, e.g. 4         */
    int32_t gap_ext;     /* stored positive, e.g. 2         */
    int32_t edit_dir;    /* ESP_EDIT_*                      */
} esp_extend_params;

/* crates/map/src/extend.rs:200-229 Extension + TouchRec (the CIGAR goes to a
 * separate caller buffer). */
typedef struct {
    uint32_t read_start;
    uint32_t read_end;
    uint32_t ref_start;
    int32_t score;
    uint32_t n_ops;      /* full CIGAR length, even when larger than the buffer */
    int32_t touch_row;   /* TouchRec.row (0 when untouched)                     */
    uint8_t touched;     /* TouchRec.touched                                    */
    uint8_t touch_left;  /* TouchRec.left                                       */
    uint8_t touch_clamped;
    uint8_t escalated;   /* extend_hint ran attempt 2 (full matrix)             */
    int32_t status;      /* ESP_OK or ESP_ECAP for this pair                    */
} esp_extension;

/* ---- handle ---- */

/* Create a handle bound to CUDA device `device` (its own stream, pinned
 * staging and grow-only device scratch).  Replaces the reference's
 * per-thread ExtendBuffer (crates/map/src/extend.rs:231-251). */
int esp_create(esp_handle **out, int device);
/* Kernel choice (no counterpart in the reference): batches of at most
 * `warp_max` pairs -- every per-call entry point included -- run one warp per
 * pair (a wavefront over the pair's strips); larger batches run one thread
 * per pair in the persistent length-binned kernel.  Both give identical
 * results.  Default 2048, or the ESP_WARP_MAX environment variable. */
int esp_set_warp_max(esp_handle *h, long warp_max);
/* Kernel variant of the thread-per-pair batches (no counterpart in the
 * reference): 0 = one pair per thread at 3 resident blocks per SM, 1 = at 4
 * blocks, 2 / 3 = two pairs of identical band geometry per thread (16x2 SIMD
 * lanes) at 3 / 4 blocks; -1 = the ESP_GOTOH_VARIANT environment variable,
 * else by size: variant 3 for batches of 2^20 pairs and more, 1 below.
 * Applies to band-mode batches and clears a previous autotuning.  Hint-mode
 * batches choose by size the same way (ESP_GOTOH_HINT_VARIANT overrides).
 * All variants give identical results. */
int esp_set_kernel_variant(esp_handle *h, int variant);
int esp_destroy(esp_handle *h);
/* Message of the last error on this handle (static storage of the handle). */
const char *esp_last_error(const esp_handle *h);
/* The handle's CUDA stream (cudaStream_t as void *). */
void *esp_stream(esp_handle *h);

/* ---- per-call drop-ins: crates/map/src/extend.rs ---- */

/* extend (extend.rs:347-354): full-window local alignment. */
int esp_extend(esp_handle *h, const uint8_t *read, size_t read_len, const uint8_t *ref_window,
               size_t window_len, const esp_extend_params *params, esp_extension *out,
               uint32_t *cigar, uint32_t cigar_cap);

/* extend_hint (extend.rs:392-428): banded attempt of half-width 30 around
 * the hint diagonal, escalating to the full matrix on a band-edge touch or a
 * score below 85% of perfect.  num/den follow DiagHint (den 0 counts as 1;
 * every reference call site passes 1/1, and run_band asserts it). */
int esp_extend_hint(esp_handle *h, const uint8_t *read, size_t read_len,
                    const uint8_t *ref_window, size_t window_len,
                    const esp_extend_params *params, int64_t hint_offset, uint32_t hint_num,
                    uint32_t hint_den, esp_extension *out, uint32_t *cigar,
                    uint32_t cigar_cap);

/* score_tail_win (crates/map/src/splice.rs:667-684): a tail scored against
 * its reference window by extend_hint along the direct diagonal (offset 0,
 * slope 1/1).  Same outputs and errors as esp_extend_hint. */
int esp_score_tail_win(esp_handle *h, const uint8_t *tail, size_t tail_len,
                       const uint8_t *ref_window, size_t window_len,
                       const esp_extend_params *params, esp_extension *out, uint32_t *cigar,
                       uint32_t cigar_cap);

/* run_band (extend.rs:606-851) with an explicit band, exposed for kernel
 * equivalence checks the way the reference's own tests call it.  half < 0
 * selects the full matrix (band_spec None). */
int esp_run_band(esp_handle *h, const uint8_t *read, size_t read_len, const uint8_t *ref_window,
                 size_t window_len, const esp_extend_params *params, int64_t band_offset,
                 int64_t band_half, esp_extension *out, uint32_t *cigar, uint32_t cigar_cap);

/* ---- batch API (new; beside the per-call drop-in) ----
 *
 * A batch is a set of read x window pairs whose bases live in one 2-bit
 * packed arena (MSB-first within each byte, the reference's contig layout,
 * crates/map/src/fasta.rs:1-5).  Positions are in bases.  Bases that are
 * not A/C/G/T are listed as half-open N intervals relative to the start of
 * their sequence (the reference keeps contig N runs the same way). */
typedef struct {
    uint64_t read_pos;   /* base offset of the read in the arena              */
    uint64_t win_pos;    /* base offset of the window in the arena            */
    uint32_t read_len;
    uint32_t win_len;
    int32_t band_offset; /* DiagHint.offset (band centre j - i)               */
    int32_t band_half;   /* run_band half-width; < 0 = full matrix            */
    uint32_t n_first;    /* first N interval of this pair                     */
    uint16_t n_read;     /* N intervals of the read (relative to read start)  */
    uint16_t n_win;      /* then N intervals of the window                    */
} esp_pair;

typedef struct {
    uint32_t start;
    uint32_t end;
} esp_n_interval;

#define ESP_MODE_BAND 0 /* run_band with each pair's band (or full matrix)       */
#define ESP_MODE_HINT 1 /* extend_hint policy with each pair's band_offset       */

/* Upper bounds over a device-resident batch, used to size DP scratch
 * (pairs beyond them are refused per pair with status ESP_EINVAL). */
typedef struct {
    uint32_t max_read_len;
    uint32_t max_win_len;
    int32_t max_half;  /* largest band_half; < 0 when any pair runs the full matrix */
} esp_batch_limits;

/* Device-resident batch: every pointer is device memory; the call is
 * asynchronous on `stream` (NULL = handle stream).  `cigar` holds
 * n_pairs * cigar_stride ops.  Returns after enqueueing. */
int esp_batch_extend_device(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                            const uint8_t *arena, uint64_t arena_bytes,
                            const esp_n_interval *n_iv, uint64_t n_iv_count,
                            const esp_batch_limits *limits, const esp_extend_params *params,
                            esp_extension *out, uint32_t *cigar, uint32_t cigar_stride,
                            void *stream);

/* Host-resident batch: copies inputs to the device, runs, copies results
 * back and synchronises (the end-to-end path). */
int esp_batch_extend_host(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                          const uint8_t *arena, uint64_t arena_bytes,
                          const esp_n_interval *n_iv, uint64_t n_iv_count,
                          const esp_extend_params *params, esp_extension *out,
                          uint32_t *cigar, uint32_t cigar_stride);

/* Autotuning per length class (no counterpart in the reference): runs the
 * band-mode batch once per DP kernel variant (esp_set_kernel_variant's 0..3)
 * on each of four length classes of its binned work list (band/window width
 * >= 196, [100, 196), [52, 100), < 52 columns) and on the whole list in one
 * launch.  Later band-mode batches of the handle run the fastest variant per
 * class when the classes' best times add up to less than the best single
 * launch, else that single launch's variant for all.  ms: 20 timings, row-
 * major (classes 0..3, then the whole list) over the four variants;
 * variants: the choice per class; either may be null.  The batch's results
 * are left in out/cigar.  Needs a batch above the warp-per-pair size. */
int esp_batch_autotune(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                       const uint8_t *arena, uint64_t arena_bytes, const esp_n_interval *n_iv,
                       uint64_t n_iv_count, const esp_batch_limits *limits,
                       const esp_extend_params *params, esp_extension *out, uint32_t *cigar,
                       uint32_t cigar_stride, void *stream, int *variants, double *ms);

/* ---- EA-Myers filters: crates/map/src/myers_ea.rs, crates/engine/src/myers.rs ----
 *
 * Editing-aware equality: read A matches reference {A}, C matches {C,T},
 * G matches {G,A}, T matches {T}; anything else matches nothing; case
 * folds.  Per-call entry points take ASCII like the reference. */

/* myers_ea::infix (myers_ea.rs:118-135): min distance of the whole read
 * against any substring of `text`.  m = 0 -> 0; m > 256 -> m; the
 * single-block entry points refuse 128 < m <= 256 (ESP_EINVAL), which the
 * reference's callers route to long:: (align.rs:878-882). */
int esp_myers_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                    size_t n, int32_t *dist);
/* myers_ea::infix_best_end (myers_ea.rs:138-155): also the earliest
 * exclusive end of a best occurrence (0 when nothing beats m). */
int esp_myers_infix_best_end(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                             size_t n, int32_t *dist, uint64_t *end);
/* myers_ea::infix_best_start(_into) (myers_ea.rs:158-185): best_end of the
 * reversed pair, start = n - reversed end. */
int esp_myers_infix_best_start(esp_handle *h, const uint8_t *read, size_t m,
                               const uint8_t *text, size_t n, int32_t *dist, uint64_t *start);
/* myers_ea::long::{infix, infix_best_end, infix_best_start(_into)}
 * (myers_ea.rs:249-310): the same for m <= 256. */
int esp_myers_long_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                         size_t n, int32_t *dist);
int esp_myers_long_infix_best_end(esp_handle *h, const uint8_t *read, size_t m,
                                  const uint8_t *text, size_t n, int32_t *dist, uint64_t *end);
int esp_myers_long_infix_best_start(esp_handle *h, const uint8_t *read, size_t m,
                                    const uint8_t *text, size_t n, int32_t *dist,
                                    uint64_t *start);
/* esperanto_engine::myers::{infix, long::infix} (engine/src/myers.rs:32-56)
 * and {global, long::global} (:42-62); 1 <= m <= 256 (the reference asserts,
 * here ESP_EINVAL). */
int esp_engine_myers_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                           size_t n, uint32_t *dist);
int esp_engine_myers_global(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                            size_t n, uint32_t *dist);

/* Batch Myers (new): pairs over a 2-bit arena as for the DP batch. */
typedef struct {
    uint64_t read_pos;
    uint64_t text_pos;
    uint32_t read_len;  /* 1..256 */
    uint32_t text_len;
    uint32_t n_first;   /* N intervals: read's, then text's */
    uint16_t n_read;
    uint16_t n_text;
} esp_myers_pair;

typedef struct {
    int32_t dist;
    int32_t status;
    uint64_t pos;       /* best end (exclusive) or best start (inclusive) */
} esp_myers_result;

#define ESP_MYERS_BEST_END 0   /* myers_ea::infix_best_end / long:: */
#define ESP_MYERS_BEST_START 1 /* myers_ea::infix_best_start / long:: */
#define ESP_MYERS_GLOBAL 2     /* engine::myers::global (pos = 0) */

int esp_batch_myers_device(esp_handle *h, int mode, const esp_myers_pair *pairs,
                           uint64_t n_pairs, uint32_t max_read_len, const uint8_t *arena,
                           uint64_t arena_bytes, const esp_n_interval *n_iv,
                           uint64_t n_iv_count, esp_myers_result *out, void *stream);
int esp_batch_myers_host(esp_handle *h, int mode, const esp_myers_pair *pairs,
                         uint64_t n_pairs, const uint8_t *arena, uint64_t arena_bytes,
                         const esp_n_interval *n_iv, uint64_t n_iv_count,
                         esp_myers_result *out);

/* ---- resident genome: crates/map/src/fasta.rs Reference / Contig ----
 *
 * The genome stays in HBM as one 2-bit arena (MSB-first, the contig layout
 * of fasta.rs:1-5); each contig is a base offset into it plus its length and
 * its merged N intervals in contig coordinates (fasta.rs:62-75). */
typedef struct {
    uint64_t base;     /* arena base position of contig coordinate 0 */
    uint32_t len;      /* contig length (bases) */
    uint32_t n_first;  /* first N interval of this contig in the genome table */
    uint32_t n_count;  /* number of its N intervals (sorted, merged) */
    uint32_t pad;
} esp_contig;

typedef struct esp_genome esp_genome;

/* Upload a genome (host arrays) to the handle's device.  The genome is
 * immutable afterwards and may be shared by handles on the same device. */
int esp_genome_create(esp_handle *h, const uint8_t *arena, uint64_t arena_bytes,
                      const esp_contig *contigs, uint32_t n_contigs,
                      const esp_n_interval *n_iv, uint64_t n_iv_count, esp_genome **out);
int esp_genome_destroy(esp_genome *g);

/* ---- paidx v1 index contigs: crates/map/src/index_io.rs ----
 *
 * The reference's index loader (index_io.rs:113-121 load, :237-354
 * decode_parts) validates the whole file and keeps its Reference: the
 * contigs, already 2-bit packed MSB-first with their N intervals.  These
 * entry points run the same strict validation (same failure messages) and
 * lay the contigs out as a resident genome, each contig starting on a byte
 * of the arena.  The seeding tables are validated, not kept. */
typedef struct {
    uint32_t k, w, freq_cutoff, contig_count;
    uint64_t kmer_count, positions_count;
    uint8_t fasta_sha256[32];
    uint64_t arena_bytes;  /* bytes of packed contigs (the genome arena) */
    uint64_t n_iv_count;   /* N intervals over all contigs */
    uint64_t names_bytes;  /* contig names, each NUL-terminated */
} esp_paidx_info;

/* Validate `data` (the whole file) and size its contents.  ESP_EFORMAT /
 * ESP_EVERSION with the reference's message in `msg` when it is malformed. */
int esp_paidx_scan(const uint8_t *data, uint64_t len, esp_paidx_info *info, char *msg,
                   size_t msg_cap);
/* Copy the contigs into caller buffers sized by esp_paidx_scan (host only). */
int esp_paidx_contigs(const uint8_t *data, uint64_t len, uint8_t *arena, uint64_t arena_bytes,
                      esp_contig *contigs, uint32_t n_contigs, esp_n_interval *n_iv,
                      uint64_t n_iv_count, char *names, uint64_t names_bytes);
/* Validate and upload: a resident genome whose contig c is the index's
 * contig c (the reference's Reference of a loaded Index). */
int esp_genome_from_paidx(esp_handle *h, const uint8_t *data, uint64_t len, esp_genome **out);

/* ---- splice-rescue flank DP: crates/map/src/split.rs ---- */

/* crates/map/src/splice.rs:21-53 SpliceParams */
typedef struct {
    uint32_t min_intron;
    uint32_t max_intron;
    int32_t gt_ag_bonus;
    int32_t gc_ag_bonus;
    int32_t at_ac_bonus;
    int32_t noncanonical_penalty;
    int32_t known_bonus;
    uint32_t refine_radius;
} esp_splice_params;

/* crates/map/src/gtf.rs:23-45 Junction and SpliceSignal */
typedef struct {
    uint32_t contig;
    uint32_t start;        /* intron start (donor side) */
    uint32_t end;          /* intron end (acceptor side, exclusive) */
    int32_t minus_strand;
} esp_junction;

#define ESP_SIG_GTAG 0
#define ESP_SIG_GCAG 1
#define ESP_SIG_ATAC 2
#define ESP_SIG_NONCANONICAL 3

/* split.rs:120-132 RetryOutcome (the two CIGARs go to caller buffers) */
typedef struct {
    int32_t found;         /* Option::is_some */
    uint32_t dro;
    uint32_t left_win_lo;
    int32_t total;
    esp_extension left;
    esp_extension right;
} esp_retry_outcome;

/* retry_tail_start (split.rs:150-223): retry the tail start +-5 around
 * `tail_start` against junction `j`: per breakpoint, extend_hint the left
 * segment in the window ending at the donor and the right segment in the
 * window starting at the acceptor, gate both on coverage and seam anchoring,
 * keep the best total (ties: lowest breakpoint).  `read` is ASCII. */
int esp_retry_tail_start(esp_handle *h, const esp_genome *g, const uint8_t *read, size_t read_len,
                         uint32_t tail_start, const esp_junction *j, int signal,
                         uint32_t support, const esp_splice_params *sp,
                         const esp_extend_params *params, esp_retry_outcome *out,
                         uint32_t *left_cigar, uint32_t *right_cigar, uint32_t cigar_cap);

/* Batch channel A (split.rs:468-570 with caller-supplied library
 * candidates; one read per record, candidates in library order):
 * retry every candidate, keep the best total (ties: first candidate), stitch
 * left + N(intron) + right (build_rescue_ext, split.rs:227-240) and validate
 * it (rescue_cigar_valid, split.rs:282-321). */
typedef struct {
    uint64_t read_pos;     /* base offset in the batch's read arena */
    uint32_t read_len;
    uint32_t tail_start;
    uint32_t contig;
    int32_t minus;         /* primary alignment strand is minus */
    uint32_t cand_first;   /* first candidate of this read */
    uint32_t cand_count;
    uint32_t n_first;      /* read N intervals (relative to the read) */
    uint32_t n_read;
} esp_splice_read;

typedef struct {
    esp_junction j;
    uint32_t support;      /* library support count */
} esp_splice_cand;

typedef struct {
    int32_t found;
    int32_t cand;          /* winning candidate (index within the read's list) */
    uint32_t dro;
    uint32_t pos;          /* left_win_lo + left.ref_start */
    int32_t score;         /* retry total */
    int32_t signal;
    uint32_t n_ops;        /* spliced CIGAR length */
    int32_t status;        /* ESP_OK, ESP_ECAP (a CIGAR did not fit), ESP_EDOMAIN */
} esp_splice_result;

int esp_batch_splice_host(esp_handle *h, const esp_genome *g, const esp_splice_read *reads,
                          uint64_t n_reads, const uint8_t *read_arena, uint64_t read_arena_bytes,
                          const esp_n_interval *read_n_iv, uint64_t read_n_iv_count,
                          const esp_splice_cand *cands, uint64_t n_cands,
                          const esp_splice_params *sp, const esp_extend_params *params,
                          esp_splice_result *out, uint32_t *cigar, uint32_t cigar_stride);

/* Device-resident variant (all pointers device memory; asynchronous on
 * `stream`, NULL = handle stream).  Reads may not exceed max_read_len. */
int esp_batch_splice_device(esp_handle *h, const esp_genome *g, const esp_splice_read *reads,
                            uint64_t n_reads, uint32_t max_read_len, const uint8_t *read_arena,
                            uint64_t read_arena_bytes, const esp_n_interval *read_n_iv,
                            uint64_t read_n_iv_count, const esp_splice_cand *cands,
                            uint64_t n_cands, const esp_splice_params *sp,
                            const esp_extend_params *params, esp_splice_result *out,
                            uint32_t *cigar, uint32_t cigar_stride, void *stream);

/* DP cells of the last batch splice call (both extension attempts counted). */
uint64_t esp_last_cells(const esp_handle *h);

/* ---- spliced pseudo-reference DP: crates/map/src/splice.rs align_spliced ----
 *
 * align_spliced (splice.rs:617-664) after prepare_spliced chose the exon
 * slices (refinement and guards upstream): the read (2-bit arena + N
 * intervals) is extended with extend_hint along the direct diagonal against
 * the concatenation of its slices [start, end) of its contig (gathered on the
 * device from the resident genome), and the CIGAR is stitched back to the
 * genome (stitch_cigar, :435-493) with an intron of exons[i+1].start -
 * exons[i].end at every seam; genomic_start (:414-424) maps the pseudo start
 * back.  CIGARs go to fixed-stride arrays. */
typedef struct {
    uint64_t read_pos;    /* base offset in the read arena */
    uint32_t read_len;
    uint32_t contig;
    uint32_t exon_first;  /* first slice of this read in the exon table */
    uint32_t exon_count;  /* >= 1, ascending and disjoint */
    uint32_t n_first;     /* the read's N intervals */
    uint32_t n_read;
} esp_spliced_read;

typedef struct {
    uint32_t start, end;  /* genomic [start, end) on the read's contig */
} esp_exon;

typedef struct {
    esp_extension ext;     /* extension against the pseudo-reference */
    uint32_t genomic_start;
    uint32_t n_ops;        /* stitched CIGAR ops */
    int32_t status;        /* ESP_OK, or ESP_ECAP when a CIGAR exceeds the stride */
    uint32_t pad;
} esp_spliced_result;

int esp_batch_spliced_host(esp_handle *h, const esp_genome *g, const esp_spliced_read *reads,
                           uint64_t n, const uint8_t *read_arena, uint64_t read_arena_bytes,
                           const esp_n_interval *read_iv, uint64_t n_read_iv,
                           const esp_exon *exons, uint64_t n_exons,
                           const esp_extend_params *params, esp_spliced_result *out,
                           uint32_t *ext_cigar, uint32_t *stitched_cigar, uint32_t cigar_stride);

/* ---- intron-chain fast path: crates/map/src/intron_chain.rs ----
 *
 * try_intron_chain_placement (intron_chain.rs:392-538) from the best
 * fragment pair on, for a batch of reads (each in alignment orientation,
 * with the pair best_frag_pair chose): the junction offset, EA-Myers
 * breakpoint refinement of both sides (refine_donor_end /
 * refine_acceptor_start, :285-343), split-read verification
 * (verify_split_read, :347-373), the anchor / intron-length / mismatch-rate
 * gates, read-aware junction refinement against the junction library
 * (splice.rs:208-313 refine_junction_read; the pair's own junction when it
 * finds none), the pseudo-reference extend_hint along the fragment's
 * diagonal and stitch_cigar, and the final gates -- on the device over the
 * resident genome.  The MEM extension, clustering and pair choice before it
 * are seeding. */
typedef struct {         /* intron_chain.rs:69-86 Frag: spans and MEM count */
    uint32_t q_lo, q_hi; /* read span [q_lo, q_hi) */
    uint32_t r_lo, r_hi; /* reference span [r_lo, r_hi) */
    uint32_t n_anchors;
} esp_frag;

typedef struct {
    uint64_t read_pos;     /* base offset in the read arena */
    uint32_t read_len;
    uint32_t contig;       /* the fragments' contig */
    uint32_t n_first;      /* the read's N intervals */
    uint32_t n_read;
    int32_t minus;         /* the fragments' strand is minus */
    uint32_t intron_start; /* best_frag_pair's intron: the fallback junction */
    uint32_t intron_end;
    esp_frag left, right;
    uint32_t pad;
} esp_intron_read;

typedef struct {         /* intron_chain.rs:21-41 IntronParams (defaults 15, 30, 50, 105000) */
    uint32_t min_frag_cov, refine_window, refine_pattern_len, intron_max;
} esp_intron_params;

typedef struct {         /* a JunctionLib entry (gtf.rs:72-149): sorted by (contig, start, end, strand) */
    esp_junction j;
    uint32_t count;
} esp_lib_junction;

#define ESP_IC_FOUND 0     /* Some(SplicedAlignment) */
#define ESP_IC_EMPTY 1     /* empty read */
#define ESP_IC_ANCHORS 2   /* fewer than two anchors */
#define ESP_IC_INTRON 3    /* refined intron length outside [20, intron_max] */
#define ESP_IC_VERIFY 4    /* split-read verification over the mismatch-rate thresholds */
#define ESP_IC_JUNCTION 5  /* chosen junction outside [20, intron_max] */
#define ESP_IC_BOUNDS 6    /* the exon bounds do not enclose the junction */
#define ESP_IC_RESULT 7    /* non-positive score, a CIGAR that loses read bases or has no intron */

typedef struct {
    int32_t found;
    int32_t stage;           /* ESP_IC_*: the gate that ended the read */
    uint32_t donor_end;      /* refine_donor_end */
    uint32_t acceptor_start; /* refine_acceptor_start */
    int32_t verify_donor;    /* verify_split_read distances (INT32_MAX when skipped) */
    int32_t verify_acceptor;
    esp_junction junction;   /* the refined junction */
    int32_t signal;          /* ESP_SIG_* */
    uint32_t support;        /* library support of the junction */
    uint32_t left_start;     /* exon bounds: (0, left_start, junction.start), */
    uint32_t right_end;      /* (junction.start - left_start, junction.end, right_end) */
    esp_extension ext;       /* extend_hint against the pseudo-reference */
    uint32_t genomic_start;  /* SplicedAlignment::genomic_start */
    uint32_t n_ops;          /* stitched CIGAR ops */
    int32_t status;          /* ESP_OK, or ESP_ECAP when a CIGAR exceeds the stride */
} esp_intron_result;

int esp_batch_intron_chain_host(esp_handle *h, const esp_genome *g, const esp_intron_read *reads,
                                uint64_t n, const uint8_t *read_arena, uint64_t read_arena_bytes,
                                const esp_n_interval *read_iv, uint64_t n_read_iv,
                                const esp_lib_junction *lib, uint64_t n_lib,
                                const esp_intron_params *ip, const esp_extend_params *params,
                                esp_intron_result *out, uint32_t *ext_cigar,
                                uint32_t *stitched_cigar, uint32_t cigar_stride);

/* ---- strict rescoring: crates/map/src/align.rs:1060-1165 rescore_with ----
 *
 * One record per placement: its query (ASCII, compared byte for byte as the
 * reference does), contig, start and CIGAR (u32 len<<4|op, ESP_OP_*), and the
 * editing direction exempted from the mismatch charge.  `lib` is the
 * junction library sorted by (contig, start, end) (JunctionLib, gtf.rs;
 * minus_strand ignored: contains_any_strand).  sp = null uses
 * SpliceParams::default() as rescore_with does. */
typedef struct {
    uint64_t query_pos;  /* byte offset of the query in the query arena */
    uint32_t query_len;
    uint32_t contig;
    uint32_t pos;        /* placement start on the contig */
    uint32_t op_first;   /* first CIGAR op in the op array */
    uint32_t op_count;
    int32_t edit_dir;    /* ESP_EDIT_* */
} esp_rescore_item;

typedef struct {         /* align.rs:188-211 StrictScore */
    int32_t score;
    uint32_t aligned, matches, mm, ea_ag, ea_tc, ins, del, clipped, n_splice;
    int32_t splice_score;
    int32_t status;      /* ESP_OK, or ESP_EINVAL for a record outside its tables */
} esp_strict_score;

/* splice.rs:119-121 intron_length_penalty through the threshold table the
 * rescoring kernel uses (host-side; equal to the reference's f64 formula for
 * every u32 length). */
int32_t esp_intron_length_penalty(uint32_t len);

int esp_batch_rescore_device(esp_handle *h, const esp_genome *g, const esp_rescore_item *items,
                             uint64_t n, const uint8_t *queries, uint64_t query_bytes,
                             const uint32_t *ops, uint64_t n_ops, const esp_junction *lib,
                             uint64_t n_lib, const esp_extend_params *params,
                             const esp_splice_params *sp, esp_strict_score *out, void *stream);
int esp_batch_rescore_host(esp_handle *h, const esp_genome *g, const esp_rescore_item *items,
                           uint64_t n, const uint8_t *queries, uint64_t query_bytes,
                           const uint32_t *ops, uint64_t n_ops, const esp_junction *lib,
                           uint64_t n_lib, const esp_extend_params *params,
                           const esp_splice_params *sp, esp_strict_score *out);

/* ---- serving loop (new): continuous batching over a resident genome ----
 *
 * Submitted requests queue FIFO.  A native worker thread turns the head of
 * the queue into DP launches of up to max_reads reads: small requests of
 * one CIGAR stride that wait together share a launch, and a request larger
 * than max_reads runs over several.  Each launch is charged the DP scratch
 * it needs (traceback words of the extend_hint policy's full-matrix attempt
 * for its longest read and window) from one device pool of
 * mem_budget_bytes shared by all in-flight slots: a launch that does not fit
 * is cut to the reads that do (at least 1,024), and when not even that fits
 * the head request waits until a running launch returns its scratch.  Each
 * read's candidate window is read in place from the resident genome, the
 * extend_hint policy runs on the slot's stream and results are copied back,
 * so requests that arrive while others run are admitted as slots and memory
 * free up, and their work overlaps on the device.  Results of a request do
 * not depend on what else is in flight. */
typedef struct {
    uint64_t read_pos;     /* base offset in the request's read arena */
    uint32_t read_len;
    uint32_t contig;
    uint32_t win_start;    /* candidate window [win_start, win_start + win_len) */
    uint32_t win_len;      /* clipped to the contig */
    int32_t hint_offset;   /* DiagHint.offset within the window */
    uint32_t pad;
} esp_serve_read;

typedef struct {
    const uint8_t *read_arena; /* host, 2-bit packed; kept alive until completion */
    uint64_t read_arena_bytes;
    const esp_serve_read *reads;
    uint64_t n_reads;
    esp_extension *out;        /* host results, n_reads records */
    uint32_t *cigar;           /* host, n_reads * cigar_stride ops */
    uint32_t cigar_stride;
} esp_serve_request;

typedef struct {
    uint32_t n_streams;        /* in-flight launch slots (default 4, at most 64) */
    uint32_t max_reads;        /* reads per launch (default 131072, below 2^20) */
    uint32_t max_read_len;     /* default 300 */
    uint32_t max_win_len;      /* default max_read_len + 128 */
    uint64_t mem_budget_bytes; /* the DP scratch pool, allocated at creation (default 16 GiB) */
} esp_server_config;

typedef struct {
    uint64_t launches;         /* DP launches completed */
    uint64_t reads;            /* reads in them */
    uint64_t merged_launches;  /* launches holding reads of more than one request */
    uint64_t split_requests;   /* requests whose reads ran in more than one launch */
    uint64_t budget_waits;     /* requests held at the head of the queue for scratch memory */
    uint64_t cut_launches;     /* launches cut short to fit the free scratch */
    uint64_t pool_bytes;       /* the scratch pool (the memory budget) */
    uint64_t pool_peak_bytes;  /* most of it charged at once */
} esp_server_stats;

typedef struct esp_server esp_server;

int esp_server_create(esp_genome *g, const esp_extend_params *params,
                      const esp_server_config *cfg, int device, esp_server **out);
/* Non-blocking; requests of any size (cigar_stride at most 64).  ESP_EBUSY:
 * even its smallest launch exceeds the whole memory budget; ESP_EINVAL: a
 * read outside its limits or tables; ESP_ECLOSED: the server is closing. */
int esp_server_submit(esp_server *s, const esp_serve_request *req, uint64_t *ticket);
/* Wait (bounded) for a ticket: ESP_OK with *status the request's status and
 * *latency_ms submit-to-results time, or ESP_ETIMEOUT. */
int esp_server_wait(esp_server *s, uint64_t ticket, int timeout_ms, int32_t *status,
                    double *latency_ms);
/* Admission and memory counters since creation. */
int esp_server_get_stats(esp_server *s, esp_server_stats *out);
/* Stop admitting: queued requests none of whose reads has started complete
 * with ESP_ECLOSED; started ones finish normally. */
int esp_server_close(esp_server *s);
int esp_server_destroy(esp_server *s);

/* ---- pipeline batching hook: a chunk collector over the batch API ----
 *
 * The reference's mapper aligns chunks of 100,000 reads, its rayon workers
 * calling the per-read entry points one read at a time
 * (crates/map/src/pipeline.rs:394-403 in run_pe, :116-250 run_se,
 * :318-450).  A collector instead gathers a chunk's calls -- from any number
 * of host threads at once; the add functions are thread-safe -- and
 * esp_chunk_run sends each kind through the batch API as one batch (one per
 * DP mode, one per Myers direction).  Each add returns the request's index
 * (input order); after the run, esp_chunk_extension / esp_chunk_myers return
 * exactly what the per-call entry point returns for it (the same guards:
 * empty reads, Myers lengths, CIGAR capacity).  A pipeline whose per-read
 * decisions depend on earlier results (Myers first, the DP only for reads
 * Myers does not settle) runs rounds: add, run, read, reset.  ASCII inputs
 * are copied at add time. */
typedef struct esp_chunk esp_chunk;

/* Kinds of esp_chunk_add_myers: myers_ea::{infix, infix_best_end,
 * infix_best_start} (myers_ea.rs:118-185), their long:: forms (:249-310),
 * esperanto_engine::myers::{infix, global} (engine/src/myers.rs:32-63). */
#define ESP_CHUNK_MYERS_INFIX 0
#define ESP_CHUNK_MYERS_BEST_END 1
#define ESP_CHUNK_MYERS_BEST_START 2
#define ESP_CHUNK_MYERS_LONG_INFIX 3
#define ESP_CHUNK_MYERS_LONG_BEST_END 4
#define ESP_CHUNK_MYERS_LONG_BEST_START 5
#define ESP_CHUNK_ENGINE_INFIX 6
#define ESP_CHUNK_ENGINE_GLOBAL 7

/* A collector running its batches on handle h (one collector per handle);
 * DP results keep cigar_stride ops per request (longer CIGARs report
 * ESP_ECAP, as the per-call entry point with that capacity does). */
int esp_chunk_create(esp_handle *h, uint32_t cigar_stride, esp_chunk **out);
/* extend_hint (extend.rs:392-428), run_band (:606-851), extend (:347-354). */
int esp_chunk_add_extend_hint(esp_chunk *c, const uint8_t *read, size_t read_len,
                              const uint8_t *ref_window, size_t window_len, int64_t hint_offset,
                              uint64_t *index);
int esp_chunk_add_run_band(esp_chunk *c, const uint8_t *read, size_t read_len,
                           const uint8_t *ref_window, size_t window_len, int64_t band_offset,
                           int64_t band_half, uint64_t *index);
int esp_chunk_add_extend(esp_chunk *c, const uint8_t *read, size_t read_len,
                         const uint8_t *ref_window, size_t window_len, uint64_t *index);
int esp_chunk_add_myers(esp_chunk *c, int kind, const uint8_t *read, size_t read_len,
                        const uint8_t *text, size_t text_len, uint64_t *index);
/* Run everything queued (one batch per kind, synchronously).  ESP_EBUSY if
 * already run since the last reset. */
int esp_chunk_run(esp_chunk *c, const esp_extend_params *params);
/* Results by request index, as the per-call entry points return them. */
int esp_chunk_extension(esp_chunk *c, uint64_t index, esp_extension *out, uint32_t *cigar,
                        uint32_t cigar_cap);
/* pos: the best end / best start of the kinds that return one, else 0. */
int esp_chunk_myers(esp_chunk *c, uint64_t index, int32_t *dist, uint64_t *pos);
uint64_t esp_chunk_size(esp_chunk *c);
/* Forget the queued requests and results (capacity is kept). */
int esp_chunk_reset(esp_chunk *c);
int esp_chunk_destroy(esp_chunk *c);

/* ---- allocation-free variant (no counterpart in the reference) ----
 *
 * esp_batch_run_band_noalloc: the same banded/full-matrix DP with traceback
 * as esp_batch_extend_device in ESP_MODE_BAND, for callers that must not
 * allocate device memory after start-up -- a host runtime that owns all
 * device memory through its own pre-sized pool, or a latency-bound request
 * path that cannot afford cudaMalloc/cudaFree (which can synchronise the
 * whole device).  It calls no cudaMalloc, cudaFree or other allocating
 * routine and needs no handle: its scratch is one fixed array of
 * ESP_NOALLOC_SCRATCH_BYTES in device memory, held by every GPU that loads
 * this library until the process exits.
 *   - Inputs and outputs are caller-owned device memory, as for
 *     esp_batch_extend_device; the call is asynchronous on `stream`
 *     (NULL = legacy default stream) on the current device.
 *   - The first call on a device looks up the array's device address for
 *     that device and keeps it for the process; make that first call before
 *     any stream capture, and do not call it after cudaDeviceReset (the
 *     address kept would belong to the destroyed context).
 *   - Every call shares the one array: calls that can overlap on the GPU
 *     (different streams, different host threads) race and must be
 *     serialised by the caller.
 *   - Work whose per-block scratch (4 warps x 32 pairs of traceback and
 *     row-buffer words, sized from `limits`) exceeds the array returns
 *     ESP_ESCRATCH, whatever n_pairs is (even a batch of a few pairs needs
 *     one block's scratch); smaller work runs with fewer resident blocks
 *     when the array cannot hold a full persistent grid, each thread taking
 *     pairs from the queue in turn.
 *   - Reads longer than the int16 domain (8191 / largest substitution
 *     score) are refused (ESP_EDOMAIN): the wide kernel needs scratch sized
 *     per pair.
 *   - Pairs run in the order given (no length binning). */
#define ESP_NOALLOC_SCRATCH_BYTES (64ull << 20)
int esp_batch_run_band_noalloc(const esp_pair *pairs, uint64_t n_pairs, const uint8_t *arena,
                               uint64_t arena_bytes, const esp_n_interval *n_iv,
                               uint64_t n_iv_count, const esp_batch_limits *limits,
                               const esp_extend_params *params, esp_extension *out,
                               uint32_t *cigar, uint32_t cigar_stride, void *stream);

/* Number of device kernel launches the last batch call enqueued. */
uint64_t esp_last_launch_count(const esp_handle *h);

#ifdef __cplusplus
}
#endif
#endif
