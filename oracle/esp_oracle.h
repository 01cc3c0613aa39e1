/*
 * esp_oracle.h -- CPU restatement of the ESPERANTO read-alignment inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle for the
 * GB300 kernels: only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark load it.  The product library never links it.
 *
 * Every function restates the reference Rust code cited beside it
 * (paths are relative to the reference project root).  The reference is a
 * Rust workspace that cannot be compiled here (no cargo, crates not
 * vendored), so this restatement is pinned instead against the literal
 * known answers in the reference's own unit tests (crates/map/src/extend.rs
 * :2033-2571, crates/map/src/split.rs:962-1029), against a brute-force
 * O(m*n) edit-distance DP for the Myers filters, and against the i16/i32
 * twin kernels agreeing on the reference's seeded sweeps.
 *
 * Conventions
 *   - sequences are byte strings (ASCII as the reference receives them);
 *   - CIGAR ops are packed u32: (len << 4) | code, code M=0 I=1 D=2 N=3 S=4
 *     (the BAM op codes; the reference folds =/X into M);
 *   - functions returning int use 0 = ok, negative = error (see ORC_E*).
 */
#ifndef ESP_ORACLE_H
#define ESP_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_OK 0
#define ORC_EINVAL (-1)   /* argument outside the reference's domain      */
#define ORC_ECAP (-2)     /* caller's CIGAR buffer too small               */
#define ORC_ENOMEM (-3)

enum { ORC_OP_M = 0, ORC_OP_I = 1, ORC_OP_D = 2, ORC_OP_N = 3, ORC_OP_S = 4 };
enum { ORC_EDIT_OFF = 0, ORC_EDIT_AG = 1, ORC_EDIT_TC = 2 };

/* crates/map/src/extend.rs:97-122 ExtendParams (mismatch stored negative,
 * gap penalties stored positive). */
typedef struct {
    int32_t match_score;
    int32_t mismatch;
    int32_t gap_open;
    int32_t gap_ext;
    int32_t edit_dir; /* ORC_EDIT_* */
} orc_params;

/* crates/map/src/extend.rs:200-214 Extension. `ops` points at caller memory
 * of `cap` entries; `n_ops` is always the full count. */
typedef struct {
    uint32_t read_start;
    uint32_t read_end;
    uint32_t ref_start;
    int32_t score;
    uint32_t n_ops;
    uint32_t cap;
    uint32_t *ops;
} orc_ext;

/* crates/map/src/extend.rs:216-229 TouchRec. */
typedef struct {
    int32_t touched;
    int64_t row;
    int32_t left;
    int32_t clamped;
} orc_touch;

/* ---- extension core (crates/map/src/extend.rs) ---- */
int orc_base_code(uint8_t b);
void orc_lut(const orc_params *p, int16_t lut[25]);
int16_t orc_i16_add(int16_t a, int16_t b);
/* run_band<T> (:606-851); wide = 0 -> i16 accumulators, 1 -> i32.
 * has_band = 0 is band_spec None (full matrix). */
int orc_run_band(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                 const orc_params *p, int wide, int has_band, int64_t offset,
                 int64_t num, int64_t den, int64_t half, orc_ext *out, orc_touch *touch);
/* run_dispatch (:293-344): pure uppercase ACGTN -> i16, else i32. */
int orc_run_dispatch(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                     const orc_params *p, int has_band, int64_t offset, int64_t num,
                     int64_t den, int64_t half, orc_ext *out, orc_touch *touch);
/* extend (:347-354) */
int orc_extend(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
               const orc_params *p, orc_ext *out);
/* extend_hint (:392-428); *escalated (may be NULL) reports attempt 2 ran. */
int orc_extend_hint(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                    const orc_params *p, int64_t offset, uint32_t num, uint32_t den,
                    orc_ext *out, int *escalated);
/* extend_hint with every attempt in the i32 flavour of run_band. */
int orc_extend_hint_i32(const uint8_t *read, int64_t m, const uint8_t *rf, int64_t n,
                    const orc_params *p, int64_t offset, uint32_t num, uint32_t den,
                    orc_ext *out, int *escalated);
/* In-window cell count of one run_band call (the GCUPS work unit). */
int64_t orc_band_cells(int64_t m, int64_t n, int has_band, int64_t offset, int64_t half);

/* ---- EA-Myers, crates/map/src/myers_ea.rs ---- */
int orc_myers_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                    int32_t *dist);
int orc_myers_infix_best_end(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                             int32_t *dist, int64_t *end);
int orc_myers_infix_best_start(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                               int32_t *dist, int64_t *start);
int orc_myers_long_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                         int32_t *dist);
int orc_myers_long_infix_best_end(const uint8_t *read, int64_t m, const uint8_t *text,
                                  int64_t n, int32_t *dist, int64_t *end);
int orc_myers_long_infix_best_start(const uint8_t *read, int64_t m, const uint8_t *text,
                                    int64_t n, int32_t *dist, int64_t *start);
/* ---- EA-Myers verifier, crates/engine/src/myers.rs ---- */
int orc_engine_infix(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                     uint32_t *dist);
int orc_engine_global(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                      uint32_t *dist);
/* Independent check: O(m*n) semi-global EA edit distance (not a
 * restatement; used to pin the two bit-parallel formulations). */
int orc_ea_edit_dp(const uint8_t *read, int64_t m, const uint8_t *text, int64_t n,
                   int32_t *dist, int64_t *end);

/* ---- reference storage, crates/map/src/fasta.rs ---- */
typedef struct {
    uint32_t len;
    const uint8_t *packed;         /* ceil(len/4) bytes, MSB-first 2-bit */
    const uint32_t *n_iv;          /* n_iv_count pairs (start, end), sorted */
    uint32_t n_iv_count;
} orc_contig;
void orc_slice_ascii(const orc_contig *c, uint32_t start, uint32_t end, uint8_t *out);
void orc_pack_2bit(const uint8_t *ascii, int64_t n, uint8_t *packed);

/* ---- splice rescue, crates/map/src/split.rs + splice.rs ---- */
enum { ORC_SIG_GTAG = 0, ORC_SIG_GCAG = 1, ORC_SIG_ATAC = 2, ORC_SIG_NONCANON = 3 };
typedef struct {
    uint32_t min_intron, max_intron;
    int32_t gt_ag_bonus, gc_ag_bonus, at_ac_bonus, noncanonical_penalty, known_bonus;
    uint32_t refine_radius;
} orc_splice_params;
typedef struct {
    uint32_t start, end;
    int32_t minus_strand;
} orc_junction;
typedef struct {
    int32_t found;
    uint32_t dro;
    uint32_t left_win_lo;
    int32_t total;
    orc_ext left, right;
} orc_retry;

void orc_splice_params_default(orc_splice_params *sp);
int orc_splice_signal(const uint8_t donor[2], const uint8_t acceptor[2], int minus);
int32_t orc_signal_score(int signal, const orc_splice_params *sp);
int orc_junction_signal(const orc_contig *c, const orc_junction *j);
uint32_t orc_cigar_ref_end(uint32_t pos, const uint32_t *ops, uint32_t n_ops);
int orc_retry_tail_start(const orc_contig *c, const uint8_t *read, uint32_t read_len,
                         uint32_t tail_start, const orc_junction *j, int signal,
                         uint32_t support, const orc_splice_params *sp, const orc_params *p,
                         orc_retry *out);
/* channel_a_with_policy (split.rs:468-570) for a right or left tail with a
 * caller-supplied candidate list (library order), either_strand = false. */
typedef struct {
    int32_t found;
    int32_t cand;        /* index of the winning candidate */
    uint32_t dro;
    uint32_t pos;
    int32_t score;
    int32_t signal;
    uint32_t n_ops;
    uint32_t cap;
    uint32_t *ops;
} orc_rescue;
int orc_channel_a(const orc_contig *c, const uint8_t *read, uint32_t read_len,
                  uint32_t tail_start, int minus, const orc_junction *cands,
                  const uint32_t *support, uint32_t n_cands, const orc_splice_params *sp,
                  const orc_params *p, orc_rescue *out);

/* ---- intron-chain fast path, crates/map/src/intron_chain.rs ---- */
typedef struct {  /* gtf.rs:72-149 JunctionLib entry, sorted (contig, start, end, minus) */
    uint32_t contig, start, end;
    int32_t minus;
    uint32_t count;
} orc_lib_entry;
typedef struct {  /* intron_chain.rs:69-86 Frag (spans and anchor count) */
    uint32_t q_lo, q_hi, r_lo, r_hi, n_anchors;
} orc_frag;
typedef struct {  /* intron_chain.rs:21-41 IntronParams */
    uint32_t min_frag_cov, refine_window, refine_pattern_len, intron_max;
} orc_intron_params;
enum {  /* the stage that ended a read */
    ORC_IC_FOUND = 0, ORC_IC_EMPTY = 1, ORC_IC_ANCHORS = 2, ORC_IC_INTRON = 3, ORC_IC_VERIFY = 4,
    ORC_IC_JUNCTION = 5, ORC_IC_BOUNDS = 6, ORC_IC_RESULT = 7
};
typedef struct {
    int32_t found, stage;
    uint32_t donor_end, acceptor_start;
    int32_t vd, va;
    orc_junction junction;
    int32_t signal;
    uint32_t support;
    uint32_t left_start, right_end;
    orc_ext ext;              /* against the pseudo-reference (ops: caller buffer) */
    uint32_t *stitched;       /* caller buffer */
    uint32_t stitched_cap, n_stitched;
} orc_intron_out;
uint32_t orc_refine_donor_end(const orc_contig *c, const uint8_t *read, uint32_t len,
                              uint32_t junction_off, uint32_t frag_ref_hi,
                              int64_t frag_implied_start, uint32_t refine_window,
                              uint32_t pattern_len);
uint32_t orc_refine_acceptor_start(const orc_contig *c, const uint8_t *read, uint32_t len,
                                   uint32_t junction_off, uint32_t frag_ref_lo,
                                   int64_t frag_implied_start, uint32_t refine_window,
                                   uint32_t pattern_len);
void orc_verify_split_read(const orc_contig *c, const uint8_t *read, uint32_t len,
                           int64_t left_off_lo, uint32_t right_r_hi, int64_t donor_end,
                           int64_t acceptor_start, int32_t *vd, int32_t *va);
uint32_t orc_lib_support(const orc_lib_entry *lib, uint64_t n, uint32_t contig, uint32_t start,
                         uint32_t end, int minus);
int orc_refine_junction_read(const orc_contig *c, uint32_t contig_id, const uint8_t *read,
                             uint32_t read_len, uint32_t naive_start, uint32_t naive_end,
                             uint32_t q_a, uint32_t q_b, int minus, const orc_lib_entry *lib,
                             uint64_t n_lib, const orc_splice_params *sp, orc_junction *out,
                             int *signal, uint32_t *support);
int orc_intron_chain(const orc_contig *c, uint32_t contig_id, const uint8_t *read,
                     uint32_t len, const orc_frag *left, const orc_frag *right,
                     uint32_t pair_intron_start, uint32_t pair_intron_end, int minus,
                     const orc_lib_entry *lib, uint64_t n_lib, const orc_intron_params *ip,
                     const orc_params *p, orc_intron_out *out);

/* ---- spliced pseudo-reference DP, crates/map/src/splice.rs ---- */
uint32_t orc_stitch_cigar(const uint32_t *ops, uint32_t n_ops, uint32_t p_start,
                          const uint32_t *bounds, uint32_t n_bounds, const uint32_t *jlen,
                          uint32_t n_j, uint32_t *out, uint32_t cap);
uint32_t orc_genomic_start(uint32_t p, const uint32_t *bounds, uint32_t n_bounds);
int orc_align_spliced_exons(const orc_contig *c, const uint8_t *read, uint32_t m,
                            const uint32_t *exons, uint32_t n_exons, const orc_params *p,
                            orc_ext *ext, uint32_t *stitched, uint32_t cap,
                            uint32_t *n_stitched, uint32_t *gstart);

/* ---- strict rescoring, crates/map/src/align.rs:1060-1165 ---- */
typedef struct {
    uint32_t contig, start, end;   /* JunctionLib entry, (contig, start, end)-sorted */
} orc_lib_junction;
typedef struct {                   /* align.rs:188-211 StrictScore */
    int32_t score;
    uint32_t aligned, matches, mm, ea_ag, ea_tc, ins, del, clipped, n_splice;
    int32_t splice_score;
} orc_strict;
int32_t orc_intron_length_penalty(uint32_t len);
void orc_rescore(const orc_contig *c, uint32_t contig_id, uint32_t pos, const uint8_t *query,
                 uint32_t qlen, const uint32_t *ops, uint32_t n_ops, const orc_lib_junction *lib,
                 uint64_t n_lib, const orc_params *p, int dir, orc_strict *s);

/* ---- batch drivers for the CPU baseline (one worker per thread, like the
 * reference's rayon map_init over per-thread buffers) ---- */
typedef struct {
    const uint8_t *seqs;      /* concatenated ASCII */
    const uint64_t *read_off; /* per pair */
    const uint32_t *read_len;
    const uint64_t *win_off;
    const uint32_t *win_len;
    const int64_t *offset;    /* band offset per pair */
    const int32_t *half;      /* band half-width per pair (<0: full matrix) */
} orc_pairs;
/* mode 0: run_dispatch with the pair's band, 1: extend_hint(offset). Outputs
 * per pair: score, read_start, read_end, ref_start, n_ops, and up to
 * ops_stride ops.  Returns total cells. */
int64_t orc_batch_extend(const orc_pairs *pr, int64_t n_pairs, const orc_params *p, int mode,
                         int threads, int32_t *score, uint32_t *rs, uint32_t *re,
                         uint32_t *fs, uint32_t *n_ops, uint32_t *ops, uint32_t ops_stride,
                         int32_t *touched);
int64_t orc_batch_myers_best_end(const uint8_t *seqs, const uint64_t *read_off,
                                 const uint32_t *read_len, const uint64_t *text_off,
                                 const uint32_t *text_len, int64_t n_pairs, int threads,
                                 int32_t *dist, int64_t *end);

/* Channel A over many reads (plus strand, default parameters), one contig
 * per read given by (cbase, clen) into a 2-bit arena without N. */
/* Optional per-read detail of orc_batch_channel_a: the winning candidate
 * (-1 when none), breakpoint, position, signal and the spliced CIGAR (the
 * first ops_stride ops per read; ops may be NULL). */
typedef struct {
    int32_t *cand;
    uint32_t *dro, *pos;
    int32_t *signal;
    uint32_t *n_ops;
    uint32_t *ops;
    uint32_t ops_stride;
} orc_ca_detail;
int orc_batch_channel_a(const uint8_t *garena, const uint64_t *cbase, const uint32_t *clen,
                        const uint8_t *reads, const uint64_t *read_off, const uint32_t *read_len,
                        const uint32_t *tail_start, const uint32_t *contig,
                        const uint32_t *cand_first, const uint32_t *cand_count,
                        const uint32_t *cstart, const uint32_t *cend, const uint32_t *csupport,
                        int64_t n_reads, int threads, int32_t *found, int32_t *score,
                        int64_t *cells, orc_ca_detail *detail);

#ifdef __cplusplus
}
#endif
#endif
