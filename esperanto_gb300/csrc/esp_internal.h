// esp_internal.h -- host-side internal interfaces between the ABI layer and
// the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "esperanto_gb300.h"

namespace esp {

// Device copy of the scoring constants (derived once per call from
// esp_extend_params; see gotoh.cu for the scaled-key arithmetic).
struct GotohConst {
    int32_t oe1;        // 4*open_ext - 1  (E open key, low bits 01)
    int32_t oe4;        // 4*open_ext      (F open key, low bits 10 after + Hp)
    int32_t ex4;        // 4*ext
    int32_t open_ext;   // -(gap_open + gap_ext)
    int32_t ext;        // -gap_ext
    int32_t match;      // match_score
    int32_t edit_dir;
    uint32_t lut4[5][2];  // per read code: bytes = 4*score vs ref codes 0..7 (4..7 = N)
    int8_t lut[25];       // SubstLut scores[read*5 + ref] (raw, for traceback deltas)
    int32_t max_m;        // longest read whose scores fit the int16 row buffer
    uint64_t dkind;       // traceback kind of a diagonal step (2 bits) by read code * 5 + ref code
};

// Validate parameters against the device domain and fill the constants.
// Returns ESP_OK or ESP_EDOMAIN.
int make_gotoh_const(const esp_extend_params &p, GotohConst &k);

// Work description for one DP launch.
struct GotohJob {
    const esp_pair *pairs;      // device
    uint64_t n_pairs;
    const uint32_t *list;       // optional: indices into pairs (device); null = 0..n-1
    const uint32_t *list_count; // optional device counter (when list is a queue)
    const uint32_t *range;      // optional device {begin, end}: items list[begin .. end)
    const uint8_t *arena;       // arena of the reads
    uint64_t arena_bases;       // bases addressable in it (excluding padding)
    const uint8_t *win_arena;   // arena of the windows (null = same as reads)
    uint64_t win_arena_bases;
    const esp_n_interval *n_iv;
    uint64_t n_iv_count;
    int mode;                   // 0 band/full per pair, 1 hint attempt 1, 2 hint attempt 2
    uint32_t *esc_list;         // mode 1: escalated pairs are appended here
    uint32_t *esc_count;
    esp_extension *out;
    uint32_t *cigar;
    uint32_t cigar_stride;
    uint32_t *tb;               // traceback scratch: slots * tb_words * 32 words
    uint64_t tb_words;          // per-thread words (>= max strips * strip stride)
    uint32_t *rb;               // row-buffer scratch: slots * rb_words * 32 words
    uint64_t rb_words;
    uint32_t *queue;            // device work counter (zeroed before launch)
    // Pairs outside the int16 domain (read longer than GotohConst::max_m):
    // the int16 kernels append them to wide_list (count in *wide_count) and
    // leave them to the wide kernel, which sets `wide` and runs them in
    // int32; without a list they are refused per pair (ESP_EINVAL).
    uint32_t *wide_list;
    uint32_t *wide_count;
    int wide;
};

// Launch the persistent DP kernel with `warps` warps total.
// variant 0: one pair per thread, 3 resident 128-thread blocks per SM (168
// registers); 1: 4 blocks.  Variants 2 / 3: two pairs of identical geometry
// per thread in 16x2 lanes (neighbours of the binned list), 3 / 4 blocks;
// their scratch per warp is twice tb_words and twice rb_words per lane.
cudaError_t launch_gotoh(const GotohJob &job, const GotohConst &k, int warps, int block,
                         cudaStream_t st, int variant);
constexpr int kGotohVariants = 4;
constexpr bool gotoh_paired(int variant) { return variant >= 2; }

// Wide DP kernel: one warp per pair of job.list (*job.list_count entries),
// int32 scores, for pairs outside the int16 domain.  job.mode 0 runs each
// pair's band (or full matrix); 1 runs the whole extend_hint policy (the
// banded attempt, then the full matrix when it escalates).  Each warp owns
// tb_words + 2 * rb_words words of job.tb (its row buffer holds H and E as
// separate words).  Same results as the int16 kernels wherever both apply.
cudaError_t launch_gotoh_wide(const GotohJob &job, const GotohConst &k, int warps,
                              cudaStream_t st);

// Warp-per-pair DP kernel (per-call drop-in, small batches): `warps` warps
// stride over the pairs; each warp owns tb_words + rb_words words of the
// traceback scratch (job.tb), job.rb unused.  Same results as launch_gotoh.
cudaError_t launch_gotoh_warp(const GotohJob &job, const GotohConst &k, int warps,
                              cudaStream_t st);

// Resident blocks per SM of the DP kernel at `block` threads.
int gotoh_blocks_per_sm(int block, int variant);

// Myers batch job.
constexpr int MYF_REVERSE = 1;
constexpr int MYF_GLOBAL = 2;
struct MyersJob {
    const esp_myers_pair *pairs;
    uint64_t n_pairs;
    const uint8_t *arena;
    const esp_n_interval *n_iv;
    int flags;
    esp_myers_result *out;
};
// nw = 32-bit limbs of the longest read (1..8).
cudaError_t launch_myers(const MyersJob &job, int nw, int num_sms, cudaStream_t st);

// Splice-rescue batch (splice.cu).
constexpr int SPL_SLOTS = 22;  // 11 breakpoints x (left, right) per candidate
constexpr int SPL_IVCAP = 6;   // N intervals one DP slot can carry (read + window)
struct SpliceItem {
    int32_t valid;   // candidate survives channel A's filters
    int32_t signal;  // ESP_SIG_*
};
struct SpliceItemOut {  // retry_tail_start outcome of one candidate
    int32_t found;
    uint32_t dro;
    uint32_t left_win_lo;
    int32_t total;
    uint64_t slot;        // DP slot of the left segment (right = slot + 1)
};
struct SpliceJob {
    int retry_only;       // per-call retry_tail_start: no channel-A filters,
    int forced_signal;    // the caller's signal is used
    SpliceItemOut *item_out;  // optional per-candidate outcome
    const esp_splice_read *reads;
    uint64_t n_reads;
    const uint8_t *read_arena;
    const esp_n_interval *read_iv;
    const uint8_t *g_arena;
    const esp_contig *contigs;
    uint32_t n_contigs;
    const esp_n_interval *g_iv;
    const esp_splice_cand *cands;
    esp_splice_params sp;
    SpliceItem *items;           // one per candidate
    int32_t *read_status;        // one per read
    esp_pair *dp_pairs;          // SPL_SLOTS per candidate
    esp_n_interval *dp_iv;       // SPL_IVCAP per slot, or null when no N anywhere
    const esp_extension *dp_out;
    const uint32_t *dp_cig;
    uint32_t dp_stride;
    esp_splice_result *out;
    uint32_t *cigar;
    uint32_t cigar_stride;
};
cudaError_t launch_splice_build(const SpliceJob &J, int num_sms, cudaStream_t st);
cudaError_t launch_splice_select(const SpliceJob &J, int num_sms, cudaStream_t st);

// DP cells of a finished batch (sum over rows of the window width of every
// attempt that ran), accumulated into *cells (u64, zeroed by the caller).
cudaError_t launch_count_cells(const esp_pair *pairs, const esp_extension *out, uint64_t n,
                               int mode, unsigned long long *cells, int num_sms,
                               cudaStream_t st);

// Counting-sort the pairs by geometry (descending cost) into `order`; the
// list length goes to *total (device).  `hist` needs bin_scratch_bytes() of
// device memory.  5 kernel launches (+1 with bounds) after 1-2 memsets.
// bounds (optional, 5 device words): the four length classes of the list.
// pad: every bin padded to an even slot count with NO_PAIR entries (order
// needs n + bin_pad_slots(n) words), for the two-pairs-per-thread kernel.
// mode: 0 band, 1 extend_hint's first attempt, 2 its full-matrix attempt.
// list / list_count (device, optional): bin only the pairs list[0 ..
// *list_count), n bounding the count (extend_hint's escalations).
cudaError_t launch_binning(const esp_pair *pairs, uint64_t n, int mode, uint32_t *hist,
                           uint32_t *order, int num_sms, cudaStream_t st, uint32_t *total,
                           uint32_t *bounds, bool pad, const uint32_t *list = nullptr,
                           const uint32_t *list_count = nullptr);
// Spare slots a padded list may add to n pairs (the list holds n + this).
uint64_t bin_pad_slots(uint64_t n);
constexpr int kLengthClasses = 4;
size_t bin_scratch_bytes();

// Traceback and row-buffer words one thread needs for a pair.
void gotoh_scratch_words(uint32_t m, uint32_t n, int32_t half, uint64_t &tb, uint64_t &rb);

}  // namespace esp
