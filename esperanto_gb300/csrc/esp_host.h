// esp_host.h -- host-side state shared by the C-ABI translation units: the
// handle, error reporting, grow-only buffers and ASCII -> 2-bit encoding.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "esp_internal.h"
#include "esperanto_gb300.h"
#include "host_pool.h"

struct esp_handle {
    std::unique_ptr<HostPool> pool;  // host scan threads, started on first use
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host-batch pipelining (created on first use)
    std::string err;
    uint64_t launches = 0;
    int gotoh_bps[esp::kGotohVariants] = {};  // resident DP blocks per SM (queried once)
    int variant = -1;   // DP kernel variant; -1 = ESP_GOTOH_VARIANT env or default
    bool variant_by_size = false;  // default variant: large band batches run paired
    int hint_variant = -2;  // variant of hint-mode batches: >= 0 forced (ESP_GOTOH_HINT_VARIANT),
                            // -1 by batch size (abi.cu hint_variant), -2 = env not read yet
    long warp_max = -1; // batches of at most this many pairs run warp-per-pair; -1 = ESP_WARP_MAX or 2048
    // CUDA graph of the last device batch: an identical submission (same
    // buffers, sizes, parameters, stream, kernel choices and scratch
    // generation) replays it instead of re-issuing its launches
    uint64_t buf_gen = 0;
    std::vector<uint64_t> graph_key, seen_key;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_launches = 0;
    int use_graphs = -1;  // -1 = ESP_GRAPHS env (default on)
    uint64_t scratch_budget = 8ull << 30;  // bytes of DP scratch one launch may use
    // d_tb / d_rb (with their caps) are a region the owner placed there, not
    // the handle's own: launches check them instead of growing them
    bool scratch_external = false;
    // grow-only device buffers
    void *d_in = nullptr;       // per-call staging: pair | n intervals | arena
    size_t d_in_cap = 0;
    void *d_res = nullptr;      // per-call results: esp_extension | cigar
    size_t d_res_cap = 0;
    uint32_t *d_tb = nullptr;
    size_t d_tb_cap = 0;        // bytes
    uint32_t *d_rb = nullptr;
    size_t d_rb_cap = 0;
    uint32_t *d_esc = nullptr;  // escalation list
    size_t d_esc_cap = 0;       // bytes
    uint32_t *d_wide = nullptr; // pairs outside the int16 domain (the wide kernel's list)
    size_t d_wide_cap = 0;      // bytes
    // d_ctr (256 B): u64 queues at [0..1] (attempt 1), [2..3] (attempt 2),
    // u32 esc count at [4], u64 class queues at [8..15], class bounds at
    // [24..28], binned list length at [29], wide-list count at [30], binned
    // escalation list length at [31]
    uint32_t *d_ctr = nullptr;
    int tune[esp::kLengthClasses] = {-1, -1, -1, -1};  // DP variant per length class (autotuned)
    bool tuned = false;
    double *autotune_ms = nullptr;  // set by esp_batch_autotune: time the classes instead
    uint32_t *d_hist = nullptr; // geometry bins
    size_t d_hist_cap = 0;
    uint32_t *d_order = nullptr;  // length-binned work list
    size_t d_order_cap = 0;
    bool binning = true;
    // host pinned staging
    void *h_in = nullptr;
    size_t h_in_cap = 0;
    void *h_res = nullptr;
    size_t h_res_cap = 0;
    // host batch staging for esp_batch_extend_host
    void *d_bat = nullptr;
    size_t d_bat_cap = 0;
    uint64_t last_cells = 0;    // DP cells of the last splice batch
    // splice batch scratch
    void *d_spl = nullptr;
    size_t d_spl_cap = 0;
    void *d_spl_io = nullptr;   // host-API staging of reads / candidates / results
    size_t d_spl_io_cap = 0;
    void *d_int = nullptr;      // intron-chain batch staging
    size_t d_int_cap = 0;
    // Myers per-call / batch staging
    void *d_my = nullptr;
    size_t d_my_cap = 0;
    void *h_my = nullptr;
    size_t h_my_cap = 0;
};

inline int fail(esp_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

inline int cuda_fail(esp_handle *h, cudaError_t e, const char *what) {
    return fail(h, ESP_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, expr)                                        \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) return cuda_fail(h, _e, #expr); \
    } while (0)

inline int grow_device(esp_handle *h, void **p, size_t *cap, size_t need) {
    if (need <= *cap) return ESP_OK;
    if (h) h->buf_gen++;  // buffers move: a captured launch graph is stale
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t sz = std::max(need, (size_t)4096);
    cudaError_t e = cudaMalloc(p, sz);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(h, ESP_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    *cap = sz;
    return ESP_OK;
}

inline int grow_host(esp_handle *h, void **p, size_t *cap, size_t need) {
    if (need <= *cap) return ESP_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    size_t sz = std::max(need * 2, (size_t)65536);
    cudaError_t e = cudaMallocHost(p, sz);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(h, ESP_ENOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    *cap = sz;
    return ESP_OK;
}

// extend.rs:150-159 base_code folded to the 2-bit arena plus N intervals.
inline int ascii_code(uint8_t b) {
    switch (b) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

// Append `len` ASCII bases at arena base position `pos` and their N runs.
inline void encode_seq(const uint8_t *s, size_t len, uint8_t *arena, uint64_t pos,
                std::vector<esp_n_interval> &iv) {
    size_t k = 0;
    while (k < len) {
        int c = ascii_code(s[k]);
        if (c == 4) {
            size_t e = k;
            while (e < len && ascii_code(s[e]) == 4) e++;
            iv.push_back({(uint32_t)k, (uint32_t)e});
            k = e;
            continue;
        }
        uint64_t p = pos + k;
        arena[p >> 2] |= (uint8_t)(c << (6 - 2 * (p & 3)));
        k++;
    }
}


struct Limits {
    uint64_t tb_words = 1, rb_words = 1;
    uint32_t max_m = 0;
};

// The handle's host worker pool (up to 16 threads with the caller).
inline HostPool &host_pool(esp_handle *h) {
    if (!h->pool) {
        unsigned T = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        h->pool.reset(new HostPool(T - 1));
    }
    return *h->pool;
}

inline void add_limits(Limits &L, uint32_t m, uint32_t n, int32_t half) {
    uint64_t tb, rb;
    esp::gotoh_scratch_words(m, n, half, tb, rb);
    L.tb_words = std::max(L.tb_words, tb);
    L.rb_words = std::max(L.rb_words, rb);
    L.max_m = std::max(L.max_m, m);
}


// Enqueue the DP launches of one batch whose inputs are on the device
// (abi.cu).  Windows come from d_win_arena when it is not null.
int enqueue_batch(esp_handle *h, int mode, const esp_pair *d_pairs, uint64_t n_pairs,
                  const uint8_t *d_arena, uint64_t arena_bytes, const esp_n_interval *d_iv,
                  uint64_t n_iv, const esp::GotohConst &K, const Limits &L1, const Limits &L2,
                  esp_extension *d_out, uint32_t *d_cigar, uint32_t cigar_stride,
                  cudaStream_t st, const uint8_t *d_win_arena = nullptr,
                  uint64_t win_arena_bytes = 0);

// Resident genome (esp_genome_create): device arena + contig table + N table,
// with host copies of the small tables for host-side validation.
struct esp_genome {
    int device = 0;
    uint8_t *d_arena = nullptr;
    uint64_t arena_bytes = 0;
    esp_contig *d_contigs = nullptr;
    std::vector<esp_contig> contigs;
    esp_n_interval *d_iv = nullptr;
    uint64_t n_iv = 0;
    std::vector<esp_n_interval> h_iv;  // host copy (serve-loop window clipping)
};

// Bytes of traceback and row-buffer scratch one enqueue_batch of n_pairs
// uses on this handle (the kernel, warps and words it would choose; abi.cu).
void dp_scratch_bytes(esp_handle *h, int mode, uint64_t n_pairs, const Limits &L1,
                      const Limits &L2, uint64_t &tb_bytes, uint64_t &rb_bytes);

// Grow a handle's escalation and binning lists once for one-pair-kernel
// batches of up to max_pairs pairs (abi.cu), so later batches of that size
// allocate nothing but their DP scratch.
int reserve_lists(esp_handle *h, uint64_t max_pairs);

// The spliced pseudo-reference DP over exon slices (spliced.cu): gather the
// pseudo-references from the genome, extend_hint along each read's hint
// diagonal (hint_offset[r], or 0 when null), stitch back to the genome.
int spliced_batch(esp_handle *h, const esp_genome *g, const esp_spliced_read *reads, uint64_t n,
                  const uint8_t *read_arena, uint64_t read_arena_bytes,
                  const esp_n_interval *read_iv, uint64_t n_read_iv, const esp_exon *exons,
                  uint64_t n_exons, const esp_extend_params *params, const int64_t *hint_offset,
                  esp_spliced_result *out, uint32_t *ext_cigar, uint32_t *stitched_cigar,
                  uint32_t cigar_stride);
