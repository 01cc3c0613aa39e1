// abi.cu -- the C ABI: handles, the per-call drop-ins of extend.rs and the
// batch-submit API.  Host-side code only; kernels live in gotoh.cu etc.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "esp_host.h"

// Kernel variant of a handle that was neither set nor tuned: the
// ESP_GOTOH_VARIANT environment variable (0..3), else 1 -- and then band
// batches of 2^20 pairs and more take the paired kernel (band_variant).
static int default_variant(bool *by_size = nullptr) {
    const char *v = getenv("ESP_GOTOH_VARIANT");
    const bool env = v && v[0] >= '0' && v[0] < '0' + esp::kGotohVariants && !v[1];
    if (by_size) *by_size = !env;
    return env ? v[0] - '0' : 1;
}

static void resolve_variant(esp_handle *h) {
    if (h->variant < 0) h->variant = default_variant(&h->variant_by_size);
}

// Variant of an untuned band batch of n pairs: the handle's, except that a
// handle left at the default runs batches of 2^20 pairs and more on the
// paired kernel (the mixed-length workload: 1,054 vs ~900 GCUPS at 2^20
// pairs, 1,148 vs 930 at 2^22; at 2^18 the one-pair kernel wins, 738 vs
// 397).  esp_batch_autotune measures instead of assuming.
static int band_variant(esp_handle *h, uint64_t n) {
    resolve_variant(h);
    if (h->variant_by_size && h->binning && n >= (1u << 20)) return 3;
    return h->variant;
}

// Kernel variant of a hint-mode batch of n pairs.  Hint batches repeat one
// geometry when their windows are cut the same way (the splice flanks: read
// segment vs segment + 30 bases at offset 0), so from 2^20 pairs on they run
// the paired kernel (measured: the 69M-pair splice flank batch 1,063 vs 974
// GCUPS); smaller ones cannot fill the GPU with two-pair items (a 65,536-pair
// batch 3.94 vs 3.14 ms, the serve loop's requests 16.0 vs 22.5 M pairs/s
// peak) and run one pair per thread.  ESP_GOTOH_HINT_VARIANT (0..3)
// overrides.
static int hint_variant(esp_handle *h, uint64_t n) {
    if (h->hint_variant < -1) {
        const char *v = getenv("ESP_GOTOH_HINT_VARIANT");
        h->hint_variant =
            (v && v[0] >= '0' && v[0] < '0' + esp::kGotohVariants && !v[1]) ? v[0] - '0' : -1;
    }
    if (h->hint_variant >= 0) return h->hint_variant;
    if (h->binning && n >= (1u << 20)) return 3;
    resolve_variant(h);
    return esp::gotoh_paired(h->variant) ? h->variant - 2 : h->variant;
}

// Whether a band batch of n pairs runs a paired kernel (set, by size, or
// chosen by autotuning for any length class).
static bool band_paired(esp_handle *h, uint64_t n) {
    if (!h->binning) return false;
    if (h->tuned) {
        for (int s = 0; s < esp::kLengthClasses; s++)
            if (esp::gotoh_paired(h->tune[s])) return true;
        return false;
    }
    return esp::gotoh_paired(band_variant(h, n));
}

// How one batch of n_pairs uses DP scratch: which kernel runs, with how
// many warps, and the traceback / row-buffer bytes they need (the choices
// enqueue_batch makes; the serve loop charges launches with it).
struct DpPlan {
    bool warp_kernel = false;
    int var = 1;             // thread-kernel variant
    bool per_class = false;  // one launch per length class of the binned list
    bool paired = false;     // a two-pairs-per-thread variant is among the launches
    uint64_t warps = 0;
    uint64_t tbw = 0, rbw = 0;  // words per thread (warp kernel: per warp)
    uint64_t tb_bytes = 0, rb_bytes = 0;
};

static DpPlan plan_dp(esp_handle *h, int mode, uint64_t n_pairs, const Limits &L1,
                      const Limits &L2) {
    DpPlan P;
    if (h->warp_max < 0) {
        const char *v = getenv("ESP_WARP_MAX");
        h->warp_max = v ? atol(v) : 2048;
    }
    P.tbw = std::max(L1.tb_words, mode == ESP_MODE_HINT ? L2.tb_words : 0);
    P.rbw = std::max(L1.rb_words, mode == ESP_MODE_HINT ? L2.rb_words : 0);
    if (n_pairs <= (uint64_t)h->warp_max) {
        // Few pairs: one warp per pair (the wavefront kernel), so a lone
        // pair is not latency-bound on a single thread.
        P.warp_kernel = true;
        uint64_t per_warp_bytes = (P.tbw + P.rbw) * 4;
        uint64_t warps = std::min<uint64_t>(n_pairs, (uint64_t)h->num_sms * 12);
        warps = std::min(warps, std::max<uint64_t>(1, h->scratch_budget / per_warp_bytes));
        P.warps = (warps + 3) / 4 * 4;  // whole blocks: every launched warp owns its scratch
        P.tb_bytes = P.warps * per_warp_bytes;
        return P;
    }
    // scratch slots: one warp per 32 pairs up to the resident limit, bounded
    // by the scratch budget
    uint64_t per_warp_bytes = (P.tbw + P.rbw) * 32 * 4;
    resolve_variant(h);
    // the paired kernels need neighbours of the binned list with one band
    // geometry
    auto usable = [&](int v) {
        return esp::gotoh_paired(v) && (mode != ESP_MODE_BAND || !h->binning) ? v - 2 : v;
    };
    int var = mode == ESP_MODE_HINT ? hint_variant(h, n_pairs) : usable(band_variant(h, n_pairs));
    // autotuned handle: one variant for every class runs as a single launch
    bool tuned_split = false;
    if (h->tuned && mode == ESP_MODE_BAND) {
        for (int s = 1; s < esp::kLengthClasses; s++) tuned_split |= h->tune[s] != h->tune[0];
        if (!tuned_split && h->tune[0] >= 0) var = usable(h->tune[0]);
    }
    // the binned list runs per length class when the handle is autotuned (or
    // is being tuned); scratch then covers the widest variant in use
    P.per_class = (tuned_split || h->autotune_ms) && h->binning && n_pairs > 32;
    int max_bps = 0;
    for (int v = 0; v < esp::kGotohVariants; v++) {
        bool used = v == var;
        if (P.per_class)
            for (int s = 0; s < esp::kLengthClasses; s++) used |= h->autotune_ms || h->tune[s] == v;
        if (!used) continue;
        if (h->gotoh_bps[v] == 0) h->gotoh_bps[v] = esp::gotoh_blocks_per_sm(128, v);
        max_bps = std::max(max_bps, h->gotoh_bps[v]);
        P.paired |= esp::gotoh_paired(v);
    }
    P.var = var;
    const uint64_t slot_pairs = P.paired ? 2 : 1;  // scratch slots per lane
    uint64_t want = std::max<uint64_t>(1, (uint64_t)h->num_sms * max_bps * 4);
    uint64_t need_warps = (n_pairs + 31) / 32;
    uint64_t warps = std::min(want, need_warps);
    uint64_t budget_warps = std::max<uint64_t>(1, h->scratch_budget / (per_warp_bytes * slot_pairs));
    warps = std::min(warps, budget_warps);
    P.warps = (warps + 3) / 4 * 4;  // whole 128-thread blocks: every launched warp owns a slot
    P.tb_bytes = P.warps * slot_pairs * P.tbw * 32 * 4;
    P.rb_bytes = P.warps * slot_pairs * P.rbw * 32 * 4;
    return P;
}

void dp_scratch_bytes(esp_handle *h, int mode, uint64_t n_pairs, const Limits &L1,
                      const Limits &L2, uint64_t &tb_bytes, uint64_t &rb_bytes) {
    const DpPlan P = plan_dp(h, mode, n_pairs, L1, L2);
    tb_bytes = P.tb_bytes;
    rb_bytes = P.rb_bytes;
}

// The traceback and row-buffer scratch of a plan (tb at least tb_min
// bytes): grown in the handle, or checked against the region the owner
// placed there (scratch_external).
static int scratch_for(esp_handle *h, const DpPlan &P, uint64_t tb_min) {
    const uint64_t tb = std::max(P.tb_bytes, tb_min);
    if (h->scratch_external) {
        if (tb > h->d_tb_cap || P.rb_bytes > h->d_rb_cap)
            return fail(h, ESP_ENOMEM, "DP scratch region too small for the launch");
        return ESP_OK;
    }
    int rc = grow_device(h, (void **)&h->d_tb, &h->d_tb_cap, tb);
    if (rc == ESP_OK && P.rb_bytes)
        rc = grow_device(h, (void **)&h->d_rb, &h->d_rb_cap, P.rb_bytes);
    return rc;
}

// Enqueue the DP launches of one batch whose inputs are on the device.
int enqueue_batch(esp_handle *h, int mode, const esp_pair *d_pairs, uint64_t n_pairs,
                  const uint8_t *d_arena, uint64_t arena_bytes, const esp_n_interval *d_iv,
                  uint64_t n_iv, const esp::GotohConst &K, const Limits &L1, const Limits &L2,
                  esp_extension *d_out, uint32_t *d_cigar, uint32_t cigar_stride,
                  cudaStream_t st, const uint8_t *d_win_arena, uint64_t win_arena_bytes) {
    h->launches = 0;
    if (n_pairs == 0) return ESP_OK;
    // list positions are u32, with up to 2^20 padding slots
    if (n_pairs > 0xffffffffull - (1ull << 21)) return fail(h, ESP_EINVAL, "batch too large");
    int rc;
    // Reads whose scores can leave the int16 domain: the int16 kernels list
    // such pairs and the wide kernel runs them afterwards (int32, one warp
    // per pair, both extend_hint attempts in-kernel), in the same scratch.
    // The int16 kernels' scratch then covers reads up to K.max_m only.
    const uint32_t max_m = std::max(L1.max_m, mode == ESP_MODE_HINT ? L2.max_m : 0u);
    const bool wide = max_m > (uint32_t)K.max_m;
    Limits N1 = L1, N2 = L2;
    if (wide) {
        const uint64_t strips = ((uint64_t)K.max_m + 7) / 8;
        for (Limits *N : {&N1, &N2}) {
            N->tb_words = std::min<uint64_t>(N->tb_words, strips * N->rb_words);
            N->max_m = std::min<uint32_t>(N->max_m, (uint32_t)K.max_m);
        }
    }
    const DpPlan P = plan_dp(h, mode, n_pairs, N1, N2);
    uint64_t wide_warps = 0, wide_bytes = 0, wide_tbw = 0, wide_rbw = 0;
    if (wide) {
        wide_tbw = std::max(L1.tb_words, mode == ESP_MODE_HINT ? L2.tb_words : 0);
        wide_rbw = std::max(L1.rb_words, mode == ESP_MODE_HINT ? L2.rb_words : 0);
        const uint64_t per_warp = (wide_tbw + 2 * wide_rbw) * 4;
        wide_warps = std::min<uint64_t>({n_pairs, (uint64_t)h->num_sms * 4,
                                         std::max<uint64_t>(1, h->scratch_budget / per_warp)});
        wide_warps = (wide_warps + 3) / 4 * 4;  // whole blocks: every warp owns its scratch
        wide_bytes = wide_warps * per_warp;
        if ((rc = grow_device(h, (void **)&h->d_wide, &h->d_wide_cap, n_pairs * 4)) != ESP_OK)
            return rc;
    }
    if ((rc = scratch_for(h, P, wide_bytes)) != ESP_OK) return rc;
    auto launch_wide = [&](const esp::GotohJob &base) -> int {
        if (!wide) return ESP_OK;
        esp::GotohJob jw = base;
        jw.list = h->d_wide;
        jw.list_count = h->d_ctr + 30;
        jw.range = nullptr;
        jw.mode = mode == ESP_MODE_HINT ? 1 : 0;
        jw.tb = h->d_tb;
        jw.tb_words = wide_tbw;
        jw.rb_words = wide_rbw;
        jw.wide_list = nullptr;
        jw.wide_count = nullptr;
        CK(h, esp::launch_gotoh_wide(jw, K, (int)wide_warps, st));
        h->launches++;
        return ESP_OK;
    };
    if (P.warp_kernel) {
        if (mode == ESP_MODE_HINT &&
            (rc = grow_device(h, (void **)&h->d_esc, &h->d_esc_cap, n_pairs * sizeof(uint32_t))) != ESP_OK)
            return rc;
        CK(h, cudaMemsetAsync(h->d_ctr, 0, 256, st));
        esp::GotohJob job{};
        job.pairs = d_pairs;
        job.n_pairs = n_pairs;
        job.arena = d_arena;
        job.arena_bases = arena_bytes * 4;
        job.win_arena = d_win_arena;
        job.win_arena_bases = win_arena_bytes * 4;
        job.n_iv = d_iv;
        job.n_iv_count = n_iv;
        job.out = d_out;
        job.cigar = d_cigar;
        job.cigar_stride = cigar_stride;
        job.tb = h->d_tb;
        job.tb_words = P.tbw;
        job.rb_words = P.rbw;
        job.esc_list = h->d_esc;
        job.esc_count = h->d_ctr + 4;
        job.mode = mode == ESP_MODE_HINT ? 1 : 0;
        job.wide_list = wide ? h->d_wide : nullptr;
        job.wide_count = h->d_ctr + 30;
        CK(h, esp::launch_gotoh_warp(job, K, (int)P.warps, st));
        h->launches++;
        if (mode == ESP_MODE_HINT) {
            esp::GotohJob j2 = job;
            j2.mode = 2;
            j2.list = h->d_esc;
            j2.list_count = h->d_ctr + 4;
            CK(h, esp::launch_gotoh_warp(j2, K, (int)P.warps, st));
            h->launches++;
        }
        return launch_wide(job);
    }
    const uint64_t tbw = P.tbw, rbw = P.rbw, warps = P.warps;
    const int var = P.var;
    const bool per_class = P.per_class, paired = P.paired;
    if (mode == ESP_MODE_HINT &&
        (rc = grow_device(h, (void **)&h->d_esc, &h->d_esc_cap, n_pairs * sizeof(uint32_t))) != ESP_OK)
        return rc;
    CK(h, cudaMemsetAsync(h->d_ctr, 0, 256, st));
    const uint32_t *order = nullptr;
    const uint32_t *list_len = nullptr;  // device word: length of a padded list
    if (h->binning && n_pairs > 32) {
        // the paired kernels want each geometry bin at an even list offset
        const uint64_t slots = n_pairs + (paired ? esp::bin_pad_slots(n_pairs) : 0);
        if ((rc = grow_device(h, (void **)&h->d_hist, &h->d_hist_cap, esp::bin_scratch_bytes())) != ESP_OK)
            return rc;
        if ((rc = grow_device(h, (void **)&h->d_order, &h->d_order_cap, slots * sizeof(uint32_t))) != ESP_OK)
            return rc;
        CK(h, esp::launch_binning(d_pairs, n_pairs, mode == ESP_MODE_HINT ? 1 : 0, h->d_hist,
                                  h->d_order, h->num_sms, st, h->d_ctr + 29,
                                  per_class ? h->d_ctr + 24 : nullptr, paired));
        h->launches += 5 + (per_class ? 1 : 0);  // kernels; the memsets are not counted
        order = h->d_order;
        if (paired) list_len = h->d_ctr + 29;
    }
    esp::GotohJob job{};
    job.list = order;
    job.list_count = list_len;
    job.pairs = d_pairs;
    job.n_pairs = n_pairs;
    job.arena = d_arena;
    job.arena_bases = arena_bytes * 4;
    job.win_arena = d_win_arena;
    job.win_arena_bases = win_arena_bytes * 4;
    job.n_iv = d_iv;
    job.n_iv_count = n_iv;
    job.out = d_out;
    job.cigar = d_cigar;
    job.cigar_stride = cigar_stride;
    job.tb = h->d_tb;
    job.tb_words = tbw;
    job.rb = h->d_rb;
    job.rb_words = rbw;
    job.queue = h->d_ctr;
    job.esc_list = h->d_esc;
    job.esc_count = h->d_ctr + 4;
    job.mode = mode == ESP_MODE_HINT ? 1 : 0;
    job.wide_list = wide ? h->d_wide : nullptr;
    job.wide_count = h->d_ctr + 30;
    if (per_class && h->autotune_ms) {
        // time every variant on every length class and, as row
        // kLengthClasses, on the whole list in one launch (best of two runs
        // each); the batch's results are those of the last run
        cudaEvent_t ev[2];
        CK(h, cudaEventCreate(&ev[0]));
        CK(h, cudaEventCreate(&ev[1]));
        for (int s = 0; s <= esp::kLengthClasses; s++)
            for (int v = 0; v < esp::kGotohVariants; v++) {
                double best = 1e30;
                for (int rep = 0; rep < 2; rep++) {
                    esp::GotohJob js = job;
                    if (s < esp::kLengthClasses) {
                        js.range = h->d_ctr + 24 + s;
                        js.queue = h->d_ctr + 8 + 2 * s;
                    }
                    CK(h, cudaMemsetAsync(js.queue, 0, 8, st));
                    // every timed run lists the wide pairs anew
                    CK(h, cudaMemsetAsync(h->d_ctr + 30, 0, 4, st));
                    CK(h, cudaEventRecord(ev[0], st));
                    CK(h, esp::launch_gotoh(js, K, (int)warps, 128, st, v));
                    CK(h, cudaEventRecord(ev[1], st));
                    CK(h, cudaEventSynchronize(ev[1]));
                    float ms = 0;
                    CK(h, cudaEventElapsedTime(&ms, ev[0], ev[1]));
                    best = std::min(best, (double)ms);
                }
                h->autotune_ms[s * esp::kGotohVariants + v] = best;
            }
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
    } else if (per_class) {
        for (int s = 0; s < esp::kLengthClasses; s++) {
            esp::GotohJob js = job;
            js.range = h->d_ctr + 24 + s;
            js.queue = h->d_ctr + 8 + 2 * s;
            CK(h, esp::launch_gotoh(js, K, (int)warps, 128, st, h->tune[s] >= 0 ? h->tune[s] : var));
            h->launches++;
        }
    } else {
        CK(h, esp::launch_gotoh(job, K, (int)warps, 128, st, var));
        h->launches++;
    }
    if (mode == ESP_MODE_HINT) {
        // extend_hint's second attempt (full matrix) over the escalations,
        // binned by their full-matrix geometry like the first attempt's
        // list (the first attempt is done with the binned list and its
        // histogram by now)
        esp::GotohJob j2 = job;
        j2.mode = 2;
        j2.list = h->d_esc;
        j2.list_count = h->d_ctr + 4;
        j2.queue = h->d_ctr + 2;
        if (order) {
            CK(h, esp::launch_binning(d_pairs, n_pairs, 2, h->d_hist, h->d_order, h->num_sms, st,
                                      h->d_ctr + 31, nullptr, paired, h->d_esc, h->d_ctr + 4));
            h->launches += 5;
            j2.list = h->d_order;
            j2.list_count = paired ? h->d_ctr + 31 : h->d_ctr + 4;
        }
        CK(h, esp::launch_gotoh(j2, K, (int)warps, 128, st, var));
        h->launches++;
    }
    return launch_wide(job);
}



int reserve_lists(esp_handle *h, uint64_t max_pairs) {
    int rc;
    if ((rc = grow_device(h, (void **)&h->d_esc, &h->d_esc_cap, max_pairs * 4)) != ESP_OK) return rc;
    if ((rc = grow_device(h, (void **)&h->d_hist, &h->d_hist_cap, esp::bin_scratch_bytes())) != ESP_OK)
        return rc;
    return grow_device(h, (void **)&h->d_order, &h->d_order_cap, max_pairs * 4);
}

extern "C" {

int esp_create(esp_handle **out, int device) {
    if (!out) return ESP_EINVAL;
    *out = nullptr;
    esp_handle *h = new (std::nothrow) esp_handle();
    if (!h) return ESP_ENOMEM;
    h->device = device;
    // DP scratch one launch may use: ESP_SCRATCH_BUDGET bytes, else 8 GiB
    // (fewer resident warps when a batch's geometry needs more)
    if (const char *v = getenv("ESP_SCRATCH_BUDGET")) {
        const unsigned long long b = strtoull(v, nullptr, 10);
        if (b >= (1ull << 20)) h->scratch_budget = b;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_ctr, 256);
    if (e != cudaSuccess) {
        delete h;
        return ESP_ECUDA;
    }
    *out = h;
    return ESP_OK;
}

int esp_set_warp_max(esp_handle *h, long warp_max) {
    if (!h || warp_max < 0) return ESP_EINVAL;
    h->warp_max = warp_max;
    return ESP_OK;
}

int esp_set_kernel_variant(esp_handle *h, int variant) {
    if (!h || variant < -1 || variant >= esp::kGotohVariants) return ESP_EINVAL;
    h->variant = variant;
    h->variant_by_size = false;  // a -1 is resolved again at the next batch
    h->tuned = false;
    for (int s = 0; s < esp::kLengthClasses; s++) h->tune[s] = -1;
    return ESP_OK;
}

int esp_destroy(esp_handle *h) {
    if (!h) return ESP_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    cudaFree(h->d_in);
    cudaFree(h->d_res);
    if (!h->scratch_external) {
        cudaFree(h->d_tb);
        cudaFree(h->d_rb);
    }
    cudaFree(h->d_esc);
    cudaFree(h->d_wide);
    cudaFree(h->d_ctr);
    cudaFree(h->d_bat);
    cudaFree(h->d_my);
    cudaFree(h->d_spl);
    cudaFree(h->d_spl_io);
    cudaFree(h->d_int);
    if (h->h_my) cudaFreeHost(h->h_my);
    cudaFree(h->d_hist);
    cudaFree(h->d_order);
    if (h->h_in) cudaFreeHost(h->h_in);
    if (h->h_res) cudaFreeHost(h->h_res);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return ESP_OK;
}

const char *esp_last_error(const esp_handle *h) { return h ? h->err.c_str() : "null handle"; }

void *esp_stream(esp_handle *h) { return h ? (void *)h->stream : nullptr; }

uint64_t esp_last_launch_count(const esp_handle *h) { return h ? h->launches : 0; }

}  // extern "C"

// One pair from ASCII through the device path (the per-call drop-in).
static int one_pair(esp_handle *h, int mode, const uint8_t *read, size_t m, const uint8_t *win,
                    size_t n, const esp_extend_params *params, int64_t offset, int64_t half,
                    esp_extension *out, uint32_t *cigar, uint32_t cap) {
    if (!h || !params || !out || (m && !read) || (n && !win)) return fail(h, ESP_EINVAL, "null argument");
    if (m > 32767 || n > 32767) return fail(h, ESP_EDOMAIN, "sequence longer than 32767");
    if (offset < -(1ll << 30) || offset > (1ll << 30)) return fail(h, ESP_EDOMAIN, "band offset out of range");
    if (half > (1ll << 30)) half = 1ll << 30;
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    CK(h, cudaSetDevice(h->device));
    std::vector<esp_n_interval> iv;
    uint64_t wpos = ((m + 63) / 64) * 64;  // window starts on a 16-byte boundary
    uint64_t bases = wpos + n;
    size_t arena_bytes = ((bases + 3) / 4 + 15) / 16 * 16 + 16;
    size_t hdr = 64 + 8 * (m + n + 2);  // pair + worst-case N intervals
    hdr = (hdr + 255) / 256 * 256;
    int rc;
    if ((rc = grow_host(h, &h->h_in, &h->h_in_cap, hdr + arena_bytes)) != ESP_OK) return rc;
    uint8_t *hin = (uint8_t *)h->h_in;
    uint8_t *harena = hin + hdr;
    memset(harena, 0, arena_bytes);
    encode_seq(read, m, harena, 0, iv);
    size_t n_read_iv = iv.size();
    encode_seq(win, n, harena, wpos, iv);
    esp_pair P{};
    P.read_pos = 0;
    P.win_pos = wpos;
    P.read_len = (uint32_t)m;
    P.win_len = (uint32_t)n;
    P.band_offset = (int32_t)offset;
    P.band_half = half < 0 ? -1 : (int32_t)half;
    P.n_first = 0;
    if (n_read_iv > 65535 || iv.size() - n_read_iv > 65535)
        return fail(h, ESP_EDOMAIN, "too many N runs");
    P.n_read = (uint16_t)n_read_iv;
    P.n_win = (uint16_t)(iv.size() - n_read_iv);
    memcpy(hin, &P, sizeof(P));
    if (!iv.empty()) memcpy(hin + 64, iv.data(), iv.size() * sizeof(esp_n_interval));
    if ((rc = grow_device(h, &h->d_in, &h->d_in_cap, hdr + arena_bytes)) != ESP_OK) return rc;
    uint32_t stride = std::max<uint32_t>(cap, 1) + 8;
    size_t res_bytes = 64 + (size_t)stride * 4;
    if ((rc = grow_device(h, &h->d_res, &h->d_res_cap, res_bytes)) != ESP_OK) return rc;
    if ((rc = grow_host(h, &h->h_res, &h->h_res_cap, res_bytes)) != ESP_OK) return rc;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(h->d_in, hin, hdr + arena_bytes, cudaMemcpyHostToDevice, st));
    uint8_t *din = (uint8_t *)h->d_in;
    Limits L1, L2;
    if (mode == ESP_MODE_HINT) {
        add_limits(L1, (uint32_t)m, (uint32_t)n, 30);
        add_limits(L2, (uint32_t)m, (uint32_t)n, -1);
    } else {
        add_limits(L1, (uint32_t)m, (uint32_t)n, P.band_half);
    }
    esp_extension *dout = (esp_extension *)h->d_res;
    uint32_t *dcig = (uint32_t *)((uint8_t *)h->d_res + 64);
    rc = enqueue_batch(h, mode, (const esp_pair *)din, 1, din + hdr, arena_bytes - 16,
                       (const esp_n_interval *)(din + 64), iv.size(), K, L1, L2, dout, dcig,
                       stride, st);
    if (rc != ESP_OK) return rc;
    CK(h, cudaMemcpyAsync(h->h_res, h->d_res, res_bytes, cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    esp_extension r;
    memcpy(&r, h->h_res, sizeof(r));
    if (r.status == ESP_EINVAL) return fail(h, ESP_EINVAL, "kernel refused the pair");
    *out = r;
    uint32_t k = std::min<uint32_t>(r.n_ops, cap);
    if (r.status == ESP_OK && cigar && k) memcpy(cigar, (uint8_t *)h->h_res + 64, k * 4);
    if (r.n_ops > cap) {
        out->status = ESP_ECAP;
        return fail(h, ESP_ECAP, "CIGAR buffer too small");
    }
    return ESP_OK;
}

extern "C" {

int esp_extend(esp_handle *h, const uint8_t *read, size_t read_len, const uint8_t *ref_window,
               size_t window_len, const esp_extend_params *params, esp_extension *out,
               uint32_t *cigar, uint32_t cigar_cap) {
    return one_pair(h, ESP_MODE_BAND, read, read_len, ref_window, window_len, params, 0, -1, out,
                    cigar, cigar_cap);
}

int esp_extend_hint(esp_handle *h, const uint8_t *read, size_t read_len,
                    const uint8_t *ref_window, size_t window_len,
                    const esp_extend_params *params, int64_t hint_offset, uint32_t hint_num,
                    uint32_t hint_den, esp_extension *out, uint32_t *cigar,
                    uint32_t cigar_cap) {
    // run_band asserts num == den == 1 (extend.rs:633); den 0 counts as 1.
    if (hint_num != 1 || (hint_den > 1)) return fail(h, ESP_EINVAL, "DiagHint slope must be 1/1");
    return one_pair(h, ESP_MODE_HINT, read, read_len, ref_window, window_len, params, hint_offset,
                    30, out, cigar, cigar_cap);
}

int esp_score_tail_win(esp_handle *h, const uint8_t *tail, size_t tail_len,
                       const uint8_t *ref_window, size_t window_len,
                       const esp_extend_params *params, esp_extension *out, uint32_t *cigar,
                       uint32_t cigar_cap) {
    return one_pair(h, ESP_MODE_HINT, tail, tail_len, ref_window, window_len, params, 0, 30, out,
                    cigar, cigar_cap);
}

int esp_run_band(esp_handle *h, const uint8_t *read, size_t read_len, const uint8_t *ref_window,
                 size_t window_len, const esp_extend_params *params, int64_t band_offset,
                 int64_t band_half, esp_extension *out, uint32_t *cigar, uint32_t cigar_cap) {
    return one_pair(h, ESP_MODE_BAND, read, read_len, ref_window, window_len, params,
                    band_half < 0 ? 0 : band_offset, band_half, out, cigar, cigar_cap);
}

// Scratch limits of a host batch (and, per chunk, the highest arena base
// its pairs touch).  Large batches are scanned by several host threads: one
// core streams ~8 GB/s, the 40-byte records of millions of pairs would
// otherwise dominate the end-to-end time.
struct ScanOut {
    Limits L1, L2;
    uint64_t arena_end = 0;
};

static void scan_range(int mode, const esp_pair *pairs, uint64_t a, uint64_t b, ScanOut &S) {
    for (uint64_t k = a; k < b; k++) {
        const esp_pair &P = pairs[k];
        if (mode == ESP_MODE_HINT) {
            add_limits(S.L1, P.read_len, P.win_len, P.win_len <= 30 ? -1 : 30);
            add_limits(S.L2, P.read_len, P.win_len, -1);
        } else {
            add_limits(S.L1, P.read_len, P.win_len, P.band_half);
        }
        S.arena_end = std::max({S.arena_end, P.read_pos + P.read_len, P.win_pos + P.win_len});
    }
}

static void merge(ScanOut &into, const ScanOut &s) {
    into.L1.tb_words = std::max(into.L1.tb_words, s.L1.tb_words);
    into.L1.rb_words = std::max(into.L1.rb_words, s.L1.rb_words);
    into.L1.max_m = std::max(into.L1.max_m, s.L1.max_m);
    into.L2.tb_words = std::max(into.L2.tb_words, s.L2.tb_words);
    into.L2.rb_words = std::max(into.L2.rb_words, s.L2.rb_words);
    into.L2.max_m = std::max(into.L2.max_m, s.L2.max_m);
    into.arena_end = std::max(into.arena_end, s.arena_end);
}

// Per-chunk scans (chunk c = pairs [bounds[c], bounds[c+1])), in parallel
// on the handle's host pool for batches of 32K pairs and more.
static void scan_chunks(esp_handle *h, int mode, const esp_pair *pairs,
                        const std::vector<uint64_t> &bounds, std::vector<ScanOut> &out) {
    const size_t C = bounds.size() - 1;
    out.assign(C, ScanOut{});
    const uint64_t n = bounds.back();
    unsigned T = n < (1u << 15) ? 1 : (unsigned)std::min<uint64_t>(16, n >> 14);
    if (T > 1) T = std::min(T, host_pool(h).size());
    // split every chunk into T slices; each worker scans slice t of every chunk
    std::vector<std::vector<ScanOut>> part(T, std::vector<ScanOut>(C));
    auto work = [&](unsigned t) {
        for (size_t c = 0; c < C; c++) {
            uint64_t a = bounds[c], b = bounds[c + 1], len = b - a;
            scan_range(mode, pairs, a + len * t / T, a + len * (t + 1) / T, part[t][c]);
        }
    };
    if (T > 1) host_pool(h).run(T, work);
    else work(0);
    for (unsigned t = 0; t < T; t++)
        for (size_t c = 0; c < C; c++) merge(out[c], part[t][c]);
}

int esp_batch_extend_host(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                          const uint8_t *arena, uint64_t arena_bytes,
                          const esp_n_interval *n_iv, uint64_t n_iv_count,
                          const esp_extend_params *params, esp_extension *out,
                          uint32_t *cigar, uint32_t cigar_stride) {
    if (!h || !params || !out || (n_pairs && (!pairs || !arena))) return fail(h, ESP_EINVAL, "null argument");
    if (mode != ESP_MODE_BAND && mode != ESP_MODE_HINT) return fail(h, ESP_EINVAL, "bad mode");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    CK(h, cudaSetDevice(h->device));
    // Large batches run as a pipeline of chunks: the inputs of chunk c+1 and
    // the results of chunk c-1 cross the host link while chunk c computes.
    // The paired kernels take two chunks, not four: an item holds two pairs,
    // so a chunk's longest items outlast its other work and smaller chunks
    // cost more in tails than their copies hide (mixed workload, 4M pairs:
    // 59.3 ms end to end in two chunks, 61.7 in one; 1M-pair launches at
    // 14.6 ms against 54.5 ms for 4M).
    const bool paired = mode == ESP_MODE_BAND ? band_paired(h, n_pairs)
                                              : esp::gotoh_paired(hint_variant(h, n_pairs));
    const uint64_t C = paired ? (n_pairs >= (1u << 21) ? 2 : 1) : (n_pairs >= (1u << 20) ? 4 : 1);
    std::vector<uint64_t> bounds(C + 1);
    for (uint64_t c = 0; c <= C; c++) bounds[c] = n_pairs * c / C;
    std::vector<ScanOut> sc;
    scan_chunks(h, mode, pairs, bounds, sc);
    ScanOut all;
    for (auto &s : sc) merge(all, s);
    const Limits &L1 = all.L1, &L2 = all.L2;
    size_t sz_pairs = (n_pairs * sizeof(esp_pair) + 255) / 256 * 256;
    size_t sz_iv = (n_iv_count * sizeof(esp_n_interval) + 255) / 256 * 256;
    size_t sz_arena = (arena_bytes + 16 + 255) / 256 * 256;
    size_t sz_out = (n_pairs * sizeof(esp_extension) + 255) / 256 * 256;
    size_t sz_cig = (n_pairs * (size_t)cigar_stride * 4 + 255) / 256 * 256;
    int rc;
    if ((rc = grow_device(h, &h->d_bat, &h->d_bat_cap, sz_pairs + sz_iv + sz_arena + sz_out + sz_cig)) != ESP_OK)
        return rc;
    uint8_t *b = (uint8_t *)h->d_bat;
    esp_pair *dp = (esp_pair *)b;
    esp_n_interval *div = (esp_n_interval *)(b + sz_pairs);
    uint8_t *da = b + sz_pairs + sz_iv;
    esp_extension *dout = (esp_extension *)(da + sz_arena);
    uint32_t *dcig = (uint32_t *)((uint8_t *)dout + sz_out);
    cudaStream_t st = h->stream;
    if (C == 1) {
        CK(h, cudaMemcpyAsync(dp, pairs, n_pairs * sizeof(esp_pair), cudaMemcpyHostToDevice, st));
        if (n_iv_count)
            CK(h, cudaMemcpyAsync(div, n_iv, n_iv_count * sizeof(esp_n_interval), cudaMemcpyHostToDevice, st));
        CK(h, cudaMemcpyAsync(da, arena, arena_bytes, cudaMemcpyHostToDevice, st));
        CK(h, cudaMemsetAsync(da + arena_bytes, 0, 16, st));
        rc = enqueue_batch(h, mode, dp, n_pairs, da, arena_bytes, div, n_iv_count, K, L1, L2, dout,
                           dcig, cigar_stride, st);
        if (rc != ESP_OK) return rc;
        CK(h, cudaMemcpyAsync(out, dout, n_pairs * sizeof(esp_extension), cudaMemcpyDeviceToHost, st));
        if (cigar && cigar_stride)
            CK(h, cudaMemcpyAsync(cigar, dcig, n_pairs * (size_t)cigar_stride * 4, cudaMemcpyDeviceToHost, st));
        CK(h, cudaStreamSynchronize(st));
        return ESP_OK;
    }
    if (!h->copy_stream) CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    cudaStream_t cs = h->copy_stream;
    std::vector<cudaEvent_t> ev(2 * C);
    for (auto &e : ev) CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // inputs, chunk by chunk: the pairs and the arena prefix the chunk reads
    // (the last chunk also gets the zero tail that 64-bit code loads read)
    if (n_iv_count)
        CK(h, cudaMemcpyAsync(div, n_iv, n_iv_count * sizeof(esp_n_interval), cudaMemcpyHostToDevice, cs));
    uint64_t copied = 0;  // arena bytes already sent
    for (uint64_t c = 0; c < C; c++) {
        const uint64_t a = bounds[c], n = bounds[c + 1] - a;
        CK(h, cudaMemcpyAsync(dp + a, pairs + a, n * sizeof(esp_pair), cudaMemcpyHostToDevice, cs));
        uint64_t need = c + 1 == C ? arena_bytes
                                   : std::min<uint64_t>(arena_bytes, (sc[c].arena_end + 3) / 4 + 16);
        if (need > copied) {
            CK(h, cudaMemcpyAsync(da + copied, arena + copied, need - copied, cudaMemcpyHostToDevice, cs));
            copied = need;
        }
        if (c + 1 == C) CK(h, cudaMemsetAsync(da + arena_bytes, 0, 16, cs));
        CK(h, cudaEventRecord(ev[c], cs));
    }
    for (uint64_t c = 0; c < C; c++) {
        const uint64_t a = bounds[c], n = bounds[c + 1] - a;
        CK(h, cudaStreamWaitEvent(st, ev[c], 0));
        rc = enqueue_batch(h, mode, dp + a, n, da, arena_bytes, div, n_iv_count, K, L1, L2,
                           dout + a, dcig + a * cigar_stride, cigar_stride, st);
        if (rc != ESP_OK) {
            for (auto &e : ev) cudaEventDestroy(e);
            return rc;
        }
        CK(h, cudaEventRecord(ev[C + c], st));
        CK(h, cudaStreamWaitEvent(cs, ev[C + c], 0));
        CK(h, cudaMemcpyAsync(out + a, dout + a, n * sizeof(esp_extension), cudaMemcpyDeviceToHost, cs));
        if (cigar && cigar_stride)
            CK(h, cudaMemcpyAsync(cigar + a * cigar_stride, dcig + a * cigar_stride,
                                  n * (size_t)cigar_stride * 4, cudaMemcpyDeviceToHost, cs));
    }
    CK(h, cudaStreamSynchronize(cs));
    CK(h, cudaStreamSynchronize(st));
    for (auto &e : ev) cudaEventDestroy(e);
    return ESP_OK;
}

int esp_batch_extend_device(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                            const uint8_t *arena, uint64_t arena_bytes,
                            const esp_n_interval *n_iv, uint64_t n_iv_count,
                            const esp_batch_limits *limits, const esp_extend_params *params,
                            esp_extension *out, uint32_t *cigar, uint32_t cigar_stride,
                            void *stream) {
    if (!h || !params || !out || !limits || (n_pairs && (!pairs || !arena)))
        return fail(h, ESP_EINVAL, "null argument");
    if (mode != ESP_MODE_BAND && mode != ESP_MODE_HINT) return fail(h, ESP_EINVAL, "bad mode");
    if (limits->max_read_len > 32767 || limits->max_win_len > 32767)
        return fail(h, ESP_EDOMAIN, "sequence longer than 32767");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    CK(h, cudaSetDevice(h->device));
    Limits L1, L2;
    if (mode == ESP_MODE_HINT) {
        add_limits(L1, limits->max_read_len, limits->max_win_len, 30);
        add_limits(L2, limits->max_read_len, limits->max_win_len, -1);
    } else {
        add_limits(L1, limits->max_read_len, limits->max_win_len,
                   limits->max_half < 0 ? -1 : limits->max_half);
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    if (h->use_graphs < 0) {
        const char *v = getenv("ESP_GRAPHS");
        h->use_graphs = (v && *v == '0') ? 0 : 1;
    }
    auto run = [&]() {
        return enqueue_batch(h, mode, pairs, n_pairs, arena, arena_bytes, n_iv, n_iv_count, K,
                             L1, L2, out, cigar, cigar_stride, st);
    };
    if (!h->use_graphs || h->autotune_ms) return run();
    // Repeated identical submissions (a resident batch re-run, a pipeline
    // reusing its buffers) replay one captured graph: the first run grows the
    // scratch, the second is captured, later ones launch the graph.
    std::vector<uint64_t> key = {
        (uint64_t)mode, (uint64_t)(uintptr_t)pairs, n_pairs, (uint64_t)(uintptr_t)arena,
        arena_bytes, (uint64_t)(uintptr_t)n_iv, n_iv_count, limits->max_read_len,
        limits->max_win_len, (uint64_t)(int64_t)limits->max_half, (uint64_t)params->match_score,
        (uint64_t)params->mismatch, (uint64_t)params->gap_open, (uint64_t)params->gap_ext,
        (uint64_t)params->edit_dir, (uint64_t)(uintptr_t)out, (uint64_t)(uintptr_t)cigar,
        cigar_stride, (uint64_t)(uintptr_t)st, (uint64_t)h->warp_max, (uint64_t)h->variant,
        (uint64_t)h->binning, (uint64_t)h->tuned};
    for (int s = 0; s < esp::kLengthClasses; s++) key.push_back((uint64_t)(int64_t)h->tune[s]);
    key.push_back(h->buf_gen);
    if (h->graph_exec && key == h->graph_key) {
        CK(h, cudaGraphLaunch(h->graph_exec, st));
        h->launches = h->graph_launches;
        return ESP_OK;
    }
    if (key != h->seen_key) {  // first sighting: run directly (grows scratch)
        int rc = run();
        key.back() = h->buf_gen;
        h->seen_key = key;
        return rc;
    }
    // second sighting with nothing regrown: capture, instantiate, launch
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
        h->graph_key.clear();
    }
    const uint64_t gen = h->buf_gen;
    CK(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = run();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc != ESP_OK || e != cudaSuccess || h->buf_gen != gen) {
        if (graph) cudaGraphDestroy(graph);
        h->seen_key.clear();
        if (rc != ESP_OK) return rc;
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
        return run();  // scratch moved during the capture: run directly
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    h->graph_exec = exec;
    h->graph_key = key;
    h->graph_launches = h->launches;
    CK(h, cudaGraphLaunch(exec, st));
    return ESP_OK;
}

int esp_batch_autotune(esp_handle *h, int mode, const esp_pair *pairs, uint64_t n_pairs,
                       const uint8_t *arena, uint64_t arena_bytes, const esp_n_interval *n_iv,
                       uint64_t n_iv_count, const esp_batch_limits *limits,
                       const esp_extend_params *params, esp_extension *out, uint32_t *cigar,
                       uint32_t cigar_stride, void *stream, int *variants, double *ms) {
    if (!h || !params || !out || !limits || !pairs || !arena) return fail(h, ESP_EINVAL, "null argument");
    if (mode != ESP_MODE_BAND) return fail(h, ESP_EINVAL, "autotuning runs band-mode batches");
    if (n_pairs <= (uint64_t)std::max<long>(32, h->warp_max < 0 ? 2048 : h->warp_max))
        return fail(h, ESP_EINVAL, "autotuning needs a batch of the persistent kernel's size");
    double t[(esp::kLengthClasses + 1) * esp::kGotohVariants];
    h->tuned = false;
    h->autotune_ms = t;
    int rc = esp_batch_extend_device(h, mode, pairs, n_pairs, arena, arena_bytes, n_iv,
                                     n_iv_count, limits, params, out, cigar, cigar_stride, stream);
    h->autotune_ms = nullptr;
    if (rc != ESP_OK) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    CK(h, cudaStreamSynchronize(st));
    // per-class launches each end in a tail of idle SMs: split only when the
    // sum of the classes' best times beats the best single launch
    auto best_of = [&](int row) {
        int b = 0;
        for (int v = 1; v < esp::kGotohVariants; v++)
            if (t[row * esp::kGotohVariants + v] < t[row * esp::kGotohVariants + b]) b = v;
        return b;
    };
    double split = 0;
    for (int s = 0; s < esp::kLengthClasses; s++)
        split += t[s * esp::kGotohVariants + best_of(s)];
    const int whole = best_of(esp::kLengthClasses);
    const bool one = t[esp::kLengthClasses * esp::kGotohVariants + whole] <= split;
    for (int s = 0; s < esp::kLengthClasses; s++) {
        h->tune[s] = one ? whole : best_of(s);
        if (variants) variants[s] = h->tune[s];
    }
    if (ms) memcpy(ms, t, sizeof(t));
    h->tuned = true;
    h->seen_key.clear();  // launches differ from any captured graph
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
        h->graph_key.clear();
    }
    return ESP_OK;
}

}  // extern "C"
