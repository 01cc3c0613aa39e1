// noalloc.cu -- a banded-Gotoh batch entry point that allocates nothing.
//
// Who needs it: callers that own all device memory through their own
// allocator or budget (a host runtime that pre-sizes one pool at start-up
// and treats any later device allocation as a failure), and latency-bound
// callers that cannot accept cudaMalloc/cudaFree on the request path because
// those calls can synchronise the whole device and stall unrelated streams.
// The regular entry points grow per-handle scratch with cudaMalloc on first
// use of a larger shape; this one never does.
//
// How: the DP kernel's scratch (a small work-queue header, the per-warp
// traceback words and the per-warp row buffers) lives in one file-scope
// __device__ array of fixed size, ESP_NOALLOC_SCRATCH_BYTES, which every GPU
// that loads this library holds until the process exits.  Host code cannot
// pass the array's name to a kernel (in host code that name is a host-side
// stand-in, not a device address), so the device address is looked up once
// per device with cudaGetSymbolAddress and cached.
//
// Sharing: every call uses the same array.  Calls that can overlap on the
// GPU (two streams, or two host threads) race on it and must be serialised
// by the caller.  Each call clears the work-queue header itself; the
// traceback and row-buffer words are always written before they are read
// within a call, so stale contents from the previous call are harmless.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "esp_internal.h"
#include "esperanto_gb300.h"

namespace {

constexpr uint64_t kScratchBytes = ESP_NOALLOC_SCRATCH_BYTES;
constexpr uint64_t kHeaderBytes = 256;  // queue counters
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};
int g_blocks_per_sm[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Per-device set-up, done by the first call on each device with that
// device current: look up the array's device address (and the SM count and
// occupancy used to size the persistent grid).  No allocation happens here.
int setup_device(int dev) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (g_scratch_addr[dev]) return ESP_OK;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return ESP_ECUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ESP_ECUDA;
    g_blocks_per_sm[dev] = esp::gotoh_blocks_per_sm(128, 1);
    g_num_sms[dev] = sms;
    g_scratch_addr[dev] = p;
    return ESP_OK;
}

}  // namespace

extern "C" int esp_batch_run_band_noalloc(const esp_pair *pairs, uint64_t n_pairs,
                                          const uint8_t *arena, uint64_t arena_bytes,
                                          const esp_n_interval *n_iv, uint64_t n_iv_count,
                                          const esp_batch_limits *limits,
                                          const esp_extend_params *params, esp_extension *out,
                                          uint32_t *cigar, uint32_t cigar_stride,
                                          void *stream) {
    if (!limits || !params || !out || (n_pairs && (!pairs || !arena))) return ESP_EINVAL;
    if (limits->max_read_len > 32767 || limits->max_win_len > 32767) return ESP_EDOMAIN;
    if (n_pairs > 0xffffffffull - 64) return ESP_EINVAL;
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK) return ESP_EDOMAIN;
    if (limits->max_read_len > (uint32_t)K.max_m) return ESP_EDOMAIN;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ESP_ECUDA;
    int rc = setup_device(dev);
    if (rc != ESP_OK) return rc;
    if (n_pairs == 0) return ESP_OK;

    uint64_t tbw, rbw;
    esp::gotoh_scratch_words(limits->max_read_len, limits->max_win_len,
                             limits->max_half < 0 ? -1 : limits->max_half, tbw, rbw);
    tbw = tbw ? tbw : 1;
    rbw = rbw ? rbw : 1;
    // Scratch per 128-thread block: 4 warps x 32 lanes x (tb + rb) words.
    const uint64_t per_block = 4ull * 32 * (tbw + rbw) * 4;
    const uint64_t room = kScratchBytes - kHeaderBytes;
    if (per_block > room) return ESP_ESCRATCH;  // one block's pairs do not fit
    uint64_t blocks = room / per_block;
    uint64_t want = (uint64_t)g_num_sms[dev] * (uint64_t)g_blocks_per_sm[dev];
    uint64_t need = (n_pairs + 127) / 128;
    if (blocks > want) blocks = want;
    if (blocks > need) blocks = need;
    const uint64_t warps = blocks * 4;

    uint8_t *base = (uint8_t *)g_scratch_addr[dev];
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(base, 0, kHeaderBytes, st) != cudaSuccess) return ESP_ECUDA;
    esp::GotohJob job{};
    job.pairs = pairs;
    job.n_pairs = n_pairs;
    job.list = nullptr;
    job.list_count = nullptr;
    job.arena = arena;
    job.arena_bases = arena_bytes * 4;
    job.n_iv = n_iv;
    job.n_iv_count = n_iv_count;
    job.mode = 0;
    job.esc_list = nullptr;
    job.esc_count = nullptr;
    job.out = out;
    job.cigar = cigar;
    job.cigar_stride = cigar_stride;
    job.queue = (uint32_t *)base;
    job.tb = (uint32_t *)(base + kHeaderBytes);
    job.tb_words = tbw;
    job.rb = job.tb + warps * 32 * tbw;
    job.rb_words = rbw;
    if (esp::launch_gotoh(job, K, (int)warps, 128, st, 1) != cudaSuccess) return ESP_ECUDA;
    return ESP_OK;
}
