// abi_myers.cu -- C ABI of the Myers filters: per-call drop-ins of
// myers_ea::* and engine::myers::*, and the batch API.
#include <cuda_runtime.h>

#include <thread>
#include <vector>

#include "esp_host.h"

namespace {

constexpr int LONG_MAX_M = 256;  // myers_ea.rs:14

// One pair through the device kernel.  Returns ESP_OK and fills dist/pos.
int one_myers(esp_handle *h, int flags, const uint8_t *read, size_t m, const uint8_t *text,
              size_t n, int32_t *dist, uint64_t *pos) {
    if (!h || (m && !read) || (n && !text)) return fail(h, ESP_EINVAL, "null argument");
    if (n > 0xffffffffull) return fail(h, ESP_EDOMAIN, "text longer than 2^32-1");
    CK(h, cudaSetDevice(h->device));
    std::vector<esp_n_interval> iv;
    uint64_t tpos = ((m + 63) / 64) * 64;
    uint64_t bases = tpos + n;
    size_t arena_bytes = ((bases + 3) / 4 + 15) / 16 * 16 + 16;
    size_t max_iv = (m + 1) / 2 + (n + 1) / 2 + 2;
    size_t hdr = (64 + max_iv * sizeof(esp_n_interval) + 255) / 256 * 256;
    int rc;
    if ((rc = grow_host(h, &h->h_my, &h->h_my_cap, hdr + arena_bytes + 64)) != ESP_OK) return rc;
    if ((rc = grow_device(h, &h->d_my, &h->d_my_cap, hdr + arena_bytes + 64)) != ESP_OK) return rc;
    uint8_t *hin = (uint8_t *)h->h_my;
    uint8_t *harena = hin + hdr;
    memset(harena, 0, arena_bytes);
    encode_seq(read, m, harena, 0, iv);
    size_t nr = iv.size();
    encode_seq(text, n, harena, tpos, iv);
    if (nr > 65535 || iv.size() - nr > 65535) return fail(h, ESP_EDOMAIN, "too many N runs");
    esp_myers_pair P{};
    P.read_pos = 0;
    P.text_pos = tpos;
    P.read_len = (uint32_t)m;
    P.text_len = (uint32_t)n;
    P.n_first = 0;
    P.n_read = (uint16_t)nr;
    P.n_text = (uint16_t)(iv.size() - nr);
    memcpy(hin, &P, sizeof(P));
    if (!iv.empty()) memcpy(hin + 64, iv.data(), iv.size() * sizeof(esp_n_interval));
    uint8_t *din = (uint8_t *)h->d_my;
    esp_myers_result *dres = (esp_myers_result *)(din + hdr + arena_bytes);
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(din, hin, hdr + arena_bytes, cudaMemcpyHostToDevice, st));
    esp::MyersJob job{};
    job.pairs = (const esp_myers_pair *)din;
    job.n_pairs = 1;
    job.arena = din + hdr;
    job.n_iv = (const esp_n_interval *)(din + 64);
    job.flags = flags;
    job.out = dres;
    CK(h, esp::launch_myers(job, (int)((m + 31) / 32), h->num_sms, st));
    h->launches = 1;
    esp_myers_result r;
    CK(h, cudaMemcpyAsync(hin + hdr + arena_bytes, dres, sizeof(r), cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    memcpy(&r, hin + hdr + arena_bytes, sizeof(r));
    if (r.status != ESP_OK) return fail(h, r.status, "myers kernel refused the pair");
    if (dist) *dist = r.dist;
    if (pos) *pos = r.pos;
    return ESP_OK;
}

// myers_ea.rs entry-point guards: m = 0 -> (0, 0); m > 256 -> (m, 0);
// single-block entries refuse 128 < m <= 256 (shift overflow in the reference).
int map_entry(esp_handle *h, bool single, int flags, const uint8_t *read, size_t m,
              const uint8_t *text, size_t n, int32_t *dist, uint64_t *pos) {
    if (m == 0) {
        if (dist) *dist = 0;
        if (pos) *pos = 0;
        return ESP_OK;
    }
    if (m > (size_t)LONG_MAX_M) {
        if (dist) *dist = (int32_t)m;
        if (pos) *pos = 0;
        return ESP_OK;
    }
    if (single && m > 128)
        return fail(h, ESP_EINVAL, "single-block Myers entry point with m > 128 (use long::)");
    return one_myers(h, flags, read, m, text, n, dist, pos);
}

}  // namespace

extern "C" {

int esp_myers_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                    size_t n, int32_t *dist) {
    return map_entry(h, true, 0, read, m, text, n, dist, nullptr);
}

int esp_myers_infix_best_end(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                             size_t n, int32_t *dist, uint64_t *end) {
    return map_entry(h, true, 0, read, m, text, n, dist, end);
}

int esp_myers_infix_best_start(esp_handle *h, const uint8_t *read, size_t m,
                               const uint8_t *text, size_t n, int32_t *dist, uint64_t *start) {
    return map_entry(h, true, esp::MYF_REVERSE, read, m, text, n, dist, start);
}

int esp_myers_long_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                         size_t n, int32_t *dist) {
    return map_entry(h, false, 0, read, m, text, n, dist, nullptr);
}

int esp_myers_long_infix_best_end(esp_handle *h, const uint8_t *read, size_t m,
                                  const uint8_t *text, size_t n, int32_t *dist, uint64_t *end) {
    return map_entry(h, false, 0, read, m, text, n, dist, end);
}

int esp_myers_long_infix_best_start(esp_handle *h, const uint8_t *read, size_t m,
                                    const uint8_t *text, size_t n, int32_t *dist,
                                    uint64_t *start) {
    return map_entry(h, false, esp::MYF_REVERSE, read, m, text, n, dist, start);
}

int esp_engine_myers_infix(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                           size_t n, uint32_t *dist) {
    if (m < 1 || m > (size_t)LONG_MAX_M)
        return fail(h, ESP_EINVAL, "EA-Myers pattern length must be in 1..=256");
    int32_t d = 0;
    int rc = one_myers(h, 0, read, m, text, n, &d, nullptr);
    if (rc == ESP_OK && dist) *dist = (uint32_t)d;
    return rc;
}

int esp_engine_myers_global(esp_handle *h, const uint8_t *read, size_t m, const uint8_t *text,
                            size_t n, uint32_t *dist) {
    if (m < 1 || m > (size_t)LONG_MAX_M)
        return fail(h, ESP_EINVAL, "EA-Myers pattern length must be in 1..=256");
    int32_t d = 0;
    int rc = one_myers(h, esp::MYF_GLOBAL, read, m, text, n, &d, nullptr);
    if (rc == ESP_OK && dist) *dist = (uint32_t)d;
    return rc;
}

static int mode_flags(int mode) {
    return mode == ESP_MYERS_BEST_START ? esp::MYF_REVERSE
                                        : (mode == ESP_MYERS_GLOBAL ? esp::MYF_GLOBAL : 0);
}

int esp_batch_myers_device(esp_handle *h, int mode, const esp_myers_pair *pairs,
                           uint64_t n_pairs, uint32_t max_read_len, const uint8_t *arena,
                           uint64_t arena_bytes, const esp_n_interval *n_iv,
                           uint64_t n_iv_count, esp_myers_result *out, void *stream) {
    (void)arena_bytes;
    (void)n_iv_count;
    if (!h || !out || (n_pairs && (!pairs || !arena))) return fail(h, ESP_EINVAL, "null argument");
    if (mode < 0 || mode > 2) return fail(h, ESP_EINVAL, "bad Myers mode");
    if (max_read_len < 1 || max_read_len > (uint32_t)LONG_MAX_M)
        return fail(h, ESP_EINVAL, "Myers read length must be in 1..=256");
    CK(h, cudaSetDevice(h->device));
    esp::MyersJob job{};
    job.pairs = pairs;
    job.n_pairs = n_pairs;
    job.arena = arena;
    job.n_iv = n_iv;
    job.flags = mode_flags(mode);
    job.out = out;
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    CK(h, esp::launch_myers(job, (int)((max_read_len + 31) / 32), h->num_sms, st));
    h->launches = 1;
    return ESP_OK;
}

int esp_batch_myers_host(esp_handle *h, int mode, const esp_myers_pair *pairs,
                         uint64_t n_pairs, const uint8_t *arena, uint64_t arena_bytes,
                         const esp_n_interval *n_iv, uint64_t n_iv_count,
                         esp_myers_result *out) {
    if (!h || !out || (n_pairs && (!pairs || !arena))) return fail(h, ESP_EINVAL, "null argument");
    // Large batches run as a pipeline of chunks: the inputs of chunk c+1 and
    // the results of chunk c-1 cross the host link while chunk c computes
    // (eight chunks: the first chunk's copy is the exposed part; measured
    // 3 % faster end to end than four on 1M pairs).
    const uint64_t C = n_pairs >= (1u << 18) ? 8 : 1;
    std::vector<uint64_t> bounds(C + 1);
    for (uint64_t c = 0; c <= C; c++) bounds[c] = n_pairs * c / C;
    // longest read (sizes the kernel's limb count) and the arena prefix each
    // chunk reads; large batches are scanned on the host pool
    uint32_t mx = 1;
    std::vector<uint64_t> arena_end(C, 0);  // bases
    {
        unsigned T = n_pairs < (1u << 16) ? 1 : (unsigned)std::min<uint64_t>(16, n_pairs >> 15);
        if (T > 1) T = std::min(T, host_pool(h).size());
        std::vector<uint32_t> part(T, 1);
        std::vector<uint64_t> ends(T * C, 0);
        auto work = [&](unsigned t) {
            uint32_t m = 1;
            for (uint64_t c = 0; c < C; c++) {
                const uint64_t a = bounds[c], len = bounds[c + 1] - a;
                uint64_t e = 0;
                for (uint64_t k = a + len * t / T, z = a + len * (t + 1) / T; k < z; k++) {
                    const esp_myers_pair &P = pairs[k];
                    m = std::max(m, P.read_len);
                    e = std::max({e, P.read_pos + P.read_len, P.text_pos + P.text_len});
                }
                ends[t * C + c] = e;
            }
            part[t] = m;
        };
        if (T > 1) host_pool(h).run(T, work);
        else work(0);
        for (uint32_t m : part) mx = std::max(mx, m);
        for (unsigned t = 0; t < T; t++)
            for (uint64_t c = 0; c < C; c++) arena_end[c] = std::max(arena_end[c], ends[t * C + c]);
    }
    if (mx > (uint32_t)LONG_MAX_M) return fail(h, ESP_EINVAL, "Myers read length must be <= 256");
    CK(h, cudaSetDevice(h->device));
    size_t sz_p = (n_pairs * sizeof(esp_myers_pair) + 255) / 256 * 256;
    size_t sz_iv = (n_iv_count * sizeof(esp_n_interval) + 255) / 256 * 256;
    size_t sz_a = (arena_bytes + 16 + 255) / 256 * 256;
    size_t sz_o = (n_pairs * sizeof(esp_myers_result) + 255) / 256 * 256;
    int rc;
    if ((rc = grow_device(h, &h->d_bat, &h->d_bat_cap, sz_p + sz_iv + sz_a + sz_o)) != ESP_OK)
        return rc;
    uint8_t *b = (uint8_t *)h->d_bat;
    esp_myers_pair *dp = (esp_myers_pair *)b;
    const esp_n_interval *div = (const esp_n_interval *)(b + sz_p);
    uint8_t *da = b + sz_p + sz_iv;
    esp_myers_result *dout = (esp_myers_result *)(b + sz_p + sz_iv + sz_a);
    cudaStream_t st = h->stream;
    if (C == 1) {
        CK(h, cudaMemcpyAsync(dp, pairs, n_pairs * sizeof(esp_myers_pair), cudaMemcpyHostToDevice, st));
        if (n_iv_count)
            CK(h, cudaMemcpyAsync((void *)div, n_iv, n_iv_count * sizeof(esp_n_interval),
                                  cudaMemcpyHostToDevice, st));
        CK(h, cudaMemcpyAsync(da, arena, arena_bytes, cudaMemcpyHostToDevice, st));
        CK(h, cudaMemsetAsync(da + arena_bytes, 0, 16, st));
        rc = esp_batch_myers_device(h, mode, dp, n_pairs, mx, da, arena_bytes, div, n_iv_count,
                                    dout, st);
        if (rc != ESP_OK) return rc;
        CK(h, cudaMemcpyAsync(out, dout, n_pairs * sizeof(esp_myers_result), cudaMemcpyDeviceToHost, st));
        CK(h, cudaStreamSynchronize(st));
        return ESP_OK;
    }
    if (!h->copy_stream) CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    cudaStream_t cs = h->copy_stream;
    std::vector<cudaEvent_t> ev(2 * C);
    for (auto &e : ev) CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    auto release = [&] {
        for (auto &e : ev) cudaEventDestroy(e);
    };
    // inputs, chunk by chunk: the pairs and the arena prefix the chunk reads
    // (the last chunk also gets the zero tail that 64-bit code loads read)
    if (n_iv_count)
        CK(h, cudaMemcpyAsync((void *)div, n_iv, n_iv_count * sizeof(esp_n_interval),
                              cudaMemcpyHostToDevice, cs));
    uint64_t copied = 0;  // arena bytes already sent
    for (uint64_t c = 0; c < C; c++) {
        const uint64_t a = bounds[c], n = bounds[c + 1] - a;
        CK(h, cudaMemcpyAsync(dp + a, pairs + a, n * sizeof(esp_myers_pair), cudaMemcpyHostToDevice, cs));
        uint64_t need = c + 1 == C ? arena_bytes
                                   : std::min<uint64_t>(arena_bytes, (arena_end[c] + 3) / 4 + 16);
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
        rc = esp_batch_myers_device(h, mode, dp + a, n, mx, da, arena_bytes, div, n_iv_count,
                                    dout + a, st);
        if (rc != ESP_OK) {
            release();
            return rc;
        }
        CK(h, cudaEventRecord(ev[C + c], st));
        CK(h, cudaStreamWaitEvent(cs, ev[C + c], 0));
        CK(h, cudaMemcpyAsync(out + a, dout + a, n * sizeof(esp_myers_result), cudaMemcpyDeviceToHost, cs));
    }
    CK(h, cudaStreamSynchronize(cs));
    CK(h, cudaStreamSynchronize(st));
    release();
    h->launches = (int)C;
    return ESP_OK;
}

}  // extern "C"
