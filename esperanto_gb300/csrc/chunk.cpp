// chunk.cpp -- the pipeline batching hook: a chunk collector over the batch
// API.
//
// The reference's mapper aligns a chunk of 100,000 reads at a time, each rayon
// worker calling extend_hint / run_band / extend and the EA-Myers filters one
// read at a time (crates/map/src/pipeline.rs:394-403, :116-250, :318-450).
// Here a chunk's workers instead queue those calls -- from any number of host
// threads -- into one collector; run() sends every queued request of a kind
// through the batch API as one batch (one device batch per DP mode and per
// Myers direction, so millions of pairs share persistent launches), and each
// caller then picks up its results by the index add() returned, in input
// order.  The per-read decisions between stages (Myers first, the DP only for
// reads Myers does not settle) become rounds: queue, run, read, reset.
// Entry-point guards (empty reads, Myers lengths) answer exactly as the
// per-call drop-ins do.
#include <mutex>
#include <vector>

#include "esp_host.h"

namespace {

enum Klass { K_HINT = 0, K_BAND = 1, K_MY_END = 2, K_MY_START = 3, K_MY_GLOBAL = 4, K_NCLASS };

// One batch of the chunk: a 2-bit arena with N intervals, the records and
// the request each record answers.
struct Batch {
    std::vector<uint8_t> arena;  // 2-bit, MSB first, +16 zero bytes kept at the end
    uint64_t bases = 0;
    std::vector<esp_n_interval> iv;
    std::vector<esp_pair> pairs;        // DP classes
    std::vector<esp_myers_pair> mpairs;  // Myers classes
    std::vector<uint64_t> req;           // request index of each record
    // results after run()
    std::vector<esp_extension> out;
    std::vector<uint32_t> cigar;
    std::vector<esp_myers_result> mout;

    // Append one sequence's bases; returns its base position.  Sequences
    // start on byte boundaries.
    uint64_t put(const uint8_t *s, size_t len) {
        uint64_t pos = (bases + 3) / 4 * 4;
        bases = pos + len;
        arena.resize((bases + 3) / 4 + 16, 0);
        encode_seq(s, len, arena.data(), pos, iv);
        return pos;
    }
    void clear() {
        arena.clear();
        bases = 0;
        iv.clear();
        pairs.clear();
        mpairs.clear();
        req.clear();
        out.clear();
        cigar.clear();
        mout.clear();
    }
};

// Where request i's answer is: a record of a batch, or settled at add time.
struct Entry {
    int8_t klass = -1;  // -1: immediate Myers answer
    bool dist_only = false;  // a Myers kind that returns a distance alone
    uint64_t rec = 0;
    int32_t dist = 0;
    uint64_t pos = 0;
};

constexpr int LONG_MAX_M = 256;  // myers_ea.rs:14

}  // namespace

struct esp_chunk {
    esp_handle *h = nullptr;
    uint32_t stride = 64;
    std::mutex mu;
    Batch b[K_NCLASS];
    std::vector<Entry> entries;
    bool ran = false;
};

namespace {

int add_dp(esp_chunk *c, int klass, const uint8_t *read, size_t m, const uint8_t *win, size_t n,
           int64_t offset, int64_t half, uint64_t *index) {
    if (!c || !index || (m && !read) || (n && !win)) return ESP_EINVAL;
    if (m > 32767 || n > 32767) return ESP_EDOMAIN;
    if (offset < -(1ll << 30) || offset > (1ll << 30)) return ESP_EDOMAIN;
    if (half > (1ll << 30)) half = 1ll << 30;
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->ran) return ESP_EBUSY;
    Batch &B = c->b[klass];
    const size_t iv0 = B.iv.size();
    esp_pair P{};
    P.read_pos = B.put(read, m);
    const size_t nr = B.iv.size() - iv0;
    P.win_pos = B.put(win, n);
    const size_t nw = B.iv.size() - iv0 - nr;
    if (nr > 65535 || nw > 65535) {
        B.iv.resize(iv0);
        return ESP_EDOMAIN;  // too many N runs
    }
    P.read_len = (uint32_t)m;
    P.win_len = (uint32_t)n;
    P.band_offset = (int32_t)offset;
    P.band_half = half < 0 ? -1 : (int32_t)half;
    P.n_first = (uint32_t)iv0;
    P.n_read = (uint16_t)nr;
    P.n_win = (uint16_t)nw;
    Entry e;
    e.klass = (int8_t)klass;
    e.rec = B.pairs.size();
    *index = c->entries.size();
    B.pairs.push_back(P);
    B.req.push_back(*index);
    c->entries.push_back(e);
    return ESP_OK;
}

int add_myers(esp_chunk *c, int kind, const uint8_t *read, size_t m, const uint8_t *text,
              size_t n, uint64_t *index) {
    if (!c || !index || (m && !read) || (n && !text)) return ESP_EINVAL;
    if (n > 0xffffffffull) return ESP_EDOMAIN;
    int klass;
    bool single = false, engine = false;
    const bool dist_only = kind == ESP_CHUNK_MYERS_INFIX || kind == ESP_CHUNK_MYERS_LONG_INFIX ||
                           kind == ESP_CHUNK_ENGINE_INFIX || kind == ESP_CHUNK_ENGINE_GLOBAL;
    switch (kind) {
    case ESP_CHUNK_MYERS_INFIX: single = true; klass = K_MY_END; break;
    case ESP_CHUNK_MYERS_BEST_END: single = true; klass = K_MY_END; break;
    case ESP_CHUNK_MYERS_BEST_START: single = true; klass = K_MY_START; break;
    case ESP_CHUNK_MYERS_LONG_INFIX: klass = K_MY_END; break;
    case ESP_CHUNK_MYERS_LONG_BEST_END: klass = K_MY_END; break;
    case ESP_CHUNK_MYERS_LONG_BEST_START: klass = K_MY_START; break;
    case ESP_CHUNK_ENGINE_INFIX: engine = true; klass = K_MY_END; break;
    case ESP_CHUNK_ENGINE_GLOBAL: engine = true; klass = K_MY_GLOBAL; break;
    default: return ESP_EINVAL;
    }
    // the per-call entry points' guards (myers_ea.rs:118-135, :189-310;
    // engine/src/myers.rs asserts 1 <= m <= 256)
    if (engine && (m < 1 || m > (size_t)LONG_MAX_M))
        return ESP_EINVAL;
    if (!engine && single && m > 128 && m <= (size_t)LONG_MAX_M)
        return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->ran) return ESP_EBUSY;
    Entry e;
    e.dist_only = dist_only;
    if (!engine && (m == 0 || m > (size_t)LONG_MAX_M)) {  // answered without a DP
        e.dist = (int32_t)(m == 0 ? 0 : m);
        *index = c->entries.size();
        c->entries.push_back(e);
        return ESP_OK;
    }
    Batch &B = c->b[klass];
    const size_t iv0 = B.iv.size();
    esp_myers_pair P{};
    P.read_pos = B.put(read, m);
    const size_t nr = B.iv.size() - iv0;
    P.text_pos = B.put(text, n);
    const size_t nt = B.iv.size() - iv0 - nr;
    if (nr > 65535 || nt > 65535) {
        B.iv.resize(iv0);
        return ESP_EDOMAIN;  // too many N runs
    }
    P.read_len = (uint32_t)m;
    P.text_len = (uint32_t)n;
    P.n_first = (uint32_t)iv0;
    P.n_read = (uint16_t)nr;
    P.n_text = (uint16_t)nt;
    e.klass = (int8_t)klass;
    e.rec = B.mpairs.size();
    *index = c->entries.size();
    B.mpairs.push_back(P);
    B.req.push_back(*index);
    c->entries.push_back(e);
    return ESP_OK;
}

}  // namespace

extern "C" {

int esp_chunk_create(esp_handle *h, uint32_t cigar_stride, esp_chunk **out) {
    if (!h || !out || cigar_stride == 0 || cigar_stride > 4096) return ESP_EINVAL;
    esp_chunk *c = new (std::nothrow) esp_chunk();
    if (!c) return ESP_ENOMEM;
    c->h = h;
    c->stride = cigar_stride;
    *out = c;
    return ESP_OK;
}

int esp_chunk_add_extend_hint(esp_chunk *c, const uint8_t *read, size_t read_len,
                              const uint8_t *ref_window, size_t window_len, int64_t hint_offset,
                              uint64_t *index) {
    return add_dp(c, K_HINT, read, read_len, ref_window, window_len, hint_offset, 30, index);
}

int esp_chunk_add_run_band(esp_chunk *c, const uint8_t *read, size_t read_len,
                           const uint8_t *ref_window, size_t window_len, int64_t band_offset,
                           int64_t band_half, uint64_t *index) {
    return add_dp(c, K_BAND, read, read_len, ref_window, window_len,
                  band_half < 0 ? 0 : band_offset, band_half, index);
}

int esp_chunk_add_extend(esp_chunk *c, const uint8_t *read, size_t read_len,
                         const uint8_t *ref_window, size_t window_len, uint64_t *index) {
    return add_dp(c, K_BAND, read, read_len, ref_window, window_len, 0, -1, index);
}

int esp_chunk_add_myers(esp_chunk *c, int kind, const uint8_t *read, size_t read_len,
                        const uint8_t *text, size_t text_len, uint64_t *index) {
    return add_myers(c, kind, read, read_len, text, text_len, index);
}

int esp_chunk_run(esp_chunk *c, const esp_extend_params *params) {
    if (!c || !params) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->ran) return fail(c->h, ESP_EBUSY, "chunk already run: reset it first");
    for (int k = 0; k < K_NCLASS; k++) {
        Batch &B = c->b[k];
        const uint64_t n = k <= K_BAND ? B.pairs.size() : B.mpairs.size();
        if (n == 0) continue;
        int rc;
        if (k <= K_BAND) {
            B.out.resize(n);
            B.cigar.resize(n * (size_t)c->stride);
            rc = esp_batch_extend_host(c->h, k == K_HINT ? ESP_MODE_HINT : ESP_MODE_BAND,
                                       B.pairs.data(), n, B.arena.data(), B.arena.size(),
                                       B.iv.empty() ? nullptr : B.iv.data(), B.iv.size(), params,
                                       B.out.data(), B.cigar.data(), c->stride);
        } else {
            B.mout.resize(n);
            const int mode = k == K_MY_END ? ESP_MYERS_BEST_END
                                           : (k == K_MY_START ? ESP_MYERS_BEST_START
                                                              : ESP_MYERS_GLOBAL);
            rc = esp_batch_myers_host(c->h, mode, B.mpairs.data(), n, B.arena.data(),
                                      B.arena.size(), B.iv.empty() ? nullptr : B.iv.data(),
                                      B.iv.size(), B.mout.data());
        }
        if (rc != ESP_OK) return rc;
    }
    c->ran = true;
    return ESP_OK;
}

int esp_chunk_extension(esp_chunk *c, uint64_t index, esp_extension *out, uint32_t *cigar,
                        uint32_t cigar_cap) {
    if (!c || !out) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->ran) return fail(c->h, ESP_EINVAL, "chunk not run");
    if (index >= c->entries.size() || c->entries[index].klass < 0 ||
        c->entries[index].klass > K_BAND)
        return fail(c->h, ESP_EINVAL, "not a DP request of this chunk");
    const Entry &e = c->entries[index];
    const Batch &B = c->b[e.klass];
    const esp_extension &r = B.out[e.rec];
    *out = r;
    if (r.status == ESP_EINVAL) return fail(c->h, ESP_EINVAL, "kernel refused the pair");
    // the chunk's stride or the caller's buffer too small: as the per-call
    // drop-in, ESP_ECAP with the full length in n_ops
    if (r.status == ESP_ECAP || r.n_ops > cigar_cap) {
        out->status = ESP_ECAP;
        return fail(c->h, ESP_ECAP, "CIGAR buffer too small");
    }
    if (cigar && r.n_ops)
        memcpy(cigar, B.cigar.data() + e.rec * (size_t)c->stride, r.n_ops * sizeof(uint32_t));
    return ESP_OK;
}

int esp_chunk_myers(esp_chunk *c, uint64_t index, int32_t *dist, uint64_t *pos) {
    if (!c) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->ran) return fail(c->h, ESP_EINVAL, "chunk not run");
    if (index >= c->entries.size() || (c->entries[index].klass >= 0 &&
                                       c->entries[index].klass <= K_BAND))
        return fail(c->h, ESP_EINVAL, "not a Myers request of this chunk");
    const Entry &e = c->entries[index];
    if (e.klass < 0) {
        if (dist) *dist = e.dist;
        if (pos) *pos = e.pos;
        return ESP_OK;
    }
    const esp_myers_result &r = c->b[e.klass].mout[e.rec];
    if (r.status != ESP_OK) return fail(c->h, r.status, "myers kernel refused the pair");
    if (dist) *dist = r.dist;
    if (pos) *pos = e.dist_only ? 0 : r.pos;
    return ESP_OK;
}

uint64_t esp_chunk_size(esp_chunk *c) {
    if (!c) return 0;
    std::lock_guard<std::mutex> lk(c->mu);
    return c->entries.size();
}

int esp_chunk_reset(esp_chunk *c) {
    if (!c) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    for (Batch &B : c->b) B.clear();
    c->entries.clear();
    c->ran = false;
    return ESP_OK;
}

int esp_chunk_destroy(esp_chunk *c) {
    delete c;
    return ESP_OK;
}

}  // extern "C"
