// serve.cpp -- continuous-batching serving loop over a resident genome.
//
// One native worker thread owns the device side: it polls the in-flight
// slots' completion events, copies finished results back to the callers'
// buffers, and admits queued requests (FIFO) to idle slots while the
// device-memory budget allows.  Each slot is a private esp_handle (stream +
// DP scratch reserved at start-up, so serving never calls cudaMalloc or
// cudaFree) plus pinned staging for one request.  Requests that arrive while
// others run are admitted as soon as a slot and budget free up, and their
// kernels overlap on the device with the ones already running.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "esp_host.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    esp_serve_request req{};
    Clock::time_point t_submit;
    uint64_t need = 0;  // admitted device bytes
    int32_t status = 1; // 1 = pending / in flight
    double latency_ms = 0;
    bool done = false;
};

struct Slot {
    esp_handle *h = nullptr;
    cudaEvent_t done = nullptr;
    Request *cur = nullptr;
    int staged_rc = ESP_OK;      // launch() status of the current request
    uint8_t *h_stage = nullptr;  // pinned: pairs | n intervals | read arena | out | cigar
    uint8_t *d_stage = nullptr;
    size_t off_iv = 0, off_arena = 0, off_out = 0, off_cig = 0, bytes = 0;
};

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

struct esp_server {
    esp_genome *g = nullptr;
    esp::GotohConst K{};
    esp_server_config cfg{};
    int device = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::unordered_map<uint64_t, Request *> all;
    uint64_t next_ticket = 1;
    uint64_t budget_free = 0;
    uint64_t per_warp_bytes = 0;
    uint64_t want_warps = 0;
    bool closing = false, stop = false;
    std::thread worker;
};

namespace {

// DP scratch one request of n reads is admitted with (the extend_hint
// policy's full-matrix attempt sizes the per-warp traceback words).
uint64_t request_need(const esp_server *s, uint64_t n) {
    uint64_t warps = std::min<uint64_t>(s->want_warps, (n + 31) / 32);
    warps = (warps + 3) / 4 * 4;
    return warps * s->per_warp_bytes;
}

// Host side of one launch: build the DP pairs (windows point straight into
// the resident genome; genome N runs are clipped into per-pair intervals),
// stage, copy, run, copy back, record completion.
int launch(esp_server *s, Slot &sl, Request *r) {
    const esp_serve_request &q = r->req;
    esp_pair *pairs = (esp_pair *)sl.h_stage;
    esp_n_interval *iv = (esp_n_interval *)(sl.h_stage + sl.off_iv);
    uint64_t niv = 0;
    const size_t iv_cap = (sl.off_arena - sl.off_iv) / sizeof(esp_n_interval);
    const esp_genome *g = s->g;
    for (uint64_t i = 0; i < q.n_reads; i++) {
        const esp_serve_read &R = q.reads[i];
        const esp_contig &C = g->contigs[R.contig];
        uint32_t ws = std::min(R.win_start, C.len);
        uint32_t we = (uint32_t)std::min<uint64_t>((uint64_t)ws + R.win_len, C.len);
        esp_pair P{};
        P.read_pos = R.read_pos;
        P.read_len = R.read_len;
        P.win_pos = C.base + ws;
        P.win_len = we - ws;
        P.band_offset = R.hint_offset;
        P.band_half = 30;
        P.n_first = 0;
        pairs[i] = P;
    }
    // genome N runs (host copy kept by the genome) -> per-pair relative lists
    if (g->n_iv) {
        for (uint64_t i = 0; i < q.n_reads; i++) {
            const esp_serve_read &R = q.reads[i];
            const esp_contig &C = g->contigs[R.contig];
            uint32_t ws = (uint32_t)(pairs[i].win_pos - C.base), we = ws + pairs[i].win_len;
            pairs[i].n_first = (uint32_t)niv;
            uint32_t cnt = 0;
            // the contig's intervals are sorted and disjoint: start at the
            // first one ending after the window start
            const esp_n_interval *cv = g->h_iv.data() + C.n_first;
            uint32_t lo = 0, hi = C.n_count;
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                if (cv[mid].end <= ws) lo = mid + 1;
                else hi = mid;
            }
            for (uint32_t k = lo; k < C.n_count && cv[k].start < we; k++) {
                uint32_t a = std::max(cv[k].start, ws), b = std::min(cv[k].end, we);
                if (a < b) {
                    if (niv >= iv_cap) return ESP_EDOMAIN;
                    iv[niv++] = {a - ws, b - ws};
                    cnt++;
                }
            }
            pairs[i].n_win = (uint16_t)cnt;
        }
    }
    memcpy(sl.h_stage + sl.off_arena, q.read_arena, q.read_arena_bytes);
    memset(sl.h_stage + sl.off_arena + q.read_arena_bytes, 0, 16);
    esp_handle *h = sl.h;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(sl.d_stage, sl.h_stage, q.n_reads * sizeof(esp_pair),
                          cudaMemcpyHostToDevice, st));
    if (niv)
        CK(h, cudaMemcpyAsync(sl.d_stage + sl.off_iv, sl.h_stage + sl.off_iv,
                              niv * sizeof(esp_n_interval), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(sl.d_stage + sl.off_arena, sl.h_stage + sl.off_arena,
                          q.read_arena_bytes + 16, cudaMemcpyHostToDevice, st));
    Limits L1, L2;
    add_limits(L1, s->cfg.max_read_len, s->cfg.max_win_len, 30);
    add_limits(L2, s->cfg.max_read_len, s->cfg.max_win_len, -1);
    int rc = enqueue_batch(h, ESP_MODE_HINT, (const esp_pair *)sl.d_stage, q.n_reads,
                           sl.d_stage + sl.off_arena, q.read_arena_bytes,
                           niv ? (const esp_n_interval *)(sl.d_stage + sl.off_iv) : nullptr, niv,
                           s->K, L1, L2, (esp_extension *)(sl.d_stage + sl.off_out),
                           (uint32_t *)(sl.d_stage + sl.off_cig), q.cigar_stride, st,
                           g->d_arena, g->arena_bytes);
    if (rc != ESP_OK) return rc;
    CK(h, cudaMemcpyAsync(sl.h_stage + sl.off_out, sl.d_stage + sl.off_out,
                          q.n_reads * sizeof(esp_extension), cudaMemcpyDeviceToHost, st));
    if (q.cigar && q.cigar_stride)
        CK(h, cudaMemcpyAsync(sl.h_stage + sl.off_cig, sl.d_stage + sl.off_cig,
                              q.n_reads * (size_t)q.cigar_stride * 4, cudaMemcpyDeviceToHost, st));
    CK(h, cudaEventRecord(sl.done, st));
    return ESP_OK;
}

// Results of a finished slot into the caller's buffers (worker thread, no
// lock held: the slot and its request belong to the worker until complete()).
void copy_out(Slot &sl) {
    const esp_serve_request &q = sl.cur->req;
    memcpy(q.out, sl.h_stage + sl.off_out, q.n_reads * sizeof(esp_extension));
    if (q.cigar && q.cigar_stride)
        memcpy(q.cigar, sl.h_stage + sl.off_cig, q.n_reads * (size_t)q.cigar_stride * 4);
}

// Publish a slot's request as done (server lock held).
void complete(esp_server *s, Slot &sl, int32_t status) {
    Request *r = sl.cur;
    r->status = status;
    r->latency_ms =
        std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
    r->done = true;
    s->budget_free += r->need;
    sl.cur = nullptr;
}

// The worker owns the slots.  The server lock guards only the queue, the
// ticket table and the budget: staging a request, launching it and copying
// results out run unlocked, so submitters and waiters are never held up by
// the bulk copies.
void worker_loop(esp_server *s) {
    cudaSetDevice(s->device);
    std::vector<std::pair<Slot *, int32_t>> done;
    std::vector<Slot *> to_launch;
    for (;;) {
        done.clear();
        for (Slot &sl : s->slots) {
            if (!sl.cur || sl.staged_rc != ESP_OK) continue;
            cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaErrorNotReady) continue;
            if (e == cudaSuccess) copy_out(sl);
            done.push_back({&sl, e == cudaSuccess ? ESP_OK : ESP_ECUDA});
        }
        to_launch.clear();
        bool inflight = false, stop = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (Slot &sl : s->slots)  // launches that failed in the previous round
                if (sl.cur && sl.staged_rc != ESP_OK) done.push_back({&sl, sl.staged_rc});
            for (auto &d : done) complete(s, *d.first, d.second);
            if (!done.empty()) s->cv_done.notify_all();
            // FIFO admission: the head request waits for a slot and for budget
            while (!s->pending.empty()) {
                Request *r = s->pending.front();
                if (s->closing) {
                    s->pending.pop_front();
                    r->status = ESP_ECLOSED;
                    r->done = true;
                    s->cv_done.notify_all();
                    continue;
                }
                Slot *idle = nullptr;
                for (Slot &sl : s->slots)
                    if (!sl.cur) {
                        idle = &sl;
                        break;
                    }
                if (!idle || r->need > s->budget_free) break;
                s->pending.pop_front();
                s->budget_free -= r->need;
                idle->cur = r;
                idle->staged_rc = ESP_OK;
                to_launch.push_back(idle);
            }
            for (Slot &sl : s->slots) inflight |= sl.cur != nullptr;
            stop = s->stop && !inflight && s->pending.empty();
            if (!stop && !inflight) {
                s->cv_work.wait(lk);
                continue;
            }
        }
        if (stop) break;
        for (Slot *sl : to_launch) sl->staged_rc = launch(s, *sl, sl->cur);
        if (to_launch.empty()) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" {

int esp_server_create(esp_genome *g, const esp_extend_params *params,
                      const esp_server_config *cfg, int device, esp_server **out) {
    if (!g || !params || !out) return ESP_EINVAL;
    *out = nullptr;
    esp_server *s = new (std::nothrow) esp_server();
    if (!s) return ESP_ENOMEM;
    if (esp::make_gotoh_const(*params, s->K) != ESP_OK) {
        delete s;
        return ESP_EDOMAIN;
    }
    esp_server_config c{};
    if (cfg) c = *cfg;
    if (!c.n_streams) c.n_streams = 4;
    if (!c.max_reads) c.max_reads = 131072;
    if (!c.max_read_len) c.max_read_len = 300;
    if (!c.max_win_len) c.max_win_len = c.max_read_len + 128;
    if (!c.mem_budget_bytes) c.mem_budget_bytes = 16ull << 30;
    if (c.max_read_len > 32767 || c.max_win_len > 32767 ||
        c.max_read_len > (uint32_t)s->K.max_m) {
        delete s;
        return ESP_EDOMAIN;
    }
    s->cfg = c;
    s->g = g;
    s->device = device;
    s->budget_free = c.mem_budget_bytes;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete s;
        return ESP_ECUDA;
    }
    s->slots.resize(c.n_streams);
    int rc = ESP_OK;
    uint64_t tb, rb;
    esp::gotoh_scratch_words(c.max_read_len, c.max_win_len, -1, tb, rb);
    s->per_warp_bytes = (tb + rb) * 32 * 4;
    for (Slot &sl : s->slots) {
        if ((rc = esp_create(&sl.h, device)) != ESP_OK) break;
        sl.h->scratch_budget = c.mem_budget_bytes / c.n_streams;
        if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            rc = ESP_ECUDA;
            break;
        }
        // reserve the slot's DP scratch for the largest request once, so the
        // serving path never reallocates
        if ((rc = reserve_dp(sl.h, c.max_reads, c.max_read_len, c.max_win_len)) != ESP_OK) break;
        const uint64_t n = c.max_reads;
        sl.off_iv = al256(n * sizeof(esp_pair));
        sl.off_arena = sl.off_iv + al256(n * 4 * sizeof(esp_n_interval));
        sl.off_out = sl.off_arena + al256(n * (uint64_t)c.max_read_len / 4 + 64);
        sl.off_cig = sl.off_out + al256(n * sizeof(esp_extension));
        sl.bytes = sl.off_cig + al256(n * 64 * 4);
        if (cudaMallocHost((void **)&sl.h_stage, sl.bytes) != cudaSuccess ||
            cudaMalloc((void **)&sl.d_stage, sl.bytes) != cudaSuccess) {
            rc = ESP_ENOMEM;
            break;
        }
    }
    if (rc == ESP_OK) {
        int bps = esp::gotoh_blocks_per_sm(128, s->slots[0].h->variant < 0 ? 1 : s->slots[0].h->variant);
        s->want_warps = (uint64_t)s->slots[0].h->num_sms * bps * 4;
        // whole 128-thread blocks within one slot's share of the budget
        uint64_t cap = (c.mem_budget_bytes / c.n_streams) / s->per_warp_bytes / 4 * 4;
        s->want_warps = std::min(s->want_warps, std::max<uint64_t>(4, cap));
    }
    if (rc != ESP_OK) {
        esp_server_destroy(s);
        return rc;
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return ESP_OK;
}

int esp_server_submit(esp_server *s, const esp_serve_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket || (req->n_reads && (!req->reads || !req->read_arena || !req->out)))
        return ESP_EINVAL;
    if (req->n_reads > s->cfg.max_reads || (req->cigar_stride > 64) ||
        req->read_arena_bytes > (uint64_t)s->cfg.max_reads * s->cfg.max_read_len / 4 + 48)
        return ESP_EBUSY;
    for (uint64_t i = 0; i < req->n_reads; i++) {
        const esp_serve_read &R = req->reads[i];
        if (R.contig >= s->g->contigs.size() || R.read_len > s->cfg.max_read_len ||
            R.win_len > s->cfg.max_win_len || R.read_pos + R.read_len > req->read_arena_bytes * 4)
            return ESP_EINVAL;
    }
    Request *r = new (std::nothrow) Request();
    if (!r) return ESP_ENOMEM;
    r->req = *req;
    r->need = request_need(s, req->n_reads);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->closing) {
        delete r;
        return ESP_ECLOSED;
    }
    if (r->need > s->cfg.mem_budget_bytes) {
        delete r;
        return ESP_EBUSY;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->all[r->ticket] = r;
    s->pending.push_back(r);
    *ticket = r->ticket;
    s->cv_work.notify_one();
    return ESP_OK;
}

int esp_server_wait(esp_server *s, uint64_t ticket, int timeout_ms, int32_t *status,
                    double *latency_ms) {
    if (!s) return ESP_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return ESP_EINVAL;
    Request *r = it->second;
    bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                  [&] { return r->done; });
    if (!ok) return ESP_ETIMEOUT;
    if (status) *status = r->status;
    if (latency_ms) *latency_ms = r->latency_ms;
    s->all.erase(it);
    delete r;
    return ESP_OK;
}

int esp_server_close(esp_server *s) {
    if (!s) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->closing = true;
    s->cv_work.notify_one();
    return ESP_OK;
}

int esp_server_destroy(esp_server *s) {
    if (!s) return ESP_OK;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->closing = true;
            s->stop = true;
            s->cv_work.notify_one();
        }
        s->worker.join();
    }
    for (Slot &sl : s->slots) {
        if (sl.h) cudaStreamSynchronize(sl.h->stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.h_stage) cudaFreeHost(sl.h_stage);
        if (sl.d_stage) cudaFree(sl.d_stage);
        if (sl.h) esp_destroy(sl.h);
    }
    for (auto &kv : s->all) delete kv.second;
    delete s;
    return ESP_OK;
}

}  // extern "C"
