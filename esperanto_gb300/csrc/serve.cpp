// serve.cpp -- continuous-batching serving loop over a resident genome.
//
// One native worker thread owns the device side.  Submitted requests queue
// FIFO; the scheduler (serve_sched.h) turns the head of the queue into
// launches of up to max_reads reads, so small requests that arrive together
// share one launch and a large request runs over several.  Each launch is
// charged the DP scratch it actually needs -- traceback words for its
// longest read and window under the extend_hint policy's full-matrix attempt
// -- from one device pool of mem_budget_bytes shared by all slots, so the
// memory budget, not the slot count, bounds how much runs at once: a launch
// that does not fit is cut to what does, and the head request waits when
// nothing fits until a running launch returns its scratch.  A slot is a CUDA
// stream (a private esp_handle whose DP scratch is the region carved for
// its launch) plus pinned staging for max_reads reads; its launches overlap
// on the device with the other slots'.  Serving allocates nothing after
// start-up.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "esp_host.h"
#include "serve_sched.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr uint64_t kMinLaunch = 1024;  // reads: a launch cut to fit memory keeps at least this many
constexpr uint32_t kMaxStride = 64;    // CIGAR ops per read the staging holds

struct Request {
    uint64_t ticket = 0;
    esp_serve_request req{};
    Clock::time_point t_submit;
    serve::Job job;
    int32_t err = ESP_OK;  // first failing launch of its reads
    int32_t status = 1;    // 1 = pending / in flight
    double latency_ms = 0;
    bool done = false;
};

struct Slot {
    esp_handle *h = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    serve::Launch L;             // the launch it runs (pieces of requests)
    uint32_t stride = 0;         // CIGAR stride of its requests
    int staged_rc = ESP_OK;      // launch() status of the current launch
    uint8_t *h_stage = nullptr;  // pinned: pairs | n intervals | read arena | out | cigar
    uint8_t *d_stage = nullptr;
    size_t off_iv = 0, off_arena = 0, off_out = 0, off_cig = 0, bytes = 0;
};

}  // namespace

struct esp_server {
    esp_genome *g = nullptr;
    esp::GotohConst K{};
    esp_server_config cfg{};
    int device = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::unordered_map<uint64_t, Request *> all;
    serve::Scheduler sched;
    uint8_t *d_pool = nullptr;  // the DP scratch pool: mem_budget_bytes of device memory
    uint64_t next_ticket = 1;
    bool closing = false, stop = false;
    std::thread worker;
};

namespace {

// Traceback / row-buffer bytes of a launch of n reads of at most m x n
// bases in extend_hint mode, as laid out in its pool region.
void launch_scratch(esp_handle *h, uint64_t n, uint32_t m, uint32_t w, uint64_t &tb,
                    uint64_t &rb) {
    Limits L1, L2;
    add_limits(L1, m, w, 30);
    add_limits(L2, m, w, -1);
    dp_scratch_bytes(h, ESP_MODE_HINT, n, L1, L2, tb, rb);
}

// Place `len` 2-bit bases of src (from base src_pos) at base dst_pos of dst.
void copy_bases(const uint8_t *src, uint64_t src_pos, uint8_t *dst, uint64_t dst_pos,
                uint64_t len) {
    for (uint64_t k = 0; k < len; k++) {
        const uint64_t s = src_pos + k, d = dst_pos + k;
        const uint8_t c = (src[s >> 2] >> (6 - 2 * (s & 3))) & 3;
        const int sh = 6 - 2 * (int)(d & 3);
        dst[d >> 2] = (uint8_t)((dst[d >> 2] & ~(3 << sh)) | (c << sh));
    }
}

// Host side of one launch: build the DP pairs of its pieces (windows point
// straight into the resident genome; genome N runs are clipped into per-pair
// intervals; each piece's read bases are staged after the previous piece's),
// point the slot's handle at the launch's pool region, copy, run, copy back,
// record completion.
int launch(esp_server *s, Slot &sl) {
    const serve::Launch &L = sl.L;
    esp_pair *pairs = (esp_pair *)sl.h_stage;
    esp_n_interval *iv = (esp_n_interval *)(sl.h_stage + sl.off_iv);
    uint8_t *arena = sl.h_stage + sl.off_arena;
    const uint64_t arena_cap = sl.off_out - sl.off_arena - 16;
    const size_t iv_cap = (sl.off_arena - sl.off_iv) / sizeof(esp_n_interval);
    const esp_genome *g = s->g;
    uint64_t niv = 0, k = 0, cursor = 0;  // pairs written; arena bytes used
    for (const serve::Piece &pc : L.pieces) {
        const esp_serve_request &q = ((Request *)pc.job->user)->req;
        // the piece's read bases: one copy of the byte span they occupy when
        // it fits the staging, else read by read
        uint64_t lo = UINT64_MAX, hi = 0;
        for (uint64_t i = pc.first; i < pc.first + pc.count; i++) {
            lo = std::min<uint64_t>(lo, q.reads[i].read_pos);
            hi = std::max<uint64_t>(hi, q.reads[i].read_pos + q.reads[i].read_len);
        }
        // (a dense span: at most the per-read share the staging is sized for)
        const uint64_t b0 = lo / 4, b1 = (hi + 3) / 4;
        const bool span = b1 - b0 <= pc.count * ((uint64_t)s->cfg.max_read_len / 4 + 2) &&
                          b1 - b0 <= arena_cap - cursor;
        if (span) memcpy(arena + cursor, q.read_arena + b0, b1 - b0);
        for (uint64_t i = pc.first; i < pc.first + pc.count; i++, k++) {
            const esp_serve_read &R = q.reads[i];
            const esp_contig &C = g->contigs[R.contig];
            uint32_t ws = std::min(R.win_start, C.len);
            uint32_t we = (uint32_t)std::min<uint64_t>((uint64_t)ws + R.win_len, C.len);
            esp_pair P{};
            if (span) {
                P.read_pos = R.read_pos - 4 * b0 + 4 * cursor;
            } else {
                if ((R.read_len + 3) / 4 > arena_cap - cursor) return ESP_EDOMAIN;
                P.read_pos = 4 * cursor;
                copy_bases(q.read_arena, R.read_pos, arena, P.read_pos, R.read_len);
                cursor += (R.read_len + 3) / 4;
            }
            P.read_len = R.read_len;
            P.win_pos = C.base + ws;
            P.win_len = we - ws;
            P.band_offset = R.hint_offset;
            P.band_half = 30;
            P.n_first = (uint32_t)niv;
            if (g->n_iv) {
                // the contig's intervals are sorted and disjoint: start at the
                // first one ending after the window start
                const esp_n_interval *cv = g->h_iv.data() + C.n_first;
                uint32_t a = 0, b = C.n_count, cnt = 0;
                while (a < b) {
                    uint32_t mid = (a + b) >> 1;
                    if (cv[mid].end <= ws) a = mid + 1;
                    else b = mid;
                }
                for (uint32_t t = a; t < C.n_count && cv[t].start < we; t++) {
                    uint32_t x = std::max(cv[t].start, ws), y = std::min(cv[t].end, we);
                    if (x < y) {
                        if (niv >= iv_cap) return ESP_EDOMAIN;
                        iv[niv++] = {x - ws, y - ws};
                        cnt++;
                    }
                }
                P.n_win = (uint16_t)cnt;
            }
            pairs[k] = P;
        }
        if (span) cursor += b1 - b0;
    }
    memset(arena + cursor, 0, 16);
    esp_handle *h = sl.h;
    // the launch's DP scratch: its region of the pool
    uint64_t tb, rb;
    launch_scratch(h, L.n, L.max_m, L.max_n, tb, rb);
    if (serve::al256(tb) + rb > L.bytes) return ESP_ENOMEM;
    h->d_tb = (uint32_t *)(s->d_pool + L.off);
    h->d_tb_cap = tb;
    h->d_rb = (uint32_t *)(s->d_pool + L.off + serve::al256(tb));
    h->d_rb_cap = rb;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(sl.d_stage, sl.h_stage, L.n * sizeof(esp_pair), cudaMemcpyHostToDevice,
                          st));
    if (niv)
        CK(h, cudaMemcpyAsync(sl.d_stage + sl.off_iv, sl.h_stage + sl.off_iv,
                              niv * sizeof(esp_n_interval), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(sl.d_stage + sl.off_arena, arena, cursor + 16, cudaMemcpyHostToDevice,
                          st));
    Limits L1, L2;
    add_limits(L1, L.max_m, L.max_n, 30);
    add_limits(L2, L.max_m, L.max_n, -1);
    int rc = enqueue_batch(h, ESP_MODE_HINT, (const esp_pair *)sl.d_stage, L.n,
                           sl.d_stage + sl.off_arena, cursor,
                           niv ? (const esp_n_interval *)(sl.d_stage + sl.off_iv) : nullptr, niv,
                           s->K, L1, L2, (esp_extension *)(sl.d_stage + sl.off_out),
                           (uint32_t *)(sl.d_stage + sl.off_cig), sl.stride, st, g->d_arena,
                           g->arena_bytes);
    if (rc != ESP_OK) return rc;
    CK(h, cudaMemcpyAsync(sl.h_stage + sl.off_out, sl.d_stage + sl.off_out,
                          L.n * sizeof(esp_extension), cudaMemcpyDeviceToHost, st));
    if (sl.stride)
        CK(h, cudaMemcpyAsync(sl.h_stage + sl.off_cig, sl.d_stage + sl.off_cig,
                              L.n * (size_t)sl.stride * 4, cudaMemcpyDeviceToHost, st));
    CK(h, cudaEventRecord(sl.done, st));
    return ESP_OK;
}

// Results of a finished launch into its requests' buffers (worker thread,
// no lock held: the slot belongs to the worker until finish()).
void copy_out(Slot &sl) {
    uint64_t k = 0;
    for (const serve::Piece &pc : sl.L.pieces) {
        const esp_serve_request &q = ((Request *)pc.job->user)->req;
        memcpy(q.out + pc.first, sl.h_stage + sl.off_out + k * sizeof(esp_extension),
               pc.count * sizeof(esp_extension));
        if (q.cigar && sl.stride)
            memcpy(q.cigar + pc.first * sl.stride, sl.h_stage + sl.off_cig + k * sl.stride * 4,
                   pc.count * (size_t)sl.stride * 4);
        k += pc.count;
    }
}

// Publish a request as done (server lock held).
void complete(Request *r, int32_t status) {
    r->status = status;
    r->latency_ms =
        std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
    r->done = true;
}

// The worker owns the slots.  The server lock guards the scheduler, the
// ticket table and the request states: staging a launch, launching it and
// copying results out run unlocked, so submitters and waiters are never held
// up by the bulk copies.
void worker_loop(esp_server *s) {
    cudaSetDevice(s->device);
    std::vector<std::pair<Slot *, int32_t>> done;
    std::vector<Slot *> to_launch;
    std::vector<serve::Job *> finished;
    for (;;) {
        done.clear();
        for (Slot &sl : s->slots) {
            if (!sl.busy || sl.staged_rc != ESP_OK) continue;
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
                if (sl.busy && sl.staged_rc != ESP_OK) done.push_back({&sl, sl.staged_rc});
            for (auto &d : done) {
                Slot &sl = *d.first;
                for (const serve::Piece &pc : sl.L.pieces) {
                    Request *r = (Request *)pc.job->user;
                    if (d.second != ESP_OK && r->err == ESP_OK) r->err = d.second;
                }
                finished.clear();
                s->sched.finish(sl.L, finished);
                for (serve::Job *j : finished) {
                    Request *r = (Request *)j->user;
                    complete(r, r->err);
                }
                sl.busy = false;
            }
            bool notify = !done.empty();
            if (s->closing) {  // requests none of whose reads started: ESP_ECLOSED
                finished.clear();
                s->sched.drop_unstarted(finished);
                for (serve::Job *j : finished) complete((Request *)j->user, ESP_ECLOSED);
                notify |= !finished.empty();
            }
            if (notify) s->cv_done.notify_all();
            // admission: every idle slot takes the next launch the scheduler
            // builds from the head of the queue (FIFO) while memory allows
            for (Slot &sl : s->slots) {
                if (sl.busy) continue;
                if (!s->sched.next(sl.L)) break;
                sl.busy = true;
                sl.staged_rc = ESP_OK;
                sl.stride = ((Request *)sl.L.pieces[0].job->user)->req.cigar_stride;
                to_launch.push_back(&sl);
            }
            for (Slot &sl : s->slots) inflight |= sl.busy;
            stop = s->stop && !inflight && s->sched.empty();
            if (!stop && !inflight) {
                s->cv_work.wait(lk);
                continue;
            }
        }
        if (stop) break;
        for (Slot *sl : to_launch) sl->staged_rc = launch(s, *sl);
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
    // a launch stays on the one-pair kernel (below the paired kernel's size)
    if (c.max_reads >= (1u << 20) || c.n_streams > 64) {
        delete s;
        return ESP_EINVAL;
    }
    if (c.max_read_len > 32767 || c.max_win_len > 32767 ||
        c.max_read_len > (uint32_t)s->K.max_m) {
        delete s;
        return ESP_EDOMAIN;
    }
    s->cfg = c;
    s->g = g;
    s->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete s;
        return ESP_ECUDA;
    }
    s->slots.resize(c.n_streams);
    int rc = ESP_OK;
    if (cudaMalloc((void **)&s->d_pool, c.mem_budget_bytes) != cudaSuccess) {
        s->d_pool = nullptr;
        rc = ESP_ENOMEM;
    }
    for (Slot &sl : s->slots) {
        if (rc != ESP_OK) break;
        if ((rc = esp_create(&sl.h, device)) != ESP_OK) break;
        sl.h->scratch_external = true;  // launches run in their pool region
        sl.h->scratch_budget = c.mem_budget_bytes;
        if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            rc = ESP_ECUDA;
            break;
        }
        // escalation and binning lists for the largest launch, so serving
        // never allocates
        if ((rc = reserve_lists(sl.h, c.max_reads)) != ESP_OK) break;
        const uint64_t n = c.max_reads;
        sl.off_iv = serve::al256(n * sizeof(esp_pair));
        sl.off_arena = sl.off_iv + serve::al256(n * 4 * sizeof(esp_n_interval));
        sl.off_out = sl.off_arena + serve::al256(n * ((uint64_t)c.max_read_len / 4 + 2) + 64);
        sl.off_cig = sl.off_out + serve::al256(n * sizeof(esp_extension));
        sl.bytes = sl.off_cig + serve::al256(n * kMaxStride * 4);
        if (cudaMallocHost((void **)&sl.h_stage, sl.bytes) != cudaSuccess ||
            cudaMalloc((void **)&sl.d_stage, sl.bytes) != cudaSuccess) {
            rc = ESP_ENOMEM;
            break;
        }
    }
    if (rc != ESP_OK) {
        esp_server_destroy(s);
        return rc;
    }
    // the slot handles' kernel choices are settled here, once, so that the
    // scheduler's scratch sizing (slot 0's handle, from any thread) only
    // reads them afterwards
    for (Slot &sl : s->slots) {
        uint64_t tb, rb;
        launch_scratch(sl.h, c.max_reads, c.max_read_len, c.max_win_len, tb, rb);
        launch_scratch(sl.h, 1, c.max_read_len, c.max_win_len, tb, rb);
    }
    esp_handle *h0 = s->slots[0].h;
    s->sched = serve::Scheduler(
        c.mem_budget_bytes, c.max_reads, kMinLaunch, [h0](uint64_t n, uint32_t m, uint32_t w) {
            uint64_t tb, rb;
            launch_scratch(h0, n, m, w, tb, rb);
            return serve::al256(tb) + rb;
        });
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return ESP_OK;
}

int esp_server_submit(esp_server *s, const esp_serve_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket || (req->n_reads && (!req->reads || !req->read_arena || !req->out)))
        return ESP_EINVAL;
    if (req->cigar_stride > kMaxStride) return ESP_EINVAL;
    Request *r = new (std::nothrow) Request();
    if (!r) return ESP_ENOMEM;
    r->req = *req;
    serve::Job &j = r->job;
    j.n = req->n_reads;
    j.group = req->cigar_stride;
    j.user = r;
    for (uint64_t i = 0; i < req->n_reads; i++) {
        const esp_serve_read &R = req->reads[i];
        if (R.contig >= s->g->contigs.size() || R.read_len > s->cfg.max_read_len ||
            R.win_len > s->cfg.max_win_len || R.read_pos + R.read_len > req->read_arena_bytes * 4) {
            delete r;
            return ESP_EINVAL;
        }
        j.max_m = std::max(j.max_m, R.read_len);
        j.max_n = std::max(j.max_n, R.win_len);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->closing) {
        delete r;
        return ESP_ECLOSED;
    }
    if (!s->sched.admissible(j)) {  // its smallest launch exceeds the whole memory budget
        delete r;
        return ESP_EBUSY;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->all[r->ticket] = r;
    if (j.n == 0) {
        complete(r, ESP_OK);
    } else {
        s->sched.push(&j);
        s->cv_work.notify_one();
    }
    *ticket = r->ticket;
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

int esp_server_get_stats(esp_server *s, esp_server_stats *out) {
    if (!s || !out) return ESP_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    const serve::Stats &t = s->sched.stats();
    out->launches = t.launches;
    out->reads = t.reads;
    out->merged_launches = t.merged;
    out->split_requests = t.split_jobs;
    out->budget_waits = t.budget_waits;
    out->cut_launches = t.cuts;
    out->pool_bytes = s->sched.pool().size();
    out->pool_peak_bytes = s->sched.pool().peak();
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
    if (s->d_pool) cudaFree(s->d_pool);
    for (auto &kv : s->all) delete kv.second;
    delete s;
    return ESP_OK;
}

}  // extern "C"
