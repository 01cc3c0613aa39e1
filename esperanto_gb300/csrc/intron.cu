// intron.cu -- the intron-chain fast path of crates/map/src/intron_chain.rs
// (try_intron_chain_placement :392-538) from the best fragment pair on, as
// device batches over a resident genome.
//
// Stage 1, intron_prepare (one thread per read): the junction offset, the
// EA-Myers breakpoint refinement of both sides (refine_donor_end /
// refine_acceptor_start :285-343: a pattern of up to 50 read bases against
// the genome within +-30 of the fragment end), the split-read verification
// (verify_split_read :347-373: each half of the read against its side,
// myers_ea::long::infix), the anchor / intron-length / dual-threshold gates,
// the read-aware junction refinement (splice.rs:208-313 refine_junction_read,
// the junction library binary-searched on the device) with the
// best_frag_pair junction as its fallback, and the exon bounds.  The Myers
// scans run per thread in 64-bit blocks, the edlib block form of
// myers_ea.rs:64-91 (every block's horizontal delta chained into the next),
// so they return the reference's distances and ends exactly.
// Stage 2: the spliced pseudo-reference DP of spliced.cu (gather the two
// exon slices, extend_hint along the read's own diagonal, stitch) for the
// reads that pass, and the last gates (positive score, a CIGAR that
// conserves the read and crosses the intron).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <vector>

#include "esp_device.cuh"
#include "esp_host.h"

namespace {

using esp::GenomeView;
using esp::genome_code;
using esp::genome_dinuc;
using esp::signal_bonus;
using esp::splice_signal_of;

constexpr int kMinIntron = 20;  // intron_chain.rs:47 MIN_INTRON

struct ReadSeq {
    const uint8_t *arena;
    uint64_t pos;
    const esp_n_interval *iv;
    uint32_t cnt;
    // base code (0..3, 4 = N) of read position q
    __device__ __forceinline__ uint32_t code(int64_t q) const {
        return esp::code5(arena, pos, iv, cnt, q);
    }
};

// myers_ea.rs:28-38 ea_matches over codes: read A {A}, C {C,T}, G {G,A},
// T {T}; a read or text N matches nothing.
__device__ __forceinline__ bool ea_match(uint32_t r, uint32_t t) {
    return t < 4 && (r == t || (r == 1 && t == 3) || (r == 2 && t == 0));
}

// Semi-global EA-Myers of read[p0, p0 + m) against contig [t0, t0 + n):
// the whole pattern against any text substring.  Returns the minimum
// distance and the earliest exclusive end reaching it (0 when nothing
// beats m), myers_ea.rs:93-155; REV scans both reversed (best start =
// n - reversed end, :158-185).
template <int NW>
__device__ void ea_scan(const ReadSeq &R, int64_t p0, int m, const GenomeView &G,
                        const esp_contig &C, uint32_t t0, uint32_t n, bool rev, int32_t &best,
                        uint32_t &best_at) {
    uint64_t peq[4][NW];
#pragma unroll
    for (int c = 0; c < 4; c++)
#pragma unroll
        for (int w = 0; w < NW; w++) peq[c][w] = 0;
    for (int i = 0; i < m; i++) {
        const uint32_t r = R.code(rev ? p0 + m - 1 - i : p0 + i);
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (ea_match(r, (uint32_t)c)) peq[c][i >> 6] |= 1ull << (i & 63);
    }
    const int last = (m - 1) >> 6;
    const uint64_t top_mask = (m & 63) ? ((1ull << (m & 63)) - 1) : ~0ull;
    uint64_t pv[NW], mv[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) {
        pv[w] = w < last ? ~0ull : (w == last ? top_mask : 0ull);
        mv[w] = 0;
    }
    int32_t score = m;
    best = m;
    best_at = 0;
    for (uint32_t j = 0; j < n; j++) {
        const uint32_t t = genome_code(G, C, rev ? t0 + n - 1 - j : t0 + j);
        int hin = 0;  // the top row of a semi-global search is free
#pragma unroll
        for (int w = 0; w < NW; w++) {
            if (w > last) break;
            const uint64_t mask = w < last ? ~0ull : top_mask;
            const uint64_t high = w < last ? (1ull << 63) : (1ull << ((m - 1) & 63));
            const uint64_t eq_in = t < 4 ? peq[t][w] : 0ull;
            const uint64_t neg = hin < 0 ? 1ull : 0ull, pos1 = hin > 0 ? 1ull : 0ull;
            const uint64_t xv = eq_in | mv[w];
            const uint64_t eq = eq_in | neg;
            const uint64_t xh = (((eq & pv[w]) + pv[w]) ^ pv[w]) | eq;
            const uint64_t ph = mv[w] | ~(xh | pv[w]);
            const uint64_t mh = pv[w] & xh;
            hin = (ph & high) ? 1 : ((mh & high) ? -1 : 0);
            const uint64_t ph_sh = (ph << 1) | pos1, mh_sh = (mh << 1) | neg;
            pv[w] = (mh_sh | ~(xv | ph_sh)) & mask;
            mv[w] = (ph_sh & xv) & mask;
        }
        score += hin;
        if (score < best) {
            best = score;
            best_at = j + 1;
        }
    }
    if (rev) best_at = n - best_at;
}

// m = 0 -> (0, 0 / n); m > 256 -> (m, 0): the entry points' guards.
__device__ void ea_search(const ReadSeq &R, int64_t p0, int m, const GenomeView &G,
                          const esp_contig &C, uint32_t t0, uint32_t n, bool rev, int32_t &best,
                          uint32_t &at) {
    if (m <= 0) {
        best = 0;
        at = 0;
        return;
    }
    if (m > 256) {
        best = m;
        at = 0;
        return;
    }
    if (m <= 64) ea_scan<1>(R, p0, m, G, C, t0, n, rev, best, at);
    else if (m <= 128) ea_scan<2>(R, p0, m, G, C, t0, n, rev, best, at);
    else if (m <= 192) ea_scan<3>(R, p0, m, G, C, t0, n, rev, best, at);
    else ea_scan<4>(R, p0, m, G, C, t0, n, rev, best, at);
}

// gtf.rs:142-149 JunctionLib::support: exact (contig, start, end, strand).
__device__ uint32_t lib_support(const esp_lib_junction *lib, uint64_t n, uint32_t contig,
                                uint32_t start, uint32_t end, int minus) {
    uint64_t lo = 0, hi = n;
    const int mb = minus != 0;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        const esp_junction &x = lib[mid].j;
        const int xb = x.minus_strand != 0;
        if (x.contig == contig && x.start == start && x.end == end && xb == mb)
            return lib[mid].count;
        const bool less = x.contig != contig ? x.contig < contig
                          : x.start != start ? x.start < start
                          : x.end != end     ? x.end < end
                                             : xb < mb;
        if (less) lo = mid + 1;
        else hi = mid;
    }
    return 0;
}

// splice.rs:316-321 edit_equiv over codes (N equals N)
__device__ __forceinline__ bool edit_equiv(uint32_t a, uint32_t b) {
    return a == b || (a == 0 && b == 2) || (a == 2 && b == 0) || (a == 3 && b == 1) ||
           (a == 1 && b == 3);
}

struct IntronJob {
    const esp_intron_read *reads;
    uint64_t n;
    const uint8_t *read_arena;
    const esp_n_interval *read_iv;
    GenomeView G;
    const esp_contig *contigs;
    const esp_lib_junction *lib;
    uint64_t n_lib;
    esp_intron_params ip;
    esp_splice_params sp;  // SpliceParams::default() with max_intron = ip.intron_max
    esp_intron_result *out;
    int64_t *hint;         // the pseudo-reference DP's hint offset per read
};

__global__ void __launch_bounds__(128) intron_prepare(IntronJob J) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < J.n;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const esp_intron_read E = J.reads[r];
        esp_intron_result o{};
        o.verify_donor = o.verify_acceptor = INT_MAX;
        o.junction.contig = E.contig;
        o.status = ESP_OK;
        J.hint[r] = 0;
        const uint32_t len = E.read_len;
        if (len == 0) {
            o.stage = ESP_IC_EMPTY;
            J.out[r] = o;
            continue;
        }
        const esp_contig C = J.contigs[E.contig];
        const ReadSeq R{J.read_arena, E.read_pos, J.read_iv + E.n_first, E.n_read};
        const esp_frag &L = E.left, &Rf = E.right;
        const int64_t left_off = (int64_t)L.r_lo - L.q_lo, right_off = (int64_t)Rf.r_lo - Rf.q_lo;
        const int64_t clen = C.len, w = J.ip.refine_window, plen = J.ip.refine_pattern_len;
        // junction offset: the read midpoint clamped into the fragments' read gap
        const uint32_t j_est = len / 2;
        uint32_t off = j_est;
        if (L.q_hi < Rf.q_lo) off = j_est < L.q_hi ? L.q_hi : (j_est > Rf.q_lo ? Rf.q_lo : j_est);
        off = off < len ? off : len;
        // refine_donor_end
        int64_t donor = L.r_hi ? (int64_t)L.r_hi - 1 : 0;
        {
            const int64_t lo = max((int64_t)L.r_hi - w, (int64_t)0);
            const int64_t hi = min((int64_t)L.r_hi + w, clen);
            if (hi > lo && off > 0) {
                const int64_t text_lo_in_read = max(lo - left_off + 2, (int64_t)0);
                const int64_t ps = max((int64_t)off - plen, max((int64_t)0, text_lo_in_read));
                if (ps < (int64_t)off) {
                    int32_t d;
                    uint32_t end;
                    ea_search(R, ps, (int)(off - ps), J.G, C, (uint32_t)lo, (uint32_t)(hi - lo),
                              false, d, end);
                    donor = lo + end;
                }
            }
        }
        // refine_acceptor_start
        int64_t acc = Rf.r_lo;
        {
            const int64_t lo = max((int64_t)Rf.r_lo - w, (int64_t)0);
            const int64_t hi = min((int64_t)Rf.r_lo + w, clen);
            if (hi > lo) {
                const int64_t text_hi_in_read = max(hi - right_off - 2, (int64_t)0);
                const int64_t pe = min(min((int64_t)off + plen, (int64_t)len), text_hi_in_read);
                if (pe > (int64_t)off) {
                    int32_t d;
                    uint32_t start;
                    ea_search(R, off, (int)(pe - off), J.G, C, (uint32_t)lo, (uint32_t)(hi - lo),
                              true, d, start);
                    acc = lo + start;
                }
            }
        }
        o.donor_end = (uint32_t)donor;
        o.acceptor_start = (uint32_t)acc;
        const int64_t intron_len = acc - donor - 1;
        // verify_split_read
        {
            const uint32_t mid = len / 2;
            const int64_t d0 = max(left_off - 30, (int64_t)0);
            const int64_t d1 = min(max(donor + 1 + 30, (int64_t)1), clen);
            const int64_t a0 = min(max(acc - 30, (int64_t)0), clen);
            const int64_t a1 = min(max((int64_t)Rf.r_hi + 30, a0 + 1), clen);
            if (d0 < d1 && a0 < a1 && mid > 0 && mid < len) {
                uint32_t at;
                ea_search(R, 0, (int)mid, J.G, C, (uint32_t)d0, (uint32_t)(d1 - d0), false,
                          o.verify_donor, at);
                ea_search(R, mid, (int)(len - mid), J.G, C, (uint32_t)a0, (uint32_t)(a1 - a0),
                          false, o.verify_acceptor, at);
            }
        }
        const int64_t max_v = max(o.verify_donor, o.verify_acceptor);
        const int64_t sum_v = (int64_t)o.verify_donor + o.verify_acceptor;
        // (f64 thresholds, intron_chain.rs:446-447: len * 0.17 / 0.24 truncated)
        const int64_t max_t = (int64_t)((double)len * 0.17), sum_t = (int64_t)((double)len * 0.24);
        if (L.n_anchors + Rf.n_anchors < 2) o.stage = ESP_IC_ANCHORS;
        else if (intron_len < kMinIntron || intron_len > (int64_t)J.ip.intron_max)
            o.stage = ESP_IC_INTRON;
        else if (max_v > max_t || sum_v > sum_t) o.stage = ESP_IC_VERIFY;
        if (o.stage) {
            J.out[r] = o;
            continue;
        }
        // refine_junction_read (splice.rs:208-313), falling back to the
        // fragment pair's own junction
        bool have = false;
        {
            const int64_t ref_gap = (int64_t)Rf.r_lo - L.r_hi, read_gap = (int64_t)Rf.q_lo - L.q_hi;
            const int64_t il = ref_gap - read_gap;
            if (read_gap <= 20 && il >= (int64_t)J.sp.min_intron && il <= (int64_t)J.sp.max_intron) {
                const int64_t lo = min(read_gap, (int64_t)0) - 2, hi = max(read_gap, (int64_t)0) + 2;
                int32_t best = 0;
                for (int64_t delta = lo; delta <= hi; delta++) {
                    const int64_t s = (int64_t)L.r_hi + delta;
                    if (s < 0) continue;
                    const int64_t e = s + il;
                    if (e < 2 || e > clen) continue;
                    const int64_t qb = (int64_t)L.q_hi + delta;
                    if (qb < 1 || qb >= (int64_t)len) continue;
                    int32_t m = 0;
                    for (int64_t i = 1; i <= 4; i++) {
                        const int64_t q1 = qb - i, g1 = s - i;
                        if (q1 >= 0 && g1 >= 0 &&
                            edit_equiv(R.code(q1), genome_code(J.G, C, (uint32_t)g1)))
                            m++;
                        const int64_t q2 = qb + i - 1, g2 = e + i - 1;
                        if (q2 < (int64_t)len && g2 < clen &&
                            edit_equiv(R.code(q2), genome_code(J.G, C, (uint32_t)g2)))
                            m++;
                    }
                    uint8_t dn[2], ac[2];
                    genome_dinuc(J.G, C, (uint32_t)s, true, dn);
                    genome_dinuc(J.G, C, (uint32_t)e, false, ac);
                    for (int t = 0; t < 2; t++) {
                        const int tm = t == 0 ? (E.minus != 0) : (E.minus == 0);
                        const int sig = splice_signal_of(dn, ac, tm != 0);
                        const uint32_t sup =
                            lib_support(J.lib, J.n_lib, E.contig, (uint32_t)s, (uint32_t)e, tm);
                        const int64_t ad = delta < 0 ? -delta : delta;
                        int32_t score = m * 50 + signal_bonus(sig, J.sp) * 5 - (int32_t)ad * 5;
                        if (sup > 0) score += J.sp.known_bonus;
                        if (!have || score > best) {
                            have = true;
                            best = score;
                            o.junction.start = (uint32_t)s;
                            o.junction.end = (uint32_t)e;
                            o.junction.minus_strand = tm;
                            o.signal = sig;
                            o.support = sup;
                        }
                    }
                }
            }
        }
        if (!have) {
            o.junction.start = E.intron_start;
            o.junction.end = E.intron_end;
            o.junction.minus_strand = E.minus != 0;
            o.support = lib_support(J.lib, J.n_lib, E.contig, E.intron_start, E.intron_end,
                                    E.minus != 0);
            uint8_t dn[2], ac[2];  // splice.rs:864-868 junction_signal
            genome_dinuc(J.G, C, E.intron_start, true, dn);
            genome_dinuc(J.G, C, E.intron_end, false, ac);
            o.signal = splice_signal_of(dn, ac, E.minus != 0);
        }
        const esp_junction &jn = o.junction;
        if (jn.end <= jn.start || jn.end - jn.start < (uint32_t)kMinIntron ||
            jn.end - jn.start > J.ip.intron_max) {
            o.stage = ESP_IC_JUNCTION;
            J.out[r] = o;
            continue;
        }
        const uint32_t left_start = L.r_lo > len ? L.r_lo - len : 0;
        const uint32_t right_end = (uint32_t)min((int64_t)Rf.r_hi + len, clen);
        if (left_start >= jn.start || jn.end >= right_end) {
            o.stage = ESP_IC_BOUNDS;
            J.out[r] = o;
            continue;
        }
        o.left_start = left_start;
        o.right_end = right_end;
        o.stage = -1;  // on to the pseudo-reference DP
        J.hint[r] = left_off - (int64_t)left_start;
        J.out[r] = o;
    }
}

}  // namespace

extern "C" int esp_batch_intron_chain_host(
    esp_handle *h, const esp_genome *g, const esp_intron_read *reads, uint64_t n,
    const uint8_t *read_arena, uint64_t read_arena_bytes, const esp_n_interval *read_iv,
    uint64_t n_read_iv, const esp_lib_junction *lib, uint64_t n_lib, const esp_intron_params *ip,
    const esp_extend_params *params, esp_intron_result *out, uint32_t *ext_cigar,
    uint32_t *stitched_cigar, uint32_t cigar_stride) {
    if (!h || !g || !params || !ip || (n && (!reads || !read_arena || !out || !ext_cigar ||
                                             !stitched_cigar)) ||
        (n_read_iv && !read_iv) || (n_lib && !lib))
        return fail(h, ESP_EINVAL, "null argument");
    if (n == 0) return ESP_OK;
    if (cigar_stride == 0) return fail(h, ESP_EINVAL, "zero CIGAR stride");
    esp::GotohConst K;
    if (esp::make_gotoh_const(*params, K) != ESP_OK)
        return fail(h, ESP_EDOMAIN, "scoring parameters outside the device domain");
    for (uint64_t r = 0; r < n; r++) {
        const esp_intron_read &E = reads[r];
        if (E.contig >= g->contigs.size() || E.read_pos + E.read_len > read_arena_bytes * 4 ||
            (uint64_t)E.n_first + E.n_read > n_read_iv || E.read_len > 32767)
            return fail(h, ESP_EINVAL, "read record outside its tables");
    }
    for (uint64_t k = 1; k < n_lib; k++) {  // the library's binary search wants its order
        const esp_junction &a = lib[k - 1].j, &b = lib[k].j;
        const bool ok = a.contig != b.contig ? a.contig < b.contig
                        : a.start != b.start ? a.start < b.start
                        : a.end != b.end     ? a.end < b.end
                                             : (a.minus_strand != 0) <= (b.minus_strand != 0);
        if (!ok) return fail(h, ESP_EINVAL, "junction library not sorted by (contig, start, end, strand)");
    }
    CK(h, cudaSetDevice(h->device));
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t o_reads = 0, o_arena = al(n * sizeof(esp_intron_read)),
                 o_iv = o_arena + al(read_arena_bytes + 16),
                 o_lib = o_iv + al(n_read_iv * sizeof(esp_n_interval) + 8),
                 o_out = o_lib + al(n_lib * sizeof(esp_lib_junction) + 8),
                 o_hint = o_out + al(n * sizeof(esp_intron_result)),
                 total = o_hint + al(n * sizeof(int64_t));
    int rc;
    if ((rc = grow_device(h, &h->d_int, &h->d_int_cap, total)) != ESP_OK) return rc;
    uint8_t *b = (uint8_t *)h->d_int;
    cudaStream_t st = h->stream;
    CK(h, cudaMemcpyAsync(b + o_reads, reads, n * sizeof(esp_intron_read), cudaMemcpyHostToDevice, st));
    CK(h, cudaMemcpyAsync(b + o_arena, read_arena, read_arena_bytes, cudaMemcpyHostToDevice, st));
    CK(h, cudaMemsetAsync(b + o_arena + read_arena_bytes, 0, 16, st));
    if (n_read_iv)
        CK(h, cudaMemcpyAsync(b + o_iv, read_iv, n_read_iv * sizeof(esp_n_interval),
                              cudaMemcpyHostToDevice, st));
    if (n_lib)
        CK(h, cudaMemcpyAsync(b + o_lib, lib, n_lib * sizeof(esp_lib_junction),
                              cudaMemcpyHostToDevice, st));
    IntronJob J{};
    J.reads = (const esp_intron_read *)(b + o_reads);
    J.n = n;
    J.read_arena = b + o_arena;
    J.read_iv = (const esp_n_interval *)(b + o_iv);
    J.G = GenomeView{g->d_arena, g->d_iv};
    J.contigs = g->d_contigs;
    J.lib = (const esp_lib_junction *)(b + o_lib);
    J.n_lib = n_lib;
    J.ip = *ip;
    // SpliceParams { max_intron: intron_max, ..SpliceParams::default() }
    J.sp = esp_splice_params{20, ip->intron_max, 4, 2, 1, 8, 6, 12};
    J.out = (esp_intron_result *)(b + o_out);
    J.hint = (int64_t *)(b + o_hint);
    const int grid = (int)std::min<uint64_t>((n + 127) / 128, (uint64_t)h->num_sms * 8);
    intron_prepare<<<grid, 128, 0, st>>>(J);
    CK(h, cudaGetLastError());
    std::vector<int64_t> hint(n);
    CK(h, cudaMemcpyAsync(out, b + o_out, n * sizeof(esp_intron_result), cudaMemcpyDeviceToHost, st));
    CK(h, cudaMemcpyAsync(hint.data(), b + o_hint, n * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    // stage 2: the pseudo-reference DP of the reads that passed
    std::vector<uint64_t> idx;
    std::vector<esp_spliced_read> sr;
    std::vector<esp_exon> ex;
    std::vector<int64_t> off;
    for (uint64_t r = 0; r < n; r++) {
        if (out[r].stage != -1) continue;
        const esp_intron_read &E = reads[r];
        const esp_intron_result &o = out[r];
        esp_spliced_read s{};
        s.read_pos = E.read_pos;
        s.read_len = E.read_len;
        s.contig = E.contig;
        s.exon_first = (uint32_t)ex.size();
        s.exon_count = 2;
        s.n_first = E.n_first;
        s.n_read = E.n_read;
        ex.push_back({o.left_start, o.junction.start});
        ex.push_back({o.junction.end, o.right_end});
        sr.push_back(s);
        off.push_back(hint[r]);
        idx.push_back(r);
    }
    const uint64_t m = idx.size();
    std::vector<esp_spliced_result> sres(m);
    std::vector<uint32_t> ec(m * (size_t)cigar_stride), sc(m * (size_t)cigar_stride);
    if (m) {
        rc = spliced_batch(h, g, sr.data(), m, read_arena, read_arena_bytes, read_iv, n_read_iv,
                           ex.data(), ex.size(), params, off.data(), sres.data(), ec.data(),
                           sc.data(), cigar_stride);
        if (rc != ESP_OK) return rc;
    }
    for (uint64_t k = 0; k < m; k++) {
        const uint64_t r = idx[k];
        esp_intron_result &o = out[r];
        const esp_spliced_result &s = sres[k];
        o.ext = s.ext;
        o.genomic_start = s.genomic_start;
        o.n_ops = s.n_ops;
        o.status = s.status;
        memcpy(ext_cigar + r * (size_t)cigar_stride, ec.data() + k * (size_t)cigar_stride,
               cigar_stride * sizeof(uint32_t));
        memcpy(stitched_cigar + r * (size_t)cigar_stride, sc.data() + k * (size_t)cigar_stride,
               cigar_stride * sizeof(uint32_t));
        if (s.status != ESP_OK) {  // a CIGAR longer than the stride: undecided
            o.stage = ESP_IC_RESULT;
            continue;
        }
        // extension.score > 0, cigar_conserving (intron_chain.rs:376-386),
        // and an intron in the stitched CIGAR
        const uint32_t *ops = stitched_cigar + r * (size_t)cigar_stride;
        uint64_t q = 0;
        bool has_n = false;
        for (uint32_t t = 0; t < s.n_ops; t++) {
            const uint32_t code = ops[t] & 15u;
            if (code == ESP_OP_M || code == ESP_OP_I || code == ESP_OP_S) q += ops[t] >> 4;
            has_n |= code == ESP_OP_N;
        }
        if (s.ext.score > 0 && q == reads[r].read_len && has_n) {
            o.found = 1;
            o.stage = ESP_IC_FOUND;
        } else {
            o.stage = ESP_IC_RESULT;
        }
    }
    return ESP_OK;
}
