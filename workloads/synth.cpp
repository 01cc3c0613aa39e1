// synth.cpp -- deterministic synthetic workloads (host side, multi-threaded).
//
// The reference ships no datasets for this path (all of its own test inputs
// are generated, crates/map/src/extend.rs:2481-2525), so every benchmark
// configuration is a seeded generator.  Each pair draws from its own
// splitmix64 stream seeded by (seed, pair index), so generation is
// parallel and independent of the thread count.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "esp_workloads.h"

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint8_t base() { return (uint8_t)(next() >> 62); }
};

uint64_t pair_seed(uint64_t seed, uint64_t idx) {
    Rng r(seed * 0x2545F4914F6CDD1Dull + idx * 0x9E3779B97F4A7C15ull + 0x1234567ull);
    r.next();
    return r.next();
}

void put2(uint8_t *arena, uint64_t p, uint8_t c) {
    arena[p >> 2] |= (uint8_t)(c << (6 - 2 * (p & 3)));
}

// Error model shared by the Gotoh configurations: 1% substitutions, 0.1%
// indels (half insertions, half deletions) of geometric length 1..3, and
// A->G at 5% of A positions on forward-strand pairs (T->C on reverse-strand
// pairs, chosen 50/50 per pair).
void derive_read(Rng &rng, const uint8_t *win, uint32_t n, uint32_t s0, uint32_t L,
                 uint8_t *out) {
    bool fwd = rng.next() & 1;
    uint32_t s = s0, k = 0;
    while (k < L) {
        double u = rng.unit();
        if (u < 0.001) {
            uint32_t len = 1;
            while (len < 3 && (rng.next() & 1)) len++;
            if (u < 0.0005) {
                for (uint32_t t = 0; t < len && k < L; t++) out[k++] = rng.base();
                continue;
            }
            s += len;
            continue;
        }
        uint8_t b = s < n ? win[s] : rng.base();
        s++;
        if (rng.unit() < 0.01) {
            b = (uint8_t)((b + 1 + rng.below(3)) & 3);
        } else if (fwd && b == 0 && rng.unit() < 0.05) {
            b = 2;  // A -> G
        } else if (!fwd && b == 3 && rng.unit() < 0.05) {
            b = 1;  // T -> C
        }
        out[k++] = b;
    }
}

struct Shape {
    uint32_t L, n, half;
};

// Shape 0 (banded batch): 150-bp reads from a 214-bp window at offset 32, band half 32.
// Shape 2 (mixed-length batch): L ~ U[50,300], half from {16,32,64,128} w.p. {.4,.3,.2,.1},
//           window L + 2*half, read drawn at offset `half`.
Shape shape_of(int shape, Rng &rng) {
    if (shape == 0) return {150, 214, 32};
    uint32_t L = 50 + rng.below(251);
    double u = rng.unit();
    uint32_t h = u < 0.4 ? 16 : (u < 0.7 ? 32 : (u < 0.9 ? 64 : 128));
    return {L, L + 2 * h, h};
}

template <class F>
void parallel_for(uint64_t n, F f) {
    unsigned T = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < 4096) T = 1;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; t++)
        th.emplace_back([&, t] {
            uint64_t lo = n * t / T, hi = n * (t + 1) / T;
            for (uint64_t i = lo; i < hi; i++) f(i);
        });
    for (auto &x : th) x.join();
}

}  // namespace

extern "C" {

// Sizes of a Gotoh workload: total arena bytes (including 16 bytes of
// padding) for `n_pairs` pairs of shape 0 or 2.
int esp_synth_gotoh_size(uint64_t seed, uint64_t n_pairs, int shape, uint64_t *arena_bytes) {
    if (!arena_bytes || (shape != 0 && shape != 2)) return ESP_EINVAL;
    std::vector<uint64_t> bases(n_pairs);
    parallel_for(n_pairs, [&](uint64_t i) {
        Rng r(pair_seed(seed, i));
        Shape s = shape_of(shape, r);
        bases[i] = s.L + s.n;
    });
    uint64_t tot = 0;
    for (uint64_t b : bases) tot += b;
    *arena_bytes = (tot + 3) / 4 + 16;
    return ESP_OK;
}

// Fill a Gotoh workload: pairs[i] gets the read and window of pair i packed
// into `arena` (zeroed by this call), band offset/half of the shape.
int esp_synth_gotoh(uint64_t seed, uint64_t n_pairs, int shape, uint8_t *arena,
                    uint64_t arena_bytes, esp_pair *pairs) {
    if (!arena || !pairs || (shape != 0 && shape != 2)) return ESP_EINVAL;
    std::vector<Shape> shp(n_pairs);
    parallel_for(n_pairs, [&](uint64_t i) {
        Rng r(pair_seed(seed, i));
        shp[i] = shape_of(shape, r);
    });
    std::vector<uint64_t> pos(n_pairs + 1, 0);
    for (uint64_t i = 0; i < n_pairs; i++) pos[i + 1] = pos[i] + shp[i].L + shp[i].n;
    if ((pos[n_pairs] + 3) / 4 + 16 > arena_bytes) return ESP_EINVAL;
    memset(arena, 0, arena_bytes);
    // Sequences are packed back to back, so the first and last byte of a
    // thread's contiguous pair range may be shared with a neighbour thread;
    // those bytes are collected and OR-ed in a serial pass afterwards.
    unsigned T = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n_pairs < 4096) T = 1;
    std::vector<std::vector<std::pair<uint64_t, uint8_t>>> edge(T);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; t++)
        th.emplace_back([&, t] {
            uint64_t lo = n_pairs * t / T, hi = n_pairs * (t + 1) / T;
            std::vector<uint8_t> win, rd;
            uint64_t first_byte = pos[lo] >> 2, last_byte = pos[hi] >> 2;
            for (uint64_t i = lo; i < hi; i++) {
                Rng r(pair_seed(seed, i));
                Shape s = shape_of(shape, r);  // same draws as the sizing pass
                win.resize(s.n);
                rd.resize(s.L);
                for (uint32_t k = 0; k < s.n; k++) win[k] = r.base();
                derive_read(r, win.data(), s.n, s.half, s.L, rd.data());
                uint64_t p = pos[i];
                for (uint32_t k = 0; k < s.L; k++, p++) {
                    uint64_t b = p >> 2;
                    uint8_t v = (uint8_t)(rd[k] << (6 - 2 * (p & 3)));
                    if (b == first_byte || b == last_byte) edge[t].push_back({b, v});
                    else arena[b] |= v;
                }
                for (uint32_t k = 0; k < s.n; k++, p++) {
                    uint64_t b = p >> 2;
                    uint8_t v = (uint8_t)(win[k] << (6 - 2 * (p & 3)));
                    if (b == first_byte || b == last_byte) edge[t].push_back({b, v});
                    else arena[b] |= v;
                }
                esp_pair &P = pairs[i];
                P.read_pos = pos[i];
                P.win_pos = pos[i] + s.L;
                P.read_len = s.L;
                P.win_len = s.n;
                P.band_offset = (int32_t)s.half;
                P.band_half = (int32_t)s.half;
                P.n_first = 0;
                P.n_read = 0;
                P.n_win = 0;
            }
        });
    for (auto &x : th) x.join();
    for (auto &e : edge)
        for (auto &bv : e) arena[bv.first] |= bv.second;
    return ESP_OK;
}

// Myers workload: 200-bp uniform text; 90% of queries are 150 bases
// sampled from the text at a uniform start in [0, 50] with U{0..8} edits
// (substitution / insertion / deletion, equally likely, at uniform read
// positions), 10% are unrelated random sequence.
static void myers_pair_seqs(uint64_t seed, uint64_t i, uint8_t *text, uint8_t *query) {
    Rng r(pair_seed(seed ^ 0x4D59455253ull, i));
    for (int k = 0; k < 200; k++) text[k] = r.base();
    if (r.unit() < 0.1) {
        for (int k = 0; k < 150; k++) query[k] = r.base();
        return;
    }
    uint32_t start = r.below(51);
    uint32_t edits = r.below(9);
    uint8_t kind[150];
    memset(kind, 0, sizeof(kind));
    for (uint32_t e = 0; e < edits; e++) kind[r.below(150)] = (uint8_t)(1 + r.below(3));
    uint32_t s = start, k = 0, p = 0;
    while (k < 150) {
        uint8_t kd = p < 150 ? kind[p] : 0;
        p++;
        if (kd == 2) {  // insertion
            query[k++] = r.base();
            continue;
        }
        if (kd == 3) {  // deletion
            s++;
            continue;
        }
        uint8_t b = s < 200 ? text[s] : r.base();
        s++;
        if (kd == 1) b = (uint8_t)((b + 1 + r.below(3)) & 3);
        query[k++] = b;
    }
}

int esp_synth_myers_size(uint64_t seed, uint64_t n_pairs, uint64_t *arena_bytes) {
    (void)seed;
    if (!arena_bytes) return ESP_EINVAL;
    *arena_bytes = (n_pairs * 350 + 3) / 4 + 16;
    return ESP_OK;
}

int esp_synth_myers(uint64_t seed, uint64_t n_pairs, uint8_t *arena, uint64_t arena_bytes,
                    esp_myers_pair *pairs) {
    if (!arena || !pairs || (n_pairs * 350 + 3) / 4 + 16 > arena_bytes) return ESP_EINVAL;
    memset(arena, 0, arena_bytes);
    // 350 bases per pair = 87.5 bytes: pairs of pairs share no byte when the
    // work is split on even pair indices (700 bases = 175 whole bytes).
    uint64_t groups = (n_pairs + 1) / 2;
    parallel_for(groups, [&](uint64_t g) {
        uint8_t text[200], query[150];
        for (uint64_t i = 2 * g; i < 2 * g + 2 && i < n_pairs; i++) {
            myers_pair_seqs(seed, i, text, query);
            uint64_t p = i * 350;
            for (int k = 0; k < 150; k++) put2(arena, p + k, query[k]);
            for (int k = 0; k < 200; k++) put2(arena, p + 150 + k, text[k]);
            esp_myers_pair &P = pairs[i];
            P.read_pos = p;
            P.text_pos = p + 150;
            P.read_len = 150;
            P.text_len = 200;
            P.n_first = 0;
            P.n_read = 0;
            P.n_text = 0;
        }
    });
    return ESP_OK;
}

// Splice workload: one contig per read.  Draw order per read (shared by
// the sizing and filling passes): intron length, breakpoint, tail jitter,
// decoy donors, decoy acceptors, supports, then sequence.
struct SpliceShape {
    uint32_t intron, b, ts;
    uint32_t n_dd, n_da;
    int8_t dd[41], da[41];   // decoy offsets from the true donor / acceptor
    uint32_t sup_true;
    uint8_t sup_d[41], sup_a[41];
};

static SpliceShape splice_shape(Rng &r) {
    SpliceShape s;
    double lu = std::log(60.0) + r.unit() * (std::log(50000.0) - std::log(60.0));
    s.intron = (uint32_t)std::exp(lu);
    if (s.intron < 60) s.intron = 60;
    s.b = 20 + r.below(111);
    int ts = (int)s.b + (int)r.below(7) - 3;
    s.ts = (uint32_t)(ts < 1 ? 1 : (ts > 149 ? 149 : ts));
    s.n_dd = s.n_da = 0;
    for (int k = -20; k <= 20; k++)
        if (k != 0 && r.below(16) == 0) s.dd[s.n_dd++] = (int8_t)k;
    for (int k = -20; k <= 20; k++)
        if (k != 0 && r.below(16) == 0) s.da[s.n_da++] = (int8_t)k;
    s.sup_true = 3 + r.below(8);
    for (uint32_t k = 0; k < s.n_dd; k++) s.sup_d[k] = (uint8_t)(1 + r.below(3));
    for (uint32_t k = 0; k < s.n_da; k++) s.sup_a[k] = (uint8_t)(1 + r.below(3));
    return s;
}

int esp_synth_splice_size(uint64_t seed, uint64_t n_reads, uint64_t *genome_bytes,
                          uint64_t *read_bytes, uint64_t *n_cands) {
    if (!genome_bytes || !read_bytes || !n_cands) return ESP_EINVAL;
    std::vector<uint64_t> g(n_reads), c(n_reads);
    parallel_for(n_reads, [&](uint64_t i) {
        Rng r(pair_seed(seed ^ 0x53504C43ull, i));
        SpliceShape s = splice_shape(r);
        g[i] = 600 + s.intron;
        c[i] = 1 + s.n_dd + s.n_da;
    });
    uint64_t gb = 0, cc = 0;
    for (uint64_t i = 0; i < n_reads; i++) {
        gb += (g[i] + 3) / 4 * 4;  // contigs start on whole bytes
        cc += c[i];
    }
    *genome_bytes = gb / 4 + 16;
    *read_bytes = (n_reads * 150 + 3) / 4 + 16;
    *n_cands = cc;
    return ESP_OK;
}

int esp_synth_splice(uint64_t seed, uint64_t n_reads, uint8_t *genome_arena,
                     uint64_t genome_bytes, esp_contig *contigs, uint8_t *read_arena,
                     uint64_t read_bytes, esp_splice_read *reads, esp_splice_cand *cands,
                     uint64_t n_cands) {
    if (!genome_arena || !contigs || !read_arena || !reads || !cands) return ESP_EINVAL;
    std::vector<SpliceShape> shp(n_reads);
    parallel_for(n_reads, [&](uint64_t i) {
        Rng r(pair_seed(seed ^ 0x53504C43ull, i));
        shp[i] = splice_shape(r);
    });
    std::vector<uint64_t> gpos(n_reads + 1, 0), cpos(n_reads + 1, 0);
    for (uint64_t i = 0; i < n_reads; i++) {
        gpos[i + 1] = gpos[i] + (600 + shp[i].intron + 3) / 4 * 4;
        cpos[i + 1] = cpos[i] + 1 + shp[i].n_dd + shp[i].n_da;
    }
    if (gpos[n_reads] / 4 + 16 > genome_bytes || cpos[n_reads] > n_cands ||
        (n_reads * 150 + 3) / 4 + 16 > read_bytes)
        return ESP_EINVAL;
    memset(genome_arena, 0, genome_bytes);
    memset(read_arena, 0, read_bytes);
    // reads pack 150 bases = 37.5 bytes: split the work on even read indices
    uint64_t groups = (n_reads + 1) / 2;
    parallel_for(groups, [&](uint64_t grp) {
        std::vector<uint8_t> ctg, src(200), rd(150);
        for (uint64_t i = 2 * grp; i < 2 * grp + 2 && i < n_reads; i++) {
            Rng r(pair_seed(seed ^ 0x53504C43ull, i));
            SpliceShape s = splice_shape(r);
            uint32_t len = 600 + s.intron, d0 = 300, a0 = 300 + s.intron;
            ctg.resize(len);
            for (uint32_t k = 0; k < len; k++) ctg[k] = r.base();
            for (uint32_t k = 0; k < s.n_dd; k++) {  // decoy GT donors
                uint32_t p = d0 + s.dd[k];
                ctg[p] = 2;
                ctg[p + 1] = 3;
            }
            for (uint32_t k = 0; k < s.n_da; k++) {  // decoy AG acceptors (end at p)
                uint32_t p = a0 + s.da[k];
                ctg[p - 2] = 0;
                ctg[p - 1] = 2;
            }
            ctg[d0] = 2;  // true GT..AG
            ctg[d0 + 1] = 3;
            ctg[a0 - 2] = 0;
            ctg[a0 - 1] = 2;
            for (uint32_t k = 0; k < len; k++) put2(genome_arena, gpos[i] + k, ctg[k]);
            // spliced source: exon1[300-b, 300) + exon2[0, ...)
            for (uint32_t k = 0; k < 200; k++)
                src[k] = k < s.b ? ctg[d0 - s.b + k] : (a0 + (k - s.b) < len ? ctg[a0 + (k - s.b)] : 0);
            derive_read(r, src.data(), 200, 0, 150, rd.data());
            for (uint32_t k = 0; k < 150; k++) put2(read_arena, i * 150 + k, rd[k]);
            esp_contig &C = contigs[i];
            C.base = gpos[i];
            C.len = len;
            C.n_first = 0;
            C.n_count = 0;
            C.pad = 0;
            esp_splice_read &R = reads[i];
            R.read_pos = i * 150;
            R.read_len = 150;
            R.tail_start = s.ts;
            R.contig = (uint32_t)i;
            R.minus = 0;
            R.cand_first = (uint32_t)cpos[i];
            R.cand_count = (uint32_t)(cpos[i + 1] - cpos[i]);
            R.n_first = 0;
            R.n_read = 0;
            // library order: sorted by (start, end)
            std::vector<esp_splice_cand> cs;
            cs.push_back({{(uint32_t)i, d0, a0, 0}, s.sup_true});
            for (uint32_t k = 0; k < s.n_dd; k++)
                cs.push_back({{(uint32_t)i, (uint32_t)(d0 + s.dd[k]), a0, 0}, s.sup_d[k]});
            for (uint32_t k = 0; k < s.n_da; k++)
                cs.push_back({{(uint32_t)i, d0, (uint32_t)(a0 + s.da[k]), 0}, s.sup_a[k]});
            std::sort(cs.begin(), cs.end(), [](const esp_splice_cand &x, const esp_splice_cand &y) {
                return x.j.start != y.j.start ? x.j.start < y.j.start : x.j.end < y.j.end;
            });
            for (size_t k = 0; k < cs.size(); k++) cands[cpos[i] + k] = cs[k];
        }
    });
    return ESP_OK;
}

// Serve workload: uniform-ACGT genome, equal contigs starting on whole
// bytes; every 4 bases are one uniformly random byte.
int esp_synth_genome(uint64_t seed, uint64_t total_bases, uint32_t n_contigs, uint8_t *arena,
                     uint64_t arena_bytes, esp_contig *contigs) {
    if (!arena || !contigs || n_contigs == 0) return ESP_EINVAL;
    uint64_t stride = ((total_bases + n_contigs - 1) / n_contigs + 3) / 4 * 4;
    if (stride > 0xffffffffull) return ESP_EDOMAIN;
    uint64_t bytes = (stride * n_contigs) / 4;
    if (bytes + 16 > arena_bytes) return ESP_EINVAL;
    const uint64_t chunk = 1 << 20;
    uint64_t nchunks = (bytes + chunk - 1) / chunk;
    parallel_for(nchunks, [&](uint64_t c) {
        Rng r(pair_seed(seed ^ 0x47454E4Full, c));
        uint64_t lo = c * chunk, hi = std::min(bytes, lo + chunk);
        for (uint64_t b = lo; b < hi; b += 8) {
            uint64_t v = r.next();
            for (uint64_t k = 0; k < 8 && b + k < hi; k++) arena[b + k] = (uint8_t)(v >> (8 * k));
        }
    });
    memset(arena + bytes, 0, arena_bytes - bytes);
    for (uint32_t c = 0; c < n_contigs; c++) {
        uint64_t base = (uint64_t)c * stride;
        uint64_t len = base >= total_bases ? 0 : std::min<uint64_t>(stride, total_bases - base);
        contigs[c].base = base;
        contigs[c].len = (uint32_t)len;
        contigs[c].n_first = 0;
        contigs[c].n_count = 0;
        contigs[c].pad = 0;
    }
    return ESP_OK;
}

// Serve requests: fragment f = reads 2f, 2f+1 (mates, 150 bp, insert
// 250..450), both as forward-strand reads of the genome with the Gotoh error
// model; window = read position -32 .. +182 (read + 2 x 32), hint offset 32.
int esp_synth_serve_reads(uint64_t seed, uint64_t request, const uint8_t *genome_arena,
                          const esp_contig *contigs, uint32_t n_contigs, uint64_t n_reads,
                          uint8_t *read_arena, uint64_t read_arena_bytes, esp_serve_read *reads) {
    if (!genome_arena || !contigs || !read_arena || !reads || n_contigs == 0) return ESP_EINVAL;
    if ((n_reads * 150 + 3) / 4 + 16 > read_arena_bytes) return ESP_EINVAL;
    memset(read_arena, 0, read_arena_bytes);
    uint64_t frags = (n_reads + 1) / 2;
    parallel_for(frags, [&](uint64_t f) {
        Rng r(pair_seed(seed ^ (0x5345525645ull + request * 0x9E3779B97F4A7C15ull), f));
        uint32_t c = r.below(n_contigs);
        const esp_contig &C = contigs[c];
        uint32_t insert = 250 + r.below(201);
        uint32_t span = insert + 32 + 32 + 200;
        uint32_t p1 = C.len > span ? 32 + r.below(C.len - span) : 32;
        uint32_t pos[2] = {p1, p1 + insert - 150};
        uint8_t win[200], rd[150];
        for (int m = 0; m < 2; m++) {
            uint64_t i = 2 * f + m;
            if (i >= n_reads) break;
            for (int k = 0; k < 200; k++) {
                uint64_t gp = C.base + pos[m] + k;
                win[k] = (uint8_t)((genome_arena[gp >> 2] >> (6 - 2 * (gp & 3))) & 3);
            }
            derive_read(r, win, 200, 0, 150, rd);
            for (int k = 0; k < 150; k++) put2(read_arena, i * 150 + k, rd[k]);
            esp_serve_read &R = reads[i];
            R.read_pos = i * 150;
            R.read_len = 150;
            R.contig = c;
            R.win_start = pos[m] >= 32 ? pos[m] - 32 : 0;
            R.win_len = 214;
            R.hint_offset = (int32_t)(pos[m] - R.win_start);
            R.pad = 0;
        }
    });
    return ESP_OK;
}

}  // extern "C"
