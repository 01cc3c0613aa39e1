// paidx.cpp -- read the contigs of a paidx v1 index (crates/map/src/index_io.rs)
// straight into the resident-genome layout.
//
// The index file already stores every contig 2-bit packed MSB-first with its
// N runs (fasta.rs:1-5), which is exactly the device genome's layout, so
// loading is a validated walk over the bytes plus one copy per contig: no
// FASTA parse and no per-base decode.  Each contig starts on a byte of the
// arena (base offset a multiple of 4).  The seeding tables that follow the
// contigs (k-mers, offsets, counts, positions) are validated the way the
// reference's loader validates them (decode_parts, index_io.rs:237-354) but
// not kept: seeding is not on this path.
#include <cstdint>
#include <cstring>
#include <string>

#include "esp_host.h"

namespace {

constexpr uint64_t kHeaderFixed = 60;  // magic 8 + five u32 + sha256 32 (index_io.rs:33)
constexpr uint64_t kCounts = 16;       // kmer_count u64 + positions_count u64

struct Cur {
    const uint8_t *d;
    uint64_t n, pos;
    bool take(uint64_t k, const uint8_t **p) {
        if (n - pos < k) return false;
        *p = d + pos;
        pos += k;
        return true;
    }
    bool u32(uint32_t *v) {
        const uint8_t *p;
        if (!take(4, &p)) return false;
        *v = (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
        return true;
    }
    bool u64(uint64_t *v) {
        uint32_t lo, hi;
        if (!u32(&lo) || !u32(&hi)) return false;
        *v = (uint64_t)hi << 32 | lo;
        return true;
    }
};

uint64_t rd64(const uint8_t *p) {
    uint64_t v = 0;
    for (int k = 7; k >= 0; k--) v = v << 8 | p[k];
    return v;
}
uint32_t rd32(const uint8_t *p) {
    return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

struct Sink {  // optional outputs of the walk (null: validate and size only)
    uint8_t *arena = nullptr;
    uint64_t arena_bytes = 0;
    esp_contig *contigs = nullptr;
    esp_n_interval *n_iv = nullptr;
    uint64_t n_iv_cap = 0;
    char *names = nullptr;
    uint64_t names_cap = 0;
};

int bad(std::string *msg, const char *m) {
    if (msg) *msg = m;
    return ESP_EFORMAT;
}

// One strict pass over the file (decode_parts order); fills `info` and,
// when given, the sink.
int walk(const uint8_t *data, uint64_t len, esp_paidx_info *info, const Sink *S,
         std::string *msg) {
    Cur c{data, len, 0};
    const uint8_t *p;
    if (!c.take(8, &p) || memcmp(p, "PAIDXfmt", 8) != 0) return bad(msg, "bad magic");
    uint32_t version;
    if (!c.u32(&version)) return bad(msg, "unexpected end of file");
    if (version != 1) {
        if (msg) *msg = "unsupported index version (supported: 1)";
        return ESP_EVERSION;
    }
    esp_paidx_info I{};
    uint32_t contig_count;
    if (!c.u32(&I.k) || !c.u32(&I.w) || !c.u32(&I.freq_cutoff) || !c.u32(&contig_count) ||
        !c.u64(&I.kmer_count) || !c.u64(&I.positions_count) || !c.take(32, &p))
        return bad(msg, "unexpected end of file");
    memcpy(I.fasta_sha256, p, 32);
    I.contig_count = contig_count;
    uint64_t contig_bytes = 0, arena = 0, niv = 0, names = 0;
    for (uint32_t k = 0; k < contig_count; k++) {
        uint32_t name_len, seq_len, packed_len, n_count;
        const uint8_t *name, *packed;
        if (!c.u32(&name_len) || !c.take(name_len, &name) || !c.u32(&seq_len) ||
            !c.u32(&packed_len))
            return bad(msg, "unexpected end of file");
        if (packed_len != (uint32_t)(((uint64_t)seq_len + 3) / 4))
            return bad(msg, "packed_len != ceil(seq_len/4)");
        if (!c.take(packed_len, &packed)) return bad(msg, "unexpected end of file");
        if (seq_len % 4 != 0 && packed_len) {  // trailing bits of the final byte are zero
            uint32_t used = 2 * (seq_len % 4);
            if (packed[packed_len - 1] & (0xFFu >> used))
                return bad(msg, "non-zero tail bits in packed contig");
        }
        if (!c.u32(&n_count)) return bad(msg, "unexpected end of file");
        const uint8_t *ivs;
        if ((uint64_t)n_count * 8 > c.n - c.pos || !c.take((uint64_t)n_count * 8, &ivs))
            return bad(msg, "unexpected end of file");
        if (S && S->contigs) {
            if (arena + packed_len > S->arena_bytes || niv + n_count > S->n_iv_cap ||
                (S->names && names + name_len + 1 > S->names_cap))
                return bad(msg, "output buffers smaller than the index needs");
            memcpy(S->arena + arena, packed, packed_len);
            esp_contig &C = S->contigs[k];
            C.base = arena * 4;
            C.len = seq_len;
            C.n_first = (uint32_t)niv;
            C.n_count = n_count;
            C.pad = 0;
            for (uint32_t q = 0; q < n_count; q++) {
                S->n_iv[niv + q].start = rd32(ivs + 8 * q);
                S->n_iv[niv + q].end = rd32(ivs + 8 * q + 4);
            }
            if (S->names) {
                memcpy(S->names + names, name, name_len);
                S->names[names + name_len] = '\0';
            }
        }
        arena += packed_len;
        niv += n_count;
        names += (uint64_t)name_len + 1;
        contig_bytes += 4 + (uint64_t)name_len + 4 + 4 + packed_len + 4 + (uint64_t)n_count * 8;
    }
    const uint64_t pad1 = (8 - (kHeaderFixed + kCounts + contig_bytes) % 8) % 8;
    if (!c.take(pad1, &p)) return bad(msg, "unexpected end of file");
    for (uint64_t k = 0; k < pad1; k++)
        if (p[k]) return bad(msg, "pad1 not zero");
    // kmers u64 | offsets u64 | counts u32, then pad2, then positions u64
    if (I.kmer_count > (UINT64_MAX / 20) || I.positions_count > (UINT64_MAX / 8))
        return bad(msg, "table size overflow");
    const uint8_t *kmers, *offsets, *counts, *positions;
    if (!c.take(I.kmer_count * 8, &kmers) || !c.take(I.kmer_count * 8, &offsets) ||
        !c.take(I.kmer_count * 4, &counts))
        return bad(msg, "unexpected end of file");
    const uint64_t pad2 =
        (8 - (kHeaderFixed + kCounts + contig_bytes + pad1 + I.kmer_count * 20) % 8) % 8;
    if (!c.take(pad2, &p)) return bad(msg, "unexpected end of file");
    for (uint64_t k = 0; k < pad2; k++)
        if (p[k]) return bad(msg, "pad2 not zero");
    if (!c.take(I.positions_count * 8, &positions)) return bad(msg, "unexpected end of file");
    if (c.pos != c.n) return bad(msg, "trailing bytes after positions table");
    for (uint64_t k = 1; k < I.kmer_count; k++)
        if (rd64(kmers + 8 * (k - 1)) >= rd64(kmers + 8 * k))
            return bad(msg, "kmers not strictly ascending");
    for (uint64_t k = 0; k < I.kmer_count; k++) {
        uint64_t o = rd64(offsets + 8 * k), n = rd32(counts + 4 * k);
        if (o > UINT64_MAX - n || o + n > I.positions_count)
            return bad(msg, "offset+count exceeds positions table");
    }
    I.arena_bytes = arena;
    I.n_iv_count = niv;
    I.names_bytes = names;
    if (info) *info = I;
    return ESP_OK;
}

}  // namespace

extern "C" {

int esp_paidx_scan(const uint8_t *data, uint64_t len, esp_paidx_info *info, char *msg,
                   size_t msg_cap) {
    if (!data || !info) return ESP_EINVAL;
    std::string m;
    int rc = walk(data, len, info, nullptr, &m);
    if (msg && msg_cap) {
        size_t k = std::min(m.size(), msg_cap - 1);
        memcpy(msg, m.data(), k);
        msg[k] = '\0';
    }
    return rc;
}

int esp_paidx_contigs(const uint8_t *data, uint64_t len, uint8_t *arena, uint64_t arena_bytes,
                      esp_contig *contigs, uint32_t n_contigs, esp_n_interval *n_iv,
                      uint64_t n_iv_count, char *names, uint64_t names_bytes) {
    if (!data || !arena || (n_contigs && !contigs)) return ESP_EINVAL;
    esp_paidx_info I;
    std::string m;
    int rc = walk(data, len, &I, nullptr, &m);
    if (rc != ESP_OK) return rc;
    if (n_contigs != I.contig_count || arena_bytes < I.arena_bytes || n_iv_count < I.n_iv_count ||
        (names && names_bytes < I.names_bytes) || (I.n_iv_count && !n_iv))
        return ESP_EINVAL;
    Sink S;
    S.arena = arena;
    S.arena_bytes = arena_bytes;
    S.contigs = contigs;
    S.n_iv = n_iv;
    S.n_iv_cap = n_iv_count;
    S.names = names;
    S.names_cap = names_bytes;
    return walk(data, len, &I, &S, &m);
}

int esp_genome_from_paidx(esp_handle *h, const uint8_t *data, uint64_t len, esp_genome **out) {
    if (!h || !data || !out) return fail(h, ESP_EINVAL, "null argument");
    esp_paidx_info I;
    std::string m;
    int rc = walk(data, len, &I, nullptr, &m);
    if (rc != ESP_OK) return fail(h, rc, "paidx: " + m);
    std::vector<uint8_t> arena(std::max<uint64_t>(1, I.arena_bytes));
    std::vector<esp_contig> contigs(I.contig_count);
    std::vector<esp_n_interval> iv(std::max<uint64_t>(1, I.n_iv_count));
    Sink S;
    S.arena = arena.data();
    S.arena_bytes = arena.size();
    S.contigs = contigs.data();
    S.n_iv = iv.data();
    S.n_iv_cap = iv.size();
    if ((rc = walk(data, len, &I, &S, &m)) != ESP_OK) return fail(h, rc, "paidx: " + m);
    return esp_genome_create(h, arena.data(), I.arena_bytes, contigs.data(), I.contig_count,
                             iv.data(), I.n_iv_count, out);
}

}  // extern "C"
