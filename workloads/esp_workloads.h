/*
 * esp_workloads.h -- benchmark and test tooling beside the GB300 alignment
 * library: seeded synthetic workloads (synth.cpp, host only) and measured
 * integer issue peaks of the GPU (probe.cu).  Neither is part of the
 * alignment path: they build into their own libraries
 * (workloads/_build/libesp_synth.so, libesp_probe.so), and the CPU
 * oracle's library carries a second build of the generators so that the
 * benchmark's reference arm makes its inputs without loading any library
 * of the GPU path.  The reference ships no datasets (all of its own test
 * inputs are generated, crates/map/src/extend.rs:2481-2525).
 */
#ifndef ESP_WORKLOADS_H
#define ESP_WORKLOADS_H

#include "esperanto_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded synthetic workloads ---- */

/* Arena bytes (16 bytes of padding included) of a Gotoh workload:
 * shape 0 = 150-bp reads vs 214-bp windows, band half 32 at offset 32;
 * shape 2 = read length U[50,300], half in {16,32,64,128} w.p.
 * {.4,.3,.2,.1}, window read + 2*half, offset half.  Error model: 1%
 * substitutions, 0.1% indels of length 1-3, A->G at 5% of A (T->C on
 * reverse-strand pairs). */
int esp_synth_gotoh_size(uint64_t seed, uint64_t n_pairs, int shape, uint64_t *arena_bytes);
/* Fill the workload into caller memory (host). */
int esp_synth_gotoh(uint64_t seed, uint64_t n_pairs, int shape, uint8_t *arena,
                    uint64_t arena_bytes, esp_pair *pairs);

/* Myers workload: 150-bp queries sampled from 200-bp uniform texts with
 * U{0..8} edits, 10% unrelated random queries. */
int esp_synth_myers_size(uint64_t seed, uint64_t n_pairs, uint64_t *arena_bytes);
int esp_synth_myers(uint64_t seed, uint64_t n_pairs, uint8_t *arena, uint64_t arena_bytes,
                    esp_myers_pair *pairs);

/* Splice workload: per read a contig exon1(300) + intron
 * (log-uniform 60..50,000, GT..AG planted) + exon2(300); the read is 150 bp
 * across the junction split at U[20,130] with the Gotoh error model;
 * candidates = the true junction plus decoys at every other GT within +-20
 * of the donor and every other AG within +-20 of the acceptor (library
 * order).  Sizes first, then fill caller memory. */
int esp_synth_splice_size(uint64_t seed, uint64_t n_reads, uint64_t *genome_bytes,
                          uint64_t *read_bytes, uint64_t *n_cands);
int esp_synth_splice(uint64_t seed, uint64_t n_reads, uint8_t *genome_arena,
                     uint64_t genome_bytes, esp_contig *contigs, uint8_t *read_arena,
                     uint64_t read_bytes, esp_splice_read *reads, esp_splice_cand *cands,
                     uint64_t n_cands);

/* Serve workload: a uniform-ACGT genome of `total_bases` in
 * `n_contigs` equal contigs (contig c starts at base c * stride, stride a
 * multiple of 4), and request reads: 2x150 paired-end fragments (insert
 * 250-450) at uniform coordinates with the Gotoh error model; each read's
 * window is read +- 32 with hint offset 32. */
int esp_synth_genome(uint64_t seed, uint64_t total_bases, uint32_t n_contigs, uint8_t *arena,
                     uint64_t arena_bytes, esp_contig *contigs);
int esp_synth_serve_reads(uint64_t seed, uint64_t request, const uint8_t *genome_arena,
                          const esp_contig *contigs, uint32_t n_contigs, uint64_t n_reads,
                          uint8_t *read_arena, uint64_t read_arena_bytes, esp_serve_read *reads);

/* ---- measured integer issue peaks of a GPU ----
 * Lane-operations per second of dependency-free streams of 3-input logic,
 * integer max, integer add and integer multiply-add on CUDA device
 * `device`: the denominators of the DP kernels' integer roofline.  Runs a
 * few milliseconds of probes.  ESP_OK, or ESP_ECUDA. */
int esp_probe_int_peaks(int device, double *lop3, double *imnmx, double *iadd, double *imad);
/* The same for the 16x2 SIMD add-then-max and three-way max the two-pairs-
 * per-thread DP kernel is built on (per 32-bit lane; each updates two 16-bit
 * values). */
int esp_probe_simd16_peaks(int device, double *addmax, double *max3);

#ifdef __cplusplus
}
#endif
#endif
