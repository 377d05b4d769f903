/*
 * hdc_synth.h -- seeded synthetic 16S-like workloads (host C++ in its own
 * library, libhdc_synth.so, kept apart from the GPU library libhdc_gb300.so).
 * They stand in for the reference's real-data front ends, which need data
 * absent here: the SILVA / Greengenes inductors
 * (db_inductors/induct_silva.py:95-181 writes taxonomy_index.tsv and one FASTA
 * per leaf) and the ART-based read simulator (tests/Make_Mixed_Sample.py:
 * 96-97,137-143,185-197,210).  Every item is derived from its own
 * std::mt19937_64 stream (seed mixed with the item's index by splitmix64), so
 * results do not depend on the thread count and match on every host.
 *
 * Output sequences are concatenated ASCII (A,C,G,T) in a caller buffer
 * described by int64 offsets and int32 lengths.
 */
#ifndef HDC_SYNTH_H
#define HDC_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A 6-rank taxonomy tree: root = uniform ACGT of root_len bases; rank r
 * (1..6) derives each child from its parent with uniform substitutions at
 * subst[r-1] (a substituted base becomes one of the other three, uniformly)
 * and a length jitter uniform in [-jitter, jitter] applied as random-position
 * insertions or deletions; leaves are clamped to [min_len, max_len].  Every
 * internal node has b = ceil(n_leaves^(1/6)) children, the last rank holding
 * exactly n_leaves leaves; node j of rank r has parent j / b.
 * Leaves are written to buf (capacity buf_cap bytes; max_len * n_leaves
 * always suffices), offsets off[n_leaves], lengths len[n_leaves].
 * nodes_per_rank[7] (optional) receives the node counts of ranks 0..6.
 * Returns 0, or -1 on a bad argument or a too small buffer. */
int hdc_synth_tree(uint64_t seed, int64_t n_leaves, int root_len, const double* subst, int jitter,
                   int min_len, int max_len, char* buf, int64_t buf_cap, int64_t* off, int32_t* len,
                   int64_t* nodes_per_rank, int threads);

/* Noisy copies of sequences: copy c of sequence i (i < n_src, c < n_copies)
 * gets uniform substitutions at rate subst; written in order (i major) as
 * n_src * n_copies segments.  Returns 0 or -1. */
int hdc_synth_copies(uint64_t seed, const char* src, const int64_t* src_off, const int32_t* src_len,
                     int64_t n_src, int n_copies, double subst, char* buf, int64_t buf_cap, int64_t* off,
                     int32_t* len, int threads);

/* Reads sampled from sources: read i picks a source uniformly (label[i]),
 * a length (read_len if sigma <= 0, else log-normal with median read_len and
 * shape sigma, clipped to [min_read, max_read] and to the source length),
 * a uniform start, then errors: with probability mixed_frac the read gets
 * errors at rate mixed_rate split substitution:insertion:deletion = 3:1:1,
 * otherwise uniform substitutions at rate subst.  Returns 0 or -1. */
int hdc_synth_reads(uint64_t seed, const char* src, const int64_t* src_off, const int32_t* src_len,
                    int64_t n_src, int64_t n_reads, int read_len, double sigma, int min_read, int max_read,
                    double subst, double mixed_frac, double mixed_rate, char* buf, int64_t buf_cap,
                    int64_t* off, int32_t* len, int32_t* label, int threads);

#ifdef __cplusplus
}
#endif
#endif /* HDC_SYNTH_H */
