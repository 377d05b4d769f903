/*
 * hdc_gb300.h -- C ABI of the GB300 (sm_103a) k-mer hypervector classifier
 * hot path: (a) k-mer hypervector encoding, (b) query x reference cosine
 * top-k search, (c) propagate-children bundling and greedy selection.
 *
 * Conventions
 *   - Every function returns an int status (HDC_OK = 0); no exception crosses
 *     this boundary.  hdc_last_error() gives a message for the calling thread.
 *   - Pointers named d_* are device pointers owned by the caller; outputs are
 *     caller-allocated.  Work is enqueued on the given CUDA stream (a
 *     cudaStream_t passed as void*; NULL is the legacy default stream) and is
 *     asynchronous unless stated otherwise.
 *   - Sizes are runtime parameters (the reference fixes them at compile time
 *     in src/config.h:5-8): dim = HV_DIM, kmer = KMER_SIZE (1..16),
 *     window = SEQUENCE_LENGTH, step = SIM_STEP.
 *   - Sequences are raw ASCII bytes.  Exactly the bytes 'A','C','G','T' are
 *     bases; a k-mer holding any other byte (N, lowercase, IUPAC codes) is
 *     skipped, as the reference CPU encoder does (src/encoder.cpp:115-117).
 *
 * Score modes (the ranking key is the float score, ties -> lower ref index)
 *   HDC_SCORE_NORM  float(2*(cos - 0.5)), -1 for a zero norm: the reference
 *                   cosine() built with NORM_COSINE (src/HV.cpp:219-242)
 *   HDC_SCORE_COS   float(cos), -1 for a zero norm: the scale the reference
 *                   GPU search reports (src/cosine.cu:270-271), but computed
 *                   from the exact integer dot and norms in FP64
 *   HDC_SCORE_DOT   float(dot): cosine() built without NORM_COSINE
 *                   (src/HV.cpp:244-252)
 */
#ifndef HDC_GB300_H
#define HDC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HDC_OK 0
#define HDC_ERR_INVALID 1     /* bad argument or unsupported size */
#define HDC_ERR_RANGE 2       /* values outside the exactly-representable range */
#define HDC_ERR_CUDA 3        /* CUDA runtime error */
#define HDC_ERR_NOMEM 4       /* device allocation failed */
#define HDC_ERR_UNSUPPORTED 5 /* device is not sm_103 or lacks a feature */
#define HDC_ERR_TIMEOUT 6     /* a bounded device-side wait gave up */

#define HDC_SCORE_NORM 0
#define HDC_SCORE_COS 1
#define HDC_SCORE_DOT 2

/* Output element kinds of the encoder. */
#define HDC_OUT_I16 0          /* int16 bundle, wraps modulo 2^16 like the reference */
#define HDC_OUT_I32 1          /* int32 bundle, exact (segments of <= 65535 k-mers) */
#define HDC_OUT_BIPOLAR_BF16 2 /* bf16 +1/-1 sign of the bundle, 0 -> +1 */
#define HDC_OUT_BIPOLAR_I16 3  /* int16 +1/-1 sign of the bundle, 0 -> +1 */
#define HDC_OUT_BIPOLAR_F16 4  /* fp16 +1/-1 sign of the bundle, 0 -> +1 (tensor-core queries) */
#define HDC_OUT_BIPOLAR_I8 5   /* int8 +1/-1 sign of the bundle, 0 -> +1 (hierarchical descent reads) */
#define HDC_OUT_F16 6          /* fp16 bundle, exact (segments of <= 2048 k-mers): count-valued
                                  tensor-core queries */
#define HDC_OUT_SIGN_BITS 7    /* the +1/-1 signs as bits (0 -> +1): bit b of uint32 word w of a
                                  row is set when element 32 w + b is >= 0, bits past dim are 0;
                                  out_stride in words (>= ceil(dim / 32)); the reads of
                                  hdc_beam_search_split_bits, which reads rows of exactly
                                  dim / 32 words: encode them with out_stride == dim / 32 */

typedef struct hdc_context hdc_context;
typedef struct hdc_refdb hdc_refdb;
typedef struct hdc_pipeline hdc_pipeline;

const char* hdc_last_error(void);
const char* hdc_status_string(int status);

/* Create a context on the current device: base hypervectors (src/HV.cpp:20-41,
 * mt19937_64 seeds A=0 C=1 T=2 G=3) are generated and uploaded. */
int hdc_context_create(int dim, int kmer, int window, int step, hdc_context** out);
void hdc_context_destroy(hdc_context* ctx);
/* The four base hypervectors in A,C,G,T order, [4][ceil(dim/64)] uint64 words (host). */
int hdc_context_base_hvs(const hdc_context* ctx, uint64_t* host_out);

/* Device memory and copies for callers without a CUDA runtime of their own
 * (FFI bindings, the GPU.cuh drop-in).  hdc_copy copies host->device when
 * to_device != 0, else device->host, asynchronously on `stream`. */
int hdc_device_alloc(size_t bytes, void** out);
int hdc_device_free(void* p);
int hdc_copy(void* dst, const void* src, size_t bytes, int to_device, void* stream);
int hdc_stream_sync(void* stream);

/* ---------------------------------------------------------------- (a) encode */

/* K-mer binder hypervectors, the values of HVCache::kmers (src/encoder.cpp:
 * 47-74), computed on the host from the context's base hypervectors: for each
 * of n k-mer codes (2 bits a base, A=0 C=1 G=2 T=3, the first base in the most
 * significant digit, below 4^kmer) the binder ~0 ^ XOR_d rot_d(base[digit d])
 * over the ring of 64 W bits with the tail masked, W = ceil(dim / 64) uint64
 * words each, into host_out [n][W].  The code is used as given: pass the
 * canonical k-mer (the smaller of the k-mer and its reverse complement). */
int hdc_binders(const hdc_context* ctx, const int64_t* codes, int64_t n, uint64_t* host_out);

/* 2-bit packing of reads on the device, the format of the reference's
 * pack_sequence (src/encode.cu:169-185): base i of the byte stream d_bytes
 * [n_bytes] goes to bits 2 (i % 16) of d_words[i / 16] (ceil(n_bytes / 16)
 * words), A/a = 0, C/c = 1, G/g = 2, T/t = 3, any other byte 0 (as A).  One
 * 128-bit load per word (a 16-byte aligned d_bytes).  Offsets into the bytes
 * stay valid as base offsets into the words: a sequence at byte offset o is
 * at base offset o of the packed stream. */
int hdc_pack_2bit(hdc_context* ctx, const char* d_bytes, int64_t n_bytes, uint32_t* d_words, void* stream);

/* hdc_encode_segments over 2-bit packed reads (hdc_pack_2bit's format, or the
 * reference's packed sequences placed at base offsets that are multiples of
 * 16): segment i is bases d_base_off[i] .. + d_len[i] - 1 of the packed
 * stream.  Every position of a packed segment is a base, so no k-mer is
 * skipped: on sequences of A, C, G, T the result equals hdc_encode_segments on
 * the ASCII bytes; bytes the packing turned into A (N, IUPAC codes) count as
 * A, as in the reference's GPU encoder (src/encode.cu:21-38), not skipped as
 * in HVCache::compute.  Same outputs, limits and errors as
 * hdc_encode_segments. */
int hdc_encode_packed(hdc_context* ctx, const uint32_t* d_words, const int64_t* d_base_off, const int32_t* d_len,
                      int64_t n_segs, int32_t max_len, int out_kind, void* d_out, int64_t out_stride,
                      int32_t* d_nkmers, void* stream);

/* Encode n_segs byte segments d_bytes[d_seg_off[i] .. d_seg_off[i]+d_seg_len[i])
 * with the whole-segment semantics of HVCache::compute (src/encoder.cpp:106-132):
 * sum over every k-mer position of the +1/-1 binder of the canonical k-mer.
 * Row i of d_out (row stride out_stride elements, >= dim) receives segment i.
 * max_len is an upper bound on the segment lengths (0: unknown), used to size
 * the device counters.  d_nkmers (optional, int32[n_segs]) receives the
 * number of k-mers bundled.  Replaces the per-window kernel hdc_encode /
 * launch_hdc_encode (src/encode.cu:69-165). */
int hdc_encode_segments(hdc_context* ctx, const char* d_bytes, const int64_t* d_seg_off,
                        const int32_t* d_seg_len, int64_t n_segs, int32_t max_len, int out_kind,
                        void* d_out, int64_t out_stride, int32_t* d_nkmers, void* stream);

/* Number of windows of a sequence of length len: (len - window)/step + 1, or 0
 * when len < window (src/encode.cu:258 without its negative-length case). */
int64_t hdc_num_windows(const hdc_context* ctx, int64_t len);

/* Window form of the encoder, the drop-in for launch_hdc_encode
 * (src/encode.cu:136-165): sequence s is d_bytes[d_seq_off[s] .. d_seq_off[s+1]),
 * its windows start at w*step and span `window` bytes, and window w of
 * sequence s is written to row d_win_off[s] + w of d_out (int16, row stride
 * dim).  d_win_off[s+1] - d_win_off[s] must equal hdc_num_windows(len s).
 * Each window gets HVCache::compute of its substring (the sequence offsets
 * are byte offsets, so every sequence of a batch is read from its own bases). */
int hdc_encode_windows(hdc_context* ctx, const char* d_bytes, const int64_t* d_seq_off,
                       const int64_t* d_win_off, int64_t n_seqs, int64_t n_windows, int16_t* d_out,
                       void* stream);

/* ---------------------------------------------------------------- (b) search */

/* Squared L2 norms (int64) and optional max |v| (int32 atomic max into
 * *d_maxabs, which the caller zeroes) of n rows of int8 (elem_bytes 1),
 * int16 (elem_bytes 2) or int32 (elem_bytes 4) hypervectors, row stride dim. */
int hdc_norms(hdc_context* ctx, const void* d_hv, int elem_bytes, int64_t n, int64_t* d_norm2,
              int32_t* d_maxabs, void* stream);
/* The same for integer-valued fp16 rows (HDC_OUT_F16 / HDC_OUT_BIPOLAR_F16 queries). */
int hdc_norms_f16(hdc_context* ctx, const void* d_hv, int64_t n, int64_t* d_norm2, int32_t* d_maxabs, void* stream);

/* Workspace the plain search needs for nq queries and top-k. */
size_t hdc_search_workspace_bytes(const hdc_context* ctx, int64_t nq, int64_t nr, int k);

/* Plain form: exact integer cosine top-k of int16 queries against int16
 * references on CUDA cores, the drop-in for launch_cosine_topk
 * (src/cosine.cu:441-496) and, with k = 1, launch_cosine_argmax
 * (src/cosine.cu:172-222).  For every query: the k best references by the
 * float score of score_mode (descending), ties to the lower reference index.
 * k is clamped to nr (src/cosine.cu:451).  Outputs are [nq][k]: d_score
 * (float), d_idx (int32), d_cos (double, FP64 cosine from the exact dot;
 * optional), d_dot (int64 exact dot; optional).  max_abs_q / max_abs_r bound
 * |element| of queries / references (from hdc_norms); products must satisfy
 * max_abs_q * max_abs_r <= 2^20 (else HDC_ERR_RANGE).  d_qnorm2 / d_rnorm2 come from hdc_norms.
 * d_work must hold hdc_search_workspace_bytes(nq, nr, k) bytes. */
int hdc_search_plain(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                     int32_t max_abs_q, const int16_t* d_r, const int64_t* d_rnorm2, int64_t nr,
                     int32_t max_abs_r, int k, int score_mode, float* d_score, int32_t* d_idx,
                     double* d_cos, int64_t* d_dot, void* d_work, size_t work_bytes, void* stream);

/* Read and clear the device status word of the context (synchronizes the
 * device): 0, 100 + the code of a bounded device-side wait that gave up in
 * a tensor-core search or descent (which then returned partial results), or
 * 200 when hdc_beam_search_split was given a max_children below the tree's. */
int hdc_context_status(hdc_context* ctx, int* status);

/* Precision form, reference side: build a tensor-core database from int16
 * (elem_bytes 2) or int32 (4) reference hypervectors [nr][dim] with
 * max |v| <= max_abs.  Each value is split into balanced base-2048 fp16
 * limbs (1 limb for |v| <= 2048, 2 for |v| <= 2048*2048+1023, ...), and the
 * exact squared norms are kept.  Synchronizes the stream.  dim must be a
 * multiple of 8.  No reference counterpart (the reference re-uploads and
 * re-normalises the database on every cosine_search call, src/cosine.cu:
 * 512-533). */
int hdc_refdb_create(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                     hdc_refdb** out, void* stream);
/* The same for queries of magnitude up to max_query_abs (1..2048; count-valued
 * queries, e.g. HDC_OUT_F16 reads): the limbs become balanced base-2^b digits
 * with every limb within T = min(2048, 2^24 / (dim * max_query_abs)) (b the
 * largest with 2^(b-1) <= T, at most 11), so that every fp32 partial sum of a
 * search with such queries is an exact integer.  max_query_abs = 1 (+1/-1
 * queries) gives the base-2048 limbs of hdc_refdb_create up to dim 16384. */
int hdc_refdb_create_ex(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                        int32_t max_query_abs, hdc_refdb** out, void* stream);
void hdc_refdb_destroy(hdc_refdb* db);
int hdc_refdb_limbs(const hdc_refdb* db);
int hdc_refdb_limb_bits(const hdc_refdb* db);

/* Persisted database (no reference counterpart: the reference re-encodes its
 * FASTA files on every run).  hdc_refdb_save writes the limbs, exact norms
 * and reciprocal roots of `db`, the context's dim / k-mer / window / step,
 * and optionally one taxonomy id per reference (h_tax_ids: nr host int32s,
 * or NULL), with a checksum; hdc_refdb_file_info reads the header;
 * hdc_refdb_load rebuilds the database on the current device (the file's dim
 * and k-mer size must equal the context's; a checksum mismatch, truncation or
 * foreign file is HDC_ERR_INVALID) and fills h_tax_ids (nr entries) when the
 * file has ids and the pointer is not NULL.  Synchronous. */
int hdc_refdb_save(hdc_context* ctx, const hdc_refdb* db, const char* path, const int32_t* h_tax_ids);
int hdc_refdb_file_info(const char* path, int* dim, int* kmer, int64_t* nr, int* limbs, int* has_tax_ids);
int hdc_refdb_load(hdc_context* ctx, const char* path, hdc_refdb** out, int32_t* h_tax_ids);
size_t hdc_search_tc_workspace_bytes(const hdc_context* ctx, const hdc_refdb* db, int64_t nq, int k);

/* Precision form: exact cosine top-k of fp16 integer queries (normally the
 * +1/-1 read hypervectors of HDC_OUT_BIPOLAR_F16, max_abs_q = 1) against a
 * tensor-core database, on tcgen05 tensor cores with fp32 accumulators per
 * limb (exact while dim * max|q| * max|limb| <= 2^24, else HDC_ERR_RANGE).
 * Same ranking rule, outputs and score modes as hdc_search_plain, whose
 * results it reproduces exactly; the replacement for launch_cosine_topk
 * (src/cosine.cu:441-496) at scale. */
int hdc_search_tc(hdc_context* ctx, const hdc_refdb* db, const void* d_q, const int64_t* d_qnorm2,
                  int64_t nq, int32_t max_abs_q, int k, int score_mode, float* d_score, int32_t* d_idx,
                  double* d_cos, int64_t* d_dot, void* d_work, size_t work_bytes, void* stream);

/* Size of the fixed device scratch used by hdc_search_plain_noalloc (16 MiB). */
#define HDC_NOALLOC_SCRATCH_BYTES (16u << 20)

/* hdc_search_plain without any device allocation, by this library or by the
 * caller: the same search, arguments, results and errors, except that the
 * workspace is a fixed HDC_NOALLOC_SCRATCH_BYTES array that the library
 * places in device memory once, when the GPU loads it.  It has no
 * counterpart in the reference (whose launch_cosine_topk allocates and frees
 * its buffers on every call, src/cosine.cu:455-494).
 *
 * For callers that cannot allocate device memory: a host application or
 * framework that owns the device memory through its own pool and does not
 * let plug-in code call cudaMalloc; code whose memory budget is already
 * reserved in full; loops that cannot afford the device-wide
 * synchronisation cudaMalloc / cudaFree imply.
 *
 * Limits and behaviour:
 *   - a batch whose workspace (hdc_search_workspace_bytes) exceeds
 *     HDC_NOALLOC_SCRATCH_BYTES is rejected with HDC_ERR_RANGE and a message
 *     naming both sizes; pass fewer queries per call;
 *   - k is checked first (1..32 after clamping to nr, else HDC_ERR_INVALID,
 *     as hdc_search_plain), then the scratch size;
 *   - the context's device must be the current device; the first call with
 *     a context looks up the scratch's device address on its device (once
 *     per context), so make that first call before any stream capture;
 *     after cudaDeviceReset create new contexts, which look it up again;
 *   - every call on a device uses the same scratch, which keeps the previous
 *     call's contents (the search overwrites every entry it reads, so
 *     nothing needs clearing); calls that overlap on the GPU (other streams,
 *     other threads) race on it: serialise them;
 *   - the scratch stays allocated on every GPU that has loaded the library
 *     until the process exits. */
int hdc_search_plain_noalloc(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                             int32_t max_abs_q, const int16_t* d_r, const int64_t* d_rnorm2, int64_t nr,
                             int32_t max_abs_r, int k, int score_mode, float* d_score, int32_t* d_idx,
                             double* d_cos, int64_t* d_dot, void* stream);

/* Schedule of hdc_search_tc on this context (no reference counterpart; the
 * knobs an autotuner varies): group_tiles = query tiles of 128 that run
 * together (0: automatic), the persistent grid being group_tiles x
 * (SMs / group_tiles) CTAs, each group's reference tiles dealt round-robin
 * to the SMs / group_tiles lanes; l2_policy = 0 no L2 hint, 1 query tiles
 * loaded evict-last, 2 also reference tiles evict-first (-1: automatic);
 * tile_n = references per tile, 128 or 256 (0: automatic); m_blocks = query
 * M-blocks of 128 rows per CTA sharing each reference tile, 1 or 2 (0:
 * automatic; 2 needs tile_n 128 and at most 2 limbs).  Results do not depend
 * on these settings, only the speed does. */
int hdc_search_tc_tuning(hdc_context* ctx, int group_tiles, int l2_policy, int tile_n, int m_blocks);

/* Shape of the last hdc_search_tc on this context (diagnostic): shape[0] =
 * CTAs per cluster, [1] = query tiles per group, [2] = reference lanes (of
 * the leading part, when the batch ran in two), [3] = 1 when each CTA pair
 * ran as one M = 256 MMA, [4] = kernels launched (a search and a merge per
 * part).  All 0 before the first search. */
int hdc_search_tc_last_shape(const hdc_context* ctx, int32_t shape[5]);

/* Further settings of a context; results do not depend on them.
 *   HDC_TC_PREFETCH: K blocks of each query/reference tile pair prefetched
 *     into L2 ahead of the shared-memory ring (0: none, -1: automatic, <= 64);
 *   HDC_TC_CLUSTER: CTAs that share an operand's blocks through a TMA
 *     multicast, 1, 2 or 4 (2 applies with tile_n 128 and one M-block; 4,
 *     two limbs with pair MMAs: two pairs on two reference lanes share their
 *     query blocks; where not every cluster of 4 can be resident, the leading
 *     whole groups that fit run as clusters of 4 and the other queries as
 *     pairs; 0 automatic: 4 up to k = 16, else 2);
 *   HDC_TC_SHARE: what a pair shares: 0 reference blocks (the pair runs two
 *     neighbouring query tiles), 1 query blocks (the pair runs one query tile
 *     on two neighbouring reference lanes; groups default to half the SMs),
 *     -1 automatic. */
#define HDC_TC_PREFETCH 1
#define HDC_TC_CLUSTER 2
#define HDC_TC_SHARE 3
#define HDC_TC_SCATTER 5   /* tensor-core search: 1 visits reference tiles in a scattered fixed
                              order (fewer top-k insertions on tree-ordered databases), 0 in
                              index order, -1 automatic */
#define HDC_TC_KBLOCK 6    /* tensor-core search: dims per K block of the paired default path,
                              32 (half the bytes per stage, a deeper ring) or 64; 0 automatic */
#define HDC_TC_PAIR_MMA 7  /* tensor-core search, two limbs: each CTA pair as one M = 256 MMA
                              (cta_group::2), 1 on, 0 off, -1 automatic */
#define HDC_TC_LANES 8     /* tensor-core search: at most this many reference lanes per query tile
                              (CTAs that split the references of one query tile); 0 automatic */
#define HDC_BEAM_GROUPED 4 /* hdc_beam_search: 1 reads grouped by candidate node, 2 the same
                              with every level but the last scored on the tensor cores
                              (entries grouped by parent), 0 one warp per read, -1
                              automatic (2 when dim % 1024 == 0 and dim <= 16384, else 0) */
#define HDC_BEAM_ONE_LAUNCH 11 /* grouped descent (HDC_BEAM_GROUPED 1 or 2): 1 runs every level
                              in one cooperative launch (one CTA per SM, the phases of a level
                              separated by bounded grid-wide barriers); 2 the same up to the
                              last level's node-ordered pairs, which a second cooperative launch
                              scores (more warps per SM than the first holds) and, past a grid
                              barrier, selects from (one warp per read): two launches a call;
                              0 a sequence of kernels per level (about 100 a call), whose
                              tensor-core kernel has more producer warps than the cooperative
                              CTA can hold (3 % faster at D = 16,384); -1 automatic (2 where
                              the cooperative CTAs fit, else 0); results are identical */
#define HDC_WAIT_LIMIT 9   /* tensor-core search and grouped descent: their bounded device-side
                              waits (pipeline mbarriers, grid barriers) give up after value x
                              1,000 SM cycles, 1 .. 4,000,000 (0: the default, 4,000,000,
                              about 2 s at 2 GHz); a wait that gives up makes the call return
                              partial results and hdc_context_status report 100 + its code
                              (120: a grid barrier of the cooperative descent) */
#define HDC_GREEDY_FORM 12 /* hdc_propagate_greedy: 1 scores every pair a decision can need in
                              bulk (tiled kernels), then decides each parent's candidates in order
                              from running maxima; 0 one CTA per parent computing each decision's
                              dots as it goes; -1 automatic (1 when dim % 8 == 0); results are
                              identical */
#define HDC_TEST_WITHHOLD_LOADS 10 /* for tests of the bounded waits only: 1 makes the
                              tensor-core search's producer issue no operand loads, so the MMA
                              issuer's and the epilogue's waits run out (after HDC_WAIT_LIMIT)
                              with nothing in flight; 2 makes the cooperative descent's first
                              CTA reach its first grid barrier four limits late, so the other
                              CTAs' waits run out and every CTA leaves there; 0 off */
int hdc_context_option(hdc_context* ctx, int option, int value);

/* Hierarchical descent (config 5; targets/identify.cpp:89-202 with one
 * prototype hypervector per taxonomy node): beam search of +1/-1 int8 read
 * hypervectors [nq][dim] down a tree whose nodes carry int32 prototypes
 * d_proto [n_nodes][dim] (squared norms d_proto_norm2), children in CSR
 * (d_child_ptr, d_child_idx).  Level 0 scores d_roots; every later level
 * scores the children of the beam entries (a node without children scores
 * itself again), ranks them by score (ties to the lower node index), stops
 * when the best score is below threshold (the reference uses 0 on the NORM
 * scale) and keeps the entries scoring >= threshold, at most `beam` (<= 8).
 * Outputs per read: the best path d_path [nq][levels] (-1 past its depth),
 * its per-level scores, and its depth.  levels <= 8; dim % 4 == 0.
 * Prototype elements must be greater than INT32_MIN.
 * Reads are scored either grouped by candidate node (each prototype row read
 * once per level for the whole batch; needs dim % 1024 == 0, dim <= 16384,
 * and device workspace from the stream-ordered allocator) or one warp per
 * read; see HDC_BEAM_GROUPED.  Both give identical results. */
int hdc_beam_search(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                    const int32_t* d_proto, const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                    const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int levels, int beam,
                    double threshold, int score_mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                    void* stream);

/* The same descent (targets/identify.cpp:89-202, as hdc_beam_search) over
 * prototypes stored in two widths.  Leaf prototypes are whole-sequence k-mer
 * counts (|v| <= sequence length) and the lowest internal ranks sums of a
 * few of them, so most of a taxonomy fits 16 bits and the descent, which
 * streams those rows from HBM, reads half the bytes.  Nodes [0, n_wide)
 * have int32 rows d_proto32 [n_wide][dim]; nodes [n_wide, n_nodes) int16
 * rows d_proto16 [n_nodes - n_wide][dim] (node n is row n - n_wide).  The
 * results are identical to hdc_beam_search on the same values.  Needs the
 * grouped descent: dim % 1024 == 0, dim <= 16384, 16-byte aligned rows and
 * reads, HDC_BEAM_GROUPED != 0 (HDC_ERR_INVALID otherwise, unless every row
 * is int32, n_wide == n_nodes).
 * max_children: the largest child count of any node, known to the caller who
 * built the tree, which sizes the call's workspace without a host
 * synchronisation; 0 has the call read it back from the device (as
 * hdc_beam_search does).  A value below the tree's is caught on the device:
 * every read stops at depth 0 and hdc_context_status reports 200. */
int hdc_beam_search_split(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                          const int32_t* d_proto32, int64_t n_wide, const int16_t* d_proto16,
                          const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                          const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                          int levels, int beam, double threshold, int score_mode, int32_t* d_path,
                          float* d_path_score, int32_t* d_depth, void* stream);
/* Diagnostic of the last one-launch descent on this context (HDC_BEAM_ONE_LAUNCH):
 * the duration in ns of each of its phases as its first CTA saw them (from the
 * launch's start to its first grid barrier, between consecutive barriers, and
 * from the last barrier to the end), at most max_n of them, their number in
 * *n_out (0 before the first such descent).  Synchronises the device. */
int hdc_beam_phase_times(const hdc_context* ctx, int64_t* out_ns, int max_n, int* n_out);

/* The same with the reads as sign bits d_qbits [nq][dim / 32] (HDC_OUT_SIGN_BITS
 * rows, 16-byte aligned): no int8 rows and no packing pass.  Row q starts at
 * word q * (dim / 32): the rows must be dense, so encode them with
 * out_stride == dim / 32 (a wider stride would be misread).  As
 * hdc_beam_search_split for everything else; needs the grouped descent. */
int hdc_beam_search_split_bits(hdc_context* ctx, const uint32_t* d_qbits, const int64_t* d_qnorm2, int64_t nq,
                               const int32_t* d_proto32, int64_t n_wide, const int16_t* d_proto16,
                               const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                               const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                               int levels, int beam, double threshold, int score_mode, int32_t* d_path,
                               float* d_path_score, int32_t* d_depth, void* stream);

/* Windowed similarity, HVCache::similarity (src/encoder.cpp:198-215), for a
 * list of (query, reference sequence) pairs.  A reference's "similarity rows"
 * are the int16 hypervectors of its windows x = 0, step, ... while
 * x + window < len (strict), in order, listed in CSR d_ref_rows [n_refs+1]
 * over d_rows [n_rows][dim] (squared norms d_row_norm2); a reference with
 * len <= window has one row, the whole sequence, flagged in d_ref_whole (may
 * be NULL when there is none) and scored unclamped.  Otherwise the score is
 * the best score over the rows starting from -1, and d_window the first row
 * reaching it (-1 when none beat -1; the reference then reports position 0).
 * Queries d_q [nq][dim] are whole-read int16 hypervectors (HVCache::get).
 * dim % 8 == 0; rows and queries 16-byte aligned. */
int hdc_similarity(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, const int16_t* d_rows,
                   const int64_t* d_row_norm2, const int64_t* d_ref_rows, const uint8_t* d_ref_whole,
                   const int32_t* d_pair_q, const int32_t* d_pair_ref, int64_t n_pairs, int score_mode,
                   float* d_score, int32_t* d_window, void* stream);

/* Hierarchical identification with the reference's own scoring
 * (targets/identify.cpp:89-202): as hdc_beam_search, but a taxonomy node is
 * scored as max(-1, similarity of the read against every sequence of the
 * node), i.e. the best over all similarity rows of the node's sequences,
 * listed in CSR d_node_rows [n_nodes+1] over d_rows [n_rows][dim] (int16,
 * squared norms d_row_norm2; a node without sequences scores -1).  Reads
 * d_q [nq][dim] are whole-read int16 hypervectors.  Outputs as
 * hdc_beam_search, plus d_stop_level [nq] (may be NULL): the level at which
 * the read stopped because its best score fell below the threshold, or -1
 * when it ran all levels.  levels <= 8; beam <= 8; dim % 8 == 0;
 * dim * 2 bytes <= 200 KiB. */
int hdc_identify(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq, const int16_t* d_rows,
                 const int64_t* d_row_norm2, const int64_t* d_node_rows, const int64_t* d_child_ptr,
                 const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int levels, int beam,
                 double threshold, int score_mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                 int32_t* d_stop_level, void* stream);

/* FASTA ingest on the device, with the reading of targets/identify.cpp:46-71:
 * lines end at '\n' only (a '\r' stays part of the line); a line starting with
 * '>' closes the current record (kept only when its sequence is not empty) and
 * names the next (the rest of the line); other lines are appended to the
 * sequence; bytes before the first header form a record with an empty name.
 * In: d_in [n] raw file bytes.  Out: d_out (n bytes) the concatenated
 * sequences; per kept record j < max_records, d_seq_off[j] / d_seq_len[j]
 * into d_out and d_name_off[j] / d_name_len[j] into d_in; *d_count (device
 * int64) = the number of kept records (may exceed max_records: then only the
 * first max_records are written).  Each record's sequence must be shorter than
 * 2^31 bytes.  Uses stream-ordered workspace of about 40 bytes per record and
 * 40 per 8 KB of input, and synchronises the stream once (to size the
 * record arrays). */
int hdc_fasta_parse(hdc_context* ctx, const char* d_in, int64_t n, char* d_out, int64_t* d_seq_off,
                    int32_t* d_seq_len, int64_t* d_name_off, int32_t* d_name_len, int64_t max_records,
                    int64_t* d_count, void* stream);

/* ---------------------------------------------------------------- batching form */

/* A reusable encode -> tensor-core search -> top-k pipeline for batches of up
 * to max_reads reads of up to max_len bases (max_bytes in total) against a
 * resident database, replayed as a CUDA graph: copies to the device, the
 * encoder's length-binned work queue (longest read first), hdc_search_tc,
 * copies back.  Reads are encoded to +1/-1 (ties to +1).  The encode()/
 * cosine_search() pair of the reference (src/GPU.cuh) at stream scale; no
 * single reference counterpart. */
int hdc_pipeline_create(hdc_context* ctx, const hdc_refdb* db, int64_t max_reads, int64_t max_bytes,
                        int32_t max_len, int k, int score_mode, hdc_pipeline** out);
void hdc_pipeline_destroy(hdc_pipeline* p);
/* Host reads bytes[off[i] .. off[i]+len[i]), i < n_reads <= max_reads; host
 * outputs [n_reads][k].  Synchronous. */
int hdc_pipeline_run(hdc_pipeline* p, const char* bytes, const int64_t* off, const int32_t* len, int64_t n_reads,
                     float* scores, int32_t* idx);
/* Replay encode + search on the batch already staged on the device, without
 * copies, asynchronously on hdc_pipeline_stream(p). */
int hdc_pipeline_launch_resident(hdc_pipeline* p);
void* hdc_pipeline_stream(hdc_pipeline* p);
/* Time the tensor-core schedules of hdc_search_tc_tuning on the pipeline's
 * buffers, keep the fastest on the context and re-capture the graphs.
 * Outputs (optional): the chosen knobs and the search time in ms. */
int hdc_pipeline_autotune(hdc_pipeline* p, int* group_tiles, int* l2_policy, int* tile_n, int* m_blocks,
                          float* ms);

/* ---------------------------------------------------------------- (c) propagate */

/* Bundling of taxonomy nodes: parent p = sum of its children's rows
 * (child_ptr[p] .. child_ptr[p+1] index child_idx, which indexes d_rows),
 * exact int32.  Rows are int16 (elem_bytes 2) or int32 (4); out is int32. */
int hdc_bundle(hdc_context* ctx, const void* d_rows, int elem_bytes, const int64_t* d_child_ptr,
               const int32_t* d_child_idx, int64_t n_parents, int32_t* d_out, void* stream);

/* Greedy representative selection of propagate-children
 * (targets/propogate-children.cpp:60-73), every parent of one rank at once.
 * Parent p visits its candidates d_cand_idx[d_cand_ptr[p] .. d_cand_ptr[p+1])
 * (indices into d_hv, the int16 whole-sequence hypervectors [n][dim] with
 * squared norms d_norm2) in order; candidate x gets
 *   best = max(0, max score(x, s) over the parent's existing sequences
 *          d_rep_idx[d_rep_ptr[p] .. d_rep_ptr[p+1]) and the candidates
 *          already appended)
 * and is appended when (double)best < threshold (the reference uses 0.75 on
 * the NORM scale).  d_selected[i] (uint8) and d_best[i] (float, optional)
 * are per candidate slot; d_scratch holds one int32 per candidate slot. */
int hdc_propagate_greedy(hdc_context* ctx, const int16_t* d_hv, const int64_t* d_norm2,
                         const int64_t* d_cand_ptr, const int32_t* d_cand_idx, const int64_t* d_rep_ptr,
                         const int32_t* d_rep_idx, int64_t n_parents, double threshold, int score_mode,
                         uint8_t* d_selected, float* d_best, int32_t* d_scratch, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HDC_GB300_H */
