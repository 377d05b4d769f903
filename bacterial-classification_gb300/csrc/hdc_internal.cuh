// Internal definitions shared by the translation units of libhdc_gb300.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "hdc_gb300.h"

struct hdc_context {
    int dim = 0;      // HV_DIM
    int kmer = 0;     // KMER_SIZE
    int window = 0;   // SEQUENCE_LENGTH
    int step = 0;     // SIM_STEP
    int words64 = 0;  // ceil(dim / 64): the reference's HV_WORDS
    int words32 = 0;  // 2 * words64: the 64*HV_WORDS-bit ring in 32-bit words
    int device = 0;
    int num_sms = 0;
    uint64_t* host_base = nullptr;  // [4][words64], A,C,G,T
    uint32_t* d_base32 = nullptr;   // [4][words32] on the device
    int* d_status = nullptr;        // device status word written by kernels that can give up
    int tc_group = 0;               // tensor-core search: query tiles per group (0: automatic)
    int tc_policy = -1;             // tensor-core search: L2 policy (-1: automatic, see hdc_search_tc_tuning)
    int tc_tile_n = 0;              // tensor-core search: references per tile, 128 or 256 (0: automatic)
    int tc_m_blocks = 0;            // tensor-core search: 128-query M-blocks per CTA, 1 or 2 (0: automatic)
    int tc_prefetch = -1;           // tensor-core search: K blocks prefetched into L2 ahead (-1: automatic)
    int tc_cluster = 0;             // tensor-core search: CTAs sharing an operand's blocks, 1 or 2 (0: automatic)
    int tc_share = -1;              // tensor-core search: 0 pairs share references, 1 queries (-1: automatic)
    mutable int tc_quad_fit = -1;   // clusters of 4 of the pair-MMA search resident at once (-1: not asked yet)
    int32_t tc_last_shape[5] = {0, 0, 0, 0, 0};  // cluster, G, S, pair MMA, kernels of the last tc search
    int tc_lanes = 0;               // tensor-core search: at most this many reference lanes (0: SMs / G)
    int tc_pair_mma = -1;           // tensor-core search: CTA pairs as one M = 256 MMA (-1: automatic)
    int tc_kblock = 0;              // tensor-core search: dims per K block, 32 or 64 (0: automatic)
    int tc_scatter = -1;            // tensor-core search: 1 scattered reference-tile order, 0 index order (-1: auto)
    int beam_grouped = -1;          // descent: 1 grouped by candidate node, 2 + tensor-core levels, 0 warp per read
    void* noalloc_scratch = nullptr;  // device address of hdc_search_plain_noalloc's fixed scratch (first call)
    int greedy_form = -1;             // propagate-children selection: 1 scored (dim % 8 == 0), 0 sequential, -1 automatic
    int beam_one = -1;                // grouped descent: 1 every level in one cooperative launch, 2 the same
                                      // with the last level in a cooperative kernel of its own, 0 a
                                      // launch sequence per level, -1 automatic (2 where it fits)
    mutable int beam_one_fit = -1;    // the one-launch descent's CTAs all fit at once (-1: not asked yet)
    unsigned long long* d_phase_ts = nullptr;  // phase clock of the last one-launch descent (diagnostic)
    long long wait_cycles = 0;        // tensor-core search and descent: limit of their bounded waits in SM
                                      // cycles (0: default)
    int test_withhold_loads = 0;      // test hook: 1 the search's producer issues no loads, 2 the cooperative
                                      // descent's first CTA reaches its first grid barrier late
};

// A tensor-core reference database (hdc_refdb_create).
struct hdc_refdb {
    int64_t nr = 0, r_pad = 0;
    int dim = 0, L = 0;
    __half* d_limbs = nullptr;  // [L][r_pad][dim]
    int64_t* d_norm2 = nullptr; // [nr]
    float* d_rsq = nullptr;     // [nr]
    double* d_sqrt = nullptr;   // [2][nr] sqrt(norm2) rounded to double (the exact score's factor), then its rounded reciprocal
    int32_t limb_max[4] = {0, 0, 0, 0};
    int limb_bits = 11;         // limbs are balanced base-2^limb_bits digits (the top one within the cap)
    int32_t max_abs = 0;
};

namespace hdc {

// Records a message for hdc_last_error() and returns the status.
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

inline bool valid_score_mode(int m) { return m == HDC_SCORE_NORM || m == HDC_SCORE_COS || m == HDC_SCORE_DOT; }

// Launchers implemented in the kernel translation units.
int launch_encode(hdc_context* ctx, const char* d_bytes, const int64_t* d_seg_off, const int32_t* d_seg_len,
                  const int64_t* d_seq_off, const int64_t* d_win_off, int64_t n_seqs, int64_t n_segs,
                  int out_kind, void* d_out, int64_t out_stride, int32_t* d_nkmers, int max_seg_len,
                  cudaStream_t stream, const int32_t* d_order = nullptr, int* d_queue = nullptr,
                  const uint32_t* d_words = nullptr);
int encode_slabs(const hdc_context* ctx);
// ASCII bytes -> 2-bit words (16 bases per word, the reference's packing)
int launch_pack_2bit(hdc_context* ctx, const char* d_bytes, int64_t n_bytes, uint32_t* d_words, cudaStream_t stream);

int launch_norms(hdc_context* ctx, const void* d_hv, int elem_bytes, int64_t n, int64_t* d_norm2,
                 int32_t* d_maxabs, cudaStream_t stream);

size_t plain_workspace_bytes(const hdc_context* ctx, int64_t nq, int64_t nr, int k);

int launch_search_plain(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, int64_t nq, int32_t maxq,
                        const int16_t* d_r, const int64_t* d_rn, int64_t nr, int32_t maxr, int k, int mode,
                        float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot, void* d_work,
                        size_t work_bytes, cudaStream_t stream);

// Merge n_lists partial top-k lists per query ([n_lists][nq][k] keys and dots)
// into the final outputs; keys whose index is not below nr count as empty.
int launch_merge(const uint64_t* ws_key, const int64_t* ws_dot, int n_lists, int64_t nq, int k, const int64_t* d_qn,
                 const int64_t* d_rn, int64_t nr, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot,
                 cudaStream_t stream);

// launch_norms element code of integer-valued fp16 rows (1, 2, 4: int8 / int16 / int32)
constexpr int kNormsF16 = -2;

int refdb_create(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                 int32_t max_query_abs, hdc_refdb** out,
                 cudaStream_t stream);
void refdb_destroy(hdc_refdb* db);
size_t tc_workspace_bytes(const hdc_context* ctx, int64_t nq, const hdc_refdb* db, int k);
int tc_default_group();
int tc_default_policy();
int tc_default_prefetch();
int tc_default_cluster();
int tc_default_share();
int tc_default_scatter();
int tc_default_kblock();
int tc_default_pair_mma();
// Fill db->d_sqrt (allocated here) from db->d_norm2.
int refdb_sqrt_table(hdc_refdb* db, cudaStream_t stream);
int tc_default_tile_n();
int tc_default_m_blocks();
int launch_search_tc(hdc_context* ctx, const hdc_refdb* db, const __half* d_q, const int64_t* d_qn, int64_t nq,
                     int32_t maxq, int k, int mode, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot,
                     void* d_work, size_t work_bytes, int* d_status, cudaStream_t stream);

int launch_propagate_greedy(hdc_context* ctx, const int16_t* d_hv, const int64_t* d_norm2,
                            const int64_t* d_cand_ptr, const int32_t* d_cand_idx, const int64_t* d_rep_ptr,
                            const int32_t* d_rep_idx, int64_t n_parents, double threshold, int mode,
                            uint8_t* d_selected, float* d_best, int32_t* d_scratch, cudaStream_t stream);

int launch_beam_search(hdc_context* ctx, const int8_t* d_q, const uint32_t* d_qbits, const int64_t* d_qn, int64_t nq, const int32_t* d_proto,
                       int64_t n32, const int16_t* d_proto16, const int64_t* d_pn, int64_t n_nodes,
                       const int64_t* d_child_ptr, const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                       int levels, int beam, double threshold, int mode, int32_t* d_path, float* d_path_score,
                       int32_t* d_depth, cudaStream_t stream);

int launch_identify(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, int64_t nq, const int16_t* d_rows,
                    const int64_t* d_rn, const int64_t* d_node_rows, const int64_t* d_child_ptr,
                    const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int levels, int beam,
                    double threshold, int mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                    int32_t* d_stop_level, cudaStream_t stream);

int launch_similarity(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, const int16_t* d_rows,
                      const int64_t* d_rn, const int64_t* d_ref_rows, const uint8_t* d_ref_whole,
                      const int32_t* d_pair_q, const int32_t* d_pair_ref, int64_t n_pairs, int mode, float* d_score,
                      int32_t* d_window, cudaStream_t stream);

// the descent with reads grouped by candidate node (beam_grouped.cu); dim % 1024 == 0, dim <= 16384;
// nodes < n32 have int32 rows in d_proto, the others int16 rows in d_proto16 (row node - n32);
// reads as int8 +1/-1 rows d_q, or as sign bits d_qbits [nq][dim / 32] (then d_q is unused)
// durations of the phases of the last one-launch descent (ns), returns how many
int beam_phase_times(const hdc_context* ctx, int64_t* out_ns, int max_n);
int launch_beam_grouped(hdc_context* ctx, const int8_t* d_q, const uint32_t* d_qbits, const int64_t* d_qn, int64_t nq, const int32_t* d_proto,
                        int64_t n32, const int16_t* d_proto16, const int64_t* d_pn, int64_t n_nodes, const int64_t* d_child_ptr, const int32_t* d_child_idx,
                        const int32_t* d_roots, int n_roots, int max_children, int levels, int beam, double threshold, int mode,
                        int32_t* d_path, float* d_path_score, int32_t* d_depth, cudaStream_t stream);

int launch_fasta_parse(hdc_context* ctx, const char* d_in, int64_t n, char* d_out, int64_t* d_seq_off,
                       int32_t* d_seq_len, int64_t* d_name_off, int32_t* d_name_len, int64_t max_records,
                       int64_t* d_count, cudaStream_t stream);

int launch_bundle(hdc_context* ctx, const void* d_rows, int elem_bytes, const int64_t* d_child_ptr,
                  const int32_t* d_child_idx, int64_t n_parents, int32_t* d_out, cudaStream_t stream);

}  // namespace hdc
