// FASTA ingest on the GPU: raw file bytes -> concatenated sequence bytes and
// per-record offsets/lengths of sequence and name, with the reading of
// targets/identify.cpp:46-71: lines end at '\n' only (a '\r' stays part of the
// line); a line starting with '>' closes the current record, kept only when
// its sequence is not empty, and its remainder names the next record; every
// other line is appended to the sequence; bytes before the first header form a
// record with an empty name.
//
// Byte-parallel: line starts, line numbers (scan), one type per line
// (header or not), kept bytes (sequence lines without their '\n') compacted by
// an exclusive scan, record index per byte (scan of header starts), then one
// pass over records for boundaries and a compaction of the non-empty ones.
// Positions are int64 (inputs beyond 2 GB); the scans recurse over their block
// sums, so any size that fits the workspace works.
#include "hdc_internal.cuh"

namespace hdc {
namespace {

constexpr int kT = 256;
constexpr int kItems = 8;
constexpr int64_t kBlk = kT * kItems;

__device__ __forceinline__ int64_t block_excl_scan64(int64_t v, int64_t* sh, int64_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < kT / 32 ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kT / 32) sh[lane] = w;
    }
    __syncthreads();
    const int64_t before = (warp ? sh[warp - 1] : 0) + x - v;
    *total = sh[kT / 32 - 1];
    __syncthreads();
    return before;
}

template <typename T>
__global__ void __launch_bounds__(kT) blk_sums(const T* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
    __shared__ int64_t sh[kT / 32];
    const int64_t base = blockIdx.x * kBlk + (int64_t)threadIdx.x * kItems;
    int64_t v = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i)
        if (base + i < n) v += (int64_t)in[base + i];
    int64_t total;
    block_excl_scan64(v, sh, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// out[i] = sum(in[0..i]) (inclusive) or sum(in[0..i)) (exclusive, and then out[n] = total);
// `offs` = exclusive scan of the block sums.  In place (out == in) is allowed.
template <typename T>
__global__ void __launch_bounds__(kT) blk_apply(const T* in, int64_t n, const int64_t* __restrict__ offs,
                                                int64_t* out, int inclusive) {
    __shared__ int64_t sh[kT / 32];
    const int64_t base = blockIdx.x * kBlk + (int64_t)threadIdx.x * kItems;
    int64_t v[kItems], s = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        v[i] = base + i < n ? (int64_t)in[base + i] : 0;
        s += v[i];
    }
    int64_t total;
    int64_t run = offs[blockIdx.x] + block_excl_scan64(s, sh, &total);
#pragma unroll
    for (int i = 0; i < kItems; ++i)
        if (base + i < n) {
            if (inclusive) run += v[i];
            out[base + i] = run;
            if (!inclusive) run += v[i];
        }
    if (!inclusive && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = offs[blockIdx.x] + total;
}

__global__ void set_zero64(int64_t* p) { *p = 0; }

int64_t scan_ws_elems(int64_t n) {  // block sums of every level
    int64_t t = 0;
    for (int64_t nb = (n + kBlk - 1) / kBlk; nb > 1; nb = (nb + kBlk - 1) / kBlk) t += nb + 1;
    return t + 2;
}

template <typename T>
void scan64(const T* in, int64_t* out, int64_t n, bool inclusive, int64_t* ws, cudaStream_t s) {
    const int64_t nb = (n + kBlk - 1) / kBlk;
    int64_t* sums = ws;
    if (nb > 1) {
        blk_sums<T><<<(unsigned)nb, kT, 0, s>>>(in, n, sums);
        scan64<int64_t>(sums, sums, nb, false, ws + nb + 1, s);  // block offsets, in place
    } else {
        set_zero64<<<1, 1, 0, s>>>(sums);
    }
    blk_apply<T><<<(unsigned)nb, kT, 0, s>>>(in, n, sums, out, inclusive ? 1 : 0);
}

// ---------------------------------------------------------------- per byte
struct FastaArgs {
    const uint8_t* in;
    int64_t n;
    uint8_t* ls;       // [n] line starts here
    uint8_t* hs;       // [n] a header line starts here
    uint8_t* keep;     // [n] sequence byte
    uint8_t* ltype;    // [n] per line: 1 header
    int64_t* ln;       // [n] inclusive scan of ls: line number + 1
    int64_t* rid;      // [n] inclusive scan of hs: record index (0 before the first header)
    int64_t* pos;      // [n + 1] exclusive scan of keep: output position
    int64_t* rec_start;  // [n + 1] first output position of record r
    int64_t* name_off;   // [n + 1]
    int64_t* name_end;   // [n + 1]
    uint8_t* nonempty;   // [n + 1]
    int64_t* ro;         // [n + 2] exclusive scan of nonempty
};

__global__ void flags_kernel(const FastaArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool ls = i == 0 || a.in[i - 1] == '\n';
        a.ls[i] = ls;
        a.hs[i] = ls && a.in[i] == '>';
    }
}

__global__ void line_type_kernel(const FastaArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x)
        if (a.ls[i]) a.ltype[a.ln[i] - 1] = a.hs[i];
}

__global__ void keep_kernel(const FastaArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x)
        a.keep[i] = !a.ltype[a.ln[i] - 1] && a.in[i] != '\n';
}

__global__ void compact_kernel(const FastaArgs a, uint8_t* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x)
        if (a.keep[i]) out[a.pos[i]] = a.in[i];
}

// record r >= 1 starts at its header byte; record 0 (before any header) at byte 0
__global__ void records_kernel(const FastaArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        if (a.hs[i]) {
            const int64_t r = a.rid[i];
            a.rec_start[r] = a.pos[i];
            a.name_off[r] = i + 1;
        }
        if (a.in[i] == '\n' && a.ltype[a.ln[i] - 1]) a.name_end[a.rid[i]] = i;  // a header line ends here
    }
}

__global__ void record_len_kernel(const FastaArgs a) {
    const int64_t H = a.rid[a.n - 1];  // records 0..H
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= a.n; r += (int64_t)gridDim.x * blockDim.x) {
        uint8_t keep = 0;
        if (r <= H) {
            const int64_t e = r < H ? a.rec_start[r + 1] : a.pos[a.n];
            keep = e > a.rec_start[r];
        }
        a.nonempty[r] = keep;
    }
}

__global__ void emit_kernel(const FastaArgs a, int64_t max_records, int64_t* __restrict__ seq_off,
                            int32_t* __restrict__ seq_len, int64_t* __restrict__ name_off,
                            int32_t* __restrict__ name_len, int64_t* __restrict__ count) {
    const int64_t H = a.rid[a.n - 1];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= H; r += (int64_t)gridDim.x * blockDim.x) {
        if (!a.nonempty[r]) continue;
        const int64_t j = a.ro[r];
        if (j >= max_records) continue;
        const int64_t s = a.rec_start[r];
        const int64_t e = r < H ? a.rec_start[r + 1] : a.pos[a.n];
        seq_off[j] = s;
        seq_len[j] = (int32_t)(e - s);
        name_off[j] = r ? a.name_off[r] : 0;
        name_len[j] = r ? (int32_t)(a.name_end[r] - a.name_off[r]) : 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = a.ro[a.n + 1];
}

__global__ void init_records_kernel(const FastaArgs a) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= a.n; r += (int64_t)gridDim.x * blockDim.x) {
        a.rec_start[r] = 0;
        a.name_off[r] = 0;
        a.name_end[r] = a.n;  // a header on the last line without '\n' ends at the end of the input
    }
}

template <typename T>
T* carve_f(uint8_t*& cur, int64_t n) {
    T* p = reinterpret_cast<T*>(cur);
    cur += ((size_t)(n > 0 ? n : 1) * sizeof(T) + 255) & ~(size_t)255;
    return p;
}

}  // namespace

int launch_fasta_parse(hdc_context* ctx, const char* d_in, int64_t n, char* d_out, int64_t* d_seq_off,
                       int32_t* d_seq_len, int64_t* d_name_off, int32_t* d_name_len, int64_t max_records,
                       int64_t* d_count, cudaStream_t stream) {
    cudaError_t e;
    if (n == 0) {
        e = cudaMemsetAsync(d_count, 0, sizeof(int64_t), stream);
        return e == cudaSuccess ? HDC_OK : cuda_fail(e, "fasta: memset");
    }
    FastaArgs a{};
    a.in = reinterpret_cast<const uint8_t*>(d_in);
    a.n = n;
    int64_t* ws_scan = nullptr;
    const int64_t ws_elems = scan_ws_elems(n + 2);
    auto carve_all = [&](uint8_t* base) {
        uint8_t* cur = base;
        a.ls = carve_f<uint8_t>(cur, n);
        a.hs = carve_f<uint8_t>(cur, n);
        a.keep = carve_f<uint8_t>(cur, n);
        a.ltype = carve_f<uint8_t>(cur, n);
        a.nonempty = carve_f<uint8_t>(cur, n + 1);
        a.ln = carve_f<int64_t>(cur, n);
        a.rid = carve_f<int64_t>(cur, n);
        a.pos = carve_f<int64_t>(cur, n + 1);
        a.rec_start = carve_f<int64_t>(cur, n + 1);
        a.name_off = carve_f<int64_t>(cur, n + 1);
        a.name_end = carve_f<int64_t>(cur, n + 1);
        a.ro = carve_f<int64_t>(cur, n + 2);
        ws_scan = carve_f<int64_t>(cur, ws_elems);
        return (size_t)(cur - base);
    };
    const size_t bytes = carve_all(nullptr);
    uint8_t* ws = nullptr;
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, stream)) != cudaSuccess)
        return cuda_fail(e, "fasta: workspace");
    carve_all(ws);
    const int grid = ctx->num_sms * 8;
    flags_kernel<<<grid, 256, 0, stream>>>(a);
    scan64<uint8_t>(a.ls, a.ln, n, true, ws_scan, stream);
    line_type_kernel<<<grid, 256, 0, stream>>>(a);
    keep_kernel<<<grid, 256, 0, stream>>>(a);
    scan64<uint8_t>(a.keep, a.pos, n, false, ws_scan, stream);
    scan64<uint8_t>(a.hs, a.rid, n, true, ws_scan, stream);
    compact_kernel<<<grid, 256, 0, stream>>>(a, reinterpret_cast<uint8_t*>(d_out));
    init_records_kernel<<<grid, 256, 0, stream>>>(a);
    records_kernel<<<grid, 256, 0, stream>>>(a);
    record_len_kernel<<<grid, 256, 0, stream>>>(a);
    scan64<uint8_t>(a.nonempty, a.ro, n + 1, false, ws_scan, stream);
    emit_kernel<<<grid, 256, 0, stream>>>(a, max_records, d_seq_off, d_seq_len, d_name_off, d_name_len, d_count);
    e = cudaGetLastError();
    cudaFreeAsync(ws, stream);
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "fasta: launch");
}

}  // namespace hdc
