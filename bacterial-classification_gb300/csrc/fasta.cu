// FASTA ingest on the GPU: raw file bytes -> concatenated sequence bytes and
// per-record offsets/lengths of sequence and name, with the reading of
// targets/identify.cpp:46-71: lines end at '\n' only (a '\r' stays part of the
// line); a line starting with '>' closes the current record, kept only when
// its sequence is not empty, and its remainder names the next record; every
// other line is appended to the sequence; bytes before the first header form a
// record with an empty name.
//
// Tiles of 8 KB, one CTA each, a thread walking its 32 bytes with the line
// state (a line is a header when its first byte is '>'):
//   1. tile_count_kernel: per tile, the bytes kept (sequence lines without
//      their '\n') and the header starts, with the bytes of the tile's first
//      line counted apart when that line started in an earlier tile (its type
//      is not known inside the tile), and the tile's last line start;
//   2. tile_scan_kernel (one CTA): the last line start before each tile gives
//      that leading line's type; then the tiles' output and record offsets;
//   3. tile_emit_kernel: the kept bytes to their output positions, and for
//      every header its record's first output position and name;
//   4. per record (record 0 holds the bytes before the first header): its
//      length, kept when not empty, compacted by an exclusive scan.
// The input is read twice and the sequences written once; the workspace is a
// few words per tile and per record (the record arrays are sized after the
// tile scan, one host synchronisation).
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

// ---------------------------------------------------------------- tiles
constexpr int kTileT = 256;
constexpr int kTileB = 32;                   // bytes per thread
constexpr int64_t kTile = kTileT * kTileB;   // bytes per tile

struct TileSum {
    int64_t last_ls;   // last line start in the tile (-1: none)
    int32_t lead_kept; // kept bytes of the tile's first line if it started earlier and is a sequence line
    int32_t kept_in;   // kept bytes of the lines that start in the tile
    int32_t n_hdr;     // header starts in the tile
    uint8_t last_hdr;  // the line starting at last_ls is a header
    uint8_t lead_hdr;  // (scan) the line running into the tile is a header
    int64_t kept_off;  // (scan) output position of the tile's first kept byte
    int64_t hdr_off;   // (scan) headers before the tile
};

struct TileArgs {
    const uint8_t* in;
    int64_t n;
    int64_t n_tiles;
    TileSum* tiles;
    int64_t* totals;   // [2] kept bytes, headers
    // records (step 3 on): record r >= 1 is the r-th header
    int64_t* rec_start;  // [H + 1] output position of the record's first kept byte
    int64_t* name_off;   // [H + 1]
    int64_t* name_end;   // [H + 1]
    uint8_t* out;
};

// This thread's bytes [b0, b0 + nb) and the byte before them.
struct Bytes {
    uint8_t c[kTileB];
    int nb;
    int64_t b0;
    bool ls0;  // b0 is a line start
};

__device__ __forceinline__ void load_bytes(const TileArgs& a, int64_t t, Bytes& x) {
    x.b0 = t * kTile + (int64_t)threadIdx.x * kTileB;
    x.nb = (int)max((int64_t)0, min((int64_t)kTileB, a.n - x.b0));
    if (x.nb == kTileB && (reinterpret_cast<uintptr_t>(a.in + x.b0) & 15) == 0) {
        const uint4 u0 = __ldg(reinterpret_cast<const uint4*>(a.in + x.b0));
        const uint4 u1 = __ldg(reinterpret_cast<const uint4*>(a.in + x.b0) + 1);
        const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
        for (int i = 0; i < kTileB; ++i) x.c[i] = (uint8_t)(w[i >> 2] >> (8 * (i & 3)));
    } else {
#pragma unroll
        for (int i = 0; i < kTileB; ++i) x.c[i] = i < x.nb ? a.in[x.b0 + i] : 0;
    }
    x.ls0 = x.b0 == 0 || (x.nb > 0 && a.in[x.b0 - 1] == '\n');
}

// Block exclusive scan of int64 sums (every thread gets its prefix and the total).
__device__ __forceinline__ int64_t tile_excl_sum(int64_t v, int64_t* sh, int64_t* total) {
    return block_excl_scan64(v, sh, total);
}

// Block exclusive "last" scan of (position, header) pairs: the largest position before this
// thread (-1: none) and its flag.
__device__ __forceinline__ void tile_excl_last(int64_t pos, int flag, int64_t* shp, int* shf, int64_t& out_pos,
                                               int& out_flag) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = pos;
    int f = flag;
    for (int o = 1; o < 32; o <<= 1) {  // inclusive, by position
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        const int g = __shfl_up_sync(0xffffffffu, f, o);
        if (lane >= o && y > x) {
            x = y;
            f = g;
        }
    }
    if (lane == 31) {
        shp[warp] = x;
        shf[warp] = f;
    }
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < kTileT / 32 ? shp[lane] : -1;
        int wf = lane < kTileT / 32 ? shf[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            const int g = __shfl_up_sync(0xffffffffu, wf, o);
            if (lane >= o && y > w) {
                w = y;
                wf = g;
            }
        }
        if (lane < kTileT / 32) {
            shp[lane] = w;
            shf[lane] = wf;
        }
    }
    __syncthreads();
    // exclusive: the previous lane's inclusive value, else the previous warp's
    int64_t px = __shfl_up_sync(0xffffffffu, x, 1);
    int pf = __shfl_up_sync(0xffffffffu, f, 1);
    if (lane == 0) {
        px = warp ? shp[warp - 1] : -1;
        pf = warp ? shf[warp - 1] : 0;
    } else if (warp && shp[warp - 1] > px) {
        px = shp[warp - 1];
        pf = shf[warp - 1];
    }
    out_pos = px;
    out_flag = pf;
    __syncthreads();
}

// The walk over a thread's bytes: hdr = the type of the line in progress at its first byte
// (or -1 while it is the tile's leading line of unknown type).  Counts kept bytes of known
// type, kept bytes of the unknown leading line, header starts; optional callbacks per kept
// byte and per header start.
template <typename KeptFn, typename HdrFn>
__device__ __forceinline__ void walk(const Bytes& x, int hdr, int& kept, int& lead_kept, int& nh, KeptFn kept_fn,
                                     HdrFn hdr_fn) {
    kept = lead_kept = nh = 0;
    bool ls = x.ls0;
#pragma unroll
    for (int i = 0; i < kTileB; ++i) {
        if (i >= x.nb) break;
        const uint8_t c = x.c[i];
        if (ls) {
            hdr = c == '>';
            if (hdr) {
                hdr_fn(i, nh);
                ++nh;
            }
        }
        if (c != '\n') {
            if (hdr == 0) {
                kept_fn(i, kept);
                ++kept;
            } else if (hdr < 0) {
                ++lead_kept;
            }
        }
        ls = c == '\n';
    }
}

__global__ void __launch_bounds__(kTileT) tile_count_kernel(const TileArgs a) {
    __shared__ int64_t shp[kTileT / 32];
    __shared__ int shf[kTileT / 32];
    __shared__ int64_t sh64[kTileT / 32];
    const int64_t t = blockIdx.x;
    Bytes x;
    load_bytes(a, t, x);
    // this thread's last line start and its type
    int64_t my_last = -1;
    int my_last_hdr = 0;
    {
        bool ls = x.ls0;
        for (int i = 0; i < x.nb; ++i) {
            if (ls) {
                my_last = x.b0 + i;
                my_last_hdr = x.c[i] == '>';
            }
            ls = x.c[i] == '\n';
        }
    }
    int64_t before;
    int before_hdr;
    tile_excl_last(my_last, my_last_hdr, shp, shf, before, before_hdr);
    int kept, lead_kept, nh;
    walk(x, before >= 0 ? before_hdr : -1, kept, lead_kept, nh, [](int, int) {}, [](int, int) {});
    int64_t tk, tl, th;
    tile_excl_sum(kept, sh64, &tk);
    tile_excl_sum(lead_kept, sh64, &tl);
    tile_excl_sum(nh, sh64, &th);
    // the tile's last line start: the last thread's inclusive value
    __shared__ int64_t last_pos;
    __shared__ int last_hdr;
    if (threadIdx.x == kTileT - 1) {
        last_pos = my_last >= 0 ? my_last : before;
        last_hdr = my_last >= 0 ? my_last_hdr : before_hdr;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        TileSum& s = a.tiles[t];
        s.last_ls = last_pos;
        s.last_hdr = (uint8_t)last_hdr;
        s.kept_in = (int32_t)tk;
        s.lead_kept = (int32_t)tl;
        s.n_hdr = (int32_t)th;
    }
}

// One CTA: the type of each tile's leading line (the line of the last line start before it),
// the tiles' kept-byte and header offsets, and the totals.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const TileArgs a) {
    __shared__ int64_t shk[32], shh[32], shp[32];
    __shared__ int shf[32];
    int64_t carry_k = 0, carry_h = 0, carry_pos = -1;
    int carry_hdr = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t c0 = 0; c0 < a.n_tiles; c0 += blockDim.x) {
        const int64_t t = c0 + threadIdx.x;
        const bool in = t < a.n_tiles;
        TileSum s{};
        if (in) s = a.tiles[t];
        else s.last_ls = -1;
        // exclusive "last line start" across the tiles: this chunk's scan, then the carry
        int64_t x = s.last_ls;
        int f = s.last_hdr;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            const int g = __shfl_up_sync(0xffffffffu, f, o);
            if (lane >= o && y > x) {
                x = y;
                f = g;
            }
        }
        if (lane == 31) {
            shp[warp] = x;
            shf[warp] = f;
        }
        __syncthreads();
        if (warp == 0) {
            int64_t w = lane < nw ? shp[lane] : -1;
            int wf = lane < nw ? shf[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
                const int g = __shfl_up_sync(0xffffffffu, wf, o);
                if (lane >= o && y > w) {
                    w = y;
                    wf = g;
                }
            }
            if (lane < nw) {
                shp[lane] = w;
                shf[lane] = wf;
            }
        }
        __syncthreads();
        int64_t px = __shfl_up_sync(0xffffffffu, x, 1);
        int pf = __shfl_up_sync(0xffffffffu, f, 1);
        if (lane == 0) {
            px = warp ? shp[warp - 1] : -1;
            pf = warp ? shf[warp - 1] : 0;
        } else if (warp && shp[warp - 1] > px) {
            px = shp[warp - 1];
            pf = shf[warp - 1];
        }
        if (carry_pos > px) {
            px = carry_pos;
            pf = carry_hdr;
        }
        // a tile whose first byte starts a line has no leading line; its lead_kept is 0
        const int lead_hdr = px >= 0 ? pf : 0;
        const int64_t kept = in ? (int64_t)s.kept_in + (lead_hdr ? 0 : s.lead_kept) : 0;
        const int64_t nh = in ? s.n_hdr : 0;
        // exclusive sums of kept bytes and headers
        int64_t vk = kept, vh = nh;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t yk = __shfl_up_sync(0xffffffffu, vk, o);
            const int64_t yh = __shfl_up_sync(0xffffffffu, vh, o);
            if (lane >= o) {
                vk += yk;
                vh += yh;
            }
        }
        if (lane == 31) {
            shk[warp] = vk;
            shh[warp] = vh;
        }
        __syncthreads();
        if (warp == 0) {
            int64_t wk = lane < nw ? shk[lane] : 0, wh = lane < nw ? shh[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t yk = __shfl_up_sync(0xffffffffu, wk, o);
                const int64_t yh = __shfl_up_sync(0xffffffffu, wh, o);
                if (lane >= o) {
                    wk += yk;
                    wh += yh;
                }
            }
            if (lane < nw) {
                shk[lane] = wk;
                shh[lane] = wh;
            }
        }
        __syncthreads();
        const int64_t ek = carry_k + (warp ? shk[warp - 1] : 0) + vk - kept;
        const int64_t eh = carry_h + (warp ? shh[warp - 1] : 0) + vh - nh;
        if (in) {
            a.tiles[t].lead_hdr = (uint8_t)lead_hdr;
            a.tiles[t].kept_off = ek;
            a.tiles[t].hdr_off = eh;
        }
        carry_k += shk[nw - 1];
        carry_h += shh[nw - 1];
        if (shp[nw - 1] > carry_pos) {
            carry_pos = shp[nw - 1];
            carry_hdr = shf[nw - 1];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.totals[0] = carry_k;
        a.totals[1] = carry_h;
    }
}

__global__ void __launch_bounds__(kTileT) tile_emit_kernel(const TileArgs a) {
    __shared__ int64_t shp[kTileT / 32];
    __shared__ int shf[kTileT / 32];
    __shared__ int64_t sh64[kTileT / 32];
    const int64_t t = blockIdx.x;
    const TileSum ts = a.tiles[t];
    Bytes x;
    load_bytes(a, t, x);
    int64_t my_last = -1;
    int my_last_hdr = 0;
    {
        bool ls = x.ls0;
        for (int i = 0; i < x.nb; ++i) {
            if (ls) {
                my_last = x.b0 + i;
                my_last_hdr = x.c[i] == '>';
            }
            ls = x.c[i] == '\n';
        }
    }
    int64_t before;
    int before_hdr;
    tile_excl_last(my_last, my_last_hdr, shp, shf, before, before_hdr);
    const int hdr0 = before >= 0 ? before_hdr : ts.lead_hdr;  // the leading line's type is known now
    int kept, lead_kept, nh;
    walk(x, hdr0, kept, lead_kept, nh, [](int, int) {}, [](int, int) {});
    int64_t tot;
    const int64_t kbase = ts.kept_off + tile_excl_sum(kept, sh64, &tot);
    const int64_t hbase = ts.hdr_off + tile_excl_sum(nh, sh64, &tot);
    // second walk: the kept bytes and the headers
    walk(
        x, hdr0, kept, lead_kept, nh, [&](int i, int k) { a.out[kbase + k] = x.c[i]; },
        [&](int i, int h) {
            const int64_t r = hbase + h + 1;  // record 0 holds the bytes before the first header
            // kept bytes of this thread before byte i: header bytes are not kept, so the count
            // of kept bytes at i is the record's first output position
            int k = 0;
            {
                int hh = -1;
                bool ls = x.ls0;
                if (!ls) hh = before >= 0 ? before_hdr : ts.lead_hdr;
                for (int j = 0; j < i; ++j) {
                    if (ls) hh = x.c[j] == '>';
                    if (x.c[j] != '\n' && hh == 0) ++k;
                    ls = x.c[j] == '\n';
                }
            }
            a.rec_start[r] = kbase + k;
            const int64_t pos = x.b0 + i;
            a.name_off[r] = pos + 1;
            int64_t e = pos + 1;
            while (e < a.n && a.in[e] != '\n') ++e;  // a header on the last line without '\n' ends at n
            a.name_end[r] = e;
        });
}

__global__ void rec_len_kernel(const int64_t* __restrict__ rec_start, const int64_t* __restrict__ totals,
                               uint8_t* __restrict__ nonempty) {
    const int64_t H = totals[1];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= H; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = r < H ? rec_start[r + 1] : totals[0];
        nonempty[r] = e > rec_start[r];
    }
}

__global__ void rec_emit_kernel(const int64_t* __restrict__ rec_start, const int64_t* __restrict__ name_off,
                                const int64_t* __restrict__ name_end, const uint8_t* __restrict__ nonempty,
                                const int64_t* __restrict__ ro, const int64_t* __restrict__ totals,
                                int64_t max_records, int64_t* __restrict__ seq_off, int32_t* __restrict__ seq_len,
                                int64_t* __restrict__ o_name_off, int32_t* __restrict__ o_name_len,
                                int64_t* __restrict__ count) {
    const int64_t H = totals[1];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= H; r += (int64_t)gridDim.x * blockDim.x) {
        if (!nonempty[r]) continue;
        const int64_t j = ro[r];
        if (j >= max_records) continue;
        const int64_t s = rec_start[r];
        const int64_t e = r < H ? rec_start[r + 1] : totals[0];
        seq_off[j] = s;
        seq_len[j] = (int32_t)(e - s);
        o_name_off[j] = r ? name_off[r] : 0;
        o_name_len[j] = r ? (int32_t)(name_end[r] - name_off[r]) : 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = ro[H + 1];
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
    TileArgs a{};
    a.in = reinterpret_cast<const uint8_t*>(d_in);
    a.n = n;
    a.n_tiles = (n + kTile - 1) / kTile;
    a.out = reinterpret_cast<uint8_t*>(d_out);
    if (a.n_tiles > 0x7fffffffLL) return fail(HDC_ERR_RANGE, "fasta: input too large");
    // tiles, then (after the scan) the records
    uint8_t* ws = nullptr;
    const size_t b_tiles = ((size_t)a.n_tiles * sizeof(TileSum) + 255) & ~(size_t)255;
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&ws), b_tiles + 256, stream)) != cudaSuccess)
        return cuda_fail(e, "fasta: workspace");
    a.tiles = reinterpret_cast<TileSum*>(ws);
    a.totals = reinterpret_cast<int64_t*>(ws + b_tiles);
    tile_count_kernel<<<(unsigned)a.n_tiles, kTileT, 0, stream>>>(a);
    tile_scan_kernel<<<1, 1024, 0, stream>>>(a);
    int64_t totals[2] = {0, 0};
    e = cudaMemcpyAsync(totals, a.totals, sizeof totals, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(ws, stream);
        return cuda_fail(e, "fasta: tile scan");
    }
    const int64_t R = totals[1] + 1;  // record 0 and one per header
    const int64_t ws_elems = scan_ws_elems(R + 1);
    uint8_t* rs = nullptr;
    int64_t* ro = nullptr;
    int64_t* ws_scan = nullptr;
    uint8_t* nonempty = nullptr;
    auto carve_all = [&](uint8_t* base) {
        uint8_t* cur = base;
        a.rec_start = carve_f<int64_t>(cur, R);
        a.name_off = carve_f<int64_t>(cur, R);
        a.name_end = carve_f<int64_t>(cur, R);
        nonempty = carve_f<uint8_t>(cur, R + 1);
        ro = carve_f<int64_t>(cur, R + 1);
        ws_scan = carve_f<int64_t>(cur, ws_elems);
        return (size_t)(cur - base);
    };
    const size_t bytes = carve_all(nullptr);
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&rs), bytes, stream)) != cudaSuccess) {
        cudaFreeAsync(ws, stream);
        return cuda_fail(e, "fasta: record workspace");
    }
    carve_all(rs);
    // record 0: the bytes before the first header, from output position 0
    cudaMemsetAsync(a.rec_start, 0, sizeof(int64_t), stream);
    tile_emit_kernel<<<(unsigned)a.n_tiles, kTileT, 0, stream>>>(a);
    const unsigned rg = (unsigned)std::max<int64_t>(1, std::min<int64_t>((R + 255) / 256, (int64_t)ctx->num_sms * 8));
    rec_len_kernel<<<rg, 256, 0, stream>>>(a.rec_start, a.totals, nonempty);
    cudaMemsetAsync(nonempty + R, 0, 1, stream);
    scan64<uint8_t>(nonempty, ro, R + 1, false, ws_scan, stream);
    rec_emit_kernel<<<rg, 256, 0, stream>>>(a.rec_start, a.name_off, a.name_end, nonempty, ro, a.totals, max_records,
                                            d_seq_off, d_seq_len, d_name_off, d_name_len, d_count);
    e = cudaGetLastError();
    cudaFreeAsync(rs, stream);
    cudaFreeAsync(ws, stream);
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "fasta: launch");
}

}  // namespace hdc
