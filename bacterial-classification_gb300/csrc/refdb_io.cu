// Persisted tensor-core reference database: the fp16 limbs, exact squared
// norms and fp32 reciprocal roots of an hdc_refdb, plus optional taxonomy ids
// (one int32 per reference), so a search can start without re-encoding the
// references.  Little-endian file:
//   128-byte header (below), then
//   limbs  [L][r_pad][dim] fp16 | norm2 [nr] int64 | rsq [nr] fp32 | ids [nr] int32 (if present)
// The payload checksum is FNV-1a over its 64-bit little-endian words (the
// tail zero-padded to a word); a load verifies it before returning.
#include <cstdio>
#include <cstring>
#include <vector>

#include "hdc_internal.cuh"

namespace {

constexpr char kMagic[8] = {'H', 'D', 'C', 'R', 'E', 'F', 'D', 'B'};
constexpr uint32_t kVersion = 1;
constexpr size_t kChunk = (size_t)64 << 20;

struct FileHeader {
    char magic[8];
    uint32_t version, header_bytes;
    int32_t dim, kmer, window, step, limbs, max_abs;
    int32_t limb_max[4];
    int64_t nr, r_pad;
    uint32_t has_ids, limb_bits;  // limb_bits 0: 11 (files written before the field)
    uint64_t payload_bytes, payload_fnv;
    uint8_t pad[128 - 8 - 8 - 24 - 16 - 16 - 8 - 16];
};
static_assert(sizeof(FileHeader) == 128, "header layout");

struct Fnv {  // FNV-1a over 64-bit words
    uint64_t h = 0xcbf29ce484222325ull;
    uint8_t tail[8];
    int nt = 0;
    void add(const uint8_t* p, size_t n) {
        while (n && nt) {
            tail[nt++] = *p++;
            --n;
            if (nt == 8) word(tail), nt = 0;
        }
        for (; n >= 8; p += 8, n -= 8) word(p);
        while (n--) tail[nt++] = *p++;
    }
    void word(const uint8_t* p) {
        uint64_t w;
        std::memcpy(&w, p, 8);
        h = (h ^ w) * 0x100000001b3ull;
    }
    uint64_t done() {
        if (nt) {
            std::memset(tail + nt, 0, 8 - nt);
            word(tail);
            nt = 0;
        }
        return h;
    }
};

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

// device -> file, in chunks; checksum as it goes
int put_device(FILE* f, const void* d, size_t bytes, std::vector<uint8_t>& buf, Fnv& fnv) {
    for (size_t o = 0; o < bytes; o += kChunk) {
        const size_t n = bytes - o < kChunk ? bytes - o : kChunk;
        cudaError_t e = cudaMemcpy(buf.data(), static_cast<const uint8_t*>(d) + o, n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return hdc::cuda_fail(e, "refdb save: copy");
        fnv.add(buf.data(), n);
        if (std::fwrite(buf.data(), 1, n, f) != n) return hdc::fail(HDC_ERR_INVALID, "refdb save: write failed");
    }
    return HDC_OK;
}

int get_device(FILE* f, void* d, size_t bytes, std::vector<uint8_t>& buf, Fnv& fnv) {
    for (size_t o = 0; o < bytes; o += kChunk) {
        const size_t n = bytes - o < kChunk ? bytes - o : kChunk;
        if (std::fread(buf.data(), 1, n, f) != n) return hdc::fail(HDC_ERR_INVALID, "refdb load: file truncated");
        fnv.add(buf.data(), n);
        cudaError_t e = cudaMemcpy(static_cast<uint8_t*>(d) + o, buf.data(), n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return hdc::cuda_fail(e, "refdb load: copy");
    }
    return HDC_OK;
}

size_t limb_bytes(const FileHeader& h) { return (size_t)h.limbs * (size_t)h.r_pad * (size_t)h.dim * 2; }
size_t payload_bytes(const FileHeader& h) {
    return limb_bytes(h) + (size_t)h.nr * (8 + 4) + (h.has_ids ? (size_t)h.nr * 4 : 0);
}

int read_header(FILE* f, FileHeader& h) {
    if (std::fread(&h, 1, sizeof h, f) != sizeof h) return hdc::fail(HDC_ERR_INVALID, "refdb file: no header");
    if (std::memcmp(h.magic, kMagic, 8) != 0) return hdc::fail(HDC_ERR_INVALID, "refdb file: not a database file");
    if (h.version != kVersion || h.header_bytes != sizeof h)
        return hdc::fail(HDC_ERR_INVALID, "refdb file: unsupported version");
    if (h.dim < 8 || h.dim % 8 || h.limbs < 1 || h.limbs > 4 || h.nr < 1 || h.r_pad < h.nr || h.r_pad % 256 ||
        h.limb_bits > 11 ||
        h.payload_bytes != payload_bytes(h))
        return hdc::fail(HDC_ERR_INVALID, "refdb file: inconsistent header");
    return HDC_OK;
}

}  // namespace

extern "C" {

int hdc_refdb_save(hdc_context* ctx, const hdc_refdb* db, const char* path, const int32_t* h_tax_ids) {
    if (!ctx || !db || !path) return hdc::fail(HDC_ERR_INVALID, "refdb save: null argument");
    if (db->dim != ctx->dim) return hdc::fail(HDC_ERR_INVALID, "refdb save: database and context dims differ");
    FileHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = sizeof h;
    h.dim = db->dim;
    h.kmer = ctx->kmer;
    h.window = ctx->window;
    h.step = ctx->step;
    h.limbs = db->L;
    h.max_abs = db->max_abs;
    for (int l = 0; l < 4; ++l) h.limb_max[l] = db->limb_max[l];
    h.nr = db->nr;
    h.r_pad = db->r_pad;
    h.has_ids = h_tax_ids ? 1 : 0;
    h.limb_bits = db->limb_bits == 11 ? 0u : (uint32_t)db->limb_bits;
    h.payload_bytes = payload_bytes(h);
    // the checksum goes into the header: write the payload after a placeholder header, then rewrite it
    File out;
    out.f = std::fopen(path, "wb");
    if (!out.f) return hdc::fail(HDC_ERR_INVALID, std::string("refdb save: cannot open ") + path);
    if (std::fwrite(&h, 1, sizeof h, out.f) != sizeof h) return hdc::fail(HDC_ERR_INVALID, "refdb save: write failed");
    std::vector<uint8_t> buf(kChunk);
    Fnv fnv;
    int st = put_device(out.f, db->d_limbs, limb_bytes(h), buf, fnv);
    if (st == HDC_OK) st = put_device(out.f, db->d_norm2, (size_t)db->nr * 8, buf, fnv);
    if (st == HDC_OK) st = put_device(out.f, db->d_rsq, (size_t)db->nr * 4, buf, fnv);
    if (st != HDC_OK) return st;
    if (h_tax_ids) {
        const size_t n = (size_t)db->nr * 4;
        fnv.add(reinterpret_cast<const uint8_t*>(h_tax_ids), n);
        if (std::fwrite(h_tax_ids, 1, n, out.f) != n) return hdc::fail(HDC_ERR_INVALID, "refdb save: write failed");
    }
    h.payload_fnv = fnv.done();
    if (std::fseek(out.f, 0, SEEK_SET) != 0 || std::fwrite(&h, 1, sizeof h, out.f) != sizeof h)
        return hdc::fail(HDC_ERR_INVALID, "refdb save: header rewrite failed");
    if (std::fclose(out.f) != 0) {
        out.f = nullptr;
        return hdc::fail(HDC_ERR_INVALID, "refdb save: close failed");
    }
    out.f = nullptr;
    return HDC_OK;
}

int hdc_refdb_file_info(const char* path, int* dim, int* kmer, int64_t* nr, int* limbs, int* has_tax_ids) {
    if (!path) return hdc::fail(HDC_ERR_INVALID, "refdb file: null path");
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return hdc::fail(HDC_ERR_INVALID, std::string("refdb file: cannot open ") + path);
    FileHeader h;
    const int st = read_header(in.f, h);
    if (st != HDC_OK) return st;
    if (dim) *dim = h.dim;
    if (kmer) *kmer = h.kmer;
    if (nr) *nr = h.nr;
    if (limbs) *limbs = h.limbs;
    if (has_tax_ids) *has_tax_ids = (int)h.has_ids;
    return HDC_OK;
}

int hdc_refdb_load(hdc_context* ctx, const char* path, hdc_refdb** out, int32_t* h_tax_ids) {
    if (!ctx || !path || !out) return hdc::fail(HDC_ERR_INVALID, "refdb load: null argument");
    *out = nullptr;
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return hdc::fail(HDC_ERR_INVALID, std::string("refdb load: cannot open ") + path);
    FileHeader h;
    int st = read_header(in.f, h);
    if (st != HDC_OK) return st;
    if (h.dim != ctx->dim || h.kmer != ctx->kmer)
        return hdc::fail(HDC_ERR_INVALID, "refdb load: the file was encoded with another dim or k-mer size");
    auto* db = new hdc_refdb();
    db->nr = h.nr;
    db->r_pad = h.r_pad;
    db->dim = h.dim;
    db->L = h.limbs;
    db->limb_bits = h.limb_bits ? (int)h.limb_bits : 11;
    db->max_abs = h.max_abs;
    for (int l = 0; l < 4; ++l) db->limb_max[l] = h.limb_max[l];
    cudaError_t e = cudaMalloc(&db->d_limbs, limb_bytes(h));
    if (e == cudaSuccess) e = cudaMalloc(&db->d_norm2, (size_t)h.nr * 8);
    if (e == cudaSuccess) e = cudaMalloc(&db->d_rsq, (size_t)h.nr * 4);
    if (e != cudaSuccess) {
        hdc::refdb_destroy(db);
        return hdc::cuda_fail(e, "refdb load: allocation");
    }
    std::vector<uint8_t> buf(kChunk);
    Fnv fnv;
    st = get_device(in.f, db->d_limbs, limb_bytes(h), buf, fnv);
    if (st == HDC_OK) st = get_device(in.f, db->d_norm2, (size_t)h.nr * 8, buf, fnv);
    if (st == HDC_OK) st = get_device(in.f, db->d_rsq, (size_t)h.nr * 4, buf, fnv);
    if (st == HDC_OK && h.has_ids) {
        std::vector<int32_t> ids((size_t)h.nr);
        if (std::fread(ids.data(), 4, (size_t)h.nr, in.f) != (size_t)h.nr)
            st = hdc::fail(HDC_ERR_INVALID, "refdb load: file truncated");
        else {
            fnv.add(reinterpret_cast<const uint8_t*>(ids.data()), (size_t)h.nr * 4);
            if (h_tax_ids) std::memcpy(h_tax_ids, ids.data(), (size_t)h.nr * 4);
        }
    }
    if (st == HDC_OK && fnv.done() != h.payload_fnv)
        st = hdc::fail(HDC_ERR_INVALID, "refdb load: checksum mismatch (corrupted file)");
    if (st == HDC_OK) st = hdc::refdb_sqrt_table(db, 0);
    if (st == HDC_OK) {
        const cudaError_t e2 = cudaStreamSynchronize(0);
        if (e2 != cudaSuccess) st = hdc::cuda_fail(e2, "refdb load: norms");
    }
    if (st != HDC_OK) {
        hdc::refdb_destroy(db);
        return st;
    }
    *out = db;
    return HDC_OK;
}

}  // extern "C"
