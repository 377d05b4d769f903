"""ctypes binding of libhdc_gb300.so (the C ABI in include/hdc_gb300.h).

This is the Python side used by the tests, the smoke check and the benchmark;
device memory and streams come from torch (plumbing only: every computation
runs in the library's own CUDA kernels).  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhdc_gb300.so")

HDC_OK = 0
ERR = {1: "HDC_ERR_INVALID", 2: "HDC_ERR_RANGE", 3: "HDC_ERR_CUDA", 4: "HDC_ERR_NOMEM",
       5: "HDC_ERR_UNSUPPORTED", 6: "HDC_ERR_TIMEOUT"}
SCORE_NORM, SCORE_COS, SCORE_DOT = 0, 1, 2
TC_PREFETCH, TC_CLUSTER, TC_SHARE, BEAM_GROUPED, TC_SCATTER, TC_KBLOCK, TC_PAIR_MMA, TC_LANES = 1, 2, 3, 4, 5, 6, 7, 8
OUT_I16, OUT_I32, OUT_BIPOLAR_BF16, OUT_BIPOLAR_I16, OUT_BIPOLAR_F16, OUT_BIPOLAR_I8, OUT_F16 = 0, 1, 2, 3, 4, 5, 6
WAIT_LIMIT, TEST_WITHHOLD_LOADS, BEAM_ONE_LAUNCH, GREEDY_FORM = 9, 10, 11, 12
OUT_SIGN_BITS = 7  # sign bits, int32 [n][dim / 32] (bit b of word w: element 32 w + b >= 0)

# (name, restype, argtypes) of every exported entry point
P, I32, I64, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_size_t
SIGNATURES = [
    ("hdc_last_error", ctypes.c_char_p, []),
    ("hdc_status_string", ctypes.c_char_p, [I32]),
    ("hdc_context_create", I32, [I32, I32, I32, I32, ctypes.POINTER(P)]),
    ("hdc_context_destroy", None, [P]),
    ("hdc_context_base_hvs", I32, [P, P]),
    ("hdc_device_alloc", I32, [SZ, ctypes.POINTER(P)]),
    ("hdc_device_free", I32, [P]),
    ("hdc_copy", I32, [P, P, SZ, I32, P]),
    ("hdc_stream_sync", I32, [P]),
    ("hdc_encode_segments", I32, [P, P, P, P, I64, ctypes.c_int32, I32, P, I64, P, P]),
    ("hdc_num_windows", I64, [P, I64]),
    ("hdc_pack_2bit", I32, [P, P, I64, P, P]),
    ("hdc_binders", I32, [P, P, I64, P]),
    ("hdc_beam_phase_times", I32, [P, P, I32, ctypes.POINTER(I32)]),
    ("hdc_encode_packed", I32, [P, P, P, P, I64, ctypes.c_int32, I32, P, I64, P, P]),
    ("hdc_encode_windows", I32, [P, P, P, P, I64, I64, P, P]),
    ("hdc_norms", I32, [P, P, I32, I64, P, P, P]),
    ("hdc_search_workspace_bytes", SZ, [P, I64, I64, I32]),
    ("hdc_search_plain", I32, [P, P, P, I64, ctypes.c_int32, P, P, I64, ctypes.c_int32, I32, I32, P, P, P, P, P,
                               SZ, P]),
    ("hdc_bundle", I32, [P, P, I32, P, P, I64, P, P]),
    ("hdc_beam_search", I32, [P, P, P, I64, P, P, I64, P, P, P, I32, I32, I32, ctypes.c_double, I32, P, P, P, P]),
    ("hdc_beam_search_split", I32, [P, P, P, I64, P, I64, P, P, I64, P, P, P, I32, I32, I32, I32, ctypes.c_double,
                                    I32, P, P, P, P]),
    ("hdc_beam_search_split_bits", I32, [P, P, P, I64, P, I64, P, P, I64, P, P, P, I32, I32, I32, I32,
                                         ctypes.c_double, I32, P, P, P, P]),
    ("hdc_similarity", I32, [P, P, P, P, P, P, P, P, P, I64, I32, P, P, P]),
    ("hdc_identify", I32, [P, P, P, I64, P, P, P, P, P, P, I32, I32, I32, ctypes.c_double, I32, P, P, P, P, P]),
    ("hdc_propagate_greedy", I32, [P, P, P, P, P, P, P, I64, ctypes.c_double, I32, P, P, P, P]),
    ("hdc_context_status", I32, [P, ctypes.POINTER(ctypes.c_int)]),
    ("hdc_search_plain_noalloc", I32, [P, P, P, I64, ctypes.c_int32, P, P, I64, ctypes.c_int32, I32, I32, P, P, P,
                                       P, P]),
    ("hdc_refdb_create", I32, [P, P, I32, I64, ctypes.c_int32, ctypes.POINTER(P), P]),
    ("hdc_refdb_destroy", None, [P]),
    ("hdc_refdb_limbs", I32, [P]),
    ("hdc_norms_f16", I32, [P, P, I64, P, P, P]),
    ("hdc_refdb_create_ex", I32, [P, P, I32, I64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(P), P]),
    ("hdc_refdb_limb_bits", I32, [P]),
    ("hdc_search_tc_workspace_bytes", SZ, [P, P, I64, I32]),
    ("hdc_refdb_save", I32, [P, P, ctypes.c_char_p, P]),
    ("hdc_refdb_file_info", I32, [ctypes.c_char_p, P, P, P, P, P]),
    ("hdc_refdb_load", I32, [P, ctypes.c_char_p, P, P]),
    ("hdc_fasta_parse", I32, [P, P, I64, P, P, P, P, P, I64, P, P]),
    ("hdc_search_tc_tuning", I32, [P, I32, I32, I32, I32]),
    ("hdc_search_tc_last_shape", I32, [P, P]),
    ("hdc_context_option", I32, [P, I32, I32]),
    ("hdc_pipeline_create", I32, [P, P, I64, I64, ctypes.c_int32, I32, I32, ctypes.POINTER(P)]),
    ("hdc_pipeline_destroy", None, [P]),
    ("hdc_pipeline_run", I32, [P, P, P, P, I64, P, P]),
    ("hdc_pipeline_launch_resident", I32, [P]),
    ("hdc_pipeline_stream", P, [P]),
    ("hdc_pipeline_autotune", I32, [P, ctypes.POINTER(I32), ctypes.POINTER(I32), ctypes.POINTER(I32),
                                    ctypes.POINTER(I32), ctypes.POINTER(ctypes.c_float)]),
    ("hdc_search_tc", I32, [P, P, P, P, I64, ctypes.c_int32, I32, I32, P, P, P, P, P, SZ, P]),
]

_lib = None


class HDCError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (ERR.get(status, status), msg))
        self.status = status


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libhdc_gb300.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != HDC_OK:
        raise HDCError(status, lib().hdc_last_error().decode())


def ptr(t):
    """Device (or host) address of a torch tensor, or None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Context:
    """One hypervector configuration (dim, kmer, window, step) on the current device."""

    def __init__(self, dim, kmer, window=150, step=10):
        self.dim, self.kmer, self.window, self.step = dim, kmer, window, step
        h = ctypes.c_void_p()
        check(lib().hdc_context_create(dim, kmer, window, step, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().hdc_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def base_hvs(self):
        import numpy as np
        out = np.zeros((4, (self.dim + 63) // 64), np.uint64)
        check(lib().hdc_context_base_hvs(self.h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    # ---------------------------------------------------------------- encode
    def encode_segments(self, d_bytes, d_off, d_len, out, out_kind=OUT_I16, max_len=0, nkmers=None, stream=None):
        n = d_off.numel()
        check(lib().hdc_encode_segments(self.h, ptr(d_bytes), ptr(d_off), ptr(d_len), n, int(max_len), out_kind,
                                        ptr(out), out.stride(0), ptr(nkmers), stream_ptr(stream)))
        return out

    def binders(self, codes):
        """Binder hypervectors [n][ceil(dim / 64)] uint64 of k-mer codes (host)."""
        import numpy as np
        c = np.ascontiguousarray(codes, np.int64)
        out = np.zeros((len(c), (self.dim + 63) // 64), np.uint64)
        check(lib().hdc_binders(self.h, c.ctypes.data_as(ctypes.c_void_p), len(c),
                                out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def pack_2bit(self, d_bytes, n_bytes=None, stream=None):
        """2-bit words (int32 tensor, ceil(n / 16)) of the first n bytes of a uint8 tensor."""
        import torch
        n = d_bytes.numel() if n_bytes is None else n_bytes
        words = torch.empty(max(1, (n + 15) // 16), dtype=torch.int32, device=d_bytes.device)
        check(lib().hdc_pack_2bit(self.h, ptr(d_bytes), n, ptr(words), stream_ptr(stream)))
        return words

    def encode_packed(self, d_words, d_base_off, d_len, out, out_kind=OUT_I16, max_len=0, nkmers=None, stream=None):
        n = d_base_off.numel()
        check(lib().hdc_encode_packed(self.h, ptr(d_words), ptr(d_base_off), ptr(d_len), n, int(max_len), out_kind,
                                      ptr(out), out.stride(0), ptr(nkmers), stream_ptr(stream)))
        return out

    def num_windows(self, length):
        return lib().hdc_num_windows(self.h, length)

    def encode_windows(self, d_bytes, d_seq_off, d_win_off, n_windows, out, stream=None):
        check(lib().hdc_encode_windows(self.h, ptr(d_bytes), ptr(d_seq_off), ptr(d_win_off), d_seq_off.numel() - 1,
                                       n_windows, ptr(out), stream_ptr(stream)))
        return out

    # ---------------------------------------------------------------- search
    def norms(self, hv, maxabs=None, stream=None):
        import torch
        n2 = torch.empty(hv.shape[0], dtype=torch.int64, device=hv.device)
        if hv.dtype == torch.float16:  # integer-valued fp16 rows
            check(lib().hdc_norms_f16(self.h, ptr(hv), hv.shape[0], ptr(n2), ptr(maxabs), stream_ptr(stream)))
        else:
            check(lib().hdc_norms(self.h, ptr(hv), hv.element_size(), hv.shape[0], ptr(n2), ptr(maxabs),
                                  stream_ptr(stream)))
        return n2

    def workspace_bytes(self, nq, nr, k):
        return lib().hdc_search_workspace_bytes(self.h, nq, nr, k)

    def search_plain(self, q, qn, maxq, r, rn, maxr, k, mode=SCORE_NORM, work=None, out=None, stream=None):
        import torch
        nq, nr = q.shape[0], r.shape[0]
        kk = min(k, nr)
        dev = q.device
        if out is None:
            out = (torch.empty((nq, kk), dtype=torch.float32, device=dev),
                   torch.empty((nq, kk), dtype=torch.int32, device=dev),
                   torch.empty((nq, kk), dtype=torch.float64, device=dev),
                   torch.empty((nq, kk), dtype=torch.int64, device=dev))
        wb = self.workspace_bytes(nq, nr, k)
        if work is None or work.numel() < wb:
            work = torch.empty(max(wb, 16), dtype=torch.uint8, device=dev)
        s, i, c, d = out
        check(lib().hdc_search_plain(self.h, ptr(q), ptr(qn), nq, int(maxq), ptr(r), ptr(rn), nr, int(maxr), k, mode,
                                     ptr(s), ptr(i), ptr(c), ptr(d), ptr(work), work.numel(), stream_ptr(stream)))
        return out

    def status(self):
        st = ctypes.c_int(0)
        check(lib().hdc_context_status(self.h, ctypes.byref(st)))
        return st.value

    def option(self, option, value):
        check(lib().hdc_context_option(self.h, option, value))

    tc_option = option

    def tc_tuning(self, group_tiles=0, l2_policy=-1, tile_n=0, m_blocks=0):
        check(lib().hdc_search_tc_tuning(self.h, group_tiles, l2_policy, tile_n, m_blocks))

    def tc_last_shape(self):
        """(CTAs per cluster, query tiles per group, reference lanes, pair MMA, kernels launched)
        of the last search_tc."""
        out = (ctypes.c_int32 * 5)()
        check(lib().hdc_search_tc_last_shape(self.h, ctypes.addressof(out)))
        return tuple(out)

    def refdb(self, refs, max_abs, stream=None, max_query_abs=0):
        return RefDB(self, refs, max_abs, stream, max_query_abs=max_query_abs)

    def search_tc(self, db, q, qn, maxq, k, mode=SCORE_NORM, work=None, out=None, stream=None):
        import torch
        nq = q.shape[0]
        kk = min(k, db.nr)
        dev = q.device
        if out is None:
            out = (torch.empty((nq, kk), dtype=torch.float32, device=dev),
                   torch.empty((nq, kk), dtype=torch.int32, device=dev),
                   torch.empty((nq, kk), dtype=torch.float64, device=dev),
                   torch.empty((nq, kk), dtype=torch.int64, device=dev))
        wb = lib().hdc_search_tc_workspace_bytes(self.h, db.h, nq, k)
        if work is None or work.numel() < wb:
            work = torch.empty(max(wb, 16), dtype=torch.uint8, device=dev)
        s, i, c, d = out
        check(lib().hdc_search_tc(self.h, db.h, ptr(q), ptr(qn), nq, int(maxq), k, mode, ptr(s), ptr(i), ptr(c),
                                  ptr(d), ptr(work), work.numel(), stream_ptr(stream)))
        return out

    # ---------------------------------------------------------------- propagate
    def propagate_greedy(self, hv, norm2, cand_ptr, cand_idx, rep_ptr, rep_idx, threshold=0.75, mode=SCORE_NORM,
                         stream=None):
        import torch
        n = cand_idx.numel()
        sel = torch.zeros(max(n, 1), dtype=torch.uint8, device=hv.device)
        best = torch.zeros(max(n, 1), dtype=torch.float32, device=hv.device)
        scratch = torch.empty(max(n, 1), dtype=torch.int32, device=hv.device)
        check(lib().hdc_propagate_greedy(self.h, ptr(hv), ptr(norm2), ptr(cand_ptr), ptr(cand_idx), ptr(rep_ptr),
                                         ptr(rep_idx), cand_ptr.numel() - 1, threshold, mode, ptr(sel), ptr(best),
                                         ptr(scratch), stream_ptr(stream)))
        return sel[:n], best[:n]

    def beam_search(self, q, qn, proto, pn, child_ptr, child_idx, roots, levels=6, beam=5, threshold=0.0,
                    mode=SCORE_NORM, stream=None):
        import torch
        nq = q.shape[0]
        path = torch.empty((nq, levels), dtype=torch.int32, device=q.device)
        score = torch.empty((nq, levels), dtype=torch.float32, device=q.device)
        depth = torch.empty(nq, dtype=torch.int32, device=q.device)
        check(lib().hdc_beam_search(self.h, ptr(q), ptr(qn), nq, ptr(proto), ptr(pn), proto.shape[0], ptr(child_ptr),
                                    ptr(child_idx),
                                    ptr(roots), roots.numel(), levels, beam, threshold, mode, ptr(path), ptr(score),
                                    ptr(depth), stream_ptr(stream)))
        return path, score, depth

    def beam_search_split(self, q, qn, proto32, proto16, pn, child_ptr, child_idx, roots, levels=6, beam=5,
                          threshold=0.0, mode=SCORE_NORM, stream=None, max_children=0):
        """hdc_beam_search_split: nodes < proto32.shape[0] have int32 rows, the
        others int16 rows in proto16 (node n is row n - proto32.shape[0]);
        max_children > 0 spares the call its host synchronisation.  q: int8
        +1/-1 rows, or int32 [nq][dim / 32] sign bits (HDC_OUT_SIGN_BITS rows,
        hdc_beam_search_split_bits)."""
        import torch
        nq = q.shape[0]
        n_wide = proto32.shape[0] if proto32 is not None else 0
        n_nodes = n_wide + (proto16.shape[0] if proto16 is not None else 0)
        path = torch.empty((nq, levels), dtype=torch.int32, device=q.device)
        score = torch.empty((nq, levels), dtype=torch.float32, device=q.device)
        depth = torch.empty(nq, dtype=torch.int32, device=q.device)
        fn = lib().hdc_beam_search_split_bits if q.dtype == torch.int32 else lib().hdc_beam_search_split
        check(fn(self.h, ptr(q), ptr(qn), nq, ptr(proto32), n_wide, ptr(proto16), ptr(pn), n_nodes, ptr(child_ptr),
                 ptr(child_idx), ptr(roots), roots.numel(), max_children, levels, beam, threshold, mode, ptr(path),
                 ptr(score), ptr(depth), stream_ptr(stream)))
        return path, score, depth

    def beam_phase_times(self):
        """Durations (ms) of the phases of the last one-launch descent, as its first CTA saw them."""
        import numpy as np
        out = np.zeros(64, np.int64)
        n = I32()
        check(lib().hdc_beam_phase_times(self.h, out.ctypes.data_as(ctypes.c_void_p), 64, ctypes.byref(n)))
        return [float(x) / 1e6 for x in out[:n.value]]

    def similarity(self, q, qn, rows, rn, ref_rows, ref_whole, pair_q, pair_ref, mode=SCORE_NORM, stream=None):
        """HVCache::similarity for (query, reference) pairs; returns (scores,
        first best window index within the reference or -1)."""
        import torch
        n = pair_q.numel()
        score = torch.empty(max(n, 1), dtype=torch.float32, device=q.device)
        win = torch.empty(max(n, 1), dtype=torch.int32, device=q.device)
        check(lib().hdc_similarity(self.h, ptr(q), ptr(qn), ptr(rows), ptr(rn), ptr(ref_rows),
                                   ptr(ref_whole) if ref_whole is not None else None, ptr(pair_q), ptr(pair_ref), n,
                                   mode, ptr(score), ptr(win), stream_ptr(stream)))
        return score[:n], win[:n]

    def identify(self, q, qn, rows, rn, node_rows, child_ptr, child_idx, roots, levels=6, beam=5, threshold=0.0,
                 mode=SCORE_NORM, stream=None):
        """identify's descent with max-over-similarity-rows node scores;
        returns (path, path scores, depth, stop level)."""
        import torch
        nq = q.shape[0]
        path = torch.empty((nq, levels), dtype=torch.int32, device=q.device)
        score = torch.empty((nq, levels), dtype=torch.float32, device=q.device)
        depth = torch.empty(nq, dtype=torch.int32, device=q.device)
        stop = torch.empty(nq, dtype=torch.int32, device=q.device)
        check(lib().hdc_identify(self.h, ptr(q), ptr(qn), nq, ptr(rows), ptr(rn), ptr(node_rows), ptr(child_ptr),
                                 ptr(child_idx), ptr(roots), roots.numel(), levels, beam, threshold, mode, ptr(path),
                                 ptr(score), ptr(depth), ptr(stop), stream_ptr(stream)))
        return path, score, depth, stop

    def fasta_parse(self, d_bytes, max_records=None, stream=None):
        """Device FASTA ingest of raw file bytes (uint8 tensor): returns (sequence bytes, seq_off,
        seq_len, name_off, name_len, number of records) with the reference's reading."""
        import torch
        n = d_bytes.numel()
        cap = (n + 1) if max_records is None else max_records
        dev = d_bytes.device
        out = torch.empty(max(n, 1), dtype=torch.uint8, device=dev)
        so = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
        sl = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
        no = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
        nl = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        check(lib().hdc_fasta_parse(self.h, ptr(d_bytes), n, ptr(out), ptr(so), ptr(sl), ptr(no), ptr(nl), cap,
                                    ptr(cnt), stream_ptr(stream)))
        c = int(cnt.item())
        m = min(c, cap)
        return out, so[:m], sl[:m], no[:m], nl[:m], c

    def bundle(self, rows, child_ptr, child_idx, out=None, stream=None):
        import torch
        npar = child_ptr.numel() - 1
        if out is None:
            out = torch.empty((npar, self.dim), dtype=torch.int32, device=rows.device)
        check(lib().hdc_bundle(self.h, ptr(rows), rows.element_size(), ptr(child_ptr), ptr(child_idx), npar,
                               ptr(out), stream_ptr(stream)))
        return out


class RefDB:
    """Tensor-core reference database (fp16 limbs + exact norms) built from int16/int32 rows,
    or loaded from a file written by save()."""

    def __init__(self, ctx, refs, max_abs, stream=None, _handle=None, _nr=0, max_query_abs=0):
        h = ctypes.c_void_p()
        if _handle is None:
            if max_query_abs:  # limbs sized for count-valued queries up to max_query_abs
                check(lib().hdc_refdb_create_ex(ctx.h, ptr(refs), refs.element_size(), refs.shape[0], int(max_abs),
                                                int(max_query_abs), ctypes.byref(h), stream_ptr(stream)))
            else:
                check(lib().hdc_refdb_create(ctx.h, ptr(refs), refs.element_size(), refs.shape[0], int(max_abs),
                                             ctypes.byref(h), stream_ptr(stream)))
            _nr = refs.shape[0]
        else:
            h = _handle
        self.h, self.nr, self.ctx = h, _nr, ctx
        self.limbs = lib().hdc_refdb_limbs(h)
        self.limb_bits = lib().hdc_refdb_limb_bits(h)

    def save(self, path, tax_ids=None):
        """Write the database (and optional int32 taxonomy ids, one per reference) to `path`."""
        import numpy as np
        ids = None if tax_ids is None else np.ascontiguousarray(tax_ids, np.int32)
        check(lib().hdc_refdb_save(self.ctx.h, self.h, str(path).encode(),
                                   None if ids is None else ids.ctypes.data_as(ctypes.c_void_p)))

    @staticmethod
    def file_info(path):
        d, k, lim, ids = I32(), I32(), I32(), I32()
        nr = ctypes.c_int64()
        check(lib().hdc_refdb_file_info(str(path).encode(), ctypes.byref(d), ctypes.byref(k), ctypes.byref(nr),
                                        ctypes.byref(lim), ctypes.byref(ids)))
        return dict(dim=d.value, kmer=k.value, nr=nr.value, limbs=lim.value, has_tax_ids=bool(ids.value))

    @classmethod
    def load(cls, ctx, path):
        """(database, taxonomy ids or None) from a file written by save()."""
        import numpy as np
        info = cls.file_info(path)
        ids = np.zeros(info["nr"], np.int32) if info["has_tax_ids"] else None
        h = ctypes.c_void_p()
        check(lib().hdc_refdb_load(ctx.h, str(path).encode(), ctypes.byref(h),
                                   None if ids is None else ids.ctypes.data_as(ctypes.c_void_p)))
        return cls(ctx, None, 0, _handle=h, _nr=info["nr"]), ids

    def close(self):
        if self.h:
            lib().hdc_refdb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pipeline:
    """Batching form: CUDA-graph encode -> tensor-core search -> top-k over host batches."""

    def __init__(self, ctx, db, max_reads, max_bytes, max_len, k, mode=SCORE_NORM):
        import numpy as np
        h = ctypes.c_void_p()
        check(lib().hdc_pipeline_create(ctx.h, db.h, max_reads, max_bytes, max_len, k, mode, ctypes.byref(h)))
        self.h, self.k, self.max_reads = h, min(k, db.nr), max_reads
        self.ctx, self.db = ctx, db  # keep alive
        self._np = np

    def run(self, seqs, n=None):
        np = self._np
        n = len(seqs) if n is None else n
        s = np.zeros((n, self.k), np.float32)
        i = np.zeros((n, self.k), np.int32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        check(lib().hdc_pipeline_run(self.h, p(seqs.buf), p(seqs.off), p(seqs.len), n, p(s), p(i)))
        return s, i

    def launch_resident(self):
        check(lib().hdc_pipeline_launch_resident(self.h))

    def stream(self):
        return lib().hdc_pipeline_stream(self.h)

    def autotune(self):
        g, pol, tn, mb = I32(), I32(), I32(), I32()
        ms = ctypes.c_float()
        check(lib().hdc_pipeline_autotune(self.h, ctypes.byref(g), ctypes.byref(pol), ctypes.byref(tn), ctypes.byref(mb),
                                          ctypes.byref(ms)))
        return dict(group_tiles=g.value, l2_policy=pol.value, tile_n=tn.value, m_blocks=mb.value, ms=ms.value)

    def close(self):
        if self.h:
            lib().hdc_pipeline_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack_sequences(seqs):
    """Host packing of ASCII sequences: (bytes uint8[total+16], offsets int64[n], lengths int32[n])."""
    import numpy as np
    bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    lens = np.fromiter((len(b) for b in bs), np.int64, len(bs))
    offs = np.zeros(len(bs), np.int64)
    if len(bs) > 1:
        offs[1:] = np.cumsum(lens)[:-1]
    buf = np.frombuffer(b"".join(bs) + b"\0" * 16, np.uint8)
    return buf, offs, lens.astype(np.int32)


# ---------------------------------------------------------------- synthetic workloads
# The generator lives in its own library (libhdc_synth.so); re-exported here for callers of this module.
from hdc_synth import Seqs, synth_copies, synth_reads, synth_tree, synth_tree_csr  # noqa: E402,F401
