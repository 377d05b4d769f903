"""ctypes front end of the CPU oracle (oracle/hdc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
check its result, and by bench.py's CPU-baseline leg; never by the product path.
Every function restates the reference CPU algorithm (see hdc_oracle.c for
the file:line citations into benlaflen/bacterial-classification).
"""
import ctypes
import os

import numpy as np

from . import build as _build

SCORE_NORM, SCORE_COS, SCORE_DOT = 0, 1, 2

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64, i32 = ctypes.c_int64, ctypes.c_int
        L.orc_mt64_stream.argtypes = [ctypes.c_uint64, i32, P]
        L.orc_base_hvs.argtypes = [i32, P]
        L.orc_base_hvs.restype = i32
        L.orc_canonical.argtypes = [ctypes.c_char_p, i32]
        L.orc_canonical.restype = i64
        L.orc_binder.argtypes = [i32, i32, i64, P]
        L.orc_encode.argtypes = [i32, i32, ctypes.c_char_p, i64, P]
        L.orc_encode.restype = i64
        L.orc_encode_segments.argtypes = [i32, i32, P, P, P, i64, i32, P, P, i32]
        L.orc_cosine_i32.argtypes = [P, P, i32, i32]
        L.orc_cosine_i32.restype = ctypes.c_float
        L.orc_topk_i32.argtypes = [P, i64, P, i64, i32, i32, i32, P, P, P, P, i32]
        L.orc_classify.argtypes = [i32, i32, P, P, P, i64, P, i32, i64, i32, i32, i32, P, P, i32]
        L.orc_classify_ex.argtypes = [i32, i32, P, P, P, i64, P, i32, i64, P, i32, i32, i32, i32, P, P, P, P, i32]
        L.orc_ref_norms.argtypes = [P, i32, i64, i32, P, i32]
        L.orc_ref_norms.restype = i32
        L.orc_encode_copy_bundles.argtypes = [i32, i32, P, P, P, i64, P, P, P, i32, P, i32]
        L.orc_encode_copy_bundles.restype = i32
        L.orc_bundle.argtypes = [P, i32, P, P, i64, P]
        L.orc_encode_bundles.argtypes = [i32, i32, P, P, P, i64, i32, P, i32]
        L.orc_scores_from.argtypes = [P, P, P, i64, i32, P]
        L.orc_propagate_greedy.argtypes = [P, i64, P, i64, i32, ctypes.c_double, i32, P, P]
        L.orc_propagate_greedy.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def nthreads_default():
    return max(1, os.cpu_count() or 1)


def mt64_stream(seed, n):
    out = np.zeros(n, np.uint64)
    lib().orc_mt64_stream(seed, n, _p(out))
    return out


def base_hvs(dim):
    W = (dim + 63) // 64
    out = np.zeros((4, W), np.uint64)
    lib().orc_base_hvs(dim, _p(out))
    return out


def canonical(kmer):
    return lib().orc_canonical(kmer.encode(), len(kmer))


def binder(dim, k, canon):
    out = np.zeros((dim + 63) // 64, np.uint64)
    lib().orc_binder(dim, k, canon, _p(out))
    return out


def pack_segments(seqs):
    """Concatenate byte strings; returns (buffer, offsets, lengths)."""
    bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    lens = np.array([len(b) for b in bs], np.int64)
    offs = np.zeros(len(bs), np.int64)
    if len(bs) > 1:
        offs[1:] = np.cumsum(lens)[:-1]
    buf = np.frombuffer(b"".join(bs) + b"\0", np.uint8).copy()
    return buf, offs, lens


def encode(seqs, dim, k, out="int16", nthreads=None):
    """HVCache::compute of every sequence. out: 'int16' | 'int32' | 'bipolar'."""
    buf, offs, lens = pack_segments(seqs)
    n = len(lens)
    kind = {"int16": 0, "int32": 1, "bipolar": 2}[out]
    dt = {0: np.int16, 1: np.int32, 2: np.int8}[kind]
    res = np.zeros((n, dim), dt)
    nk = np.zeros(n, np.int64)
    lib().orc_encode_segments(dim, k, _p(buf), _p(offs), _p(lens), n, kind, _p(res), _p(nk),
                              nthreads or nthreads_default())
    return res, nk


def encode_bundles(buf, off, lens, dim, k, group=1, nthreads=None):
    """Fast CPU encoder for large reference sets: exact int32 encodings of the
    segments buf[off[i]:off[i]+lens[i]], summed in consecutive groups."""
    buf = np.ascontiguousarray(buf, np.uint8)
    off = np.ascontiguousarray(off, np.int64)
    lens = np.ascontiguousarray(lens, np.int64)
    n = len(off)
    out = np.zeros((n // group, dim), np.int32)
    if lib().orc_encode_bundles(dim, k, _p(buf), _p(off), _p(lens), n, group, _p(out),
                                nthreads or nthreads_default()) != 0:
        raise ValueError("encode_bundles: bad group")
    return out


def encode_copy_bundles(leaves, copies, group, dim, k, nthreads=None):
    """Rows of the sums of `group` consecutive noisy copies of each leaf (exact
    int32): the same rows as encode_bundles(copies, group), computed from each
    leaf's encoding plus the k-mers its copies change.  leaves / copies:
    objects with buf, off, len (copies[i * group + c] is a copy of leaf i)."""
    lb, lo, ll = (np.ascontiguousarray(leaves.buf, np.uint8), np.ascontiguousarray(leaves.off, np.int64),
                  np.ascontiguousarray(leaves.len, np.int64))
    cb, co, cl = (np.ascontiguousarray(copies.buf, np.uint8), np.ascontiguousarray(copies.off, np.int64),
                  np.ascontiguousarray(copies.len, np.int64))
    n = len(lo)
    if len(co) != n * group:
        raise ValueError("encode_copy_bundles: %d copies for %d leaves x %d" % (len(co), n, group))
    out = np.zeros((n, dim), np.int32)
    if lib().orc_encode_copy_bundles(dim, k, _p(lb), _p(lo), _p(ll), n, _p(cb), _p(co), _p(cl), group, _p(out),
                                     nthreads or nthreads_default()) != 0:
        raise ValueError("encode_copy_bundles: bad group")
    return out


def pack_2bit(data):
    """The reference's 2-bit packing (src/encode.cu:169-185, pack_sequence) of a
    byte string as one stream: base i at bits 2 (i % 16) of word i // 16,
    A/a = 0, C/c = 1, G/g = 2, T/t = 3, any other byte 0.  Returns uint32
    words, ceil(len / 16) of them."""
    b = np.frombuffer(bytes(data), np.uint8)
    n = len(b)
    code = np.zeros(((n + 15) // 16) * 16, np.uint32)
    up = b & 0xDF
    code[:n] = np.select([up == ord("C"), up == ord("G"), up == ord("T")], [1, 2, 3], 0)
    code = code.reshape(-1, 16) << (2 * np.arange(16, dtype=np.uint32))
    return np.bitwise_or.reduce(code, axis=1).astype(np.uint32)


def packed_view(seq):
    """The sequence the packed encoder sees: every byte a base by pack_2bit's
    codes (lowercase as its base, any other byte as A)."""
    return "".join(ch.upper() if ch.upper() in "CGT" else "A" for ch in seq)


def window_segments(seqs, window, step):
    """Windows of every sequence: (len-window)//step+1 of them (none when
    len < window), window w covering [w*step, w*step+window)."""
    out = []
    for s in seqs:
        if len(s) < window:
            continue
        for w in range((len(s) - window) // step + 1):
            out.append(s[w * step: w * step + window])
    return out


def cosine(a, b, mode=SCORE_NORM):
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    return lib().orc_cosine_i32(_p(a), _p(b), a.shape[-1], mode)


def topk(q, r, k, mode=SCORE_NORM, nthreads=None):
    """Brute-force top-k: returns (scores f32, idx i32, cos f64, dot i64), each [nq, k]."""
    q = np.ascontiguousarray(q, np.int32)
    r = np.ascontiguousarray(r, np.int32)
    nq, dim = q.shape
    nr = r.shape[0]
    s = np.zeros((nq, k), np.float32)
    i = np.zeros((nq, k), np.int32)
    c = np.zeros((nq, k), np.float64)
    d = np.zeros((nq, k), np.int64)
    lib().orc_topk_i32(_p(q), nq, _p(r), nr, dim, k, mode, _p(s), _p(i), _p(c), _p(d),
                       nthreads or nthreads_default())
    return s, i, c, d


_NORMS = {}  # id of a reference array -> (array, squared norms, max |element|)


def ref_norms(refs, nthreads=None):
    """(squared norms int64 [nr], max |element|) of reference rows, computed
    once per array object (the array must not change in place afterwards)."""
    hit = _NORMS.get(id(refs))
    if hit is not None and hit[0] is refs:
        return hit[1], hit[2]
    r = np.ascontiguousarray(refs)
    rn = np.zeros(r.shape[0], np.int64)
    mx = lib().orc_ref_norms(_p(r), r.dtype.itemsize, r.shape[0], r.shape[1], _p(rn), nthreads or nthreads_default())
    _NORMS.clear()
    _NORMS[id(refs)] = (refs, rn, mx)
    return rn, mx


def classify(reads, refs, dim, kmer, k, mode=SCORE_NORM, bipolar=False, nthreads=None, exact=False):
    """Encode every read and rank it against refs [nr, dim] (int16 or int32): the CPU path.
    Returns (scores f32, idx i32), or with exact=True also (FP64 cosines, int64 dots) of the hits.
    The references' norms are computed on the first call with an array and reused."""
    buf, offs, lens = pack_segments(reads)
    if refs.dtype not in (np.int16, np.int32):
        refs = np.ascontiguousarray(refs, np.int32)
    if not refs.flags.c_contiguous:
        refs = np.ascontiguousarray(refs)
    rn, mx = ref_norms(refs, nthreads)
    n = len(lens)
    s = np.zeros((n, k), np.float32)
    i = np.zeros((n, k), np.int32)
    c = np.zeros((n, k), np.float64) if exact else None
    d = np.zeros((n, k), np.int64) if exact else None
    lib().orc_classify_ex(dim, kmer, _p(buf), _p(offs), _p(lens), n, _p(refs), refs.dtype.itemsize, refs.shape[0],
                          _p(rn), mx, k, mode, int(bipolar), _p(s), _p(i), None if c is None else _p(c),
                          None if d is None else _p(d), nthreads or nthreads_default())
    return (s, i, c, d) if exact else (s, i)


def bundle(rows, child_ptr, child_idx):
    rows = np.ascontiguousarray(rows, np.int32)
    child_ptr = np.ascontiguousarray(child_ptr, np.int64)
    child_idx = np.ascontiguousarray(child_idx, np.int32)
    npar = len(child_ptr) - 1
    out = np.zeros((npar, rows.shape[1]), np.int32)
    lib().orc_bundle(_p(rows), rows.shape[1], _p(child_ptr), _p(child_idx), npar, _p(out))
    return out


def propagate_greedy(reps, cands, threshold=0.75, mode=SCORE_NORM):
    reps = np.ascontiguousarray(reps, np.int32).reshape(-1, cands.shape[1]) if len(reps) else \
        np.zeros((0, cands.shape[1]), np.int32)
    cands = np.ascontiguousarray(cands, np.int32)
    sel = np.zeros(cands.shape[0], np.uint8)
    best = np.zeros(cands.shape[0], np.float32)
    lib().orc_propagate_greedy(_p(reps), reps.shape[0], _p(cands), cands.shape[0], cands.shape[1],
                               threshold, mode, _p(sel), _p(best))
    return sel.astype(bool), best


def scores_from(dot, nl, nr, mode=SCORE_NORM):
    """Reference float scores from exact int64 dots and squared norms."""
    dot = np.ascontiguousarray(dot, np.int64).ravel()
    nl = np.ascontiguousarray(np.broadcast_to(nl, dot.shape), np.int64)
    nr = np.ascontiguousarray(np.broadcast_to(nr, dot.shape), np.int64)
    out = np.zeros(dot.shape, np.float32)
    lib().orc_scores_from(_p(dot), _p(nl), _p(nr), dot.size, mode, _p(out))
    return out


def similarity_rows(seqs, window, step):
    """Similarity rows of every reference sequence, HVCache::similarity
    (src/encoder.cpp:198-215): a sequence with len <= window is one
    whole-sequence row (:200-203); otherwise the windows x = 0, step, ...
    while x + window < len (strict, :205).  Returns (row strings, CSR
    ref_rows [n+1], whole flags [n])."""
    rows, ptr, whole = [], [0], []
    for s in seqs:
        if len(s) <= window:
            rows.append(s)
            whole.append(1)
        else:
            rows.extend(s[x: x + window] for x in range(0, len(s) - window, step))
            whole.append(0)
        ptr.append(len(rows))
    return rows, np.array(ptr, np.int64), np.array(whole, np.uint8)


def similarity(q, rows, ref_rows, whole, pair_q, pair_ref, mode=SCORE_NORM):
    """HVCache::similarity (src/encoder.cpp:198-215) over int16 hypervectors:
    for a whole-sequence reference the unclamped score of its one row, else
    the best score over its rows starting from -1, with the first row that
    beats the running best (strict >, :208-212).  Returns (scores, window
    index within the reference, -1 when no row beat -1)."""
    q = np.asarray(q, np.int64)
    rows = np.asarray(rows, np.int64)
    qn = (q * q).sum(1)
    rn = (rows * rows).sum(1)
    out_s = np.zeros(len(pair_q), np.float32)
    out_w = np.zeros(len(pair_q), np.int32)
    for p, (qi, ri) in enumerate(zip(pair_q, pair_ref)):
        r0, r1 = int(ref_rows[ri]), int(ref_rows[ri + 1])
        sc = scores_from(rows[r0:r1] @ q[qi], qn[qi], rn[r0:r1], mode)
        if whole[ri]:
            out_s[p], out_w[p] = sc[0], 0
            continue
        best, win = np.float32(-1.0), -1
        for j, v in enumerate(sc):
            if v > best:
                best, win = v, j
        out_s[p], out_w[p] = best, win
    return out_s, out_w


def _descent(node_score, nq, child_ptr, child_idx, roots, levels, beam, threshold):
    """The level loop of targets/identify.cpp:89-202.  node_score(r, nodes)
    gives read r's float scores of the candidate nodes.  Returns per read
    (path list, score list, stop level or -1)."""
    out = []
    for r in range(nq):
        beams = [([], [])]
        result = None
        for L in range(levels):
            cands = []
            for path, sc in beams:
                if L == 0:
                    kids = list(roots)
                else:
                    node = path[-1]
                    kids = list(child_idx[child_ptr[node]:child_ptr[node + 1]]) or [node]
                for c in kids:
                    cands.append((path, sc, int(c)))
            nodes = np.array([c[2] for c in cands], np.int64)
            s = node_score(r, nodes) if len(nodes) else np.zeros(0, np.float32)
            order = sorted(range(len(cands)), key=lambda i: (-float(s[i]), int(nodes[i])))
            ranked = [(cands[i][0] + [cands[i][2]], cands[i][1] + [float(s[i])]) for i in order]
            if not ranked or ranked[0][1][-1] < threshold:
                result = (ranked[0] if ranked else beams[0]) + (L,)
                break
            beams = [e for e in ranked[:beam] if e[1][-1] >= threshold]
            if L == levels - 1:
                result = beams[0] + (-1,)
        out.append(result)
    return out


def beam_search(q, proto, child_ptr, child_idx, roots, levels=6, beam=5, threshold=0.0, mode=SCORE_NORM, pn=None):
    """Beam descent of targets/identify.cpp:89-202 with one prototype per node:
    level 0 scores `roots`; each later level expands every beam entry to its
    children (a node without children to itself, :28-33); candidates are
    ranked by score with ties to the lower node index; a read stops with its
    best path when the best score is below threshold (:174-189), else keeps
    the entries with score >= threshold, at most `beam` (:191-199).
    `pn` (squared prototype norms) may be given; prototype rows are widened
    to int64 only when gathered.  Returns per read (path list, score list)."""
    q = np.asarray(q, np.int64)
    if pn is None:
        pn = np.array([int((np.asarray(row, np.int64) ** 2).sum()) for row in proto], np.int64)
    qn = (q * q).sum(1)

    def score(r, nodes):
        return scores_from(np.asarray(proto[nodes], np.int64) @ q[r], qn[r], pn[nodes], mode)

    return [(p, s) for p, s, _ in _descent(score, q.shape[0], child_ptr, child_idx, roots, levels, beam, threshold)]


def identify(q, rows, node_rows, child_ptr, child_idx, roots, levels=6, beam=5, threshold=0.0, mode=SCORE_NORM):
    """targets/identify.cpp:89-202 with its own node score: max(-1, best
    score of the read against every similarity row of every sequence of the
    node) (:127, :138-159), rows of node n at rows[node_rows[n]:node_rows[n+1]].
    Returns per read (path list, score list, stop level or -1)."""
    q = np.asarray(q, np.int64)
    rows = np.asarray(rows, np.int64)
    qn = (q * q).sum(1)
    rn = (rows * rows).sum(1)

    def score(r, nodes):
        out = np.full(len(nodes), -1.0, np.float32)
        for i, n in enumerate(nodes):
            r0, r1 = int(node_rows[n]), int(node_rows[n + 1])
            if r1 > r0:
                out[i] = max(np.float32(-1.0), scores_from(rows[r0:r1] @ q[r], qn[r], rn[r0:r1], mode).max())
        return out

    return _descent(score, q.shape[0], child_ptr, child_idx, roots, levels, beam, threshold)


def fasta_records(data):
    """The FASTA reading of targets/identify.cpp:46-71 over raw bytes: lines
    split on b'\\n' only (a '\\r' stays part of the line); a line starting with
    '>' closes the current record (kept only when its sequence is non-empty)
    and names the next one (the rest of the line); any other line is appended
    to the sequence; the sequence before the first header has an empty name.
    Returns [(name bytes, sequence bytes)] in file order."""
    out = []
    seq, name = [], b""
    lines = data.split(b"\n")
    if data.endswith(b"\n"):
        lines = lines[:-1]  # getline reads no empty line after a final newline
    for line in lines:
        if line.startswith(b">"):
            if seq:
                out.append((name, b"".join(seq)))
                seq = []
            name = line[1:]
        else:
            if line:
                seq.append(line)
    if seq:
        out.append((name, b"".join(seq)))
    return out
