"""ctypes binding of libhdc_synth.so (include/hdc_synth.h): seeded synthetic
16S-like workloads -- taxonomy trees, noisy copies and reads -- standing in for
real data.  Host code only; it maps no GPU library, so a CPU-only process (the
benchmark's reference arm) can build the same workloads."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhdc_synth.so")

P, I32, I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
SIGNATURES = [
    ("hdc_synth_tree", I32, [ctypes.c_uint64, I64, I32, P, I32, I32, I32, P, I64, P, P, P, I32]),
    ("hdc_synth_copies", I32, [ctypes.c_uint64, P, P, P, I64, I32, ctypes.c_double, P, I64, P, P, I32]),
    ("hdc_synth_reads", I32, [ctypes.c_uint64, P, P, P, I64, I64, I32, ctypes.c_double, I32, I32, ctypes.c_double,
                              ctypes.c_double, ctypes.c_double, P, I64, P, P, P, I32]),
]

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libhdc_synth.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class Seqs:
    """Concatenated ASCII sequences on the host: buf uint8, off int64, len int32."""

    def __init__(self, buf, off, ln, label=None):
        self.buf, self.off, self.len, self.label = buf, off, ln, label

    def __len__(self):
        return len(self.off)

    def get(self, i):
        o = int(self.off[i])
        return bytes(self.buf[o:o + int(self.len[i])]).decode()

    def max_len(self):
        return int(self.len.max()) if len(self.len) else 0


def _np_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def synth_tree(seed, n_leaves, root_len=1500, subst=(0.04, 0.03, 0.02, 0.015, 0.01, 0.005), jitter=20,
               min_len=1400, max_len=1600, threads=0):
    import numpy as np
    sub = np.array(subst, np.float64)
    buf = np.zeros(n_leaves * max_len + 16, np.uint8)
    off = np.zeros(n_leaves, np.int64)
    ln = np.zeros(n_leaves, np.int32)
    ranks = np.zeros(7, np.int64)
    if lib().hdc_synth_tree(seed, n_leaves, root_len, _np_ptr(sub), jitter, min_len, max_len, _np_ptr(buf),
                            buf.size, _np_ptr(off), _np_ptr(ln), _np_ptr(ranks), threads) != 0:
        raise ValueError("hdc_synth_tree failed")
    s = Seqs(buf, off, ln)
    s.nodes_per_rank = ranks
    return s


def synth_tree_csr(n_leaves):
    """Node numbering of the taxonomy hdc_synth_tree generates: branching
    b = ceil(n_leaves^(1/6)), ranks 1..6 numbered rank by rank, node j of a
    rank the child of node j // b of the rank above.  Returns (b, base
    [7] first node of each rank, counts [6], child_ptr [n_nodes+1] int64,
    child_idx int32)."""
    import numpy as np
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    counts = [(n_leaves + b ** (6 - r) - 1) // b ** (6 - r) for r in range(1, 7)]
    base = np.cumsum([0] + counts)
    n_child = np.zeros(int(base[-1]), np.int64)
    idx = []
    for r in range(1, 6):
        kids = np.arange(counts[r], dtype=np.int64)
        n_child[base[r - 1]:base[r]] = np.bincount(kids // b, minlength=counts[r - 1])
        idx.append(base[r] + kids)
    ptr = np.zeros(int(base[-1]) + 1, np.int64)
    ptr[1:] = np.cumsum(n_child)
    return b, base, counts, ptr, np.concatenate(idx).astype(np.int32)


def synth_copies(seed, src, n_copies, subst, threads=0):
    import numpy as np
    n = len(src) * n_copies
    buf = np.zeros(int(src.len.astype(np.int64).sum()) * n_copies + 16, np.uint8)
    off = np.zeros(n, np.int64)
    ln = np.zeros(n, np.int32)
    if lib().hdc_synth_copies(seed, _np_ptr(src.buf), _np_ptr(src.off), _np_ptr(src.len), len(src), n_copies,
                              subst, _np_ptr(buf), buf.size, _np_ptr(off), _np_ptr(ln), threads) != 0:
        raise ValueError("hdc_synth_copies failed")
    return Seqs(buf, off, ln)


def synth_reads(seed, src, n_reads, read_len, subst=0.01, sigma=0.0, min_read=100, max_read=1600,
                mixed_frac=0.0, mixed_rate=0.0, threads=0):
    import numpy as np
    cap_len = max(read_len, max_read if sigma > 0 else read_len)
    cap = n_reads * (cap_len + cap_len // 4 + 8) + 16
    buf = np.zeros(cap, np.uint8)
    off = np.zeros(n_reads, np.int64)
    ln = np.zeros(n_reads, np.int32)
    lab = np.zeros(n_reads, np.int32)
    if lib().hdc_synth_reads(seed, _np_ptr(src.buf), _np_ptr(src.off), _np_ptr(src.len), len(src), n_reads,
                             read_len, sigma, min_read, max_read, subst, mixed_frac, mixed_rate, _np_ptr(buf),
                             buf.size, _np_ptr(off), _np_ptr(ln), _np_ptr(lab), threads) != 0:
        raise ValueError("hdc_synth_reads failed")
    return Seqs(buf, off, ln, lab)
