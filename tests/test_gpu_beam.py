"""Hierarchical descent (config 5 shape): beam search of bipolar reads down
a bundled taxonomy (leaf encodings, internal nodes = exact int32 sums of
their children) against the oracle's restatement of targets/identify.cpp's
level loop: identical paths, per-level scores and stopping depths."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tree_csr(n_leaves, b):
    """(base, counts, child_ptr, child_idx) of the hdc_synth_tree layout."""
    import hdc_gb300
    bb, base, counts, ptr, idx = hdc_gb300.synth_tree_csr(n_leaves)
    assert bb == b
    return base, counts, ptr, idx


def _drop_children(ptr, idx, nodes):
    """The CSR with the children of `nodes` removed (those nodes become
    childless internal nodes, which the descent re-scores)."""
    kids = [list(idx[ptr[n]:ptr[n + 1]]) for n in range(len(ptr) - 1)]
    for n in nodes:
        kids[n] = []
    out_ptr = np.zeros(len(ptr), np.int64)
    out_ptr[1:] = np.cumsum([len(k) for k in kids])
    return out_ptr, np.array([x for k in kids for x in k], np.int32)


def _first_int16_node(proto):
    """The smallest n such that every row >= n fits int16."""
    import torch
    fits = (proto.abs().amax(dim=1) <= 32767).cpu().numpy()
    n = len(fits)
    while n > 0 and fits[n - 1]:
        n -= 1
    return n


# grouped: 1 reads grouped by candidate node, 2 the same with the levels above the last on
# the tensor cores, 0 one warp per read (identical results)
@pytest.mark.parametrize("grouped,one", [(0, 0), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2)])
@pytest.mark.parametrize("dim,kmer,n_leaves,beam,threshold,childless", [
    (1024, 10, 200, 5, 0.0, False), (2048, 12, 300, 3, 0.0, False), (1024, 8, 150, 5, 0.6, False),
    (2048, 10, 300, 5, -2.0, True), (1024, 10, 200, 8, float("-inf"), True)])
def test_beam_descent_matches_oracle(hdc, orc, cuda, dim, kmer, n_leaves, beam, threshold, childless, grouped, one):
    import torch
    H = hdc
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    tree = H.synth_tree(41 + n_leaves, n_leaves)
    reads = H.synth_reads(42, tree, 64, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, kmer, 250, 10)
    ctx.option(H.BEAM_GROUPED, grouped)
    ctx.option(H.BEAM_ONE_LAUNCH, one)  # grouped: every level in one launch, or kernels per level
    base, counts, ptr, idx = _tree_csr(n_leaves, b)
    n_nodes = int(base[-1])
    proto = torch.zeros((n_nodes, dim), dtype=torch.int32, device=cuda)
    leaves = proto[int(base[5]):]
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), leaves, H.OUT_I32, tree.max_len())
    for r in range(4, -1, -1):  # internal nodes: bundles of their children, bottom-up
        lo, hi = int(base[r]), int(base[r + 1])
        cp = torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda)
        proto[lo:hi] = ctx.bundle(proto, cp, torch.from_numpy(idx).to(cuda))
    q8 = torch.empty((len(reads), dim), dtype=torch.int8, device=cuda)
    ctx.encode_segments(torch.from_numpy(reads.buf).to(cuda), torch.from_numpy(reads.off).to(cuda),
                        torch.from_numpy(reads.len).to(cuda), q8, H.OUT_BIPOLAR_I8, reads.max_len())
    qn = ctx.norms(q8)
    pn = ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    if childless:  # some internal nodes lose their children: the descent scores them again
        ptr, idx = _drop_children(ptr, idx, list(range(int(base[2]), int(base[3]), 3)) + [int(base[1])])
    path, score, depth = ctx.beam_search(q8, qn, proto, pn, torch.from_numpy(ptr).to(cuda),
                                         torch.from_numpy(idx).to(cuda), roots, 6, beam, threshold)
    if grouped:  # the same descent over int16 rows from the first node whose rows all fit 16 bits
        n_wide = _first_int16_node(proto)
        split = ctx.beam_search_split(q8, qn, proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16), pn,
                                      torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda), roots, 6, beam,
                                      threshold)
        for x, y in zip((path, score, depth), split):
            assert torch.equal(x, y)
    torch.cuda.synchronize()
    want = orc.beam_search(q8.cpu().numpy(), proto.cpu().numpy(), ptr, idx, list(range(counts[0])), 6, beam,
                           threshold)
    path, score, depth = path.cpu().numpy(), score.cpu().numpy(), depth.cpu().numpy()
    for r, (wp, ws) in enumerate(want):
        assert depth[r] == len(wp), r
        assert list(path[r, :len(wp)]) == wp, r
        assert np.array_equal(score[r, :len(wp)], np.array(ws, np.float32)), r


def test_beam_grouped_equals_per_read(hdc, cuda):
    """A larger tree and batch: the grouped descent and the one-warp-per-read
    descent return identical paths, scores and depths."""
    import torch
    H = hdc
    dim, n_leaves, nq = 2048, 20000, 3000
    b, base, counts, ptr, idx = H.synth_tree_csr(n_leaves)
    tree = H.synth_tree(7, n_leaves)
    reads = H.synth_reads(8, tree, nq, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, 12, 250, 10)
    proto = torch.zeros((int(base[-1]), dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), proto[int(base[5]):], H.OUT_I32, tree.max_len())
    d_idx = torch.from_numpy(idx).to(cuda)
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        ctx.bundle(proto, torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda), d_idx, out=proto[lo:hi])
    q8 = torch.empty((nq, dim), dtype=torch.int8, device=cuda)
    ctx.encode_segments(torch.from_numpy(reads.buf).to(cuda), torch.from_numpy(reads.off).to(cuda),
                        torch.from_numpy(reads.len).to(cuda), q8, H.OUT_BIPOLAR_I8, reads.max_len())
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    out = []
    for grouped in (0, 1, 2):
        ctx.option(H.BEAM_GROUPED, grouped)
        for threshold in (0.0, float("-inf")):
            res = ctx.beam_search(q8, qn, proto, pn, torch.from_numpy(ptr).to(cuda), d_idx, roots, 6, 5, threshold)
            out.append([x.cpu().numpy() for x in res])
    torch.cuda.synchronize()
    for a, b_ in zip(out[:2], out[2:4]):
        for x, y in zip(a, b_):
            assert np.array_equal(x, y)
    for a, b_ in zip(out[:2], out[4:]):
        for x, y in zip(a, b_):
            assert np.array_equal(x, y)
    assert (out[3][2] == 6).all()  # no early stop: every read reaches a leaf


def test_beam_tensor_core_levels_wide_nodes_and_limbs(hdc, cuda):
    """The tensor-core levels against the CUDA-core grouped descent on a tree
    that stresses them: 3 roots with 40 children each (items of 32 children
    and a remainder of 8), 2 leaves per level-1 node, 300 reads (more than 128
    entries per parent), prototype values up to 2^26 in magnitude (three
    non-zero limbs) with rows at the limb edges, D = 1,024."""
    import torch
    H = hdc
    g = np.random.default_rng(61)
    dim, nq = 1024, 300
    n0, n1 = 3, 3 * 40
    n2 = 2 * n1
    ptr = np.zeros(n0 + n1 + n2 + 1, np.int64)
    idx = []
    for r in range(n0):
        idx += list(range(n0 + 40 * r, n0 + 40 * (r + 1)))
        ptr[r + 1] = len(idx)
    for v in range(n1):
        idx += [n0 + n1 + 2 * v, n0 + n1 + 2 * v + 1]
        ptr[n0 + v + 1] = len(idx)
    ptr[n0 + n1 + 1:] = len(idx)
    idx = np.array(idx, np.int32)
    lim = 1 << 26
    proto_h = g.integers(-lim, lim + 1, (n0 + n1 + n2, dim)).astype(np.int32)
    proto_h[5, :] = lim
    proto_h[6, :] = -lim
    proto_h[7, ::2] = 1023
    proto_h[7, 1::2] = -1024
    proto_h[8, :] = 2048 * 2048 - 1
    proto_h[9, :] = -(2048 * 2048) + 1
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    q[:40] = np.where(proto_h[n0 + 7] >= 0, 1, -1)  # many reads follow one level-1 node
    proto = torch.from_numpy(proto_h).to(cuda)
    q8 = torch.from_numpy(q).to(cuda)
    ctx = H.Context(dim, 10, 250, 10)
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, n0, dtype=torch.int32, device=cuda)
    d_ptr, d_idx = torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda)
    out = []
    cases = [(levels, beam, threshold) for levels in (1, 2, 3)  # 1: no tensor-core level; 2: level 0 only
             for beam, threshold in ((5, float("-inf")), (8, 0.0), (3, -0.5))]
    for grouped in (1, 2):
        ctx.option(H.BEAM_GROUPED, grouped)
        for levels, beam, threshold in cases:
            res = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, levels, beam, threshold)
            out.append([x.cpu().numpy() for x in res])
    torch.cuda.synchronize()
    assert ctx.status() == 0
    n = len(cases)
    for a, b_ in zip(out[:n], out[n:]):
        for x, y in zip(a, b_):
            assert np.array_equal(x, y)



def test_beam_tensor_core_two_limb_items(hdc, cuda):
    """Items whose children all have squared norms <= 2^42 (so every element
    |v| <= 2^21) run with two fp16 limbs; the others with three.  Seven roots:
    0-2 with 40 children each (items of their own), 3-6 with 10 children each
    (two parents to a shared item when they have <= 64 entries, which reads
    0-29 make them).  Children of roots 0, 3 and 5-6 fit two limbs, with rows
    at the edge (one element +-2^21, norm exactly 2^42; all elements +-2^16);
    roots 1 and 4 each have one child of norm 2^42 + 1; root 2's children
    reach 2^26.  The tensor-core descent (every form) equals the CUDA-core
    one, D = 1,024."""
    import torch
    H = hdc
    g = np.random.default_rng(73)
    dim, nq = 1024, 300
    fan = [40, 40, 40, 10, 10, 10, 10]
    n0, n1 = len(fan), sum(fan)
    n2 = 2 * n1
    ptr = np.zeros(n0 + n1 + n2 + 1, np.int64)
    idx, first = [], [n0 + sum(fan[:r]) for r in range(n0)]
    for r in range(n0):
        idx += list(range(first[r], first[r] + fan[r]))
        ptr[r + 1] = len(idx)
    for v in range(n1):
        idx += [n0 + n1 + 2 * v, n0 + n1 + 2 * v + 1]
        ptr[n0 + v + 1] = len(idx)
    ptr[n0 + n1 + 1:] = len(idx)
    idx = np.array(idx, np.int32)
    u = np.where(g.random(dim) < 0.5, -1, 1).astype(np.int64)
    proto_h = np.zeros((n0 + n1 + n2, dim), np.int64)
    for r in range(n0):
        proto_h[r] = (1000 if r < 3 else -1000) * u + g.integers(-200, 201, dim)
    e16 = 1 << 16
    for r in range(n0):  # children leaning towards their root's reads (some pass threshold 0, some stop)
        rows = slice(first[r], first[r] + fan[r])
        h = (1 << 25) if r == 2 else e16 // 2
        proto_h[rows] = (h if r < 3 else -h) * u + g.integers(-h, h + 1, (fan[r], dim))
    c = first[0]
    proto_h[c] = 0
    proto_h[c, 0] = 1 << 21
    proto_h[c + 1] = 0
    proto_h[c + 1, 5] = -(1 << 21)
    proto_h[c + 2, ::2], proto_h[c + 2, 1::2] = e16, -e16
    proto_h[c + 3] = 0
    proto_h[c + 3, 0], proto_h[c + 3, 1] = (1 << 21) - 1, 2047
    for r in (1, 4):  # one child just over the bound: the parent's items take three limbs
        c = first[r] + 1
        proto_h[c] = 0
        proto_h[c, 0], proto_h[c, 1] = 1 << 21, 1
    proto_h[first[5]] = 0
    proto_h[first[5], 3] = -(1 << 21)
    proto_h[n0 + n1:] = g.integers(-30000, 30001, (n2, dim))
    sq = (proto_h.astype(np.float64) ** 2).sum(axis=1)
    assert sq[first[0]] == 2.0 ** 42 and sq[first[1] + 1] == 2.0 ** 42 + 1
    flips = g.random((nq, dim)) < 0.2
    q = np.where(flips, -u, u)
    q[:30] = -q[:30]  # these reads follow roots 3-6 (few entries each: shared items)
    proto = torch.from_numpy(proto_h.astype(np.int32)).to(cuda)
    q8 = torch.from_numpy(q.astype(np.int8)).to(cuda)
    ctx = H.Context(dim, 10, 250, 10)
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    assert int(pn[first[0]]) == 1 << 42 and int(pn[first[4] + 1]) == (1 << 42) + 1
    roots = torch.arange(0, n0, dtype=torch.int32, device=cuda)
    d_ptr, d_idx = torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda)
    cases = [(levels, beam, threshold) for levels in (2, 3)
             for beam, threshold in ((5, 0.0), (8, float("-inf")), (3, 0.0))]
    forms = [(1, 0), (2, 0), (2, 1), (2, 2)]  # (HDC_BEAM_GROUPED, HDC_BEAM_ONE_LAUNCH)
    out = {}
    for grouped, one in forms:
        ctx.option(H.BEAM_GROUPED, grouped)
        ctx.option(H.BEAM_ONE_LAUNCH, one)
        for case in cases:
            res = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, *case)
            out[(grouped, one) + case] = [x.cpu().numpy() for x in res]
    torch.cuda.synchronize()
    assert ctx.status() == 0
    for case in cases:
        ref = out[(1, 0) + case]
        assert (ref[2] == case[0]).any()  # some reads reach the last level
        for form in forms[1:]:
            for x, y in zip(ref, out[form + case]):
                assert np.array_equal(x, y), (form, case)


def test_beam_split_rows_equal_int32(hdc, cuda):
    """hdc_beam_search_split (nodes from n_wide on as int16 rows) returns the
    paths, scores and depths of hdc_beam_search on the same values, in both
    grouped forms, with the cut at the leaves, at the first node whose rows
    fit 16 bits, at 0 (every row int16) where they all fit, and at n_nodes
    (every row int32); the one-warp-per-read form refuses int16 rows."""
    import torch
    H = hdc
    dim, n_leaves, nq = 2048, 20000, 3000
    b, base, counts, ptr, idx = H.synth_tree_csr(n_leaves)
    tree = H.synth_tree(17, n_leaves)
    reads = H.synth_reads(18, tree, nq, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, 12, 250, 10)
    proto = torch.zeros((int(base[-1]), dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), proto[int(base[5]):], H.OUT_I32, tree.max_len())
    d_idx = torch.from_numpy(idx).to(cuda)
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        ctx.bundle(proto, torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda), d_idx, out=proto[lo:hi])
    q8 = torch.empty((nq, dim), dtype=torch.int8, device=cuda)
    ctx.encode_segments(torch.from_numpy(reads.buf).to(cuda), torch.from_numpy(reads.off).to(cuda),
                        torch.from_numpy(reads.len).to(cuda), q8, H.OUT_BIPOLAR_I8, reads.max_len())
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    d_ptr = torch.from_numpy(ptr).to(cuda)
    first16 = _first_int16_node(proto)
    assert first16 < int(base[5])  # the lowest internal rank fits 16 bits too
    n_nodes = proto.shape[0]
    for grouped in (1, 2):
        ctx.option(H.BEAM_GROUPED, grouped)
        for threshold in (0.0, float("-inf")):
            want = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, 6, 5, threshold)
            for n_wide in (int(base[5]), first16, n_nodes):
                got = ctx.beam_search_split(q8, qn, proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16),
                                            pn, d_ptr, d_idx, roots, 6, 5, threshold)
                for x, y in zip(want, got):
                    assert torch.equal(x, y), (grouped, threshold, n_wide)
        # the largest child count given by the caller (no host synchronisation): the same results;
        # one below the tree's stops every read at depth 0 and sets status 200
        maxc = int(np.diff(ptr).max())
        for given in (maxc, maxc + 3):
            got = ctx.beam_search_split(q8, qn, proto[:first16].contiguous(), proto[first16:].to(torch.int16), pn,
                                        d_ptr, d_idx, roots, 6, 5, 0.0, max_children=given)
            want = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, 6, 5, 0.0)
            for x, y in zip(want, got):
                assert torch.equal(x, y), (grouped, given)
        assert ctx.status() == 0
        _, _, depth = ctx.beam_search_split(q8, qn, proto[:first16].contiguous(), proto[first16:].to(torch.int16),
                                            pn, d_ptr, d_idx, roots, 6, 5, 0.0, max_children=maxc - 1)
        assert (depth == 0).all()
        assert ctx.status() == 200
        assert ctx.status() == 0  # read and cleared
    ctx.option(H.BEAM_GROUPED, 0)
    with pytest.raises(H.HDCError):
        ctx.beam_search_split(q8, qn, proto[:first16].contiguous(), proto[first16:].to(torch.int16), pn, d_ptr,
                              d_idx, roots, 6, 5, 0.0)
    torch.cuda.synchronize()
    assert ctx.status() == 0


def test_beam_split_tensor_core_levels_int16_children(hdc, cuda):
    """The tensor-core levels with int16 children: the wide tree (3 roots of 40
    children, items of 32 + 8) with values in the int16 range, rows at its
    edges (32767, -32768, alternating), every row int16 (n_wide = 0), all but
    the roots, or a cut between the 21st and 22nd child of the first root (one
    item, and one producer warp, with both widths), against the int32 descent."""
    import torch
    H = hdc
    g = np.random.default_rng(62)
    dim, nq = 1024, 300
    n0, n1 = 3, 3 * 40
    n2 = 2 * n1
    ptr = np.zeros(n0 + n1 + n2 + 1, np.int64)
    idx = []
    for r in range(n0):
        idx += list(range(n0 + 40 * r, n0 + 40 * (r + 1)))
        ptr[r + 1] = len(idx)
    for v in range(n1):
        idx += [n0 + n1 + 2 * v, n0 + n1 + 2 * v + 1]
        ptr[n0 + v + 1] = len(idx)
    ptr[n0 + n1 + 1:] = len(idx)
    idx = np.array(idx, np.int32)
    proto_h = g.integers(-32768, 32768, (n0 + n1 + n2, dim)).astype(np.int32)
    proto_h[5, :] = 32767
    proto_h[6, :] = -32768
    proto_h[7, ::2] = 32767
    proto_h[7, 1::2] = -32768
    proto_h[n0 + n1 + 3, :] = -32768
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    q[:40] = np.where(proto_h[n0 + 7] >= 0, 1, -1)
    proto = torch.from_numpy(proto_h).to(cuda)
    q8 = torch.from_numpy(q).to(cuda)
    ctx = H.Context(dim, 10, 250, 10)
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, n0, dtype=torch.int32, device=cuda)
    d_ptr, d_idx = torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda)
    for grouped in (1, 2):
        ctx.option(H.BEAM_GROUPED, grouped)
        for levels, beam, threshold in ((1, 5, float("-inf")), (2, 8, 0.0), (3, 5, float("-inf")), (3, 3, -0.5)):
            want = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, levels, beam, threshold)
            for n_wide in (0, n0, n0 + 21):
                got = ctx.beam_search_split(q8, qn, proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16),
                                            pn, d_ptr, d_idx, roots, levels, beam, threshold)
                for x, y in zip(want, got):
                    assert torch.equal(x, y), (grouped, levels, beam, threshold, n_wide)
    torch.cuda.synchronize()
    assert ctx.status() == 0


def _pack_signs(q8, dim):
    """int64 [n][ceil(dim / 32)] words of the +1 signs of int8 rows (bit b of word w: element 32 w + b > 0)."""
    import torch
    n = q8.shape[0]
    words = (dim + 31) // 32
    pos = torch.zeros((n, words * 32), dtype=torch.int64, device=q8.device)
    pos[:, :dim] = (q8[:, :dim] > 0).to(torch.int64)
    weights = (torch.ones(32, dtype=torch.int64, device=q8.device) << torch.arange(32, device=q8.device))
    return (pos.view(n, words, 32) * weights).sum(dim=2)


@pytest.mark.parametrize("dim,kmer", [(1000, 8), (1024, 12), (2048, 10), (200, 3), (1056, 8), (96, 5)])
def test_sign_bits_output_equals_packed_bipolar(hdc, cuda, dim, kmer):
    """HDC_OUT_SIGN_BITS rows are the packed signs of HDC_OUT_BIPOLAR_I8 rows
    (0 -> +1, bits past dim 0), for segments of 0 to 1,600 bytes (counters of
    4, 8 and 12 high planes) with N and lowercase bytes; dense rows of
    ceil(dim / 32) words and nothing written past them (dims 200, 1056, 96:
    one 32-bit word fewer than the ring of 64-bit words holds)."""
    import torch
    H = hdc
    rng = np.random.default_rng(dim + kmer)
    lens = [0, 1, kmer - 1, kmer, kmer + 1, 255 + kmer, 300, 1600] + list(rng.integers(100, 1600, 40))
    seqs = ["".join(rng.choice(list("ACGTACGTACGTNa"), n)) for n in lens]
    ctx = H.Context(dim, kmer, 250, 10)
    short = [x for x in seqs if len(x) <= 200]
    # max_len picks the counter width: <= 255 k-mers 4 high planes, <= 4095 8, else 12
    for batch, max_len in ((short, 200), (seqs, 1600), (seqs, 5000)):
        buf, off, ln = H.pack_sequences(batch)
        d_buf, d_off, d_len = (torch.from_numpy(x.copy()).to(cuda) for x in (buf, off, ln))
        q8 = torch.empty((len(batch), dim), dtype=torch.int8, device=cuda)
        ctx.encode_segments(d_buf, d_off, d_len, q8, H.OUT_BIPOLAR_I8, max_len)
        words = (dim + 31) // 32
        guard = torch.full((len(batch) * words + 64,), 0x5A5A5A5A, dtype=torch.int32, device=cuda)
        bits = guard[:len(batch) * words].view(len(batch), words)
        ctx.encode_segments(d_buf, d_off, d_len, bits, H.OUT_SIGN_BITS, max_len)
        want = _pack_signs(q8, dim)
        assert torch.equal(bits.to(torch.int64) & 0xFFFFFFFF, want), max_len
        assert (guard[len(batch) * words:] == 0x5A5A5A5A).all()  # nothing past the last row


def test_beam_split_bit_reads_equal_int8_reads(hdc, cuda):
    """hdc_beam_search_split_bits over HDC_OUT_SIGN_BITS reads returns what
    hdc_beam_search_split returns over the same reads as int8 rows, in both
    grouped forms."""
    import torch
    H = hdc
    dim, n_leaves, nq = 2048, 20000, 3000
    b, base, counts, ptr, idx = H.synth_tree_csr(n_leaves)
    tree = H.synth_tree(27, n_leaves)
    reads = H.synth_reads(28, tree, nq, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, 12, 250, 10)
    proto = torch.zeros((int(base[-1]), dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), proto[int(base[5]):], H.OUT_I32, tree.max_len())
    d_idx = torch.from_numpy(idx).to(cuda)
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        ctx.bundle(proto, torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda), d_idx, out=proto[lo:hi])
    rb, ro, rl = (torch.from_numpy(x).to(cuda) for x in (reads.buf, reads.off, reads.len))
    q8 = torch.empty((nq, dim), dtype=torch.int8, device=cuda)
    ctx.encode_segments(rb, ro, rl, q8, H.OUT_BIPOLAR_I8, reads.max_len())
    qbits = torch.empty((nq, dim // 32), dtype=torch.int32, device=cuda)
    ctx.encode_segments(rb, ro, rl, qbits, H.OUT_SIGN_BITS, reads.max_len())
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    d_ptr = torch.from_numpy(ptr).to(cuda)
    n_wide = int(base[5])
    p32, p16 = proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16)
    maxc = int(np.diff(ptr).max())
    for grouped in (1, 2):
        ctx.option(H.BEAM_GROUPED, grouped)
        for threshold in (0.0, float("-inf")):
            want = ctx.beam_search_split(q8, qn, p32, p16, pn, d_ptr, d_idx, roots, 6, 5, threshold)
            got = ctx.beam_search_split(qbits, qn, p32, p16, pn, d_ptr, d_idx, roots, 6, 5, threshold,
                                        max_children=maxc)
            for x, y in zip(want, got):
                assert torch.equal(x, y), (grouped, threshold)
    torch.cuda.synchronize()
    assert ctx.status() == 0


def test_beam_one_launch_equals_level_kernels(hdc, cuda):
    """The one-launch descent (descent_one_kernel: every level in one cooperative
    launch, and the same with the last level scored and selected by kernels of
    their own) against the
    same grouped descent run as kernels per level, on a
    20,000-leaf tree with 3,000 reads: identical paths, scores and depths for
    int32 rows and for split int16 rows with sign-bit reads, both grouped forms,
    thresholds 0 and -inf, 6 and 3 levels, a caller-given child count (equal,
    over, and under the tree's: every read stops at depth 0, status 200), and a
    tree with childless internal nodes."""
    import torch
    H = hdc
    dim, n_leaves, nq = 2048, 20000, 3000
    b, base, counts, ptr, idx = H.synth_tree_csr(n_leaves)
    tree = H.synth_tree(23, n_leaves)
    reads = H.synth_reads(24, tree, nq, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, 12, 250, 10)
    proto = torch.zeros((int(base[-1]), dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), proto[int(base[5]):], H.OUT_I32, tree.max_len())
    d_idx = torch.from_numpy(idx).to(cuda)
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        ctx.bundle(proto, torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda), d_idx, out=proto[lo:hi])
    rb, ro, rl = (torch.from_numpy(x).to(cuda) for x in (reads.buf, reads.off, reads.len))
    q8 = torch.empty((nq, dim), dtype=torch.int8, device=cuda)
    qbits = torch.empty((nq, dim // 32), dtype=torch.int32, device=cuda)
    ctx.encode_segments(rb, ro, rl, q8, H.OUT_BIPOLAR_I8, reads.max_len())
    ctx.encode_segments(rb, ro, rl, qbits, H.OUT_SIGN_BITS, reads.max_len())
    qn, pn = ctx.norms(q8), ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    d_ptr = torch.from_numpy(ptr).to(cuda)
    n_wide = int(base[5])
    p32, p16 = proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16)
    maxc = int(np.diff(ptr).max())
    cptr, cidx = _drop_children(ptr, idx, list(range(int(base[2]), int(base[3]), 5)) + [int(base[1])])
    c_ptr, c_idx = torch.from_numpy(cptr).to(cuda), torch.from_numpy(cidx).to(cuda)

    def runs():
        out = []
        for grouped in (1, 2):
            ctx.option(H.BEAM_GROUPED, grouped)
            for levels, threshold in ((6, 0.0), (6, float("-inf")), (3, 0.0)):
                out.append(ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, levels, 5, threshold))
                out.append(ctx.beam_search_split(qbits, qn, p32, p16, pn, d_ptr, d_idx, roots, levels, 5, threshold,
                                                 max_children=maxc))
            out.append(ctx.beam_search_split(qbits, qn, p32, p16, pn, d_ptr, d_idx, roots, 6, 5, 0.0,
                                             max_children=maxc + 2))
            out.append(ctx.beam_search(q8, qn, proto, pn, c_ptr, c_idx, roots, 6, 4, -2.0))
        torch.cuda.synchronize()
        assert ctx.status() == 0
        return [[x.cpu().numpy() for x in res] for res in out]

    ctx.option(H.BEAM_ONE_LAUNCH, 0)
    want = runs()
    for one in (1, 2):  # every level in one launch; the same with the last level in the leaf kernel
        ctx.option(H.BEAM_ONE_LAUNCH, one)
        got = runs()
        for w, g in zip(want, got):
            for x, y in zip(w, g):
                assert np.array_equal(x, y), one
    # a child count below the tree's: every read stops at depth 0 and the status reports it
    _, _, depth = ctx.beam_search_split(qbits, qn, p32, p16, pn, d_ptr, d_idx, roots, 6, 5, 0.0,
                                        max_children=maxc - 1)
    torch.cuda.synchronize()
    assert (depth == 0).all()
    assert ctx.status() == 200
    assert ctx.status() == 0


def test_beam_grid_barrier_wait_runs_out_and_context_recovers(hdc, cuda):
    """A bounded grid-barrier wait of the cooperative descent that runs out,
    without faulting anything: with HDC_TEST_WITHHOLD_LOADS 2 the first CTA
    reaches its first grid barrier four wait limits late (HDC_WAIT_LIMIT), so
    the other CTAs' waits give up and raise the abort word; every CTA leaves
    at that barrier (no phase runs on incomplete data), the leaf launch does
    nothing, TMEM is freed and the context status reports 120.  The next call
    on the same context (hook off, default limit) equals the per-level
    kernels, for both cooperative forms."""
    import torch
    H = hdc
    dim, n_leaves, nq = 2048, 2000, 600
    b, base, counts, ptr, idx = H.synth_tree_csr(n_leaves)
    tree = H.synth_tree(31, n_leaves)
    reads = H.synth_reads(32, tree, nq, 250, subst=0.01)
    ctx = H.Context(dim, 12, 250, 10)
    proto = torch.zeros((int(base[-1]), dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), proto[int(base[5]):], H.OUT_I32, tree.max_len())
    d_idx = torch.from_numpy(idx).to(cuda)
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        ctx.bundle(proto, torch.from_numpy(ptr[lo:hi + 1].copy()).to(cuda), d_idx, out=proto[lo:hi])
    rb, ro, rl = (torch.from_numpy(x).to(cuda) for x in (reads.buf, reads.off, reads.len))
    qbits = torch.empty((nq, dim // 32), dtype=torch.int32, device=cuda)
    ctx.encode_segments(rb, ro, rl, qbits, H.OUT_SIGN_BITS, reads.max_len())
    qn = torch.full((nq,), dim, dtype=torch.int64, device=cuda)
    pn = ctx.norms(proto)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=cuda)
    d_ptr = torch.from_numpy(ptr).to(cuda)
    n_wide = int(base[5])
    p32, p16 = proto[:n_wide].contiguous(), proto[n_wide:].to(torch.int16)
    maxc = int(np.diff(ptr).max())

    def call():
        res = ctx.beam_search_split(qbits, qn, p32, p16, pn, d_ptr, d_idx, roots, 6, 5, float("-inf"),
                                    max_children=maxc)
        torch.cuda.synchronize()
        return [x.cpu().numpy() for x in res]

    ctx.option(H.BEAM_GROUPED, 2)
    ctx.option(H.BEAM_ONE_LAUNCH, 0)
    want = call()
    assert ctx.status() == 0
    for one in (1, 2):
        ctx.option(H.BEAM_ONE_LAUNCH, one)
        ctx.option(H.WAIT_LIMIT, 1000)  # 10^6 SM cycles, about half a millisecond
        ctx.option(H.TEST_WITHHOLD_LOADS, 2)
        call()
        assert ctx.status() == 120, one  # a grid barrier gave up
        ctx.option(H.TEST_WITHHOLD_LOADS, 0)
        ctx.option(H.WAIT_LIMIT, 0)
        got = call()
        assert ctx.status() == 0
        for x, y in zip(want, got):
            assert np.array_equal(x, y), one
