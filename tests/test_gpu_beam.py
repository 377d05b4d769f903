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


# grouped: 1 reads grouped by candidate node, 0 one warp per read (identical results)
@pytest.mark.parametrize("grouped", [0, 1])
@pytest.mark.parametrize("dim,kmer,n_leaves,beam,threshold,childless", [
    (1024, 10, 200, 5, 0.0, False), (2048, 12, 300, 3, 0.0, False), (1024, 8, 150, 5, 0.6, False),
    (2048, 10, 300, 5, -2.0, True), (1024, 10, 200, 8, float("-inf"), True)])
def test_beam_descent_matches_oracle(hdc, orc, cuda, dim, kmer, n_leaves, beam, threshold, childless, grouped):
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
    for grouped in (0, 1):
        ctx.option(H.BEAM_GROUPED, grouped)
        for threshold in (0.0, float("-inf")):
            res = ctx.beam_search(q8, qn, proto, pn, torch.from_numpy(ptr).to(cuda), d_idx, roots, 6, 5, threshold)
            out.append([x.cpu().numpy() for x in res])
    torch.cuda.synchronize()
    for a, b_ in zip(out[:2], out[2:]):
        for x, y in zip(a, b_):
            assert np.array_equal(x, y)
    assert (out[3][2] == 6).all()  # no early stop: every read reaches a leaf
