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


@pytest.mark.parametrize("dim,kmer,n_leaves,beam,threshold", [(1024, 10, 200, 5, 0.0), (2048, 12, 300, 3, 0.0),
                                                              (1024, 8, 150, 5, 0.6)])
def test_beam_descent_matches_oracle(hdc, orc, cuda, dim, kmer, n_leaves, beam, threshold):
    import torch
    H = hdc
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    tree = H.synth_tree(41 + n_leaves, n_leaves)
    reads = H.synth_reads(42, tree, 64, 250, subst=0.01, sigma=0.5, min_read=100, max_read=800,
                          mixed_frac=0.2, mixed_rate=0.06)
    ctx = H.Context(dim, kmer, 250, 10)
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
