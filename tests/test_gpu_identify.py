"""Windowed similarity (HVCache::similarity) and the identify descent with
the reference's own node scoring, on the GPU, against the reference's
similarity() golden vectors and the oracle's restatements: identical float
scores, window positions, paths, per-level scores and stop levels."""
import json
import os
import random

import numpy as np
import pytest

from test_gpu_beam import _tree_csr

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _encode(H, ctx, seqs, dim, dev):
    """int16 compute-semantics encodes of strings, and their squared norms."""
    import torch
    from oracle.oracle import pack_segments
    buf, off, lens = pack_segments(seqs)
    out = torch.zeros((max(len(seqs), 1), dim), dtype=torch.int16, device=dev)
    if seqs:
        ctx.encode_segments(torch.from_numpy(buf).to(dev), torch.from_numpy(off).to(dev),
                            torch.from_numpy(lens.astype(np.int32)).to(dev), out, H.OUT_I16, int(lens.max()))
    return out, ctx.norms(out)


def _similarity(H, orc, dev, dim, kmer, window, step, queries, refs, pq, pr):
    import torch
    ctx = H.Context(dim, kmer, window, step)
    rows, ref_rows, whole = orc.similarity_rows(refs, window, step)
    q, qn = _encode(H, ctx, queries, dim, dev)
    r, rn = _encode(H, ctx, rows, dim, dev)
    s, w = ctx.similarity(q, qn, r, rn, torch.from_numpy(ref_rows).to(dev), torch.from_numpy(whole).to(dev),
                          torch.from_numpy(np.asarray(pq, np.int32)).to(dev),
                          torch.from_numpy(np.asarray(pr, np.int32)).to(dev))
    torch.cuda.synchronize()
    return s.cpu().numpy(), w.cpu().numpy(), (q.cpu().numpy(), r.cpu().numpy(), ref_rows, whole)


@pytest.mark.parametrize("g", json.load(open(os.path.join(GOLD, "similarity.json"))),
                         ids=lambda g: "D%d_k%d" % (g["dim"], g["kmer"]))
def test_similarity_matches_reference(hdc, orc, cuda, g):
    res = np.array(g["results"], np.float64)
    pq, pr = res[:, 0].astype(np.int32), res[:, 1].astype(np.int32)
    s, w, _ = _similarity(hdc, orc, cuda, g["dim"], g["kmer"], g["window"], g["step"], g["queries"], g["refs"],
                          pq, pr)
    assert np.array_equal(s, res[:, 2].astype(np.float32))
    assert np.array_equal(np.where(w < 0, 0, w * g["step"]), res[:, 3].astype(np.int64))


def test_similarity_random_vs_oracle(hdc, orc, cuda):
    rng = random.Random(11)
    root = "".join(rng.choice("ACGT") for _ in range(3000))
    refs = [root[s:s + n] for s, n in ((rng.randrange(0, 1500), rng.randrange(50, 1500)) for _ in range(40))]
    queries = [root[s:s + 250] for s in (rng.randrange(0, 2700) for _ in range(24))]
    pq = np.repeat(np.arange(24), 40).astype(np.int32)
    pr = np.tile(np.arange(40), 24).astype(np.int32)
    s, w, (q, r, ref_rows, whole) = _similarity(hdc, orc, cuda, 4096, 10, 250, 10, queries, refs, pq, pr)
    ws, ww = orc.similarity(q, r, ref_rows, whole, pq, pr)
    assert np.array_equal(s, ws)
    assert np.array_equal(w, ww)


@pytest.mark.parametrize("dim,kmer,n_leaves,beam,threshold", [(1024, 8, 60, 5, 0.0), (2048, 10, 90, 3, 0.0),
                                                              (1024, 6, 40, 5, -2.0)])
def test_identify_matches_oracle(hdc, orc, cuda, dim, kmer, n_leaves, beam, threshold):
    """Nodes carry sequences (leaves: their two copies; internal nodes: one
    copy of every descendant leaf, some cut short; some nodes none) cut into
    similarity rows; reads descend with identify's scoring."""
    import torch
    H = hdc
    window, step = 150, 10
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    tree = H.synth_tree(300 + n_leaves, n_leaves)
    copies = H.synth_copies(301, tree, 2, 0.02)
    base, counts, ptr, idx = _tree_csr(n_leaves, b)
    n_nodes = int(base[-1])
    rng = random.Random(n_leaves)
    leaf_of = lambda node: [node - int(base[5])]
    desc = {}
    for node in range(n_nodes - 1, -1, -1):
        kids = idx[ptr[node]:ptr[node + 1]]
        desc[node] = leaf_of(node) if node >= base[5] else [x for c in kids for x in desc[int(c)]]
    node_seqs = []
    for node in range(n_nodes):
        if node >= base[5]:
            node_seqs.append([copies.get(2 * desc[node][0] + c) for c in range(2)])
        elif rng.random() < 0.1:
            node_seqs.append([])  # a node without sequences scores -1
        else:  # one copy of every descendant leaf, some cut short (whole-sequence rows)
            node_seqs.append([copies.get(2 * j)[:rng.choice([100, 150, 400, 2000, 2000, 2000])] for j in desc[node]])
    rows, node_rows = [], [0]
    for seqs in node_seqs:
        r, _, _ = orc.similarity_rows(seqs, window, step)
        rows.extend(r)
        node_rows.append(len(rows))
    node_rows = np.array(node_rows, np.int64)
    reads = H.synth_reads(302, copies, 48, 150, subst=0.01, sigma=0.3, min_read=80, max_read=300)
    ctx = H.Context(dim, kmer, window, step)
    q, qn = _encode(H, ctx, [reads.get(i) for i in range(len(reads))], dim, cuda)
    r, rn = _encode(H, ctx, rows, dim, cuda)
    roots = list(range(counts[0]))
    path, score, depth, stop = ctx.identify(q, qn, r, rn, torch.from_numpy(node_rows).to(cuda),
                                            torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda),
                                            torch.tensor(roots, dtype=torch.int32, device=cuda), 6, beam, threshold)
    torch.cuda.synchronize()
    want = orc.identify(q.cpu().numpy(), r.cpu().numpy(), node_rows, ptr, idx, roots, 6, beam, threshold)
    path, score, depth, stop = path.cpu().numpy(), score.cpu().numpy(), depth.cpu().numpy(), stop.cpu().numpy()
    assert any(s == -1 for _, _, s in want)  # some reads run every level
    for i, (wp, ws, wstop) in enumerate(want):
        assert depth[i] == len(wp), i
        assert list(path[i, :len(wp)]) == wp, i
        assert np.array_equal(score[i, :len(wp)], np.array(ws, np.float32)), i
        assert stop[i] == wstop, i
