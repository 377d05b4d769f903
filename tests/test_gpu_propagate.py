"""propagate-children on the GPU against the oracle: greedy representative
selection (decisions and best scores bit-exact) and the bundling of parents
as the sum of their children."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tree_parents(n_leaves, b):
    """Parents of every internal rank with their descendant leaves in order,
    for the tree layout of hdc_synth_tree (node j of rank r has parent j // b)."""
    groups = []
    for r in range(1, 6):  # ranks p..g hold the leaves' ancestors
        span = b ** (6 - r)
        n_nodes = (n_leaves + span - 1) // span
        for j in range(n_nodes):
            groups.append(list(range(j * span, min(n_leaves, (j + 1) * span))))
    return groups


@pytest.mark.parametrize("dim,kmer,n_leaves,threshold", [(1024, 8, 64, 0.75), (2048, 5, 81, 0.75),
                                                          (1000, 8, 30, 0.2)])
def test_greedy_matches_oracle(hdc, orc, cuda, dim, kmer, n_leaves, threshold):
    import torch
    H = hdc
    tree = H.synth_tree(31 + n_leaves, n_leaves)
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    ctx = H.Context(dim, kmer, 150, 10)
    hv = torch.empty((n_leaves, dim), dtype=torch.int16, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), hv, H.OUT_I16, tree.max_len())
    norm2 = ctx.norms(hv)
    groups = _tree_parents(n_leaves, b)
    # some parents already hold sequences (a re-run of the reference appends to them)
    reps = [g[::7][:2] if i % 3 == 0 else [] for i, g in enumerate(groups)]
    cand_ptr = np.zeros(len(groups) + 1, np.int64)
    cand_ptr[1:] = np.cumsum([len(g) for g in groups])
    rep_ptr = np.zeros(len(groups) + 1, np.int64)
    rep_ptr[1:] = np.cumsum([len(r) for r in reps])
    cand_idx = np.array([x for g in groups for x in g], np.int32)
    rep_idx = np.array([x for r in reps for x in r] or [0], np.int32)
    t = lambda a: torch.from_numpy(a).to(cuda)
    sel, best = ctx.propagate_greedy(hv, norm2, t(cand_ptr), t(cand_idx), t(rep_ptr), t(rep_idx), threshold)
    torch.cuda.synchronize()
    sel, best = sel.cpu().numpy().astype(bool), best.cpu().numpy()
    hv_np = hv.cpu().numpy()
    ref_hv, _ = orc.encode([tree.get(i) for i in range(n_leaves)], dim, kmer, "int16")
    assert np.array_equal(hv_np, ref_hv)
    n_sel = 0
    for p, g in enumerate(groups):
        o_sel, o_best = orc.propagate_greedy(hv_np[reps[p]] if reps[p] else [], hv_np[g], threshold)
        a, z = cand_ptr[p], cand_ptr[p + 1]
        assert np.array_equal(sel[a:z], o_sel), p
        assert np.array_equal(best[a:z], o_best), p
        n_sel += int(o_sel.sum())
    assert 0 < n_sel < len(cand_idx)  # the threshold actually splits the candidates


def test_bundle_tree_levels(hdc, orc, cuda):
    """Internal-node prototypes: each parent is the exact int32 sum of its
    children, built bottom-up rank by rank."""
    import torch
    H = hdc
    n_leaves, b, dim = 100, 3, 512
    tree = H.synth_tree(5, n_leaves)
    ctx = H.Context(dim, 8, 150, 10)
    level = torch.empty((n_leaves, dim), dtype=torch.int32, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), level, H.OUT_I32, tree.max_len())
    host = level.cpu().numpy()
    n = n_leaves
    while n > 1:
        npar = (n + b - 1) // b
        ptr = np.array([min(n, i * b) for i in range(npar + 1)], np.int64)
        idx = np.arange(n, dtype=np.int32)
        level = ctx.bundle(level, torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda))
        host = orc.bundle(host, ptr, idx)
        assert np.array_equal(level.cpu().numpy(), host)
        n = npar


@pytest.mark.parametrize("dim,kmer", [(1024, 8), (2048, 10)])
def test_greedy_scored_equals_sequential(hdc, cuda, dim, kmer):
    """The scored form (pair scores in bulk, then the decisions in order from running
    maxima) against the sequential form (each decision's dots computed as it is made):
    identical decisions and best scores, for parents of 2,600 candidates (three blocks of
    1,024), 1,100 candidates with existing sequences (their columns and the earlier
    blocks' appended candidates in the fixed-column tiles), block-edge sizes 1,024 and
    1,025, single candidates, an empty parent, and thresholds that select some, all
    (2.0) or none (-2.0) of them."""
    import torch
    H = hdc
    n_leaves = 2600
    tree = H.synth_tree(77, n_leaves)
    ctx = H.Context(dim, kmer, 150, 10)
    hv = torch.empty((n_leaves, dim), dtype=torch.int16, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), hv, H.OUT_I16, tree.max_len())
    norm2 = ctx.norms(hv)
    groups = [list(range(n_leaves)), list(range(0, n_leaves, 2))[:1100], list(range(7)), list(range(40, 73)), [9],
              [], list(range(1024)), list(range(500, 1525)), list(range(2599, 1500, -1))]
    reps = [[], [5, 17, 901], [3], [], [1, 2], [4], [], [0, 1, 2, 3], []]
    cand_ptr = np.zeros(len(groups) + 1, np.int64)
    cand_ptr[1:] = np.cumsum([len(g) for g in groups])
    rep_ptr = np.zeros(len(groups) + 1, np.int64)
    rep_ptr[1:] = np.cumsum([len(r) for r in reps])
    cand_idx = np.array([x for g in groups for x in g], np.int32)
    rep_idx = np.array([x for r in reps for x in r], np.int32)
    t = lambda a: torch.from_numpy(a).to(cuda)
    for threshold in (0.75, 0.9, 2.0, -2.0):
        out = []
        for form in (0, 1):
            ctx.option(H.GREEDY_FORM, form)
            sel, best = ctx.propagate_greedy(hv, norm2, t(cand_ptr), t(cand_idx), t(rep_ptr), t(rep_idx), threshold)
            torch.cuda.synchronize()
            out.append((sel.cpu().numpy(), best.cpu().numpy()))
        assert ctx.status() == 0
        assert np.array_equal(out[0][0], out[1][0]), threshold
        assert np.array_equal(out[0][1], out[1][1]), threshold
        if threshold == 0.75:
            assert 0 < out[0][0].sum() < len(cand_idx)
        if threshold == 2.0:
            assert out[0][0].all()
        if threshold == -2.0:
            assert not out[0][0].any()
