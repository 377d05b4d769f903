"""Batching form: the CUDA-graph pipeline (length-binned encode -> tensor-core
search -> top-k) on reads of uneven length with indels and N bases, checked
against the oracle's encode + brute-force ranking (bipolar queries); results
must not change after autotuning or on replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pipeline_matches_oracle_and_survives_autotune(hdc, orc, cuda):
    import torch
    H = hdc
    dim, kmer, K = 2048, 10, 10
    tree = H.synth_tree(17, 300)
    reads = H.synth_reads(18, tree, 700, 250, subst=0.01, sigma=0.5, min_read=100, max_read=1600,
                          mixed_frac=0.2, mixed_rate=0.06)
    # a few reads with N bases and one shorter than k
    buf = reads.buf.copy()
    for i in range(0, 700, 97):
        buf[reads.off[i] + 5] = ord("N")
    reads = H.Seqs(buf, reads.off, reads.len.copy(), reads.label)
    reads.len[3] = 5
    ctx = H.Context(dim, kmer, 250, 10)
    refs = torch.empty((len(tree), dim), dtype=torch.int16, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), refs, H.OUT_I16, tree.max_len())
    db = ctx.refdb(refs, int(refs.abs().max().item()))
    total = int(reads.len.astype(np.int64).sum())
    pipe = H.Pipeline(ctx, db, 1024, total + 4096, 1600, K)
    s1, i1 = pipe.run(reads)
    o_s, o_i = orc.classify([reads.get(j) for j in range(len(reads))], refs.cpu().numpy(), dim, kmer, K,
                            orc.SCORE_NORM, bipolar=True)
    assert np.array_equal(i1, o_i)
    assert np.array_equal(s1, o_s)
    best = pipe.autotune()
    assert best["tile_n"] in (128, 256)
    s2, i2 = pipe.run(reads)
    assert np.array_equal(i2, i1) and np.array_equal(s2, s1)
    pipe.launch_resident()
    torch.cuda.synchronize()
    s3, i3 = pipe.run(reads)  # a replay after a resident launch gives the same answer
    assert np.array_equal(i3, i1)
    assert ctx.status() == 0
