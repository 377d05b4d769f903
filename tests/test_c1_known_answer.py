"""The plain method at full size against the reference's own answers
(tests/golden/c1_known_answer.json, made by tests/golden/make_c1_golden.py
from the compiled reference): 2,000 references, D = 8,192, k = 8, 10,000
reads of 150 bp, top-5 by cosine (NORM scale).

  * CPU: the oracle on the first 1,000 reads gives the reference's indices
    and float scores (pins the oracle at this size);
  * GPU: the GPU encoder + the plain drop-in search (hdc_search_plain) on all
    10,000 reads, and the precision form on the same count-valued reads
    (hdc_search_tc against a database whose limbs are sized for counts up to
    143), give the reference's indices and float scores for every read."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_c1_golden import C1, digests, workload  # noqa: E402

GOLD = json.load(open(os.path.join(HERE, "golden", "c1_known_answer.json")))


def _synth():
    import build as pkg_build
    pkg_build.build_synth()
    import hdc_synth
    return hdc_synth


def test_golden_matches_its_workload_definition():
    assert GOLD["workload"] == C1
    assert len(GOLD["chunks"]) == C1["n_reads"] // C1["chunk"]


def test_c1_oracle_first_chunk(orc):
    S = _synth()
    tree, reads = workload(S)
    refs = orc.encode_bundles(tree.buf, tree.off, tree.len, C1["dim"], C1["kmer"], 1).astype(np.int16)
    n = C1["chunk"]
    seqs = [reads.get(i) for i in range(n)]
    s, i = orc.classify(seqs, refs, C1["dim"], C1["kmer"], C1["k"], orc.SCORE_NORM)
    d = digests(i, s)
    assert d["chunks"][0] == GOLD["chunks"][0]
    assert np.array_equal(i[:8], np.array(GOLD["first_rows"]["idx"]))


@pytest.mark.gpu
def test_c1_gpu_plain_and_precision_forms_all_reads(hdc, cuda):
    import torch
    H = hdc
    S = _synth()
    tree, reads = workload(S)
    dim, kmer, k = C1["dim"], C1["kmer"], C1["k"]
    ctx = H.Context(dim, kmer, C1["window"], C1["step"])
    refs = torch.empty((len(tree), dim), dtype=torch.int16, device=cuda)
    ctx.encode_segments(torch.from_numpy(tree.buf).to(cuda), torch.from_numpy(tree.off).to(cuda),
                        torch.from_numpy(tree.len).to(cuda), refs, H.OUT_I16, tree.max_len())
    q = torch.empty((len(reads), dim), dtype=torch.int16, device=cuda)
    rb, ro, rl = (torch.from_numpy(x).to(cuda) for x in (reads.buf, reads.off, reads.len))
    ctx.encode_segments(rb, ro, rl, q, H.OUT_I16, reads.max_len())
    mq = torch.zeros(1, dtype=torch.int32, device=cuda)
    mr = torch.zeros(1, dtype=torch.int32, device=cuda)
    qn, rn = ctx.norms(q, mq), ctx.norms(refs, mr)
    torch.cuda.synchronize()
    s, i, _, _ = ctx.search_plain(q, qn, int(mq.item()), refs, rn, int(mr.item()), k, H.SCORE_NORM)
    torch.cuda.synchronize()
    d = digests(i.cpu().numpy(), s.cpu().numpy())
    for key in ("idx_sha256", "score_sha256", "top1_sha256", "chunks"):
        assert d[key] == GOLD[key], key
    # precision form: the same count-valued reads as fp16 on the tensor cores
    maxq = C1["read_len"] - kmer + 1
    db = ctx.refdb(refs, int(mr.item()), max_query_abs=maxq)
    q16 = torch.empty((len(reads), dim), dtype=torch.float16, device=cuda)
    ctx.encode_segments(rb, ro, rl, q16, H.OUT_F16, reads.max_len())
    ts, ti, _, _ = ctx.search_tc(db, q16, qn, maxq, k, H.SCORE_NORM)
    torch.cuda.synchronize()
    assert ctx.status() == 0
    d = digests(ti.cpu().numpy(), ts.cpu().numpy())
    for key in ("idx_sha256", "score_sha256", "chunks"):
        assert d[key] == GOLD[key], key
