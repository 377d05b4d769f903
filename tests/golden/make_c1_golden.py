"""Known answers of the plain method at full size (the CPU-runnable workload):
2,000 leaf references of a seeded 6-rank synthetic tree (1,400-1,600 bp), HV
dimension 8,192, k = 8, and 10,000 reads of 150 bp with 1 % substitutions;
every read encoded and ranked against every reference by cosine, top-5.

The answers come from the reference itself: its unmodified CPU sources
(src/HV.cpp, src/encoder.cpp: HVCache::get = compute, cosine with
NORM_COSINE), compiled by oracle/build_ref.sh 8192 8 150 10 with
oracle/ref_driver.cpp's `topk` command (brute force, order by score
descending, ties to the lower reference index).  The reads are split over
processes; each process encodes every reference itself.

Stored (tests/golden/c1_known_answer.json): the workload's parameters and
seeds, sha256 of the top-5 reference indices (int32, little endian) and of
their float scores (float32) per chunk of 1,000 reads and over all reads, the
top-1 indices' sha256, the first rows in clear, and the top-1 accuracy
against the generator's labels.  Needs the reference checkout; run from the
repo root:
    python tests/golden/make_c1_golden.py
"""
import concurrent.futures
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (ROOT, os.path.join(ROOT, "bacterial-classification_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

C1 = dict(n_leaves=2000, dim=8192, kmer=8, window=150, step=10, n_reads=10000, read_len=150, subst=0.01,
          tree_seed=1, read_seed=101, k=5, chunk=1000)
OUT = os.path.join(HERE, "c1_known_answer.json")


def workload(S, c=C1):
    """(references, reads) of the workload from the seeded generator (hdc_synth)."""
    tree = S.synth_tree(c["tree_seed"], c["n_leaves"])
    reads = S.synth_reads(c["read_seed"], tree, c["n_reads"], c["read_len"], subst=c["subst"])
    return tree, reads


def digests(idx, score, c=C1):
    """The stored digests of top-k indices [n][k] and float scores [n][k]."""
    idx = np.ascontiguousarray(idx, "<i4")
    score = np.ascontiguousarray(score, "<f4")
    h = lambda a: hashlib.sha256(a.tobytes()).hexdigest()
    ch = c["chunk"]
    return {"idx_sha256": h(idx), "score_sha256": h(score), "top1_sha256": h(np.ascontiguousarray(idx[:, 0])),
            "chunks": [{"first": a, "idx_sha256": h(idx[a:a + ch]), "score_sha256": h(score[a:a + ch])}
                       for a in range(0, idx.shape[0], ch)]}


def _run_shard(exe, refs_txt, reads, k, tmp, s):
    q = os.path.join(tmp, "q%d.txt" % s)
    out = os.path.join(tmp, "out%d.txt" % s)
    with open(q, "w") as f:
        f.write("\n".join(reads) + "\n")
    subprocess.check_call([exe, "topk", q, refs_txt, str(k), out], stderr=subprocess.DEVNULL)
    rows = np.loadtxt(out, dtype=np.float64, ndmin=2)
    n = len(reads)
    idx = np.full((n, k), -1, np.int32)
    score = np.zeros((n, k), np.float32)
    for qi, t, i, sc in rows:
        idx[int(qi), int(t)] = int(i)
        score[int(qi), int(t)] = np.float32(sc)
    return idx, score


def main():
    from oracle import build as B
    import build as pkg_build
    pkg_build.build_synth()
    import hdc_synth as S
    if not B.reference_available():
        sys.exit("reference checkout not found: the known answers come from the reference itself")
    c = C1
    exe = B.build_ref(c["dim"], c["kmer"], c["window"], c["step"])
    tree, reads = workload(S)
    seqs = [reads.get(i) for i in range(len(reads))]
    procs = max(1, os.cpu_count() or 1)
    with tempfile.TemporaryDirectory() as tmp:
        refs_txt = os.path.join(tmp, "refs.txt")
        with open(refs_txt, "w") as f:
            f.write("\n".join(tree.get(i) for i in range(len(tree))) + "\n")
        bounds = np.linspace(0, len(seqs), procs + 1).astype(int)
        with concurrent.futures.ThreadPoolExecutor(procs) as ex:
            parts = list(ex.map(lambda s: _run_shard(exe, refs_txt, seqs[bounds[s]:bounds[s + 1]], c["k"], tmp, s),
                                range(procs)))
    idx = np.concatenate([p[0] for p in parts])
    score = np.concatenate([p[1] for p in parts])
    assert (idx >= 0).all()
    doc = {"workload": c, "source": "reference src/HV.cpp + src/encoder.cpp (NORM_COSINE), oracle/ref_driver.cpp topk",
           "top1_accuracy": float((idx[:, 0] == reads.label).mean()),
           "first_rows": {"idx": idx[:8].tolist(), "score": [[float(x) for x in r] for r in score[:8]]}}
    doc.update(digests(idx, score))
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote %s (top-1 accuracy %.4f)" % (OUT, doc["top1_accuracy"]))


if __name__ == "__main__":
    main()
