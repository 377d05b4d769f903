"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's unmodified CPU sources (src/HV.cpp, src/encoder.cpp of
benlaflen/bacterial-classification), compiled per configuration by
oracle/build_ref.sh with oracle/ref_driver.cpp as the front end, on seeded
synthetic inputs, and stores what they return:

  base      the four base hypervectors (A,C,G,T) as uint64 words
  binder    cache.kmers[kmer] for homopolymers, palindromes and random k-mers
  encode    HVCache::get(seq) for random sequences, sequences holding N /
            lowercase / other bytes, and the edge lengths 0, k-1, k, k+1
  windows   HVCache::get(seq.substr(w*step, L)) for every window
  topk      the reference cosine (NORM_COSINE) ranked (score desc, index asc)
  cosine    cosine() of HV pairs, including zero-norm vectors
  simtest   the eight 30-mers of tests/sim-test.cpp, all pairs (D=10000, k=5)

Needs the reference checkout; run from the repo root:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import random
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as B  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# (dim, kmer, window, step, store_full_hvs)
CONFIGS = [
    (10000, 5, 125, 10, True),   # the reference's own config.h
    (1024, 8, 150, 10, True),
    (200, 3, 20, 5, True),       # dim not a multiple of 64
    (8192, 8, 150, 10, False),   # plain-form shape (configs 1-2)
    (10240, 10, 250, 10, False),  # precision-form shape (configs 3-4)
    (16384, 12, 250, 10, False),  # hierarchical shape (config 5)
]

SIMTEST = [
    "AAAAAAAAAAAAAAAAAAAAAAAAAAAAAA", "AAGAAGAAGAAGAAGAAGAAGAAGAAGAAG",
    "GAGAAGAGAAGAGAAGAGAAGAGAAGAGAA", "GAGAGAGAGAGAGAGAGAGAGAGAGAGAGA",
    "GAGGAGAGGAGAGGAGAGGAGAGGAGAGGA", "GGAGGAGGAGGAGGAGGAGGAGGAGGAGGA",
    "GGAGGGGAGGGGAGGGGAGGGGAGGGGAGG", "GGGGGGGGGGGGGGGGGGGGGGGGGGGGGG",
]


def rseq(rng, n, alphabet="ACGT"):
    return "".join(rng.choice(alphabet) for _ in range(n))


def mutate(rng, s, rate):
    out = list(s)
    for i in range(len(out)):
        if rng.random() < rate:
            out[i] = rng.choice([c for c in "ACGT" if c != out[i]])
    return "".join(out)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run(exe, *args):
    subprocess.check_call([exe] + [str(a) for a in args])


def sequences_for(rng, k, window):
    seqs = [rseq(rng, rng.randint(k + 2, 3 * window)) for _ in range(10)]
    seqs.append("")
    seqs.append(rseq(rng, k - 1) if k > 1 else "")
    seqs.append(rseq(rng, k))
    seqs.append(rseq(rng, k + 1))
    seqs.append("A" * (window + 7))
    seqs.append(("ACGT" * window)[: window + 3])
    s = list(rseq(rng, 2 * window))
    for pos in rng.sample(range(len(s)), 6):
        s[pos] = rng.choice("NnacgtRY-")
    seqs.append("".join(s))
    seqs.append(rseq(rng, window).lower() + rseq(rng, window))
    return seqs


def make_config(dim, k, window, step, full, tmp):
    exe = B.build_ref(dim, k, window, step)
    rng = random.Random(1000 * dim + k)
    W = (dim + 63) // 64
    res = {"dim": dim, "kmer": k, "window": window, "step": step}
    arrays = {}

    run(exe, "base", f"{tmp}/base.bin")
    base = np.fromfile(f"{tmp}/base.bin", np.uint64).reshape(4, W)
    arrays["base_head"] = base[:, :4].copy()
    arrays["base_tail"] = base[:, -2:].copy()
    res["base_sha"] = sha(base)

    kmers = ["A" * k, "T" * k, "C" * k, "G" * k, ("AC" * k)[:k], ("ACGT" * k)[:k], ("TG" * k)[:k]]
    kmers += [rseq(rng, k) for _ in range(24)]
    with open(f"{tmp}/k.txt", "w") as f:
        f.write("\n".join(kmers) + "\n")
    run(exe, "binder", f"{tmp}/k.txt", f"{tmp}/b.bin")
    binders = np.fromfile(f"{tmp}/b.bin", np.uint64).reshape(len(kmers), W)
    res["binder_kmers"] = kmers
    res["binder_sha"] = [sha(b) for b in binders]
    if full:
        arrays["binders"] = binders

    seqs = sequences_for(rng, k, window)
    with open(f"{tmp}/s.txt", "w") as f:
        f.write("\n".join(seqs) + "\n")
    run(exe, "encode", f"{tmp}/s.txt", f"{tmp}/e.bin")
    enc = np.fromfile(f"{tmp}/e.bin", np.int16).reshape(len(seqs), dim)
    res["encode_seqs"] = seqs
    res["encode_sha"] = [sha(e) for e in enc]
    if full:
        arrays["encode"] = enc
    else:
        arrays["encode_head"] = enc[:, :64].copy()

    wseqs = [rseq(rng, window + step * rng.randint(0, 4) + rng.randint(0, step - 1)) for _ in range(3)]
    with open(f"{tmp}/w.txt", "w") as f:
        f.write("\n".join(wseqs) + "\n")
    run(exe, "windows", f"{tmp}/w.txt", f"{tmp}/w.bin")
    win = np.fromfile(f"{tmp}/w.bin", np.int16).reshape(-1, dim)
    res["window_seqs"] = wseqs
    res["windows_sha"] = [sha(w) for w in win]

    # top-k: references are noisy relatives of a few roots, queries are
    # mutated windows of the references (so the ranking is informative)
    roots = [rseq(rng, 3 * window) for _ in range(3)]
    refs = [mutate(rng, roots[i % 3], 0.03 * (1 + i // 3)) for i in range(12)]
    refs.append(refs[0])  # an exact duplicate: a tie broken by the lower index
    queries = []
    for i in range(8):
        r = refs[rng.randrange(len(refs))]
        st = rng.randint(0, len(r) - window)
        queries.append(mutate(rng, r[st: st + window], 0.01))
    with open(f"{tmp}/q.txt", "w") as f:
        f.write("\n".join(queries) + "\n")
    with open(f"{tmp}/r.txt", "w") as f:
        f.write("\n".join(refs) + "\n")
    run(exe, "topk", f"{tmp}/q.txt", f"{tmp}/r.txt", 5, f"{tmp}/t.txt")
    rows = [l.split() for l in open(f"{tmp}/t.txt").read().splitlines()]
    res["topk_queries"] = queries
    res["topk_refs"] = refs
    res["topk_idx"] = [[int(r[2]) for r in rows if int(r[0]) == q] for q in range(len(queries))]
    res["topk_score"] = [[float(r[3]) for r in rows if int(r[0]) == q] for q in range(len(queries))]

    # cosine of raw int16 pairs, including a zero vector and extreme values
    a = np.random.default_rng(dim).integers(-300, 300, (6, dim)).astype(np.int16)
    b = np.random.default_rng(dim + 1).integers(-300, 300, (6, dim)).astype(np.int16)
    a[1] = 0
    b[2] = a[2]
    b[3] = -a[3]
    a[4] = 32767
    b[4] = -32768
    a.tofile(f"{tmp}/ca.bin")
    b.tofile(f"{tmp}/cb.bin")
    run(exe, "cosine", f"{tmp}/ca.bin", f"{tmp}/cb.bin", len(a), f"{tmp}/c.txt")
    arrays["cos_a"] = a
    arrays["cos_b"] = b
    res["cosine"] = [float(x) for x in open(f"{tmp}/c.txt").read().split()]

    name = f"ref_D{dim}_k{k}_L{window}_s{step}"
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)
    with open(os.path.join(OUT, name + ".json"), "w") as f:
        json.dump(res, f, indent=0)
    return name


def make_simtest(tmp):
    exe = B.build_ref(10000, 5, 125, 10)
    with open(f"{tmp}/s.txt", "w") as f:
        f.write("\n".join(SIMTEST) + "\n")
    run(exe, "encode", f"{tmp}/s.txt", f"{tmp}/e.bin")
    enc = np.fromfile(f"{tmp}/e.bin", np.int16).reshape(len(SIMTEST), 10000)
    n = len(SIMTEST)
    a = np.repeat(enc, n, axis=0)
    b = np.tile(enc, (n, 1))
    a.tofile(f"{tmp}/a.bin")
    b.tofile(f"{tmp}/b.bin")
    run(exe, "cosine", f"{tmp}/a.bin", f"{tmp}/b.bin", n * n, f"{tmp}/c.txt")
    cos = [float(x) for x in open(f"{tmp}/c.txt").read().split()]
    with open(os.path.join(OUT, "simtest_D10000_k5.json"), "w") as f:
        json.dump({"seqs": SIMTEST, "encode_sha": [sha(e) for e in enc], "cosine": cos}, f, indent=0)


def main():
    if not B.reference_available():
        sys.exit("reference checkout not found: golden vectors come from the reference itself")
    with tempfile.TemporaryDirectory() as tmp:
        for cfg in CONFIGS:
            print("golden:", make_config(*cfg, tmp))
        make_simtest(tmp)
        print("golden: simtest")


if __name__ == "__main__":
    main()
