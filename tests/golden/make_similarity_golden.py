"""Golden vectors for HVCache::similarity (src/encoder.cpp:198-215): the
reference driver (oracle/ref_driver.cpp, built by oracle/build_ref.sh from
the reference's own HV.cpp/encoder.cpp) scores every (query, reference) pair
with windows of compute semantics (no precompute).  References cover the
edges of the window rule: shorter than k, shorter than / equal to / one past
the window, exactly one step past it (the strict x + L < len drops that
window), long sequences, N and lowercase bases.  Run from the repo root:
    python tests/golden/make_similarity_golden.py"""
import json
import os
import random
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.build import build_ref  # noqa: E402

CONFIGS = [(1024, 8, 150, 10), (200, 3, 20, 5)]


def mutate(rng, s, n):
    s = list(s)
    for p in rng.sample(range(len(s)), min(n, len(s))):
        s[p] = rng.choice("ACGT".replace(s[p], "") if s[p] in "ACGT" else "ACGT")
    return "".join(s)


def cases(L, step, k, seed):
    rng = random.Random(seed)
    root = "".join(rng.choice("ACGT") for _ in range(12 * L))
    lens = [0, k - 1, L // 2, L - 1, L, L + 1, L + step - 1, L + step, L + step + 1, L + 2 * step, 3 * L, 10 * L]
    refs = []
    for i, n in enumerate(lens):
        start = rng.randrange(0, len(root) - n + 1)
        refs.append(mutate(rng, root[start:start + n], n // 50))
    long = refs[-1]
    refs.append(long[: 2 * L] + "N" * 3 + long[2 * L + 3: 4 * L])  # N bases
    refs.append(long[L: 3 * L].lower())                               # lowercase
    refs.append("".join(rng.choice("ACGT") for _ in range(4 * L)))     # unrelated
    queries = []
    for n in (L, L // 2, L + L // 2):
        start = rng.randrange(0, len(long) - n + 1)
        queries.append(mutate(rng, long[start:start + n], max(1, n // 60)))
    queries.append("".join(rng.choice("ACGT") for _ in range(L)))
    q = list(queries[0])
    q[L // 3] = "N"
    queries.append("".join(q))
    return queries, refs


def main():
    out = []
    for dim, k, L, step in CONFIGS:
        exe = build_ref(dim, k, L, step)
        queries, refs = cases(L, step, k, 1000 + dim)
        with tempfile.TemporaryDirectory() as tmp:
            qf, rf, of = (os.path.join(tmp, n) for n in ("q.txt", "r.txt", "o.txt"))
            open(qf, "w").write("\n".join(queries) + "\n")
            open(rf, "w").write("\n".join(refs) + "\n")
            subprocess.check_call([exe, "similarity", qf, rf, of])
            rows = [l.split() for l in open(of).read().splitlines()]
        res = [[int(a), int(b), float(c), int(d)] for a, b, c, d in rows]
        out.append(dict(dim=dim, kmer=k, window=L, step=step, queries=queries, refs=refs, results=res))
        print(dim, k, L, step, len(res), "pairs")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "similarity.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()
