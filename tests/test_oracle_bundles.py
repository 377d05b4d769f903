"""CPU checks of the oracle's helpers for large workloads: the bundle-of-copies
encoder built from differences gives the rows of the direct encoder, and the
classify call's FP64 cosines and dots agree with its float scores."""
import numpy as np
import pytest


class _Seqs:
    def __init__(self, seqs):
        bs = [s.encode() for s in seqs]
        self.len = np.array([len(b) for b in bs], np.int64)
        self.off = np.zeros(len(bs), np.int64)
        self.off[1:] = np.cumsum(self.len)[:-1]
        self.buf = np.frombuffer(b"".join(bs) + b"\0" * 16, np.uint8).copy()


def _mutate(rng, s, rate, indel=False):
    out = []
    for ch in s:
        if rng.random() < rate:
            if indel and rng.random() < 0.3:
                if rng.random() < 0.5:
                    continue  # deletion
                out.append(rng.choice("ACGT"))  # insertion before the base
            else:
                ch = rng.choice([b for b in "ACGT" if b != ch])
        out.append(ch)
    return "".join(out)


@pytest.mark.parametrize("dim,k,group", [(1024, 8, 8), (200, 3, 3), (10240, 10, 2)])
def test_copy_bundles_equal_direct_bundles(orc, dim, k, group):
    import random
    rng = random.Random(dim + k)
    leaves = ["".join(rng.choice("ACGT") for _ in range(rng.randint(k - 1, 400))) for _ in range(12)]
    leaves[3] = leaves[3][:50] + "NNacgt" + leaves[3][50:]  # skipped k-mers in the leaf
    copies = []
    for i, s in enumerate(leaves):
        for c in range(group):
            # copy 0 of leaf 5 changes length (encoded whole); one copy is unchanged; others substitute
            copies.append(_mutate(rng, s, 0.05, indel=(i == 5 and c == 0)) if (i, c) != (2, 1) else s)
    ls, cs = _Seqs(leaves), _Seqs(copies)
    direct = orc.encode_bundles(cs.buf, cs.off, cs.len, dim, k, group, 2)
    delta = orc.encode_copy_bundles(ls, cs, group, dim, k, 3)
    assert np.array_equal(direct, delta)


def test_copy_bundles_reject_a_wrong_copy_count(orc):
    ls, cs = _Seqs(["ACGTACGTAC"]), _Seqs(["ACGTACGTAC"] * 3)
    with pytest.raises(ValueError):
        orc.encode_copy_bundles(ls, cs, 2, 64, 3)


def test_classify_exact_outputs_match_scores(orc):
    import random
    rng = random.Random(5)
    dim, k = 1024, 8
    refs_s = ["".join(rng.choice("ACGT") for _ in range(300)) for _ in range(40)]
    refs, _ = orc.encode(refs_s, dim, k, "int16")
    reads = [refs_s[rng.randrange(40)][a:a + 120] for a in (0, 30, 90, 150)]
    s, i = orc.classify(reads, refs, dim, k, 5)
    s2, i2, c, d = orc.classify(reads, refs, dim, k, 5, exact=True)
    assert np.array_equal(s, s2) and np.array_equal(i, i2)
    q, _ = orc.encode(reads, dim, k, "int16")
    dots = q.astype(np.int64) @ refs.astype(np.int64).T
    qn = (q.astype(np.int64) ** 2).sum(1)
    rn = (refs.astype(np.int64) ** 2).sum(1)
    for r in range(len(reads)):
        assert np.array_equal(d[r], dots[r, i[r]])
        want = dots[r, i[r]] / (np.sqrt(qn[r].astype(np.float64)) * np.sqrt(rn[i[r]].astype(np.float64)))
        assert np.array_equal(c[r], want)
        assert np.array_equal(s[r], orc.scores_from(d[r], qn[r], rn[i[r]]))
