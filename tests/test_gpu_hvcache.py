"""The GPU-backed encoder.h drop-in (dropin/encoder.h, encoder_gpu.cpp):
class HVCache with the reference's interface, driven through that interface
by dropin/hvcache_selftest.cpp, against the oracle -- get() is
HVCache::compute (also after evictions, with a cache of 3 entries),
precompute() then get() of every window gives each window's compute,
similarity() gives HVCache::similarity's position and score, and kmers[]
holds the binder of each k-mer's canonical form."""
import os
import random
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIM, K, L, STEP = 1024, 8, 150, 10


def _selftest(hdc, tmp, seqs, pairs, kmers, capacity):
    import build as pkg_build
    out = pkg_build.build_dropin(DIM, K, L, STEP)
    for name, rows in (("seqs.txt", seqs), ("pairs.txt", ["%d %d" % p for p in pairs]), ("kmers.txt", kmers)):
        with open(os.path.join(tmp, name), "w") as f:
            f.write("\n".join(rows) + "\n")
    pre = os.path.join(tmp, "out%d" % capacity)
    r = subprocess.run([os.path.join(out, "hvcache_selftest")] + [os.path.join(tmp, n) for n in
                                                                  ("seqs.txt", "pairs.txt", "kmers.txt")] +
                       [str(capacity), pre], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["kmers", str(4 ** K)]
    return pre


@pytest.mark.parametrize("capacity", [3, 100000])
def test_hvcache_drop_in_matches_oracle(hdc, orc, cuda, capacity):
    rng = random.Random(17)
    base = ["".join(rng.choice("ACGT") for _ in range(n)) for n in (1500, 600, 400)]
    seqs = [base[0], base[1], base[2], base[0][100:250], base[0][300:450] + "N" + base[0][451:460],
            "acgt" + base[1][:146], "", "ACGTACG", base[2][:L], base[2][:L + STEP], base[1][:L + 1]]
    seqs += [base[rng.randrange(3)][a:a + rng.choice((L, 120, 300))] for a in range(0, 200, 23)]
    pairs = [(q, r) for q in (3, 4, 5, 12) for r in range(len(seqs))]
    kmers = ["A" * K, "T" * K, "ACGTACGT"[:K], "GGGCCCAA"[:K], base[0][:K], base[1][7:7 + K]]
    with tempfile.TemporaryDirectory() as tmp:
        pre = _selftest(hdc, tmp, seqs, pairs, kmers, capacity)
        got = np.fromfile(pre + ".get.bin", np.int16).reshape(-1, DIM)
        want, _ = orc.encode(seqs, DIM, K, "int16")
        assert np.array_equal(got, np.concatenate([want, want]))
        wins = [s[x:x + L] for s in seqs if len(s) >= L for x in range(0, len(s), STEP) if x == 0 or x + L < len(s)]
        got = np.fromfile(pre + ".windows.bin", np.int16).reshape(-1, DIM)
        want, _ = orc.encode(wins, DIM, K, "int16")
        assert np.array_equal(got, want)
        rows, ptr, whole = orc.similarity_rows(seqs, L, STEP)
        q, _ = orc.encode(seqs, DIM, K, "int16")
        rv, _ = orc.encode(rows, DIM, K, "int16") if rows else (np.zeros((0, DIM), np.int16), None)
        ws, ww = orc.similarity(q, rv, ptr, whole, [p[0] for p in pairs], [p[1] for p in pairs], orc.SCORE_NORM)
        lines = open(pre + ".sim.txt").read().split("\n")[:-1]
        assert len(lines) == len(pairs)
        for (pos, score), s_, w_ in zip((l.split() for l in lines), ws, ww):
            assert int(pos) == (max(int(w_), 0) * STEP)
            assert np.float32(float(score)) == s_
        got = np.fromfile(pre + ".kmers.bin", np.uint64).reshape(len(kmers), -1)
        for row, km in zip(got, kmers):
            assert np.array_equal(row, orc.binder(DIM, K, orc.canonical(km)))


def test_binders_entry_point_matches_oracle(hdc, orc, cuda):
    for dim, k in ((1024, 8), (200, 3), (10240, 10)):
        ctx = hdc.Context(dim, k, 150, 10)
        codes = np.array([0, 1, 4 ** k - 1, 12345 % 4 ** k, 4 ** k // 3], np.int64)
        got = ctx.binders(codes)
        for c, row in zip(codes, got):
            assert np.array_equal(row, orc.binder(dim, k, int(c)))
        with pytest.raises(hdc.HDCError):
            ctx.binders([4 ** k])
