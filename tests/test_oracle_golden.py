"""The CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py runs the reference's src/HV.cpp and
src/encoder.cpp).  Bit-exact for every integer output; the float cosine
scores are compared exactly as well (same double expression, same cast)."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CONFIGS = sorted(glob.glob(os.path.join(GOLD, "ref_D*.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(path):
    meta = json.load(open(path))
    arr = np.load(path[:-5] + ".npz")
    return meta, arr


def test_mt19937_64_known_answer(orc):
    # C++ standard [rand.predef]: the 10000th output of a default-constructed
    # mt19937_64 (seed 5489) is 9981545732273789042.
    assert int(orc.mt64_stream(5489, 10000)[-1]) == 9981545732273789042


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_base_hvs(orc, path):
    meta, arr = load(path)
    base = orc.base_hvs(meta["dim"])
    assert sha(base) == meta["base_sha"]
    assert (base[:, :4] == arr["base_head"]).all()
    assert (base[:, -2:] == arr["base_tail"]).all()


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_binders(orc, path):
    meta, arr = load(path)
    for km, h in zip(meta["binder_kmers"], meta["binder_sha"]):
        b = orc.binder(meta["dim"], meta["kmer"], orc.canonical(km))
        assert sha(b) == h, km


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_encode(orc, path):
    meta, arr = load(path)
    enc, nk = orc.encode(meta["encode_seqs"], meta["dim"], meta["kmer"])
    assert [sha(e) for e in enc] == meta["encode_sha"]
    if "encode" in arr:
        assert (enc == arr["encode"]).all()


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_windows(orc, path):
    meta, arr = load(path)
    segs = orc.window_segments(meta["window_seqs"], meta["window"], meta["step"])
    enc, _ = orc.encode(segs, meta["dim"], meta["kmer"])
    assert [sha(e) for e in enc] == meta["windows_sha"]


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_topk(orc, path):
    meta, arr = load(path)
    q, _ = orc.encode(meta["topk_queries"], meta["dim"], meta["kmer"])
    r, _ = orc.encode(meta["topk_refs"], meta["dim"], meta["kmer"])
    s, i, c, d = orc.topk(q, r, 5, orc.SCORE_NORM)
    assert i.tolist() == meta["topk_idx"]
    assert np.array_equal(s, np.array(meta["topk_score"], np.float32))


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_cosine(orc, path):
    meta, arr = load(path)
    got = [orc.cosine(a, b) for a, b in zip(arr["cos_a"], arr["cos_b"])]
    assert np.array_equal(np.array(got, np.float32), np.array(meta["cosine"], np.float32))


def test_simtest_pairs(orc):
    """tests/sim-test.cpp: all pairs of eight 30-mers at the reference's own
    configuration (D=10000, k=5)."""
    meta = json.load(open(os.path.join(GOLD, "simtest_D10000_k5.json")))
    enc, _ = orc.encode(meta["seqs"], 10000, 5)
    assert [sha(e) for e in enc] == meta["encode_sha"]
    n = len(meta["seqs"])
    got = [orc.cosine(enc[i], enc[j]) for i in range(n) for j in range(n)]
    assert np.array_equal(np.array(got, np.float32), np.array(meta["cosine"], np.float32))
    for i in range(n):  # self-similarity prints 1.000000 in the reference
        assert got[i * n + i] == np.float32(1.0)


def test_fast_bundle_encoder_matches_oracle(orc):
    """The fast CPU encoder used only to build large reference sets for the
    CPU baseline equals the oracle's encoder bit for bit (and sums groups)."""
    import random
    rng = random.Random(9)
    seqs = ["".join(rng.choice("ACGT") for _ in range(rng.randint(0, 900))) for _ in range(40)]
    seqs += ["ACGTNNACGTacgtACGTACGTAGCTAGCTAGCT" * 5, "A" * 9, ""]
    buf, off, ln = orc.pack_segments(seqs)
    for dim, k in [(1024, 8), (200, 3), (2048, 10), (4096, 12), (512, 16)]:
        ref, _ = orc.encode(seqs, dim, k, "int32")
        assert np.array_equal(orc.encode_bundles(buf, off, ln, dim, k), ref), (dim, k)
    ref, _ = orc.encode(seqs[:40], 1024, 8, "int32")
    got = orc.encode_bundles(buf, off[:40], ln[:40], 1024, 8, group=8)
    assert np.array_equal(got, ref.reshape(5, 8, -1).sum(1))


SIM_GOLDEN = json.load(open(os.path.join(GOLD, "similarity.json")))


@pytest.mark.parametrize("g", SIM_GOLDEN, ids=lambda g: "D%d_k%d" % (g["dim"], g["kmer"]))
def test_similarity_matches_reference(orc, g):
    """HVCache::similarity over the oracle's window rows equals the
    reference's own similarity() (score bit-exact as float, position)."""
    rows, ref_rows, whole = orc.similarity_rows(g["refs"], g["window"], g["step"])
    q, _ = orc.encode(g["queries"], g["dim"], g["kmer"])
    r, _ = orc.encode(rows, g["dim"], g["kmer"])
    res = np.array(g["results"], dtype=np.float64)
    pq, pr = res[:, 0].astype(np.int64), res[:, 1].astype(np.int64)
    s, w = orc.similarity(q, r, ref_rows, whole, pq, pr)
    assert np.array_equal(s, res[:, 2].astype(np.float32))
    pos = np.where(w < 0, 0, w * g["step"])
    assert np.array_equal(pos, res[:, 3].astype(np.int64))
