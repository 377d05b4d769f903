"""Precision form: the tcgen05 tensor-core search against the CPU oracle and
the plain CUDA-core search.  Dots must be exact (int64 equal), labels and
order identical, float scores equal, FP64 cosines equal (the cosine error
against the FP64 oracle is therefore zero; the stated bound is 1e-12
relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(hdc, dev, refs, q_bipolar, dim):
    import torch
    ctx = hdc.Context(dim, 10, 250, 10)
    tr = torch.from_numpy(refs).to(dev)
    db = ctx.refdb(tr, int(np.abs(refs).max()))
    q16 = torch.from_numpy(q_bipolar.astype(np.float16)).to(dev)
    qi = torch.from_numpy(q_bipolar.astype(np.int16)).to(dev)
    qn = ctx.norms(qi)
    return ctx, db, tr, q16, qi, qn


def _run_tc(ctx, db, q16, qn, maxq, k, mode, tile_n=0, group=0, m_blocks=0, cluster=0, share=-1, pair=-1):
    import torch
    import hdc_gb300
    ctx.tc_tuning(group, -1, tile_n, m_blocks)
    ctx.tc_option(hdc_gb300.TC_CLUSTER, cluster)
    ctx.tc_option(hdc_gb300.TC_SHARE, share)
    ctx.tc_option(hdc_gb300.TC_PAIR_MMA, pair)
    s, i, c, d = ctx.search_tc(db, q16, qn, maxq, k, mode)
    torch.cuda.synchronize()
    assert ctx.status() == 0
    return s.cpu().numpy(), i.cpu().numpy(), c.cpu().numpy(), d.cpu().numpy()


# cluster 2, share 0: CTA pairs sharing reference blocks by multicast; groups of 3
# query tiles round down to 2, and odd tile counts leave a CTA of the last pair
# without a tile.  share 1: pairs sharing query blocks over two reference lanes
# (groups of 3 and 50 query tiles: 50 and 2 lanes).
@pytest.mark.parametrize("tile_n,group,m_blocks,cluster,share", [
    (128, 0, 1, 1, 0), (128, 0, 2, 1, 0), (256, 0, 1, 1, 0), (128, 3, 2, 1, 0), (128, 0, 1, 2, 0),
    (128, 3, 1, 2, 0), (128, 4, 1, 2, 0), (128, 0, 1, 2, 1), (128, 3, 1, 2, 1), (128, 50, 1, 2, 1)])
@pytest.mark.parametrize("dim,nq,nr,k,mode,vmax,dtype", [
    (1024, 200, 1000, 5, 0, 2000, np.int16),     # one fp16 limb (|v| <= 2048)
    (2048, 130, 3000, 10, 0, 12000, np.int16),   # two limbs (bundle of 8 copies)
    (1024, 300, 777, 1, 1, 12000, np.int16),     # argmax, COS scale, ragged sizes
    (512, 64, 500, 32, 2, 3000, np.int16),       # DOT scale, largest k
    (1024, 100, 600, 5, 0, 3000000, np.int32),   # two limbs, the top one above 1024
    (1024, 100, 600, 5, 0, 20000000, np.int32),  # three limbs (int32 internal-node sums)
    (640, 50, 400, 5, 0, 100000000, np.int32),   # three limbs, top limb ~ 24
    (10240, 129, 300, 5, 0, 12728, np.int16),    # precision-form dimension
])
def test_tc_vs_oracle(hdc, orc, cuda, dim, nq, nr, k, mode, vmax, dtype, tile_n, group, m_blocks, cluster, share):
    g = np.random.default_rng(dim + nq + nr)
    refs = g.integers(-vmax, vmax + 1, (nr, dim)).astype(dtype)
    refs[3] = refs[1]                       # tie: lower index first
    refs[4] = 0                             # zero norm
    refs[5, :] = vmax                       # extreme limbs
    refs[6, ::2] = -vmax
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    q[0] = np.where(refs[1] >= 0, 1, -1)    # a query aligned with reference 1
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    s, i, c, d = _run_tc(ctx, db, q16, qn, 1, k, mode, tile_n, group, m_blocks, cluster, share)
    os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), min(k, nr), mode)
    assert np.array_equal(i, oi)
    assert np.array_equal(d, od)
    assert np.array_equal(s, os_)
    assert np.array_equal(c, oc)


def test_tc_matches_plain_form(hdc, cuda):
    """Same bipolar queries and references through both GPU forms."""
    import torch
    g = np.random.default_rng(1)
    dim, nq, nr = 2048, 500, 4000
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    rn = ctx.norms(tr)
    a = ctx.search_plain(qi, qn, 1, tr, rn, 12000, 5, hdc.SCORE_NORM)
    b = ctx.search_tc(db, q16, qn, 1, 5, hdc.SCORE_NORM)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)


def test_tc_exact_worst_case_accumulators(hdc, orc, cuda):
    """Every query element +1 against limbs at their extremes: each per-limb
    accumulator reaches dim * 1024 (= 2^23 at dim 8192) with no rounding."""
    dim, nq, nr = 8192, 4, 130
    refs = np.full((nr, dim), -1024 + 2048 * 7, np.int16)   # low limb -1024, high limb 7
    refs[1] = 1023
    refs[2] = -1024
    refs[3] = 2047 * 5 + 1023
    q = np.ones((nq, dim), np.int8)
    q[1] = -1
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    s, i, c, d = _run_tc(ctx, db, q16, qn, 1, 5, hdc.SCORE_DOT, 256)
    os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), 5, orc.SCORE_DOT)
    assert np.array_equal(d, od) and np.array_equal(i, oi)


def _vector_with_sums(g, n, s1, s2):
    """An integer vector of length n with sum s1 and sum of squares s2 exactly:
    n - 3 random entries, then the last three from a perfect-square condition."""
    import math
    mean = s1 / n
    sd = math.sqrt(s2 / n - mean * mean)
    c = np.arange(-3 * int(sd), 3 * int(sd) + int(mean) + 1, dtype=np.int64)
    for _ in range(200):
        r = np.rint(g.normal(mean, sd, n - 3)).astype(np.int64)
        u1 = s1 - int(r.sum()) - c
        x = 2 * (s2 - int((r * r).sum()) - c * c) - u1 * u1
        ok = x >= 0
        s = np.floor(np.sqrt(np.where(ok, x, 0).astype(np.float64))).astype(np.int64)
        for dd in (-1, 0, 1):
            hit = ok & (s + dd >= 0) & ((s + dd) ** 2 == x) & (((u1 + s + dd) & 1) == 0)
            if hit.any():
                j = int(np.flatnonzero(hit)[0])
                sq = int(s[j] + dd)
                out = np.concatenate([r, [int(c[j]), (int(u1[j]) + sq) // 2, (int(u1[j]) - sq) // 2]])
                assert int(out.sum()) == s1 and int((out * out).sum()) == s2
                return out
    raise RuntimeError("no vector with these sums")


@pytest.mark.parametrize("mode", [0, 1])
def test_tc_scores_at_float_midpoints(hdc, orc, cuda, mode):
    """Cosines exactly on a midpoint between two floats, and their neighbours.

    With an all-ones query of dim 4096 (sqrt(nq) = 64) and references of norm2
    4^21 (sqrt = 2^21) the cosine is dot / 2^27 exactly, so dots can place it (or
    NORM's c - 0.5) on a float midpoint, where the reference's rounding ties to
    even and the search's reciprocal-product score must defer to the exact
    divide; the neighbours (dot +- 2) take the fast path.  Negated queries give
    the mirrored cosines."""
    g = np.random.default_rng(21)
    dim = 4096
    mids = [2**26 + 4, 2**26 + 12, 3 * 2**25 + 2, 3 * 2**25 + 6, 2**25 - 2]
    dots = mids + [x + d for x in mids for d in (-2, 2)]
    refs = np.stack([_vector_with_sums(g, dim, x, 4**21) for x in dots]).astype(np.int32)
    q = np.ones((2, dim), np.int8)
    q[1] = -1
    # the construction: COS 0.5 + 2^-25 ties down to 0.5, NORM 2 (0.25 + 2^-26) to 0.5
    assert np.float32(mids[0] / 2.0**27) == np.float32(0.5)
    assert np.float32(2 * (mids[2] / 2.0**27 - 0.5)) == np.float32(0.5)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    k = len(dots)
    s, i, c, d = _run_tc(ctx, db, q16, qn, 1, k, mode)
    os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), k, mode)
    assert np.array_equal(d, od) and np.array_equal(i, oi)
    assert np.array_equal(s.view(np.uint32), os_.view(np.uint32))
    assert np.array_equal(c, oc)


def test_tc_rejects_inexact_range(hdc, cuda):
    import torch
    dim = 16384 + 64
    refs = np.full((8, dim), 2000, np.int16)    # one limb of 2000: 16448 * 2000 > 2^24
    q = np.ones((2, dim), np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    with pytest.raises(hdc.HDCError) as e:
        ctx.search_tc(db, q16, qn, 1, 1)
    assert e.value.status == 2


def test_tc_encoded_bipolar_reads(hdc, orc, cuda):
    """End to end: bundled references (8 noisy copies) and bipolar reads encoded
    on the GPU, searched on the tensor cores, checked against the oracle's
    encode + brute-force ranking of the same sequences."""
    import torch
    H = hdc
    dim, kmer = 2048, 10
    tree = H.synth_tree(7, 64)
    copies = H.synth_copies(8, tree, 8, 0.01)
    reads = H.synth_reads(9, tree, 100, 250, subst=0.01)
    ctx = H.Context(dim, kmer, 250, 10)

    def enc(seqs, kind, dt):
        out = torch.empty((len(seqs), dim), dtype=dt, device=cuda)
        ctx.encode_segments(torch.from_numpy(seqs.buf).to(cuda), torch.from_numpy(seqs.off).to(cuda),
                            torch.from_numpy(seqs.len).to(cuda), out, kind, seqs.max_len())
        return out

    cp = enc(copies, H.OUT_I32, torch.int32)
    ptr = torch.arange(0, len(copies) + 1, 8, dtype=torch.int64, device=cuda)
    refs = ctx.bundle(cp, ptr, torch.arange(len(copies), dtype=torch.int32, device=cuda))
    q16 = enc(reads, H.OUT_BIPOLAR_F16, torch.float16)
    qi = enc(reads, H.OUT_BIPOLAR_I16, torch.int16)
    qn = ctx.norms(qi)
    db = ctx.refdb(refs, int(refs.abs().max().item()))
    s, i, c, d = ctx.search_tc(db, q16, qn, 1, 5, H.SCORE_NORM)
    torch.cuda.synchronize()
    ref_np = orc.encode([copies.get(j) for j in range(len(copies))], dim, kmer, "int32")[0]
    ref_np = ref_np.reshape(64, 8, dim).sum(1)
    assert np.array_equal(refs.cpu().numpy(), ref_np)
    os_, oi = orc.classify([reads.get(j) for j in range(len(reads))], ref_np, dim, kmer, 5, orc.SCORE_NORM,
                           bipolar=True)
    assert np.array_equal(i.cpu().numpy(), oi)
    assert np.array_equal(s.cpu().numpy(), os_)


@pytest.mark.parametrize("group,share", [(0, 0), (38, 0), (76, 0), (0, 1), (38, 1), (19, 1)])
def test_tc_cluster_many_pairs(hdc, cuda, group, share):
    """Every SM busy: 41 query tiles (odd) and 22 reference tiles in groups
    spread over all SMs, the paired multicast forms against the unpaired one,
    bit for bit."""
    g = np.random.default_rng(77 + group)
    dim, nq, nr = 2048, 41 * 128 - 5, 2600
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    one = _run_tc(ctx, db, q16, qn, 1, 7, 0, 128, group, 1, 1, 0)
    two = _run_tc(ctx, db, q16, qn, 1, 7, 0, 128, group, 1, 2, share)
    for a, b in zip(one, two):
        assert np.array_equal(a, b)


def test_tc_tile_order_does_not_change_results(hdc, cuda):
    """Reference tiles visited in index order or in the scattered order:
    identical scores, indices, cosines and dots (k = 1, 5, 32)."""
    import torch
    import hdc_gb300
    g = np.random.default_rng(31)
    dim, nq, nr = 2048, 700, 9000
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    for k in (1, 5, 32):
        res = []
        for scatter in (0, 1):
            ctx.option(hdc_gb300.TC_SCATTER, scatter)
            res.append(_run_tc(ctx, db, q16, qn, 1, k, 0))
        for a, b in zip(*res):
            assert np.array_equal(a, b)

def test_tc_kblock32_equals_kblock64(hdc, cuda):
    """The paired search with 32-dim K blocks (64-byte swizzle, deeper ring)
    and with 64-dim K blocks: identical scores, indices, cosines and dots,
    including a dim that is not a multiple of 64 (k = 1, 5, 32)."""
    import hdc_gb300
    g = np.random.default_rng(37)
    for dim, nr, lim in ((2048, 9000, 12000), (1056, 5000, 20000000)):
        nq = 700
        refs = g.integers(-lim, lim + 1, (nr, dim)).astype(np.int32 if lim > 32767 else np.int16)
        q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
        ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
        for k in (1, 5, 32):
            res = []
            for kb in (64, 32):
                ctx.option(hdc_gb300.TC_KBLOCK, kb)
                res.append(_run_tc(ctx, db, q16, qn, 1, k, 0))
            for a, b in zip(*res):
                assert np.array_equal(a, b)


# CTA pairs as one M = 256 MMA (two limbs only; other limb counts take the
# multicast form whatever the option says).  Groups of 3 query tiles round down
# to 2; 129 / 300 queries leave the odd CTA of the last pair without a tile.
@pytest.mark.parametrize("group", [0, 3, 4])
@pytest.mark.parametrize("dim,nq,nr,k,mode,vmax,dtype", [
    (2048, 130, 3000, 10, 0, 12000, np.int16),   # two limbs
    (1024, 300, 777, 1, 1, 12000, np.int16),     # argmax, COS scale, ragged sizes
    (512, 64, 500, 32, 2, 3000, np.int16),       # DOT scale, largest k
    (1024, 100, 600, 5, 0, 3000000, np.int32),   # two limbs, the top one above 1024
    (1056, 200, 900, 5, 0, 12000, np.int16),     # dim not a multiple of the 64-dim K block
    (10240, 129, 300, 5, 0, 12728, np.int16),    # precision-form dimension
    (1024, 100, 600, 5, 0, 20000000, np.int32),  # three limbs: multicast form
    (1024, 200, 1000, 5, 0, 2000, np.int16),     # one limb: multicast form
])
def test_tc_pair_mma_vs_oracle(hdc, orc, cuda, dim, nq, nr, k, mode, vmax, dtype, group):
    g = np.random.default_rng(dim + nq + nr + 7)
    refs = g.integers(-vmax, vmax + 1, (nr, dim)).astype(dtype)
    refs[3] = refs[1]
    refs[4] = 0
    refs[5, :] = vmax
    refs[6, ::2] = -vmax
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    q[0] = np.where(refs[1] >= 0, 1, -1)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    s, i, c, d = _run_tc(ctx, db, q16, qn, 1, k, mode, 128, group, 1, 2, 0, 1)
    os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), min(k, nr), mode)
    assert np.array_equal(i, oi)
    assert np.array_equal(d, od)
    assert np.array_equal(s, os_)
    assert np.array_equal(c, oc)


def test_tc_pair_mma_equals_multicast(hdc, cuda):
    """Pairs as one M = 256 MMA and pairs sharing reference blocks by
    multicast: identical scores, indices, cosines and dots (k = 1, 5, 32) on a
    grid with many pairs and reference lanes."""
    g = np.random.default_rng(41)
    dim, nq, nr = 2048, 5000, 20000
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    import torch
    for k in (1, 5, 32):
        a = _run_tc(ctx, db, q16, qn, 1, k, 0, pair=0)
        b = _run_tc(ctx, db, q16, qn, 1, k, 0, pair=1)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    # clusters of 4: two pair MMAs on two reference lanes sharing query blocks
    for k in (1, 32):
        ref = _run_tc(ctx, db, q16, qn, 1, k, 0, pair=0)
        c4 = _run_tc(ctx, db, q16, qn, 1, k, 0, cluster=4, pair=1)
        for x, y in zip(ref, c4):
            assert np.array_equal(x, y)
    # with L2 eviction hints on the pair loads (queries evict-last, + references evict-first)
    import hdc_gb300
    ctx.tc_option(hdc_gb300.TC_CLUSTER, 0)
    for policy in (1, 2):
        ctx.tc_tuning(8, policy, 0, 0)
        c = ctx.search_tc(db, q16, qn, 1, 32, 0)
        torch.cuda.synchronize()
        assert ctx.status() == 0
        for x, y in zip(a, c):
            assert np.array_equal(x, y.cpu().numpy())



_LANE_ORACLE = {}


# Reference lanes of one query tile exchange their k-th best scores (2 to 4
# lanes) and filter by them.  A clustered database (rows near a few centres,
# so many references score close to a query's best) with duplicated rows
# placed in other lanes' tiles (equal scores across lanes: ties go to the
# lower index) checks that no reference of the final top-k is dropped.
# With pair MMAs, k = 9..16 keeps the lists' keys in registers (k = 9 and 16
# are its bounds).  Forms: multicast pairs, pair MMAs, and clusters of 4 (two
# pair MMAs on two lanes sharing query blocks; 3 lanes round down to 2, and 94
# reference tiles over 4 lanes leave two lanes an empty last tile).
@pytest.mark.parametrize("lanes", [2, 3, 4, 8])
@pytest.mark.parametrize("pair,cluster", [(0, 2), (1, 2), (1, 4)])
@pytest.mark.parametrize("k,mode", [(1, 0), (5, 0), (32, 0), (5, 2), (10, 1), (9, 0), (16, 0)])
def test_tc_lane_exchange_vs_oracle(hdc, orc, cuda, lanes, pair, cluster, k, mode):
    import hdc_gb300
    g = np.random.default_rng(100 + k)
    dim, nq, nr = 512, 520, 12000
    centres = g.integers(-9000, 9001, (6, dim))
    refs = (centres[g.integers(0, 6, nr)] + g.integers(-400, 401, (nr, dim))).astype(np.int16)
    src = g.choice(nr // 2, 300, replace=False)
    dst = nr // 2 + g.choice(nr // 2, 300, replace=False)
    refs[dst] = refs[src]                  # equal scores in other reference tiles
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    q[:64] = np.where(centres[g.integers(0, 6, 64)] >= 0, 1, -1)  # queries near a centre
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    ctx.option(hdc_gb300.TC_LANES, lanes)
    s, i, c, d = _run_tc(ctx, db, q16, qn, 1, k, mode, 128, 0, 1, cluster, 0, pair)
    assert ctx.status() == 0
    if (k, mode) not in _LANE_ORACLE:  # the same inputs for every lane count and form
        _LANE_ORACLE[(k, mode)] = orc.topk(q.astype(np.int32), refs.astype(np.int32), min(k, nr), mode)
    os_, oi, oc, od = _LANE_ORACLE[(k, mode)]
    assert np.array_equal(i, oi)
    assert np.array_equal(d, od)
    assert np.array_equal(s, os_)
    assert np.array_equal(c, oc)


def test_tc_quad_split_vs_pairs_and_oracle(hdc, orc, cuda):
    """A batch whose clusters of 4 do not all fit (75 query tiles: 74 x 2
    lanes = 148 CTAs, of which 144 can run as clusters of 4): the leading 72
    tiles run as clusters of 4, the other 293 queries as pairs.  Identical to
    pairs for the whole batch, and to the oracle on sampled rows, including
    rows on both sides of the split."""
    import hdc_gb300
    g = np.random.default_rng(53)
    dim, nr, nq = 1024, 4000, 75 * 128 - 91
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    for k, mode in ((5, 0), (32, 2)):
        pairs = _run_tc(ctx, db, q16, qn, 1, k, mode, cluster=2, pair=1)
        quads = _run_tc(ctx, db, q16, qn, 1, k, mode, cluster=4, pair=1)
        shape = ctx.tc_last_shape()
        assert shape[3] == 1 and shape[0] in (2, 4)
        for x, y in zip(pairs, quads):
            assert np.array_equal(x, y)
        rows = np.concatenate([np.arange(9200, 9240), g.choice(nq, 120, replace=False)])
        os_, oi, oc, od = orc.topk(q[rows].astype(np.int32), refs.astype(np.int32), k, mode)
        s, i, c, d = quads
        assert np.array_equal(i[rows], oi)
        assert np.array_equal(d[rows], od)
        assert np.array_equal(s[rows], os_)
        assert np.array_equal(c[rows], oc)


# Count-valued queries (e.g. fp16 k-mer counts of reads): the database's limbs are sized for
# the largest query magnitude (hdc_refdb_create_ex), every fp32 partial sum stays exact.
@pytest.mark.parametrize("dim,nq,nr,k,mode,qmax,vmax,dtype,bits,limbs", [
    (2048, 140, 3000, 5, 0, 200, 30000, np.int16, 6, 3),     # base 64
    (1024, 100, 900, 10, 1, 2048, 1600, np.int16, 4, 3),     # base 16: |q| up to 2048
    (1056, 200, 700, 1, 2, 143, 1000000, np.int32, 7, 3),    # base 128, int32 references
])
def test_tc_count_queries_vs_oracle(hdc, orc, cuda, dim, nq, nr, k, mode, qmax, vmax, dtype, bits, limbs):
    import torch
    g = np.random.default_rng(dim + qmax)
    refs = g.integers(-vmax, vmax + 1, (nr, dim)).astype(dtype)
    refs[3] = refs[1]
    refs[5, :] = vmax
    refs[6, ::2] = -vmax
    q = g.integers(-qmax, qmax + 1, (nq, dim)).astype(np.int16)
    q[0, :] = qmax
    q[1] = np.where(refs[1] >= 0, qmax, -qmax)
    ctx = hdc.Context(dim, 10, 250, 10)
    tr = torch.from_numpy(refs).to(cuda)
    db = ctx.refdb(tr, int(np.abs(refs).max()), max_query_abs=qmax)
    assert (db.limb_bits, db.limbs) == (bits, limbs)
    q16 = torch.from_numpy(q.astype(np.float16)).to(cuda)
    qn = ctx.norms(q16)  # integer-valued fp16 rows (hdc_norms_f16)
    assert torch.equal(qn, ctx.norms(torch.from_numpy(q).to(cuda)))
    for cluster, pair in ((0, -1), (2, 0)):
        s, i, c, d = _run_tc(ctx, db, q16, qn, qmax, k, mode, cluster=cluster, pair=pair)
        os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), min(k, nr), mode)
        assert np.array_equal(i, oi)
        assert np.array_equal(d, od)
        assert np.array_equal(s, os_)
        assert np.array_equal(c, oc)



# schedules: one CTA per tile; multicast pairs sharing references; pairs sharing queries;
# pair MMA (cta_group::2); pair MMAs in clusters of 4
@pytest.mark.parametrize("cluster,share,pair", [(1, 0, 0), (2, 0, 0), (2, 1, 0), (2, 0, 1), (4, 0, 1)])
def test_tc_bounded_wait_runs_out_and_context_recovers(hdc, orc, cuda, cluster, share, pair):
    """A bounded device-side wait that runs out, without faulting anything:
    with HDC_TEST_WITHHOLD_LOADS the producer issues no operand load, so the
    MMA issuer's wait for the first stage (and the epilogue's for the first
    accumulators) runs out after HDC_WAIT_LIMIT with no copy and no MMA in
    flight; every role leaves its loop, TMEM is freed and the context status
    reports 100 + the wait's code.  The next search on the same context (hook
    off, default limit) returns the oracle's results."""
    import torch
    H = hdc
    g = np.random.default_rng(77)
    dim, nq, nr, k = 1024, 512, 1500, 5
    refs = g.integers(-12000, 12001, (nr, dim)).astype(np.int16)  # two limbs
    q = np.where(g.random((nq, dim)) < 0.5, -1, 1).astype(np.int8)
    ctx, db, tr, q16, qi, qn = _setup(hdc, cuda, refs, q, dim)
    ctx.tc_option(H.TC_CLUSTER, cluster)
    ctx.tc_option(H.TC_SHARE, share)
    ctx.tc_option(H.TC_PAIR_MMA, pair)
    assert ctx.status() == 0
    ctx.option(H.WAIT_LIMIT, 1000)  # 10^6 SM cycles, about half a millisecond
    ctx.option(H.TEST_WITHHOLD_LOADS, 1)
    ctx.search_tc(db, q16, qn, 1, k, H.SCORE_NORM)
    torch.cuda.synchronize()
    st = ctx.status()
    assert 101 <= st <= 104, st  # a pipeline wait of the search gave up
    assert ctx.tc_last_shape()[0] == cluster
    ctx.option(H.TEST_WITHHOLD_LOADS, 0)
    ctx.option(H.WAIT_LIMIT, 0)
    s, i, c, d = ctx.search_tc(db, q16, qn, 1, k, H.SCORE_NORM)
    torch.cuda.synchronize()
    assert ctx.status() == 0
    os_, oi, oc, od = orc.topk(q.astype(np.int32), refs.astype(np.int32), k, H.SCORE_NORM)
    assert np.array_equal(i.cpu().numpy(), oi) and np.array_equal(d.cpu().numpy(), od)
    assert np.array_equal(s.cpu().numpy(), os_) and np.array_equal(c.cpu().numpy(), oc)


def test_wait_options_are_checked(hdc, cuda):
    H = hdc
    ctx = H.Context(1024, 10, 250, 10)
    for opt, bad in ((H.WAIT_LIMIT, -1), (H.WAIT_LIMIT, 4000001), (H.TEST_WITHHOLD_LOADS, 3),
                     (H.TEST_WITHHOLD_LOADS, -1)):
        with pytest.raises(H.HDCError):
            ctx.option(opt, bad)
