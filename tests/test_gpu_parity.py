"""GPU parity of the CUDA path with the CPU oracle and the reference's golden
vectors.  Integer outputs (hypervectors, dots, indices) must be bit-exact;
float scores must be equal (they are the reference's own double expression
rounded to float), FP64 cosines equal to the oracle's double value."""
import glob
import hashlib
import json
import os
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CONFIGS = sorted(glob.glob(os.path.join(GOLD, "ref_D*.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def upload(seqs, dev):
    import torch
    import hdc_gb300 as H
    buf, off, ln = H.pack_sequences(seqs)
    return (torch.from_numpy(buf.copy()).to(dev), torch.from_numpy(off).to(dev), torch.from_numpy(ln).to(dev),
            int(ln.max()) if len(ln) else 0)


def gpu_encode(ctx, seqs, dev, kind=0, max_len=None):
    import torch
    b, o, l, mx = upload(seqs, dev)
    dt = {0: torch.int16, 1: torch.int32, 2: torch.bfloat16, 3: torch.int16, 4: torch.float16, 5: torch.int8,
          6: torch.float16}[kind]
    out = torch.full((len(seqs), ctx.dim), 7, dtype=dt, device=dev)
    nk = torch.zeros(len(seqs), dtype=torch.int32, device=dev)
    ctx.encode_segments(b, o, l, out, kind, mx if max_len is None else max_len, nk)
    torch.cuda.synchronize()
    return out.cpu(), nk.cpu().numpy()


def rseq(rng, n, alphabet="ACGT"):
    return "".join(rng.choice(alphabet) for _ in range(n))


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_base_hvs_match_golden(hdc, cuda, path):
    meta = json.load(open(path))
    ctx = hdc.Context(meta["dim"], meta["kmer"], meta["window"], meta["step"])
    assert sha(ctx.base_hvs()) == meta["base_sha"]


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_encode_matches_golden(hdc, cuda, path):
    meta = json.load(open(path))
    ctx = hdc.Context(meta["dim"], meta["kmer"], meta["window"], meta["step"])
    out, nk = gpu_encode(ctx, meta["encode_seqs"], cuda)
    assert [sha(r) for r in out.numpy()] == meta["encode_sha"]


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_encode_windows_match_golden(hdc, cuda, path):
    import torch
    meta = json.load(open(path))
    ctx = hdc.Context(meta["dim"], meta["kmer"], meta["window"], meta["step"])
    seqs = meta["window_seqs"]
    buf, off, ln = hdc.pack_sequences(seqs)
    seq_off = np.zeros(len(seqs) + 1, np.int64)
    seq_off[1:] = np.cumsum(ln)
    nw = [ctx.num_windows(int(x)) for x in ln]
    win_off = np.zeros(len(seqs) + 1, np.int64)
    win_off[1:] = np.cumsum(nw)
    out = torch.zeros((int(win_off[-1]), ctx.dim), dtype=torch.int16, device=cuda)
    ctx.encode_windows(torch.from_numpy(buf.copy()).to(cuda), torch.from_numpy(seq_off).to(cuda),
                       torch.from_numpy(win_off).to(cuda), int(win_off[-1]), out)
    torch.cuda.synchronize()
    assert [sha(r) for r in out.cpu().numpy()] == meta["windows_sha"]


@pytest.mark.parametrize("dim,k", [(1024, 8), (200, 3), (2048, 10), (4096, 12), (1024, 16), (512, 1), (10000, 5)])
def test_encode_random_all_kinds(hdc, orc, cuda, dim, k):
    import torch
    rng = random.Random(dim * 31 + k)
    seqs = [rseq(rng, rng.randint(0, 600)) for _ in range(60)]
    seqs += [rseq(rng, 300, "ACGTACGTACGTNacgt") for _ in range(10)]  # N and lowercase
    seqs += ["", "A" * (k - 1), "C" * k, "G" * (k + 1), rseq(rng, 5000), rseq(rng, 70000)]
    ctx = hdc.Context(dim, k, 150, 10)
    ref16, nk_ref = orc.encode(seqs, dim, k, "int16")
    ref32, _ = orc.encode(seqs, dim, k, "int32")
    out, nk = gpu_encode(ctx, seqs, cuda, 0)
    assert np.array_equal(out.numpy(), ref16)
    assert np.array_equal(nk, nk_ref)
    # exact int32 and the bipolar forms: segments up to 65535 k-mers
    short = [i for i, s in enumerate(seqs) if len(s) - k + 1 <= 65535]
    sub = [seqs[i] for i in short]
    out32, _ = gpu_encode(ctx, sub, cuda, 1)
    assert np.array_equal(out32.numpy(), ref32[short])
    bip = np.where(ref32[short] >= 0, 1, -1)
    outb, _ = gpu_encode(ctx, sub, cuda, 3)
    assert np.array_equal(outb.numpy(), bip)
    outbf, _ = gpu_encode(ctx, sub, cuda, 2)
    assert np.array_equal(outbf.float().numpy(), bip.astype(np.float32))
    outh, _ = gpu_encode(ctx, sub, cuda, 4)
    assert np.array_equal(outh.float().numpy(), bip.astype(np.float32))
    out8, _ = gpu_encode(ctx, sub, cuda, 5)
    assert np.array_equal(out8.numpy(), bip)
    # fp16 counts (exact): segments up to 2048 k-mers; longer ones are refused
    f16 = [i for i, s in enumerate(seqs) if len(s) - k + 1 <= 2048]
    outf, _ = gpu_encode(ctx, [seqs[i] for i in f16], cuda, 6)
    assert np.array_equal(outf.float().numpy(), ref32[f16].astype(np.float32))
    with pytest.raises(hdc.HDCError):
        gpu_encode(ctx, [seqs[i] for i in range(len(seqs)) if len(seqs[i]) - k + 1 > 2048][:1], cuda, 6)


def test_search_rejects_inexact_range(hdc, cuda):
    import torch
    ctx = hdc.Context(256, 8, 150, 10)
    q = torch.zeros((4, 256), dtype=torch.int16, device=cuda)
    n = ctx.norms(q)
    with pytest.raises(hdc.HDCError) as e:
        ctx.search_plain(q, n, 1100, q, n, 1000, 1)  # 1.1e6 > 2^20
    assert e.value.status == 2


def test_encode_max_len_hint_is_checked(hdc, cuda):
    ctx = hdc.Context(1024, 8, 150, 10)
    with pytest.raises(hdc.HDCError):
        gpu_encode(ctx, ["A" * 70000], cuda, 1, max_len=70000)  # exact int32 needs <= 65535 k-mers


def _search(hdc, ctx, q, r, k, mode, dev):
    import torch
    tq = torch.from_numpy(np.ascontiguousarray(q, np.int16)).to(dev)
    tr = torch.from_numpy(np.ascontiguousarray(r, np.int16)).to(dev)
    mq = torch.zeros(1, dtype=torch.int32, device=dev)
    mr = torch.zeros(1, dtype=torch.int32, device=dev)
    qn = ctx.norms(tq, mq)
    rn = ctx.norms(tr, mr)
    torch.cuda.synchronize()
    s, i, c, d = ctx.search_plain(tq, qn, int(mq.item()), tr, rn, int(mr.item()), k, mode)
    torch.cuda.synchronize()
    return s.cpu().numpy(), i.cpu().numpy(), c.cpu().numpy(), d.cpu().numpy()


@pytest.mark.parametrize("path", CONFIGS, ids=os.path.basename)
def test_search_matches_golden_topk(hdc, cuda, path):
    meta = json.load(open(path))
    ctx = hdc.Context(meta["dim"], meta["kmer"], meta["window"], meta["step"])
    q, _ = gpu_encode(ctx, meta["topk_queries"], cuda)
    r, _ = gpu_encode(ctx, meta["topk_refs"], cuda)
    s, i, c, d = _search(hdc, ctx, q.numpy(), r.numpy(), 5, hdc.SCORE_NORM, cuda)
    assert i.tolist() == meta["topk_idx"]
    assert np.array_equal(s, np.array(meta["topk_score"], np.float32))


@pytest.mark.parametrize("dim,nq,nr,k,mode,vmax", [
    (1024, 37, 300, 5, 0, 150),      # nq, nr not multiples of the tiles
    (1024, 200, 1000, 1, 0, 150),    # argmax
    (2048, 130, 2000, 10, 1, 300),   # COS scale
    (512, 64, 777, 32, 2, 100),      # DOT scale, largest k
    (1000, 50, 500, 5, 0, 150),      # dim not a multiple of 8: scalar loads
    (4096, 40, 600, 5, 0, 1000),     # int64 accumulation path (max*max*dim >= 2^31)
    (256, 20, 3, 5, 0, 50),          # k clamped to nr
])
def test_search_plain_vs_oracle(hdc, orc, cuda, dim, nq, nr, k, mode, vmax):
    g = np.random.default_rng(dim + nq + nr + k)
    r = g.integers(-vmax, vmax + 1, (nr, dim)).astype(np.int16)
    q = g.integers(-vmax, vmax + 1, (nq, dim)).astype(np.int16)
    if nr > 5:
        r[5] = r[3]                  # duplicates: ties to the lower index
    r[min(7, nr - 1)] = 0            # zero norm: score -1
    q[1] = r[min(3, nr - 1)]         # exact matches
    q[2] = 0
    ctx = hdc.Context(dim, 8, 150, 10)
    s, i, c, d = _search(hdc, ctx, q, r, k, mode, cuda)
    os_, oi, oc, od = orc.topk(q, r, min(k, nr), mode)
    assert np.array_equal(i, oi)
    assert np.array_equal(s, os_)
    assert np.array_equal(d, od)
    assert np.array_equal(c, oc)


def test_search_encoded_reads(hdc, orc, cuda):
    """Reads sampled from mutated references: the realistic ranking case."""
    rng = random.Random(5)
    dim, k = 2048, 8
    roots = [rseq(rng, 1500) for _ in range(4)]
    refs = []
    for i in range(300):
        s = list(roots[i % 4])
        for p in rng.sample(range(1500), 20 + i % 50):
            s[p] = rng.choice("ACGT")
        refs.append("".join(s))
    reads = []
    for i in range(200):
        r = refs[rng.randrange(len(refs))]
        st = rng.randint(0, 1350)
        reads.append(r[st:st + 150])
    ctx = hdc.Context(dim, k, 150, 10)
    q, _ = gpu_encode(ctx, reads, cuda)
    R, _ = gpu_encode(ctx, refs, cuda)
    s, i, c, d = _search(hdc, ctx, q.numpy(), R.numpy(), 5, hdc.SCORE_NORM, cuda)
    os_, oi = orc.classify(reads, R.numpy().astype(np.int32), dim, k, 5, orc.SCORE_NORM)
    assert np.array_equal(i, oi)
    assert np.array_equal(s, os_)


def test_bundle_vs_oracle(hdc, orc, cuda):
    import torch
    g = np.random.default_rng(3)
    dim = 1536
    rows = g.integers(-2000, 2000, (500, dim)).astype(np.int16)
    counts = g.integers(0, 9, 80)
    ptr = np.zeros(81, np.int64)
    ptr[1:] = np.cumsum(counts)
    idx = g.integers(0, 500, int(ptr[-1])).astype(np.int32)
    ctx = hdc.Context(dim, 8, 150, 10)
    out = ctx.bundle(torch.from_numpy(rows).to(cuda), torch.from_numpy(ptr).to(cuda), torch.from_numpy(idx).to(cuda))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), orc.bundle(rows, ptr, idx))


def test_self_retrieval_full_size(hdc, cuda):
    """Full plain-form reference size (50,000 references, D=8192): a sample
    of references queried against the whole database each rank themselves
    first with cos = 1 (to the last FP64 bit of sqrt(n)*sqrt(n)), a
    size-independent property of the exact search."""
    import torch
    g = torch.Generator(device=cuda).manual_seed(11)
    nr, dim = 50000, 8192
    r = torch.randint(-1000, 1001, (nr, dim), dtype=torch.int16, device=cuda, generator=g)
    ctx = hdc.Context(dim, 8, 150, 10)
    mr = torch.zeros(1, dtype=torch.int32, device=cuda)
    rn = ctx.norms(r, mr)
    sel = torch.arange(0, nr, 997, device=cuda)
    q = r[sel].clone()
    mq = torch.zeros(1, dtype=torch.int32, device=cuda)
    qn = ctx.norms(q, mq)
    s, i, c, d = ctx.search_plain(q, qn, int(mq.item()), r, rn, int(mr.item()), 5, hdc.SCORE_COS)
    torch.cuda.synchronize()
    assert torch.equal(i[:, 0].long(), sel)
    assert torch.equal(d[:, 0], rn[sel])
    assert bool((c[:, 0] >= 1 - 1e-15).all())
