"""Persisted tensor-core database: save -> load gives the same search results
bit for bit and the same taxonomy ids; a corrupted byte, a truncated file, a
foreign file and a file of another k-mer size are rejected."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _db(hdc, cuda, dim=1024, nr=700, vmax=12000, seed=5):
    import torch
    g = np.random.default_rng(seed)
    refs = g.integers(-vmax, vmax + 1, (nr, dim)).astype(np.int16)
    ctx = hdc.Context(dim, 10, 250, 10)
    tr = torch.from_numpy(refs).to(cuda)
    db = ctx.refdb(tr, int(np.abs(refs).max()))
    q = np.where(g.random((300, dim)) < 0.5, -1, 1)
    q16 = torch.from_numpy(q.astype(np.float16)).to(cuda)
    qn = torch.full((300,), dim, dtype=torch.int64, device=cuda)
    return ctx, db, q16, qn


def _search(ctx, db, q16, qn):
    import torch
    out = ctx.search_tc(db, q16, qn, 1, 5)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in out]


def test_save_load_roundtrip(hdc, cuda, tmp_path):
    ctx, db, q16, qn = _db(hdc, cuda)
    ids = np.arange(db.nr, dtype=np.int32) * 7 + 3
    path = tmp_path / "refs.hdcdb"
    db.save(path, ids)
    info = hdc.RefDB.file_info(path)
    assert info == dict(dim=1024, kmer=10, nr=db.nr, limbs=db.limbs, has_tax_ids=True)
    db2, ids2 = hdc.RefDB.load(ctx, path)
    assert np.array_equal(ids2, ids) and db2.limbs == db.limbs and db2.nr == db.nr
    for a, b in zip(_search(ctx, db, q16, qn), _search(ctx, db2, q16, qn)):
        assert np.array_equal(a, b)
    db.save(tmp_path / "noids.hdcdb")
    db3, ids3 = hdc.RefDB.load(ctx, tmp_path / "noids.hdcdb")
    assert ids3 is None and db3.nr == db.nr


def test_load_rejects_bad_files(hdc, cuda, tmp_path):
    ctx, db, q16, qn = _db(hdc, cuda, nr=300)
    path = tmp_path / "refs.hdcdb"
    db.save(path)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.hdcdb"
    raw[128 + 1000] ^= 0x40  # one payload bit
    bad.write_bytes(bytes(raw))
    with pytest.raises(RuntimeError, match="checksum"):
        hdc.RefDB.load(ctx, bad)
    bad.write_bytes(path.read_bytes()[:-10])
    with pytest.raises(RuntimeError, match="truncated|inconsistent"):
        hdc.RefDB.load(ctx, bad)
    bad.write_bytes(b"not a database" * 20)
    with pytest.raises(RuntimeError, match="not a database"):
        hdc.RefDB.load(ctx, bad)
    other = hdc.Context(1024, 12, 250, 10)
    with pytest.raises(RuntimeError, match="k-mer"):
        hdc.RefDB.load(other, path)


def test_save_load_keeps_limb_base(hdc, cuda, tmp_path):
    """A database sized for count-valued queries (base-64 limbs) survives the
    file round trip: same limbs, same limb base, identical search results."""
    import torch
    g = np.random.default_rng(9)
    dim, nr, nq = 1024, 500, 60
    refs = g.integers(-30000, 30001, (nr, dim)).astype(np.int16)
    q = g.integers(-300, 301, (nq, dim)).astype(np.int16)
    ctx = hdc.Context(dim, 10, 250, 10)
    db = ctx.refdb(torch.from_numpy(refs).to(cuda), 30000, max_query_abs=300)
    q16 = torch.from_numpy(q.astype(np.float16)).to(cuda)
    qn = ctx.norms(torch.from_numpy(q).to(cuda))
    path = tmp_path / "counts.hdcdb"
    db.save(path)
    db2, _ = hdc.RefDB.load(ctx, path)
    assert (db2.limbs, db2.limb_bits) == (db.limbs, db.limb_bits) and db.limb_bits < 11
    a = ctx.search_tc(db, q16, qn, 300, 5)
    b = ctx.search_tc(db2, q16, qn, 300, 5)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)

