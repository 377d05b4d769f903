"""2-bit packed reads (the reference's pack_sequence format, src/encode.cu:
169-185): the device packing (hdc_pack_2bit) against the oracle's
restatement, and the encoder over packed reads (hdc_encode_packed) against
the encoder over the same ASCII bytes (A, C, G, T sequences, bit-exact with
HVCache::compute through the golden-pinned ASCII path) and against the
oracle's encode of what the packing makes of N, IUPAC and lowercase bytes."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pack_2bit_matches_oracle(hdc, orc, cuda):
    import torch
    rng = random.Random(3)
    for n in (0, 1, 15, 16, 17, 255, 4096, 100003):
        data = bytes(rng.choice(b"ACGTacgtNRYx\0\xff") for _ in range(n))
        d = torch.from_numpy(np.frombuffer(data + b"\0" * 16, np.uint8).copy()).to(cuda)
        ctx = hdc.Context(1024, 8, 150, 10)
        words = ctx.pack_2bit(d, n)
        torch.cuda.synchronize()
        want = orc.pack_2bit(data)
        assert np.array_equal(words.cpu().numpy()[:len(want)].view(np.uint32), want), n


@pytest.mark.parametrize("dim,k", [(1024, 8), (10240, 10), (16384, 12), (200, 3), (8192, 16)])
def test_encode_packed_equals_ascii(hdc, cuda, dim, k):
    import torch
    H = hdc
    rng = random.Random(dim + k)
    lens = [0, k - 1, k, 16, 17, 150, 250, 1600, 3001] + [rng.randint(100, 1600) for _ in range(40)]
    seqs = ["".join(rng.choice("ACGT") for _ in range(n)) for n in lens]
    # segments at arbitrary byte (= base) offsets: a random gap before each
    buf, off = b"", []
    for s in seqs:
        buf += bytes(rng.choice(b"ACGTN") for _ in range(rng.randint(0, 21)))
        off.append(len(buf))
        buf += s.encode()
    d_bytes = torch.from_numpy(np.frombuffer(buf + b"\0" * 32, np.uint8).copy()).to(cuda)
    d_off = torch.tensor(off, dtype=torch.int64, device=cuda)
    d_len = torch.tensor(lens, dtype=torch.int32, device=cuda)
    ctx = H.Context(dim, k, 150, 10)
    words = ctx.pack_2bit(d_bytes, len(buf))
    for kind, dt, width in ((H.OUT_I16, torch.int16, dim), (H.OUT_I32, torch.int32, dim),
                            (H.OUT_SIGN_BITS, torch.int32, (dim + 31) // 32),
                            (H.OUT_BIPOLAR_F16, torch.float16, dim)):
        a = torch.zeros((len(seqs), width), dtype=dt, device=cuda)
        b = torch.ones((len(seqs), width), dtype=dt, device=cuda)
        na = torch.zeros(len(seqs), dtype=torch.int32, device=cuda)
        nb = torch.ones(len(seqs), dtype=torch.int32, device=cuda)
        ctx.encode_segments(d_bytes, d_off, d_len, a, kind, max(lens), nkmers=na)
        ctx.encode_packed(words, d_off, d_len, b, kind, max(lens), nkmers=nb)
        torch.cuda.synchronize()
        assert torch.equal(a, b), kind
        assert torch.equal(na, nb)


def test_encode_packed_reads_other_bytes_as_the_packing_codes(hdc, orc, cuda):
    """N and other bytes pack as A and lowercase as its base, so the packed
    encode of a sequence equals HVCache::compute of its packed view."""
    import torch
    H = hdc
    rng = random.Random(9)
    dim, k = 1024, 8
    seqs = ["".join(rng.choice("ACGTacgtNNRY") for _ in range(n)) for n in (8, 40, 150, 300, 999)]
    buf = "".join(seqs).encode()
    off = np.cumsum([0] + [len(s) for s in seqs[:-1]])
    ctx = H.Context(dim, k, 150, 10)
    d_bytes = torch.from_numpy(np.frombuffer(buf + b"\0" * 16, np.uint8).copy()).to(cuda)
    words = ctx.pack_2bit(d_bytes, len(buf))
    out = torch.empty((len(seqs), dim), dtype=torch.int32, device=cuda)
    ctx.encode_packed(words, torch.tensor(off, dtype=torch.int64, device=cuda),
                      torch.tensor([len(s) for s in seqs], dtype=torch.int32, device=cuda), out, H.OUT_I32, 999)
    torch.cuda.synchronize()
    want, _ = orc.encode([orc.packed_view(s) for s in seqs], dim, k, "int32")
    assert np.array_equal(out.cpu().numpy(), want)
