"""GPU FASTA ingest against the oracle's restatement of the reference's reading
(targets/identify.cpp:46-71): records, names and sequences byte for byte, on
edge cases (CRLF, empty records, text before the first header, blank lines,
'>' inside a line, no final newline, header only, empty input) and on a large
random file."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    b"",
    b"\n",
    b">only header",
    b">h\n",
    b"ACGT",
    b"AC\n>r1\nACGT\nTT\n>empty\n>r2 x\r\nGG\r\n\n>\nA",
    b">a\nAC>GT\n\n\nTT\n>b\n>c\nG",
    b">a b c\nNNNN\n>a b c\nNNNN\n",
    b"\n\n>x\n\nA\n\n",
]


def _parse(hdc, ctx, data, cuda, max_records=None):
    import torch
    d = torch.frombuffer(bytearray(data), dtype=torch.uint8).to(cuda) if data else \
        torch.empty(0, dtype=torch.uint8, device=cuda)
    out, so, sl, no, nl, c = ctx.fasta_parse(d, max_records)
    torch.cuda.synchronize()
    ob = out.cpu().numpy().tobytes()
    so, sl, no, nl = (x.cpu().numpy() for x in (so, sl, no, nl))
    recs = [(data[no[j]:no[j] + nl[j]], ob[so[j]:so[j] + sl[j]]) for j in range(len(so))]
    return recs, c


@pytest.mark.parametrize("data", CASES)
def test_fasta_edge_cases(hdc, orc, cuda, data):
    ctx = hdc.Context(1024, 8, 150, 10)
    recs, c = _parse(hdc, ctx, data, cuda)
    want = orc.fasta_records(data)
    assert c == len(want)
    assert recs == want


def test_fasta_large_random(hdc, orc, cuda):
    rng = random.Random(9)
    parts = []
    for i in range(30000):
        parts.append(b">read%d some description\n" % i)
        seq = "".join(rng.choice("ACGTN") for _ in range(rng.randint(0, 400)))
        for j in range(0, len(seq), rng.choice([60, 80, 1000])):
            parts.append(seq[j:j + 80].encode() + (b"\r\n" if i % 7 == 0 else b"\n"))
    data = b"".join(parts)
    ctx = hdc.Context(1024, 8, 150, 10)
    recs, c = _parse(hdc, ctx, data, cuda)
    want = orc.fasta_records(data)
    assert c == len(want) and recs == want


def test_fasta_capacity(hdc, orc, cuda):
    data = b"".join(b">r%d\nACGT\n" % i for i in range(50))
    ctx = hdc.Context(1024, 8, 150, 10)
    recs, c = _parse(hdc, ctx, data, cuda, max_records=20)
    assert c == 50 and recs == orc.fasta_records(data)[:20]


def test_fasta_lines_across_tiles(hdc, orc, cuda):
    """Lines longer than the parser's 8 KB tiles: text before the first header
    over several tiles, a 20 KB header line, a 100 KB sequence line without
    '\\n', CRLF lines, headers at tile edges and an input ending inside a
    header."""
    rng = random.Random(5)
    seq = lambda n: "".join(rng.choice("ACGTN") for _ in range(n)).encode()
    parts = [seq(30000), b"\n", seq(5000), b"\n>", b"h" * 20000, b"\n", seq(100000), b"\n"]
    for i in range(200):  # short records of random sizes, some lines ending in CRLF
        parts.append(b">r%d\n" % i)
        parts.append(seq(rng.randint(0, 9000)) + (b"\r\n" if i % 3 == 0 else b"\n"))
    data = b"".join(parts)
    # headers placed exactly at multiples of 8 KB
    edge = bytearray(b"A" * (8192 * 3 + 5))
    for p in (8192 - 1, 2 * 8192 - 1):
        edge[p] = ord("\n")
        edge[p + 1] = ord(">")
    data += bytes(edge) + b"\n>tail header without newline"
    ctx = hdc.Context(1024, 8, 150, 10)
    recs, c = _parse(hdc, ctx, data, cuda)
    want = orc.fasta_records(data)
    assert c == len(want) and recs == want
