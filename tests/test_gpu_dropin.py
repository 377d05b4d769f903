"""The GPU.cuh drop-in (encode, cosine_search) driven through the reference's
call surface by dropin/selftest.cpp, checked against the oracle: window
hypervectors bit-exact, ranked matches identical (cosine scale)."""
import os
import random
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dropin_encode_and_cosine_search(hdc, orc, cuda):
    import build as pkg_build
    out = pkg_build.build_dropin(1024, 8, 150, 10)
    rng = random.Random(3)
    roots = ["".join(rng.choice("ACGT") for _ in range(400)) for _ in range(3)]
    seqs = []
    for i in range(24):
        s = list(roots[i % 3])
        for p in rng.sample(range(400), 6):
            s[p] = rng.choice("ACGT")
        seqs.append("".join(s)[: rng.randint(120, 400)])  # some shorter than one window
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "s.txt"), "w") as f:
            f.write("\n".join(seqs) + "\n")
        r = subprocess.run([os.path.join(out, "selftest"), os.path.join(tmp, "s.txt"), "5",
                            os.path.join(tmp, "w.bin"), os.path.join(tmp, "m.txt")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        win = np.fromfile(os.path.join(tmp, "w.bin"), np.int16).reshape(-1, 1024)
        rows = [l.split() for l in open(os.path.join(tmp, "m.txt")).read().splitlines()]
    per_seq = [orc.window_segments([s], 150, 10) for s in seqs]
    ref_win, _ = orc.encode([w for ws in per_seq for w in ws], 1024, 8)
    assert np.array_equal(win, ref_win)
    half = len(seqs) // 2
    q_rows, db_rows, pos = [], [], 0
    for i, ws in enumerate(per_seq):
        if i < half and ws:
            q_rows.append(pos)
        if i >= half:
            db_rows.extend(range(pos, pos + len(ws)))
        pos += len(ws)
    s, idx, _, _ = orc.topk(ref_win[q_rows], ref_win[db_rows], 5, orc.SCORE_COS)
    got_idx = np.array([[int(r[2]) for r in rows if int(r[0]) == q] for q in range(len(q_rows))])
    got_s = np.array([[float(r[3]) for r in rows if int(r[0]) == q] for q in range(len(q_rows))], np.float32)
    assert np.array_equal(got_idx, idx)
    assert np.array_equal(got_s, s)
