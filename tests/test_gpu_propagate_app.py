"""propagate-children end to end: the GPU driver (dropin/propagate_gpu.cpp
over hdc_encode_segments + hdc_propagate_greedy, with the Hierarchy mirror)
run on the synthetic taxonomy must append exactly what the reference's own
targets/propogate-children.cpp appended (sha256 of every changed FASTA and the
printed total, recorded by tests/golden/make_propagate_golden.py)."""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from taxonomy_fixture import fasta_digest, input_digest, make_taxonomy_dir  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(HERE, "golden", "propagate_children.json")))


@pytest.mark.parametrize("g", GOLDEN, ids=lambda g: "D%d_k%d" % (g["case"]["dim"], g["case"]["kmer"]))
def test_propagate_children_matches_reference(hdc, cuda, g):
    import build as pkg_build
    c = g["case"]
    out = pkg_build.build_dropin(c["dim"], c["kmer"], c["window"], c["step"])
    with tempfile.TemporaryDirectory() as tmp:
        seq_dir, tax = make_taxonomy_dir(tmp, hdc, c["n_leaves"], c["per_species"], c["seed"])
        assert input_digest(tmp) == g["input_sha256"]
        before = fasta_digest(seq_dir)
        r = subprocess.run([os.path.join(out, "propagate-children"), seq_dir, tax], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        after = fasta_digest(seq_dir)
    changed = {k: hashlib.sha256(v.encode()).hexdigest() for k, v in after.items() if before.get(k) != v}
    assert int(r.stdout.strip().split("Propogated:")[-1]) == g["total"]
    assert changed == g["appended_files"]
