"""identify end to end: the GPU application (dropin/identify_gpu.cpp over
hdc_encode_segments + hdc_identify, with the Hierarchy mirror) writes the
same result text as the reference's targets/identify.cpp (built with
precompute off, compute-semantics windows) on the synthetic taxonomy after
propagate-children, for the same reads (recorded by
tests/golden/make_identify_golden.py)."""
import json
import os
import subprocess
import sys
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from taxonomy_fixture import input_digest, make_reads, make_taxonomy_dir  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(HERE, "golden", "identify.json")))


@pytest.mark.parametrize("g", GOLDEN, ids=lambda g: "D%d_k%d" % (g["case"]["dim"], g["case"]["kmer"]))
def test_identify_matches_reference(hdc, cuda, g):
    import build as pkg_build
    c = g["case"]
    out = pkg_build.build_dropin(c["dim"], c["kmer"], c["window"], c["step"])
    with tempfile.TemporaryDirectory() as tmp:
        seq_dir, tax = make_taxonomy_dir(tmp, hdc, c["n_leaves"], c["per_species"], c["seed"])
        r = subprocess.run([os.path.join(out, "propagate-children"), seq_dir, tax], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert input_digest(tmp) == g["propagated_sha256"]
        reads = make_reads(tmp, c["n_reads"], c["window"], c["read_seed"])
        res = os.path.join(tmp, "result.txt")
        open(res, "w").close()
        r = subprocess.run([os.path.join(out, "identify"), seq_dir, tax, reads, res], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        text = open(res).read()
    assert text == g["output"]
