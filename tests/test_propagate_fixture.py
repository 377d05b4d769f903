"""The synthetic taxonomy behind the propagate-children golden vectors is
reproducible: rebuilding it gives the bytes the reference binary ran on."""
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from taxonomy_fixture import input_digest, make_taxonomy_dir  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "propagate_children.json")))


def test_fixture_reproducible(hdc):
    for g in GOLDEN:
        c = g["case"]
        with tempfile.TemporaryDirectory() as tmp:
            make_taxonomy_dir(tmp, hdc, c["n_leaves"], c["per_species"], c["seed"])
            assert input_digest(tmp) == g["input_sha256"]
