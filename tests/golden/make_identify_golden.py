"""Golden output of the reference's identify application
(targets/identify.cpp, built with precompute off by
oracle/build_ref_identify.sh) on the synthetic taxonomy of
taxonomy_fixture.py after the reference's own propagate-children ran on it,
for the reads of taxonomy_fixture.make_reads.  Stores the digest of the
propagated taxonomy and the text identify writes to its output file.  Needs
the reference checkout; run from the repo root:
    python tests/golden/make_identify_golden.py"""
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "bacterial-classification_gb300"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as pkg_build  # noqa: E402
import hdc_gb300 as H  # noqa: E402
from taxonomy_fixture import input_digest, make_reads, make_taxonomy_dir  # noqa: E402

CASES = [dict(dim=1024, kmer=6, window=150, step=10, n_leaves=40, per_species=2, seed=71, n_reads=40, read_seed=5),
         dict(dim=2048, kmer=8, window=150, step=10, n_leaves=60, per_species=3, seed=72, n_reads=30, read_seed=6)]


def sh(script, c):
    return subprocess.check_output(["sh", os.path.join(ROOT, "oracle", script), str(c["dim"]), str(c["kmer"]),
                                    str(c["window"]), str(c["step"])], text=True).strip()


def main():
    pkg_build.build()
    out = []
    for c in CASES:
        prop, ident = sh("build_ref_propagate.sh", c), sh("build_ref_identify.sh", c)
        with tempfile.TemporaryDirectory() as tmp:
            seq_dir, tax = make_taxonomy_dir(tmp, H, c["n_leaves"], c["per_species"], c["seed"])
            subprocess.run([prop, seq_dir, tax], capture_output=True, check=True)
            digest = input_digest(tmp)
            reads = make_reads(tmp, c["n_reads"], c["window"], c["read_seed"])
            res = os.path.join(tmp, "result.txt")
            open(res, "w").close()
            t0 = time.time()
            subprocess.run([ident, seq_dir, tax, reads, res], stdout=subprocess.DEVNULL, check=True)
            dt = time.time() - t0
            text = open(res).read()
        out.append(dict(case=c, propagated_sha256=digest, output=text, reference_seconds=round(dt, 2)))
        print(c, "%.1f s" % dt)
        print(text[:400])
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "identify.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
