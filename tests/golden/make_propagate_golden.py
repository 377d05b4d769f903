"""Golden output of the reference's propagate-children application: run the
reference binary (oracle/build_ref_propagate.sh) on the synthetic taxonomy
of taxonomy_fixture.py and store the sha256 of every FASTA file it appended
to.  Needs the reference checkout; run from the repo root:
    python tests/golden/make_propagate_golden.py"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "bacterial-classification_gb300"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as pkg_build  # noqa: E402
import hdc_gb300 as H  # noqa: E402
from taxonomy_fixture import fasta_digest, input_digest, make_taxonomy_dir  # noqa: E402

CASES = [dict(dim=1024, kmer=6, window=150, step=10, n_leaves=40, per_species=2, seed=71),
         dict(dim=2048, kmer=8, window=150, step=10, n_leaves=60, per_species=3, seed=72)]


def main():
    pkg_build.build()
    out = []
    for c in CASES:
        exe = subprocess.check_output(["sh", os.path.join(ROOT, "oracle", "build_ref_propagate.sh"), str(c["dim"]),
                                       str(c["kmer"]), str(c["window"]), str(c["step"])], text=True).strip()
        with tempfile.TemporaryDirectory() as tmp:
            seq_dir, tax = make_taxonomy_dir(tmp, H, c["n_leaves"], c["per_species"], c["seed"])
            before = fasta_digest(seq_dir)
            digest = input_digest(tmp)
            r = subprocess.run([exe, seq_dir, tax], capture_output=True, text=True, check=True)
            after = fasta_digest(seq_dir)
        changed = {k: hashlib.sha256(v.encode()).hexdigest() for k, v in after.items() if before.get(k) != v}
        total = int(r.stdout.strip().split("Propogated:")[-1])
        out.append(dict(case=c, input_sha256=digest, appended_files=changed, total=total))
        print(c, "appended", total, "to", len(changed), "files")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "propagate_children.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
