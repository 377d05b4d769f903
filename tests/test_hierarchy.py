"""The drop-in's Hierarchy (dropin/hierarchy.cpp, the taxonomy tree and FASTA
store of the GPU applications) against the reference's own src/hierarchy.cpp,
compiled unchanged: the same driver (tests/hierarchy_dump.cpp) built against
each prints identical orders, children, sequences and appended files for the
synthetic taxonomy of the application tests and for a hand-written index with
the format's edge cases.  Build and run on the CPU; skipped without the
reference checkout."""
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

from oracle.build import REF_ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DROPIN = os.path.join(ROOT, "bacterial-classification_gb300", "dropin")
sys.path.insert(0, os.path.join(HERE, "golden"))

EDGE_INDEX = (
    "header\tignored\tk__X;p__Y\n"
    "a\ts__One\tk__Bacteria; p__Firmi cutes;c__Bacilli;o__;f__Fam One;g__G1;s__G1 sp\n"
    "\n"
    "b\ts__Two\t  k__Bacteria;p__Firmi cutes;c__Bacilli;o__Ord;f__Fam Two;g__G2;s__G2 sp;\n"
    "c\tonly two fields\n"
    "d\tno taxonomy\t\n"
    "e\ts__Three\tk__Bacteria;p__Proteo;c__Gamma;o__Ent;f__Ent;g__Esch;s__E coli\textra\tfields\n"
    "f\ts__Four\tk__Bacteria;p__Proteo;c__Gamma;o__Ent;f__Ent;g__Salm;s__S enterica\r\n"
    "g\ts__Five\tk__Bacteria;p__Proteo;c__Gamma;o__Ent;f__Ent;g__Esch;s__E albertii\n"
    "h\tno marks\tBacteria;Proteo;;__;x__\n"
    "i\ts__Six\tk__Bacteria;p__Actino;c__Act;o__Strep;f__Strep;g__Strep;s__S griseus")

EDGE_FASTA = {
    "s__G1_sp": ">a\nACGT\nAC\n>b\n>c\nGG\n",
    "s__E_coli": ">x\nAAAA\n>y\nCCCC",  # no final newline
    "g__Esch": "",
    "s__S_griseus": "TTTT\n>z\nGGGG\n\n>w\n",  # a record before the first header, an empty record
}


def _build(tmp, impl_src, name):
    exe = os.path.join(tmp, name)
    subprocess.check_call(["g++", "-O1", "-std=c++20", "-I" + os.path.dirname(impl_src),
                           os.path.join(HERE, "hierarchy_dump.cpp"), impl_src, "-o", exe])
    return exe


def _run(exe, tree_dir, cats):
    seq_dir = os.path.join(tree_dir, "sequences_by_category")
    r = subprocess.run([exe, seq_dir, os.path.join(tree_dir, "taxonomy_index.tsv")] + cats, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _edge_dir(path):
    seq_dir = os.path.join(path, "sequences_by_category")
    os.makedirs(seq_dir)
    with open(os.path.join(path, "taxonomy_index.tsv"), "w", newline="") as f:
        f.write(EDGE_INDEX)
    for name, text in EDGE_FASTA.items():
        with open(os.path.join(seq_dir, name + ".fasta"), "w", newline="") as f:
            f.write(text)


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_ROOT, "src", "hierarchy.cpp")),
                    reason="reference checkout absent")
@pytest.mark.parametrize("case", ["synthetic", "edges"])
def test_hierarchy_matches_reference(case):
    from taxonomy_fixture import make_taxonomy_dir
    import hdc_synth
    import build as pkg_build
    pkg_build.build_synth()
    with tempfile.TemporaryDirectory() as tmp:
        ref_exe = _build(tmp, os.path.join(REF_ROOT, "src", "hierarchy.cpp"), "dump_ref")
        our_exe = _build(tmp, os.path.join(DROPIN, "hierarchy.cpp"), "dump_ours")
        src = os.path.join(tmp, "tree")
        if case == "synthetic":
            make_taxonomy_dir(src, hdc_synth, 300, 2, 71)
            cats = ["s__S3", "g__G1", "p__P0"]
        else:
            _edge_dir(src)
            cats = ["s__G1 sp", "s__E_coli", "g__Esch"]
        outs = []
        for exe in (ref_exe, our_exe):
            work = os.path.join(tmp, "run_" + os.path.basename(exe))
            shutil.copytree(src, work)
            outs.append(_run(exe, work, cats))
        assert outs[0].count("\n") > 20
        assert outs[0] == outs[1]
