"""A seeded synthetic taxonomy in the reference's on-disk format
(db_inductors/induct_silva.py:156-179): taxonomy_index.tsv with a header
and one line per sequence (id, lowest rank, "k__...;p__...;...;s__..."), and
sequences_by_category/<category>.fasta -- the species' sequences, empty
files for every internal node.  Shared by the golden-vector maker and the
GPU test so both build the same directory."""
import os

import numpy as np

RANKS = ["p", "c", "o", "f", "g", "s"]


def make_taxonomy_dir(path, H, n_leaves=40, per_species=2, seed=71):
    tree = H.synth_tree(seed, n_leaves)
    copies = H.synth_copies(seed + 1, tree, per_species, 0.02)
    b = 1
    while b ** 6 < n_leaves:
        b += 1
    seq_dir = os.path.join(path, "sequences_by_category")
    os.makedirs(seq_dir, exist_ok=True)
    lines = ["id\tlowest\ttaxonomy"]
    nodes = set()
    for j in range(n_leaves):
        lineage = ["k__Bacteria"] + ["%s__%s%d" % (r, r.upper(), j // b ** (5 - i)) for i, r in enumerate(RANKS)]
        nodes.update(lineage)
        for c in range(per_species):
            lines.append("seq%d_%d\t%s\t%s" % (j, c, lineage[-1], ";".join(lineage)))
        with open(os.path.join(seq_dir, lineage[-1] + ".fasta"), "w") as f:
            for c in range(per_species):
                f.write(">seq%d_%d\n%s\n" % (j, c, copies.get(j * per_species + c)))
    for n in nodes:
        fp = os.path.join(seq_dir, n + ".fasta")
        if not os.path.exists(fp):
            open(fp, "w").close()
    with open(os.path.join(path, "taxonomy_index.tsv"), "w") as f:
        f.write("\n".join(lines) + "\n")
    return seq_dir, os.path.join(path, "taxonomy_index.tsv")


def fasta_digest(seq_dir):
    """{file name: content} of every non-empty FASTA."""
    out = {}
    for name in sorted(os.listdir(seq_dir)):
        with open(os.path.join(seq_dir, name)) as f:
            text = f.read()
        if text:
            out[name] = text
    return out


def input_digest(path):
    """sha256 over taxonomy_index.tsv and every FASTA (name and content)."""
    import hashlib
    h = hashlib.sha256()
    with open(os.path.join(path, "taxonomy_index.tsv"), "rb") as f:
        h.update(f.read())
    seq_dir = os.path.join(path, "sequences_by_category")
    for name in sorted(os.listdir(seq_dir)):
        h.update(name.encode() + b"\0")
        with open(os.path.join(seq_dir, name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()
