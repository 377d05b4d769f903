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


def _mutate(rng, s, rate):
    s = list(s)
    for p in range(len(s)):
        if rng.random() < rate:
            s[p] = rng.choice([b for b in "ACGT" if b != s[p]])
    return "".join(s)


def make_reads(path, n_reads, window, seed):
    """reads.fasta beside the taxonomy: n_reads distinct reads cut from
    species sequences (lengths window, window/2 and 3*window/2, 1% substitution),
    plus an unrelated random read and one with an N.  Returns its path."""
    import random
    rng = random.Random(seed)
    seq_dir = os.path.join(path, "sequences_by_category")
    species = sorted(f for f in os.listdir(seq_dir) if f.startswith("s__"))
    reads, seen = [], set()
    while len(reads) < n_reads:
        sp = rng.choice(species)
        with open(os.path.join(seq_dir, sp)) as f:
            seqs = [l.strip() for l in f if l.strip() and not l.startswith(">")]
        s = rng.choice(seqs)
        n = rng.choice([window, window, window // 2, window + window // 2])
        start = rng.randrange(0, len(s) - n + 1)
        r = _mutate(rng, s[start:start + n], 0.01)
        if r not in seen:
            seen.add(r)
            reads.append(("read%d %s" % (len(reads), sp[:-6]), r))
    reads.append(("random", "".join(rng.choice("ACGT") for _ in range(window))))
    r = list(reads[0][1])
    r[len(r) // 3] = "N"
    reads.append(("with_n", "".join(r)))
    out = os.path.join(path, "reads.fasta")
    with open(out, "w") as f:
        for name, r in reads:
            f.write(">%s\n%s\n" % (name, r))
    return out


if __name__ == "__main__":
    # python tests/golden/taxonomy_fixture.py <dir> <n_leaves> <per_species> <seed> [<n_reads> <window> <read_seed>]
    # writes the taxonomy (and reads.fasta) into <dir>, for timing the applications by hand
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(os.path.dirname(here))
    sys.path.insert(0, os.path.join(root, "bacterial-classification_gb300"))
    import build as pkg_build
    pkg_build.build()
    import hdc_gb300
    a = sys.argv[1:]
    os.makedirs(a[0], exist_ok=True)
    make_taxonomy_dir(a[0], hdc_gb300, int(a[1]), int(a[2]), int(a[3]))
    if len(a) > 4:
        make_reads(a[0], int(a[4]), int(a[5]), int(a[6]))
    print(input_digest(a[0]) if len(a) <= 4 else a[0])
