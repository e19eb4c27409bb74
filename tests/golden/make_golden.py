"""Generates the golden fixtures under tests/golden/ from the reference tree.

Run once where the reference source tree is checked out, with its path as
the only argument; the outputs are committed, and no test reads the
reference at run time.

Outputs
  arisong.npz   the Arisong alignment of tutorial/updated_Arisong.sto in Easel
                RNA digital codes (A,C,G,U=0..3, gap=4, degenerate 5..14, N=15,
                '*'=16, '~'=17), unfiltered, plus its SS_cons string.
  arisong_gtp.json  the GTp table R-scape's tutorial documents for this
                alignment (documentation/tutorial.tex:186-212): alignment
                coordinates (1-based), score, E-value, p-value, nseff.
"""
import json
import os
import re
import sys

import numpy as np

EASEL_RNA = "ACGU-RYMKSWHBVDN*~"


def digitize(seq):
    out = np.empty(len(seq), dtype=np.uint8)
    for k, ch in enumerate(seq.upper()):
        if ch in ".-_":
            out[k] = 4
        elif ch == "T":
            out[k] = 3
        else:
            out[k] = EASEL_RNA.index(ch)
    return out


def read_stockholm(path):
    names, seqs, ss = [], {}, ""
    with open(path) as fh:
        for line in fh:
            line = line.rstrip("\n")
            if not line or line.startswith("//"):
                continue
            if line.startswith("#=GC SS_cons"):
                ss += line.split()[-1]
                continue
            if line.startswith("#"):
                continue
            name, seq = line.split()
            if name not in seqs:
                names.append(name)
                seqs[name] = ""
            seqs[name] += seq
    return names, [seqs[n] for n in names], ss


def read_tutorial_table(path):
    """The 11-row GTp table that follows the two-set command in the tutorial."""
    rows = []
    with open(path) as fh:
        lines = fh.read().splitlines()
    start = None
    for k, line in enumerate(lines):
        if "R-scape -s tutorial/updated" in line:
            start = k
            break
    pat = re.compile(r"^\*\s+(\d+)\s+(\d+)\s+([0-9.]+)\s+([0-9.e+-]+)\s+([0-9.e+-]+)\s+\d+\s+[0-9.]+\s+([0-9.]+)")
    for line in lines[start:]:
        m = pat.match(line)
        if m:
            rows.append(dict(left=int(m.group(1)), right=int(m.group(2)), score=float(m.group(3)),
                             evalue=float(m.group(4)), pvalue=float(m.group(5)), nseff=float(m.group(6))))
        elif rows and line.startswith("\\end{sreoutput}"):
            break
    return rows


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <R-scape source tree>")
    ref = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    names, seqs, ss = read_stockholm(os.path.join(ref, "tutorial", "updated_Arisong.sto"))
    ax = np.stack([digitize(s) for s in seqs])
    np.savez_compressed(os.path.join(here, "arisong.npz"), ax=ax, ss_cons=np.array(ss))
    rows = read_tutorial_table(os.path.join(ref, "documentation", "tutorial.tex"))
    with open(os.path.join(here, "arisong_gtp.json"), "w") as fh:
        json.dump({"source": "documentation/tutorial.tex:186-212", "nseq": 95, "alen_filtered": 66,
                   "alen": int(ax.shape[1]), "pairs": rows}, fh, indent=1)
    print("nseq %d alen %d, %d golden pairs" % (ax.shape[0], ax.shape[1], len(rows)))


if __name__ == "__main__":
    main()
