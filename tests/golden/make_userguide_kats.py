"""Extracts the printed sample outputs of the JADAMILU user guide into JSON.

The reference ships no test suite; its only result-pinning artefacts are the
sample outputs printed in Doc/userguide.ps (eigenvalues to 16 digits, residual
norms and MATVEC counts).  This script reads that PostScript as text, takes
the numbers between the known line anchors and writes userguide_kats.json.
Run it once where the reference is available:

    python tests/golden/make_userguide_kats.py <JADAMILU source tree>
"""
import json
import os
import re
import sys

# (name, first line, last line, sample program / matrix, driver parameters)
ANCHORS = [
    ("EXAMPLE1", 7598, 7613, dict(matrix="tridiag", diag_offset=-1.0, diag_scale=1.0, isearch=2, sigma=0.0,
                                  driver="dpjd")),
    ("EXAMPLE2", 7915, 7945, dict(matrix="tridiag", diag_offset=-1.0, diag_scale=1.0, isearch=0, driver="dpjd")),
    ("EXAMPLE5", 9335, 9385, dict(matrix="tridiag", diag_offset=-1.0, diag_scale=0.0, isearch=0,
                                  driver="dpjdrevcom", rank1=0.1)),
    ("EXAMPLE6", 9595, 9625, dict(matrix="tridiag", diag_offset=-1.0, diag_scale=0.0, isearch=0,
                                  driver="dpjdrevcom", rank1=0.1, icntl2=1)),
    ("EXAMPLE9", 12225, 12255, dict(matrix="tridiag", diag_offset=0.0, diag_scale=1.0, isearch=0,
                                    driver="dpjdrevcom_diag")),
    ("EXAMPLE10", 13120, 13170, dict(matrix="tridiag", diag_offset=0.0, diag_scale=1.0, isearch=0,
                                     driver="dpjdrevcom_diag", icntl1=2, icntl2=1)),
]

NUM = re.compile(r"\((-?\d\.\d{12,}E[-+]\d+)\)|(?<=[ )])(-?\d\.\d{12,}E[-+]\d+)")
MV = re.compile(r"needed:\)\d+ b\((\d+)\)|\((\d+)\)\d* b\(;\)")


def extract(lines):
    text = "".join(lines)
    eigs = [float(a or b) for a, b in NUM.findall(text)]
    m = re.search(r"MATVEC\)[^(]*\(needed:\)\s*\d+\s*b\((\d+)\)", text) or re.search(r"needed:\)\s*\d+\s*b\((\d+)\)", text)
    mv = int(m.group(1)) if m else None
    return eigs, mv


def main(ref):
    path = os.path.join(ref, "Doc", "userguide.ps")
    with open(path, "r", errors="replace") as f:
        lines = f.readlines()
    out = {}
    for name, a, b, meta in ANCHORS:
        eigs, mv = extract(lines[a - 1:b])
        out[name] = dict(eigenvalues=eigs[:5], matvec=mv, source=f"Doc/userguide.ps:{a}-{b}", **meta)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "userguide_kats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_userguide_kats.py <path of the JADAMILU source tree>")
    main(sys.argv[1])
