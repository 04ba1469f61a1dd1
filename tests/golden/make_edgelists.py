"""Generate the edge-list fixtures: tests/golden/edgelists/<name>.el and
tests/golden/edgelists.json, the SHA-256 of the .bcsr the reference's own
converter (tools/convert_from_txt.cc, compiled in place into
oracle/_ref/converter_txt by ``make -C oracle ref``) writes for each.

    python tests/golden/make_edgelists.py

The files mix what the converter has to handle: comment and header lines,
blank lines and lines with leading blanks (skipped), tab and space
separators, CRLF line ends, a third column, self loops, repeated and reversed
edges, and sparse ids with gaps (isolated ids removed).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "edgelists")
EXE = os.path.join(ROOT, "oracle", "_ref", "converter_txt")


def files():
    f = {}
    f["tiny"] = ("% a KONECT-style header\n# a comment\n1 2\n2 1\n2 3\n3 3\n\n 7 9\n1\t5\n5 1\n9 2\n"
                 "9 2\n4 4\n")
    rng = np.random.default_rng(7)
    lines = ["# sparse ids, duplicates, self loops, weights\n"]
    ids = np.sort(rng.choice(1_000_000, 900, replace=False))
    for _ in range(3000):
        a, b = (int(x) for x in rng.choice(ids, 2))
        if rng.random() < 0.02:
            b = a
        sep = "\t" if rng.random() < 0.3 else " "
        tail = " %.3f" % rng.random() if rng.random() < 0.2 else ""
        end = "\r\n" if rng.random() < 0.1 else "\n"
        lines.append(f"{a}{sep}{b}{tail}{end}")
        if rng.random() < 0.05:
            lines.append(f"{b} {a}\n")
    f["sparse3000"] = "".join(lines)
    lines = [f"0 {v}\n" for v in range(1, 400)] + [f"{v} {v + 1}\n" for v in range(400, 900)]
    f["star_chain"] = "".join(lines)
    rng = np.random.default_rng(11)
    e = rng.integers(0, 3000, (8000, 2))
    f["dense8000"] = "".join(f"{a} {b}\n" for a, b in e)
    return f


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OUT)
    rows = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, text in files().items():
            with open(os.path.join(OUT, name + ".el"), "w", newline="") as fh:
                fh.write(text)
            el = os.path.join(tmp, name + ".el")
            shutil.copy(os.path.join(OUT, name + ".el"), el)
            subprocess.run([EXE, el], check=True, capture_output=True)
            raw = open(os.path.join(tmp, name + ".bcsr"), "rb").read()
            V = int(np.frombuffer(raw, np.uint32, 1)[0])
            E = int(np.frombuffer(raw, np.uint64, 1, 4)[0])
            rows[name] = {"sha256": hashlib.sha256(raw).hexdigest(), "V": V, "E": E}
    with open(os.path.join(HERE, "edgelists.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_edgelists.py", "reference": "tools/convert_from_txt.cc",
                   "bcsr": rows}, fh, indent=1)
    print(rows)


if __name__ == "__main__":
    main()
