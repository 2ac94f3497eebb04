"""Regenerate the golden fixtures in this folder from the reference checkout.

Run once in a container where the reference tree is mounted, giving its path:

    python tests/golden/make_golden.py <reference checkout>

It copies the reference's small binary CSR fixtures (Tests/*) byte for byte
and transcribes the known answers its readme files record into
``golden.json``:

  * Tests/spike/penta_10.readme:1-21 -- the full 8x8 reduced system R and its
    right-hand side for penta_10.bin with p = 2, b = 1 (5 decimals), and the
    SPIKE error 3.51E-16;
  * Tests/solve_small/readme.txt:1-4 -- the solution of tridiagonal.bin with
    b = 1 (3 decimals) and its relative residual 1.110223E-16;
  * Tests/bandwidth/readme.txt:1-9 -- ku = 2, kl = 4 for banded.bin (the same
    check as OpenMP/bandwidth.c:32-41);
  * Tests/split/Readme.txt + OpenMP/split.c:43-74 -- block1.bin and block2.bin
    are A[0:5,0:5] and A[5:10,5:10] of matrix.bin.

Nothing at test time reads the reference tree; the tests read only this folder.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

FIXTURES = [
    "spike/penta_10.bin", "spike/penta_15.bin", "spike/penta_15.z",
    "solve_small/tridiagonal.bin", "bandwidth/banded.bin",
    "split/matrix.bin", "split/block1.bin", "split/block2.bin",
    "pentadiagonal/small.bin", "heptadiagonal/small.bin", "heptadiagonal/medium.bin",
    "dummy/tridiagonal.bin", "complex16/penta_15.z", "complex16/penta_1k.z",
]


def _floats(text):
    return [float(v) for v in re.findall(r"-?\d+\.\d*(?:[eE][-+]?\d+)?", text)]


def main(ref_root: str) -> None:
    tests = os.path.join(ref_root, "Tests")
    for rel in FIXTURES:
        dst = os.path.join(HERE, rel.replace("/", "__"))
        shutil.copyfile(os.path.join(tests, rel), dst)

    golden = {}
    txt = open(os.path.join(tests, "spike/penta_10.readme")).read()
    rpart, rest = txt.split("RHS of the reduced system")
    rhs_part, err_part = rest.split("00-th RHS")
    R = _floats(rpart)
    rhs = _floats(rhs_part)
    assert len(R) == 64 and len(rhs) == 8, (len(R), len(rhs))
    golden["penta_10"] = {
        "file": "spike__penta_10.bin", "partitions": 2, "b": 1.0, "decimals": 5,
        "R": [R[i * 8:(i + 1) * 8] for i in range(8)], "rhs": rhs,
        "spike_error": float(re.search(r"SPIKE error:\s*([0-9.Ee+-]+)", err_part).group(1)),
    }

    txt = open(os.path.join(tests, "solve_small/readme.txt")).read()
    first = txt.splitlines()[0]
    golden["solve_small"] = {
        "file": "solve_small__tridiagonal.bin", "b": 1.0, "decimals": 3,
        "x": [float(v) for v in first.strip("[] \n").split()],
        "relative_residual": float(re.search(r"Relative residual\s+([0-9.Ee+-]+)", txt).group(1)),
    }

    txt = open(os.path.join(tests, "bandwidth/readme.txt")).read()
    golden["bandwidth"] = {
        "file": "bandwidth__banded.bin",
        "ku": int(re.search(r"upper bandwidth\s*:\s*(\d+)", txt).group(1)),
        "kl": int(re.search(r"lower bandwidth\s*:\s*(\d+)", txt).group(1)),
    }
    golden["split"] = {
        "matrix": "split__matrix.bin",
        "blocks": [["split__block1.bin", 0, 5], ["split__block2.bin", 5, 10]],
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print("wrote", len(FIXTURES), "fixtures and golden.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
