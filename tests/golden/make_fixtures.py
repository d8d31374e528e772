"""Regenerates tests/golden/reference_scans.npz from the reference's own test clouds.

Reads tests/data/scan.2d.txt, scan.3d.txt and scan.3d.large.txt of libnabo
(the clouds its CTest suite validates on, tests/CMakeLists.txt:9-14) with
the reference's parsing rule (tests/helpers.h:46-80: tokens separated by
space, tab, comma or semicolon; the first line fixes the dimension; values
parsed as double), and stores them as float64 arrays of shape (n, dim).
Run in a checkout that has the reference next to it:

    python tests/golden/make_fixtures.py /path/to/libnabo
"""
import os
import re
import sys

import numpy as np

NAMES = ("scan.2d.txt", "scan.3d.txt", "scan.3d.large.txt")


def load_reference_txt(path: str) -> np.ndarray:
    data, dim = [], None
    with open(path) as f:
        for line in f:
            toks = [t for t in re.split(r"[ \t,;]+", line.strip()) if t]
            if dim is None:
                dim = len(toks)
            data.extend(float(t) for t in toks)
    return np.asarray(data, dtype=np.float64).reshape(-1, dim)


def main(ref_root: str) -> None:
    out = {}
    for name in NAMES:
        arr = load_reference_txt(os.path.join(ref_root, "tests", "data", name))
        out[name.replace(".txt", "").replace(".", "_")] = arr
        print(name, arr.shape)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_scans.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py /path/to/libnabo")
    main(sys.argv[1])
