#!/usr/bin/env python3
"""Generate tests/golden/io/ (small synthetic Matrix Market and CSV inputs,
seeded) and tests/golden/io_golden.npz (what the REFERENCE readers make of
them: readMtx_info_and_coo + Converter_Coo2Csr, src/readMTX.c:8-135 and
src/matrixType.c:4-52, and parseCSV, src/common.c:16-48, compiled by
oracle/build.py).  The reference ships no matrices or RHS files of its own.
Needs the reference tree; run from the repo root:

    python tests/golden/make_io_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

IO = os.path.join(HERE, "io")


def lap2d_lower(N):
    """Lower triangle (i >= j) of the 2-D 5-point Laplacian on an N x N grid."""
    ent = []
    for y in range(N):
        for x in range(N):
            r = y * N + x
            ent.append((r, r, 4.0))
            if x > 0:
                ent.append((r, r - 1, -1.0))
            if y > 0:
                ent.append((r, r - N, -1.0))
    return ent


def write_mtx(name, banner, nr, nc, ent, comments=("% synthetic test matrix",), fmt="%.17g"):
    with open(os.path.join(IO, name), "w") as f:
        f.write(banner + "\n")
        for c in comments:
            f.write(c + "\n")
        f.write("%d %d %d\n" % (nr, nc, len(ent)))
        for e in ent:
            if len(e) == 2:
                f.write("%d %d\n" % (e[0] + 1, e[1] + 1))
            else:
                f.write(("%d %d " + fmt + "\n") % (e[0] + 1, e[1] + 1, e[2]))


def main():
    os.makedirs(IO, exist_ok=True)
    rng = np.random.default_rng(7)
    out = {}
    # 1. symmetric real, lower triangle in shuffled order, two comment lines
    ent = lap2d_lower(12)
    ent = [ent[i] for i in rng.permutation(len(ent))]
    write_mtx("lap2d_12_sym.mtx", "%%MatrixMarket matrix coordinate real symmetric", 144, 144,
              ent, comments=("% 2-D 5-point Laplacian, 12 x 12 grid", "%"))
    # 2. general real, unsorted, one duplicate entry, upper-case tokens
    ent = [(int(rng.integers(0, 30)), int(rng.integers(0, 25)), float(rng.normal()))
           for _ in range(120)]
    ent.append(ent[5])
    write_mtx("general_30x25.mtx", "%%MatrixMarket MATRIX Coordinate REAL General", 30, 25, ent)
    # 3. pattern symmetric
    ent = sorted({(int(i), int(j)) for i, j in rng.integers(0, 15, (40, 2)) if i >= j})
    ent = [ent[i] for i in rng.permutation(len(ent))]
    write_mtx("pattern_15_sym.mtx", "%%MatrixMarket matrix coordinate pattern symmetric", 15,
              15, ent)
    # 4. integer general
    ent = [(int(rng.integers(0, 20)), int(rng.integers(0, 20)), int(rng.integers(-9, 10)))
           for _ in range(50)]
    write_mtx("integer_20.mtx", "%%MatrixMarket matrix coordinate integer general", 20, 20,
              ent, fmt="%d")
    # 5. skew-symmetric (read as stored)
    ent = [(i, j, float(rng.normal())) for i in range(1, 10) for j in range(i) if (i + j) % 3]
    write_mtx("skew_10.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric", 10, 10,
              ent)
    for name in sorted(os.listdir(IO)):
        if name.endswith(".mtx"):
            rp, ci, v, shape = O.ref_read_mtx(os.path.join(IO, name))
            key = name[:-4]
            out[key + "/rp"], out[key + "/ci"], out[key + "/v"] = rp, ci, v
            out[key + "/shape"] = np.array(shape)
    # 6. RHS files in the reference's RHS format (one row per line, %.18e, ',')
    B = rng.uniform(-1.0, 1.0, (144, 4))
    with open(os.path.join(IO, "rhs_144x4.csv"), "w") as f:
        for row in B:
            f.write(",".join("%.18e" % x for x in row) + "\n")
    out["rhs_144x4"] = O.ref_parse_csv(os.path.join(IO, "rhs_144x4.csv"), 144, 4)
    # fewer lines than requested: the reference leaves the rest zero
    with open(os.path.join(IO, "rhs_short.csv"), "w") as f:
        for row in B[:5, :3]:
            f.write(",".join("%.18e" % x for x in row) + "\n")
    out["rhs_short"] = O.ref_parse_csv(os.path.join(IO, "rhs_short.csv"), 8, 3)
    np.savez(os.path.join(HERE, "io_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
