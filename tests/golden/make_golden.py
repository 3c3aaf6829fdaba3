"""Convert the reference's golden stiffness matrices into small numpy fixtures.

Reads the PETSc-binary AIJ files that Underworld/Rheology/tests/ViscousSuite.c compares against
(Underworld/Rheology/tests/expected/test*2D.matrix, testArrheniusWithLimiter.matrix) and the one
StgFEM's isoviscous assembly test compares against (StgFEM/Assembly/tests/expected/
testIsoviscousSiffness.matrix, the file's own spelling) from the read-only reference tree, and
writes them as CSR arrays to tests/golden/viscous_golden.npz.
Run once with the reference tree's path as the only argument; the fixtures are committed.

PETSc binary layout (big-endian): int32 MAT_FILE_CLASSID (1211216), int32 rows, int32 cols,
int32 total nnz, int32 row lengths[rows], int32 column indices[nnz], float64 values[nnz].
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit(f"usage: python {os.path.basename(__file__)} <path of the Underworld 1.x source tree>")
REF = sys.argv[1]
SRC = os.path.join(REF, "Underworld/Rheology/tests/expected")
NAMES = ["testMaterialViscosity2D", "testArrhenius2D", "testArrheniusWithLimiter", "testFrankKamenetskii2D"]
SOURCES = {name: os.path.join(SRC, name + ".matrix") for name in NAMES}
SOURCES["testIsoviscousSiffness"] = os.path.join(REF, "StgFEM/Assembly/tests/expected/testIsoviscousSiffness.matrix")


def read_petsc_aij(path):
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw, dtype=">i4", count=4)
    assert hdr[0] == 1211216, "not a PETSc Mat file"
    m, n, nz = int(hdr[1]), int(hdr[2]), int(hdr[3])
    off = 16
    rowlen = np.frombuffer(raw, dtype=">i4", count=m, offset=off).astype(np.int64)
    off += 4 * m
    cols = np.frombuffer(raw, dtype=">i4", count=nz, offset=off).astype(np.int64)
    off += 4 * nz
    vals = np.frombuffer(raw, dtype=">f8", count=nz, offset=off).astype(np.float64)
    rowptr = np.concatenate([[0], np.cumsum(rowlen)])
    return m, n, rowptr, cols, vals


def main():
    out = {}
    for name, path in SOURCES.items():
        m, n, rp, ci, v = read_petsc_aij(path)
        out[name + "_shape"] = np.array([m, n])
        out[name + "_rowptr"] = rp
        out[name + "_cols"] = ci
        out[name + "_vals"] = v
        print(name, m, n, len(v))
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "viscous_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
