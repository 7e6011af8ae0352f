"""Pin the snapshot-file layout on the reference's own Python readers.

Writes a seeded 2D and a seeded 3D state with openmhd_gb300.fileio (the C ABI
writer, omhd_fileio_output), reads each file back with the reference's readers
(visualization/openmhd2d.py and visualization/openmhd3d.py, `data_read`),
checks here that they return exactly the written time, coordinates, the five
U planes they keep (rho, B, psi) and the four V planes, and stores what they
returned together with the SHA-256 of each file in
tests/golden/fileio_reference_reader.npz.  tests/test_fileio.py writes the same
states again and checks the file bytes and our reader against that record.

    python tests/golden/make_fileio_golden.py <path of the OpenMHD checkout>
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "fileio_reference_reader.npz")
SHAPES = {2: (6, 7), 3: (5, 4, 6)}  # (jx, ix) and (kx, jx, ix)
TIME = {2: 0.625, 3: 1.75}


def seeded_case(nd: int):
    """The state written for an nd-dimensional file: (t, x, y, z, U, V)."""
    shape = SHAPES[nd]
    rng = np.random.default_rng(20 + nd)
    U = rng.standard_normal((9,) + shape)
    V = rng.standard_normal((4,) + shape)
    x = np.linspace(-1.0, 1.0, shape[-1])
    y = np.linspace(0.5, 2.0, shape[-2])
    z = np.linspace(3.0, 4.0, shape[0]) if nd == 3 else None
    return TIME[nd], x, y, z, U, V


def write_case(nd: int, path: str) -> str:
    from openmhd_gb300 import fileio

    t, x, y, z, U, V = seeded_case(nd)
    fileio.write(path, t, x, y, U, V, z=z)
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def main(ref: str) -> None:
    from openmhd_gb300.build import build

    build()
    sys.path.insert(0, os.path.join(ref, "visualization"))
    import openmhd2d
    import openmhd3d

    rec = {}
    with tempfile.TemporaryDirectory() as d:
        for nd in (2, 3):
            path = os.path.join(d, f"field-0000{nd}.dat")
            rec[f"sha256_{nd}d"] = np.array(write_case(nd, path))
            t, x, y, z, U, V = seeded_case(nd)
            if nd == 2:
                xr, yr, tr, data = openmhd2d.data_read(path, silent=True)
                field = lambda a: a.T  # noqa: E731  (jx, ix) -> reader's (ix, jx)
            else:
                xr, yr, zr, tr, data = openmhd3d.data_read(path, silent=True)
                field = lambda a: a.transpose(2, 1, 0)  # noqa: E731
                assert np.array_equal(zr, z)
                rec["z_3d"] = zr
            assert tr == t and np.array_equal(xr, x) and np.array_equal(yr, y)
            for q in range(4):  # reader slots 0-3: the four V planes
                assert np.array_equal(data[..., q], field(V[q]))
            for q in range(4, 9):  # reader slots 4-8: U planes rho, bx, by, bz, psi
                assert np.array_equal(data[..., q], field(U[q]))
            rec[f"t_{nd}d"] = np.array(tr)
            rec[f"x_{nd}d"] = xr
            rec[f"y_{nd}d"] = yr
            rec[f"data_{nd}d"] = data
    np.savez_compressed(OUT, **rec)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fileio_golden.py <path of the OpenMHD checkout>")
    main(sys.argv[1])
