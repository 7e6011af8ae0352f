"""Snapshot files in the reference's layout (2D_basic/fileio.f90:16-115,
3D_basic/fileio.f90:16-122).  The CPU tests write through the C ABI with host
arrays and read back with an independent numpy reader that follows the
reference's record order (t, ix, jx[, kx], x, y[, z], nine U planes, four V
planes); the GPU tests write a solver's state and restart from it."""
import numpy as np
import pytest

from helpers import random_state


@pytest.fixture(scope="module")
def lib():
    from openmhd_gb300 import _lib
    from openmhd_gb300.build import build

    build()
    return _lib.load()


def numpy_reader(path, nd):
    """The reference's reader logic (openmhd2d.py data_read / fileio_input)."""
    with open(path, "rb") as f:
        t = np.fromfile(f, dtype=np.float64, count=1)[0]
        dims = np.fromfile(f, dtype=np.int32, count=nd)
        coords = [np.fromfile(f, dtype=np.float64, count=int(n)) for n in dims]
        n = int(np.prod(dims))
        U = np.fromfile(f, dtype=np.float64, count=9 * n).reshape((9,) + tuple(int(d) for d in dims[::-1]))
        V = np.fromfile(f, dtype=np.float64, count=4 * n).reshape((4,) + tuple(int(d) for d in dims[::-1]))
        rest = f.read()
    return t, dims, coords, U, V, rest


@pytest.mark.parametrize("nd", [2, 3])
def test_output_layout_and_input(lib, tmp_path, nd):
    from openmhd_gb300 import fileio

    shape = (7, 6) if nd == 2 else (5, 4, 6)
    U = random_state(shape, 3)
    V = np.random.default_rng(1).standard_normal((4,) + shape)
    x = np.linspace(0.0, 1.0, shape[-1])
    y = np.linspace(-1.0, 2.0, shape[-2])
    z = np.linspace(3.0, 4.0, shape[0]) if nd == 3 else None
    path = tmp_path / "field-00001.dat"
    fileio.write(path, 0.625, x, y, U, V, z=z)
    t, dims, coords, U2, V2, rest = numpy_reader(path, nd)
    assert t == 0.625 and rest == b""
    assert list(dims) == list(shape[::-1])
    assert np.array_equal(coords[0], x) and np.array_equal(coords[1], y)
    if nd == 3:
        assert np.array_equal(coords[2], z)
    assert np.array_equal(U2, U) and np.array_equal(V2, V)
    kx = shape[0] if nd == 3 else 1
    t3, x3, y3, z3, U3 = fileio.read(path, nd, shape[-1], shape[-2], kx)
    assert t3 == 0.625 and np.array_equal(U3, U) and np.array_equal(x3, x) and np.array_equal(y3, y)


def test_input_rejects_other_sizes(lib, tmp_path):
    from openmhd_gb300 import OmhdError, fileio

    U = random_state((6, 7), 1)
    path = tmp_path / "f.dat"
    fileio.write(path, 1.0, np.zeros(7), np.zeros(6), U, np.zeros((4, 6, 7)))
    with pytest.raises(OmhdError) as e:
        fileio.read(path, 2, 8, 6)
    assert e.value.code == 4  # OMHD_BAD_ARG, fileio.f90:77-82 "parameter mismatch"


def test_wrong_shapes_and_types_are_refused_before_the_library(lib, tmp_path):
    """The library trusts ix/jx/kx: coordinates, V or U that are smaller than
    the sizes U implies, or of another type, are refused in Python, and the C
    entry point refuses sizes below 1, before anything is read or written."""
    import ctypes as C

    import torch

    from openmhd_gb300 import fileio
    from openmhd_gb300.solver import OMHD_BAD_ARG

    U = random_state((6, 7), 3)
    path = tmp_path / "f.dat"
    x, y = np.zeros(7), np.zeros(6)
    bad = [
        dict(x=np.zeros(6), y=y, U=U),
        dict(x=x, y=np.zeros(5), U=U),
        dict(x=x, y=y, U=U, V=np.zeros((4, 6, 6))),
        dict(x=x, y=y, U=U[:8]),
        dict(x=x, y=y, U=random_state((5, 6, 7), 4)),  # 3D without z
        dict(x=x, y=y, U=random_state((5, 6, 7), 4), z=np.zeros(4)),
    ]
    for kw in bad:
        with pytest.raises(ValueError):
            fileio.write(path, 0.0, kw.pop("x"), kw.pop("y"), kw.pop("U"), **kw)
    with pytest.raises(TypeError):
        fileio.write(path, 0.0, x, y, torch.from_numpy(U).float())
    assert not path.exists()
    for sizes in ((2, 0, 6), (3, 7, 6, 0), (4, 7, 6)):
        with pytest.raises(ValueError):
            fileio.read(path, *sizes)
    t = C.c_double()
    buf = np.zeros(9 * 7 * 6)
    for nd, ix, jx, kx in ((2, 7, 0, 1), (3, 7, 6, 0), (3, -1, 6, 5)):
        st = lib.omhd_fileio_input(str(path).encode(), nd, ix, jx, kx, C.byref(t), buf.ctypes.data,
                                   buf.ctypes.data, buf.ctypes.data, buf.ctypes.data)
        assert st == OMHD_BAD_ARG, (nd, ix, jx, kx)


def test_input_reports_missing_and_truncated_files(lib, tmp_path):
    """A missing file and a file cut short in its header, coordinates or planes
    are reported as OMHD_IO_ERR (the reference's read would stop)."""
    from openmhd_gb300 import OmhdError, fileio
    from openmhd_gb300.solver import OMHD_IO_ERR

    U = random_state((6, 7), 2)
    path = tmp_path / "f.dat"
    fileio.write(path, 1.0, np.zeros(7), np.zeros(6), U, np.zeros((4, 6, 7)))
    data = path.read_bytes()
    with pytest.raises(OmhdError) as e:
        fileio.read(tmp_path / "missing.dat", 2, 7, 6)
    assert e.value.code == OMHD_IO_ERR
    for cut in (4, 8 + 4, 8 + 8 + 7 * 8 + 3, len(data) - 4 * 6 * 7 * 8 - 8):
        short = tmp_path / f"short{cut}.dat"
        short.write_bytes(data[:cut])
        with pytest.raises(OmhdError) as e:
            fileio.read(short, 2, 7, 6)
        assert e.value.code == OMHD_IO_ERR, cut


@pytest.mark.gpu
def test_solver_snapshot_and_restart(cuda_lib, tmp_path, oracle_mod):
    from openmhd_gb300 import Solver, orszag_tang

    cfg, model = orszag_tang(48)
    a = Solver(cfg).init_model(model)
    a.step(5)
    path = tmp_path / "field-00005.dat"
    a.write_snapshot(path)
    info = a.sync()
    t, dims, coords, U, V, rest = numpy_reader(path, 2)
    assert rest == b"" and t == info.t
    assert np.array_equal(U, a.get_state_numpy())
    assert np.array_equal(coords[0], a.coords()[0])
    Vo, st, _ = oracle_mod.u2v(U.copy(), 2)  # primitives as u2v.f90 computes them
    assert st == 0 and np.array_equal(V, Vo)
    # restart: continuing from the file equals continuing the run
    b = Solver(cfg).read_snapshot(path)
    a.step(4)
    b.step(4)
    ia, ib = a.sync(), b.sync()
    assert ia.t == ib.t
    assert np.array_equal(a.get_state_numpy(), b.get_state_numpy())


@pytest.mark.gpu
def test_run_with_output_restart_from_newest_file(cuda_lib, tmp_path):
    """The driver-level restart (2D_basic/mainp.f90:85-118) on the GPU solver:
    a run to t = 0.3 with output every 0.1, then a fresh solver with
    n_start = -1 finds the newest file, continues with the next file number
    and ends on the state an uninterrupted run reaches, bit for bit (the
    output times only set where the device stops between files, never dt)."""
    import os

    from openmhd_gb300 import Solver, orszag_tang

    cfg, model = orszag_tang(48)
    out = str(tmp_path / "data")
    first = Solver(cfg).init_model(model).run_with_output(0.3, 0.1, outdir=out)
    assert [os.path.basename(p) for p in first] == ["field-%05d.dat" % n for n in range(4)]
    b = Solver(cfg).init_model(model)
    second = b.run_with_output(0.6, 0.1, outdir=out, n_start=-1)
    assert os.path.basename(second[0]) == "field-00004.dat"
    whole = Solver(cfg).init_model(model)
    whole.run_until(0.6)
    ib, iw = b.sync(), whole.sync()
    assert ib.t == iw.t and ib.t >= 0.6
    assert np.array_equal(b.get_state_numpy(), whole.get_state_numpy())


def test_layout_pinned_by_reference_readers(lib, tmp_path):
    """The files written for the seeded states of tests/golden/make_fileio_golden.py
    are byte for byte the files that the reference's own readers
    (visualization/openmhd2d.py, openmhd3d.py) parsed into the recorded arrays,
    those arrays are the written state, and our reader returns the same."""
    import os
    import sys

    from openmhd_gb300 import fileio

    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, golden)
    import make_fileio_golden as G

    rec = np.load(os.path.join(golden, "fileio_reference_reader.npz"))
    for nd in (2, 3):
        path = str(tmp_path / f"field-0000{nd}.dat")
        assert G.write_case(nd, path) == str(rec[f"sha256_{nd}d"])
        t, x, y, z, U, V = G.seeded_case(nd)
        field = (lambda a: a.T) if nd == 2 else (lambda a: a.transpose(2, 1, 0))
        data = rec[f"data_{nd}d"]
        assert float(rec[f"t_{nd}d"]) == t
        assert np.array_equal(rec[f"x_{nd}d"], x) and np.array_equal(rec[f"y_{nd}d"], y)
        if nd == 3:
            assert np.array_equal(rec["z_3d"], z)
        for q in range(4):
            assert np.array_equal(data[..., q], field(V[q]))
        for q in range(4, 9):
            assert np.array_equal(data[..., q], field(U[q]))
        shape = G.SHAPES[nd]
        t2, x2, y2, z2, U2 = fileio.read(path, nd, shape[-1], shape[-2], shape[0] if nd == 3 else 1)
        assert t2 == t and np.array_equal(U2, U) and np.array_equal(x2, x) and np.array_equal(y2, y)
        if nd == 3:
            assert np.array_equal(z2, z)
