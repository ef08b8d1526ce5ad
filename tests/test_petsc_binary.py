"""PETSc binary files (the format of VecView/MatView to a binary viewer, as
c/ch12/obstacle.c:138-144 dumps solutions and c/ch2/loadsolve.c loads
systems): byte-exact known answers, round trips, several objects per file,
and rejection of malformed files.  Host code: runs without a GPU."""
import struct

import numpy as np
import pytest


def test_vec_known_bytes(built, tmp_path):
    import p4pdes_gb300 as fg
    f = tmp_path / "v.dat"
    fg.petsc_vec_write(f, np.array([1.0, 2.5, -3.0]))
    assert f.read_bytes() == struct.pack(">ii3d", 1211214, 3, 1.0, 2.5, -3.0)
    assert np.array_equal(fg.petsc_vec_read(f), [1.0, 2.5, -3.0])


def test_vec_round_trip_and_append(built, tmp_path):
    import p4pdes_gb300 as fg
    rng = np.random.default_rng(0)
    u, psi = rng.standard_normal(9 * 9), rng.standard_normal(12345)
    f = tmp_path / "dump.dat"
    fg.petsc_vec_write(f, u)
    fg.petsc_vec_write(f, psi, append=True)     # obstacle.c writes u then the obstacle
    assert np.array_equal(fg.petsc_vec_read(f, 0), u)
    assert np.array_equal(fg.petsc_vec_read(f, 1), psi)
    with pytest.raises(fg.FishError):
        fg.petsc_vec_read(f, 2)


def test_mat_known_bytes_and_round_trip(built, tmp_path):
    import scipy.sparse as sp
    import p4pdes_gb300 as fg
    A = sp.csr_matrix(np.array([[2.0, -1.0, 0.0], [-1.0, 2.0, -1.0], [0.0, -1.0, 2.0]]))
    f = tmp_path / "A.dat"
    fg.petsc_mat_write(f, A)
    want = struct.pack(">4i", 1211216, 3, 3, 7) + struct.pack(">3i", 2, 3, 2) + \
        struct.pack(">7i", 0, 1, 0, 1, 2, 1, 2) + struct.pack(">7d", 2, -1, -1, 2, -1, -1, 2)
    assert f.read_bytes() == want
    fg.petsc_vec_write(f, np.ones(3), append=True)  # A then b, as loadsolve reads them
    M, N, rp, col, val = fg.petsc_mat_read(f, 0)
    B = sp.csr_matrix((val, col, rp), shape=(M, N))
    assert (B != A).nnz == 0
    assert np.array_equal(fg.petsc_vec_read(f, 1), np.ones(3))
    with pytest.raises(fg.FishError):
        fg.petsc_mat_read(f, 1)                 # object 1 is a Vec


def test_malformed_files_are_rejected(built, tmp_path):
    import p4pdes_gb300 as fg
    bad = tmp_path / "bad.dat"
    bad.write_bytes(struct.pack(">ii", 1234, 3) + b"\0" * 24)
    with pytest.raises(fg.FishError):
        fg.petsc_vec_read(bad)
    short = tmp_path / "short.dat"
    short.write_bytes(struct.pack(">ii2d", 1211214, 3, 1.0, 2.0))
    with pytest.raises(fg.FishError):
        fg.petsc_vec_read(short)
    with pytest.raises(fg.FishError):
        fg.petsc_vec_read(tmp_path / "missing.dat")
