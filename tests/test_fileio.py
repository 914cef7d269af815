"""The reference's file formats (.bcsm[.gz], .vector, Vector3Array .dat) and
the file-driven solver (src/pcg_solver.cpp).

Byte layouts: SPARSE_MATRIX::readFromBinary(GZ) (SPARSE_MATRIX.cpp:1612-1708),
VECTOR::read (VECTOR_FAST.cpp:247-270), readVector (STLUtil.h:105-118).
"""
import gzip
import struct

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from rank_structured_cholesky_gb300 import fileio, pcg_solver


def _small_csc():
    # 3 x 3 SPD tridiagonal, full symmetric storage
    colptr = np.array([0, 2, 5, 7], np.int32)
    rowind = np.array([0, 1, 0, 1, 2, 1, 2], np.int32)
    vals = np.array([4.0, -1.0, -1.0, 4.0, -1.0, -1.0, 4.0])
    return colptr, rowind, vals


def test_bcsm_bytes_match_the_reference_layout(tmp_path):
    colptr, rowind, vals = _small_csc()
    raw = struct.pack("<3Q", 7, 3, 3) + colptr.astype("<i4").tobytes() + rowind.astype("<i4").tobytes() + \
        vals.astype("<f8").tobytes()
    for name, data in (("a.bcsm", raw), ("a.bcsm.gz", gzip.compress(raw))):
        p = tmp_path / name
        p.write_bytes(data)
        n, cp, ri, v = fileio.read_bcsm(str(p))
        assert n == 3 and np.array_equal(cp, colptr) and np.array_equal(ri, rowind) and np.array_equal(v, vals)
    fileio.write_bcsm(str(tmp_path / "b.bcsm"), colptr, rowind, vals)
    assert (tmp_path / "b.bcsm").read_bytes() == raw


def test_vector_and_positions_round_trip(tmp_path):
    v = np.arange(5, dtype=np.float64) * 0.5 - 1.0
    fileio.write_vector(str(tmp_path / "r.vector"), v)
    assert (tmp_path / "r.vector").read_bytes() == struct.pack("<i", 5) + v.astype("<f8").tobytes()
    assert np.array_equal(fileio.read_vector(str(tmp_path / "r.vector")), v)
    xyz = np.random.default_rng(0).standard_normal((4, 3))
    fileio.write_positions(str(tmp_path / "p.dat"), xyz)
    assert np.array_equal(fileio.read_positions(str(tmp_path / "p.dat")), xyz)


def test_malformed_files_are_rejected(tmp_path):
    colptr, rowind, vals = _small_csc()
    good = struct.pack("<3Q", 7, 3, 3) + colptr.astype("<i4").tobytes() + rowind.astype("<i4").tobytes() + \
        vals.astype("<f8").tobytes()
    (tmp_path / "t.bcsm").write_bytes(good[:-8])                     # truncated values
    with pytest.raises(fileio.FormatError):
        fileio.read_bcsm(str(tmp_path / "t.bcsm"))
    bad = bytearray(good)
    bad[24 + 4:24 + 8] = struct.pack("<i", 9)                        # colptr[1] > nnz
    (tmp_path / "c.bcsm").write_bytes(bytes(bad))
    with pytest.raises(fileio.FormatError):
        fileio.read_bcsm(str(tmp_path / "c.bcsm"))
    (tmp_path / "r.vector").write_bytes(struct.pack("<i", 3) + b"\0" * 16)
    with pytest.raises(fileio.FormatError):
        fileio.read_vector(str(tmp_path / "r.vector"))


def test_cli_reports_missing_files(tmp_path, capsys):
    assert pcg_solver.main([str(tmp_path / "nothing")]) == 1
    assert "pcg_solver:" in capsys.readouterr().err


def _write_problem(prefix, prob, positions):
    fileio.write_bcsm(prefix + "_system.bcsm.gz", prob.colptr, prob.rowind, prob.vals)
    fileio.write_vector(prefix + "_rhs.vector", prob.rhs[0])
    if positions:
        fileio.write_positions(prefix + "_meshPositions.dat", prob.xyz)


@pytest.mark.gpu
@pytest.mark.parametrize("positions", [True, False])
def test_cli_solves_like_the_library(tmp_path, positions):
    prob = rs.diffusion(3, 16, sigma=1.0, seed=7)
    prefix = str(tmp_path / "sys")
    _write_problem(prefix, prob, positions)
    out = str(tmp_path / "x.vector")
    assert pcg_solver.main([prefix, "--out", out]) == 0
    x = fileio.read_vector(out)
    A = prob.scipy()
    b = prob.rhs[0]
    assert np.linalg.norm(b - A @ x) <= 1.5e-6 * np.linalg.norm(b)   # the driver's 1e-6 tolerance
    ctx = rs.Context(max_dense_block=200, max_diag_block=400, reorder_separators=1 if positions else 0)
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, prob.xyz if positions else None)
    x_lib, _ = G.pcg(b, eps=1e-6, maxit=10000)
    assert np.array_equal(x, x_lib)
