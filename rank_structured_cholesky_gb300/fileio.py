"""The reference's file formats for systems, vectors and mesh positions.

* ``<name>.bcsm`` / ``<name>.bcsm.gz`` -- a CSC matrix (full symmetric storage),
  as written by ``SPARSE_MATRIX::writeToBinary``
  (src/rschol/linearalgebra/SPARSE_MATRIX.cpp:1557) and read by
  ``SPARSE_MATRIX::readFromBinary`` / ``readFromBinaryGZ`` (same file,
  1612-1708): three native
  ``size_t`` (nnz, rows, columns), then ``int32`` column pointers (columns + 1),
  ``int32`` row indices (nnz) and ``float64`` values (nnz); ``.gz`` is the same
  byte stream gzip-compressed.
* ``<name>.vector`` -- ``VECTOR::write`` / ``VECTOR::read``
  (src/rschol/linearalgebra/VECTOR_FAST.cpp:194-270): an ``int32`` size, then
  ``float64`` entries.
* ``<name>.dat`` positions -- ``writeVector`` / ``readVector`` of a
  ``Vector3Array`` (src/rschol/util/STLUtil.h:75-138): an ``int32`` count, then
  count x 3 ``float64``.

All integers are little-endian, as on the machines the reference targets.
"""
import gzip
import struct

import numpy as np


class FormatError(ValueError):
    pass


def _open(path, mode):
    return gzip.open(path, mode) if str(path).endswith(".gz") else open(path, mode)


def _read_exact(f, n, what):
    b = f.read(n)
    if len(b) != n:
        raise FormatError("%s: expected %d bytes, found %d" % (what, n, len(b)))
    return b


def read_bcsm(path):
    """(n_rows, colptr, rowind, vals) of a .bcsm or .bcsm.gz file."""
    with _open(path, "rb") as f:
        nnz, nrow, ncol = struct.unpack("<3Q", _read_exact(f, 24, "header"))
        if nrow != ncol:
            raise FormatError("matrix is %d x %d, not square" % (nrow, ncol))
        colptr = np.frombuffer(_read_exact(f, 4 * (ncol + 1), "column pointers"), dtype="<i4").astype(np.int32)
        rowind = np.frombuffer(_read_exact(f, 4 * nnz, "row indices"), dtype="<i4").astype(np.int32)
        vals = np.frombuffer(_read_exact(f, 8 * nnz, "values"), dtype="<f8").astype(np.float64)
    if colptr[0] != 0 or colptr[-1] != nnz or np.any(np.diff(colptr) < 0):
        raise FormatError("inconsistent column pointers")
    if nnz and (rowind.min() < 0 or rowind.max() >= nrow):
        raise FormatError("row index out of range")
    return int(nrow), colptr, rowind, vals


def write_bcsm(path, colptr, rowind, vals):
    colptr = np.ascontiguousarray(colptr, "<i4")
    rowind = np.ascontiguousarray(rowind, "<i4")
    vals = np.ascontiguousarray(vals, "<f8")
    n = len(colptr) - 1
    with _open(path, "wb") as f:
        f.write(struct.pack("<3Q", len(rowind), n, n))
        f.write(colptr.tobytes())
        f.write(rowind.tobytes())
        f.write(vals.tobytes())


def read_vector(path):
    with _open(path, "rb") as f:
        (n,) = struct.unpack("<i", _read_exact(f, 4, "size"))
        if n < 0:
            raise FormatError("negative vector size")
        return np.frombuffer(_read_exact(f, 8 * n, "entries"), dtype="<f8").astype(np.float64)


def write_vector(path, v):
    v = np.ascontiguousarray(v, "<f8")
    with _open(path, "wb") as f:
        f.write(struct.pack("<i", len(v)))
        f.write(v.tobytes())


def read_positions(path):
    """n x 3 positions of a Vector3Array file."""
    with _open(path, "rb") as f:
        (n,) = struct.unpack("<i", _read_exact(f, 4, "count"))
        if n < 0:
            raise FormatError("negative position count")
        return np.frombuffer(_read_exact(f, 24 * n, "positions"), dtype="<f8").astype(np.float64).reshape(n, 3)


def write_positions(path, xyz):
    xyz = np.ascontiguousarray(xyz, "<f8").reshape(-1, 3)
    with _open(path, "wb") as f:
        f.write(struct.pack("<i", len(xyz)))
        f.write(xyz.tobytes())
