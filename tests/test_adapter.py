"""The C++ PRECONDITIONER adapter (include/rschol_gpu_preconditioner.hpp).

The adapter must compile as a concrete PRECONDITIONER (all three pure
virtuals of src/rschol/linearalgebra/PRECONDITIONER.h:54-56 implemented)
against the reference's declarations, here the stand-ins under
tests/adapter_standin/ that repeat the reference's signatures
(PRECONDITIONER, VECTOR, SPARSE_MATRIX::SparseColumnMatrix, the factor-type
enums).  tests/adapter_driver.cpp uses it the way src/pcg_solver.cpp uses
FactorPreconditioner.  On CPU the driver must link and report the missing
device as an exception (never abort); on a GPU its PRECONDITIONER::solve,
a host CG loop through that interface, and its device PCG must agree with
the library's own entry points.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import rank_structured_cholesky_gb300 as rs
from rank_structured_cholesky_gb300 import _build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
EXE = os.path.join(_build.OUT, "adapter_driver")


def build_driver():
    lib = _build.build_library()
    src = os.path.join(HERE, "adapter_driver.cpp")
    hdr = os.path.join(ROOT, "include", "rschol_gpu_preconditioner.hpp")
    if _build._stale(EXE, [src, hdr, lib]):
        cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-Werror", "-I", os.path.join(HERE, "adapter_standin"),
               "-I", os.path.join(ROOT, "include"), src, "-o", EXE, "-L", os.path.dirname(lib), "-lrschol_gb300",
               "-Wl,-rpath," + os.path.dirname(lib)]
        subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return EXE


def write_system(path, prob, b):
    with open(path, "wb") as f:
        np.array([prob.n, len(prob.rowind)], np.int32).tofile(f)
        prob.colptr.astype(np.int32).tofile(f)
        prob.rowind.astype(np.int32).tofile(f)
        prob.vals.astype(np.float64).tofile(f)
        np.ascontiguousarray(b, np.float64).tofile(f)


def test_adapter_is_a_concrete_preconditioner():
    """The header alone compiles as an instantiable PRECONDITIONER subclass."""
    src = ('#include "rschol_gpu_preconditioner.hpp"\n'
           'static PRECONDITIONER *make() { return new GpuFactorPreconditioner(); }\n'
           'int main() { PRECONDITIONER *p = make(); p->init(); delete p; return 0; }\n')
    subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-Wall", "-Werror", "-x", "c++", "-",
                    "-I", os.path.join(HERE, "adapter_standin"), "-I", os.path.join(ROOT, "include")],
                   input=src, text=True, check=True)


def test_adapter_reports_missing_device_without_abort(tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present: covered by the GPU test")
    except ImportError:
        pass
    exe = build_driver()
    prob = rs.diffusion(2, 12, sigma=1.0, seed=3)
    write_system(tmp_path / "in.bin", prob, prob.rhs[0])
    p = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert p.returncode == 3, (p.returncode, p.stdout, p.stderr)
    assert "rschol_factor_create returned status 7" in p.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [rs.FP64, rs.MIXED])
def test_adapter_drives_the_gpu_factor(tmp_path, precision):
    exe = build_driver()
    prob = rs.diffusion(2, 64, sigma=1.0, seed=3)
    b = prob.rhs[0]
    write_system(tmp_path / "in.bin", prob, b)
    p = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(precision)],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, (p.stdout, p.stderr)
    n = prob.n
    raw = open(tmp_path / "out.bin", "rb").read()
    vecs = np.frombuffer(raw[:24 * n], np.float64).reshape(3, n)
    host_it, dev_it = np.frombuffer(raw[24 * n:], np.int32)
    # the library's own entry points, same driver settings (maxDense 200, maxDiag 400, no positions)
    ctx = rs.Context(max_dense_block=200, max_diag_block=400, reorder_separators=0, precision=precision)
    G = rs.GpuFactor(ctx, prob.colptr, prob.rowind, prob.vals, None)
    z = G.apply(b)
    assert np.linalg.norm(vecs[0] - z) <= 1e-12 * np.linalg.norm(z)
    x, info = G.pcg(b, 1e-8, 1000)
    assert dev_it == info["iterations"]
    assert abs(int(host_it) - info["iterations"]) <= 1
    A = prob.scipy()
    for k in (1, 2):
        assert np.linalg.norm(b - A @ vecs[k]) / np.linalg.norm(b) <= 1e-8
