"""Synthetic workload generators (sizes, symmetry, positive definiteness)."""
import numpy as np
import scipy.sparse as sp

import rank_structured_cholesky_gb300 as rs


def test_poisson_2d_128_nnz():
    p = rs.diffusion(2, 128, sigma=0.0, seed=0)
    assert p.n == 16384 and len(p.vals) == 81408
    A = p.scipy()
    assert abs(A - A.T).max() == 0
    assert np.allclose(A.diagonal(), 4.0)


def test_diffusion_3d_symmetric_spd():
    p = rs.diffusion(3, 6, sigma=1.0, seed=1)
    A = p.scipy().toarray()
    assert np.allclose(A, A.T)
    assert np.linalg.eigvalsh(A).min() > 0


def test_elasticity_size_and_spd():
    p = rs.elasticity(4, seed=2)
    assert p.n == 4 * 5 * 5 * 3        # x = 0 face clamped
    A = p.scipy().toarray()
    assert np.allclose(A, A.T, atol=1e-12)
    assert np.linalg.eigvalsh(A).min() > 0
    assert np.all(np.abs(p.rhs) <= 1.0)


def test_generator_is_seeded():
    a = rs.diffusion(2, 16, sigma=2.0, seed=3, nrhs=2)
    b = rs.diffusion(2, 16, sigma=2.0, seed=3, nrhs=2)
    assert np.array_equal(a.vals, b.vals) and np.array_equal(a.rhs, b.rhs)
    assert a.rhs.shape == (2, 256)
