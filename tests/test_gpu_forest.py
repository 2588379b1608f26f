"""Batched solve of many independent meshes as one forest on the device.

Every same-generation front of all meshes shares a launch, so a forest of
meshes of one shape takes as many launches as one of them, not the sum.
Each mesh's part of the solution must match the oracle's solve of that mesh
alone (FP64 path, 1e-10 relative), and in the mixed path each mesh must reach
backward error 1e-12 on its own operator (checked on the CPU with the
assembled matrix of that mesh)."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _parts(n_rhs):
    return [hpfem.poisson3d(8, 4, seed=31, n_rhs=n_rhs),
            hpfem.poisson3d(5, 3, seed=32, n_rhs=n_rhs),
            hpfem.diffusion3d(6, 2, seed=33, contrast=1e4, n_rhs=n_rhs),
            hpfem.poisson2d(12, 4, seed=34, n_rhs=n_rhs),
            hpfem.poisson3d(4, 5, seed=35, n_rhs=n_rhs)]


def _slices(parts):
    o = 0
    for p in parts:
        yield p, slice(o, o + p.n_dof())
        o += p.n_dof()


def _solve(spec, mode=0, prec=api.PREC_FP32):
    m = api.load_spec(spec)
    if mode:
        m.set_mode(1, prec, TOL, 10)
    m.factor(uo.CHOL)
    m.solve(uo.CHOL)
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)
    return m, x


def test_forest_fp64_matches_oracle_per_mesh(native_lib):
    parts = _parts(4)
    f = hpfem.forest(parts)
    _, x = _solve(f)
    for p, sl in _slices(parts):
        ref = uo.solve_mesh(p, uo.CHOL).x
        rel = np.abs(x[sl] - ref).max() / np.abs(ref).max()
        assert rel < 1e-10, rel


@pytest.mark.parametrize("prec", [api.PREC_FP32, api.PREC_BF16X3])
def test_forest_mixed_meets_tolerance_per_mesh(native_lib, prec):
    parts = _parts(16)
    f = hpfem.forest(parts)
    m, x = _solve(f, mode=1, prec=prec)
    assert m.status() == 0
    for p, sl in _slices(parts):
        A, b = uo.assemble(p)
        assert uo.backward_error(p, x[sl], A, b) <= 2 * TOL


def test_forest_shares_launches(native_lib):
    # meshes of one shape: every level's launches are shared by all of them
    parts = [hpfem.poisson3d(5, 3, seed=40 + k) for k in range(4)]

    def n_ops(spec):
        m = api.load_spec(spec)
        m.set_mode(1, api.PREC_FP32, TOL, 10)
        m.factor(uo.CHOL)
        m.set_profiling(True)
        m.factor(uo.CHOL)
        n = len(m.op_log())
        m.set_profiling(False)
        return n

    separate = sum(n_ops(p) for p in parts)
    joined = n_ops(hpfem.forest(parts))
    assert joined <= 0.3 * separate, (joined, separate)
