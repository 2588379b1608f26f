"""Mixed precision (FP32 / BF16-split fronts) with FP64 iterative refinement on
the unassembled element matrices: the refined solution must reach a backward
error <= 1e-12 and agree with the FP64 oracle."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _mixed(spec, method, prec, tol=TOL):
    m = api.load_spec(spec)
    m.set_mode(1, prec, tol, 10)
    m.factor(method)
    m.solve(method)
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)
    return m, x


@pytest.mark.parametrize("prec", [api.PREC_FP32, api.PREC_BF16X3, api.PREC_BF16X6])
@pytest.mark.parametrize("name,make,method", [
    ("3d_8_p4", lambda: hpfem.poisson3d(8, 4, seed=21), uo.CHOL),
    ("2d_16_p4", lambda: hpfem.poisson2d(16, 4, seed=22), uo.CHOL),
    ("diff_6_p3_c1e4", lambda: hpfem.diffusion3d(6, 3, seed=23, merges=[3, 2]), uo.CHOL),
    ("cd_4_p3", lambda: hpfem.convdiff3d(4, 3, seed=24), uo.LU_PIV),
    ("cd_12_p3_tall", lambda: hpfem.convdiff3d(12, 3, seed=25), uo.LU_PIV),
])
def test_mixed_refines_to_fp64(native_lib, name, make, method, prec):
    spec = make()
    ref = uo.solve_mesh(spec, method)
    m, x = _mixed(spec, method, prec)
    t = m.timing()
    assert m.status() in (0, api.STATUS_RECOMPUTED_FP64)
    assert m.status() == 0, "refinement fell back to FP64"
    assert t["berr"] <= TOL, t
    # independent check on the CPU with the assembled operator
    A, b = uo.assemble(spec)
    assert uo.backward_error(spec, x, A, b) <= 2 * TOL
    rel = np.abs(x - ref.x).max() / np.abs(ref.x).max()
    assert rel < 1e-6, rel


@pytest.mark.parametrize("prec,first_tol", [(api.PREC_BF16X3, 1e-5), (api.PREC_BF16X6, 1e-6)])
def test_tensor_core_schur_update_accuracy(native_lib, prec, first_tol):
    """Large fronts (ss >= 128) take the tcgen05 path: the backward error of
    the first solve shows the factor is accurate to split-BF16 level, and the
    refinement then reaches 1e-12."""
    spec = hpfem.poisson3d(8, 4, seed=27)
    m, x = _mixed(spec, uo.CHOL, prec)
    t = m.timing()
    assert t["berr"] <= TOL
    assert 0 < m.first_backward_error() < first_tol, m.first_backward_error()


def test_backward_error_matches_oracle(native_lib):
    spec = hpfem.poisson3d(4, 3, seed=25)
    m, x = _mixed(spec, uo.CHOL, api.PREC_FP32)
    A, b = uo.assemble(spec)
    be_cpu = uo.backward_error(spec, x, A, b)
    be_gpu = m.backward_error()
    assert abs(be_gpu - be_cpu) <= 1e-3 * be_cpu + 1e-18


def test_unreachable_tolerance_recomputes_in_fp64(native_lib):
    spec = hpfem.poisson3d(4, 3, seed=26)
    ref = uo.solve_mesh(spec, uo.CHOL)
    m = api.load_spec(spec)
    m.set_mode(1, api.PREC_FP32, 1e-30, 1)   # cannot be met: forces the FP64 redo
    m.chol_with_free()
    m.solve_chol()
    assert m.status() == api.STATUS_RECOMPUTED_FP64
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof)
    assert np.abs(x - ref.x).max() / np.abs(ref.x).max() < 1e-10
