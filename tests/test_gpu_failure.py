"""Failure detection on the device without faulting it.

Every spin-wait inside the kernels (the flag hand-offs of the tree solves,
the grid barrier of the cooperative LU panel, the allocation-free solve) has
an iteration limit.  These tests lower the limit to 0, so that a wait not
satisfied at its first look gives up, and check that the call reports status
14, that the device stays usable, and that the next call with the default
limit gives the oracle's answer.  Bad inputs (a NaN in a right-hand side)
must come back as status 13, not as a silent NaN solution or a crash.

The reference has no device waits and does not check its inputs for NaN
(LINAL/src/dense/chol.cxx:67 ignores a breakdown), so this is behaviour of
this library only."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _rel(x, ref):
    return float(np.abs(x - ref).max() / np.abs(ref).max())


def test_tree_solve_wait_runs_out_returns_14(native_lib):
    # 8^3 p=4: root front 2791 with flag-driven block solves on the large fronts
    spec = hpfem.poisson3d(8, 4, seed=21)
    ref = uo.solve_mesh(spec, uo.CHOL)
    m = api.load_spec(spec)
    m.chol_with_free()
    api.set_wait_limit(0)
    try:
        with pytest.raises(api.UHMError) as ei:
            m.solve_chol()
    finally:
        api.set_wait_limit(-1)
    assert ei.value.code == 14
    m.solve_chol()                      # same factors, default limit
    assert m.status() == 0
    assert _rel(_x(m, spec), ref.x) < REL_TOL


def test_lu_panel_grid_barrier_runs_out_returns_14(native_lib):
    # root front 6938 rows: LU panels on many CTAs behind a grid barrier
    spec = hpfem.convdiff3d(12, 3, seed=14)
    m = api.load_spec(spec)
    api.set_wait_limit(0)
    try:
        with pytest.raises(api.UHMError) as ei:
            m.lu_piv_with_free()
    finally:
        api.set_wait_limit(-1)
    assert ei.value.code == 14
    with pytest.raises(api.UHMError):
        m.solve_lu_piv()                # the failed factorisation is not solved with
    m.lu_piv_with_free()
    m.solve_lu_piv()
    assert m.status() == 0
    ref = uo.solve_mesh(spec, uo.LU_PIV)
    assert _rel(_x(m, spec), ref.x) < REL_TOL


@pytest.mark.parametrize("mode,prec", [(0, api.PREC_FP64), (1, api.PREC_FP32)], ids=["plain", "mixed"])
def test_nan_rhs_reports_status_13(native_lib, mode, prec):
    spec = hpfem.poisson3d(4, 3, seed=22)
    spec.rhs = spec.rhs.copy()
    spec.rhs.reshape(-1)[7] = np.nan
    m = api.load_spec(spec)
    m.set_mode(mode, prec, 1e-12, 10)
    m.chol_with_free()                  # the factors do not depend on the right-hand side
    with pytest.raises(api.UHMError) as ei:
        m.solve_chol()
    assert ei.value.code == 13
    # a finite right-hand side on the same mesh solves normally afterwards
    good = hpfem.poisson3d(4, 3, seed=22)
    m.copy_in_leaves(api.UHM_RHS, good.rhs)
    m.solve_chol()
    assert m.status() in (0, api.STATUS_RECOMPUTED_FP64)
    ref = uo.solve_mesh(good, uo.CHOL)
    assert _rel(_x(m, good), ref.x) < (REL_TOL if mode == 0 else 1e-8)
