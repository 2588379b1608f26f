"""The forward solve of large Cholesky fronts with 256-row CTAs
(solve_rows = 256, k_fwd_hand4) against the 64-row flag-driven kernels
(solve_rows = 64) and the oracle.

Each 256-row CTA takes the column blocks left of it from other CTAs as
hand-off words and solves its own four 64-row blocks in turn, so there is one
hand-off between CTAs per 256 rows.  The reference's steps are the same
triangular solves (UHM/src/matrix/uhm/fla/chol/solve.cxx:152-202); only the
order of the additions within a row differs between the two forms.

Checked: mixed precision (FP32 fronts) and plain FP64 fronts, a root front
with a ragged last block, ABL rows (fronts below the root), several
right-hand sides in two launch groups (4 + 3 and 4 + 2, which take the 4-
and 2-wide 64-row kernels), and that both forms give the same first-solve
backward error (same factors)."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

REL_TOL_FP64 = 1e-10
REL_TOL_MIXED = 1e-8


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _solve(spec, mode, prec, **tun):
    m = api.load_spec(spec)
    m.set_tunables(**tun)
    m.set_mode(mode, prec, 1e-12, 10)
    m.chol_with_free()
    m.solve_chol()
    assert m.status() == 0, m.last_error()
    return m, m.timing()


CASES = [
    ("3d_8_p4_mixed", lambda: hpfem.poisson3d(8, 4, seed=71), 1, api.PREC_BF16X3, REL_TOL_MIXED),
    ("3d_8_p4_fp32", lambda: hpfem.poisson3d(8, 4, seed=72), 1, api.PREC_FP32, REL_TOL_MIXED),
    ("3d_8_p3_fp64", lambda: hpfem.poisson3d(8, 3, seed=73), 0, api.PREC_FP64, REL_TOL_FP64),
    ("3d_6_p4_rhs7", lambda: hpfem.poisson3d(6, 4, seed=74, n_rhs=7), 1, api.PREC_FP32, REL_TOL_MIXED),
    # launch groups of 4 and 2 right-hand sides (the 4- and 2-wide kernels)
    ("3d_6_p4_rhs6", lambda: hpfem.poisson3d(6, 4, seed=76, n_rhs=6), 1, api.PREC_FP32, REL_TOL_MIXED),
    ("diff_8_p3", lambda: hpfem.diffusion3d(8, 3, seed=75, contrast=1e3), 1, api.PREC_FP32, REL_TOL_MIXED),
]


@pytest.mark.parametrize("name,make,mode,prec,tol", CASES, ids=[c[0] for c in CASES])
def test_solve_rows_256_matches_oracle_and_64(native_lib, name, make, mode, prec, tol):
    spec = make()
    ref = uo.solve_mesh(spec, uo.CHOL)
    m4, t4 = _solve(spec, mode, prec, solve_rows=256)
    m1, t1 = _solve(spec, mode, prec, solve_rows=64)
    for m in (m4, m1):
        rel = np.abs(_x(m, spec) - ref.x).max() / np.abs(ref.x).max()
        assert rel < tol, (name, rel)
    if mode == 1:
        assert t4["berr"] <= 1e-12 and t1["berr"] <= 1e-12
        # the same factors: first-solve errors of one order
        assert t4["berr_first"] < 10 * t1["berr_first"] + 1e-14, (t4["berr_first"], t1["berr_first"])
        assert t1["berr_first"] < 10 * t4["berr_first"] + 1e-14, (t4["berr_first"], t1["berr_first"])
