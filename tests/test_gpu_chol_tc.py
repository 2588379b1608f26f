"""The cooperative-panel Cholesky path of BF16X3 fronts (k_chol_tc.cu).

Each tensor-core front is factored panel by panel: with panels of 256
columns a cooperative launch factors the diagonal block and forms its
inverse and the rows below are solved on the tensor cores (X = A Linv^T);
with panels of 512 columns the cooperative launch factors the whole panel.
The factor block's trailing columns are updated on the tensor cores after
every panel, and the Schur complement ABR once at the end with the whole
factor block as K.  Iterative refinement
would hide a wrong update, so the tests check the first solve's backward
error (BF16X3 factors give about 1e-8 on these meshes; a missed or doubled
update region gives 1e-3 or worse) as well as the refined solution against
the oracle (1e-8 relative, max norm) and the step-by-step tensor-core path
(tc_panel = 0) on the same mesh."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

FIRST_BERR = 1e-6
REL_TOL_MIXED = 1e-8


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _solve(spec, tc_panel, tc_min_n=512):
    m = api.load_spec(spec)
    m.set_tunables(tc_panel=tc_panel, tc_min_n=tc_min_n)
    m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
    m.chol_with_free()
    m.solve_chol()
    assert m.status() == 0, m.last_error()
    return m, m.timing()


CASES = [
    # root 2791 (fs = n), level-3 fronts (631, 1538): panels of both widths,
    # ragged last panels, ABR passes with K = 631
    ("3d_8_p4", lambda: hpfem.poisson3d(8, 4, seed=31), 512),
    ("3d_8_p4_w256", lambda: hpfem.poisson3d(8, 4, seed=32), 256),
    ("3d_8_p4_w512_b", lambda: hpfem.poisson3d(8, 4, seed=37), 512),
    # heterogeneous coefficients, fronts from n = 256 on the tensor cores
    ("diff_8_p3", lambda: hpfem.diffusion3d(8, 3, seed=33, contrast=1e3), 256),
    ("diff_8_p3_w512", lambda: hpfem.diffusion3d(8, 3, seed=33, contrast=1e3), 512),
    # two right-hand sides and a 3-way top merge (one large root front)
    ("3d_6_p4_merge32_rhs2", lambda: hpfem.poisson3d(6, 4, seed=34, merges=[3, 2], n_rhs=2), 256),
    # seven right-hand sides: the solves' second group holds three
    ("3d_6_p3_rhs7", lambda: hpfem.poisson3d(6, 3, seed=38, n_rhs=7), 256),
]


@pytest.mark.parametrize("name,make,w1", CASES, ids=[c[0] for c in CASES])
def test_panel_path_matches_oracle(native_lib, name, make, w1):
    spec = make()
    ref = uo.solve_mesh(spec, uo.CHOL)
    m, t = _solve(spec, w1, tc_min_n=256)
    prec = m.front_precision()[0]
    assert (prec == api.PREC_BF16X3).any()
    assert t["berr_first"] < FIRST_BERR, (name, t["berr_first"])
    assert t["berr"] <= 1e-12
    rel = np.abs(_x(m, spec) - ref.x).max() / np.abs(ref.x).max()
    assert rel < REL_TOL_MIXED, (name, rel)


def test_panel_path_agrees_with_step_path(native_lib):
    spec = hpfem.poisson3d(8, 4, seed=35)
    _, t_new = _solve(spec, 512)
    _, t_old = _solve(spec, 0)
    # both are BF16X3 factorisations of the same fronts: first-solve errors of one order
    assert t_new["berr_first"] < 10 * t_old["berr_first"] + 1e-12, (t_new["berr_first"], t_old["berr_first"])


@pytest.mark.parametrize("w1,kinds", [(512, ("chol_panel", "tc_chol_trail", "tc_chol_schur")),
                                      (256, ("chol_diag", "chol_pack", "tc_chol_trsm", "tc_chol_trail",
                                             "tc_chol_schur"))])
def test_panel_path_launches_its_kernels(native_lib, w1, kinds):
    spec = hpfem.poisson3d(8, 4, seed=36)
    m = api.load_spec(spec)
    m.set_tunables(tc_panel=w1)
    m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
    m.set_profiling(True)
    m.chol_with_free()
    m.solve_chol()
    prof = m.profile()
    for k in kinds:
        assert prof[k]["launches"] > 0, k
    # no front of this mesh went through the step-by-step tensor-core path
    assert "tc_syrk_bf16" not in prof and "tc_pack" not in prof
