"""Parity of the device factor/solve against the CPU oracle (seeded hp-FEM
meshes, sizes the oracle finishes in seconds).

Tolerance: the plain FP64 path must match the oracle's solution within 1e-10
relative (max-norm), and its backward error must be at FP64 level."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _solve_gpu(spec, method, bulk=True):
    m = api.load_spec(spec, bulk=bulk)
    m.factor(method)
    m.solve(method)
    ids = spec.node_id.astype(np.int32)
    x = m.node_solution(ids, spec.node_ndof, spec.n_rhs)
    return m, x


CASES = [
    ("2d_4x4_p2", lambda: hpfem.poisson2d(4, 2, seed=1), uo.CHOL),
    ("2d_16x16_p4", lambda: hpfem.poisson2d(16, 4, seed=2), uo.CHOL),
    ("3d_4_p3", lambda: hpfem.poisson3d(4, 3, seed=3), uo.CHOL),
    ("3d_8_p4", lambda: hpfem.poisson3d(8, 4, seed=4), uo.CHOL),
    ("3d_6_p2_merge32", lambda: hpfem.poisson3d(6, 2, seed=5, merges=[3, 2]), uo.CHOL),
    ("3d_7_p3_ragged", lambda: hpfem.poisson3d(7, 3, seed=15), uo.CHOL),
    ("cd_4_p3_lupiv", lambda: hpfem.convdiff3d(4, 3, seed=6), uo.LU_PIV),
    ("cd_6_p3_lupiv", lambda: hpfem.convdiff3d(6, 3, seed=7, merges=[3, 2]), uo.LU_PIV),
    ("cd_4_p2_lunopiv", lambda: hpfem.convdiff3d(4, 2, seed=8, pe=1.0), uo.LU_NOPIV),
    # root front 6938 rows: LU panels on many CTAs (cooperative launch) + row interchanges
    ("cd_12_p3_lupiv_tall", lambda: hpfem.convdiff3d(12, 3, seed=14), uo.LU_PIV),
    ("3d_4_p3_rhs4", lambda: hpfem.poisson3d(4, 3, seed=9, n_rhs=4), uo.CHOL),
    # 16 right-hand sides through the flag-driven solves of the large fronts (four launches of four)
    ("3d_8_p4_rhs16", lambda: hpfem.poisson3d(8, 4, seed=12, n_rhs=16), uo.CHOL),
    ("3d_6_p3_rhs7", lambda: hpfem.poisson3d(6, 3, seed=13, n_rhs=7), uo.CHOL),
    ("diff_4_varp", lambda: hpfem.build_mesh(3, 4, np.random.default_rng(3).integers(2, 6, 64),
                                              seed=10), uo.CHOL),
]


@pytest.mark.parametrize("name,make,method", CASES, ids=[c[0] for c in CASES])
def test_fp64_matches_oracle(native_lib, name, make, method):
    spec = make()
    ref = uo.solve_mesh(spec, method)
    m, x = _solve_gpu(spec, method)
    rel = np.abs(x - ref.x).max() / np.abs(ref.x).max()
    assert rel < REL_TOL, (name, rel)
    berr = m.backward_error()
    A, b = uo.assemble(spec)
    berr_ref = uo.backward_error(spec, ref.x, A, b)
    assert berr < 1e-14, (name, berr, berr_ref)


def test_per_element_copy_in_matches_bulk(native_lib):
    spec = hpfem.poisson3d(4, 3, seed=11)
    _, x1 = _solve_gpu(spec, uo.CHOL, bulk=True)
    _, x2 = _solve_gpu(spec, uo.CHOL, bulk=False)
    assert np.array_equal(x1, x2)


def test_copy_out_element_order(native_lib):
    spec = hpfem.poisson2d(4, 3, seed=12)
    ref = uo.solve_mesh(spec, uo.CHOL)
    m, _ = _solve_gpu(spec, uo.CHOL)
    for e in (0, 5, spec.n_leaves - 1):
        xe = m.copy_out(m._elts[e], spec.element_nodes(e), int(spec.elem_m[e]))
        xr = uo.element_solution(spec, ref.x, e)
        assert np.allclose(xe, xr, rtol=0, atol=1e-12 * np.abs(ref.x).max())


def test_rerun_is_bitwise_reproducible(native_lib):
    spec = hpfem.poisson3d(4, 4, seed=13)
    _, x1 = _solve_gpu(spec, uo.CHOL)
    _, x2 = _solve_gpu(spec, uo.CHOL)
    assert np.array_equal(x1, x2)


def test_indefinite_front_reports_status(native_lib):
    spec = hpfem.poisson2d(4, 2, seed=14)
    spec.mats = -spec.mats           # negative definite: Cholesky must break down
    m = api.load_spec(spec)
    with pytest.raises(api.UHMError) as ei:
        m.chol_with_free()
    assert ei.value.code == 11
