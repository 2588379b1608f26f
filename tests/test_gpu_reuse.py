"""Factor reuse on the device (Element_::set_reuse / Mesh_::check_reuse, the
reference's UHM/src/operation/element.cxx:202-205 skipping the merge and
factorisation of a reusable element).

After one leaf's element matrix changes (copy_in adds c I to it), a
factorisation with every element flagged reusable redoes only that leaf and
its ancestors, keeps the other fronts' factors from the previous
factorisation, and gives the solution a fresh factorisation of the changed
mesh gives (FP64: to 1e-12 relative; FP32 fronts with FP64 refinement: both
within the refinement's accuracy of the oracle).  Unchanged meshes keep every
front; unflagged meshes redo every front; a flag alone never keeps a front
whose subtree changed (the reference's check_reuse can leave such a flag
set)."""
import dataclasses

import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _bumped(spec, k, c):
    mats = spec.mats.copy()
    mk, o = int(spec.elem_m[k]), int(spec.mat_off[k])
    blk = mats[o:o + mk * mk].reshape(mk, mk, order="F")
    blk[np.diag_indices(mk)] += c
    return dataclasses.replace(spec, mats=mats)


def _path(spec, k):
    p, e = [], k
    while e >= 0:
        p.append(e)
        e = int(spec.parent[e])
    return p


def _run(spec, method, mixed):
    m = api.load_spec(spec)
    if mixed:
        m.set_mode(1, api.PREC_FP32, 1e-12, 10)
    m.factor(method)
    m.solve(method)
    return m


CASES = [
    ("diff_6_p3_chol", lambda: hpfem.diffusion3d(6, 3, seed=71, contrast=1e2), uo.CHOL, False),
    ("cd_6_p3_lupiv", lambda: hpfem.convdiff3d(6, 3, seed=72), uo.LU_PIV, False),
    ("poisson_8_p3_fp32", lambda: hpfem.poisson3d(8, 3, seed=73), uo.CHOL, True),
]


@pytest.mark.parametrize("name,make,method,mixed", CASES, ids=[c[0] for c in CASES])
def test_refactor_redoes_only_the_changed_path(native_lib, name, make, method, mixed):
    spec = make()
    n_fronts = spec.n_elements
    m = _run(spec, method, mixed)
    assert m.n_refactored() == n_fronts
    x0 = _x(m, spec)
    for e in m._elts:
        m.set_reuse(e, True)
    # nothing changed: every front kept, the same solution
    m.factor(method)
    m.solve(method)
    assert m.n_refactored() == 0
    assert np.array_equal(_x(m, spec), x0)
    # one leaf changed: it and its ancestors are redone
    k = spec.n_leaves // 2
    mk = int(spec.elem_m[k])
    c = 0.5 * float(np.abs(spec.element_matrix(k)).max())
    m.copy_in(m._elts[k], spec.element_nodes(k), api.UHM_LHS, c * np.eye(mk))
    m.factor(method)
    m.solve(method)
    assert m.n_refactored() == len(_path(spec, k))
    x1 = _x(m, spec)
    spec2 = _bumped(spec, k, c)
    ref = uo.solve_mesh(spec2, method).x
    assert not np.allclose(x1, x0)
    if mixed:
        assert np.abs(x1 - ref).max() <= 1e-8 * np.abs(ref).max()
        assert m.backward_error() <= 1e-12
    else:
        x2 = _x(_run(spec2, method, mixed), spec2)
        assert np.abs(x1 - x2).max() <= 1e-12 * np.abs(x2).max()
        assert np.abs(x1 - ref).max() <= 1e-10 * np.abs(ref).max()
    # flags cleared: every front redone, the same solution
    for e in m._elts:
        m.set_reuse(e, False)
    m.factor(method)
    m.solve(method)
    assert m.n_refactored() == n_fronts
    assert np.abs(_x(m, spec) - x1).max() <= 1e-12 * np.abs(x1).max()


def test_check_reuse_flags_drive_the_factorisation(native_lib):
    """check_reuse on an unchanged mesh flags everything: nothing is redone."""
    spec = hpfem.poisson3d(6, 3, seed=74)
    m = _run(spec, uo.CHOL, False)
    b = api.Mesh()
    m.backup(b)
    m.check_reuse(b)
    m.factor(uo.CHOL)
    assert m.n_refactored() == 0
    m.solve(uo.CHOL)
    ref = uo.solve_mesh(spec, uo.CHOL).x
    assert np.abs(_x(m, spec) - ref).max() <= 1e-10 * np.abs(ref).max()


def test_flagged_front_with_changed_child_is_redone(native_lib):
    """Only the changed leaf is left unflagged; its ancestors keep their flags
    (as the reference's check_reuse can leave them), yet they are redone."""
    spec = hpfem.poisson3d(6, 3, seed=75)
    m = _run(spec, uo.CHOL, False)
    for e in m._elts:
        m.set_reuse(e, True)
    k = 3
    m.set_reuse(m._elts[k], False)
    mk = int(spec.elem_m[k])
    m.copy_in(m._elts[k], spec.element_nodes(k), api.UHM_LHS, 2.0 * np.eye(mk))
    m.factor(uo.CHOL)
    assert m.n_refactored() == len(_path(spec, k))
    m.solve(uo.CHOL)
    ref = uo.solve_mesh(_bumped(spec, k, 2.0), uo.CHOL).x
    assert np.abs(_x(m, spec) - ref).max() <= 1e-10 * np.abs(ref).max()
