"""Many independent meshes joined into one forest (hpfem.forest), no GPU.

The oracle solves the forest and each mesh on its own: the forest's solution
is the concatenation of the separate ones, its fronts are the union of theirs,
and the native symbolic phase (Mesh_::lock through the C ABI) gives the same
front structure as the oracle.  The device side is covered by
test_gpu_forest.py."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem


def _parts():
    return [hpfem.poisson2d(3, 2, seed=1, n_rhs=2),
            hpfem.poisson3d(2, 2, seed=2, n_rhs=2),
            hpfem.diffusion3d(2, 3, seed=3, contrast=1e3, n_rhs=2),
            hpfem.poisson2d(4, 3, seed=4, n_rhs=2)]


def test_forest_layout():
    parts = _parts()
    f = hpfem.forest(parts)
    assert f.n_leaves == sum(p.n_leaves for p in parts)
    assert f.n_elements == sum(p.n_elements for p in parts)
    assert f.n_dof() == sum(p.n_dof() for p in parts)
    assert int((f.parent < 0).sum()) == len(parts)
    assert len(np.unique(f.node_id)) == f.n_nodes
    # every child points back to its parent, and generations decrease towards the roots
    for e in range(f.n_elements):
        for c in f.children(e):
            assert f.parent[c] == e and f.generation[c] > f.generation[e]
    # element matrices are carried over unchanged
    for k, p in enumerate(parts):
        lo = f.info["parts"][k]["leaves"][0]
        for e in (0, p.n_leaves - 1):
            assert np.array_equal(f.element_matrix(lo + e), p.element_matrix(e))
            assert np.array_equal(f.element_rhs(lo + e), p.element_rhs(e))


def test_forest_rejects_mixed_rhs_counts():
    with pytest.raises(ValueError):
        hpfem.forest([hpfem.poisson2d(2, 2, n_rhs=1), hpfem.poisson2d(2, 2, n_rhs=2)])


def test_oracle_forest_equals_separate_solves():
    parts = _parts()
    f = hpfem.forest(parts)
    xf = uo.solve_mesh(f, uo.CHOL).x
    xs = np.concatenate([uo.solve_mesh(p, uo.CHOL).x for p in parts])
    assert xf.shape == xs.shape
    assert np.abs(xf - xs).max() <= 1e-12 * np.abs(xs).max()
    fs_f = sorted(map(tuple, uo.symbolic(f).fs_ss().tolist()))
    fs_s = sorted(t for p in parts for t in map(tuple, uo.symbolic(p).fs_ss().tolist()))
    assert fs_f == fs_s


def test_native_lock_of_forest_matches_oracle(native_lib):
    f = hpfem.forest(_parts())
    m = api.load_spec(f)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((f.n_elements, 2), np.int64)
    got[eid] = np.stack([fs, ss], axis=1)
    plan = uo.symbolic(f)
    assert np.array_equal(got, plan.fs_ss())
    assert m.get_n_dof() == f.n_dof()


def test_ragged_nested_dissection_structure(native_lib):
    """n = 7 has no exact 2/3/5 merge plan: ceiling halving 7 -> 4 -> 2 -> 1,
    with parents of fewer than 8 children at the far faces; the native
    symbolic phase must give the oracle's fronts."""
    spec = hpfem.poisson3d(7, 2, seed=6)
    assert spec.info["merges"] == [2, 2, 2]
    kids = np.diff(spec.child_ptr)[spec.n_leaves:]
    assert kids.min() == 1 and kids.max() == 8
    m = api.load_spec(spec)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((spec.n_elements, 2), np.int64)
    got[eid] = np.stack([fs, ss], axis=1)
    assert np.array_equal(got, uo.symbolic(spec).fs_ss())
