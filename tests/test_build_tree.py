"""Assembly tree built by the library (uhm_build_tree_, heavy-edge matching
after UHM/src/operation/build_tree_var1.cxx:53-181), no GPU.

Leaves only go in; after build_tree and lock, the tree must be a valid
assembly tree over every leaf (children before parents in generation, one
root per connected part), every interior front must eliminate something,
the native symbolic fronts must equal the oracle's on the same tree, and the
oracle's solution on the built tree must equal its solution on the mesh's
nested-dissection tree."""
import dataclasses

import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem


def _leaves_only(spec):
    m = api.Mesh()
    nods = {nid: m.add_node(nid, nd, p)
            for nid, nd, p in zip(spec.node_id.tolist(), spec.node_ndof.tolist(), spec.node_p.tolist())}
    elts = [m.add_element(0) for _ in range(spec.n_leaves)]
    for e in range(spec.n_leaves):
        for nid in spec.element_nodes(e).tolist():
            m.element_add_node(elts[e], nods[nid])
    return m


def _as_spec(spec, m):
    """the spec with the mesh's tree: leaves first, interior elements by id"""
    eid, par, gen, kids = m.tree()
    L = spec.n_leaves
    order = list(range(L)) + sorted(int(e) for e in eid if e >= L)
    idx = {e: i for i, e in enumerate(order)}
    pmap = dict(zip(eid.tolist(), par.tolist()))
    gmap = dict(zip(eid.tolist(), gen.tolist()))
    parent = np.array([idx[pmap[e]] if pmap[e] >= 0 else -1 for e in order])
    generation = np.array([gmap[e] for e in order])
    cp, ci = [0], []
    for e in order:
        ci += [idx[c] for c in kids[e]]
        cp.append(len(ci))
    s = dataclasses.replace(spec, parent=parent, generation=generation, child_ptr=np.array(cp),
                            child_idx=np.array(ci, dtype=np.int64))
    return s, idx


def _built(spec):
    m = _leaves_only(spec)
    m.build_tree()
    m.lock()
    m.create_matrix_without_buffer(api.UHM_REAL, spec.n_rhs)
    return m


CASES = [
    ("poisson3d_4_p3", lambda: hpfem.poisson3d(4, 3, seed=1), uo.CHOL),
    ("convdiff3d_4_p2", lambda: hpfem.convdiff3d(4, 2, seed=2), uo.LU_PIV),
    ("poisson2d_8_p2", lambda: hpfem.poisson2d(8, 2, seed=3), uo.CHOL),
    ("poisson3d_4_p1", lambda: hpfem.poisson3d(4, 1, seed=4), uo.CHOL),
    ("varp3d_3", lambda: hpfem.build_mesh(3, 3, np.random.default_rng(5).integers(1, 5, 27), seed=5), uo.CHOL),
]


@pytest.mark.parametrize("name,make,method", CASES, ids=[c[0] for c in CASES])
def test_built_tree_is_valid_and_solves_like_the_original(native_lib, name, make, method):
    spec = make()
    m = _built(spec)
    s2, idx = _as_spec(spec, m)
    L = spec.n_leaves
    assert (s2.parent < 0).sum() == 1
    for e in range(s2.n_elements):
        if s2.parent[e] >= 0:
            assert s2.generation[e] > s2.generation[s2.parent[e]]
        kids = s2.child_idx[s2.child_ptr[e]:s2.child_ptr[e + 1]]
        assert (len(kids) == 0) == (e < L)
        assert all(s2.parent[c] == e for c in kids)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((s2.n_elements, 2), np.int64)
    for e, f, s in zip(eid.tolist(), fs.tolist(), ss.tolist()):
        got[idx[e]] = (f, s)
    assert np.array_equal(got, uo.symbolic(s2).fs_ss())
    assert (got[L:, 0] > 0).all()                       # every interior front eliminates something
    x_built = uo.solve_mesh(s2, method).x
    x_nd = uo.solve_mesh(spec, method).x
    assert np.abs(x_built - x_nd).max() <= 1e-10 * np.abs(x_nd).max()


def test_disconnected_parts_become_separate_trees(native_lib):
    parts = [hpfem.poisson3d(2, 2, seed=6), hpfem.poisson2d(3, 2, seed=7)]
    f = hpfem.forest(parts)
    m = _built(f)
    s2, _ = _as_spec(f, m)
    assert (s2.parent < 0).sum() == 2
    x = uo.solve_mesh(s2, uo.CHOL).x
    xs = np.concatenate([uo.solve_mesh(p, uo.CHOL).x for p in parts])
    assert np.abs(x - xs).max() <= 1e-10 * np.abs(xs).max()


def test_build_is_deterministic(native_lib):
    spec = hpfem.poisson3d(4, 2, seed=8)
    t1 = _built(spec).tree()
    t2 = _built(spec).tree()
    assert all(np.array_equal(a, b) for a, b in zip(t1[:3], t2[:3]))
    assert t1[3] == t2[3]


def test_built_mesh_takes_the_usual_calls(native_lib):
    """build_tree then lock, create_matrix, bulk copy_in: the reference's
    Fortran sequence (UHM/example/f90/ex1.f90) up to the factorisation."""
    spec = hpfem.poisson3d(3, 2, seed=9)
    m = _built(spec)
    m.copy_in_leaves(api.UHM_LHS, spec.mats, spec.elem_node.astype(np.int32))
    m.copy_in_leaves(api.UHM_RHS, spec.rhs)
    assert m.status() == 0
    assert m.get_n_dof() == spec.n_dof()


def _write_uhm(spec, path, extra_node=False):
    """the leaves of a spec in the .uhm text format Mesh_::import_file reads
    (UHM/src/mesh/mesh.cxx:511-579): nodes "id phy n_dof p kind", then per
    element its node count and "id phy" lines"""
    lines = ["# written for the import test", "UHM", str(spec.n_nodes + (1 if extra_node else 0))]
    for i, d, p, k in zip(spec.node_id, spec.node_ndof, spec.node_p, spec.node_kind):
        lines.append(f"{int(i)} 0 {int(d)} {int(p)} {int(k)}")
    if extra_node:
        lines.append(f"{int(spec.node_id.max()) + 1} 0 5 2 0")     # owned by no element: dropped
    lines.append(str(spec.n_leaves))
    for e in range(spec.n_leaves):
        nl = spec.element_nodes(e)
        lines.append(str(len(nl)))
        lines += [f"{int(n)} 0" for n in nl]
    path.write_text("\n".join(lines) + "\n")


def test_import_then_build_tree(native_lib, tmp_path):
    """The reference's file-driven flow: import_file (leaves only), build_tree,
    lock, create_matrix, copy_in -- fronts equal the oracle's on the built tree."""
    spec = hpfem.convdiff3d(3, 2, seed=10)
    f = tmp_path / "mesh.uhm"
    _write_uhm(spec, f, extra_node=True)
    m = api.Mesh()
    m.import_file(str(f))
    m.build_tree()
    m.lock()
    m.create_matrix_without_buffer(api.UHM_REAL, spec.n_rhs)
    assert m.get_n_dof() == spec.n_dof()                 # the orphan node's 5 dofs are gone
    m.copy_in_leaves(api.UHM_LHS, spec.mats, spec.elem_node.astype(np.int32))
    assert m.status() == 0
    s2, idx = _as_spec(spec, m)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((s2.n_elements, 2), np.int64)
    for e, a, b in zip(eid.tolist(), fs.tolist(), ss.tolist()):
        got[idx[e]] = (a, b)
    assert np.array_equal(got, uo.symbolic(s2).fs_ss())
    x = uo.solve_mesh(s2, uo.LU_PIV).x
    ref = uo.solve_mesh(spec, uo.LU_PIV).x
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("bad", ["header", "node"])
def test_import_rejects_bad_files(native_lib, tmp_path, bad):
    spec = hpfem.poisson2d(2, 2, seed=11)
    f = tmp_path / "bad.uhm"
    _write_uhm(spec, f)
    text = f.read_text()
    if bad == "header":
        text = text.replace("UHM", "XYZ", 1)
    else:
        text = text.rstrip("\n") + "\n1\n999999 0\n"
        text = text.replace(f"\n{spec.n_leaves}\n", f"\n{spec.n_leaves + 1}\n", 1)
    f.write_text(text)
    m = api.Mesh()
    with pytest.raises(api.UHMError):
        m.import_file(str(f))
    assert m.status() != 0
