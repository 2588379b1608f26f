"""Sparse export of the assembled operator (uhm_gpu_export_sparse, the
reference's DSparse_: UHM/src/interf/sparse.cxx:188-460), host only.

The exported matrix and right-hand sides must equal the oracle's assembly
(oracle.uhm_oracle.assemble) after renumbering its canonical dofs into the
mesh's numbering (uhm_gpu_get_node_offsets).  The values must equal, bit for
bit, the reference's accumulation restated here: a map keyed by (row, col)
whose first contribution inserts and whose later ones add, leaves in order.
The compressed, symmetric, column-major and Fortran-numbered forms must
describe the same matrix."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem


def _native_dofs(m, spec):
    """canonical dof -> the mesh's global dof"""
    offs = m.node_offsets(spec.node_id)
    perm = np.zeros(spec.n_dof(), np.int64)
    coff = uo.node_dof_offsets(spec.node_ndof)
    for k in range(spec.n_nodes):
        nd = int(spec.node_ndof[k])
        perm[coff[k]:coff[k] + nd] = offs[k] + np.arange(nd)
    return perm


def _map_accumulate(spec, perm):
    acc = {}
    for e in range(spec.n_leaves):
        d = perm[uo.element_dofs(spec, e)]
        A = spec.element_matrix(e)
        for j in range(len(d)):
            for i in range(len(d)):
                key = (int(d[i]), int(d[j]))
                if key in acc:
                    acc[key] = acc[key] + A[i, j]
                else:
                    acc[key] = A[i, j]
    return acc


MESHES = [
    ("poisson2d", lambda: hpfem.poisson2d(4, 3, seed=81, n_rhs=2)),
    ("convdiff3d", lambda: hpfem.convdiff3d(2, 2, seed=82)),
    ("varp3d", lambda: hpfem.build_mesh(3, 2, [2, 3, 2, 4, 3, 2, 2, 3], seed=83)),
]


@pytest.mark.parametrize("name,make", MESHES, ids=[c[0] for c in MESHES])
def test_triplets_equal_the_oracle_assembly(native_lib, name, make):
    spec = make()
    m = api.load_spec(spec)
    s = m.export_sparse()
    n = spec.n_dof()
    assert s["n_dof"] == n and s["n_rhs"] == spec.n_rhs
    assert len(s["ia"]) == len(s["ja"]) == len(s["a"])
    keys = s["ia"].astype(np.int64) * n + s["ja"]
    assert np.all(np.diff(keys) > 0)                     # key order, no duplicates
    perm = _native_dofs(m, spec)
    A, b = uo.assemble(spec)
    P = sp.csr_matrix((np.ones(n), (perm, np.arange(n))), shape=(n, n))
    Ao = (P @ A @ P.T).tocoo()
    Ae = sp.csr_matrix((s["a"], (s["ia"], s["ja"])), shape=(n, n))
    assert abs(Ae - Ao).max() <= 1e-14 * abs(Ao).max()
    bo = np.zeros_like(b)
    bo[perm] = b
    assert np.abs(s["b"] - bo).max() <= 1e-14 * np.abs(bo).max()
    # bit-identical to the reference's map accumulation (leaf order)
    acc = _map_accumulate(spec, perm)
    assert len(acc) == len(s["a"])
    got = {(int(i), int(j)): v for i, j, v in zip(s["ia"], s["ja"], s["a"])}
    assert all(got[k] == v for k, v in acc.items())


def test_forms_describe_one_matrix(native_lib):
    spec = hpfem.poisson3d(2, 3, seed=84, n_rhs=3)
    m = api.load_spec(spec)
    n = spec.n_dof()
    full = m.export_sparse()
    A = sp.csr_matrix((full["a"], (full["ia"], full["ja"])), shape=(n, n))
    # compressed rows
    c = m.export_sparse(compress=True)
    assert c["n_dof"] == n and len(c["ia"]) == n + 1
    assert (sp.csr_matrix((c["a"], c["ja"], c["ia"]), shape=(n, n)) != A).nnz == 0
    # compressed columns, Fortran numbering
    cf = m.export_sparse(compress=True, cs=True, fort=True)
    assert cf["ja"][0] == 1 and cf["ja"][-1] == len(cf["a"]) + 1
    Acsc = sp.csc_matrix((cf["a"], cf["ia"] - 1, cf["ja"] - 1), shape=(n, n))
    assert (Acsc.tocsr() != A).nnz == 0
    # symmetric: upper triangle by rows (cs = 0) or lower by columns' keys (cs = 1)
    su = m.export_sparse(is_sym=True)
    assert np.all(su["ja"] >= su["ia"])
    assert (sp.csr_matrix((su["a"], (su["ia"], su["ja"])), shape=(n, n)) != sp.triu(A).tocsr()).nnz == 0
    sl = m.export_sparse(is_sym=True, cs=True)
    assert np.all(sl["ia"] >= sl["ja"])
    assert (sp.csr_matrix((sl["a"], (sl["ia"], sl["ja"])), shape=(n, n)) != sp.tril(A).tocsr()).nnz == 0
    assert np.array_equal(full["b"], c["b"])
    assert full["b"].shape == (n, 3)


def test_axpy_off_keeps_the_first_contribution(native_lib):
    spec = hpfem.poisson2d(2, 2, seed=85)
    m = api.load_spec(spec)
    s = m.export_sparse(axpy=False)
    perm = _native_dofs(m, spec)
    first = {}
    for e in range(spec.n_leaves):
        d = perm[uo.element_dofs(spec, e)]
        A = spec.element_matrix(e)
        for j in range(len(d)):
            for i in range(len(d)):
                first.setdefault((int(d[i]), int(d[j])), A[i, j])
    got = {(int(i), int(j)): v for i, j, v in zip(s["ia"], s["ja"], s["a"])}
    assert got == first


def test_export_needs_element_matrices(native_lib):
    spec = hpfem.poisson2d(2, 2, seed=86)
    m = api.load_spec(spec, lhs=False)
    with pytest.raises(api.UHMError):
        m.export_sparse()


def test_export_without_right_hand_sides(native_lib):
    spec = hpfem.poisson2d(3, 2, seed=87)
    m = api.Mesh()
    nods = {nid: m.add_node(nid, nd, p)
            for nid, nd, p in zip(spec.node_id.tolist(), spec.node_ndof.tolist(), spec.node_p.tolist())}
    elts = [m.add_element(int(g)) for g in spec.generation.tolist()]
    for e in range(spec.n_leaves):
        for nid in spec.element_nodes(e).tolist():
            m.element_add_node(elts[e], nods[nid])
    for e in range(spec.n_elements):
        for c in spec.children(e).tolist():
            m.set_parent(elts[c], elts[e])
            m.add_child(elts[e], elts[c])
    m.lock()
    m.create_matrix_without_buffer(api.UHM_REAL, 1)
    m.copy_in_leaves(api.UHM_LHS, spec.mats, spec.elem_node.astype(np.int32))
    s = m.export_sparse()
    full = api.load_spec(spec).export_sparse()
    assert s["n_rhs"] == 0 and s["b"].size == 0
    assert np.array_equal(s["ia"], full["ia"]) and np.array_equal(s["a"], full["a"])


# ---- pinned to the reference's own DSparse_ (tests/golden/sparse_*.npz) ----
import importlib.util  # noqa: E402
import os  # noqa: E402

from oracle import ref_runner  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_gs = importlib.util.spec_from_file_location("golden_cases_sparse", os.path.join(GOLDEN, "cases.py"))
golden_cases = importlib.util.module_from_spec(_gs)
_gs.loader.exec_module(golden_cases)
SPARSE_CASES = golden_cases.SPARSE_CASES


def _by_node_dof(offsets, spec, ia, ja, a):
    """triplets keyed by ((node index, dof k), (node index, dof k)), whatever
    the numbering that produced them"""
    owner = {}
    for i, (o, d) in enumerate(zip(offsets.tolist(), spec.node_ndof.tolist())):
        for k in range(d):
            owner[o + k] = (i, k)
    return {(owner[int(r)], owner[int(c)]): v for r, c, v in zip(ia, ja, a)}, owner


def _compare_with_reference(m, spec, ref):
    s = m.export_sparse()
    ours, our_owner = _by_node_dof(m.node_offsets(spec.node_id), spec, s["ia"], s["ja"], s["a"])
    theirs, ref_owner = _by_node_dof(ref["offsets"], spec, ref["ia"], ref["ja"], ref["a"])
    assert ours.keys() == theirs.keys()
    assert all(ours[k] == theirs[k] for k in theirs)                 # bit for bit
    n, nr = spec.n_dof(), spec.n_rhs
    assert ref["n_dof"] == n - 1                                     # the reference's triplet: its last row index
    rb = np.asarray(ref["b"]).reshape(nr, n).T                       # column-major over the reference's rows
    ob = s["b"]
    for g_ref, key in ref_owner.items():
        g_our = [g for g, kk in our_owner.items() if kk == key][0]
        assert np.array_equal(ob[g_our], rb[g_ref])


@pytest.mark.parametrize("name,gen,kw", SPARSE_CASES, ids=[c[0] for c in SPARSE_CASES])
def test_export_equals_reference_fixture(native_lib, name, gen, kw):
    g = dict(np.load(os.path.join(GOLDEN, "sparse_" + name + ".npz")))
    spec = golden_cases.make_spec(gen, kw)
    assert golden_cases.spec_digest(spec) == str(g["digest"]), "mesh generator changed: regenerate fixtures"
    _compare_with_reference(api.load_spec(spec), spec, g)


@pytest.mark.skipif(not ref_runner.available(), reason="reference solver not built here (make -C oracle)")
def test_export_equals_live_reference(native_lib):
    spec = hpfem.diffusion3d(3, 3, seed=24, contrast=1e3, n_rhs=2)
    _compare_with_reference(api.load_spec(spec), spec, ref_runner.run_sparse(spec))
