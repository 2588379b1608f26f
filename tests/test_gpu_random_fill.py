"""Random element matrices (uhm_random_spd_matrix_ / uhm_random_matrix_, the
reference's benchmark fills) factored and solved on the device: Cholesky on
the SPD fill, LU with partial pivoting on the general one, each to a backward
error of 1e-12 on the assembled operator."""
import numpy as np
import pytest

from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("spd,method", [(True, api.UHM_CHOL), (False, api.UHM_LU_PIV)], ids=["spd_chol", "gen_lupiv"])
def test_random_fill_factor_solve(native_lib, spd, method):
    spec = hpfem.poisson3d(4, 3, seed=3, n_rhs=2)
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
    m.create_matrix_without_buffer(api.UHM_REAL, spec.n_rhs)
    (m.random_spd_matrix if spd else m.random_matrix)()
    m.factor(method)
    m.solve(method)
    assert m.status() == 0
    assert m.backward_error() <= 1e-12
    # the solution against a dense solve of the exported operator
    s = m.export_sparse()
    n = s["n_dof"]
    A = np.zeros((n, n))
    A[s["ia"], s["ja"]] = s["a"]
    x = np.linalg.solve(A, s["b"])
    offs = m.node_offsets(spec.node_id)
    got = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)
    rows = np.concatenate([np.arange(o, o + d) for o, d in zip(offs, spec.node_ndof) if d])
    assert np.abs(got - x[rows]).max() <= 1e-10 * np.abs(x).max()
