"""Per-front blocks read back through uhm::Matrix_ (uhm_gpu_get_front_block).

A leaf front's assembled matrix is its element matrix, so its blocks can be
checked independently of the solver: with the element matrix permuted into
front order (factor nodes first, then Schur nodes, each node's dofs in
order), ATL must hold L = chol(A_ff), ABL = A_sf L^{-T}, ABR = A_ss -
ABL ABL^T (lower triangles), to 1e-12 relative in FP64.  The mesh is 3D
p = 6, so the leaf fronts (n = 343) take the blocked kernels, whose 64 x 64
diagonal blocks are held by their inverses on the device.  After the solve,
XT / XB must equal the solution at the front's rows."""
import numpy as np
import pytest

from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu


def _front_perm(m, spec, e):
    fac, sch = m.front_nodes(e)
    rows, pos = {}, 0
    for nid in spec.element_nodes(e).tolist():
        k = int(spec.node_ndof[nid])
        rows[nid] = list(range(pos, pos + k))
        pos += k
    perm = [r for nid in list(fac) + list(sch) for r in rows[int(nid)]]
    nf = sum(int(spec.node_ndof[nid]) for nid in fac)
    return np.array(perm), nf


def test_leaf_front_blocks_match_dense_partial_factorisation(native_lib):
    spec = hpfem.poisson3d(2, 6, seed=41)
    m = api.load_spec(spec)
    m.set_mode(0)
    m.chol_with_free()
    eid, _, fs, ss = m.fronts()
    e = 0
    k = int(np.nonzero(eid == e)[0][0])
    assert fs[k] + ss[k] > 160            # a blocked front
    perm, nf = _front_perm(m, spec, e)
    A = spec.element_matrix(e)[np.ix_(perm, perm)]
    L11 = np.linalg.cholesky(A[:nf, :nf])
    L21 = np.linalg.solve(L11, A[:nf, nf:]).T
    S = A[nf:, nf:] - L21 @ L21.T
    scale = np.abs(A).max()
    assert np.abs(m.front_block(e, "ATL") - L11).max() <= 1e-12 * scale
    assert np.abs(m.front_block(e, "ABL") - L21).max() <= 1e-12 * scale
    assert np.abs(m.front_block(e, "ABR") - np.tril(S)).max() <= 1e-12 * scale
    # after the solve: the front's rows of the solution
    m.solve_chol()
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, 1)[:, 0]
    fac, sch = m.front_nodes(e)
    starts = np.concatenate([[0], np.cumsum(spec.node_ndof)])
    want = np.concatenate([x[starts[n]:starts[n + 1]] for n in list(fac) + list(sch)])
    xt, xb = m.front_block(e, "XT")[:, 0], m.front_block(e, "XB")[:, 0]
    got = np.concatenate([xt, xb])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(x).max()


def test_lu_front_pivots_and_blocks_read_back(native_lib):
    spec = hpfem.convdiff3d(2, 3, seed=42)
    m = api.load_spec(spec)
    m.set_mode(0)
    m.lu_piv_with_free()
    eid, _, fs, ss = m.fronts()
    root = int(eid[-1])
    p = m.front_block(root, "P")
    assert p.shape == (int(fs[-1]),) and (p >= 0).all() and (p < fs[-1] + ss[-1]).all()
    atl = m.front_block(root, "ATL")
    assert atl.shape == (int(fs[-1]), int(fs[-1])) and np.isfinite(atl).all()
