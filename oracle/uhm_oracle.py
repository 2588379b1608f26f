"""CPU oracle for the UHM multifrontal factor/solve path (TEST INFRASTRUCTURE).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm may
import it.  It is a numpy/scipy restatement of the reference's algorithm, one
function per reference step, each citing the reference file:line it follows
(paths relative to the UHM project root).  Dense kernels go through scipy's
LAPACK/BLAS, as the reference's go through libflame/BLAS.

Pinning: ``tests/golden/`` holds outputs of the reference's own C++ sources
(UHM + LINAL, compiled against a project-written FLAME-subset shim, recipe in
``oracle/Makefile``); ``tests/test_oracle_golden.py`` checks this module
against them.  The dense arithmetic of the shim is OpenBLAS, not libflame, so
fidelity to libflame's own rounding is not pinned (libflame is absent).

Differences from the reference that are deliberate:
* ``numbering`` visits an element's factor nodes in node-id order.  The
  reference walks ``std::map<Node_*,int>`` (pointer order,
  UHM/src/mesh/element.cxx:383-392), which depends on heap addresses; node
  *sets*, (fs, ss) sizes and the tree are unaffected.
* the forward solve merges the right-hand side of each child once (b and the
  child update together); the reference merges b during the factorisation
  (op_merge_full_* with x=1, UHM/src/operation/element.cxx:135-185) and the
  update during solve_*_1.  The sums are mathematically identical.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla
from scipy.linalg import blas as fblas
from scipy.linalg import lapack as flapack

CHOL, LU_NOPIV, LU_PIV = 1, 2, 3      # UHM/include/uhm/const.hxx:82-86 (enum UHM_CHOL=1, ...)


# ----------------------------------------------------------------------------
# LAWN-41 flop model  (LINAL/src/util.cxx:60-116)
# ----------------------------------------------------------------------------
def flop_gemm(m, n, k):
    return 2.0 * m * n * k


def flop_syrk(k, n):
    return 2.0 * 0.5 * k * n * (n + 1.0)


def flop_trsm_lower(m, n):
    return 0.5 * n * m * (m + 1.0) + 0.5 * n * m * (m - 1.0)


def flop_trsm_upper(m, n):
    return 0.5 * m * n * (n + 1.0) + 0.5 * m * n * (n - 1.0)


def flop_chol(n):
    return ((1.0 / 6.0) * n ** 3 + 0.5 * n * n + (1.0 / 3.0) * n) + ((1.0 / 6.0) * n ** 3 - (1.0 / 6.0) * n)


def flop_lu(m, n):
    if m > n:
        return ((0.5 * m * n * n - (1.0 / 6.0) * n ** 3 + 0.5 * m * n - 0.5 * n * n + (2.0 / 3.0) * n)
                + (0.5 * m * n * n - (1.0 / 6.0) * n ** 3 - 0.5 * m * n + (1.0 / 6.0) * n))
    return ((0.5 * n * m * m - (1.0 / 6.0) * m ** 3 + 0.5 * n * m - 0.5 * m * m + (2.0 / 3.0) * m)
            + (0.5 * n * m * m - (1.0 / 6.0) * m ** 3 - 0.5 * n * m + (1.0 / 6.0) * m))


def front_cost(method, fs, ss, n_rhs):
    """Element_::estimate_cost (UHM/src/mesh/element.cxx:128-195), real case."""
    if method == CHOL:
        dec = flop_chol(fs) + flop_trsm_lower(fs, ss) + flop_syrk(fs, ss)
    else:
        dec = flop_lu(fs, fs) + flop_trsm_lower(fs, ss) + flop_trsm_upper(ss, fs) + flop_gemm(ss, ss, fs)
    sol = (flop_trsm_lower(fs, n_rhs) + flop_gemm(ss, n_rhs, fs) + flop_trsm_upper(n_rhs, fs)
           + flop_gemm(fs, n_rhs, ss))
    return dec, sol


# ----------------------------------------------------------------------------
# Symbolic analysis: Mesh_::lock  (UHM/src/mesh/mesh.cxx:438-456)
# ----------------------------------------------------------------------------
@dataclass
class Front:
    eid: int
    gen: int
    parent: int
    children: list
    factor: list = field(default_factory=list)   # [(node, offset_in_block)]
    schur: list = field(default_factory=list)
    fs: int = 0
    ss: int = 0


@dataclass
class Plan:
    fronts: list
    node_ndof: np.ndarray
    node_offset: np.ndarray       # global offset (elimination numbering)
    order_leaf2root: list         # element ids, generation descending, id ascending
    owner_front: np.ndarray       # per node: front where it is FACTOR (-1: zero dof / none)
    node_pos: np.ndarray          # per node: offset inside owner's factor block

    def fs_ss(self):
        return np.array([[f.fs, f.ss] for f in self.fronts], dtype=np.int64)


def symbolic(spec) -> Plan:
    """Restates Mesh_::lock: Scheduler_::load grouping by generation
    (UHM/src/operation/scheduler.cxx:157-178), op_restore_connectivity on the
    leaves (UHM/src/mesh/element.cxx:362-381), op_update_connectivity leaf to
    root = merge_nodes_from_children + separate_nodes (element.cxx:336-360,
    272-286), op_numbering (element.cxx:383-392) and op_arrange_nodes
    (element.cxx:288-334)."""
    n_el = spec.n_elements
    gen = spec.generation
    # Scheduler_::load: std::map<int gen, vector<Element>> filled in element-id order;
    # execute_elements_seq(leaf2root) walks generations from the highest down.
    order = sorted(range(n_el), key=lambda e: (-int(gen[e]), e))
    kind = spec.node_kind
    ndof = spec.node_ndof
    owners = [set() for _ in range(spec.n_nodes)]
    nodes = [dict() for _ in range(n_el)]            # node -> separation flag
    # restore_connectivity: leaves own their initial nodes
    for e in range(spec.n_leaves):
        for nd in spec.element_nodes(e):
            nd = int(nd)
            nodes[e][nd] = 0
            owners[nd].add(e)
    is_leaf = [spec.child_ptr[e + 1] == spec.child_ptr[e] for e in range(n_el)]
    for e in order:
        if not is_leaf[e]:
            nodes[e] = {}
            for c in spec.children(e):
                c = int(c)
                for nd, sep in nodes[c].items():
                    if sep == 2:                      # UHM_SEPARATED_SCHUR
                        if nd not in nodes[e]:
                            nodes[e][nd] = 0
                            owners[nd].add(e)
                        owners[nd].discard(c)
        for nd in nodes[e]:
            assert owners[nd], "node without owner"
            nodes[e][nd] = 1 if (len(owners[nd]) == 1 and kind[nd] == 0) else 2
    # numbering (node-id order inside an element; see module docstring)
    offset = np.zeros(spec.n_nodes, dtype=np.int64)
    g = 0
    for e in order:
        for nd in sorted(nodes[e]):
            if nodes[e][nd] == 1:
                offset[nd] = g
                g += int(ndof[nd])
    fronts = []
    owner_front = np.full(spec.n_nodes, -1, dtype=np.int64)
    node_pos = np.zeros(spec.n_nodes, dtype=np.int64)
    for e in range(n_el):
        f = Front(eid=e, gen=int(gen[e]), parent=int(spec.parent[e]),
                  children=[int(c) for c in spec.children(e)])
        fac = sorted((int(offset[nd]), nd) for nd, s in nodes[e].items() if s == 1 and ndof[nd])
        sch = sorted((int(offset[nd]), nd) for nd, s in nodes[e].items() if s == 2 and ndof[nd])
        o = 0
        for _, nd in fac:
            f.factor.append((nd, o))
            owner_front[nd] = e
            node_pos[nd] = o
            o += int(ndof[nd])
        f.fs = o
        o = 0
        for _, nd in sch:
            f.schur.append((nd, o))
            o += int(ndof[nd])
        f.ss = o
        fronts.append(f)
    return Plan(fronts, ndof.copy(), offset, order, owner_front, node_pos)


def _front_index(front: Front, ndof):
    """node -> (part, offset): part 0 = factor (top), 1 = schur (bottom)."""
    d = {}
    for nd, o in front.factor:
        d[nd] = (0, o)
    for nd, o in front.schur:
        d[nd] = (1, o)
    return d


def child_map(plan: Plan, parent: int, child: int):
    """Helper_::set_mapper (UHM/include/uhm/matrix/uhm/helper.hxx:98-158) at dof
    granularity: for every schur dof of the child, (part, index) in the parent."""
    ndof = plan.node_ndof
    pidx = _front_index(plan.fronts[parent], ndof)
    part = []
    pos = []
    for nd, _o in plan.fronts[child].schur:
        pp, po = pidx[nd]
        for k in range(int(ndof[nd])):
            part.append(pp)
            pos.append(po + k)
    return np.asarray(part, dtype=np.int64), np.asarray(pos, dtype=np.int64)


def element_map(plan: Plan, spec, e: int):
    """Mesh_::copy_in's phony child (UHM/src/mesh/interf.cxx:108-204): the user
    dof order is the element's node order with each node's dofs contiguous."""
    ndof = plan.node_ndof
    idx = _front_index(plan.fronts[e], ndof)
    part = []
    pos = []
    for nd in spec.element_nodes(e):
        nd = int(nd)
        for k in range(int(ndof[nd])):
            pp, po = idx[nd]
            part.append(pp)
            pos.append(po + k)
    return np.asarray(part, dtype=np.int64), np.asarray(pos, dtype=np.int64)


# ----------------------------------------------------------------------------
# Numeric factorisation
# ----------------------------------------------------------------------------
class FrontData:
    __slots__ = ("ATL", "ATR", "ABL", "ABR", "piv", "bt", "bb", "xt", "xb")


def _scatter_add(blocks, part, pos, src):
    """Helper_::_merge_A / Matrix_FLA_::merge (helper.hxx:191-222,
    UHM/src/matrix/uhm/fla/matrix.cxx:284-303): parent[rows, cols] += src."""
    t = np.nonzero(part == 0)[0]
    b = np.nonzero(part == 1)[0]
    ATL, ATR, ABL, ABR = blocks
    pt, pb = pos[t], pos[b]
    if len(t):
        ATL[np.ix_(pt, pt)] += src[np.ix_(t, t)]
    if len(t) and len(b):
        ATR[np.ix_(pt, pb)] += src[np.ix_(t, b)]
        ABL[np.ix_(pb, pt)] += src[np.ix_(b, t)]
    if len(b):
        ABR[np.ix_(pb, pb)] += src[np.ix_(b, b)]


def _lu_nopiv_inplace(A):
    """Right-looking LU without pivoting (LINAL/src/dense/lu_nopiv.cxx:104-146
    with FLA_LU_nopiv on the diagonal block)."""
    n = A.shape[0]
    nb = 64
    for k in range(0, n, nb):
        e = min(k + nb, n)
        for j in range(k, e):
            A[j + 1:, j] /= A[j, j]
            A[j + 1:, j + 1:e] -= np.outer(A[j + 1:, j], A[j, j + 1:e])
        if e < n:
            L11 = np.tril(A[k:e, k:e], -1) + np.eye(e - k)
            A[k:e, e:] = sla.solve_triangular(L11, A[k:e, e:], lower=True, unit_diagonal=True)
            A[e:, e:] -= A[e:, k:e] @ A[k:e, e:]
    return A


def factor_front(method, d: FrontData, fs: int, ss: int):
    """Matrix_FLA_::chol / lu_nopiv / lu_piv of one front:
    chol_hier (UHM/src/matrix/uhm/fla/chol/decompose.cxx:85-98),
    lu_nopiv_hier (fla/lu_nopiv/decompose.cxx:95-121),
    lu_piv_hier (fla/lu_piv/decompose.cxx:124-153)."""
    if method == CHOL:
        if fs:
            c, info = flapack.dpotrf(d.ATL, lower=1, clean=1, overwrite_a=1)
            if info != 0:
                raise np.linalg.LinAlgError(f"front not positive definite (info={info})")
            d.ATL = c
        if fs and ss:
            d.ABL = fblas.dtrsm(1.0, d.ATL, d.ABL, side=1, lower=1, trans_a=1, diag=0, overwrite_b=1)
            d.ABR = fblas.dsyrk(-1.0, d.ABL, beta=1.0, c=d.ABR, trans=0, lower=1, overwrite_c=1)
    elif method == LU_PIV:
        if fs:
            lu, piv, info = flapack.dgetrf(d.ATL, overwrite_a=1)
            if info > 0:
                raise np.linalg.LinAlgError(f"singular front (info={info})")
            d.ATL = lu
            d.piv = piv
        if fs and ss:
            d.ATR = _apply_piv(d.ATR, d.piv)
            d.ATR = fblas.dtrsm(1.0, d.ATL, d.ATR, side=0, lower=1, trans_a=0, diag=1, overwrite_b=1)
            d.ABL = fblas.dtrsm(1.0, d.ATL, d.ABL, side=1, lower=0, trans_a=0, diag=0, overwrite_b=1)
            d.ABR = fblas.dgemm(-1.0, d.ABL, d.ATR, beta=1.0, c=d.ABR, overwrite_c=1)
    elif method == LU_NOPIV:
        if fs:
            _lu_nopiv_inplace(d.ATL)
        if fs and ss:
            d.ATR = fblas.dtrsm(1.0, d.ATL, d.ATR, side=0, lower=1, trans_a=0, diag=1, overwrite_b=1)
            d.ABL = fblas.dtrsm(1.0, d.ATL, d.ABL, side=1, lower=0, trans_a=0, diag=0, overwrite_b=1)
            d.ABR = fblas.dgemm(-1.0, d.ABL, d.ATR, beta=1.0, c=d.ABR, overwrite_c=1)
    else:
        raise ValueError(method)


def _apply_piv(B, piv):
    """FLA_Apply_pivots(LEFT, NO_TRANSPOSE): sequential row interchanges
    (LINAL/src/dense/pivot.cxx:46-91), LAPACK ipiv convention (0-based here)."""
    B = np.asfortranarray(B)
    for i, p in enumerate(piv):
        if p != i:
            B[[i, p], :] = B[[p, i], :]
    return B


@dataclass
class Result:
    plan: Plan
    data: list
    x: np.ndarray            # canonical solution: node-id order, dofs contiguous
    timings: dict


def _zeros(m, n):
    return np.zeros((m, n), dtype=np.float64, order="F")


def solve_mesh(spec, method=CHOL, plan: Plan | None = None, timing: bool = False) -> Result:
    """Full pipeline of UHM/test/performance/uhmtest.cxx: lock, create matrices,
    copy_in element matrices and RHS, *_with_free, solve_*, gather x."""
    import time
    t0 = time.perf_counter()
    plan = plan or symbolic(spec)
    t1 = time.perf_counter()
    nrhs = spec.n_rhs
    data = []
    for f in plan.fronts:
        d = FrontData()
        d.ATL, d.ATR, d.ABL, d.ABR = _zeros(f.fs, f.fs), _zeros(f.fs, f.ss), _zeros(f.ss, f.fs), _zeros(f.ss, f.ss)
        d.piv = None
        d.bt, d.bb = _zeros(f.fs, nrhs), _zeros(f.ss, nrhs)
        data.append(d)
    # copy_in (LHS and RHS) for every leaf element
    emaps = {}
    for e in range(spec.n_leaves):
        part, pos = element_map(plan, spec, e)
        emaps[e] = (part, pos)
        d = data[e]
        _scatter_add((d.ATL, d.ATR, d.ABL, d.ABR), part, pos, spec.element_matrix(e))
        rhs = spec.element_rhs(e)
        t = part == 0
        d.bt[pos[t]] += rhs[t]
        d.bb[pos[~t]] += rhs[~t]
    cmaps = {}
    t2 = time.perf_counter()
    # factorisation leaf -> root (Scheduler_::execute_tree post-order;
    # op_decompose, UHM/src/operation/element.cxx:202-241)
    for e in plan.order_leaf2root:
        f = plan.fronts[e]
        d = data[e]
        for c in f.children:
            cm = child_map(plan, e, c)
            cmaps[c] = cm
            _scatter_add((d.ATL, d.ATR, d.ABL, d.ABR), cm[0], cm[1], data[c].ABR)
            data[c].ABR = None          # *_with_free: child ABR released
        factor_front(method, d, f.fs, f.ss)
    t3 = time.perf_counter()
    # forward solve leaf -> root (solve_*_1, e.g. chol/solve.cxx:152-168 + merge_rhs_x)
    for e in plan.order_leaf2root:
        f = plan.fronts[e]
        d = data[e]
        zt, zb = d.bt.copy(order="F"), d.bb.copy(order="F")
        for c in f.children:
            part, pos = cmaps[c]
            xb_c = data[c].xb
            t = part == 0
            zt[pos[t]] += xb_c[t]
            zb[pos[~t]] += xb_c[~t]
        if f.fs:
            if method == LU_PIV:
                zt = _apply_piv(zt, d.piv)
                zt = fblas.dtrsm(1.0, d.ATL, zt, side=0, lower=1, trans_a=0, diag=1, overwrite_b=1)
            elif method == LU_NOPIV:
                zt = fblas.dtrsm(1.0, d.ATL, zt, side=0, lower=1, trans_a=0, diag=1, overwrite_b=1)
            else:
                zt = fblas.dtrsm(1.0, d.ATL, zt, side=0, lower=1, trans_a=0, diag=0, overwrite_b=1)
        if f.fs and f.ss:
            zb = fblas.dgemm(-1.0, d.ABL, zt, beta=1.0, c=zb, overwrite_c=1)
        d.xt, d.xb = zt, zb
    # backward solve root -> leaf (solve_*_2 + branch_rhs_x, helper.hxx:302-331)
    for e in reversed(plan.order_leaf2root):
        f = plan.fronts[e]
        d = data[e]
        if f.parent >= 0 and f.ss:
            part, pos = cmaps[e]
            p = data[f.parent]
            xb = np.empty((f.ss, nrhs), order="F")
            t = part == 0
            xb[t] = p.xt[pos[t]]
            xb[~t] = p.xb[pos[~t]]
            d.xb = xb
        if f.fs and f.ss:
            if method == CHOL:
                d.xt = fblas.dgemm(-1.0, d.ABL, d.xb, beta=1.0, c=d.xt, trans_a=1, overwrite_c=1)
            else:
                d.xt = fblas.dgemm(-1.0, d.ATR, d.xb, beta=1.0, c=d.xt, overwrite_c=1)
        if f.fs:
            if method == CHOL:
                d.xt = fblas.dtrsm(1.0, d.ATL, d.xt, side=0, lower=1, trans_a=1, diag=0, overwrite_b=1)
            else:
                d.xt = fblas.dtrsm(1.0, d.ATL, d.xt, side=0, lower=0, trans_a=0, diag=0, overwrite_b=1)
    t4 = time.perf_counter()
    x = gather_solution(plan, data, nrhs)
    timings = dict(symbolic=t1 - t0, assemble=t2 - t1, factor=t3 - t2, solve=t4 - t3)
    return Result(plan, data, x, timings)


def node_dof_offsets(ndof):
    return np.concatenate([[0], np.cumsum(ndof)]).astype(np.int64)


def gather_solution(plan: Plan, data, nrhs):
    """Canonical solution vector: node-id order, each node's dofs contiguous."""
    off = node_dof_offsets(plan.node_ndof)
    x = np.zeros((int(off[-1]), nrhs))
    for nd in range(len(plan.node_ndof)):
        k = int(plan.node_ndof[nd])
        if not k:
            continue
        f = int(plan.owner_front[nd])
        o = int(plan.node_pos[nd])
        x[off[nd]:off[nd] + k] = data[f].xt[o:o + k]
    return x


def element_solution(spec, x, e):
    """Mesh_::copy_out(UHM_RHS) for leaf e: x in the element's dof order."""
    off = node_dof_offsets(spec.node_ndof)
    rows = []
    for nd in spec.element_nodes(e):
        nd = int(nd)
        rows.extend(range(off[nd], off[nd + 1]))
    return x[np.asarray(rows, dtype=np.int64)]


# ----------------------------------------------------------------------------
# Assembled operator (test-only cross-checks) and backward error
# ----------------------------------------------------------------------------
def element_dofs(spec, e):
    off = node_dof_offsets(spec.node_ndof)
    rows = []
    for nd in spec.element_nodes(e):
        nd = int(nd)
        rows.extend(range(off[nd], off[nd + 1]))
    return np.asarray(rows, dtype=np.int64)


def assemble(spec):
    """Global sparse A and b (the idea of DSparse_::import_element,
    UHM/src/interf/sparse.cxx:196-267), canonical dof order."""
    import scipy.sparse as sp
    n = spec.n_dof()
    I, J, V = [], [], []
    b = np.zeros((n, spec.n_rhs))
    for e in range(spec.n_leaves):
        dofs = element_dofs(spec, e)
        A = spec.element_matrix(e)
        I.append(np.repeat(dofs, len(dofs)))
        J.append(np.tile(dofs, len(dofs)))
        V.append(A.reshape(-1, order="C"))
        b[dofs] += spec.element_rhs(e)
    A = sp.csr_matrix((np.concatenate(V), (np.concatenate(I), np.concatenate(J))), shape=(n, n))
    A.sum_duplicates()
    return A, b


def backward_error(spec, x, A=None, b=None):
    """||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), A assembled."""
    if A is None:
        A, b = assemble(spec)
    r = b - A @ x
    anorm = abs(A).sum(axis=1).max()
    return float(np.abs(r).max() / (anorm * np.abs(x).max() + np.abs(b).max()))


def residual_unassembled(spec, x):
    """r = b - sum_e P_e^T A_e P_e x, element by element, canonical order."""
    r = np.zeros_like(x)
    for e in range(spec.n_leaves):
        dofs = element_dofs(spec, e)
        r[dofs] += spec.element_rhs(e) - spec.element_matrix(e) @ x[dofs]
    return r


def mesh_cost(plan: Plan, method=CHOL, n_rhs=1):
    """Mesh_::estimate_cost (UHM/src/mesh/matrix.cxx:210-239)."""
    dec = sol = 0.0
    for f in plan.fronts:
        a, b = front_cost(method, f.fs, f.ss, n_rhs)
        dec += a
        sol += b
    return dec, sol
