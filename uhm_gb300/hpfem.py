"""Seeded synthetic hp-FEM meshes for the UHM multifrontal path.

The reference library has no finite-element assembly of its own: its tests feed
random SPD element matrices (UHM/src/mesh/matrix.cxx:295-309,
UHM/test/performance/uhmtest.cxx:60-68).  The workloads this package is
measured on are Poisson / diffusion / convection-diffusion problems on uniform
quad and hex meshes, discretised with tensor-product integrated-Legendre
(Lobatto) shape functions of order p.  This module builds, for such a mesh:

* the UHM nodes (one per topological entity: vertex, edge, face, cell
  interior) with ``n_dof`` = number of hierarchic modes on that entity, and
  ``n_dof = 0`` for entities on the Dirichlet boundary (UHM skips zero-dof
  nodes, UHM/src/mesh/element.cxx:302 and UHM/src/mesh/interf.cxx:139);
* the leaf elements with their node lists;
* a geometric nested-dissection tree (2^d-ary merges, or the per-level merge
  factors given) whose generations follow Element_::update_generation
  (UHM/src/mesh/element.cxx:63-72): leaves 0, parent = min(children) - 1;
* FP64 element matrices by Gauss quadrature with p_max+1 points per direction
  (exact for these polynomial integrands), and element right-hand sides.

Everything is deterministic in ``seed`` (numpy PCG64).

Conventions
-----------
Element (i, j[, k]) covers [i h, (i+1) h] x ...; elements are numbered
lexicographically, x fastest.  All edges and faces carry the global axis
orientation, so odd Lobatto modes match between neighbours without sign flips.
Within an entity the bubble modes are ordered lexicographically, lowest axis
fastest.  Variable order uses the minimum rule: an edge/face takes the minimum
order of the elements sharing it.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = ["MeshSpec", "poisson2d", "poisson3d", "convdiff3d", "diffusion3d",
           "build_mesh", "lobatto_1d", "forest", "batch3d", "element_recipe"]


# ----------------------------------------------------------------------------
# 1D integrated-Legendre basis and reference matrices
# ----------------------------------------------------------------------------
def _legendre(k: int, x: np.ndarray) -> np.ndarray:
    c = np.zeros(k + 1)
    c[k] = 1.0
    return np.polynomial.legendre.legval(x, c)


def lobatto_1d(p: int, nq: int | None = None):
    """Reference 1D matrices on [-1, 1] for modes 0..p.

    Mode 0 = (1-x)/2, mode 1 = (1+x)/2, mode k>=2 = (P_k - P_{k-2})/sqrt(2(2k-1)).
    Returns (M, K, C) with M_ij = int phi_i phi_j, K_ij = int phi_i' phi_j',
    C_ij = int phi_i phi_j' (test i, trial j), all by nq-point Gauss quadrature.
    """
    nq = nq or (p + 1)
    xq, wq = np.polynomial.legendre.leggauss(nq)
    phi = np.zeros((p + 1, nq))
    dphi = np.zeros((p + 1, nq))
    phi[0] = 0.5 * (1 - xq)
    phi[1] = 0.5 * (1 + xq)
    dphi[0] = -0.5
    dphi[1] = 0.5
    for k in range(2, p + 1):
        phi[k] = (_legendre(k, xq) - _legendre(k - 2, xq)) / math.sqrt(2.0 * (2 * k - 1))
        dphi[k] = math.sqrt((2 * k - 1) / 2.0) * _legendre(k - 1, xq)
    M = (phi * wq) @ phi.T
    K = (dphi * wq) @ dphi.T
    C = (phi * wq) @ dphi.T
    return M, K, C


# ----------------------------------------------------------------------------
# Mesh container
# ----------------------------------------------------------------------------
@dataclass
class MeshSpec:
    """A mesh ready to be fed through the UHM Mesh_ API.

    Node ids are (id, phy=0).  ``elem_ptr/elem_node`` list, for each leaf
    element e, its node ids in the order used for its element matrix (dofs of
    a node contiguous; zero-dof nodes contribute no rows).  Elements
    0..n_leaves-1 are the leaves; the tree arrays cover all elements in the
    order they are added through ``add_element(gen)``.
    """

    dim: int
    node_id: np.ndarray
    node_ndof: np.ndarray
    node_p: np.ndarray
    node_kind: np.ndarray
    elem_ptr: np.ndarray
    elem_node: np.ndarray
    n_leaves: int
    parent: np.ndarray            # per element, -1 for the root
    generation: np.ndarray        # per element
    child_ptr: np.ndarray         # CSR of children, in add_child order
    child_idx: np.ndarray
    elem_m: np.ndarray            # rows of each leaf element matrix
    mat_off: np.ndarray           # offset of each m*m block (column-major)
    mats: np.ndarray              # flat float64
    n_rhs: int
    rhs_off: np.ndarray           # offset of each m*n_rhs block (column-major)
    rhs: np.ndarray               # flat float64
    symmetric: bool
    info: dict = field(default_factory=dict)

    @property
    def n_elements(self) -> int:
        return len(self.parent)

    @property
    def n_nodes(self) -> int:
        return len(self.node_id)

    def element_nodes(self, e: int) -> np.ndarray:
        return self.elem_node[self.elem_ptr[e]:self.elem_ptr[e + 1]]

    def element_matrix(self, e: int) -> np.ndarray:
        m = int(self.elem_m[e])
        o = int(self.mat_off[e])
        return self.mats[o:o + m * m].reshape(m, m, order="F")

    def element_rhs(self, e: int) -> np.ndarray:
        m = int(self.elem_m[e])
        o = int(self.rhs_off[e])
        return self.rhs[o:o + m * self.n_rhs].reshape(m, self.n_rhs, order="F")

    def children(self, e: int) -> np.ndarray:
        return self.child_idx[self.child_ptr[e]:self.child_ptr[e + 1]]

    def n_dof(self) -> int:
        return int(self.node_ndof.sum())


# ----------------------------------------------------------------------------
# Structured-grid topology
# ----------------------------------------------------------------------------
def _entities(dim: int, n: tuple):
    """Enumerate topological entities of an n[0] x ... grid.

    Returns a dict mapping (bubble_axes tuple, grid coordinate tuple) -> node id
    generator function, plus arrays describing each node.  Entities are
    numbered block by block: vertices, then edges by axis, faces by normal
    axis, then cell interiors, each block lexicographic with x fastest.
    """
    import itertools

    blocks = []
    axes = list(range(dim))
    for nb in range(dim + 1):
        for bub in itertools.combinations(axes, nb):
            shape = tuple(n[a] if a in bub else n[a] + 1 for a in axes)
            blocks.append((bub, shape))
    base = {}
    off = 0
    for bub, shape in blocks:
        base[bub] = (off, shape)
        off += int(np.prod(shape))
    return base, off


def _entity_id(base, bub, coord):
    off, shape = base[bub]
    idx = 0
    stride = 1
    for a in range(len(shape)):
        idx += coord[a] * stride
        stride *= shape[a]
    return off + idx


def _merge_plan(n: int, merges):
    """Per-level merge factors reducing n cells to 1 along one axis.

    When n factors into 2, 3 and 5 the plan is exact (smallest factors
    first, 2s at the leaves).  Otherwise (a prime factor above 5, e.g. n = 11
    or 14) exact merges would put a 7-, 11- or 13-way merge, and with it one
    huge separator, at a single level; the plan then halves the cell count
    with ceiling division at every level (nested dissection with a ragged
    last block: 11 -> 6 -> 3 -> 2 -> 1), which build_mesh supports."""
    if merges is not None:
        assert int(np.prod(merges)) == n, (n, merges)
        return list(merges)
    plan = []
    m = n
    while m > 1:
        if m % 2 == 0:
            plan.append(2)
            m //= 2
        else:
            # smallest odd prime factor
            f = 3
            while m % f:
                f += 2
            if f > 5:
                return [2] * int(math.ceil(math.log2(n)))
            plan.append(f)
            m //= f
    return plan


def build_mesh(dim: int, n: int, p, *, kappa=None, beta=None, react=None, seed: int = 0,
               n_rhs: int = 1, merges=None, h: float | None = None) -> MeshSpec:
    """Build a uniform quad (dim=2) or hex (dim=3) mesh of n^dim elements.

    p      : int, or an integer array of per-element orders (minimum rule)
    kappa  : None (1.0) or per-element diffusion coefficients
    beta   : None or a length-dim convection velocity (nonsymmetric matrices)
    react  : None or per-element reaction coefficients c (adds c * mass; a
             negative c shifts the operator towards its first eigenvalue)
    merges : per-level merge factors of the nested-dissection tree (product n);
             default: factors of 2 first, then odd primes.
    """
    import itertools

    rng = np.random.default_rng(seed)
    h = h if h is not None else 1.0 / n
    nn = (n,) * dim
    n_el = n ** dim
    p_el = np.broadcast_to(np.asarray(p, dtype=np.int64), (n_el,)).copy()
    assert p_el.min() >= 1
    kap = np.ones(n_el) if kappa is None else np.asarray(kappa, dtype=np.float64)
    rea = None if react is None else np.broadcast_to(np.asarray(react, dtype=np.float64), (n_el,))
    symmetric = beta is None

    base, n_nodes = _entities(dim, nn)
    # entity order = min over the elements touching it
    ent_p = np.full(n_nodes, 1 << 30, dtype=np.int64)
    ent_bub = [None] * n_nodes
    ent_coord = [None] * n_nodes

    el_coords = list(itertools.product(*[range(n)] * dim))
    el_coords = [tuple(reversed(c)) for c in el_coords]  # x fastest
    # local entity list per element: (bubble axes, vertex offsets)
    local_ents = []
    for nb in range(dim + 1):
        for bub in itertools.combinations(range(dim), nb):
            others = [a for a in range(dim) if a not in bub]
            for offs in itertools.product(*[(0, 1)] * len(others)):
                offs = tuple(reversed(offs))
                local_ents.append((bub, dict(zip(others, offs))))
    el_nodes = np.zeros((n_el, len(local_ents)), dtype=np.int64)
    for e, c in enumerate(el_coords):
        for li, (bub, vo) in enumerate(local_ents):
            g = tuple(c[a] + vo.get(a, 0) for a in range(dim))
            nid = _entity_id(base, bub, g)
            el_nodes[e, li] = nid
            ent_p[nid] = min(ent_p[nid], p_el[e])
            ent_bub[nid] = bub
            ent_coord[nid] = g
    # dofs per entity, Dirichlet on the whole boundary
    node_ndof = np.zeros(n_nodes, dtype=np.int64)
    node_p = np.zeros(n_nodes, dtype=np.int64)
    for nid in range(n_nodes):
        bub, g = ent_bub[nid], ent_coord[nid]
        pe = int(ent_p[nid])
        node_p[nid] = pe
        on_bnd = any((a not in bub) and (g[a] == 0 or g[a] == n) for a in range(dim))
        node_ndof[nid] = 0 if on_bnd else (pe - 1) ** len(bub)

    # element matrices: local tensor modes -> retained modes in node order
    cache = {}
    elem_m = np.zeros(n_el, dtype=np.int64)
    mats_list = []
    sel_list = []
    for e in range(n_el):
        pe = int(p_el[e])
        sel = []
        for li, (bub, vo) in enumerate(local_ents):
            nid = el_nodes[e, li]
            if node_ndof[nid] == 0:
                continue
            pn = int(node_p[nid])
            # bubble modes 2..pn along bub axes, lowest axis fastest
            ranges = [range(2, pn + 1)] * len(bub)
            for modes in itertools.product(*ranges):
                modes = tuple(reversed(modes))
                mi = [0] * dim
                for a in range(dim):
                    mi[a] = vo[a] if a not in bub else modes[bub.index(a)]
                flat = 0
                stride = 1
                for a in range(dim):
                    flat += mi[a] * stride
                    stride *= (pe + 1)
                sel.append(flat)
        sel = np.asarray(sel, dtype=np.int64)
        elem_m[e] = len(sel)
        sel_list.append(sel)

    def ref_mats(pe):
        key = pe
        if key not in cache:
            M, K, C = lobatto_1d(pe, pe + 1)
            if dim == 2:
                diff = np.kron(M, K) + np.kron(K, M)
                mass = (h / 2) ** 2 * np.kron(M, M)
                conv = []
                if beta is not None:
                    conv = [(h / 2) * np.kron(M, C), (h / 2) * np.kron(C, M)]
            else:
                diff = (h / 2) * (np.kron(M, np.kron(M, K)) + np.kron(M, np.kron(K, M))
                                  + np.kron(K, np.kron(M, M)))
                mass = (h / 2) ** 3 * np.kron(M, np.kron(M, M))
                conv = []
                if beta is not None:
                    s = (h / 2) ** 2
                    conv = [s * np.kron(M, np.kron(M, C)), s * np.kron(M, np.kron(C, M)),
                            s * np.kron(C, np.kron(M, M))]
            cache[key] = (diff, conv, mass)
        return cache[key]

    mat_off = np.zeros(n_el, dtype=np.int64)
    off = 0
    for e in range(n_el):
        mat_off[e] = off
        off += int(elem_m[e]) ** 2
    mats = np.empty(off, dtype=np.float64)
    for e in range(n_el):
        diff, conv, mass = ref_mats(int(p_el[e]))
        sel = sel_list[e]
        A = kap[e] * diff[np.ix_(sel, sel)]
        if rea is not None and rea[e] != 0.0:
            A = A + rea[e] * mass[np.ix_(sel, sel)]
        if beta is not None:
            for a in range(dim):
                A = A + beta[a] * conv[a][np.ix_(sel, sel)]
        m = int(elem_m[e])
        mats[mat_off[e]:mat_off[e] + m * m] = A.reshape(-1, order="F")

    # right-hand side: i.i.d. N(0,1) per global dof, placed in the element of
    # lowest index containing the node (assembled RHS = the random vector)
    gb = rng.standard_normal((int(node_ndof.sum()), n_rhs))
    node_first = np.full(n_nodes, -1, dtype=np.int64)
    node_dof0 = np.concatenate([[0], np.cumsum(node_ndof)])[:-1]
    rhs_off = np.zeros(n_el, dtype=np.int64)
    off = 0
    for e in range(n_el):
        rhs_off[e] = off
        off += int(elem_m[e]) * n_rhs
    rhs = np.zeros(off, dtype=np.float64)
    for e in range(n_el):
        r = 0
        blk = np.zeros((int(elem_m[e]), n_rhs))
        for nid in el_nodes[e]:
            nd = int(node_ndof[nid])
            if nd == 0:
                continue
            if node_first[nid] < 0:
                node_first[nid] = e
                blk[r:r + nd] = gb[node_dof0[nid]:node_dof0[nid] + nd]
            r += nd
        rhs[rhs_off[e]:rhs_off[e] + blk.size] = blk.reshape(-1, order="F")

    # nested-dissection tree through add_element(gen)
    plan = _merge_plan(n, merges)
    parent = [-1] * n_el
    generation = [0] * n_el
    children = [[] for _ in range(n_el)]
    # current level: dict block coord -> element index
    cur = {c: e for e, c in enumerate(el_coords)}
    cur_n = n
    for f in plan:
        nxt_n = -(-cur_n // f)         # the last block of a ragged halving is smaller
        blocks = list(itertools.product(*[range(nxt_n)] * dim))
        blocks = [tuple(reversed(b)) for b in blocks]
        nxt = {}
        for b in blocks:
            kids = []
            for sub in itertools.product(*[range(f)] * dim):
                sub = tuple(reversed(sub))
                cc = tuple(b[a] * f + sub[a] for a in range(dim))
                if all(x < cur_n for x in cc):
                    kids.append(cur[cc])
            pid = len(parent)
            parent.append(-1)
            generation.append(min(generation[k] for k in kids) - 1)
            children.append(list(kids))
            for k in kids:
                parent[k] = pid
            nxt[b] = pid
        cur = nxt
        cur_n = nxt_n
    child_ptr = np.zeros(len(parent) + 1, dtype=np.int64)
    for e in range(len(parent)):
        child_ptr[e + 1] = child_ptr[e] + len(children[e])
    child_idx = np.asarray([k for ch in children for k in ch], dtype=np.int64)

    elem_ptr = np.arange(0, (n_el + 1) * len(local_ents), len(local_ents), dtype=np.int64)
    return MeshSpec(
        dim=dim,
        node_id=np.arange(n_nodes, dtype=np.int64),
        node_ndof=node_ndof,
        node_p=node_p,
        node_kind=np.zeros(n_nodes, dtype=np.int64),
        elem_ptr=elem_ptr,
        elem_node=el_nodes.reshape(-1),
        n_leaves=n_el,
        parent=np.asarray(parent, dtype=np.int64),
        generation=np.asarray(generation, dtype=np.int64),
        child_ptr=child_ptr,
        child_idx=child_idx,
        elem_m=elem_m,
        mat_off=mat_off,
        mats=mats,
        n_rhs=n_rhs,
        rhs_off=rhs_off,
        rhs=rhs,
        symmetric=symmetric,
        info=dict(dim=dim, n=n, p=(int(p_el[0]) if np.all(p_el == p_el[0]) else "var"),
                  merges=plan, seed=seed, n_rhs=n_rhs, h=h,
                  # what a device-side generator needs to rebuild the element
                  # matrices (element_recipe): per element its order,
                  # coefficients and retained tensor modes
                  recipe=dict(p_el=p_el, kappa=kap, react=rea, beta=beta,
                              sel_ptr=np.concatenate([[0], np.cumsum([len(v) for v in sel_list])]).astype(np.int64),
                              sel=(np.concatenate(sel_list).astype(np.int32) if sel_list
                                   else np.zeros(0, np.int32)))),
    )


# ----------------------------------------------------------------------------
# Named workloads
# ----------------------------------------------------------------------------
def poisson2d(n: int = 16, p: int = 4, seed: int = 0, n_rhs: int = 1) -> MeshSpec:
    """-Laplace(u) = f on the unit square, n x n quads, order p, Dirichlet u=0."""
    return build_mesh(2, n, p, seed=seed, n_rhs=n_rhs)


def poisson3d(n: int = 16, p: int = 4, seed: int = 0, n_rhs: int = 1,
              merges=None) -> MeshSpec:
    """-Laplace(u) = f on the unit cube, n^3 hexes, order p, Dirichlet u=0."""
    return build_mesh(3, n, p, seed=seed, n_rhs=n_rhs, merges=merges)


def diffusion3d(n: int, p, seed: int = 0, contrast: float = 1e4, n_rhs: int = 1,
                sigma: float = 2.0, merges=None) -> MeshSpec:
    """-div(kappa grad u) = f, kappa lognormal per element, log-clipped so that
    max/min kappa <= contrast."""
    rng = np.random.default_rng(seed + 7919)
    lk = sigma * rng.standard_normal(n ** 3)
    c = 0.5 * math.log(contrast)
    kappa = np.exp(np.clip(lk, -c, c))
    return build_mesh(3, n, p, kappa=kappa, seed=seed, n_rhs=n_rhs, merges=merges)


def convdiff3d(n: int = 24, p: int = 3, seed: int = 0, pe: float = 100.0,
               contrast: float = 1e4, sigma: float = 2.0, n_rhs: int = 1,
               merges=None) -> MeshSpec:
    """-div(kappa grad u) + beta.grad u = f, beta = (1, .5, .25) * Pe."""
    rng = np.random.default_rng(seed + 7919)
    lk = sigma * rng.standard_normal(n ** 3)
    c = 0.5 * math.log(contrast)
    kappa = np.exp(np.clip(lk, -c, c))
    beta = np.array([1.0, 0.5, 0.25]) * pe
    return build_mesh(3, n, p, kappa=kappa, beta=beta, seed=seed, n_rhs=n_rhs,
                      merges=merges)


# ----------------------------------------------------------------------------
# Many independent meshes as one forest
# ----------------------------------------------------------------------------
def forest(specs) -> MeshSpec:
    """Join independent meshes into one MeshSpec whose tree is a forest.

    The reference's Mesh_ holds any set of elements: ``lock`` groups them by
    generation over the whole mesh (UHM/src/operation/scheduler.cxx:45-70) and
    every element without a parent is a root whose nodes are all factored
    (UHM/src/mesh/element.cxx:272-286), so a mesh made of several disjoint
    trees factors and solves each tree independently.  Same-generation fronts
    of all meshes then fall into the same level and share each launch.

    Node ids of mesh k are shifted past those of meshes 0..k-1; the leaves of
    all meshes come first (mesh by mesh), then the interior elements.  Every
    spec must have the same ``n_rhs`` and symmetry.  ``info["parts"]`` lists,
    per mesh, its node-id offset, number of nodes, leaf range and dofs.
    """
    specs = list(specs)
    if not specs:
        raise ValueError("forest: no meshes")
    n_rhs = specs[0].n_rhs
    sym = specs[0].symmetric
    if any(s.n_rhs != n_rhs or s.symmetric != sym for s in specs):
        raise ValueError("forest: meshes differ in n_rhs or symmetry")
    leaf_base, int_base = [], []
    nl = sum(s.n_leaves for s in specs)
    lo, io = 0, nl
    for s in specs:
        leaf_base.append(lo)
        int_base.append(io)
        lo += s.n_leaves
        io += s.n_elements - s.n_leaves

    def remap(k, e):
        s = specs[k]
        e = np.asarray(e, dtype=np.int64)
        return np.where(e < s.n_leaves, leaf_base[k] + e, int_base[k] + (e - s.n_leaves))

    n_el = io
    parent = np.full(n_el, -1, dtype=np.int64)
    generation = np.zeros(n_el, dtype=np.int64)
    children = [None] * n_el
    node_id, node_ndof, node_p, node_kind = [], [], [], []
    elem_node, elem_m, mats, rhs = [], [], [], []
    parts = []
    nid_off = 0
    for k, s in enumerate(specs):
        idx = remap(k, np.arange(s.n_elements))
        par = s.parent
        parent[idx] = np.where(par < 0, -1, remap(k, np.maximum(par, 0)))
        generation[idx] = s.generation
        for e in range(s.n_elements):
            children[idx[e]] = remap(k, s.children(e))
        node_id.append(s.node_id + nid_off)
        node_ndof.append(s.node_ndof)
        node_p.append(s.node_p)
        node_kind.append(s.node_kind)
        elem_node.append(s.elem_node + nid_off)
        elem_m.append(s.elem_m)
        mats.append(s.mats)
        rhs.append(s.rhs)
        parts.append(dict(node_off=nid_off, n_nodes=s.n_nodes, leaves=(leaf_base[k],
                          leaf_base[k] + s.n_leaves), n_dof=s.n_dof(), info=s.info))
        nid_off += int(s.node_id.max()) + 1
    child_ptr = np.zeros(n_el + 1, dtype=np.int64)
    for e in range(n_el):
        child_ptr[e + 1] = child_ptr[e] + len(children[e])
    child_idx = (np.concatenate([c for c in children if len(c)]).astype(np.int64)
                 if child_ptr[-1] else np.zeros(0, dtype=np.int64))
    elem_m = np.concatenate(elem_m)
    sizes = elem_m.astype(np.int64)
    mat_off = np.concatenate([[0], np.cumsum(sizes * sizes)[:-1]]).astype(np.int64)
    rhs_off = np.concatenate([[0], np.cumsum(sizes * n_rhs)[:-1]]).astype(np.int64)
    lens = np.concatenate([np.diff(s.elem_ptr) for s in specs])
    elem_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return MeshSpec(
        dim=specs[0].dim,
        node_id=np.concatenate(node_id).astype(np.int64),
        node_ndof=np.concatenate(node_ndof),
        node_p=np.concatenate(node_p),
        node_kind=np.concatenate(node_kind),
        elem_ptr=elem_ptr,
        elem_node=np.concatenate(elem_node).astype(np.int64),
        n_leaves=nl,
        parent=parent,
        generation=generation,
        child_ptr=child_ptr,
        child_idx=child_idx,
        elem_m=elem_m,
        mat_off=mat_off,
        mats=np.concatenate(mats),
        n_rhs=n_rhs,
        rhs_off=rhs_off,
        rhs=np.concatenate(rhs),
        symmetric=sym,
        info=dict(forest=len(specs), parts=parts, n_rhs=n_rhs),
    )


def batch3d(n_meshes: int, seed: int = 0, n_range=(8, 20), p_range=(2, 6), n_rhs: int = 16):
    """The batched workload: independent 3D Poisson meshes with n uniform in
    ``n_range`` (hexes per side) and p uniform in ``p_range``, ``n_rhs``
    i.i.d. N(0,1) right-hand sides each, all drawn from ``seed``.  Returns
    the list of specs (join them with :func:`forest`)."""
    rng = np.random.default_rng(seed + 104729)
    out = []
    for k in range(n_meshes):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        p = int(rng.integers(p_range[0], p_range[1] + 1))
        out.append(poisson3d(n, p, seed=seed * 100003 + k, n_rhs=n_rhs))
    return out


def element_recipe(spec: MeshSpec) -> dict:
    """Inputs of the device-side element-matrix generator
    (uhm_gpu_generate_lobatto_elements) for a mesh from build_mesh: the
    1D Lobatto matrices (M, K, C) of every order in use, stored back to back
    with per-order offsets, and per element its order, coefficients and
    retained tensor modes (flat index mi[0] + mi[1] (p+1) + mi[2] (p+1)^2)
    in the element's row order.  The generator combines them exactly as
    build_mesh does (same products and sums in the same order, no fused
    multiply-add), so the matrices come out bit-identical."""
    r = spec.info.get("recipe")
    if r is None:
        raise ValueError("element_recipe: the mesh was not built by build_mesh")
    dim, h = spec.dim, spec.info["h"]
    pmax = int(r["p_el"].max())
    ref_off = np.zeros(pmax + 2, np.int64)
    parts = []
    for p in range(1, pmax + 1):
        M, K, C = lobatto_1d(p, p + 1)
        ref_off[p] = sum(x.size for x in parts)
        parts += [M.ravel(order="C"), K.ravel(order="C"), C.ravel(order="C")]
    ref = np.concatenate(parts)
    n_el = spec.n_leaves
    react = r["react"]
    beta = r["beta"]
    # scale factors exactly as build_mesh forms them
    hh = h / 2
    cmass = (h / 2) ** 3 if dim == 3 else (h / 2) ** 2
    cconv = (h / 2) ** 2 if dim == 3 else (h / 2)
    return dict(dim=dim, h=float(h), hh=float(hh), cmass=float(cmass), cconv=float(cconv),
                n_el=n_el, ref=ref, ref_off=ref_off,
                p_el=np.ascontiguousarray(r["p_el"], np.int32),
                kappa=np.ascontiguousarray(r["kappa"], np.float64),
                react=None if react is None else np.ascontiguousarray(react, np.float64),
                beta=None if beta is None else np.ascontiguousarray(beta, np.float64),
                sel_ptr=np.ascontiguousarray(r["sel_ptr"], np.int64),
                sel=np.ascontiguousarray(r["sel"], np.int32))
