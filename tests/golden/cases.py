"""Golden cases: seeded meshes solved by the reference's own C++ solver.

Each case is (name, generator, keyword arguments, method).  The generator is a
function of ``uhm_gb300.hpfem``; ``make_golden.py`` runs the reference solver
(built by ``oracle/Makefile``) on the mesh and stores its solution, its front
sizes and its LAWN-41 flop estimates in ``<name>.npz`` beside a digest of the
mesh's inputs, so a change of the generator is caught instead of compared.
Methods: 1 Cholesky, 2 LU without pivoting, 3 LU with partial pivoting, 4 LU
with incremental pivoting (UHM/include/uhm/const.hxx:76; solved by
solve_lu_piv, as the reference's Fortran flow does).
"""
import hashlib

import numpy as np

from uhm_gb300 import hpfem

CHOL, LU_NOPIV, LU_PIV, LU_INCPIV = 1, 2, 3, 4

CASES = [
    ("2d_4x4_p2", "poisson2d", dict(n=4, p=2, seed=1), CHOL),
    ("2d_4x4_p1", "poisson2d", dict(n=4, p=1, seed=2), CHOL),
    ("2d_2x2_p2_lupiv", "poisson2d", dict(n=2, p=2, seed=3), LU_PIV),
    ("2d_16x16_p4", "poisson2d", dict(n=16, p=4, seed=2), CHOL),
    ("3d_1_p3_single_element", "poisson3d", dict(n=1, p=3, seed=1), CHOL),
    ("3d_4_p3", "poisson3d", dict(n=4, p=3, seed=3), CHOL),
    ("3d_4_p3_lunopiv", "poisson3d", dict(n=4, p=3, seed=3), LU_NOPIV),
    ("3d_4_p3_lupiv", "poisson3d", dict(n=4, p=3, seed=3), LU_PIV),
    ("3d_6_p2_merge32", "poisson3d", dict(n=6, p=2, seed=5, merges=[3, 2]), CHOL),
    ("3d_4_p3_rhs4", "poisson3d", dict(n=4, p=3, seed=9, n_rhs=4), CHOL),
    ("diff_4_p3_contrast", "diffusion3d", dict(n=4, p=3, seed=4), CHOL),
    ("cd_4_p3_lupiv", "convdiff3d", dict(n=4, p=3, seed=6), LU_PIV),
    ("cd_6_p3_lupiv_merge32", "convdiff3d", dict(n=6, p=3, seed=7, merges=[3, 2]), LU_PIV),
    ("cd_4_p2_lunopiv", "convdiff3d", dict(n=4, p=2, seed=8, pe=1.0), LU_NOPIV),
    ("cd_4_p3_lu_incpiv", "convdiff3d", dict(n=4, p=3, seed=12), LU_INCPIV),
    ("varp_4_3d", "build_mesh", dict(dim=3, n=4, p=[int(v) for v in np.random.default_rng(3).integers(2, 6, 64)],
                                     seed=10), CHOL),
]

# meshes whose assembled operator the reference exports (DSparse_::triplet);
# stored as sparse_<name>.npz
SPARSE_CASES = [
    ("2d_4x4_p2_rhs2", "poisson2d", dict(n=4, p=2, seed=21, n_rhs=2)),
    ("cd_3_p2", "convdiff3d", dict(n=3, p=2, seed=22)),
    ("varp_3_3d", "build_mesh", dict(dim=3, n=3, p=[int(v) for v in np.random.default_rng(23).integers(1, 5, 27)],
                                     seed=23)),
]


def make_spec(gen, kwargs):
    kw = dict(kwargs)
    if gen == "build_mesh":
        kw["p"] = np.asarray(kw["p"], dtype=np.int64)
        return hpfem.build_mesh(kw.pop("dim"), kw.pop("n"), kw.pop("p"), **kw)
    return getattr(hpfem, gen)(**kw)


def spec_digest(spec) -> str:
    """sha256 over every input the solver sees (topology, tree, matrices, rhs)."""
    h = hashlib.sha256()
    for a in (spec.node_id, spec.node_ndof, spec.node_p, spec.node_kind, spec.elem_ptr, spec.elem_node,
              spec.generation, spec.child_ptr, spec.child_idx):
        h.update(np.ascontiguousarray(a, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(spec.mats, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(spec.rhs, dtype=np.float64).tobytes())
    return h.hexdigest()
