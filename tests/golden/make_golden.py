"""Regenerates the golden fixtures in this folder from the reference solver.

    make -C oracle REF=<reference checkout>    # builds oracle/_ref/<machine>/uhm_ref_driver
    python tests/golden/make_golden.py

For every case in ``cases.py`` the mesh is generated, solved by the
reference's own C++ sources (UHM + LINAL compiled against the FLAME-subset
shim in ``oracle/flame_shim``, numerics by OpenBLAS) and stored as
``<name>.npz``: the solution ``x`` (node order, dofs of a node contiguous,
one column per right-hand side), per-element ``fronts`` (factor dofs, schur
dofs), ``flops`` (decompose, solve) from Mesh_::estimate_cost and the input
``digest``.  For every case in ``SPARSE_CASES`` the reference's own sparse
export (DSparse_::import_element + triplet) is stored as
``sparse_<name>.npz``: the triplets, the right-hand sides, the reference's
first global dof of every node and the input ``digest``.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from cases import CASES, SPARSE_CASES, make_spec, spec_digest  # noqa: E402
from oracle import ref_runner  # noqa: E402


def main():
    if not ref_runner.available():
        ref_runner.build()
    for name, gen, kw, method in CASES:
        spec = make_spec(gen, kw)
        r = ref_runner.run(spec, method)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), x=r.x, fronts=r.fronts.astype(np.int32),
                            flops=np.array([r.flop_decompose, r.flop_solve]), method=np.int32(method),
                            digest=np.array(spec_digest(spec)))
        print(f"{name:28s} n_dof={spec.n_dof():6d} fronts={spec.n_elements:5d} method={method}")
    for name, gen, kw in SPARSE_CASES:
        spec = make_spec(gen, kw)
        r = ref_runner.run_sparse(spec)
        np.savez_compressed(os.path.join(HERE, "sparse_" + name + ".npz"), offsets=r["offsets"],
                            n_dof=np.int32(r["n_dof"]), n_rhs=np.int32(r["n_rhs"]), ia=r["ia"], ja=r["ja"],
                            a=r["a"], b=r["b"], digest=np.array(spec_digest(spec)))
        print(f"sparse_{name:21s} n_dof={spec.n_dof():6d} nnz={len(r['a']):7d}")


if __name__ == "__main__":
    main()
