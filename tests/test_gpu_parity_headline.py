"""Parity at the full sizes of the benchmark workloads.

- 3D Poisson 16^3 hex p=4, Cholesky fronts (the benchmark mesh, 250,047
  dofs, root front 11,719): the plain FP64 device path against the oracle
  within 1e-10 relative (max norm), and the mixed path (BF16-split / FP32
  fronts, FP64 refinement to backward error 1e-12) within 1e-8.
- 3D convection-diffusion 24^3 hex p=3, LU with partial pivoting inside the
  eliminated block, nested-dissection merges 3, 2, 2, 2 (357,911 dofs, root
  front 14,911): the plain FP64 device
  path against the reference's own solver built from its sources when it
  builds on this machine (oracle/Makefile), else against the oracle, within
  1e-10.

The reference's corresponding flow is Mesh_::chol_with_free + solve_chol
(UHM/src/mesh/chol.cxx:49-98) and lu_piv_with_free + solve_lu_piv."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

REL_TOL_FP64 = 1e-10
REL_TOL_MIXED = 1e-8


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _rel(x, ref):
    return float(np.abs(x - ref).max() / np.abs(ref).max())


def test_poisson3d_16_p4_matches_oracle(native_lib):
    spec = hpfem.poisson3d(16, 4, seed=0)
    assert spec.n_dof() == 250047
    ref = uo.solve_mesh(spec, uo.CHOL)
    m = api.load_spec(spec)
    _, _, fs, ss = m.fronts()
    assert int((fs + ss).max()) == 11719
    m.set_mode(0)
    m.chol_with_free()
    m.solve_chol()
    rel64 = _rel(_x(m, spec), ref.x)
    assert rel64 < REL_TOL_FP64, rel64
    assert m.backward_error() < 1e-15
    for prec in (api.PREC_BF16X3, api.PREC_FP32):
        m.set_mode(1, prec, 1e-12, 10)
        m.chol_with_free()
        m.solve_chol()
        assert m.status() == 0, m.last_error()
        t = m.timing()
        assert t["berr"] <= 1e-12
        relm = _rel(_x(m, spec), ref.x)
        assert relm < REL_TOL_MIXED, (prec, relm)


def test_convdiff3d_24_p3_lupiv_matches_reference(native_lib):
    spec = hpfem.convdiff3d(24, 3, seed=0, merges=[3, 2, 2, 2])
    assert spec.n_dof() == 357911
    ref_x = None
    try:
        import os
        from oracle import ref_runner
        if ref_runner.build(jobs=os.cpu_count() or 8):
            ref_x = ref_runner.run(spec, uo.LU_PIV, threads=os.cpu_count() or 8).x
    except Exception:
        ref_x = None
    if ref_x is None:
        ref_x = uo.solve_mesh(spec, uo.LU_PIV).x
    m = api.load_spec(spec)
    m.set_mode(0)
    m.lu_piv_with_free()
    m.solve_lu_piv()
    rel64 = _rel(_x(m, spec), ref_x)
    assert rel64 < REL_TOL_FP64, rel64
    m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
    m.lu_piv_with_free()
    m.solve_lu_piv()
    assert m.status() == 0, m.last_error()
    assert m.timing()["berr"] <= 1e-12
    assert _rel(_x(m, spec), ref_x) < REL_TOL_MIXED
