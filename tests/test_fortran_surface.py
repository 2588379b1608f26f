"""The rest of the reference's Fortran/C interface (UHM/include/uhm/wrapper/
fort.hxx), no GPU: every entry point it declares is exported; QR and SVD
fronts record status 30; the SVD thresholds are kept; the random fills give
solvable systems of the mesh's shape (symmetric positive definite for
random_spd_matrix); lu_incpiv is accepted (its numbers are checked on the GPU
against the reference's own incremental-pivoting solution,
tests/golden/cd_4_p3_lu_incpiv.npz)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from uhm_gb300 import api, hpfem

# the reference header, read from the checkout ($UHM_REFERENCE) or from the
# staged copy of its sources (oracle/_ref/src) when either is present
_REL = os.path.join("UHM", "include", "uhm", "wrapper", "fort.hxx")
_ROOTS = [os.environ.get("UHM_REFERENCE", ""),
          os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "src")]
FORT = next((os.path.join(r, _REL) for r in _ROOTS if r and os.path.exists(os.path.join(r, _REL))),
            os.path.join("/root/reference", _REL))


@pytest.mark.skipif(not os.path.exists(FORT), reason="reference checkout absent")
def test_every_reference_entry_point_is_exported(native_lib):
    names = re.findall(r"UHM_C2F\((\w+)\)", open(FORT).read())
    assert len(names) == 60
    missing = [n for n in names if not hasattr(native_lib, n + "_")]
    assert not missing, missing


def _mesh(spec):
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
    return m


def test_qr_and_svd_report_unsupported(native_lib):
    m = api.load_spec(hpfem.poisson2d(2, 2, seed=1))
    with pytest.raises(api.UHMError) as e:
        m.qr_with_free()
    assert e.value.code == 30
    for fn in ("uhm_svd_with_free_", "uhm_solve_qr_", "uhm_solve_svd_", "uhm_check_qr_", "uhm_check_svd_"):
        m2 = api.load_spec(hpfem.poisson2d(2, 2, seed=1))
        getattr(native_lib, fn)(C.byref(m2.h))
        assert m2.status() == 30, fn


def test_svd_thresholds_round_trip(native_lib):
    for setter, getter, v in (("set_svd_relative_threshold_", "get_svd_relative_threshold_", 1e-9),
                              ("set_svd_absolute_threshold_", "get_svd_absolute_threshold_", 2.5e-14)):
        getattr(native_lib, setter)(C.byref(C.c_double(v)))
        out = C.c_double(0)
        getattr(native_lib, getter)(C.byref(out))
        assert out.value == v
    native_lib.set_svd_cutoff_small_(C.byref(C.c_int(1)))
    f = C.c_int(0)
    native_lib.get_svd_cutoff_small_(C.byref(f))
    assert f.value == 1


@pytest.mark.parametrize("spd", [True, False])
def test_random_fill_gives_a_solvable_system(native_lib, spd):
    spec = hpfem.poisson3d(2, 3, seed=2, n_rhs=2)
    m = _mesh(spec)
    (m.random_spd_matrix if spd else m.random_matrix)()
    m.triangularize()                      # no effect here (kernels read lower triangles)
    assert m.status() == 0
    s = m.export_sparse()
    n = s["n_dof"]
    A = np.zeros((n, n))
    A[s["ia"], s["ja"]] = s["a"]
    d = np.abs(np.diag(A))
    assert np.all(d > np.abs(A).sum(axis=1) - d)          # strictly diagonally dominant
    if spd:
        assert np.array_equal(A, A.T)
        assert np.linalg.eigvalsh(A).min() > 0
    else:
        assert not np.array_equal(A, A.T)
    assert s["b"].shape == (n, 2) and np.abs(s["b"]).max() > 0
    # deterministic: a second mesh gets the same first fill
    m2 = _mesh(spec)
    (m2.random_spd_matrix if spd else m2.random_matrix)()
    assert np.array_equal(m2.export_sparse()["a"], s["a"])


def test_lu_incpiv_entry_is_exported_and_maps_to_the_pivoted_lu(native_lib):
    assert api.UHM_LU_INCPIV == 4
    assert hasattr(native_lib, "uhm_lu_incpiv_with_free_") and hasattr(native_lib, "uhm_solve_lu_incpiv_")
