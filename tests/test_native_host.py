"""Host side of the native library, no GPU: the C ABI exports every function
that include/uhm_gb300.h declares, and the symbolic phase (Mesh_::lock) run
through that ABI gives the reference's front structure and flop estimates."""
import importlib.util
import os
import re

import numpy as np
import pytest

from uhm_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
_spec = importlib.util.spec_from_file_location("golden_cases", os.path.join(GOLDEN, "cases.py"))
golden_cases = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(golden_cases)


def _declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith("uhm_"):
                names.append(name)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared_functions()
    assert len(names) > 40
    assert "uhm_chol_with_free_" in names and "uhm_solve_chol_" in names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in _declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def _topology_mesh(spec):
    m = api.Mesh()
    nods = {}
    for nid, nd, p in zip(spec.node_id.tolist(), spec.node_ndof.tolist(), spec.node_p.tolist()):
        nods[nid] = m.add_node(nid, nd, p)
    elts = [m.add_element(int(g)) for g in spec.generation]
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


@pytest.mark.parametrize("case", golden_cases.CASES, ids=[c[0] for c in golden_cases.CASES])
def test_symbolic_matches_reference(native_lib, case):
    name, gen, kw, method = case
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    spec = golden_cases.make_spec(gen, kw)
    m = _topology_mesh(spec)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((spec.n_elements, 2), np.int64)
    got[eid] = np.stack([fs, ss], axis=1)
    assert np.array_equal(got, g["fronts"])
    fd, fsv = m.estimate_cost(method, spec.n_rhs)
    assert fd == pytest.approx(g["flops"][0], rel=1e-14)
    assert fsv == pytest.approx(g["flops"][1], rel=1e-14)


def test_tunables_round_trip_and_limits(native_lib):
    m = api.Mesh()
    assert m.tunables() == dict(small_max_f64=160, small_max_f32=224, tc_min_n=512, gc_min_rows=512,
                                fuse_potrf_trsm=2, tc_nbo=256, tc_panel=256,
                                solve_rows=64, lookahead=1, solve_chain=0)
    m.set_tunables(tc_min_n=768, small_max_f32=128)
    assert m.tunables()["tc_min_n"] == 768 and m.tunables()["small_max_f32"] == 128
    # whole-front shared-memory kernels hold at most 160 (FP64) / 224 (FP32) rows
    with pytest.raises(api.UHMError):
        m.set_tunables(small_max_f64=161)
    with pytest.raises(api.UHMError):
        m.set_tunables(small_max_f32=225)
    with pytest.raises(api.UHMError):
        m.set_tunables(tc_nbo=384)
    # the cooperative panel kernel holds 256 or 512 columns (0: not used)
    with pytest.raises(api.UHMError):
        m.set_tunables(tc_panel=128)
    m.set_tunables(tc_panel=0)
    assert m.tunables()["tc_panel"] == 0
    assert m.tunables()["small_max_f32"] == 128
