"""Device factor/solve against the reference's own solver (golden fixtures
in tests/golden, produced by the reference's C++ sources).

Tolerance: the plain FP64 device path matches the reference solution to 1e-10
relative in the max norm; the mixed-precision path with iterative refinement
reaches a backward error of 1e-12 and matches the reference to 1e-8 relative
(forward error is bounded by the condition number times the backward error)."""
import importlib.util
import os

import numpy as np
import pytest

from uhm_gb300 import api

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_spec = importlib.util.spec_from_file_location("golden_cases", os.path.join(GOLDEN, "cases.py"))
golden_cases = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(golden_cases)
CASES = golden_cases.CASES
IDS = [c[0] for c in CASES]


def _run(spec, method, mixed=False):
    m = api.load_spec(spec)
    if mixed:
        m.set_mode(1, api.PREC_FP32, 1e-12, 10)
    m.factor(method)
    m.solve(method)
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)
    return m, x


@pytest.mark.parametrize("name,gen,kw,method", CASES, ids=IDS)
def test_fp64_matches_reference(native_lib, name, gen, kw, method):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    spec = golden_cases.make_spec(gen, kw)
    m, x = _run(spec, method)
    eid, _, fs, ss = m.fronts()
    got = np.zeros((spec.n_elements, 2), np.int64)
    got[eid] = np.stack([fs, ss], axis=1)
    assert np.array_equal(got, g["fronts"])
    rel = np.abs(x - g["x"]).max() / np.abs(g["x"]).max()
    assert rel < 1e-10, rel


@pytest.mark.parametrize("name,gen,kw,method", [c for c in CASES if c[3] == 1], ids=[c[0] for c in CASES if c[3] == 1])
def test_mixed_ir_matches_reference(native_lib, name, gen, kw, method):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    spec = golden_cases.make_spec(gen, kw)
    m, x = _run(spec, method, mixed=True)
    assert m.backward_error() <= 1e-12
    rel = np.abs(x - g["x"]).max() / np.abs(g["x"]).max()
    assert rel < 1e-8, rel
