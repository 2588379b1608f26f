"""The oracle pinned against the reference's own solver (CPU only).

``tests/golden/*.npz`` hold outputs of the reference's C++ sources (UHM +
LINAL) built by ``oracle/Makefile`` and run by ``tests/golden/make_golden.py``.
Tolerances: solutions agree to 1e-12 relative in the max norm (both sides are
FP64 with different BLAS blocking, so bit equality is not expected); front
sizes and flop estimates are integers / exact sums and must be equal.
"""
import importlib.util
import os

import numpy as np
import pytest

from oracle import ref_runner
from oracle import uhm_oracle as uo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_spec = importlib.util.spec_from_file_location("golden_cases", os.path.join(GOLDEN, "cases.py"))
golden_cases = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(golden_cases)
CASES = golden_cases.CASES
IDS = [c[0] for c in CASES]
X_TOL = 1e-12


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("name,gen,kw,method", CASES, ids=IDS)
def test_generator_reproduces_golden_inputs(name, gen, kw, method):
    g = _load(name)
    spec = golden_cases.make_spec(gen, kw)
    assert golden_cases.spec_digest(spec) == str(g["digest"]), "mesh generator changed: regenerate fixtures"
    assert int(g["method"]) == method


@pytest.mark.parametrize("name,gen,kw,method", CASES, ids=IDS)
def test_oracle_matches_reference(name, gen, kw, method):
    g = _load(name)
    spec = golden_cases.make_spec(gen, kw)
    # 4 (lu_incpiv): the reference pivots within each diagonal block; the
    # oracle's LU with partial pivoting must give its solution to rounding
    method = uo.LU_PIV if method == 4 else method
    res = uo.solve_mesh(spec, method)
    assert np.array_equal(res.plan.fs_ss(), g["fronts"]), "front (factor, schur) sizes differ"
    scale = max(np.abs(g["x"]).max(), 1e-300)
    assert np.abs(res.x - g["x"]).max() / scale < X_TOL
    fd, fsv = uo.mesh_cost(res.plan, method, spec.n_rhs)
    assert fd == pytest.approx(g["flops"][0], rel=1e-14)
    assert fsv == pytest.approx(g["flops"][1], rel=1e-14)


def test_oracle_catches_a_planted_error():
    """A wrong extend-add (one child contribution dropped) must fail the pin."""
    name, gen, kw, method = CASES[5]
    g = _load(name)
    spec = golden_cases.make_spec(gen, kw)
    spec.rhs = spec.rhs.copy()
    spec.rhs[: int(spec.elem_m[0])] *= 1.0 + 1e-9     # perturb one element's load
    res = uo.solve_mesh(spec, method)
    assert np.abs(res.x - g["x"]).max() / np.abs(g["x"]).max() > X_TOL


@pytest.mark.skipif(not ref_runner.available(), reason="reference solver not built here (make -C oracle)")
@pytest.mark.parametrize("name", ["3d_4_p3_lupiv", "3d_4_p3_rhs4"])
def test_live_reference_reproduces_golden(name):
    case = next(c for c in CASES if c[0] == name)
    g = _load(name)
    spec = golden_cases.make_spec(case[1], case[2])
    r = ref_runner.run(spec, case[3])
    assert np.array_equal(r.fronts, g["fronts"])
    assert np.abs(r.x - g["x"]).max() <= 1e-14 * np.abs(g["x"]).max()
