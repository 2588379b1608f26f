"""Element matrices generated on the device (uhm_gpu_generate_lobatto_elements)
instead of built on the host and copied in.  The generator forms every entry
with the host generator's products and sums in the same order, so the FP64
solutions must be bit-identical to those from copied-in matrices, for
diffusion, convection-diffusion (LU), 2D, variable-order and reaction meshes
(and 2D convection with reaction);
generating over copied-in matrices gives the same solution too."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

CASES = [
    ("diff_4_p3", lambda: hpfem.diffusion3d(4, 3, seed=61, contrast=1e3), uo.CHOL),
    ("cd_4_p3", lambda: hpfem.convdiff3d(4, 3, seed=62), uo.LU_PIV),
    ("2d_8_p4", lambda: hpfem.poisson2d(8, 4, seed=63), uo.CHOL),
    ("varp_3", lambda: hpfem.build_mesh(3, 3, np.random.default_rng(4).integers(2, 6, 27), seed=64), uo.CHOL),
    ("react_3_p3", lambda: hpfem.build_mesh(3, 3, 3, react=-3.0, seed=65), uo.CHOL),
    ("cd2d_react_8_p3", lambda: hpfem.build_mesh(2, 8, 3, beta=(30.0, -20.0), react=0.5, seed=67), uo.LU_PIV),
]


def _solve(m, spec, method):
    m.factor(method)
    m.solve(method)
    assert m.status() == 0
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


@pytest.mark.parametrize("name,make,method", CASES, ids=[c[0] for c in CASES])
def test_generated_elements_match_copied_in(native_lib, name, make, method):
    spec = make()
    recipe = hpfem.element_recipe(spec)
    x_copy = _solve(api.load_spec(spec), spec, method)
    m = api.load_spec(spec, lhs=False)
    m.generate_elements(recipe, method)
    x_gen = _solve(m, spec, method)
    assert np.array_equal(x_gen, x_copy)
    # regenerate over the same mesh (its matrices already on the device)
    m.generate_elements(recipe, method)
    assert np.array_equal(_solve(m, spec, method), x_copy)
    ref = uo.solve_mesh(spec, method).x
    assert np.abs(x_gen - ref).max() <= 1e-10 * np.abs(ref).max()


def test_generator_rejects_mismatched_recipe(native_lib):
    spec = hpfem.poisson3d(2, 3, seed=66)
    other = hpfem.poisson3d(2, 2, seed=66)
    m = api.load_spec(spec, lhs=False)
    with pytest.raises(api.UHMError):
        m.generate_elements(hpfem.element_recipe(other), uo.CHOL)
