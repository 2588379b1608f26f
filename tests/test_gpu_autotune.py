"""The threshold autotuner (uhm_gpu_autotune): it times candidate values of
the kernel-selection thresholds on the mesh at hand, keeps valid values and
leaves a solution that meets the refinement tolerance; a mesh tuned and then
solved again with the chosen values still matches the oracle."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,make,method,prec", [
    ("3d_8_p4_bf16", lambda: hpfem.poisson3d(8, 4, seed=51), uo.CHOL, api.PREC_BF16X3),
    ("cd_12_p3_fp32", lambda: hpfem.convdiff3d(12, 3, seed=52), uo.LU_PIV, api.PREC_FP32),
])
def test_autotune_keeps_valid_thresholds(native_lib, name, make, method, prec):
    spec = make()
    m = api.load_spec(spec)
    m.set_mode(1, prec, 1e-12, 10)
    r = m.autotune(method, reps=1)
    assert r["timed"] >= 1
    assert r["small_max_f64"] in (64, 96, 128, 160)
    assert r["small_max_f32"] in (96, 128, 160, 192, 224)
    assert r["tc_min_n"] in (384, 512, 768, 1024, 1536, 1 << 30)
    assert r["gc_min_rows"] in (256, 512, 1024, 2048, 1 << 30)
    assert r["fuse_potrf_trsm"] in (0, 1, 2, 4)
    assert r["tc_nbo"] in (128, 256, 512)
    assert m.timing()["berr"] <= 1e-12
    m.factor(method)
    m.solve(method)
    assert m.status() == 0 and m.timing()["berr"] <= 1e-12
    x = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)
    ref = uo.solve_mesh(spec, method).x
    assert np.abs(x - ref).max() <= 1e-8 * np.abs(ref).max()
