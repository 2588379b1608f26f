"""The chain solves of large FP32 Cholesky fronts (k_fwd_chain / k_bwd_chain),
the solve_chain = 1 form of the 64-row solves (the default, 0, runs the
flag-driven kernels).

One CTA per front solves the 64-row diagonal blocks in turn from shared
memory, applying the CH_K = 3 blocks next to the diagonal itself; helper
CTAs sum the blocks further away and hand their partial sums over as
self-validating words.  The reference's steps are the same triangular
solves (UHM/src/matrix/uhm/fla/chol/solve.cxx:152-202); only the order of
the additions within a row differs from the flag-driven kernels.

Checked: the chain solves give the oracle's solution and the flag-driven
kernels' first-solve backward error (same FP32 factors) on fronts with many
blocks (root 2791), with ABL rows (level-3 fronts), with ragged last blocks,
with several right-hand sides (two launch groups), and on a configuration
where the leaf level has more large fronts than may run as chains (those
levels fall back to the flag-driven kernels); the profile shows the chain
kernels."""
import numpy as np
import pytest

from oracle import uhm_oracle as uo
from uhm_gb300 import api, hpfem

pytestmark = pytest.mark.gpu

REL_TOL_MIXED = 1e-8


def _x(m, spec):
    return m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof, spec.n_rhs)


def _solve(spec, **tun):
    m = api.load_spec(spec)
    m.set_tunables(**tun)
    m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
    m.chol_with_free()
    m.solve_chol()
    assert m.status() == 0, m.last_error()
    return m, m.timing()


CASES = [
    ("3d_8_p4", lambda: hpfem.poisson3d(8, 4, seed=61), {}),
    ("diff_8_p3_fp32_fronts", lambda: hpfem.diffusion3d(8, 3, seed=62, contrast=1e3), {"tc_min_n": 1 << 30}),
    ("3d_6_p4_rhs7", lambda: hpfem.poisson3d(6, 4, seed=63, n_rhs=7), {}),
    # large leaf fronts: 512 per level, beyond the chains one launch may hold
    ("3d_8_p4_small96", lambda: hpfem.poisson3d(8, 4, seed=64), {"small_max_f32": 96}),
]


@pytest.mark.parametrize("name,make,tun", CASES, ids=[c[0] for c in CASES])
def test_chain_matches_oracle_and_flag_kernels(native_lib, name, make, tun):
    spec = make()
    ref = uo.solve_mesh(spec, uo.CHOL)
    m1, t1 = _solve(spec, solve_chain=1, **tun)
    m0, t0 = _solve(spec, solve_chain=0, **tun)
    for m, t in ((m1, t1), (m0, t0)):
        assert t["berr"] <= 1e-12
        rel = np.abs(_x(m, spec) - ref.x).max() / np.abs(ref.x).max()
        assert rel < REL_TOL_MIXED, (name, rel)
    # the same FP32 factors: first-solve errors of one order
    assert t1["berr_first"] < 10 * t0["berr_first"] + 1e-14, (t1["berr_first"], t0["berr_first"])
    assert t0["berr_first"] < 10 * t1["berr_first"] + 1e-14, (t1["berr_first"], t0["berr_first"])


def test_chain_kernels_launch(native_lib):
    spec = hpfem.poisson3d(8, 4, seed=65)
    m = api.load_spec(spec)
    m.set_tunables(solve_chain=1)
    m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
    m.set_profiling(True)
    m.chol_with_free()
    m.solve_chol()
    prof = m.profile()
    assert prof["fwd_chain"]["launches"] > 0 and prof["bwd_chain"]["launches"] > 0
