"""The allocation-free dense solve (uhm_gpu_dense_chol_solve_noalloc).

Callers that may not allocate device memory hold their own Cholesky factor
and right-hand side in device buffers; this entry point solves with them
using only a fixed scratch array inside the library.  It is checked here
against the library's regular path - a mesh with one element holding the
whole dense matrix, factorised and solved through the reference-style
interface - on two calls in a row (the second call must not see stale
scratch from the first).  Tolerance: 1e-10 relative in the max norm, as
for the other FP64 parity tests.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from uhm_gb300 import api

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    return B @ B.T / n + np.eye(n)


def _mesh_solve(A, b):
    """x = A^{-1} b through the regular entry points: one element, n nodes of one dof."""
    n = A.shape[0]
    m = api.Mesh()
    nods = [m.add_node(i, 1, 1) for i in range(n)]
    e = m.add_element(0)
    for nd in nods:
        m.element_add_node(e, nd)
    m.lock()
    m.create_matrix_without_buffer(api.UHM_REAL, 1)
    ids = np.arange(n, dtype=np.int32)
    m.copy_in(e, ids, api.UHM_LHS, np.asfortranarray(A))
    m.copy_in(e, ids, api.UHM_RHS, b.reshape(n, 1))
    m.chol_with_free()
    m.solve_chol()
    return m.node_solution(ids, np.ones(n, np.int64), 1)[:, 0]


def _entry(native_lib):
    fn = native_lib.uhm_gpu_dense_chol_solve_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch, torch.device("cuda:0")


# n = 700: 11 blocks, the last one ragged; n = 37: a single partial block
# (the backward block waits on its own forward flag); ld = n + 13: a padded
# column-major factor; a stream made for the test instead of torch's current one
CASES = [(700, 0, False), (37, 0, False), (700, 13, False), (300, 5, True)]


@pytest.mark.parametrize("n,pad,own_stream", CASES)
def test_noalloc_dense_solve_matches_mesh_solve(native_lib, n, pad, own_stream):
    torch, dev = _device()
    fn = _entry(native_lib)
    A = _spd(n, 3)
    b = np.random.default_rng(4).standard_normal(n)
    x_ref = _mesh_solve(A, b)
    L = np.linalg.cholesky(A)
    ld = n + pad
    Lp = np.zeros((ld, n))
    Lp[:n, :] = L
    L_dev = torch.from_numpy(np.ascontiguousarray(Lp.T)).to(dev)   # column-major L, leading dimension ld
    stream = torch.cuda.Stream(dev) if own_stream else torch.cuda.current_stream(dev)
    for call in range(2):
        x_dev = torch.from_numpy(b.copy()).to(dev)
        torch.cuda.synchronize(dev)
        rc = fn(L_dev.data_ptr(), n, ld, x_dev.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert rc == 0, (call, rc)
        torch.cuda.synchronize(dev)
        x = x_dev.cpu().numpy()
        rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
        assert rel < REL_TOL, (call, rel)


def test_noalloc_wait_that_runs_out_returns_14(native_lib):
    """With the wait limit at 0 every wait that is not satisfied at its first
    look gives up: the call returns 14 and the device stays usable, so the
    next call (default limit) solves correctly."""
    torch, dev = _device()
    fn = _entry(native_lib)
    setl = native_lib.uhm_gpu_set_wait_limit
    setl.argtypes = [C.c_longlong]
    setl.restype = C.c_int
    n = 700
    A = _spd(n, 5)
    b = np.random.default_rng(6).standard_normal(n)
    L = np.linalg.cholesky(A)
    L_dev = torch.from_numpy(np.ascontiguousarray(L.T)).to(dev)
    stream = torch.cuda.current_stream(dev)
    x_dev = torch.from_numpy(b.copy()).to(dev)
    torch.cuda.synchronize(dev)
    assert setl(0) == 0
    try:
        rc = fn(L_dev.data_ptr(), n, n, x_dev.data_ptr(), C.c_void_p(stream.cuda_stream))
    finally:
        assert setl(-1) == 0
    assert rc == 14
    x_dev = torch.from_numpy(b.copy()).to(dev)
    torch.cuda.synchronize(dev)
    assert fn(L_dev.data_ptr(), n, n, x_dev.data_ptr(), C.c_void_p(stream.cuda_stream)) == 0
    x_ref = np.linalg.solve(A, b)
    x = x_dev.cpu().numpy()
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() < REL_TOL


def test_noalloc_rejects_bad_sizes(native_lib):
    fn = _entry(native_lib)
    dummy = C.c_void_p(16)                     # never dereferenced: the sizes are rejected first
    assert fn(dummy, 262144 + 1, 262144 + 1, dummy, None) == 30
    assert fn(dummy, 0, 1, dummy, None) == 7
    assert fn(dummy, 10, 5, dummy, None) == 7
