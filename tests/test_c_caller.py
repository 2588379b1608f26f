"""A C program calling the Fortran-style interface (tests/c_caller/two_elements.c,
the call order of the reference's UHM/example/f90/ex1.f90): the header
compiles as C99 with warnings on, the library links and, on the host, the
sequence up to copy_in runs (uhm_build_tree_ included); on the GPU the LU
factorisation, solve and copy_out give the solution of the assembled system
(numpy on the same pseudo-random matrices)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "two_elements.c")
LIBDIR = os.path.join(ROOT, "uhm_gb300")


def _build(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "two_elements")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                        "-L", LIBDIR, "-luhm_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, mode):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = {}
    xs = {}
    for line in r.stdout.splitlines():
        f = line.split()
        if f[0] == "x":
            xs[(int(f[1]), int(f[2]))] = float(f[3])
        else:
            out[f[0]] = float(f[1])
    return out, xs


def _expected():
    """the same numbers as the C program, and the assembled system's solution
    in each element's row order"""
    mask = (1 << 64) - 1
    s = 100
    vals = []
    for _ in range(15 * 15 + 15):
        s = (s * 6364136223846793005 + 1442695040888963407) & mask
        vals.append((s >> 11) * (1.0 / 9007199254740992.0))
    A = np.array(vals[:225]).reshape(15, 15, order="F")
    B = np.array(vals[225:])
    nodes = [[3, 4, 5, 7, 9, 8, 1], [4, 6, 5, 10, 11, 9, 2]]
    nd = [1, 1, 1, 3, 3, 3, 3]
    ndof = {n: nd[k] for e in nodes for k, n in enumerate(e)}
    off, o = {}, 0
    for n in sorted(ndof):
        off[n] = o
        o += ndof[n]
    G = np.zeros((o, o))
    b = np.zeros(o)
    rows = []
    for e in nodes:
        r = np.concatenate([np.arange(off[n], off[n] + ndof[n]) for n in e])
        rows.append(r)
        G[np.ix_(r, r)] += A
        b[r] += B
    x = np.linalg.solve(G, b)
    return o, [x[r] for r in rows]


def test_c_caller_host_sequence(native_lib, tmp_path):
    exe = _build(tmp_path)
    out, _ = _run(exe, "host")
    assert out["n_dof"] == _expected()[0] == 25
    assert out["status"] == 0


@pytest.mark.gpu
def test_c_caller_factor_solve(native_lib, tmp_path):
    exe = _build(tmp_path)
    out, xs = _run(exe, "full")
    assert out["status"] == 0 and out["solve_status"] == 0
    _, want = _expected()
    scale = max(np.abs(w).max() for w in want)
    for j in range(2):
        got = np.array([xs[(j, i)] for i in range(15)])
        assert np.abs(got - want[j]).max() <= 1e-10 * scale
    assert out["residual"] <= 1e-10 * scale
