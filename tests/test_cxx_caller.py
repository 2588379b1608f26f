"""A C++ program written against uhm_gb300/csrc/mesh.hpp the way a user of
the reference's uhm::Mesh_ writes it (tests/cxx_caller/two_elements.cpp: the
free functions and Mesh_ / Element_ calls of UHM/example/cxx/ex1.cxx): it
compiles with warnings on, links the library, and its sizes and LAWN-41 cost
equal those of the same mesh built through the C ABI."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from uhm_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx_caller", "two_elements.cpp")
LIBDIR = os.path.join(ROOT, "uhm_gb300")


def test_cxx_caller(native_lib, tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "two_elements_cxx")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "uhm_gb300", "csrc"),
                        SRC, "-L", LIBDIR, "-luhm_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {k: float(v) for k, v in (line.split() for line in r.stdout.splitlines())}
    assert out["n_elements"] == 3 and out["n_dof"] == 25
    assert out["threads"] == 2 and out["block"] == 128
    # the same mesh through the C ABI
    m = api.Mesh()
    nods = [[3, 4, 5, 7, 9, 8, 1], [4, 6, 5, 10, 11, 9, 2]]
    nd = [1, 1, 1, 3, 3, 3, 3]
    made = {}
    for j in range(2):
        e = m.add_element(0)
        for i, n in enumerate(nods[j]):
            if n not in made:
                made[n] = m.add_node(n, nd[i], nd[i])
            m.element_add_node(e, made[n])
    m.build_tree()
    m.lock()
    m.create_matrix_without_buffer(api.UHM_REAL, 1)
    fd, _ = m.estimate_cost(api.UHM_LU_PIV, 1)
    assert out["flop_decompose"] == fd
