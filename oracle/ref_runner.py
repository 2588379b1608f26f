"""Runs the reference solver built by ``oracle/Makefile`` (TEST INFRASTRUCTURE).

Writes a :class:`uhm_gb300.hpfem.MeshSpec` in the binary layout that
``oracle/ref_driver.cpp`` reads, runs ``oracle/_ref/<machine>/uhm_ref_driver`` and
parses its output.  Only the fixture generator (``tests/golden/make_golden.py``)
and tests that skip when the binary is absent use this module; the reference
checkout is needed only to build the binary.
"""
from __future__ import annotations

import os
import platform
import subprocess
import tempfile
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MACHINE = platform.machine()
DRIVER = os.path.join(HERE, "_ref", MACHINE, "uhm_ref_driver")
STAGED = os.path.join(HERE, "_ref", "src")          # git-ignored copy of the sources the recipe needs


def reference_root() -> str:
    """Where the reference checkout is read from: $UHM_REFERENCE, else the
    checkout's usual place in the build container."""
    return os.environ.get("UHM_REFERENCE", "/root/reference")


@dataclass
class RefResult:
    x: np.ndarray          # (n_dof, n_rhs), node order of the spec, dofs of a node contiguous
    fronts: np.ndarray     # (n_elements, 2): (factor dofs, schur dofs) per element
    t_factor: float
    t_solve: float
    flop_decompose: float
    flop_solve: float
    t_lock: float = float("nan")   # the symbolic phase (Mesh_::lock), seconds
    rep_times: np.ndarray | None = None   # (reps, 2): factor and solve seconds of each repetition


def available() -> bool:
    return os.path.exists(DRIVER)


def build(ref_root: str | None = None, jobs: int = 16) -> bool:
    """Compile the reference solver for this machine.  With the checkout
    present, its sources are also staged into oracle/_ref/src (git-ignored),
    which travels with the working tree, so that a machine without the
    checkout (the GPU host, another architecture) can build the same solver
    from the staged copy.  Returns whether the driver binary exists."""
    ref_root = ref_root or reference_root()
    if os.path.isdir(os.path.join(ref_root, "UHM", "src")):
        subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF={ref_root}"], check=True)
        src = ref_root
    elif os.path.isdir(os.path.join(STAGED, "UHM", "src")):
        src = os.path.join("_ref", "src")
    else:
        return available()
    subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs}", f"REF={src}"], check=True)
    return available()


def write_spec(spec, method: int, path: str) -> None:
    i32 = lambda a: np.asarray(a, dtype="<i4").tobytes()
    with open(path, "wb") as f:
        f.write(b"UHMS" + i32([1]))
        f.write(i32([spec.n_nodes]))
        f.write(i32(np.stack([spec.node_id, spec.node_ndof, spec.node_p, spec.node_kind], axis=1).ravel()))
        f.write(i32([spec.n_elements, spec.n_leaves, spec.n_rhs, method]))
        f.write(i32(spec.generation))
        f.write(i32(spec.child_ptr))
        f.write(i32(spec.child_idx))
        f.write(i32(spec.elem_ptr))
        f.write(i32(spec.elem_node))
        for e in range(spec.n_leaves):
            f.write(np.asarray(spec.element_matrix(e), dtype="<f8").ravel(order="F").tobytes())
            f.write(np.asarray(spec.element_rhs(e), dtype="<f8").ravel(order="F").tobytes())


def read_result(path: str, spec) -> RefResult:
    buf = open(path, "rb").read()
    if buf[:4] != b"UHMR":
        raise ValueError("bad reference output")
    p = 4
    ver, n_nodes, n_rhs = np.frombuffer(buf, "<i4", 3, p)
    p += 12
    assert ver == 1 and n_nodes == spec.n_nodes
    n_dof = int(spec.node_ndof.sum())
    x = np.frombuffer(buf, "<f8", n_dof * n_rhs, p).reshape(n_dof, n_rhs).copy()
    p += 8 * n_dof * n_rhs
    n_el = int(np.frombuffer(buf, "<i4", 1, p)[0])
    p += 4
    fronts = np.frombuffer(buf, "<i4", 2 * n_el, p).reshape(n_el, 2).astype(np.int64)
    p += 8 * n_el
    tf, ts, fd, fs = np.frombuffer(buf, "<f8", 4, p)
    p += 32
    tl = float(np.frombuffer(buf, "<f8", 1, p)[0]) if len(buf) >= p + 8 else float("nan")
    p += 8
    reps = None
    if len(buf) >= p + 4:
        nrep = int(np.frombuffer(buf, "<i4", 1, p)[0])
        p += 4
        reps = np.frombuffer(buf, "<f8", 2 * nrep, p).reshape(nrep, 2).copy()
    return RefResult(x, fronts, float(tf), float(ts), float(fd), float(fs), tl, reps)


def run(spec, method: int, threads: int = 1, reps: int = 1) -> RefResult:
    """Factor and solve the spec with the reference solver on `threads` OpenMP
    threads (sequential OpenBLAS inside each task, as the reference's own
    builds use); with reps > 1 the numeric work is repeated and every
    repetition's factor and solve times are returned in rep_times."""
    if not available():
        raise RuntimeError("reference solver not built (make -C oracle)")
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        write_spec(spec, method, fin)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
        subprocess.run([DRIVER, fin, fout, str(threads), str(max(1, int(reps)))], check=True, env=env,
                       stdout=subprocess.DEVNULL)
        return read_result(fout, spec)


def run_sparse(spec) -> dict:
    """The reference's own sparse export of the spec's leaves (DSparse_ with
    C numbering, row keys: import_element of every leaf in order, then
    triplet without symmetry), with each node's first global dof in the
    reference's numbering."""
    if not available():
        raise RuntimeError("reference solver not built (make -C oracle)")
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        write_spec(spec, 1, fin)
        env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
        subprocess.run([DRIVER, fin, fout, "1", "sparse"], check=True, env=env, stdout=subprocess.DEVNULL)
        buf = open(fout, "rb").read()
    if buf[:4] != b"UHMP":
        raise ValueError("bad reference sparse output")
    p = 4
    ver, n_nodes = np.frombuffer(buf, "<i4", 2, p)
    p += 8
    assert ver == 1 and n_nodes == spec.n_nodes
    offsets = np.frombuffer(buf, "<i4", n_nodes, p).copy()
    p += 4 * n_nodes
    n_dof, n_rhs, nnz = (int(v) for v in np.frombuffer(buf, "<i4", 3, p))
    p += 12
    ia = np.frombuffer(buf, "<i4", nnz, p).copy()
    p += 4 * nnz
    ja = np.frombuffer(buf, "<i4", nnz, p).copy()
    p += 4 * nnz
    a = np.frombuffer(buf, "<f8", nnz, p).copy()
    p += 8 * nnz
    nb = int(np.frombuffer(buf, "<i4", 1, p)[0])
    p += 4
    b = np.frombuffer(buf, "<f8", nb, p).copy()
    return dict(offsets=offsets, n_dof=n_dof, n_rhs=n_rhs, ia=ia, ja=ja, a=a, b=b)
