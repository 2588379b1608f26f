"""Python mirror of UHM's Mesh API over the C ABI of include/uhm_gb300.h.

Method names and argument meaning follow ``uhm::Mesh_`` / the Fortran
interface (UHM/include/uhm/mesh/mesh.hxx:82-293,
UHM/include/uhm/wrapper/fort.hxx:47-190).  Every call goes through
``libuhm_gb300.so``; there is no Python or CPU fallback for the numerics: if
the library cannot be loaded, importing this module fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libuhm_gb300.so")

UHM_REAL, UHM_COMPLEX = 101, 103
UHM_LHS, UHM_RHS = 1, 2
UHM_PHYSICS_SINGLE, UHM_PHYSICS_MULTI = 1, 2
UHM_CHOL, UHM_LU_NOPIV, UHM_LU_PIV, UHM_LU_INCPIV = 1, 2, 3, 4
PREC_FP64, PREC_FP32, PREC_BF16X3, PREC_BF16X6, PREC_LEARNED = 0, 1, 2, 3, 4
STATUS_RECOMPUTED_FP64 = 20     # refinement missed; the solution was recomputed in FP64

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"uhm_gb300 native library missing: {LIB_PATH} "
                               "(build it with `python -m uhm_gb300.build`)")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_P = C.POINTER
_l, _i, _d = C.c_long, C.c_int, C.c_double


def _declare(L):
    def sig(name, args, res=None):
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    sig("uhm_mesh_create_", [_P(_l)])
    sig("uhm_gpu_set_wait_limit", [C.c_longlong], _i)
    sig("uhm_mesh_delete_", [_P(_l)])
    sig("uhm_add_element_", [_P(_l), _P(_l)])
    sig("uhm_add_node_", [_P(_l), _P(_i), _P(_i), _P(_i), _P(_i), _P(_l)])
    sig("uhm_element_add_node_", [_P(_l), _P(_l)])
    sig("uhm_copy_in_", [_P(_l), _P(_l), _P(_i), _P(_i), _P(_i), _P(_i), _P(_i), _P(_i), _P(_d)])
    sig("uhm_copy_out_", [_P(_l), _P(_l), _P(_i), _P(_i), _P(_i), _P(_i), _P(_i), _P(_i), _P(_d)])
    sig("uhm_get_n_dof_", [_P(_l), _P(_i)])
    sig("uhm_get_n_nonzero_", [_P(_l), _P(_i)])
    sig("uhm_estimate_cost_", [_P(_l), _P(_i), _P(_i), _P(_i), _P(_d), _P(_d), _P(C.c_uint), _P(_d)])
    sig("uhm_mesh_import_", [_P(_l), C.c_char_p])
    sig("uhm_build_tree_", [_P(_l)])
    sig("uhm_create_matrix_without_buffer_", [_P(_l), _P(_i), _P(_i)])
    sig("uhm_create_leaf_matrix_buffer_", [_P(_l)])
    sig("uhm_create_element_matrix_buffer_", [_P(_l), _P(_i)])
    sig("uhm_set_rhs_", [_P(_l)])
    sig("uhm_lock_", [_P(_l)])
    sig("uhm_unlock_", [_P(_l)])
    for n in ("chol_with_free", "lu_nopiv_with_free", "lu_piv_with_free", "solve_chol",
              "solve_lu_nopiv", "solve_lu_piv", "check_chol", "check_lu_nopiv", "check_lu_piv"):
        sig(f"uhm_{n}_", [_P(_l)])
    sig("uhm_get_residual_", [_P(_l), _P(_d)])
    sig("uhm_get_flop_", [_P(_d)])
    sig("uhm_reset_flop_", [])
    sig("uhm_set_num_threads_", [_P(_i)])
    sig("uhm_gpu_add_element_with_generation", [_P(_l), _P(_i), _P(_l)], _i)
    sig("uhm_gpu_element_set_parent", [_P(_l), _P(_l)], _i)
    sig("uhm_gpu_element_add_child", [_P(_l), _P(_l)], _i)
    sig("uhm_gpu_get_status", [_P(_l)], _i)
    sig("uhm_gpu_get_last_error", [_P(_l), C.c_char_p, _i], _i)
    sig("uhm_gpu_set_mode", [_P(_l), _i, _i, _d, _i], _i)
    sig("uhm_gpu_set_front_precision", [_P(_l), _i, _P(_i)], _i)
    sig("uhm_gpu_copy_in_leaves", [_P(_l), _i, _P(_i), _P(_d), _l], _i)
    sig("uhm_gpu_copy_out_leaves", [_P(_l), _P(_d), _l], _i)
    sig("uhm_gpu_get_node_solution", [_P(_l), _i, _P(_i), _P(_d), _l], _i)
    sig("uhm_gpu_backward_error", [_P(_l), _P(_d)], _i)
    sig("uhm_gpu_get_timing", [_P(_l), _P(_d)], _i)
    sig("uhm_gpu_get_n_fronts", [_P(_l), _P(_i)], _i)
    sig("uhm_gpu_get_fronts", [_P(_l), _i, _P(_i), _P(_i), _P(_i), _P(_i)], _i)
    sig("uhm_gpu_get_front_nodes", [_P(_l), _i, _i, _P(_i), _P(_i), _P(_i)], _i)
    sig("uhm_gpu_set_profiling", [_P(_l), _i], _i)
    sig("uhm_gpu_get_profile", [_P(_l), _i, _P(_d), _P(_d), _P(_d), _P(_l)], _i)
    sig("uhm_gpu_host_alloc", [_l], C.c_void_p)
    sig("uhm_gpu_host_free", [C.c_void_p])
    _f = C.c_float
    sig("uhm_gpu_set_selector", [_P(_l), _P(_f), _i], _i)
    sig("uhm_gpu_set_tunables", [_P(_l), _P(_i)], _i)
    sig("uhm_gpu_get_tunables", [_P(_l), _P(_i)], _i)
    sig("uhm_gpu_autotune", [_P(_l), _i, _i, _P(_i)], _i)
    sig("uhm_gpu_generate_lobatto_elements", [_P(_l), _i, _i, _d, _d, _d, _i, _P(_d), _P(_l), _i, _P(_i),
                                              _P(_d), _P(_d), _P(_d), _P(_l), _P(_i)], _i)
    sig("uhm_gpu_element_set_reuse", [_P(_l), _i], _i)
    sig("uhm_gpu_element_get_reuse", [_P(_l), _P(_i)], _i)
    sig("uhm_gpu_mesh_backup", [_P(_l), _P(_l)], _i)
    sig("uhm_gpu_mesh_check_reuse", [_P(_l), _P(_l)], _i)
    sig("uhm_gpu_get_n_refactored", [_P(_l), _P(_i)], _i)
    sig("uhm_gpu_export_sparse", [_P(_l), _i, _i, _i, _i, _i, _P(_i), _P(_i), _P(_l), _P(_l), _P(_l),
                                  _P(_i), _P(_i), _P(_d), _P(_d)], _i)
    sig("uhm_gpu_get_node_offsets", [_P(_l), _i, _P(_i), _P(_i)], _i)
    sig("uhm_gpu_get_tree", [_P(_l), _i, _P(_i), _P(_i), _P(_i), _P(_i)], _i)
    sig("uhm_gpu_get_children", [_P(_l), _i, _i, _P(_i), _P(_i)], _i)
    sig("uhm_gpu_get_op_log", [_P(_l), _i, _P(_i), _P(_i), _P(_d), _P(_i)], _i)
    sig("uhm_gpu_get_front_features", [_P(_l), _i, _i, _P(_f)], _i)
    sig("uhm_gpu_get_front_precision", [_P(_l), _i, _P(_i), _P(_i)], _i)
    sig("uhm_gpu_mlp_n_params", [], _i)
    sig("uhm_gpu_mlp_n_features", [], _i)
    sig("uhm_gpu_mlp_predict", [_P(_f), _i, _P(_f), _P(_i), _P(_f)], _i)
    sig("uhm_gpu_mlp_gradient", [_P(_f), _P(_i), _P(_f), _i, _P(_f), _P(_f), _P(_f)], _i)
    sig("uhm_gpu_mlp_train", [_P(_f), _P(_i), _P(_f), _i, _P(_f), _i, _i, _f, C.c_ulonglong, _P(_f)], _i)


class UHMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def _ip(v):
    return C.byref(_i(int(v)))


def _arr(a, dtype, ctype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data_as(_P(ctype))


class Mesh:
    """Handle to a ``uhm::Mesh_`` living in the native library."""

    def __init__(self):
        self.L = lib()
        self.h = _l(0)
        self.L.uhm_mesh_create_(C.byref(self.h))
        self._elements = {}
        self.n_rhs = 1

    def __del__(self):
        try:
            if self.h.value:
                self.L.uhm_mesh_delete_(C.byref(self.h))
        except Exception:
            pass

    # -- errors --------------------------------------------------------
    def status(self) -> int:
        return int(self.L.uhm_gpu_get_status(C.byref(self.h)))

    def last_error(self) -> str:
        buf = C.create_string_buffer(1024)
        self.L.uhm_gpu_get_last_error(C.byref(self.h), buf, 1024)
        return buf.value.decode()

    def _check(self, code=None):
        st = self.status() if code is None else code
        if st and st != STATUS_RECOMPUTED_FP64:
            raise UHMError(st, self.last_error())

    # -- topology --------------------------------------------------------
    def add_node(self, id, n_dof, p=None, phy=0):
        nod = _l(0)
        self.L.uhm_add_node_(C.byref(self.h), _ip(id), _ip(phy), _ip(n_dof),
                             _ip(n_dof if p is None else p), C.byref(nod))
        return nod.value

    def add_element(self, gen=None):
        e = _l(0)
        if gen is None:
            self.L.uhm_add_element_(C.byref(self.h), C.byref(e))
        else:
            self.L.uhm_gpu_add_element_with_generation(C.byref(self.h), _ip(gen), C.byref(e))
        return e.value

    def element_add_node(self, elt, nod):
        self.L.uhm_element_add_node_(C.byref(_l(elt)), C.byref(_l(nod)))

    def set_parent(self, elt, parent):
        self.L.uhm_gpu_element_set_parent(C.byref(_l(elt)), C.byref(_l(parent)))

    def add_child(self, elt, child):
        self.L.uhm_gpu_element_add_child(C.byref(_l(elt)), C.byref(_l(child)))

    # -- factor reuse (Mesh_::backup / check_reuse, Element_::set_reuse) ----
    def set_reuse(self, elt, flag=True):
        self.L.uhm_gpu_element_set_reuse(C.byref(_l(elt)), int(bool(flag)))

    def get_reuse(self, elt) -> bool:
        f = _i(0)
        self.L.uhm_gpu_element_get_reuse(C.byref(_l(elt)), C.byref(f))
        return bool(f.value)

    def backup(self, other: "Mesh"):
        self._check(self.L.uhm_gpu_mesh_backup(C.byref(self.h), C.byref(other.h)))

    def check_reuse(self, other: "Mesh"):
        self._check(self.L.uhm_gpu_mesh_check_reuse(C.byref(self.h), C.byref(other.h)))

    def n_refactored(self) -> int:
        n = _i(0)
        self._check(self.L.uhm_gpu_get_n_refactored(C.byref(self.h), C.byref(n)))
        return n.value

    # -- sparse export (DSparse_::import_element + triplet / compress) --------
    def export_sparse(self, is_sym=False, fort=False, cs=False, compress=False, axpy=True) -> dict:
        nd, nr = _i(0), _i(0)
        lia, lja, nnz = _l(0), _l(0), _l(0)
        flags = [int(bool(v)) for v in (is_sym, fort, cs, compress, axpy)]
        self._check(self.L.uhm_gpu_export_sparse(C.byref(self.h), *flags, C.byref(nd), C.byref(nr),
                                                 C.byref(lia), C.byref(lja), C.byref(nnz),
                                                 None, None, None, None))
        ia = np.zeros(lia.value, np.int32)
        ja = np.zeros(lja.value, np.int32)
        a = np.zeros(nnz.value)
        b = np.zeros(nd.value * nr.value)
        self._check(self.L.uhm_gpu_export_sparse(C.byref(self.h), *flags, C.byref(nd), C.byref(nr),
                                                 C.byref(lia), C.byref(lja), C.byref(nnz),
                                                 ia.ctypes.data_as(_P(_i)), ja.ctypes.data_as(_P(_i)),
                                                 a.ctypes.data_as(_P(_d)), b.ctypes.data_as(_P(_d))))
        return dict(n_dof=nd.value, n_rhs=nr.value, ia=ia, ja=ja, a=a, b=b.reshape(nr.value, nd.value).T)

    def build_tree(self):
        self.L.uhm_build_tree_(C.byref(self.h))
        self._check()

    def tree(self):
        """(element ids, parent ids (-1 for roots), generations, {id: children})"""
        n = _i(0)
        self._check(self.L.uhm_gpu_get_tree(C.byref(self.h), 0, None, None, None, C.byref(n)))
        eid, par, gen = (np.zeros(n.value, np.int32) for _ in range(3))
        self._check(self.L.uhm_gpu_get_tree(C.byref(self.h), n.value, eid.ctypes.data_as(_P(_i)),
                                            par.ctypes.data_as(_P(_i)), gen.ctypes.data_as(_P(_i)),
                                            C.byref(n)))
        kids = {}
        buf = np.zeros(1 << 16, np.int32)
        for e in eid.tolist():
            k = _i(0)
            self._check(self.L.uhm_gpu_get_children(C.byref(self.h), e, len(buf),
                                                    buf.ctypes.data_as(_P(_i)), C.byref(k)))
            kids[e] = buf[:k.value].tolist()
        return eid, par, gen, kids

    def node_offsets(self, ids) -> np.ndarray:
        ids = np.ascontiguousarray(ids, np.int32)
        out = np.zeros(len(ids), np.int32)
        self._check(self.L.uhm_gpu_get_node_offsets(C.byref(self.h), len(ids), ids.ctypes.data_as(_P(_i)),
                                                    out.ctypes.data_as(_P(_i))))
        return out

    def lock(self):
        self.L.uhm_lock_(C.byref(self.h))
        self._check()

    def unlock(self):
        self.L.uhm_unlock_(C.byref(self.h))

    def import_file(self, path: str):
        self.L.uhm_mesh_import_(C.byref(self.h), path.encode())
        self._check()

    # -- matrices ----------------------------------------------------------
    def create_matrix_without_buffer(self, datatype=UHM_REAL, n_rhs=1):
        self.n_rhs = n_rhs
        self.L.uhm_create_matrix_without_buffer_(C.byref(self.h), _ip(datatype), _ip(n_rhs))
        self._check()

    def create_matrix_buffer(self):
        self.L.uhm_create_element_matrix_buffer_(C.byref(self.h), _ip(0))

    def copy_in(self, elt, nods, side, buf, datatype=UHM_REAL):
        buf = np.asfortranarray(buf, dtype=np.float64)
        m = buf.shape[0]
        n = buf.shape[1] if buf.ndim == 2 else 1
        nods_a, nods_p = _arr(nods, np.int32, _i)
        self.L.uhm_copy_in_(C.byref(self.h), C.byref(_l(elt)), _ip(datatype), _ip(m), _ip(n),
                            _ip(UHM_PHYSICS_SINGLE), nods_p, _ip(side),
                            buf.ctypes.data_as(_P(_d)))
        self._check()

    def copy_out(self, elt, nods, m, n=1, datatype=UHM_REAL):
        out = np.zeros((m, n), order="F")
        nods_a, nods_p = _arr(nods, np.int32, _i)
        self.L.uhm_copy_out_(C.byref(self.h), C.byref(_l(elt)), _ip(datatype), _ip(m), _ip(n),
                             _ip(UHM_PHYSICS_SINGLE), nods_p, _ip(UHM_RHS),
                             out.ctypes.data_as(_P(_d)))
        self._check()
        return out

    def set_rhs(self):
        self.L.uhm_set_rhs_(C.byref(self.h))

    # -- factor / solve ------------------------------------------------------
    def _call(self, name):
        getattr(self.L, f"uhm_{name}_")(C.byref(self.h))
        self._check()

    def chol_with_free(self):
        self._call("chol_with_free")

    def lu_piv_with_free(self):
        self._call("lu_piv_with_free")

    def lu_nopiv_with_free(self):
        self._call("lu_nopiv_with_free")

    def lu_incpiv_with_free(self):
        self._call("lu_incpiv_with_free")

    def qr_with_free(self):
        self._call("qr_with_free")

    def random_spd_matrix(self):
        self._call("random_spd_matrix")

    def random_matrix(self):
        self._call("random_matrix")

    def triangularize(self):
        self._call("triangularize")

    def solve_chol(self):
        self._call("solve_chol")

    def solve_lu_piv(self):
        self._call("solve_lu_piv")

    def solve_lu_nopiv(self):
        self._call("solve_lu_nopiv")

    def factor(self, method):
        {UHM_CHOL: self.chol_with_free, UHM_LU_PIV: self.lu_piv_with_free,
         UHM_LU_NOPIV: self.lu_nopiv_with_free, UHM_LU_INCPIV: self.lu_incpiv_with_free}[method]()

    def solve(self, method):
        # an lu_incpiv factorisation is solved by solve_lu_piv, as in the reference
        {UHM_CHOL: self.solve_chol, UHM_LU_PIV: self.solve_lu_piv,
         UHM_LU_NOPIV: self.solve_lu_nopiv, UHM_LU_INCPIV: self.solve_lu_piv}[method]()

    def get_residual(self) -> float:
        r = _d(0)
        self.L.uhm_get_residual_(C.byref(self.h), C.byref(r))
        self._check()
        return r.value

    def backward_error(self) -> float:
        r = _d(0)
        self._check(self.L.uhm_gpu_backward_error(C.byref(self.h), C.byref(r)))
        return r.value

    def set_mode(self, mode=0, default_prec=PREC_FP32, tol=1e-12, max_iter=10):
        self._check(self.L.uhm_gpu_set_mode(C.byref(self.h), mode, default_prec, tol, max_iter))

    def set_front_precision(self, prec_by_element_id):
        a, p = _arr(prec_by_element_id, np.int32, _i)
        self._check(self.L.uhm_gpu_set_front_precision(C.byref(self.h), len(a), p))

    def first_backward_error(self) -> float:
        out = (_d * 9)()
        self.L.uhm_gpu_get_timing(C.byref(self.h), out)
        return out[8]

    def timing(self) -> dict:
        out = (_d * 9)()
        self.L.uhm_gpu_get_timing(C.byref(self.h), out)
        keys = ["upload_ms", "factor_ms", "solve_ms", "refine_ms", "total_ms", "ir_iters",
                "berr", "kernel_launches", "berr_first"]
        return dict(zip(keys, list(out)))

    OP_NAMES = ["assemble", "small_factor", "potrf_diag", "trsm_panel", "syrk_update",
                "getrf_panel", "lu_row_update", "gemm_update", "fwd_gather", "fwd_small",
                "trsv_fwd_step", "gemv_fwd", "bwd_prepare", "bwd_small", "gemv_bwd", "trsv_bwd_step",
                "bwd_store", "tc_pack", "tc_syrk_bf16", "fwd_flags", "bwd_flags", "getrf_coop",
                "laswp", "potrf_trsm", "assemble_scatter", "tc_gemm_bf16", "chol_panel", "tc_chol_trail",
                "tc_chol_schur", "clear_flags", "chol_diag", "chol_pack", "tc_chol_trsm", "event_record",
                "event_wait", "fwd_chain", "bwd_chain"] + [f"op{k}" for k in range(37, 40)]

    def set_profiling(self, on=True):
        self._check(self.L.uhm_gpu_set_profiling(C.byref(self.h), int(on)))

    def profile(self) -> dict:
        n = len(self.OP_NAMES)
        ms, fl, by = (_d * n)(), (_d * n)(), (_d * n)()
        la = (_l * n)()
        self._check(self.L.uhm_gpu_get_profile(C.byref(self.h), n, ms, fl, by, la))
        return {self.OP_NAMES[k]: dict(ms=ms[k], flops=fl[k], bytes=by[k], launches=la[k])
                for k in range(n) if la[k]}

    def get_n_dof(self) -> int:
        n = _i(0)
        self.L.uhm_get_n_dof_(C.byref(self.h), C.byref(n))
        return n.value

    def estimate_cost(self, method, n_rhs=1):
        fd, fs, buf = _d(0), _d(0), _d(0)
        nnz = C.c_uint(0)
        self.L.uhm_estimate_cost_(C.byref(self.h), _ip(method), _ip(UHM_REAL), _ip(n_rhs),
                                  C.byref(fd), C.byref(fs), C.byref(nnz), C.byref(buf))
        return fd.value, fs.value

    # -- structure ------------------------------------------------------------
    def fronts(self):
        n = _i(0)
        self.L.uhm_gpu_get_n_fronts(C.byref(self.h), C.byref(n))
        self._check()
        n = n.value
        eid, gen, fs, ss = (np.zeros(n, np.int32) for _ in range(4))
        self.L.uhm_gpu_get_fronts(C.byref(self.h), n, eid.ctypes.data_as(_P(_i)),
                                  gen.ctypes.data_as(_P(_i)), fs.ctypes.data_as(_P(_i)),
                                  ss.ctypes.data_as(_P(_i)))
        return eid, gen, fs, ss

    FRONT_BLOCKS = {"ATL": 1, "ATR": 2, "ABL": 3, "ABR": 4, "P": 5, "XT": 7, "XB": 8}

    def front_block(self, elt_id, name):
        """One block of a front (uhm_gpu_get_front_block), column-major as a
        numpy array; P as int32 pivots."""
        eid, _, fs, ss = self.fronts()
        k = int(np.nonzero(eid == elt_id)[0][0])
        f, s_ = int(fs[k]), int(ss[k])
        dims = {"ATL": (f, f), "ATR": (f, s_), "ABL": (s_, f), "ABR": (s_, s_), "P": (f, 1),
                "XT": (f, self.n_rhs), "XB": (s_, self.n_rhs)}[name]
        out = np.zeros(dims[0] * dims[1], np.int32 if name == "P" else np.float64)
        self._check(self.L.uhm_gpu_get_front_block(C.byref(self.h), int(elt_id), self.FRONT_BLOCKS[name],
                                                   dims[0], dims[1], out.ctypes.data_as(C.c_void_p)))
        return out if name == "P" else out.reshape(dims[1], dims[0]).T

    def front_nodes(self, elt_id, cap=1 << 20):
        ids = np.zeros(cap, np.int32)
        nf, ns = _i(0), _i(0)
        self._check(self.L.uhm_gpu_get_front_nodes(C.byref(self.h), elt_id, cap,
                                                   ids.ctypes.data_as(_P(_i)), C.byref(nf), C.byref(ns)))
        return ids[:nf.value], ids[nf.value:nf.value + ns.value]

    def op_log(self, cap=1 << 16):
        """Profiled launches in order: list of (op name, items, ms)."""
        kind, items = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        ms = np.zeros(cap, np.float64)
        n = _i(0)
        self._check(self.L.uhm_gpu_get_op_log(C.byref(self.h), cap, kind.ctypes.data_as(_P(_i)),
                                              items.ctypes.data_as(_P(_i)), ms.ctypes.data_as(_P(_d)), C.byref(n)))
        k = min(n.value, cap)
        return [(self.OP_NAMES[kind[i]], int(items[i]), float(ms[i])) for i in range(k)]

    # -- learned precision selector ------------------------------------------
    # -- element matrices generated on the device -------------------------------
    def generate_elements(self, recipe, method=UHM_CHOL):
        """Build every leaf's element matrix on the device from
        hpfem.element_recipe(spec) (uhm_gpu_generate_lobatto_elements)
        instead of copying it in; the element node lists must be known (a
        bulk copy_in_leaves with node lists, e.g. of the right-hand sides)."""
        r = recipe
        keep = []

        def ptr(a, dt, ct):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data_as(_P(ct))
        self._check(self.L.uhm_gpu_generate_lobatto_elements(
            C.byref(self.h), method, r["dim"], r["hh"], r["cmass"], r["cconv"], r["n_el"],
            ptr(r["ref"], np.float64, _d), ptr(r["ref_off"], np.int64, _l), len(r["ref_off"]),
            ptr(r["p_el"], np.int32, _i), ptr(r["kappa"], np.float64, _d), ptr(r["react"], np.float64, _d),
            ptr(r["beta"], np.float64, _d), ptr(r["sel_ptr"], np.int64, _l), ptr(r["sel"], np.int32, _i)))

    # -- kernel-selection thresholds --------------------------------------------
    TUNABLES = ("small_max_f64", "small_max_f32", "tc_min_n", "gc_min_rows", "fuse_potrf_trsm", "tc_nbo",
                "tc_panel", "solve_rows", "lookahead", "solve_chain")

    def tunables(self) -> dict:
        v = np.zeros(len(self.TUNABLES), np.int32)
        self._check(self.L.uhm_gpu_get_tunables(C.byref(self.h), v.ctypes.data_as(_P(_i))))
        return dict(zip(self.TUNABLES, v.tolist()))

    def set_tunables(self, **kw):
        cur = self.tunables()
        cur.update(kw)
        v = np.asarray([cur[k] for k in self.TUNABLES], np.int32)
        self._check(self.L.uhm_gpu_set_tunables(C.byref(self.h), v.ctypes.data_as(_P(_i))))

    def autotune(self, method=UHM_CHOL, reps=2) -> dict:
        """Time candidate thresholds on this mesh and keep the fastest
        (uhm_gpu_autotune); returns the chosen values and the number of
        candidates timed."""
        n = _i(0)
        self._check(self.L.uhm_gpu_autotune(C.byref(self.h), method, reps, C.byref(n)))
        return dict(self.tunables(), timed=n.value)

    def set_selector(self, params):
        a, p = _arr(params, np.float32, C.c_float)
        self._check(self.L.uhm_gpu_set_selector(C.byref(self.h), p, len(a)))

    def front_features(self, method=UHM_CHOL):
        """Selector features per front, in the order of fronts()."""
        n = len(self.fronts()[0])
        out = np.zeros((n, mlp_n_features()), np.float32)
        self._check(self.L.uhm_gpu_get_front_features(C.byref(self.h), method, n,
                                                      out.ctypes.data_as(_P(C.c_float))))
        return out

    def front_precision(self):
        """(precision of each front in the last plan, selector class or -1)."""
        n = len(self.fronts()[0])
        prec, cls = np.zeros(n, np.int32), np.zeros(n, np.int32)
        self._check(self.L.uhm_gpu_get_front_precision(C.byref(self.h), n, prec.ctypes.data_as(_P(_i)),
                                                       cls.ctypes.data_as(_P(_i))))
        return prec, cls

    def node_solution(self, node_ids, ndof, n_rhs=1):
        ids, p = _arr(node_ids, np.int32, _i)
        rows = int(np.asarray(ndof)[ids].sum())
        out = np.zeros((rows, n_rhs), order="F")
        self._check(self.L.uhm_gpu_get_node_solution(C.byref(self.h), len(ids), p,
                                                     out.ctypes.data_as(_P(_d)), rows * n_rhs))
        return out

    # -- bulk ------------------------------------------------------------------
    def copy_in_leaves(self, side, buf, nods_all=None):
        buf = np.ascontiguousarray(buf, dtype=np.float64)
        np_ = None
        if nods_all is not None:
            nods_all, np_ = _arr(nods_all, np.int32, _i)
        self._check(self.L.uhm_gpu_copy_in_leaves(C.byref(self.h), side, np_,
                                                  buf.ctypes.data_as(_P(_d)), buf.size))

    def copy_out_leaves(self, n_values, out=None):
        if out is None:
            out = np.zeros(n_values)
        self._check(self.L.uhm_gpu_copy_out_leaves(C.byref(self.h), out.ctypes.data_as(_P(_d)),
                                                   n_values))
        return out


def set_wait_limit(iters: int) -> None:
    """Iteration limit of every bounded wait inside the device kernels
    (uhm_gpu_set_wait_limit); iters < 0 restores the defaults."""
    rc = lib().uhm_gpu_set_wait_limit(int(iters))
    if rc:
        raise UHMError(rc, "uhm_gpu_set_wait_limit failed")


def pinned_empty(n: int, dtype=np.float64):
    """numpy array backed by page-locked host memory (freed with the array)."""
    L = lib()
    nbytes = int(n) * np.dtype(dtype).itemsize
    ptr = L.uhm_gpu_host_alloc(max(nbytes, 16))
    if not ptr:
        raise MemoryError("uhm_gpu_host_alloc failed")
    buf = (C.c_char * nbytes).from_address(ptr)
    arr = np.frombuffer(buf, dtype=dtype, count=n)

    class _Owner:
        def __del__(self_inner):
            L.uhm_gpu_host_free(C.c_void_p(ptr))
    arr_owner = _Owner()
    arr = arr.view()
    arr.flags.writeable = True
    _keep[id(arr)] = arr_owner
    return arr


_keep = {}


def mlp_n_params() -> int:
    return int(lib().uhm_gpu_mlp_n_params())


def mlp_n_features() -> int:
    return int(lib().uhm_gpu_mlp_n_features())


def _mlp_check(code):
    if code:
        raise UHMError(code, "selector network call failed")


def mlp_predict(X, params):
    """Selector classes and probabilities for samples X (N x 12), on the device."""
    X, px = _arr(X, np.float32, C.c_float)
    P, pp = _arr(params, np.float32, C.c_float)
    n = X.shape[0]
    cls = np.zeros(n, np.int32)
    prob = np.zeros((n, 3), np.float32)
    _mlp_check(lib().uhm_gpu_mlp_predict(px, n, pp, cls.ctypes.data_as(_P(_i)), prob.ctypes.data_as(_P(C.c_float))))
    return cls, prob


def mlp_gradient(X, y, params, class_weight=None):
    """(loss, gradient) of the class-weighted mean cross-entropy over all samples."""
    X, px = _arr(X, np.float32, C.c_float)
    y, py = _arr(y, np.int32, _i)
    P, pp = _arr(params, np.float32, C.c_float)
    w = None if class_weight is None else np.ascontiguousarray(class_weight, np.float32)
    pw = None if w is None else w.ctypes.data_as(_P(C.c_float))
    g = np.zeros(mlp_n_params(), np.float32)
    loss = np.zeros(1, np.float32)
    _mlp_check(lib().uhm_gpu_mlp_gradient(px, py, pw, X.shape[0], pp, g.ctypes.data_as(_P(C.c_float)),
                                          loss.ctypes.data_as(_P(C.c_float))))
    return float(loss[0]), g


def mlp_train(X, y, params, epochs=20, batch=512, lr=1e-3, seed=0, class_weight=None):
    """Adam on the device; returns (trained parameters, mean loss per epoch)."""
    X, px = _arr(X, np.float32, C.c_float)
    y, py = _arr(y, np.int32, _i)
    P = np.array(params, dtype=np.float32, copy=True)
    w = None if class_weight is None else np.ascontiguousarray(class_weight, np.float32)
    pw = None if w is None else w.ctypes.data_as(_P(C.c_float))
    hist = np.zeros(max(1, epochs), np.float32)
    _mlp_check(lib().uhm_gpu_mlp_train(px, py, pw, X.shape[0], P.ctypes.data_as(_P(C.c_float)), epochs, batch,
                                       float(lr), int(seed), hist.ctypes.data_as(_P(C.c_float))))
    return P, hist[:epochs]


def load_spec(spec, n_rhs=None, bulk=True, pinned=False, lhs=True):
    """Feed a uhm_gb300.hpfem.MeshSpec through the Mesh API: nodes, leaf
    elements (add_element + element_add_node), the tree through
    add_element(gen) / set_parent / add_child, lock,
    create_matrix_without_buffer, copy_in of every element matrix and rhs."""
    n_rhs = spec.n_rhs if n_rhs is None else n_rhs
    m = Mesh()
    nods = {}
    for nid, nd, p in zip(spec.node_id.tolist(), spec.node_ndof.tolist(), spec.node_p.tolist()):
        nods[nid] = m.add_node(nid, nd, p)
    elts = []
    gen = spec.generation.tolist()
    for e in range(spec.n_elements):
        elts.append(m.add_element(gen[e]))
    for e in range(spec.n_leaves):
        for nid in spec.element_nodes(e).tolist():
            m.element_add_node(elts[e], nods[nid])
    for e in range(spec.n_elements):
        for c in spec.children(e).tolist():
            m.set_parent(elts[c], elts[e])
            m.add_child(elts[e], elts[c])
    m.lock()
    m.create_matrix_without_buffer(UHM_REAL, n_rhs)
    m._elts = elts
    if not lhs:
        # right-hand sides (and the element node lists) only: the element
        # matrices come from the device generator (generate_elements)
        m.copy_in_leaves(UHM_RHS, spec.rhs, spec.elem_node.astype(np.int32))
    elif bulk:
        nods_all = spec.elem_node.astype(np.int32)
        m.copy_in_leaves(UHM_LHS, spec.mats, nods_all)
        m.copy_in_leaves(UHM_RHS, spec.rhs)
    else:
        for e in range(spec.n_leaves):
            nl = spec.element_nodes(e)
            m.copy_in(elts[e], nl, UHM_LHS, spec.element_matrix(e))
            m.copy_in(elts[e], nl, UHM_RHS, spec.element_rhs(e))
    return m
