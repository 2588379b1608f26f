"""Factor-reuse flags on the host (Mesh_::backup / check_reuse,
UHM/src/mesh/mesh.cxx:113-225; Element_::set_reuse, element.cxx:75), no GPU.

check_reuse is restated here from the reference: every element starts
reusable; in element-id order an element is reusable when an element of its
id is in the backup with the same factor and schur nodes (same node, same
n_dof + p + kind, same order), and one that is not clears the flag on itself
and every ancestor -- which a later (higher-id) ancestor can set again from
its own comparison.  The native flags must equal the restatement's.  The
factorisation never relies on such a flag alone: it also requires every
child to be kept (test_gpu_reuse.py)."""
import numpy as np

from uhm_gb300 import api, hpfem


def _lists(m, spec, extra_val=None):
    """element id -> (factor nodes, schur nodes), each as (node id, n_dof + p + kind)."""
    val = {int(i): int(d) + int(p) + int(k) for i, d, p, k in
           zip(spec.node_id, spec.node_ndof, spec.node_p, spec.node_kind)}
    val.update(extra_val or {})
    eid, _, _, _ = m.fronts()
    out = {}
    for e in eid.tolist():
        f, s = m.front_nodes(e)
        out[e] = (tuple((int(i), val[int(i)]) for i in f), tuple((int(i), val[int(i)]) for i in s))
    return out


def _check_reuse(before, after, parent):
    flags = {e: True for e in after}
    for e in sorted(after):
        flags[e] = e in before and before[e] == after[e]
        if not flags[e]:
            u = e
            while u >= 0:
                flags[u] = False
                u = parent[u]
    return flags


def test_set_and_get_reuse(native_lib):
    spec = hpfem.poisson3d(2, 2, seed=1)
    m = api.load_spec(spec)
    assert not any(m.get_reuse(x) for x in m._elts)        # the reference's default: 0
    m.set_reuse(m._elts[3], True)
    assert m.get_reuse(m._elts[3]) and not m.get_reuse(m._elts[2])
    m.set_reuse(m._elts[3], False)
    assert not m.get_reuse(m._elts[3])


def test_unchanged_mesh_is_all_reusable(native_lib):
    spec = hpfem.poisson3d(3, 2, seed=2)
    m = api.load_spec(spec)
    b = api.Mesh()
    m.backup(b)
    m.check_reuse(b)
    assert all(m.get_reuse(x) for x in m._elts)


def test_flags_after_a_leaf_gains_a_node(native_lib):
    spec = hpfem.poisson3d(4, 2, seed=3)
    m = api.load_spec(spec)
    before = _lists(m, spec)
    b = api.Mesh()
    m.backup(b)
    m.unlock()
    nid = int(spec.node_id.max()) + 1
    m.element_add_node(m._elts[9], m.add_node(nid, 2, 1))
    m.lock()
    m.check_reuse(b)
    after = _lists(m, spec, {nid: 3})
    want = _check_reuse(before, after, spec.parent.tolist())
    got = {e: m.get_reuse(m._elts[e]) for e in after}
    assert got == want
    assert not got[9]
    assert sum(not v for v in got.values()) >= 1


def test_flags_against_an_empty_backup(native_lib):
    spec = hpfem.poisson3d(2, 2, seed=4)
    m = api.load_spec(spec)
    m.check_reuse(api.Mesh())
    assert not any(m.get_reuse(x) for x in m._elts)


def test_backup_rejects_itself(native_lib):
    m = api.load_spec(hpfem.poisson3d(2, 2, seed=5))
    try:
        m.backup(m)
    except api.UHMError as e:
        assert e.code != 0
    else:
        raise AssertionError("backup into the same mesh must fail")
