"""The device element generator's recipe and arithmetic, on the CPU.

hpfem.element_recipe(spec) feeds uhm_gpu_generate_lobatto_elements.  A numpy
restatement of the two device passes (k_gen_tables: per order, the
element-independent factors over all mode pairs; k_gen_lobatto: the
per-element coefficients times table entries; the same products and sums in
the same order, elementwise, no fused multiply-add) must rebuild the host generator's matrices bit for bit from the recipe alone,
and the C ABI must reject recipes whose indices would leave the tensor grid
or the element's size before it touches the device."""
import numpy as np
import pytest

from uhm_gb300 import api, hpfem


def _tables(R, q, dim, hh, cm, cc, has_react, has_beta):
    """k_gen_tables: per order, the element-independent factors over all
    pairs (ga, gb) of tensor-grid modes, ga fastest, table after table."""
    G = q ** 3 if dim == 3 else q ** 2
    i = np.arange(G * G)
    ga, gb = i % G, i // G
    xa = (ga % q) * q + gb % q
    ya = ((ga // q) % q) * q + (gb // q) % q
    za = (ga // (q * q)) * q + gb // (q * q)
    M, K, Cv = R[:q * q], R[q * q:2 * q * q], R[2 * q * q:3 * q * q]
    t = []
    if dim == 3:
        t1 = M[za] * (M[ya] * K[xa])
        t2 = M[za] * (K[ya] * M[xa])
        t3 = K[za] * (M[ya] * M[xa])
        t.append(hh * ((t1 + t2) + t3))
        if has_react:
            t.append(cm * (M[za] * (M[ya] * M[xa])))
        if has_beta:
            t += [cc * (M[za] * (M[ya] * Cv[xa])), cc * (M[za] * (Cv[ya] * M[xa])),
                  cc * (Cv[za] * (M[ya] * M[xa]))]
    else:
        t.append(M[ya] * K[xa] + K[ya] * M[xa])
        if has_react:
            t.append(cm * (M[ya] * M[xa]))
        if has_beta:
            t += [cc * (M[ya] * Cv[xa]), cc * (Cv[ya] * M[xa])]
    return np.concatenate(t), G


def _generate(r):
    """k_gen_lobatto: entry (a, b) = kappa S[k] [+ react Rm[k]] [+ beta_d C_d[k]],
    k = sel_a + sel_b G."""
    dim = r["dim"]
    has_react, has_beta = r["react"] is not None, r["beta"] is not None
    tabs = {}
    for p in sorted(set(r["p_el"].tolist())):
        q, o = p + 1, int(r["ref_off"][p])
        tabs[p] = _tables(r["ref"][o:o + 3 * q * q], q, dim, r["hh"], r["cmass"], r["cconv"],
                          has_react, has_beta)
    out = []
    for e in range(r["n_el"]):
        T, G = tabs[int(r["p_el"][e])]
        GG = G * G
        s = r["sel"][r["sel_ptr"][e]:r["sel_ptr"][e + 1]].astype(np.int64)
        k = s[:, None] + s[None, :] * G
        v = r["kappa"][e] * T[:GG][k]
        rea = r["react"][e] if has_react else 0.0
        if rea != 0.0:
            v = v + rea * T[GG:2 * GG][k]
        if has_beta:
            c0 = 2 * GG if has_react else GG
            for d in range(dim):
                v = v + r["beta"][d] * T[c0 + d * GG:c0 + (d + 1) * GG][k]
        out.append(v.reshape(-1, order="F"))
    return np.concatenate(out)


CASES = [
    ("diff3d", lambda: hpfem.diffusion3d(3, 3, seed=61, contrast=1e3)),
    ("convdiff3d", lambda: hpfem.convdiff3d(3, 2, seed=62)),
    ("poisson2d", lambda: hpfem.poisson2d(6, 4, seed=63)),
    ("varp3d", lambda: hpfem.build_mesh(3, 2, [2, 3, 2, 4, 3, 2, 2, 3], seed=64)),
    ("react3d", lambda: hpfem.build_mesh(3, 2, 3, react=-2.5, seed=65)),
    ("convreact2d", lambda: hpfem.build_mesh(2, 5, 3, beta=(30.0, -20.0), react=0.5, seed=67)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_recipe_rebuilds_host_matrices_bitwise(name, make):
    spec = make()
    got = _generate(hpfem.element_recipe(spec))
    assert got.shape == spec.mats.shape
    assert np.array_equal(got, spec.mats)


def test_recipe_requires_build_mesh():
    spec = hpfem.poisson3d(2, 2, seed=1)
    spec.info.pop("recipe")
    with pytest.raises(ValueError):
        hpfem.element_recipe(spec)


def _bad(mutate):
    spec = hpfem.poisson3d(2, 3, seed=66)
    r = hpfem.element_recipe(spec)
    mutate(r, spec)
    m = api.load_spec(spec, lhs=False)
    with pytest.raises(api.UHMError) as ei:
        m.generate_elements(r)
    assert ei.value.code == 7


def test_rejects_mode_outside_grid(native_lib):
    def f(r, spec):
        r["sel"] = r["sel"].copy(); r["sel"][5] = 4 ** 3     # p=3: modes 0..63
    _bad(f)


def test_rejects_order_outside_range(native_lib):
    def f(r, spec):
        r["p_el"] = r["p_el"].copy(); r["p_el"][0] = 8
    _bad(f)


def test_rejects_wrong_element_count(native_lib):
    def f(r, spec):
        r["n_el"] = r["n_el"] - 1
    _bad(f)


def test_rejects_mode_count_mismatch(native_lib):
    other = hpfem.element_recipe(hpfem.poisson3d(2, 2, seed=66))

    def f(r, spec):
        r.update(other)
    _bad(f)
