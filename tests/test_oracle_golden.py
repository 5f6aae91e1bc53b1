"""The CPU oracle pinned against upstream impurityModel outputs (no GPU).

Fixtures come from running upstream itself (``tests/golden/make_golden.py``); the NiO case
uses upstream's own shipped inputs (``data.npz``) and thermal spectrum (``XAS.dat``).
"""

import os

import numpy as np
import pytest

import oracle.ed_oracle as O
from impuritymodel_gb300 import codec
from impuritymodel_gb300 import models as M
from tests.golden.fixtures import decode_op, decode_psi, decode_restrictions, decode_states, load


@pytest.fixture(scope="module")
def c1():
    z = load("config1.npz")
    n = int(z["n_spin_orbitals"])
    return dict(z=z, n=n, hop=decode_op(z, "hop"), restr=decode_restrictions(z, "restr"),
                basis=tuple(decode_states(z["basis"], n)), es=z["es"],
                psis=[decode_psi(z, "eig%d" % i, n) for i in range(len(z["es"]))])


# --- known answers of upstream's unit tests, restated ---------------------------------


def test_codec_known_answer():
    # state (2, 5) among 7 spin-orbitals is "0010010", int 18, bytes b"$"
    # (upstream impurityModel/test/test_product_state_representation.py:55-60)
    assert O.tuple_to_bytes((2, 5), 7) == b"$"
    assert codec.tuple_to_bytes((2, 5), 7) == b"$"
    assert O.bytes_to_tuple(b"$", 7) == (2, 5)
    w = codec.bytes_to_words([b"$"], 7)
    assert int(w[0, 0]) == 0x24 << 56
    assert codec.words_to_bytes(w, 7) == [b"$"]


def test_sign_known_answers():
    # create at 3 in (2, 5): one electron below -> -1 (upstream test_create.py:52-70)
    v = int.from_bytes(O.tuple_to_bytes((2, 5), 7), "big")
    v2, s = O.create_sign(v, 3, 8)
    assert s == -1 and O.bytes_to_tuple(v2.to_bytes(1, "big"), 7) == (2, 3, 5)
    assert O.create_sign(v2, 3, 8)[1] == 0  # Pauli blocked
    # remove 3 from (2, 3, 5) -> -1, then remove 2 -> +1 (upstream test_remove.py:25-30)
    v3, s = O.remove_sign(v2, 3, 8)
    assert s == -1
    v4, s = O.remove_sign(v3, 2, 8)
    assert s == 1 and O.bytes_to_tuple(v4.to_bytes(1, "big"), 7) == (5,)
    assert O.remove_sign(v4, 2, 8)[1] == 0


def test_applyop_semantics_known_answers():
    # upstream test_applyOp.py: two creations sign 7*9*(2*(i<j)-1), equal final states merge,
    # restrictions block doubly occupied restricted sets
    n = 6
    vac = {O.tuple_to_bytes((), n): 7}
    for i in range(n):
        for j in range(n):
            out = O.apply_op(n, {((i, "c"), (j, "c")): 9}, vac)
            if i == j:
                assert out == {}
            else:
                assert out == {O.tuple_to_bytes(tuple(sorted((i, j))), n): 7 * 9 * (2 * (i < j) - 1)}
    psi = {O.tuple_to_bytes((1, 2), n): 7}
    out = O.apply_op(n, {((1, "c"), (1, "a")): 9, ((2, "c"), (2, "a")): 11}, psi)
    assert out == {O.tuple_to_bytes((1, 2), n): 7 * (9 + 11)}
    restr = {frozenset([1, 4, 5]): (0, 1)}
    out = O.apply_op(n, {((1, "c"), (4, "c")): 9}, vac, restrictions=restr)
    assert out == {}
    # a wrong result stored in opResult is used as is
    memo = {O.tuple_to_bytes((), n): {O.tuple_to_bytes(tuple(range(n)), n): 2}}
    out = O.apply_op(n, {((0, "c"),): 9}, vac, opResult=memo)
    assert out == {O.tuple_to_bytes(tuple(range(n)), n): 7 * 2}


# --- fixtures produced by upstream ----------------------------------------------------


def test_basis_matches_upstream(c1):
    mod = M.make_model("config1")
    assert O.get_basis(*mod.basis_args()) == c1["basis"]
    z2 = load("config2.npz")
    mod2 = M.make_model("config2")
    assert len(O.get_basis(*mod2.basis_args())) == int(z2["n_basis"])


def test_generator_reproduces_fixture_operator(c1):
    mod = M.make_model("config1")
    assert list(mod.hOp.keys()) == list(c1["hop"].keys())
    assert all(complex(mod.hOp[k]) == c1["hop"][k] for k in mod.hOp)
    assert M.dagger_op(mod.hOp) == mod.hOp


def test_gaunt_known_values():
    # upstream's convention (finite.gauntC): c^k = (-1)^m sqrt((2l+1)(2l'+1)) (l k l'; 0 0 0)
    # (l k l'; -m m-m' m'), so c^2(2 0; 2 0) = 5 * 2/35 = 2/7 and c^4(2 0; 2 0) = 2/7
    assert abs(M.gaunt_c(2, 2, 0, 2, 0) - 2.0 / 7.0) < 1e-15
    assert abs(M.gaunt_c(4, 2, 0, 2, 0) - 2.0 / 7.0) < 1e-15
    assert M.gaunt_c(1, 2, 0, 2, 0) == 0.0


def test_applyop_matches_upstream(c1):
    n = c1["n"]
    z = load("applyop_config1.npz")
    psi_in = decode_psi(z, "hpsi_in", n)
    out = O.apply_op(n, c1["hop"], psi_in, 1e-12, None, None)
    ref = decode_psi(z, "hpsi_out", n)
    assert list(out) == list(ref)
    assert all(out[s] == ref[s] for s in ref)
    out = O.apply_op(n, c1["hop"], psi_in, 1e-12, c1["restr"], None)
    assert out == decode_psi(z, "hpsi_restr_out", n)
    mod = M.make_model("config1")
    tops = mod.xas_ops()
    memo = {}
    for k, i in enumerate([0, 1, 2, 0]):
        psi = {s: complex(a) for s, a in c1["psis"][i].items()}
        out = O.apply_op(n, tops[k % 3], psi, 1e-7, c1["restr"], memo)
        assert out == decode_psi(z, "memo%d" % k, n)


def test_h_columns_vectorised_equals_dict_apply(c1):
    n = c1["n"]
    words = O.bytes_to_words(list(c1["basis"][:60]), n)
    colptr, out, val = O.h_columns(words, O.TermTable(c1["hop"]), O.restriction_masks(c1["restr"], n), 1e-12)
    outs = O.words_to_bytes(out, n)
    for j, b in enumerate(c1["basis"][:60]):
        ref = O.apply_op(n, c1["hop"], {b: 1}, 1e-12, c1["restr"])
        got = {outs[e]: val[e] for e in range(colptr[j], colptr[j + 1])}
        assert list(got) == list(ref)
        assert all(got[s] == ref[s] for s in ref)


def test_hamiltonian_bit_exact(c1):
    z = c1["z"]
    h = O.get_hamiltonian_matrix(c1["n"], c1["hop"], c1["basis"]).tocoo()
    ref = {(int(r), int(c)): v for r, c, v in zip(z["h_row"], z["h_col"], z["h_val"])}
    got = {(int(r), int(c)): v for r, c, v in zip(h.row, h.col, h.data)}
    assert set(ref) == set(got) and all(got[k] == ref[k] for k in ref)


def test_expand_and_lanczos_match_upstream(c1):
    z = c1["z"]
    n = c1["n"]
    psi1 = decode_psi(z, "psi1", n)
    b = O.expand_basis(n, None, c1["hop"], tuple(psi1.keys()), c1["restr"])
    assert b == tuple(decode_states(z["exp_basis"], n))
    h, idx = O.expand_basis_and_hamiltonian(n, None, c1["hop"], tuple(psi1.keys()), c1["restr"])
    nrm = np.sqrt(O.norm2(psi1))
    psi0 = np.zeros(len(idx), dtype=complex)
    for s, a in psi1.items():
        psi0[idx[s]] = a / nrm
    a, bb = O.get_tridiagonal_krylov_vectors(h, psi0, 150)
    assert np.abs(a[:20] - z["alpha"][:20]).max() < 1e-10
    assert np.abs(bb[:20] - z["beta"][:20]).max() < 1e-10


def test_eigensystem_matches_upstream(c1):
    es, _ = O.eigensystem(c1["n"], c1["hop"], c1["basis"], 3, groundDiagMode="full")
    assert np.abs(es - c1["es"]).max() < 1e-9


def test_xas_and_rixs_match_upstream(c1):
    z = c1["z"]
    mod = M.make_model("config1")
    gs = O.get_spectra(c1["n"], c1["hop"], mod.xas_ops(), c1["psis"], c1["es"], z["w"], 0.1, c1["restr"])
    assert np.abs(gs - z["gs_xas"]).max() <= 1e-6 * np.abs(z["gs_xas"]).max()
    g = O.get_rixs_map(c1["n"], c1["hop"], mod.xas_ops(), mod.rixs_out_ops(), c1["psis"][:1], c1["es"][:1],
                       z["w_in"], z["w_loss"], 0.2, 0.05, c1["restr"])
    assert np.abs(g - z["gs_rixs"]).max() <= 1e-6 * np.abs(z["gs_rixs"]).max()


def test_config2_ground_state_matches_upstream():
    z = load("config2.npz")
    mod = M.make_model("config2")
    n = mod.n_spin_orbitals
    basis = O.get_basis(*mod.basis_args())
    es, _ = O.eigensystem(n, mod.hOp, basis, 5, groundDiagMode="full")
    assert np.abs(es - z["es"]).max() < 1e-8


def test_nio_shipped_xas_dat():
    """Upstream's shipped NiO 50-bath run: E0 (output.txt) and the thermal XAS.dat."""
    z = load("nio50.npz")
    n = int(z["n_spin_orbitals"])
    hop = decode_op(z, "hop")
    restr = decode_restrictions(z, "restr")
    from collections import OrderedDict

    nb = OrderedDict([(1, 0), (2, 50)])
    basis = O.get_basis(nb, OrderedDict([(1, 0), (2, 50)]), OrderedDict([(1, 0), (2, 2)]),
                        OrderedDict([(1, 0), (2, 0)]), OrderedDict([(1, 0), (2, 2)]), OrderedDict([(1, 6), (2, 8)]))
    assert len(basis) == 1770
    es, psis = O.eigensystem(n, hop, basis, 5)
    assert abs(es[0] - (-903.8237)) < 5e-5
    keep = [i for i in range(len(es)) if es[i] - es[0] < 10 * O.K_B * 300]
    w = np.linspace(-25, 25, 3000)
    eps = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    tops = [M.dipole_op(nb, e) for e in eps]
    gs = O.get_spectra(n, hop, tops, [psis[i] for i in keep], es[: len(keep)], w, 0.2, restr)
    a = O.thermal_average(es[: len(keep)], -gs.imag, T=300)
    dat = z["xas_dat"]
    assert np.abs(dat[:, 0] - w).max() < 1e-4
    assert np.abs(a.sum(axis=0) - dat[:, 1]).max() < 1.5e-4  # "%8.4f" columns


def _dense(d, key):
    out = np.zeros((10, 10), dtype=complex)
    for k, v in d.items():
        out[key(k)] = v
    return out


@pytest.mark.parametrize("tag,cfg,fname", [("c1", "config1", "config1.npz")])
def test_observables_match_upstream(tag, cfg, fname):
    """3d observables (finite.py:843-1298) on upstream's eigenstates against upstream's own
    values (golden fixture observables.npz), 1e-12."""
    z = load("observables.npz")
    zc = load(fname)
    mod = M.make_model(cfg)
    n = int(zc["n_spin_orbitals"])
    nb = mod.nBaths
    for i in range(int(z[tag + "_n_states"])):
        psi = decode_psi(zc, "eig%d" % i, n)
        dm = _dense(O.density_matrix(nb, psi), lambda k: (k[0][1] * 5 + k[0][2] + 2, k[1][1] * 5 + k[1][2] + 2))
        assert np.abs(dm - z[tag + "_dm"][i]).max() < 1e-12
        dmc = _dense(O.density_matrix_cubic(nb, psi), lambda k: (k[0][0] * 5 + k[0][1], k[1][0] * 5 + k[1][1]))
        assert np.abs(dmc - z[tag + "_dm_cubic"][i]).max() < 1e-12
        vals = [O.trace_density_matrix(nb, psi), *np.real(O.eg_t2g_occupation(nb, psi)), O.lz3d(nb, psi),
                O.sz3d(nb, psi), O.lsqr3d(nb, psi), O.ssqr3d(nb, psi)]
        assert np.abs(np.array(vals) - z[tag + "_values"][i]).max() < 1e-11
    psi0 = decode_psi(zc, "eig0", n)
    for kind, name in (("Sz", "applySz3d"), ("Lz", "applyLz3d"), ("S+", "applySplus3d"), ("L+", "applyLplus3d"),
                       ("S-", "applySminus3d"), ("L-", "applyLminus3d")):
        ref = decode_psi(z, tag + "_" + name, n)
        got = O.apply_one_body_3d(nb, psi0, kind)
        keys = set(ref) | set(got)
        assert max(abs(ref.get(s, 0) - got.get(s, 0)) for s in keys) < 1e-13
