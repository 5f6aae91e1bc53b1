"""Host-side drop-in functions against upstream's own outputs (no GPU): ``finite.get_basis``
(upstream finite.py:294-374) for the 26- and 66-spin-orbital models, state for state and in
upstream's order, and ``finite.get_hamiltonian_matrix_from_h_dict`` (finite.py:1613-1693) on
the h_dict that upstream's expand_basis filled, entry for entry (fixtures written by
tests/golden/make_golden.py from upstream itself)."""

import numpy as np

from impuritymodel_gb300 import finite
from impuritymodel_gb300 import models as M
from tests.golden.fixtures import decode_states, load


def test_get_basis_matches_upstream_26_orbitals():
    mod = M.make_model("config1")
    z = load("config1.npz")
    basis = finite.get_basis(*mod.basis_args())
    assert isinstance(basis, tuple)
    assert list(basis) == decode_states(z["basis"], mod.n_spin_orbitals)


def test_get_basis_matches_upstream_66_orbitals():
    mod = M.make_model("config2")
    z = load("dropin.npz")
    basis = finite.get_basis(*mod.basis_args())
    ref = decode_states(z["basis2"], mod.n_spin_orbitals)
    assert len(basis) == len(ref) == 1770
    assert list(basis) == ref


def _h_dict(z, n):
    keys = decode_states(z["hd_keys"], n)
    outs = decode_states(z["hd_out"], n)
    ptr = z["hd_ptr"]
    vals = z["hd_val"]
    return {k: {outs[e]: complex(vals[e]) for e in range(ptr[i], ptr[i + 1])} for i, k in enumerate(keys)}


def test_hamiltonian_from_h_dict_matches_upstream():
    n = M.make_model("config1").n_spin_orbitals
    z = load("dropin.npz")
    h_dict = _h_dict(z, n)
    basis = tuple(decode_states(z["hd_basis"], n))
    h, index = finite.get_hamiltonian_matrix_from_h_dict(h_dict, basis)
    assert index == {b: i for i, b in enumerate(basis)}
    got = h.tocoo()
    ref = {(int(r), int(c)): v for r, c, v in zip(z["hd_row"], z["hd_col"], z["hd_h"])}
    mine = {(int(r), int(c)): v for r, c, v in zip(got.row, got.col, got.data)}
    assert set(mine) == set(ref)
    assert all(mine[k] == ref[k] for k in ref)
    dense, index2 = finite.get_hamiltonian_matrix_from_h_dict(h_dict, basis, mode="dense")
    assert index2 == index
    assert np.array_equal(dense, h.toarray())


def test_hamiltonian_from_h_dict_errors_like_upstream():
    import pytest

    with pytest.raises(Exception, match="Wrong input parameters"):
        finite.get_hamiltonian_matrix_from_h_dict({}, (), mode="csc")
