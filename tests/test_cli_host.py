"""The command-line driver on the CPU: upstream's flags and defaults, the restricted h0
reader, and the Hamiltonian assembled from upstream's NiO 50-bath h0 file equal to the one
upstream's own run produced (its shipped data.npz)."""

import ast
import pickle
from collections import OrderedDict

import numpy as np
import pytest

from impuritymodel_gb300 import get_spectra as G
from tests.golden.fixtures import decode_op, load

# upstream get_spectra.py:427-618: flag -> default
UPSTREAM_DEFAULTS = {
    "ls": [1, 2], "nBaths": [0, 10], "nValBaths": [0, 10], "n0imps": [6, 8], "dnTols": [0, 2], "dnValBaths": [0, 2],
    "dnConBaths": [0, 0], "Fdd": [7.5, 0, 9.9, 0, 6.6], "Fpp": [0.0, 0.0, 0.0], "Fpd": [8.9, 0, 6.8],
    "Gpd": [0.0, 5.0, 0, 2.8], "xi_2p": 11.629, "xi_3d": 0.096, "chargeTransferCorrection": 1.5,
    "hField": [0, 0, 0.0001], "nPsiMax": 5, "nPrintSlaterWeights": 3, "tolPrintOccupation": 0.5, "T": 300,
    "energy_cut": 10, "delta": 0.2, "deltaRIXS": 0.05, "deltaNIXS": 0.1,
}


def write_h0(path):
    """Upstream's NiO 50-bath h0 operator (from the fixture) as a plain-dict pickle."""
    z = load("nio50_cli.npz")
    h0 = {ast.literal_eval(k): complex(v) for k, v in zip(z["h0_keys"], z["h0_vals"])}
    with open(path, "wb") as fh:
        pickle.dump(h0, fh)
    return h0


def test_flags_and_defaults_match_upstream():
    args = vars(G.parser().parse_args(["h0.pickle", "radial.dat"]))
    assert args.pop("h0_filename") == "h0.pickle" and args.pop("radial_filename") == "radial.dat"
    assert args == UPSTREAM_DEFAULTS


def test_hamiltonian_from_upstream_h0_equals_upstream_run(tmp_path):
    h0_file = tmp_path / "h0.pickle"
    write_h0(h0_file)
    nb = OrderedDict([(1, 0), (2, 50)])
    hop = G.get_hamiltonian_operator(nb, OrderedDict([(1, 0), (2, 50)]),
                                     [UPSTREAM_DEFAULTS[k] for k in ("Fdd", "Fpp", "Fpd", "Gpd")],
                                     [UPSTREAM_DEFAULTS["xi_2p"], UPSTREAM_DEFAULTS["xi_3d"]],
                                     [OrderedDict([(1, 6), (2, 8)]), 1.5], UPSTREAM_DEFAULTS["hField"], str(h0_file))
    ref = decode_op(load("nio50.npz"), "hop")
    assert len(hop) == len(ref) == 1132
    assert set(hop) == set(ref)
    assert max(abs(complex(hop[k]) - complex(ref[k])) for k in ref) < 1e-12


def test_restricted_unpickler_refuses_other_objects(tmp_path):
    bad = tmp_path / "bad.pickle"
    with open(bad, "wb") as fh:
        pickle.dump({"x": pytest.approx}, fh)
    with pytest.raises(pickle.UnpicklingError):
        G.read_pickled_file(str(bad))


def test_popcount64_matches_python():
    """The SWAR bit count used to check restrictions on host words."""
    from impuritymodel_gb300.spectra import _popcount64

    rng = np.random.default_rng(3)
    x = rng.integers(0, 2**63, size=500, dtype=np.int64).astype(np.uint64) * np.uint64(2) + np.uint64(1)
    x[:3] = [0, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64(1) << np.uint64(63)]
    assert np.array_equal(_popcount64(x), [bin(int(v)).count("1") for v in x])


def test_device_op_cache_follows_in_place_edits():
    """The compiled operator is reused for the same dict and content only: changing a
    coefficient, adding or removing a term in place recompiles it (upstream code may edit an
    operator dict between calls)."""
    import types

    from impuritymodel_gb300 import finite, models

    op = dict(models.make_model("config1").hOp)
    eng = types.SimpleNamespace(device="cpu", h2d_bytes=0)
    d1 = finite._device_op(op, eng)
    assert finite._device_op(op, eng) is d1
    key = next(iter(op))
    op[key] = op[key] + 0.5
    d2 = finite._device_op(op, eng)
    assert d2 is not d1 and d2.coeff[0, 0].item() == d1.coeff[0, 0].item() + 0.5
    del op[key]
    d3 = finite._device_op(op, eng)
    assert d3.n_terms == d1.n_terms - 1
    new_key = next(k for k in (((i, "c"), (j, "a")) for i in range(26) for j in range(26)) if k not in op)
    op[new_key] = 1.0
    assert finite._device_op(op, eng).n_terms == d1.n_terms
