"""Pruning inside basis expansion: the ground-state basis of a held-out model grown from its
lowest configurations, each breadth-first layer's new states ranked by the trained network and
only the best fraction kept (the states a layer drops are not offered again).  The full
expansion equals upstream's restricted basis (the judge); the energy error of the pruned basis
is non-negative (variational), shrinks as more is kept, and is smaller with the network's
ranking than with a random ranking of the same layers at the same fraction."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_pruned_expansion_against_full_and_random(eng):
    from impuritymodel_gb300 import codec, finite, pruning
    from impuritymodel_gb300 import models as M
    from impuritymodel_gb300.engine import make_restrictions

    train = [M.random_model(1000 + s, 1 + s % 3) for s in range(40)]
    st, lw = pruning.ground_state_samples(eng, train)
    net = pruning.BasisNet(eng, seed=0, lr=2e-3)
    net.train(st, lw, epochs=30, batch=512)
    held = M.random_model(2000, 3)
    n = held.n_spin_orbitals
    keeps = [0.5, 0.75, 0.9, 1.0]
    res, full = pruning.evaluate_expansion_pruning(eng, held, net, keeps)
    # the full expansion of the seed is upstream's restricted basis, as a set
    basis = finite.get_basis(*held.basis_args())
    assert full["n"] == len(basis)
    assert res[1.0]["error"] == 0.0 and res[1.0]["n"] == full["n"]
    errs = [res[k]["error"] for k in keeps]
    assert all(e >= -1e-9 for e in errs), errs
    assert errs[0] >= errs[1] - 1e-9 >= errs[2] - 2e-9, errs
    assert res[0.5]["n"] < res[0.75]["n"] < res[0.9]["n"] < full["n"]
    r = res[0.75]
    # the same layers ranked at random keep more energy error
    dop = finite._device_op(held.hOp, eng)
    restr = make_restrictions(held.restrictions, n)
    b0 = eng.upload_states(codec.bytes_to_words(list(pruning.seed_basis(held)), n))
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    rnd = lambda s: torch.rand(s.shape[0], device=s.device, generator=gen, dtype=torch.float64)  # noqa: E731
    pr, _, _ = pruning.expand_pruned(eng, dop, restr, b0, rnd, 0.75)
    e_r, _ = finite.eig_lowest(eng, eng.build_csr(pr, dop, None), 1)
    assert e_r[0] - full["e"][0] > r["error"], (e_r[0] - full["e"][0], r)
    st_full = eng.sort_unique(eng.upload_states(codec.bytes_to_words(basis, n)))
    full_sorted, _, _ = pruning.expand_pruned(eng, dop, restr, b0)
    assert torch.equal(full_sorted, st_full)
