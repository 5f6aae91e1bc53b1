"""Host logic of the large-sector row order (CPU tensors, no GPU): CsrMatrix.permuted is
P H P^T with each row's entries in their stored order, and locality_order sorts by the non-lead
orbitals first and the lead orbitals last."""

import numpy as np
import torch

from impuritymodel_gb300.engine import CsrMatrix
from impuritymodel_gb300.large import locality_order


def _random_csr(n, rng, complex_=False):
    dense = np.where(rng.random((n, n)) < 0.2, rng.standard_normal((n, n)), 0.0)
    rows, cols = np.nonzero(dense)
    # a row's entries in a scrambled (non-sorted) order, as the term order may leave them
    order = np.lexsort((rng.random(rows.size), rows))
    rows, cols = rows[order], cols[order]
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    v = dense[rows, cols]
    if complex_:
        val = torch.from_numpy(np.stack([v, 0.5 * v], 1))
        return CsrMatrix(torch.from_numpy(rp), torch.from_numpy(cols.astype(np.int32)), val_c=val), dense * (1 + 0.5j)
    return CsrMatrix(torch.from_numpy(rp), torch.from_numpy(cols.astype(np.int32)), val_r=torch.from_numpy(v)), dense


def _dense(csr):
    n = csr.n
    out = np.zeros((n, n), dtype=np.complex128)
    rp, col = csr.row_ptr.numpy(), csr.col.numpy()
    val = csr.val_r.numpy() if csr.val_r is not None else csr.val_c.numpy() @ np.array([1, 1j])
    for i in range(n):
        for e in range(rp[i], rp[i + 1]):
            out[i, col[e]] += val[e]
    return out


def test_permuted_is_pap():
    rng = np.random.default_rng(0)
    for complex_ in (False, True):
        csr, dense = _random_csr(40, rng, complex_)
        perm = torch.from_numpy(rng.permutation(40))
        p = csr.permuted(perm)
        pn = perm.numpy()
        assert np.allclose(_dense(p), dense[np.ix_(pn, pn)], rtol=0, atol=0)
        # every new row holds its old row's entries in the stored order
        for k in range(40):
            old = pn[k]
            a, b = int(csr.row_ptr[old]), int(csr.row_ptr[old + 1])
            c, d = int(p.row_ptr[k]), int(p.row_ptr[k + 1])
            inv = np.argsort(pn)
            assert np.array_equal(p.col[c:d].numpy(), inv[csr.col[a:b].numpy()])


class _Op:
    def __init__(self, moves):
        self.moves = np.asarray(moves)


def _words(states, n_orb):
    w = (n_orb + 63) // 64
    out = np.zeros((len(states), w), dtype=np.uint64)
    for k, occ in enumerate(states):
        for o in occ:
            out[k, o // 64] |= np.uint64(1) << np.uint64(63 - o % 64)
    return out


def test_locality_order_blocks_by_non_lead_orbitals():
    rng = np.random.default_rng(1)
    n_orb = 70  # two words; lead orbitals 0..3 and 66 (one in each word)
    lead = [0, 1, 2, 3, 66]
    moves = np.full(n_orb, 2)
    moves[lead] = 50
    states = sorted({tuple(sorted(rng.choice(n_orb, 6, replace=False).tolist())) for _ in range(300)})
    words = _words(states, n_orb)
    # the sorted basis as the engine keeps it (unsigned lexicographic)
    srt = np.lexsort(words.T[::-1])
    words = words[srt]
    basis = torch.from_numpy(words.view(np.int64))
    perm = locality_order(basis, _Op(moves)).numpy()
    assert sorted(perm.tolist()) == list(range(len(words)))
    mask = _words([lead], n_orb)[0]
    key = [tuple((r & ~mask).tolist()) + tuple((r & mask).tolist()) for r in words[perm]]
    assert key == sorted(key)
    # no orbital stands out: the sorted order is kept
    assert locality_order(basis, _Op(np.full(n_orb, 3))) is None


def test_combination_masks_follow_itertools_order():
    import itertools

    from impuritymodel_gb300.finite import _combination_masks

    for m in range(0, 9):
        idx = list(range(3, 3 + m))
        for k in range(0, m + 2):
            cs = list(itertools.combinations(idx, k))
            ref = np.zeros((len(cs), 16), dtype=bool)
            for i, c in enumerate(cs):
                ref[i, list(c)] = True
            got = _combination_masks(idx, k, 16)
            assert got.shape == ref.shape and (got == ref).all(), (m, k)


def test_get_basis_equals_upstream_order():
    """The bit-mask basis enumeration gives upstream's basis in upstream's order (the oracle
    restates upstream's itertools loops), for the 26- and 316-spin-orbital models and random
    models."""
    import oracle.ed_oracle as O
    from impuritymodel_gb300 import finite, models

    for mod in [models.make_model("config1"), models.make_model("config4")] + [
            models.random_model(s, 1 + s % 5) for s in range(4)]:
        args = mod.basis_args()
        assert finite.get_basis(*args) == tuple(O.get_basis(*args))
