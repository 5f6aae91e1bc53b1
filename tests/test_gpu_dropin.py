"""Drop-in functions on the GPU against upstream's own outputs (tests/golden/dropin.npz):

* ``spectra.getGreen`` (upstream spectra.py:551-681) on a 60-state closure with Krylov size
  = dimension: the continued fraction at 1e-6 relative, and the caller's ``h_dict`` filled
  with the same states, in the same order, as upstream fills it;
* ``finite.eigensystem`` (finite.py:58-118) on a model whose spectrum is made of exactly
  degenerate spin triplets: every copy of each level is returned (energies against dense
  diagonalisation at 1e-8 eV; eigenvectors orthonormal with residuals at solver precision).
  Upstream's ARPACK call returns only two of the three copies of each triplet on this model
  (the fixture holds its output), so every upstream energy is one of ours, not the reverse.
"""

import numpy as np
import pytest

import oracle.ed_oracle as O
from impuritymodel_gb300 import finite, spectra
from impuritymodel_gb300 import models as M
from tests.golden.fixtures import decode_psi, decode_states, load

pytestmark = pytest.mark.gpu


def test_get_green_matches_upstream_and_fills_h_dict(eng):
    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    z1 = load("config1.npz")
    z = load("dropin.npz")
    psi1 = decode_psi(z1, "psi1", n)
    nrm = np.sqrt(finite.norm2(psi1))
    psin = {s: a / nrm for s, a in psi1.items()}
    h_dict = {}
    g = spectra.getGreen(n, float(z1["es"][0]), psin, mod.hOp, z["green_w"], 0.1, 150, 1e-7, mod.restrictions,
                         h_dict)
    ref = z["green_g"]
    assert np.abs(g - ref).max() <= 1e-6 * np.abs(ref).max()
    assert list(h_dict.keys()) == decode_states(z["green_keys"], n)
    assert [len(v) for v in h_dict.values()] == list(z["green_nout"])
    # entries equal upstream's applyOp(hOp, {b: 1}, restrictions) (oracle restatement)
    for b in list(h_dict)[:10]:
        ref_b = O.apply_op(n, mod.hOp, {b: 1}, 1e-12, mod.restrictions)
        assert h_dict[b].keys() == ref_b.keys()
        assert all(h_dict[b][s] == ref_b[s] for s in ref_b)
    # a second call reuses the filled memo and gives the same function
    g2 = spectra.getGreen(n, float(z1["es"][0]), psin, mod.hOp, z["green_w"], 0.1, 150, 1e-7, mod.restrictions,
                          h_dict)
    assert np.abs(g2 - g).max() <= 1e-12 * np.abs(g).max()


@pytest.mark.parametrize("precision", [0, 3])
def test_eigensystem_returns_every_copy_of_degenerate_levels(eng, precision):
    mod = M.make_model("config1", hfield=(0.0, 0.0, 0.0), xi_3d=0.0)
    n = mod.n_spin_orbitals
    basis = finite.get_basis(*mod.basis_args())
    k = 6
    es, psis = finite.eigensystem(n, mod.hOp, basis, k, precision=precision)
    es_x, _ = O.eigensystem(n, mod.hOp, basis, k, groundDiagMode="full")
    assert len(es) == k
    assert np.abs(es - es_x).max() < 1e-8, (es, es_x)
    # two triplets: three copies each
    assert np.abs(es[:3] - es[0]).max() < 1e-8 and np.abs(es[3:] - es[3]).max() < 1e-8
    assert es[3] - es[0] > 1e-2
    # upstream's own call found two copies of each triplet (and then higher levels): each of
    # its energies is an eigenvalue, but the lowest six counted with multiplicity are ours
    up = load("dropin.npz")["deg_es"]
    es_all, _ = O.eigensystem(n, mod.hOp, basis, 12, groundDiagMode="full")
    for e in up:
        assert np.abs(es_all - e).min() < 1e-8
    assert np.sum(np.abs(up - es[0]) < 1e-8) == 2
    # eigenvectors: orthonormal and eigenvectors of H (dense check on the 190-state basis)
    h = O.get_hamiltonian_matrix(n, mod.hOp, basis).toarray()
    idx = {b: i for i, b in enumerate(basis)}
    vecs = np.zeros((len(basis), k), dtype=complex)
    for q, p in enumerate(psis):
        for s, a in p.items():
            vecs[idx[s], q] = a
    gram = vecs.conj().T @ vecs
    assert np.abs(gram - np.diag(np.diag(gram))).max() < 1e-6  # truncated at |amp|^2 < 1e-7
    res = np.linalg.norm(h @ vecs - vecs * es[None, :], axis=0) / np.linalg.norm(vecs, axis=0)
    assert res.max() < 1e-2  # the 1e-7 weight truncation of upstream's dicts dominates
    # the device form keeps the full vectors: residuals at solver precision
    eng_ = eng
    dop = finite._device_op(mod.hOp, eng_)
    sb = finite._SortedBasis(eng_, list(basis), n)
    csr = finite._device_hamiltonian(eng_, dop, sb)
    e2, X = finite.eig_lowest(eng_, csr, k, tol_rel=1e-12, precision=precision)
    assert np.abs(e2 - es_x).max() < 1e-8
    Xh = X.cpu().numpy()
    g2 = Xh.conj() @ Xh.T
    assert np.abs(g2 - np.eye(k)).max() < 1e-8


def test_session_sectors_give_the_same_spectra(eng):
    """eigensystem -> getSpectra -> getRIXSmap through the dict API with the sectors kept by
    the session (XAS closure reused as the RIXS core-hole sector, the ground-state basis as the
    final-state sector) equals the same calls with the cache cleared before each."""
    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    basis = finite.get_basis(*mod.basis_args())
    w = np.linspace(-10, 20, 200)
    wl = np.linspace(-2, 12, 150)
    finite.clear_sector_cache()
    es, psis = finite.eigensystem(n, mod.hOp, basis, 3)
    g1 = spectra.getSpectra(n, mod.hOp, mod.xas_ops(), psis, es, w, 0.2, mod.restrictions)
    r1 = spectra.getRIXSmap(n, mod.hOp, mod.xas_ops(), mod.rixs_out_ops(), psis, es, w[::40], wl, 0.2, 0.05,
                            mod.restrictions)
    assert len(eng.sectors) >= 2
    finite.clear_sector_cache()
    g2 = spectra.getSpectra(n, mod.hOp, mod.xas_ops(), psis, es, w, 0.2, mod.restrictions)
    finite.clear_sector_cache()
    r2 = spectra.getRIXSmap(n, mod.hOp, mod.xas_ops(), mod.rixs_out_ops(), psis, es, w[::40], wl, 0.2, 0.05,
                            mod.restrictions)
    assert np.abs(g1 - g2).max() <= 1e-10 * np.abs(g2).max()
    # the final states run on the ground-state sector or on their own closure: the same
    # Krylov spaces (closures are unions of components)
    assert np.abs(r1 - r2).max() <= 1e-6 * np.abs(r2).max()
