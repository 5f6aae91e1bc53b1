"""Ragged ensemble batches on the GPU: the one-launch Lanczos over many models' sectors
against the single-sector kernels, and ensemble ground states + XAS against the oracle's
dense eigensystems and the single-model drop-in API."""

import numpy as np
import pytest
import torch

import oracle.ed_oracle as O
from impuritymodel_gb300 import ensemble, finite, spectra
from impuritymodel_gb300 import models as M

pytestmark = pytest.mark.gpu

# (seed, bath levels per 3d spin-orbital); the last model has two words per state, the
# others one (ragged batches mix state widths)
MODELS = [(11, 1), (12, 2), (13, 1), (14, 5)]


@pytest.fixture(scope="module")
def members():
    return [M.random_model(seed, levels) for seed, levels in MODELS]


def test_ragged_lanczos_equals_single_sector_kernel(eng, members):
    """Same recurrence and reduction order as the single-sector shared-memory kernel: the
    ragged launch reproduces its alpha/beta (first 20 steps to 1e-12 relative, all 40 to
    1e-8; the unreorthogonalised recurrence amplifies rounding differences)."""
    secs = [ensemble.ModelSectors(eng, m) for m in members]
    batch = ensemble.RaggedBatch(eng, [s.csr for s in secs], [0, 1, 2, 1])
    K = 40
    k = np.array([min(K, secs[s].csr.n) for s in batch.run_sec_h], dtype=np.int32)
    starts = [ensemble._random_start(eng, secs[s].csr.n, 100 + r) for r, s in enumerate(batch.run_sec_h)]
    a, b = eng.lanczos_ragged(batch, torch.cat(starts), k)
    for r, s in enumerate(batch.run_sec_h):
        a1, b1 = eng.lanczos(secs[s].csr, starts[r].reshape(-1, 1), k[r : r + 1])
        kr = int(k[r])
        ah, a1h = a[r, :kr].cpu().numpy(), a1[0, :kr].cpu().numpy()
        bh, b1h = b[r, : kr - 1].cpu().numpy(), b1[0, : kr - 1].cpu().numpy()
        scale = np.abs(a1h).max()
        assert np.abs(ah[:20] - a1h[:20]).max() <= 1e-12 * scale
        assert np.abs(bh[:19] - b1h[:19]).max() <= 1e-12 * scale
        assert np.abs(ah - a1h).max() <= 1e-8 * scale
        assert np.abs(bh - b1h).max() <= 1e-8 * scale


def test_ensemble_ground_states_and_xas(eng, members):
    """Energies against dense diagonalisation (1e-8 eV); XAS against the single-model
    getSpectra on the same model (1e-6 relative); the graph-captured solve agrees."""
    w = np.linspace(-10.0, 20.0, 400)
    es, gs = ensemble.ensemble_gs_xas(members, w, 0.2, n_states=3)
    es_g, gs_g = ensemble.ensemble_gs_xas(members, w, 0.2, n_states=3, graph=True)
    for m, mod in enumerate(members):
        n = mod.n_spin_orbitals
        basis = finite.get_basis(*mod.basis_args())
        ex, _ = O.eigensystem(n, mod.hOp, basis, 3, groundDiagMode="full")
        assert np.abs(es[m] - ex[:3]).max() < 1e-8
        e1, psis1 = finite.eigensystem(n, mod.hOp, basis, 3)
        g1 = spectra.getSpectra(n, mod.hOp, mod.xas_ops(), psis1, e1, w, 0.2, mod.restrictions)
        assert gs[m].shape == g1.shape
        assert np.abs(gs[m] - g1).max() / np.abs(g1).max() < 1e-6
        assert np.abs(gs_g[m] - gs[m]).max() / np.abs(gs[m]).max() < 1e-9


def test_graph_replay_equals_direct_launches(eng, members):
    """The CUDA-graph replay of the ragged XAS solve issues the same two kernels on the same
    buffers: its output equals the direct launches' bit for bit."""
    w = np.linspace(-10.0, 20.0, 200)
    secs = [ensemble.ModelSectors(eng, m) for m in members]
    es, psis = ensemble.ensemble_ground_states(eng, secs, 3)
    solve, _ = ensemble.ensemble_xas_setup(eng, secs, es, psis, w, 0.2)
    g_direct = solve.run().clone()
    solve.capture()
    solve.g.zero_()
    g_graph = solve.replay()
    assert torch.equal(g_direct, g_graph)
