"""3d observables on the GPU against upstream's own values (golden fixture observables.npz,
made by running upstream's finite.py:843-1298 on its eigenstates of the 26- and 66-spin-orbital
models): density matrices and expectation values 1e-12, operator results 1e-13."""

import numpy as np
import pytest

from impuritymodel_gb300 import finite, observables
from impuritymodel_gb300 import models as M
from tests.golden.fixtures import decode_psi, load

pytestmark = pytest.mark.gpu

CASES = [("c1", "config1", "config1.npz"), ("c2", "config2", "config2.npz")]


def _dense(d, key):
    out = np.zeros((10, 10), dtype=complex)
    for k, v in d.items():
        out[key(k)] = v
    return out


@pytest.mark.parametrize("tag,cfg,fname", CASES)
def test_upstream_api_observables(eng, tag, cfg, fname):
    z = load("observables.npz")
    zc = load(fname)
    mod = M.make_model(cfg)
    n = int(zc["n_spin_orbitals"])
    nb = mod.nBaths
    for i in range(int(z[tag + "_n_states"])):
        psi = decode_psi(zc, "eig%d" % i, n)
        dm = _dense(finite.getDensityMatrix(nb, psi), lambda k: (k[0][1] * 5 + k[0][2] + 2, k[1][1] * 5 + k[1][2] + 2))
        assert np.abs(dm - z[tag + "_dm"][i]).max() < 1e-12
        dmc = _dense(finite.getDensityMatrixCubic(nb, psi), lambda k: (k[0][0] * 5 + k[0][1], k[1][0] * 5 + k[1][1]))
        assert np.abs(dmc - z[tag + "_dm_cubic"][i]).max() < 1e-12
        vals = [finite.getTraceDensityMatrix(nb, psi), *finite.getEgT2gOccupation(nb, psi), finite.getLz3d(nb, psi),
                finite.getSz3d(nb, psi), finite.getLsqr3d(nb, psi), finite.getSsqr3d(nb, psi)]
        assert np.abs(np.array(vals) - z[tag + "_values"][i]).max() < 1e-11
    psi0 = decode_psi(zc, "eig0", n)
    for name in ("applySz3d", "applyLz3d", "applySplus3d", "applyLplus3d", "applySminus3d", "applyLminus3d"):
        ref = decode_psi(z, tag + "_" + name, n)
        got = getattr(finite, name)(nb, psi0)
        keys = set(ref) | set(got)
        assert max(abs(ref.get(s, 0) - got.get(s, 0)) for s in keys) < 1e-13, name


@pytest.mark.parametrize("tag,cfg,fname", CASES)
def test_batched_expectation_values(eng, tag, cfg, fname):
    """All eigenstates of a model in one density-matrix launch (+ one operator launch per
    ladder operator): same values as upstream's per-state loops."""
    z = load("observables.npz")
    zc = load(fname)
    mod = M.make_model(cfg)
    n = int(zc["n_spin_orbitals"])
    from impuritymodel_gb300 import codec

    pt = []
    for i in range(int(z[tag + "_n_states"])):
        words, amps = codec.psi_to_arrays(decode_psi(zc, "eig%d" % i, n), n)
        pt.append((eng.upload_states(words), eng.to_device(amps)))
    r = observables.expectation_values(eng, pt, mod.nBaths)
    vals = np.stack([r[k] for k in ("n3d", "eg_dn", "eg_up", "t2g_dn", "t2g_up", "lz", "sz", "l2", "s2")], 1)
    assert np.abs(vals - z[tag + "_values"]).max() < 1e-11
    assert np.abs(r["dm"] - z[tag + "_dm"]).max() < 1e-12
    assert np.abs(r["dm_cubic"] - z[tag + "_dm_cubic"]).max() < 1e-12
