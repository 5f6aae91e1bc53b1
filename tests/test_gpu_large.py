"""Large-sector path on the GPU (impuritymodel_gb300.large): matrix-free H·v and the batched
reorthogonalised Lanczos in complex64 with FP64 reductions, against the CSR path in
complex128.

Tolerances: matrix-free H·v against the CSR product at 1e-13 (complex128; the same matrix
elements summed in another order) and 2e-6 (complex64 with float32 accumulation), relative
to the row-sum scale; the reorthogonalised recurrence's first 20 alpha/beta against
upstream's plain recurrence at 1e-9 (before orthogonality is lost, both compute the same
Krylov space); complex64 spectra against the complex128 reference at 1e-3 relative L1 per
spectrum.  The model is the 316-spin-orbital one (5-word states) with at most one bath hole,
so its sectors fit a test.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small316(eng):
    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions
    from impuritymodel_gb300.large import MatfreeOp

    mod = models.make_model("config4", bath_holes=1)
    n = mod.n_spin_orbitals
    basis = finite.get_basis(*mod.basis_args())
    dop = DeviceOp(mod.hOp, eng.device)
    mop = MatfreeOp(mod.hOp, n, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    sb = finite._SortedBasis(eng, list(basis), n)
    return dict(mod=mod, n=n, dop=dop, mop=mop, restr=restr, sb=sb)


def _check_hv(eng, basis, csr, mop, restr, widths):
    from impuritymodel_gb300.large import hv_diag, hv_matfree_into, state_hash

    n = basis.shape[0]
    d = hv_diag(eng, basis, mop)
    table = state_hash(eng, basis)
    rng = np.random.default_rng(4)
    rows = torch.repeat_interleave(torch.arange(n, device=eng.device), csr.row_ptr[1:] - csr.row_ptr[:-1])
    vals = csr.val_r.abs() if csr.val_r is not None else torch.view_as_complex(csr.val_c).abs()
    for precision, Rs in widths:
        for R in Rs:
            x = torch.from_numpy(rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))).to(eng.device)
            ref = eng.spmv(csr, x)
            scale = float(torch.zeros(n, dtype=torch.float64, device=eng.device).index_add_(
                0, rows, vals * x.abs().max()).max())
            for shift, tab in ((0.0, None), (3.0, None), (0.0, table)):
                xt = x.to(torch.complex64) if precision else x
                y = torch.empty_like(xt)
                hv_matfree_into(eng, basis, mop, restr, d, xt, y, shift, tab)
                err = float((y.to(torch.complex128) + shift * xt.to(torch.complex128) - ref).abs().max()) / scale
                tol = 2e-6 if precision else 1e-13
                assert err < tol, (precision, R, shift, err)


def test_matfree_hv_matches_csr_316_orbitals(eng, small316):
    from impuritymodel_gb300 import finite

    s = small316
    csr = finite._device_hamiltonian(eng, s["dop"], s["sb"])
    assert s["sb"].sorted.shape[1] == 5
    _check_hv(eng, s["sb"].sorted, csr, s["mop"], s["restr"], ((0, (1, 2, 16)), (1, (2, 8, 16))))


def test_matfree_hv_matches_csr_26_orbitals(eng):
    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions
    from impuritymodel_gb300.large import MatfreeOp

    mod = models.make_model("config1")
    n = mod.n_spin_orbitals
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    dop = DeviceOp(mod.hOp, eng.device)
    csr = finite._device_hamiltonian(eng, dop, sb)
    _check_hv(eng, sb.sorted, csr, MatfreeOp(mod.hOp, n, eng.device), make_restrictions(mod.restrictions, n),
              ((0, (1, 4)), (1, (2, 4))))


def test_reorth_lanczos_and_spectra_316_orbitals(eng, small316):
    from impuritymodel_gb300 import finite
    from impuritymodel_gb300.engine import DeviceOp
    from impuritymodel_gb300.large import lanczos_reorth_batched, spectra_large

    s = small316
    mod = s["mod"]
    es, psi_t = finite.eigensystem_device(eng, s["dop"], s["sb"], 1)
    w = np.linspace(-15, 15, 600)
    ps = [DeviceOp(t, eng.device) for t in mod.ps_ops()[:4]]
    g64, info = spectra_large(eng, s["dop"], s["mop"], s["restr"], ps, psi_t, es, -w, -0.2, K=120, precision=1)
    sector = info["sector_obj"]
    assert info["runs"] == 4 and info["sector"] > 1000
    g128, _ = spectra_large(eng, s["dop"], s["mop"], s["restr"], ps, psi_t, es, -w, -0.2, K=120, precision=0,
                            sector=sector)
    g64c, _ = spectra_large(eng, s["dop"], s["mop"], s["restr"], ps, psi_t, es, -w, -0.2, K=120, precision=1,
                            matfree=False, sector=sector)
    for o in range(4):
        ref = g128[0, o].imag
        assert np.abs(ref).sum() > 0
        for g in (g64, g64c):
            err = np.abs(g[0, o].imag - ref).sum() / np.abs(ref).sum()
            assert err < 1e-3, (o, err)
    # the first steps of the reorthogonalised recurrence equal upstream's plain recurrence
    n = sector.n
    rng = np.random.default_rng(2)
    v0 = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    v0 /= np.linalg.norm(v0, axis=0)
    v0t = torch.from_numpy(v0).to(eng.device)
    a_p, b_p = eng.lanczos(sector.csr, v0t, [40, 40], precision=0)

    def apply_h(x, y):
        y.copy_(eng.spmv(sector.csr, x))

    a_r, b_r, k_len = lanczos_reorth_batched(eng, apply_h, v0t, 40, precision=0)
    assert list(k_len) == [40, 40]
    assert np.abs(a_r[:, :20] - a_p.cpu().numpy()[:, :20]).max() < 1e-9
    assert np.abs(b_r[:, :20] - b_p.cpu().numpy()[:, :20]).max() < 1e-9
