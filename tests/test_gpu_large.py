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
    g64, info = spectra_large(eng, s["dop"], s["mop"], s["restr"], ps, psi_t, es, -w, -0.2, K=120, precision=1,
                              matfree=True)
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
    # one Gram-Schmidt pass per step (second only where DGKS asks) against two every step:
    # both keep the basis orthogonal, so all 40 coefficients agree
    a_2, b_2, _ = lanczos_reorth_batched(eng, apply_h, v0t, 40, precision=0, reorth="cgs2")
    assert np.abs(a_r - a_2).max() < 1e-9 and np.abs(b_r - b_2).max() < 1e-9


def test_locality_order_is_a_relabelling(eng, small316):
    """The sector in locality order: a permutation whose blocks agree on every non-lead
    orbital; H.v of the reordered CSR and of the matrix-free product on the reordered basis
    equal the sorted-order products permuted, bit for bit (each row keeps its term order)."""
    from impuritymodel_gb300 import finite
    from impuritymodel_gb300.large import hv_diag, hv_matfree_into, locality_order, state_hash

    s = small316
    basis = s["sb"].sorted
    n = basis.shape[0]
    perm = locality_order(basis, s["dop"])
    assert perm is not None
    assert torch.equal(torch.sort(perm).values, torch.arange(n, device=eng.device))
    moves = s["dop"].moves
    lead = set(np.nonzero(moves > 4.0 * np.median(moves[moves > 0]))[0].tolist())
    assert lead and all(o < 16 for o in lead)  # the 2p and 3d spin-orbitals of this model
    words = basis[perm].cpu().numpy().view(np.uint64)
    mask = np.zeros(words.shape[1], dtype=np.uint64)
    for o in lead:
        mask[o // 64] |= np.uint64(1) << np.uint64(63 - o % 64)
    major = [tuple(r) for r in (words & ~mask)]
    assert major == sorted(major)  # non-decreasing bath part: contiguous blocks
    csr = finite._device_hamiltonian(eng, s["dop"], s["sb"])
    csr_p = csr.permuted(perm)
    assert csr_p.nnz == csr.nnz
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.standard_normal((n, 4)) + 1j * rng.standard_normal((n, 4))).to(eng.device)
    y = eng.spmv(csr, x)
    y_p = eng.spmv(csr_p, x[perm].contiguous())
    assert torch.equal(y_p, y[perm])
    bp = basis[perm].contiguous()
    d, d_p = hv_diag(eng, basis, s["mop"]), hv_diag(eng, bp, s["mop"])
    assert torch.equal(d_p, d[perm])
    ym = torch.empty_like(x)
    ym_p = torch.empty_like(x)
    hv_matfree_into(eng, basis, s["mop"], s["restr"], d, x, ym, 0.0, state_hash(eng, basis))
    hv_matfree_into(eng, bp, s["mop"], s["restr"], d_p, x[perm].contiguous(), ym_p, 0.0, state_hash(eng, bp))
    assert torch.equal(ym_p, ym[perm])


def test_spectra_locality_order_matches_sorted(eng, small316):
    from impuritymodel_gb300 import finite
    from impuritymodel_gb300.engine import DeviceOp
    from impuritymodel_gb300.large import spectra_large

    s = small316
    es, psi_t = finite.eigensystem_device(eng, s["dop"], s["sb"], 1)
    w = np.linspace(-15, 15, 400)
    ps = [DeviceOp(t, eng.device) for t in s["mod"].ps_ops()[:2]]
    args = (eng, s["dop"], s["mop"], s["restr"], ps, psi_t, es, -w, -0.2)
    g_o, info = spectra_large(*args, K=100, precision=0, order=True)
    g_s, _ = spectra_large(*args, K=100, precision=0, order=False, sector=info["sector_obj"])
    for o in range(2):
        ref = g_s[0, o].imag
        # complex128 both ways: the orders differ only in the summation order of the dots
        assert np.abs(g_o[0, o].imag - ref).sum() / np.abs(ref).sum() < 1e-9


@pytest.mark.parametrize("precision,R", [(1, 16), (1, 3), (1, 1), (0, 16), (0, 5)])
def test_krylov_pieces_match_torch(eng, precision, R):
    """edgpu_krylov_dot / _project / _normalize against the same operations in complex128
    torch arithmetic, for paired (even R) and single complex64 lanes and for complex128:
    dots and norms at 1e-5 (complex64 inputs, FP64 accumulation above chunks of 8 products)
    or 1e-12 (complex128) relative to the vector norms."""
    import ctypes as C

    from impuritymodel_gb300 import _lib as L
    from impuritymodel_gb300.engine import _ptr

    lib = eng.lib
    n, K, m = 20011, 9, 7
    dt = torch.complex64 if precision else torch.complex128
    g = torch.Generator(device=eng.device).manual_seed(3)
    V = torch.randn((K, n, R), dtype=dt, device=eng.device, generator=g)
    w = torch.randn((n, R), dtype=dt, device=eng.device, generator=g)
    h = torch.zeros((K, R), dtype=torch.complex128, device=eng.device)
    wsn = lib.edgpu_krylov_workspace(n, R, K)
    ws = torch.empty(wsn, dtype=torch.uint8, device=eng.device)
    st = eng.stream
    Vr = torch.view_as_real(V)
    L.check(lib.edgpu_krylov_dot(precision, _ptr(Vr), n * R, m, n, R, _ptr(torch.view_as_real(w)),
                                 _ptr(torch.view_as_real(h)), C.c_void_p(ws.data_ptr()), wsn, st), "dot")
    V64, w64 = V.to(torch.complex128), w.to(torch.complex128)
    ref = torch.einsum("kir,ir->kr", V64[:m].conj(), w64)
    tol = 1e-5 if precision else 1e-12
    scale = float(torch.linalg.vector_norm(w64)) * float(torch.linalg.vector_norm(V64[0]))
    assert float((h[:m] - ref).abs().max()) < tol * scale
    # project with norms, then normalise
    w_ref = w64 - torch.einsum("kr,kir->ir", h[:m], V64[:m])
    L.check(lib.edgpu_krylov_project(precision, _ptr(Vr), n * R, m, n, R, _ptr(torch.view_as_real(h)),
                                     _ptr(torch.view_as_real(w)), 1, C.c_void_p(ws.data_ptr()), wsn, st), "project")
    assert float((w.to(torch.complex128) - w_ref).abs().max()) < (5e-5 if precision else 1e-11) * float(
        w_ref.abs().max())
    beta = torch.zeros(R, dtype=torch.float64, device=eng.device)
    v = torch.empty_like(w)
    eng.reset_status()
    L.check(lib.edgpu_krylov_normalize(precision, n, R, _ptr(torch.view_as_real(w)), _ptr(torch.view_as_real(v)),
                                       _ptr(beta), _ptr(eng.status), C.c_void_p(ws.data_ptr()), wsn, st), "normalize")
    b_ref = torch.linalg.vector_norm(w.to(torch.complex128), dim=0)
    assert float(((beta - b_ref) / b_ref).abs().max()) < (1e-6 if precision else 1e-13)
    assert float((v.to(torch.complex128) - w.to(torch.complex128) / b_ref).abs().max()) < (1e-6 if precision else 1e-13)
    assert int(eng.status.item()) == 0


def test_bucketed_application_equals_all_terms_kernel(eng):
    """The bucketed operator application (index of the terms by created orbital, diagonal
    sums one state per lane in 19-state warp groups for this 47 895-state basis, hash-merged
    outputs) builds the same CSR and expands to the same closure, bit for bit, as the kernel
    that tries every term on every state (selected by a scratch capacity that is not a power
    of two)."""
    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    mod = models.make_model("config4")
    n = mod.n_spin_orbitals
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    assert sb.sorted.shape[0] > 40000
    saved = eng.scratch_entries
    try:
        eng.scratch_entries = 256
        a = eng.build_csr(sb.sorted, dop, restr)
        ps = DeviceOp(mod.ps_ops()[0], eng.device)
        amps = torch.zeros((sb.sorted.shape[0], 2), dtype=torch.float64, device=eng.device)
        amps[:, 0] = 1.0
        (st, _), = eng.apply_vectors([sb.sorted], [amps], ps, restr, 0.0)
        start = eng.sort_unique(st[:2000])
        ea_s, ea_l = eng.expand(start, dop, restr)
        eng.scratch_entries = 300
        b = eng.build_csr(sb.sorted, dop, restr)
        eb_s, eb_l = eng.expand(start, dop, restr)
    finally:
        eng.scratch_entries = saved
    assert torch.equal(a.row_ptr, b.row_ptr) and torch.equal(a.col, b.col) and torch.equal(a.val_r, b.val_r)
    assert torch.equal(ea_s, eb_s) and torch.equal(ea_l, eb_l)
