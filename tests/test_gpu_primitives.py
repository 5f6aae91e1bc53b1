"""GPU primitives against NumPy and the oracle: scan, radix sort, unique, merge, lookup,
per-state operator application (bit-exact against the oracle's term-order sums)."""

import numpy as np
import pytest
import torch

import oracle.ed_oracle as O
from impuritymodel_gb300 import models as M

pytestmark = pytest.mark.gpu


def _rand_states(rng, n, n_orb, n_el):
    out = np.zeros((n, (n_orb + 63) // 64), dtype=np.uint64)
    for k in range(n):
        occ = rng.choice(n_orb, n_el, replace=False)
        for i in occ:
            out[k, i // 64] |= np.uint64(1) << np.uint64(63 - i % 64)
    return out


@pytest.mark.parametrize("n", [0, 1, 7, 2048, 2049, 100_000])
def test_scan(eng, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 50, size=n).astype(np.int64)
    out = eng.scan(torch.from_numpy(x).to(eng.device)).cpu().numpy()
    ref = np.zeros(n + 1, np.int64)
    np.cumsum(x, out=ref[1:])
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("w,n", [(1, 5000), (2, 70_000), (5, 9000)])
def test_sort_unique_merge_lookup(eng, w, n):
    rng = np.random.default_rng(w * 7 + n)
    n_orb = 64 * w - 3
    pool = _rand_states(rng, n // 3 + 1, n_orb, n_orb // 4)
    keys = pool[rng.integers(0, pool.shape[0], size=n)]
    kt = eng.upload_states(keys)
    pay = torch.arange(n, dtype=torch.int32, device=eng.device)
    eng.sort_states(kt, pay)
    got = eng.download_states(kt)
    order = np.lexsort([keys[:, q] for q in range(w - 1, -1, -1)])  # stable
    assert np.array_equal(got, keys[order])
    assert np.array_equal(pay.cpu().numpy(), order.astype(np.int32))
    u, first, _ = eng.unique_sorted(kt, pay)
    ref_u = np.unique(keys, axis=0)
    # np.unique sorts rows lexicographically as unsigned: same order
    assert np.array_equal(eng.download_states(u), ref_u)
    # merge two disjoint halves
    a = ref_u[::2]
    b = ref_u[1::2]
    m = eng.merge(eng.upload_states(a), eng.upload_states(b))
    assert np.array_equal(eng.download_states(m), ref_u)
    q = np.concatenate([ref_u[:50], _rand_states(rng, 50, n_orb, n_orb // 4 + 1)])
    idx = eng.lookup(u, eng.upload_states(q)).cpu().numpy()
    assert np.array_equal(idx[:50], np.arange(50))
    assert np.all(idx[50:] == -1)


@pytest.mark.parametrize("config", ["config1", "config2"])
def test_apply_columns_bit_exact(eng, config):
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    mod = M.make_model(config)
    n = mod.n_spin_orbitals
    basis = O.get_basis(*mod.basis_args())
    words = O.bytes_to_words(list(basis[:700]), n)
    tab = O.TermTable(mod.hOp)
    masks = O.restriction_masks(mod.restrictions, n)
    colptr, out, val = O.h_columns(words, tab, masks, 1e-12)
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    offs, so, _, sv = eng.apply_columns(eng.upload_states(words), dop, restr, 1e-12, want_states=True, want_vals=True)
    assert np.array_equal(offs.cpu().numpy(), colptr)
    assert np.array_equal(eng.download_states(so), out)
    v = sv.cpu().numpy()
    assert np.array_equal(v[:, 0], val.real) and np.array_equal(v[:, 1], val.imag)


@pytest.mark.parametrize("config,k_cap", [("config1", 120), ("config2", 160)])
def test_reorth_fused_matches_per_step_kernels(eng, config, k_cap):
    """Reorthogonalised Lanczos as one cooperative launch per chunk against the seven
    grid-wide kernels per step, from the same start vector on the ground-state sector: alpha/beta to
    1e-9 relative, the 5 lowest Ritz values to 1e-10 eV, Krylov basis orthonormal to 1e-12."""
    import scipy.linalg

    from impuritymodel_gb300 import finite

    mod = M.make_model(config)
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    csr = finite._device_hamiltonian(eng, dop, sb)
    g = torch.Generator(device=eng.device)
    g.manual_seed(7)
    v0 = torch.randn(csr.n, dtype=torch.complex128, device=eng.device, generator=g)
    v0 = v0 / torch.linalg.vector_norm(v0)
    out = {}
    try:
        for fused in (1, 0):
            eng.lib.edgpu_set_reorth_fused(fused)
            V, a, b = eng.krylov_reorth(csr, v0, k_cap, chunk=40)
            gram = V @ V.conj().t()
            err = (gram - torch.eye(V.shape[0], dtype=gram.dtype, device=gram.device)).abs().max().item()
            assert err < 1e-12, (fused, err)
            out[fused] = (a, b)
    finally:
        eng.lib.edgpu_set_reorth_fused(1)
    (a1, b1), (a0, b0) = out[1], out[0]
    assert a1.shape == a0.shape
    scale = np.abs(a0).max()
    assert np.abs(a1 - a0).max() < 1e-9 * scale
    assert np.abs(b1[:-1] - b0[:-1]).max() < 1e-9 * scale
    th1 = scipy.linalg.eigh_tridiagonal(a1, b1[:-1], eigvals_only=True)[:5]
    th0 = scipy.linalg.eigh_tridiagonal(a0, b0[:-1], eigvals_only=True)[:5]
    assert np.abs(th1 - th0).max() < 1e-10


def test_apply_vectors_multi_equals_per_operator_calls(eng):
    """All operators at once (one scan/sort/unique) give bit for bit the per-operator results."""
    from impuritymodel_gb300 import finite

    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    es, psi_t = finite.eigensystem_device(eng, finite._device_op(mod.hOp, eng),
                                          finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n), 3)
    from impuritymodel_gb300.engine import make_restrictions

    restr = make_restrictions(mod.restrictions, n)
    dops = [finite._device_op(t, eng) for t in mod.xas_ops() + mod.ps_ops()[:2]]
    multi = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t], dops, restr, 1e-7)
    for o, dop in enumerate(dops):
        single = eng.apply_vectors([p[0] for p in psi_t], [p[1] for p in psi_t], dop, restr, 1e-7)
        for (s1, a1), (s2, a2) in zip(single, multi[o]):
            assert torch.equal(s1, s2) and torch.equal(a1, a2)


def test_components_kernel_equals_label_propagation(eng):
    """One-launch component labels equal scipy's connected components (smallest member index
    as label) on the XAS sector of the 26-orbital model."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components

    from impuritymodel_gb300 import finite, spectra
    from impuritymodel_gb300.engine import make_restrictions

    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    restr = make_restrictions(mod.restrictions, n)
    es, psi_t = finite.eigensystem_device(eng, dop, finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n), 3)
    outs = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t],
                                   [finite._device_op(t, eng) for t in mod.xas_ops()], restr, 1e-7)
    sec = spectra.Sector(eng, dop, restr, torch.cat([s for row in outs for s, _ in row]))
    csr = sec.csr
    lab = eng.components(csr).cpu().numpy()
    H = sp.csr_matrix((np.ones(csr.nnz), csr.col.cpu().numpy(), csr.row_ptr.cpu().numpy()), shape=(csr.n, csr.n))
    nc, cc = connected_components(H, directed=False)
    ref = np.array([np.nonzero(cc == cc[i])[0].min() for i in range(csr.n)])
    assert np.array_equal(lab, ref)


@pytest.mark.parametrize("precision", [0, 3])
def test_shifted_solve_against_dense(eng, precision):
    """x = (z - H)^{-1} y for 40 shifts and 3 right-hand sides on the RIXS core-hole sector of
    the 66-orbital model: the FP64 and the double-float recurrences against a dense solve,
    1e-7 relative (residual tolerance 1e-10 times the resolvent norm bound 1 / Im z, against
    |x| >= |y| / max |z - lambda|)."""
    from impuritymodel_gb300 import finite, spectra
    from impuritymodel_gb300.engine import make_restrictions

    mod = M.make_model("config2")
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    restr = make_restrictions(mod.restrictions, n)
    es, psi_t = finite.eigensystem_device(eng, dop, finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n), 1)
    outs = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t],
                                   [finite._device_op(t, eng) for t in mod.xas_ops()], restr, 1e-7)
    sec = spectra.Sector(eng, dop, restr, torch.cat([s for row in outs for s, _ in row]))
    csr = sec.csr
    assert csr.val_c is None  # real H: precision 3 takes the double-float kernel
    H = np.zeros((csr.n, csr.n))
    rp, col, val = csr.row_ptr.cpu().numpy(), csr.col.cpu().numpy(), csr.val_r.cpu().numpy()
    for i in range(csr.n):
        H[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    rng = np.random.default_rng(5)
    Y = rng.standard_normal((3, csr.n)) + 1j * rng.standard_normal((3, csr.n))
    w = np.linspace(-10.0, 20.0, 40)
    zs = np.array([w + 0.2j + es[0] + 0.5 * r for r in range(3)])
    X, m = eng.shifted_solve(csr, torch.from_numpy(Y).to(eng.device), zs, 1e-10, min(6 * csr.n + 50, 2000), precision)
    X = X.cpu().numpy()
    for r in range(3):
        for k in range(len(w)):
            ref = np.linalg.solve(zs[r, k] * np.eye(csr.n) - H, Y[r])
            assert np.linalg.norm(X[r, k] - ref) <= 1e-7 * np.linalg.norm(ref), (r, k)
    assert np.all(m.cpu().numpy() > 0)


@pytest.mark.parametrize("config", ["config1", "config2"])
def test_reorth_double_float_matches_fp64(eng, config):
    """The double-float cooperative reorthogonalised Lanczos against the FP64 one on the
    ground-state sector: the 5 lowest energies to 1e-10 eV, eigenpair residuals
    ||H x - e x|| below 1e-9 (degenerate levels make single eigenvectors arbitrary), and its
    Krylov basis orthonormal to 1e-12."""
    from impuritymodel_gb300 import finite

    mod = M.make_model(config)
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    csr = finite._device_hamiltonian(eng, dop, sb)
    if csr.val_c is not None:
        pytest.skip("complex H: the double-float form runs in FP64")
    e0, x0 = finite.eig_lowest(eng, csr, 5, tol_rel=1e-12, precision=0)
    e3, x3 = finite.eig_lowest(eng, csr, 5, tol_rel=1e-12, precision=3)
    assert np.abs(e3 - e0).max() < 1e-10
    hx = eng.spmv(csr, x3.t().contiguous()).t()
    res = torch.linalg.vector_norm(hx - torch.as_tensor(e3, device=eng.device).view(-1, 1) * x3, dim=1)
    assert res.max().item() < 1e-9, res
    g = torch.Generator(device=eng.device)
    g.manual_seed(3)
    v0 = torch.randn(csr.n, dtype=torch.complex128, device=eng.device, generator=g)
    v0 = v0 / torch.linalg.vector_norm(v0)
    V, a, b = eng.krylov_reorth(csr, v0, 120, chunk=40, precision=3)
    gram = V @ V.conj().t()
    err = (gram - torch.eye(V.shape[0], dtype=gram.dtype, device=gram.device)).abs().max().item()
    assert err < 1e-12, err


@pytest.mark.parametrize("runs", [5, 300, 750, 1000])
def test_small_double_float_lanczos_matches_fp64(eng, runs):
    """The one-CTA-per-run double-float Lanczos (one shared-memory vector per run, the
    previous vector in the workspace; the CTA size follows the run count: 512 threads for a
    few runs, 160 for hundreds) against the FP64 recurrence on the 1770-row ground-state
    sector of the 66-orbital model: the first 25 alphas and betas to 1e-9 relative, ragged
    step counts honoured (k_max 0 leaves a run's coefficients zero)."""
    from impuritymodel_gb300 import finite

    mod = M.make_model("config2")
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    csr = finite._device_hamiltonian(eng, dop, sb)
    assert csr.val_c is None
    g = torch.Generator(device=eng.device)
    g.manual_seed(runs)
    v0 = torch.randn(csr.n, runs, dtype=torch.complex128, device=eng.device, generator=g)
    v0 = v0 / torch.linalg.vector_norm(v0, dim=0, keepdim=True)
    rng = np.random.default_rng(runs)
    k_max = rng.integers(25, 41, size=runs).astype(np.int32)
    k_max[0] = 0
    k_max[-1] = 1
    a0, b0 = eng.lanczos(csr, v0, k_max, precision=0)
    a3, b3 = eng.lanczos(csr, v0, k_max, precision=3)
    a0, b0, a3, b3 = (x.cpu().numpy() for x in (a0, b0, a3, b3))
    assert not a3[0].any() and not b3[0].any()
    assert a3[-1, 0] != 0.0 and not a3[-1, 1:].any() and not b3[-1].any()
    live = np.arange(1, runs - 1)
    for x0, x3 in ((a0, a3), (b0, b3)):
        d = np.abs(x3[live, :24] - x0[live, :24]) / np.maximum(np.abs(x0[live, :24]), 1e-300)
        assert d.max() < 1e-9, d.max()
    for r in live[:50]:
        assert not a3[r, k_max[r]:].any() and not b3[r, k_max[r] - 1:].any()


@pytest.mark.parametrize("n,runs", [(100, 1000), (777, 400), (2000, 300)])
def test_sliced_double_float_lanczos_irregular_rows(eng, n, runs):
    """The sliced layout (rows sorted by length into 32-row column-major slices, columns
    stored as slots) on symmetric matrices whose rows range from empty-ish to a few hundred
    entries, n not a multiple of 32: the double-float alphas and betas against the FP64
    recurrence over the first 20 steps (1e-9 relative), for every run."""
    import scipy.sparse as sp
    from impuritymodel_gb300 import finite

    rng = np.random.default_rng(n)
    A = sp.random(n, n, density=4.0 / n, random_state=n, format="coo")
    heavy = rng.choice(n, size=max(1, n // 50), replace=False)  # a few rows with many entries
    rows = np.repeat(heavy, min(n, 300))
    cols = rng.integers(0, n, size=rows.size)
    B = sp.coo_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(n, n))
    H = (A + B).tocsr()
    H = (H + H.T).tocsr() + sp.diags(rng.uniform(-5.0, 5.0, n))
    csr = finite._scipy_to_device_csr(eng, H)
    assert csr.val_c is None
    g = torch.Generator(device=eng.device)
    g.manual_seed(n)
    v0 = torch.randn(n, runs, dtype=torch.complex128, device=eng.device, generator=g)
    v0 = v0 / torch.linalg.vector_norm(v0, dim=0, keepdim=True)
    k_max = np.full(runs, 20, dtype=np.int32)
    a0, b0 = eng.lanczos(csr, v0, k_max, precision=0)
    a3, b3 = eng.lanczos(csr, v0, k_max, precision=3)
    a0, b0, a3, b3 = (x.cpu().numpy() for x in (a0, b0, a3, b3))
    assert np.abs(a3 - a0).max() <= 1e-9 * np.abs(a0).max()
    assert (np.abs(b3[:, :19] - b0[:, :19]) / b0[:, :19]).max() < 1e-9


@pytest.mark.parametrize("precision", [0, 3])
def test_concurrent_xas_rixs_equals_sequential(eng, precision):
    """xas_rixs_device (RIXS on the current stream, XAS on a side stream taking the RIXS
    job's T_in psi and core-hole sector, the ground-state sector reused for the final states)
    gives the same bits as spectra_device and rixs_device called one after the other."""
    from impuritymodel_gb300 import finite, spectra
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    mod = M.make_model("config2")
    n = mod.n_spin_orbitals
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    xas = [DeviceOp(t, eng.device) for t in mod.xas_ops()]
    outs = [DeviceOp(t, eng.device) for t in mod.rixs_out_ops()]
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    es, psi_t, h = finite.eigensystem_device(eng, dop, sb, 2, precision=precision, with_hamiltonian=True)
    gs_sector = spectra.closed_sector(eng, dop, restr, sb.sorted, h, sb.words)
    w = np.linspace(-25.0, 25.0, 300)
    w_in = np.linspace(-10.0, 20.0, 4)
    w_loss = np.linspace(-2.0, 12.0, 250)
    gx1, gr1 = spectra.xas_rixs_device(eng, dop, restr, xas, xas, outs, psi_t, es, w, 0.2, w_in, w_loss, 0.2, 0.05,
                                       150, 1e-7, precision, final_sector=gs_sector)
    gx2 = spectra.spectra_device(eng, dop, restr, xas, psi_t, es, w, 0.2, 150, 1e-7, precision)
    gr2 = spectra.rixs_device(eng, dop, restr, xas, outs, psi_t, es, w_in, w_loss, 0.2, 0.05, 150, 1e-7, precision,
                              final_sector=gs_sector)
    torch.cuda.synchronize()
    assert torch.equal(gx1, gx2)
    assert torch.equal(gr1, gr2)
    assert gx1.abs().max().item() > 0 and gr1.abs().max().item() > 0


def test_closed_ground_sector_serves_green_functions(eng):
    """The ground-state sector of the 66-orbital model is closed under the restricted H, so
    Green's-function runs starting inside it can use it instead of a fresh expansion.  When
    the runs' closure is the whole sector (random start states spread over it) the spectra
    are bit-identical to the expanded ones; a start state outside it falls back to the
    expansion."""
    from impuritymodel_gb300 import finite, spectra
    from impuritymodel_gb300.engine import make_restrictions

    mod = M.make_model("config2")
    n = mod.n_spin_orbitals
    dop = finite._device_op(mod.hOp, eng)
    restr = make_restrictions(mod.restrictions, n)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    es, psi_t, h = finite.eigensystem_device(eng, dop, sb, 1, precision=3, with_hamiltonian=True)
    sec = spectra.closed_sector(eng, dop, restr, sb.sorted, h, sb.words)
    assert sec is not None and sec.n == sb.sorted.shape[0]
    rng = np.random.default_rng(11)
    run_states, run_amps = [], []
    for r in range(4):
        idx = torch.as_tensor(np.sort(rng.choice(sec.n, 300, replace=False)), device=eng.device)
        run_states.append(sb.sorted[idx].contiguous())
        run_amps.append(torch.as_tensor(rng.standard_normal((300, 2)), device=eng.device))
    w = np.linspace(-5.0, 15.0, 200)
    e_runs = [es[0]] * 4
    st = spectra.green_setup(eng, dop, restr, run_states, run_amps, 150, 3)
    assert st.sector.n == sec.n  # the expanded closure is the whole sector
    g1 = spectra.green_batch(eng, dop, restr, run_states, run_amps, e_runs, w, 0.1, 150, 3)
    g2 = spectra._drive(spectra._green_batch_steps(eng, dop, restr, run_states, run_amps, e_runs, w, 0.1, 150, 3,
                                                   sector_hint=sec))
    assert torch.equal(g1, g2)
    # a start state outside the hinted sector: falls back to the expansion
    small = spectra.Sector.from_parts(sb.sorted[:10].contiguous(), h)
    g3 = spectra._drive(spectra._green_batch_steps(eng, dop, restr, run_states, run_amps, e_runs, w, 0.1, 150, 3,
                                                   sector_hint=small))
    assert torch.equal(g1, g3)


@pytest.mark.parametrize("w,n", [(1, 2), (2, 300), (3, 4097), (2, 8192), (8, 1500)])
def test_small_sort_is_stable(eng, w, n):
    """The one-CTA bitonic path sorts like the stable radix sort: keys with many duplicates,
    payloads in their original relative order within equal keys."""
    rng = np.random.default_rng(n + w)
    pool = _rand_states(rng, max(2, n // 7), 64 * w - 5, 5)
    keys = pool[rng.integers(0, pool.shape[0], size=n)]
    kt = eng.upload_states(keys)
    pay = torch.arange(n, dtype=torch.int32, device=eng.device)
    eng.sort_states(kt, pay)
    order = np.lexsort([keys[:, q] for q in range(w - 1, -1, -1)])  # stable
    assert np.array_equal(eng.download_states(kt), keys[order])
    assert np.array_equal(pay.cpu().numpy(), order.astype(np.int32))
