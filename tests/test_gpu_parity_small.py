"""Drop-in API on the GPU against upstream's own outputs (golden fixtures of the 26-orbital
seeded model) and against the oracle.

Tolerances: basis, sparsity pattern and signs bit-exact; H values bit-exact (same
term-order sums); energies 1e-8 eV; spectra 1e-6 relative (max |dg| / max |g|).
"""

import numpy as np
import pytest

import oracle.ed_oracle as O
from impuritymodel_gb300 import finite, spectra
from tests.golden.fixtures import decode_op, decode_psi, decode_restrictions, decode_states, load

pytestmark = pytest.mark.gpu

E_TOL = 1e-8
SPEC_RTOL = 1e-6


@pytest.fixture(scope="module")
def c1():
    z = load("config1.npz")
    n = int(z["n_spin_orbitals"])
    d = dict(
        z=z,
        n=n,
        hop=decode_op(z, "hop"),
        restr=decode_restrictions(z, "restr"),
        basis=tuple(decode_states(z["basis"], n)),
        es=z["es"],
        psis=[decode_psi(z, "eig%d" % i, n) for i in range(len(z["es"]))],
    )
    return d


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_applyop_matches_golden(eng, c1):
    n = c1["n"]
    z = load("applyop_config1.npz")
    psi_in = decode_psi(z, "hpsi_in", n)
    out = finite.applyOp(n, c1["hop"], psi_in, 1e-12, None, None)
    ref = decode_psi(z, "hpsi_out", n)
    assert list(out.keys()) == list(ref.keys())  # same states, same dict order
    a = np.array([out[s] for s in ref])
    b = np.array([ref[s] for s in ref])
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    out = finite.applyOp(n, c1["hop"], psi_in, 1e-12, c1["restr"], None)
    ref = decode_psi(z, "hpsi_restr_out", n)
    assert list(out.keys()) == list(ref.keys())


def test_applyop_memo_matches_golden(eng, c1):
    from impuritymodel_gb300 import models as M

    n = c1["n"]
    z = load("applyop_config1.npz")
    mod = M.make_model("config1")
    tops = mod.xas_ops()
    t_big = {}
    for k, i in enumerate([0, 1, 2, 0]):
        psi = {s: complex(a) for s, a in c1["psis"][i].items()}
        out = finite.applyOp(n, tops[k % 3], psi, 1e-7, c1["restr"], t_big)
        ref = decode_psi(z, "memo%d" % k, n)
        assert set(out) == set(ref)
        a = np.array([out[s] for s in ref])
        b = np.array([ref[s] for s in ref])
        assert np.abs(a - b).max() <= 1e-12


def test_hamiltonian_bit_exact(eng, c1):
    z = c1["z"]
    n = c1["n"]
    h = finite.get_hamiltonian_matrix(n, c1["hop"], c1["basis"]).tocoo()
    ref = {(int(r), int(c)): v for r, c, v in zip(z["h_row"], z["h_col"], z["h_val"])}
    got = {(int(r), int(c)): v for r, c, v in zip(h.row, h.col, h.data)}
    assert set(ref) == set(got)
    assert all(got[k] == ref[k] for k in ref)


def test_expand_basis_matches_golden(eng, c1):
    z = c1["z"]
    n = c1["n"]
    psi1 = decode_psi(z, "psi1", n)
    h_dict = {}
    b = finite.expand_basis(n, h_dict, c1["hop"], tuple(psi1.keys()), c1["restr"])
    assert b == tuple(decode_states(z["exp_basis"], n))
    assert set(h_dict) == set(b)


def test_lanczos_matches_golden(eng, c1):
    """alpha/beta of upstream's plain Lanczos on a 60-state sector with K = dim.

    Without reorthogonalisation the late coefficients amplify rounding, so the first 20
    are compared at 1e-9 and the continued fraction (exact for K = dim) at 1e-6."""
    z = c1["z"]
    n = c1["n"]
    psi1 = decode_psi(z, "psi1", n)
    h, idx = finite.expand_basis_and_hamiltonian(n, {}, c1["hop"], tuple(psi1.keys()), c1["restr"])
    nrm = np.sqrt(finite.norm2(psi1))
    psi0 = np.zeros(len(idx), dtype=complex)
    for s, a in psi1.items():
        psi0[idx[s]] = a / nrm
    alpha, beta = finite.get_tridiagonal_krylov_vectors(h, psi0, 150)
    assert alpha.shape == z["alpha"].shape and beta.shape == z["beta"].shape
    assert np.abs(alpha[:20] - z["alpha"][:20]).max() < 1e-9
    assert np.abs(beta[:20] - z["beta"][:20]).max() < 1e-9
    w = np.linspace(-30, 30, 1500)
    g = O.continued_fraction(alpha, beta, w, 0.1, -700.0)
    g_ref = O.continued_fraction(z["alpha"], z["beta"], w, 0.1, -700.0)
    assert _rel(g, g_ref) < SPEC_RTOL


def test_eigensystem(eng, c1):
    """Energies against upstream (ARPACK) at 1e-8 eV; eigenvectors against the exact dense
    eigenvectors (upstream's own ARPACK vectors are converged only to its tol=1e-9)."""
    n = c1["n"]
    es, psis = finite.eigensystem(n, c1["hop"], c1["basis"], 3)
    assert np.abs(es - c1["es"]).max() < E_TOL
    es_x, psis_x = O.eigensystem(n, c1["hop"], c1["basis"], 3, groundDiagMode="full")
    assert np.abs(es - es_x).max() < E_TOL
    for p, q in zip(psis, psis_x):
        # both dicts drop |amp|^2 < 1e-7 (upstream truncation), so normalise the overlap
        ov = abs(sum(np.conj(q[s]) * p.get(s, 0) for s in q)) / np.sqrt(finite.norm2(p) * finite.norm2(q))
        assert ov > 1 - 1e-9


def test_xas_matches_golden(eng, c1):
    z = c1["z"]
    from impuritymodel_gb300 import models as M

    mod = M.make_model("config1")
    gs = spectra.getSpectra(c1["n"], c1["hop"], mod.xas_ops(), c1["psis"], c1["es"], z["w"], 0.1, c1["restr"])
    assert gs.shape == z["gs_xas"].shape
    assert _rel(gs, z["gs_xas"]) < SPEC_RTOL


def _ensemble(fn, members=4, eps=1e-15):
    """Upstream's algorithm (oracle) rerun with start vectors perturbed at rounding level."""
    return [fn(perturb=(eps, np.random.default_rng(k))) for k in range(members)]


def _accuracy_class(g, ensemble, g_exact, g_ref=None, envelope=5e-3):
    """Krylov results with K < sector dimension.  Upstream's recurrence (no
    reorthogonalisation) turns rounding-level differences into ~1e-4..1e-3 changes of the
    spectrum: the oracle's own RIXS map on this model is 1.4e-4 from the exact resolvent on
    x86-64 and 5.5e-5 on aarch64 (same code, different floating-point contraction).  The
    GPU result must be as close to the exact resolvent as the worst member of an ensemble
    of oracle runs with 1e-15 start-vector perturbations, within that 3x architecture
    spread, and within the envelope of upstream's own (golden) result."""
    e_gpu = _rel(g, g_exact)
    e_ens = max(_rel(x, g_exact) for x in ensemble)
    assert e_gpu <= 3.0 * e_ens + SPEC_RTOL, (e_gpu, e_ens)
    if g_ref is not None:
        assert _rel(g, g_ref) < envelope


def test_ps_ips_match_golden(eng, c1):
    z = c1["z"]
    from impuritymodel_gb300 import models as M

    mod = M.make_model("config1")
    w = z["w"]
    n, hop, restr, psis, es = c1["n"], c1["hop"], c1["restr"], c1["psis"], c1["es"]
    for ops, sign, ref in ((mod.ps_ops()[:3], -1, z["gs_ps"]), (mod.ips_ops()[:3], 1, z["gs_ips"])):
        args = (n, hop, ops, psis, es, sign * w, sign * 0.1, restr)
        gs = spectra.getSpectra(*args)
        gx = O.get_spectra(*args, exact=True)
        ens = _ensemble(lambda perturb: O.get_spectra(*args, perturb=perturb))
        _accuracy_class(gs, ens, gx, ref)


def test_rixs_against_oracle(eng, c1):
    z = c1["z"]
    from impuritymodel_gb300 import models as M

    mod = M.make_model("config1")
    args = (c1["n"], c1["hop"], mod.xas_ops(), mod.rixs_out_ops(), c1["psis"][:1], c1["es"][:1], z["w_in"],
            z["w_loss"], 0.2, 0.05, c1["restr"])
    gs = spectra.getRIXSmap(*args)
    # identical outgoing-channel slices: upstream's shared outgoing memo
    assert np.array_equal(gs[:, :, 0], gs[:, :, 1]) and np.array_equal(gs[:, :, 0], gs[:, :, 2])
    exact = O.get_rixs_map(*args, solver="direct", exact=True)
    ens = _ensemble(lambda perturb: O.get_rixs_map(*args, solver="direct", perturb=perturb), members=3)
    # against upstream's own BiCGSTAB (rtol 1e-5) map: its noise floor
    _accuracy_class(gs, ens, exact, z["gs_rixs"])


def test_double_float_lanczos_tracks_fp64(eng, c1):
    """The double-float Lanczos (precision 3, ~48-bit significands) on the 60-state sector of
    the golden Lanczos case: the first 20 alpha/beta agree with upstream's at 1e-9 like the
    FP64 form, and the continued fraction (K = dim) at 1e-6."""
    z = c1["z"]
    n = c1["n"]
    psi1 = decode_psi(z, "psi1", n)
    dop = finite._device_op(c1["hop"], eng)
    restr = spectra.make_restrictions(c1["restr"], n)
    st, am = spectra._psi_tensors(eng, psi1, n)
    out = {}
    for prec in (0, 3):
        _, (alpha, beta, k_h, _) = spectra.green_batch(eng, dop, restr, [st], [am], [0.0], [0.0], 0.1, 150, prec,
                                                       return_coeffs=True)
        out[prec] = (alpha.cpu().numpy()[0, : k_h[0]], beta.cpu().numpy()[0, : k_h[0]])
    a3, b3 = out[3]
    assert a3.shape == z["alpha"].shape
    assert np.abs(a3[:20] - z["alpha"][:20]).max() < 1e-9
    assert np.abs(b3[:20] - z["beta"][:20]).max() < 1e-9
    assert np.abs(a3[:20] - out[0][0][:20]).max() < 1e-9
    w = np.linspace(-30, 30, 1500)
    g = O.continued_fraction(a3, b3, w, 0.1, -700.0)
    g_ref = O.continued_fraction(z["alpha"], z["beta"], w, 0.1, -700.0)
    assert _rel(g, g_ref) < SPEC_RTOL


@pytest.mark.parametrize("precision", [2, 3])
def test_reduced_forms_accuracy(eng, c1, precision):
    """FP32 continued fractions (2) and double-float Lanczos with FP32 continued fractions
    (3): XAS against upstream at 1e-5 relative (float32 resolvents), PS and RIXS in the
    same accuracy class against the exact resolvent as the FP64 form."""
    z = c1["z"]
    from impuritymodel_gb300 import models as M

    mod = M.make_model("config1")
    n, hop, restr, psis, es = c1["n"], c1["hop"], c1["restr"], c1["psis"], c1["es"]
    gs = spectra.getSpectra(n, hop, mod.xas_ops(), psis, es, z["w"], 0.1, restr, precision=precision)
    assert _rel(gs, z["gs_xas"]) < 1e-5
    args = (n, hop, mod.ps_ops()[:3], psis, es, -z["w"], -0.1, restr)
    gs = spectra.getSpectra(*args, precision=precision)
    gx = O.get_spectra(*args, exact=True)
    ens = _ensemble(lambda perturb: O.get_spectra(*args, perturb=perturb))
    _accuracy_class(gs, ens, gx, z["gs_ps"])
    rargs = (n, hop, mod.xas_ops(), mod.rixs_out_ops(), psis[:1], es[:1], z["w_in"], z["w_loss"], 0.2, 0.05, restr)
    gr = spectra.getRIXSmap(*rargs, precision=precision)
    exact = O.get_rixs_map(*rargs, solver="direct", exact=True)
    ens = _ensemble(lambda perturb: O.get_rixs_map(*rargs, solver="direct", perturb=perturb), members=3)
    _accuracy_class(gr, ens, exact, z["gs_rixs"])
