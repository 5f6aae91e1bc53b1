"""The path driven through the C ABI alone, as a non-Python host would: expand -> build CSR ->
lowest eigenpairs -> Lanczos -> continued fraction, each one library call (torch only holds
the buffers), against upstream's own outputs for the 26-spin-orbital model
(tests/golden/config1.npz): the expanded basis in upstream's order, bit for bit; energies at
1e-8 eV; the first 20 Lanczos coefficients at 1e-9 and the continued fraction (Krylov size =
dimension) at 1e-6 relative.  The CSR is also compared bit for bit with the Python engine's.
"""

import ctypes as C

import numpy as np
import pytest
import torch

import oracle.ed_oracle as O
from tests.golden.fixtures import decode_op, decode_psi, decode_restrictions, decode_states, load

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def _words(states, n):
    return torch.from_numpy(O.bytes_to_words(list(states), n).view(np.int64)).cuda()


@pytest.fixture(scope="module")
def cfg(eng):
    from impuritymodel_gb300 import _lib as L
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    z = load("config1.npz")
    n = int(z["n_spin_orbitals"])
    hop = decode_op(z, "hop")
    restr = decode_restrictions(z, "restr")
    return dict(L=L, lib=L.load(), z=z, n=n, dop=DeviceOp(hop, eng.device), restr=make_restrictions(restr, n),
                stream=C.c_void_p(torch.cuda.current_stream().cuda_stream))


def _expand(c, basis0_words, capacity=4096, emit_cap=1024):
    L, lib = c["L"], c["lib"]
    w = basis0_words.shape[1]
    out_s = torch.empty((capacity, w), dtype=torch.int64, device="cuda")
    out_l = torch.empty((capacity, w), dtype=torch.int64, device="cuda")
    n_out = C.c_int64(0)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    wsn = lib.edgpu_expand_workspace(w, capacity, emit_cap)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    rc = lib.edgpu_expand(w, C.byref(c["dop"].terms), C.byref(c["restr"]), 1e-12, _p(basis0_words),
                          basis0_words.shape[0], capacity, emit_cap, _p(out_s), _p(out_l), C.byref(n_out), _p(st),
                          _p(ws), wsn, c["stream"])
    assert rc == L.EDGPU_OK, rc
    return out_s[: n_out.value], out_l[: n_out.value]


def _build_csr(c, basis_sorted, real=True):
    L, lib = c["L"], c["lib"]
    n, w = basis_sorted.shape
    rp = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    nnz = C.c_int64(0)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    wsn = lib.edgpu_build_csr_workspace(w, n, 0)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    rc = lib.edgpu_build_csr(w, C.byref(c["dop"].terms), C.byref(c["restr"]), 1e-12, _p(basis_sorted), n, int(real),
                             _p(rp), None, None, 0, C.byref(nnz), _p(st), _p(ws), wsn, c["stream"])
    assert rc == L.EDGPU_ERR_OVERFLOW and nnz.value > 0  # the size query
    col = torch.empty(nnz.value, dtype=torch.int32, device="cuda")
    val = torch.empty(nnz.value if real else (nnz.value, 2), dtype=torch.float64, device="cuda")
    wsn = lib.edgpu_build_csr_workspace(w, n, nnz.value)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    rc = lib.edgpu_build_csr(w, C.byref(c["dop"].terms), C.byref(c["restr"]), 1e-12, _p(basis_sorted), n, int(real),
                             _p(rp), _p(col), _p(val), nnz.value, C.byref(nnz), _p(st), _p(ws), wsn, c["stream"])
    assert rc == L.EDGPU_OK, rc
    s = L.CSR()
    s.n, s.nnz = n, nnz.value
    s.row_ptr, s.col = rp.data_ptr(), col.data_ptr()
    if real:
        s.val_r = val.data_ptr()
    else:
        s.val_c = val.data_ptr()
    return s, (rp, col, val)


def test_capi_expand_matches_upstream_order(eng, cfg):
    z, n = cfg["z"], cfg["n"]
    psi1 = decode_psi(z, "psi1", n)
    srt, lay = _expand(cfg, _words(psi1.keys(), n))
    ref = decode_states(z["exp_basis"], n)
    got = O.words_to_bytes(lay.cpu().numpy().view(np.uint64), n)
    assert got == ref
    assert O.words_to_bytes(srt.cpu().numpy().view(np.uint64), n) == sorted(ref)
    # small emit capacity: the frontier is split into chunks, same result
    srt2, lay2 = _expand(cfg, _words(psi1.keys(), n), emit_cap=16)
    assert torch.equal(srt, srt2) and torch.equal(lay, lay2)


def test_capi_csr_eig_lanczos_cfrac(eng, cfg):
    from impuritymodel_gb300.engine import CsrMatrix

    L, lib, z, n = cfg["L"], cfg["lib"], cfg["z"], cfg["n"]
    basis = decode_states(z["basis"], n)
    sb = _words(sorted(basis), n)
    csr, keep = _build_csr(cfg, sb)
    # bit for bit the Python engine's CSR
    ref = eng.build_csr(sb, cfg["dop"], cfg["restr"])
    assert torch.equal(keep[0], ref.row_ptr) and torch.equal(keep[1], ref.col) and torch.equal(keep[2], ref.val_r)
    # lowest three eigenpairs
    k, k_cap = 3, 190
    evals = (C.c_double * k)()
    evecs = torch.empty((k, sb.shape[0], 2), dtype=torch.float64, device="cuda")
    k_found = C.c_int(0)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    wsn = lib.edgpu_eig_lowest_workspace(sb.shape[0], k_cap)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    rc = lib.edgpu_eig_lowest(C.byref(csr), k, 1e-12, k_cap, 7, evals, _p(evecs), C.byref(k_found), _p(st), _p(ws),
                              wsn, cfg["stream"])
    assert rc == L.EDGPU_OK and k_found.value == k, rc
    es = np.array(evals[:k])
    assert np.abs(es - z["es"]).max() < 1e-8
    # eigenvectors: residual of H X = X diag(es) through the engine's product
    X = torch.view_as_complex(evecs).t().contiguous()
    HX = eng.spmv(CsrMatrix(keep[0], keep[1], val_r=keep[2]), X)
    res = (HX - X * torch.from_numpy(es).cuda()).abs().max().item()
    assert res < 1e-6
    # Lanczos on the closure of psi1 (upstream's golden run) and its continued fraction
    psi1 = decode_psi(z, "psi1", n)
    srt, _ = _expand(cfg, _words(psi1.keys(), n))
    csr2, keep2 = _build_csr(cfg, srt)
    rows = O.words_to_bytes(srt.cpu().numpy().view(np.uint64), n)
    idx = {s: i for i, s in enumerate(rows)}
    nrm = np.sqrt(sum(abs(a) ** 2 for a in psi1.values()))
    v0 = np.zeros(len(rows), dtype=np.complex128)
    for s, a in psi1.items():
        v0[idx[s]] = a / nrm
    v0t = torch.view_as_real(torch.from_numpy(v0).cuda()).contiguous()
    K = len(rows)
    kmax = torch.full((1,), K, dtype=torch.int32, device="cuda")
    alpha = torch.zeros((1, K), dtype=torch.float64, device="cuda")
    beta = torch.zeros((1, K), dtype=torch.float64, device="cuda")
    st.zero_()
    wsn = lib.edgpu_lanczos_workspace(K, 1, K, 0)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    rc = lib.edgpu_lanczos(C.byref(csr2), _p(v0t), 1, _p(kmax), K, 0, _p(alpha), _p(beta), _p(st), _p(ws), wsn,
                           cfg["stream"])
    assert rc == L.EDGPU_OK
    a = alpha.cpu().numpy()[0]
    b = beta.cpu().numpy()[0]
    assert np.abs(a[:20] - z["alpha"][:20]).max() < 1e-9 and np.abs(b[:20] - z["beta"][:20]).max() < 1e-9
    w = np.linspace(-30, 30, 1500)
    om = torch.from_numpy(w).cuda()
    e = torch.tensor([-700.0], dtype=torch.float64, device="cuda")
    sc = torch.ones(1, dtype=torch.float64, device="cuda")
    g = torch.empty((1, w.size, 2), dtype=torch.float64, device="cuda")
    rc = lib.edgpu_cfrac(_p(alpha), _p(beta), _p(kmax), K, 1, _p(om), w.size, 0.1, _p(e), _p(sc), _p(g),
                         cfg["stream"])
    assert rc == L.EDGPU_OK
    gc = torch.view_as_complex(g).cpu().numpy()[0]
    g_ref = O.continued_fraction(z["alpha"], z["beta"], w, 0.1, -700.0)
    assert np.abs(gc - g_ref).max() < 1e-6 * np.abs(g_ref).max()
