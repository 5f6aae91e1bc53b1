"""The allocation-free Lanczos entry point (edgpu_lanczos_noalloc) through the C ABI.

Callers that cannot allocate device memory (a host code whose memory manager owns the GPU,
or a solver loop where an allocation would synchronise the device) pass only inputs and
outputs; the library keeps the scratch in a static device array.  Its results must equal
those of edgpu_lanczos with a caller-provided workspace, on two calls in a row (the array
keeps the previous call's contents), and sizes beyond the array are rejected.

Collected last (file name) so that a run stopping at the first failure has already run
every other test.
"""

import ctypes as C

import numpy as np
import pytest
import scipy.sparse
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _hermitian_csr(n, seed, complex_vals):
    rng = np.random.default_rng(seed)
    a = scipy.sparse.random(n, n, density=6.0 / n, random_state=rng, format="csr")
    if complex_vals:
        a = a + 1j * scipy.sparse.random(n, n, density=6.0 / n, random_state=rng, format="csr")
    h = a + a.conj().T + scipy.sparse.diags(rng.uniform(-810.0, -790.0, n))
    h = scipy.sparse.csr_matrix(h)
    h.sort_indices()
    return h


def _device_csr(h, precision, complex_vals, L, dev):
    keep = {}
    keep["rp"] = torch.from_numpy(h.indptr.astype(np.int64)).to(dev)
    keep["col"] = torch.from_numpy(h.indices.astype(np.int32)).to(dev)
    s = L.CSR()
    s.n = h.shape[0]
    s.nnz = h.nnz
    s.row_ptr = keep["rp"].data_ptr()
    s.col = keep["col"].data_ptr()
    data = np.asarray(h.data, dtype=np.complex128)
    if complex_vals:
        t = torch.view_as_real(torch.from_numpy(data).to(dev)).contiguous()
        keep["v"] = t if precision == 0 else t.to(torch.float32)
        if precision == 0:
            s.val_c = keep["v"].data_ptr()
        else:
            s.val_cf = keep["v"].data_ptr()
    else:
        t = torch.from_numpy(np.ascontiguousarray(data.real)).to(dev)
        keep["v"] = t if precision == 0 else t.to(torch.float32)
        if precision == 0:
            s.val_r = keep["v"].data_ptr()
        else:
            s.val_rf = keep["v"].data_ptr()
    return s, keep


@pytest.mark.parametrize("precision,complex_vals", [(0, False), (0, True), (1, False)])
def test_noalloc_lanczos_matches_workspace_entry_point(precision, complex_vals):
    from impuritymodel_gb300 import _lib as L
    from impuritymodel_gb300 import build

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build()
    lib = L.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    # large enough that edgpu_lanczos also takes the grid-wide (scratch-using) path
    n = 6000 if precision == 0 else 9000
    R, K = 3, 60
    h = _hermitian_csr(n, 11 + precision, complex_vals)
    csr, keep = _device_csr(h, precision, complex_vals, L, dev)
    rng = np.random.default_rng(5)
    v0 = rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))
    v0 /= np.linalg.norm(v0, axis=0, keepdims=True)
    v0_t = torch.view_as_real(torch.from_numpy(np.ascontiguousarray(v0)).to(dev)).contiguous()
    kmax = torch.full((R,), K, dtype=torch.int32, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def outputs():
        return (torch.zeros((R, K), dtype=torch.float64, device=dev),
                torch.zeros((R, K), dtype=torch.float64, device=dev),
                torch.zeros(1, dtype=torch.int32, device=dev))

    a_ref, b_ref, st = outputs()
    ws_bytes = lib.edgpu_lanczos_workspace(n, R, K, precision)
    assert ws_bytes <= L.noalloc_bytes()
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    rc = lib.edgpu_lanczos(C.byref(csr), C.c_void_p(v0_t.data_ptr()), R, C.c_void_p(kmax.data_ptr()), K, precision,
                           C.c_void_p(a_ref.data_ptr()), C.c_void_p(b_ref.data_ptr()), C.c_void_p(st.data_ptr()),
                           C.c_void_p(ws.data_ptr()), ws_bytes, stream)
    assert rc == L.EDGPU_OK
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    for _ in range(2):
        a, b, st2 = outputs()
        rc = lib.edgpu_lanczos_noalloc(C.byref(csr), C.c_void_p(v0_t.data_ptr()), R, C.c_void_p(kmax.data_ptr()), K,
                                       precision, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                       C.c_void_p(st2.data_ptr()), stream)
        assert rc == L.EDGPU_OK
        torch.cuda.synchronize()
        assert int(st2.item()) == 0
        np.testing.assert_allclose(a.cpu().numpy(), a_ref.cpu().numpy(), rtol=RTOL, atol=RTOL)
        np.testing.assert_allclose(b[:, : K - 1].cpu().numpy(), b_ref[:, : K - 1].cpu().numpy(), rtol=RTOL,
                                   atol=RTOL)
    # a problem whose scratch exceeds the static array is rejected before anything runs
    big_r = 4096
    assert lib.edgpu_lanczos_workspace(n, big_r, K, precision) > L.noalloc_bytes()
    rc = lib.edgpu_lanczos_noalloc(C.byref(csr), C.c_void_p(v0_t.data_ptr()), big_r, C.c_void_p(kmax.data_ptr()), K,
                                   precision, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                   C.c_void_p(st2.data_ptr()), stream)
    assert rc == L.EDGPU_ERR_WORKSPACE
    del keep
