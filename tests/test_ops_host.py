"""The torch.ops.edgpu.* operators without a GPU: they are registered with the dispatcher and
their fake kernels give the output shapes and dtypes (what tracing and torch.compile see)."""

import torch
from torch._subclasses.fake_tensor import FakeTensorMode

import impuritymodel_gb300  # noqa: F401  (registers the operators)


def test_operators_are_registered():
    for name in ("spmv", "lanczos", "cfrac", "build_csr", "expand"):
        assert hasattr(torch.ops.edgpu, name), name


def test_fake_kernels_shapes():
    with FakeTensorMode(allow_non_fake_inputs=False, shape_env=None):
        n, nnz, R, K, nw = 100, 700, 4, 30, 50
        rp = torch.empty(n + 1, dtype=torch.int64)
        col = torch.empty(nnz, dtype=torch.int32)
        val = torch.empty(nnz, dtype=torch.float64)
        x = torch.empty((n, R), dtype=torch.complex128)
        y = torch.ops.edgpu.spmv(rp, col, val, x)
        assert y.shape == (n, R) and y.dtype == torch.complex128
        a, b = torch.ops.edgpu.lanczos(rp, col, val, x, torch.empty(R, dtype=torch.int32), K, 0)
        assert a.shape == (R, K) and b.shape == (R, K) and a.dtype == torch.float64
        g = torch.ops.edgpu.cfrac(a, b, torch.empty(R, dtype=torch.int32), torch.empty(nw, dtype=torch.float64), 0.1,
                                  torch.empty(R, dtype=torch.float64), torch.empty(R, dtype=torch.float64))
        assert g.shape == (R, nw) and g.dtype == torch.complex128
