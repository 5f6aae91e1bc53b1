"""Basis-pruning network kernels on the GPU: the tcgen05 BF16 GEMM against exact integer
products, and (below) the forward/backward passes against the NumPy oracle."""

import numpy as np
import pytest
import torch

from impuritymodel_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _ptr(t):
    return t.data_ptr()


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (256, 64, 320), (384, 48, 128), (128, 16, 64), (256, 320, 256)])
def test_gemm_bf16_exact(eng, M, N, K):
    """Small integers are exact in BF16 and their products' sums exact in FP32, so the tensor
    core result must equal the integer product bit for bit (checks operand layouts,
    descriptors and the accumulator read-back)."""
    rng = np.random.default_rng(M + N + K)
    a = rng.integers(-4, 5, size=(M, K)).astype(np.float32)
    b = rng.integers(-4, 5, size=(N, K)).astype(np.float32)
    A = torch.from_numpy(a).to(eng.device).to(torch.bfloat16).contiguous()
    B = torch.from_numpy(b).to(eng.device).to(torch.bfloat16).contiguous()
    C = torch.full((M, N), np.nan, dtype=torch.float32, device=eng.device)
    eng.reset_status()
    L.check(eng.lib.edgpu_gemm_bf16(_ptr(A), _ptr(B), M, N, K, _ptr(C), _ptr(eng.status), eng.stream), "gemm")
    eng.read_status("gemm")
    assert np.array_equal(C.cpu().numpy(), a @ b.T)
