"""The autotuner's Lanczos launch choice: for a batch of 96 double-float runs on the
26-spin-orbital model's sector, every CTA size gives the same alpha/beta to double-float
precision (only the order of block reductions differs), the tuner records a time for each
and reuses its choice."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_lanczos_cta_choices_agree_and_are_cached(eng):
    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions
    from impuritymodel_gb300.tuner import bucket, get_tuner

    mod = models.make_model("config1")
    n = mod.n_spin_orbitals
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    csr = eng.build_csr(sb.sorted, DeviceOp(mod.hOp, eng.device), make_restrictions(mod.restrictions, n))
    R, K = 96, 60
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    v0 = torch.randn((csr.n, R), dtype=torch.complex128, device="cuda", generator=g)
    v0 /= torch.linalg.vector_norm(v0, dim=0, keepdim=True)
    kmax = np.full(R, K, dtype=np.int32)
    eng.tune_lanczos = False
    ref = eng.lanczos(csr, v0, kmax, precision=3)
    outs = []
    for c in eng.LANCZOS_CTAS:
        eng.lib.edgpu_set_lanczos_cta(c)
        try:
            outs.append(eng.lanczos(csr, v0, kmax, precision=3))
        finally:
            eng.lib.edgpu_set_lanczos_cta(-1)
    for a, b in outs:
        assert torch.allclose(a[:, :30], ref[0][:, :30], rtol=0, atol=1e-9)
        assert torch.allclose(b[:, :30], ref[1][:, :30], rtol=0, atol=1e-9)
    eng.tune_lanczos = True
    a, b = eng.lanczos(csr, v0, kmax, precision=3)
    key = (bucket(csr.n), bucket(R), bucket(K))
    choice = get_tuner().lookup("lanczos_cta", key)
    assert choice is not None and choice[0] in eng.LANCZOS_CTAS
    times = get_tuner().report("lanczos_cta")["lanczos_cta|" + ",".join(str(k) for k in key)]["times_us"]
    assert len(times) == len(eng.LANCZOS_CTAS)
    assert torch.allclose(a[:, :30], ref[0][:, :30], rtol=0, atol=1e-9)
