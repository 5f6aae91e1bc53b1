"""torch.ops.edgpu.* on the GPU: torch.library.opcheck (schema, fake kernel against the real
one, dispatch) for spmv, lanczos and cfrac, and build_csr / expand equal to the engine's
results bit for bit (26-spin-orbital model)."""

import numpy as np
import pytest
import torch

import impuritymodel_gb300  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sector(eng):
    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    mod = models.make_model("config1")
    n = mod.n_spin_orbitals
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    return dict(sb=sb, dop=dop, restr=restr, csr=eng.build_csr(sb.sorted, dop, restr))


def test_opcheck_spmv_lanczos_cfrac(eng, sector):
    csr = sector["csr"]
    n = csr.n
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.randn((n, 4), dtype=torch.complex128, device="cuda", generator=g)
    args = (csr.row_ptr, csr.col, csr.val_r, x)
    torch.library.opcheck(torch.ops.edgpu.spmv.default, args)
    y = torch.ops.edgpu.spmv(*args)
    assert torch.allclose(y, eng.spmv(csr, x), rtol=0, atol=0)
    v0 = x / torch.linalg.vector_norm(x, dim=0, keepdim=True)
    kmax = torch.full((4,), 40, dtype=torch.int32, device="cuda")
    largs = (csr.row_ptr, csr.col, csr.val_r, v0, kmax, 40, 0)
    torch.library.opcheck(torch.ops.edgpu.lanczos.default, largs)
    a, b = torch.ops.edgpu.lanczos(*largs)
    a2, b2 = eng.lanczos(csr, v0, np.full(4, 40, dtype=np.int32))
    assert torch.equal(a, a2) and torch.equal(b, b2)
    om = torch.linspace(-20, 20, 300, dtype=torch.float64, device="cuda")
    e = torch.full((4,), -700.0, dtype=torch.float64, device="cuda")
    sc = torch.ones(4, dtype=torch.float64, device="cuda")
    cargs = (a, b, kmax, om, 0.1, e, sc)
    torch.library.opcheck(torch.ops.edgpu.cfrac.default, cargs)
    gc = torch.ops.edgpu.cfrac(*cargs)
    assert gc.shape == (4, 300) and torch.isfinite(torch.view_as_real(gc)).all()


def test_build_csr_and_expand_ops_equal_engine(eng, sector):
    from impuritymodel_gb300 import ops

    sb, dop, restr = sector["sb"], sector["dop"], sector["restr"]
    lo, hi, mask = ops.restriction_tensors(restr, eng.device)
    rp, col, val = torch.ops.edgpu.build_csr(sb.sorted, *ops.term_tensors(dop), lo, hi, mask, 1e-12)
    ref = sector["csr"]
    assert torch.equal(rp, ref.row_ptr) and torch.equal(col, ref.col) and torch.equal(val, ref.val_r)
    b0 = sb.sorted[:5].contiguous()
    s1, l1 = torch.ops.edgpu.expand(b0, *ops.term_tensors(dop), lo, hi, mask, 1e-12)
    s2, l2 = eng.expand(b0, dop, restr)
    assert torch.equal(s1, s2) and torch.equal(l1, l2)
