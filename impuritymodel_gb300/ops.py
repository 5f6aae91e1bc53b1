"""PyTorch custom operators over the C ABI: ``torch.ops.edgpu.*``.

The device entry points of the engine as dispatcher operators with fake (meta) kernels, so
that tensor programs (``torch.compile``, tracing, ``torch.library.opcheck``) can call them;
the work runs in ``libedgpu.so`` on the current stream.  Sparse matrices travel as their CSR
tensors (``row_ptr`` int64 [n + 1], ``col`` int32 [nnz], ``val`` float64 [nnz] for a real H or
[nnz, 2] for complex), product states as int64 [N, W] word tensors, operators as the three
term-table tensors of ``edgpu_terms`` (``ops`` int64, ``coeff`` float64 [T, 2], ``flags``
int32) and restrictions as ``lo``/``hi`` int32 [r] with ``mask`` int64 [r, 8].

Upstream counterparts: ``spmv`` is h.dot of get_tridiagonal_krylov_vectors
(impurityModel/ed/finite.py:1946-1989), ``lanczos`` that function itself (finite.py:1897-1995),
``cfrac`` the continued fraction of getGreen (spectra.py:678-680), ``build_csr``
get_hamiltonian_matrix (finite.py:1514-1610) and ``expand`` expand_basis (finite.py:1696-1803).
"""



import torch
from torch import Tensor

from . import _lib as L


def _engine():
    from .engine import get_engine

    return get_engine()


def _csr(row_ptr, col, val, ncols=None):
    from .engine import CsrMatrix

    if val.dim() == 2:
        return CsrMatrix(row_ptr, col, val_c=val, ncols=ncols)
    return CsrMatrix(row_ptr, col, val_r=val, ncols=ncols)


class _TermView:
    """An operator given as term-table tensors, shaped like DeviceOp for the engine."""

    def __init__(self, ops, coeff, flags):
        self.ops, self.coeff, self.flags = ops, coeff, flags
        self.n_terms = int(ops.numel())
        self.is_real = bool((coeff[:, 1] == 0).all().item()) if self.n_terms else True
        self.terms = L.Terms(ops.data_ptr() if self.n_terms else 0, coeff.data_ptr() if self.n_terms else 0,
                             flags.data_ptr() if self.n_terms else 0, self.n_terms)


def _restr(lo, hi, mask):
    if lo.numel() == 0:
        return None
    r = L.Restrictions()
    lo_h, hi_h, m_h = lo.cpu().tolist(), hi.cpu().tolist(), mask.cpu().tolist()
    if len(lo_h) > L.MAX_RESTRICTIONS:
        raise ValueError("at most %d restrictions are supported" % L.MAX_RESTRICTIONS)
    r.n = len(lo_h)
    for k in range(r.n):
        r.lo[k], r.hi[k] = int(lo_h[k]), int(hi_h[k])
        for q in range(L.MAX_WORDS):
            r.mask[k][q] = int(m_h[k][q]) & 0xFFFFFFFFFFFFFFFF
    return r


@torch.library.custom_op("edgpu::spmv", mutates_args=())
def spmv(row_ptr: Tensor, col: Tensor, val: Tensor, x: Tensor) -> Tensor:
    """y [n, R] = H x for x [ncols, R] complex128."""
    eng = _engine()
    return eng.spmv(_csr(row_ptr, col, val, ncols=x.shape[0]), x.contiguous())


@spmv.register_fake
def _(row_ptr, col, val, x):
    return x.new_empty((row_ptr.shape[0] - 1, x.shape[1]))


@torch.library.custom_op("edgpu::lanczos", mutates_args=())
def lanczos(row_ptr: Tensor, col: Tensor, val: Tensor, v0: Tensor, k_max: Tensor, K: int,
            precision: int) -> tuple[Tensor, Tensor]:
    """Batched Lanczos (upstream's recurrence) of R normalised start vectors v0 [n, R]
    complex128; k_max int32 [R] (each <= K).  Returns alpha, beta float64 [R, K]."""
    eng = _engine()
    csr = _csr(row_ptr, col, val)
    k_h = k_max.to("cpu", torch.int32)
    if int(k_h.max()) != K:
        raise ValueError("lanczos: K must equal max(k_max)")
    return eng.lanczos(csr, v0.contiguous(), k_h.numpy(), precision=precision)


@lanczos.register_fake
def _(row_ptr, col, val, v0, k_max, K, precision):
    r = v0.shape[1]
    return v0.new_empty((r, K), dtype=torch.float64), v0.new_empty((r, K), dtype=torch.float64)


@torch.library.custom_op("edgpu::cfrac", mutates_args=())
def cfrac(alpha: Tensor, beta: Tensor, k_len: Tensor, omega: Tensor, delta: float, e: Tensor,
          scale: Tensor) -> Tensor:
    """Continued fractions g [R, n_omega] complex128 of the R runs' alpha/beta [R, K]."""
    eng = _engine()
    r, K = alpha.shape
    g = torch.empty((r, omega.numel()), dtype=torch.complex128, device=alpha.device)
    return eng.cfrac_device(alpha.contiguous(), beta.contiguous(), k_len.to(torch.int32).contiguous(),
                            omega.contiguous(), float(delta), e.contiguous(), scale.contiguous(), g)


@cfrac.register_fake
def _(alpha, beta, k_len, omega, delta, e, scale):
    return alpha.new_empty((alpha.shape[0], omega.numel()), dtype=torch.complex128)


@torch.library.custom_op("edgpu::build_csr", mutates_args=())
def build_csr(basis: Tensor, ops: Tensor, coeff: Tensor, flags: Tensor, lo: Tensor, hi: Tensor, mask: Tensor,
              weight_min: float) -> tuple[Tensor, Tensor, Tensor]:
    """Sector Hamiltonian on a sorted basis [n, W]: (row_ptr, col, val); val float64 [nnz] when
    every coefficient is real, else [nnz, 2]."""
    eng = _engine()
    csr = eng.build_csr(basis.contiguous(), _TermView(ops, coeff, flags), _restr(lo, hi, mask), weight_min)
    val = csr.val_r if csr.val_r is not None else csr.val_c
    return csr.row_ptr, csr.col, val


@build_csr.register_fake
def _(basis, ops, coeff, flags, lo, hi, mask, weight_min):
    nnz = torch.library.get_ctx().new_dynamic_size()
    rp = basis.new_empty((basis.shape[0] + 1,), dtype=torch.int64)
    return rp, basis.new_empty((nnz,), dtype=torch.int32), basis.new_empty((nnz,), dtype=torch.float64)


@torch.library.custom_op("edgpu::expand", mutates_args=())
def expand(basis0: Tensor, ops: Tensor, coeff: Tensor, flags: Tensor, lo: Tensor, hi: Tensor, mask: Tensor,
           weight_min: float) -> tuple[Tensor, Tensor]:
    """Closure of basis0 [n0, W]: (sorted basis, upstream's layered order), both [N, W]."""
    eng = _engine()
    return eng.expand(basis0.contiguous(), _TermView(ops, coeff, flags), _restr(lo, hi, mask), weight_min)


@expand.register_fake
def _(basis0, ops, coeff, flags, lo, hi, mask, weight_min):
    n = torch.library.get_ctx().new_dynamic_size()
    return basis0.new_empty((n, basis0.shape[1])), basis0.new_empty((n, basis0.shape[1]))


def term_tensors(dop):
    """(ops, coeff, flags) tensors of a compiled operator (engine.DeviceOp)."""
    return dop.ops, dop.coeff, dop.flags


def restriction_tensors(restr, device):
    """(lo, hi, mask) tensors of an edgpu_restrictions structure (or None)."""
    if restr is None:
        return (torch.zeros(0, dtype=torch.int32, device=device), torch.zeros(0, dtype=torch.int32, device=device),
                torch.zeros((0, L.MAX_WORDS), dtype=torch.int64, device=device))
    n = int(restr.n)
    lo = torch.tensor([restr.lo[k] for k in range(n)], dtype=torch.int32, device=device)
    hi = torch.tensor([restr.hi[k] for k in range(n)], dtype=torch.int32, device=device)
    m = [[int(restr.mask[k][q]) for q in range(L.MAX_WORDS)] for k in range(n)]
    mask = torch.tensor([[x - (1 << 64) if x >= (1 << 63) else x for x in row] for row in m], dtype=torch.int64,
                        device=device)
    return lo, hi, mask
