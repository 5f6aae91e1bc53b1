"""Large sectors: matrix-free H·v and the batched reorthogonalised Lanczos in complex64 or
complex128 with FP64-accumulated reductions, and Green's functions on them.

For the 316-spin-orbital model (300 bath spin-orbitals, at most two bath holes) the
photoemission and core-hole sectors hold 2.9e5-4.6e5 states.  There:

* H is applied matrix-free (``edgpu_hv_matfree``): the diagonal is summed once per sector,
  the off-diagonal terms are bucketed by the orbital they fill, and each row applies only the
  buckets of its empty orbitals, looks the results up in the sorted basis and gathers x;
* the Krylov recurrence keeps its vectors in complex64 (``precision=1``) with every
  reduction (alpha, beta, the Gram-Schmidt dot products) accumulated in FP64 and two
  Gram-Schmidt passes per step against the whole basis, because a complex64 recurrence
  without reorthogonalisation loses orthogonality within a few dozen steps;
* the same recurrence in complex128 on the CSR Hamiltonian is the FP64 reference the
  complex64 spectra are judged against (per-spectrum relative L1 error).

Upstream computes these Green's functions with getGreen (impurityModel/ed/spectra.py:551-681)
on sparse matrices built from applyOp, and the Lanczos coefficients with
get_tridiagonal_krylov_vectors (impurityModel/ed/finite.py:1897-1995) without
reorthogonalisation.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .engine import DeviceOp, _ptr


class MatfreeOp:
    """An operator dict split for matrix-free application: diagonal terms (a product state
    onto itself) and off-diagonal terms bucketed by key orbital (the first orbital a term
    creates without annihilating it; the term can act only where that orbital is empty).
    Within each part the upstream term order is kept."""

    def __init__(self, op, n_orb, device):
        diag, off = {}, []
        for pos, (key, v) in enumerate(op.items()):
            cre = [int(i) for i, a in key if a == "c"]
            ann = [int(i) for i, a in key if a == "a"]
            if sorted(cre) == sorted(ann):
                diag[key] = v
                continue
            keys = [i for i in cre if i not in ann]
            if not keys:
                raise ValueError("matrix-free application needs every off-diagonal term to create an electron")
            off.append((keys[0], pos, key, v))
        off.sort(key=lambda t: (t[0], t[1]))
        self.n_orb = int(n_orb)
        if any(k >= self.n_orb for k, _, _, _ in off):
            raise ValueError("term orbital beyond the spin-orbital count")
        self.diag = DeviceOp(diag, device)
        self.off = DeviceOp({key: v for _, _, key, v in off}, device)
        counts = np.bincount(np.array([k for k, _, _, _ in off], dtype=np.int64), minlength=self.n_orb)
        bucket = np.zeros(self.n_orb + 1, dtype=np.int32)
        bucket[1:] = np.cumsum(counts)
        self.bucket = torch.from_numpy(bucket).to(device)
        self.is_real = self.diag.is_real and self.off.is_real


def hv_diag(eng, basis_sorted, mop):
    """Diagonal of H on a sorted basis (FP64, [n])."""
    n, w = basis_sorted.shape
    d = torch.empty(n, dtype=torch.float64, device=eng.device)
    L.check(eng.lib.edgpu_hv_diag(w, _ptr(basis_sorted), n, C.byref(mop.diag.terms), _ptr(d), eng.stream), "hv_diag")
    return d


def state_hash(eng, basis_sorted):
    """Hash table of the basis states (int32 slots, a power of two >= 2n) for matrix-free
    lookups."""
    n, w = basis_sorted.shape
    size = 1 << max(4, int(2 * n - 1).bit_length())
    table = torch.empty(size, dtype=torch.int32, device=eng.device)
    L.check(eng.lib.edgpu_state_hash_build(w, _ptr(basis_sorted), n, _ptr(table), size, eng.stream), "state_hash")
    return table


def hv_matfree_into(eng, basis_sorted, mop, restr, diag, x, y, shift=0.0, table=None):
    """y = (H - shift I) x for x, y [n, R] complex (complex64 or complex128), matrix-free;
    ``table`` (from :func:`state_hash`) replaces the binary searches by hash lookups."""
    n, w = basis_sorted.shape
    R = x.shape[1]
    rp = C.byref(restr) if restr is not None else None
    if x.dtype == torch.complex64:
        fn = eng.lib.edgpu_hv_matfree_c64
    else:
        fn = eng.lib.edgpu_hv_matfree
    tsize = 0 if table is None else int(table.numel())
    L.check(fn(w, _ptr(basis_sorted), n, _ptr(table), tsize, mop.n_orb, _ptr(mop.bucket), C.byref(mop.off.terms),
               0 if mop.off.is_real else 1, rp, _ptr(diag), float(shift), _ptr(torch.view_as_real(x)),
               _ptr(torch.view_as_real(y)), R, eng.stream), "hv_matfree")
    return y


def lanczos_reorth_batched(eng, apply_h, v0, K, precision=1, shift=0.0):
    """Batched Lanczos with two classical Gram-Schmidt passes per step against the whole
    basis, for R runs at once.

    ``v0`` [n, R] complex128, each column normalised; ``apply_h(x, y)`` writes y = (H - shift)
    x for [n, R] vectors of the run dtype (complex64 for ``precision=1``, complex128 for 0).
    Returns (alpha [R, K], beta [R, K] host float64 with ``shift`` added back to alpha,
    k_len [R]: the Krylov size of each run, cut at its first zero beta)."""
    n, R = v0.shape
    dt = torch.complex64 if precision else torch.complex128
    K = int(min(K, n))
    V = torch.zeros((K, n, R), dtype=dt, device=eng.device)
    V[0] = v0.to(dt)
    w = torch.empty((n, R), dtype=dt, device=eng.device)
    h1 = torch.zeros((K, K, R), dtype=torch.complex128, device=eng.device)
    h2 = torch.zeros((K, K, R), dtype=torch.complex128, device=eng.device)
    beta = torch.zeros((K, R), dtype=torch.float64, device=eng.device)
    scratch = torch.empty((n, R), dtype=dt, device=eng.device)
    ws, wsn = eng.workspace(eng.lib.edgpu_krylov_workspace(n, R, K))
    eng.reset_status()
    stride = n * R
    Vp = torch.view_as_real(V)
    lib = eng.lib
    for j in range(K):
        apply_h(V[j], w)
        m = j + 1
        for hbuf, last in ((h1, False), (h2, True)):
            L.check(lib.edgpu_krylov_dot(precision, _ptr(Vp), stride, m, n, R, _ptr(torch.view_as_real(w)),
                                         _ptr(torch.view_as_real(hbuf[j])), ws, wsn, eng.stream), "krylov_dot")
            L.check(lib.edgpu_krylov_project(precision, _ptr(Vp), stride, m, n, R,
                                             _ptr(torch.view_as_real(hbuf[j])), _ptr(torch.view_as_real(w)),
                                             1 if last else 0, ws, wsn, eng.stream), "krylov_project")
        dst = V[j + 1] if j + 1 < K else scratch
        L.check(lib.edgpu_krylov_normalize(precision, n, R, _ptr(torch.view_as_real(w)),
                                           _ptr(torch.view_as_real(dst)), _ptr(beta[j]), _ptr(eng.status), ws, wsn,
                                           eng.stream), "krylov_normalize")
    idx = torch.arange(K, device=eng.device)
    alpha = (h1[idx, idx].real + h2[idx, idx].real).t().contiguous() + shift
    a = alpha.cpu().numpy()
    b = beta.t().contiguous().cpu().numpy()
    k_len = np.full(R, K, dtype=np.int32)
    for r in range(R):
        z = np.nonzero(b[r] == 0.0)[0]
        if z.size:
            k_len[r] = int(z[0]) + 1
    return a, b, k_len


def green_large(eng, dop, mop, restr, sector, v0, scale, e_runs, omega, delta, K=150, precision=1, matfree=True):
    """Continued-fraction Green's functions of R normalised start vectors ``v0`` [n, R] on a
    large ``sector`` (its sorted basis and, for the CSR path, its Hamiltonian).

    ``precision=1``: complex64 vectors, H matrix-free (or the complex64 CSR copy), FP64
    reductions; ``precision=0``: complex128 vectors on the FP64 CSR (the reference).  Returns
    (g [R, n_omega] complex128 host, alpha, beta, k_len)."""
    csr = sector.csr
    shift = 0.0
    if precision:
        if matfree:
            diag = hv_diag(eng, sector.basis, mop)
            shift = float(diag.mean().item())
            table = state_hash(eng, sector.basis)

            def apply_h(x, y):
                hv_matfree_into(eng, sector.basis, mop, restr, diag, x, y, shift, table)
        else:
            csr.mixed()
            shift = csr.mixed_shift

            def apply_h(x, y):
                eng.spmv_into(csr, torch.view_as_real(x), torch.view_as_real(y), x.shape[1], precision=1)
    else:
        def apply_h(x, y):
            if eng.spmv_planned_ok(x.shape[1], 0):
                eng.spmv_into(csr, torch.view_as_real(x), torch.view_as_real(y), x.shape[1], precision=0)
            else:
                y.copy_(eng.spmv(csr, x))
    # the H.v kernels serve R / (complex numbers per 16 bytes) lanes per row, a divisor of
    # 32: the run count is padded with empty runs (they stop at their first step)
    R = v0.shape[1]
    runs16 = 2 if precision else 1
    if R > 32 * runs16:  # more runs than one H.v launch serves: in chunks
        parts = [green_large(eng, dop, mop, restr, sector, v0[:, c:c + 32 * runs16], scale[c:c + 32 * runs16],
                             e_runs[c:c + 32 * runs16], omega, delta, K, precision, matfree)
                 for c in range(0, R, 32 * runs16)]
        Kc = max(p[1].shape[1] for p in parts)
        pad = lambda x: np.pad(x, ((0, 0), (0, Kc - x.shape[1])))  # noqa: E731
        return (np.concatenate([p[0] for p in parts]), np.concatenate([pad(p[1]) for p in parts]),
                np.concatenate([pad(p[2]) for p in parts]), np.concatenate([p[3] for p in parts]))
    Rp = runs16
    while Rp < R:
        Rp *= 2
    if Rp != R:
        v0 = torch.cat([v0, torch.zeros((v0.shape[0], Rp - R), dtype=v0.dtype, device=v0.device)], 1)
    a, b, k_len = lanczos_reorth_batched(eng, apply_h, v0, K, precision, shift)
    a, b, k_len = a[:R], b[:R], k_len[:R]
    at = torch.from_numpy(np.ascontiguousarray(a)).to(eng.device)
    bt = torch.from_numpy(np.ascontiguousarray(b)).to(eng.device)
    g = eng.cfrac(at, bt, k_len, omega, delta, np.asarray(e_runs, dtype=np.float64),
                  np.asarray(scale, dtype=np.float64))
    return eng.to_host(g), a, b, k_len


def spectra_large(eng, dop, mop, restr, t_dops, psi_t, es, w, delta, K=150, precision=1, matfree=True,
                  slaterWeightMin=1e-7, sector=None):
    """Spectra ``g[n_states, n_ops, n_w]`` of transition operators on large sectors (upstream
    getSpectra, impurityModel/ed/spectra.py:684-806: T psi, normalised, Green's function
    scaled by the squared norm), every (operator, state) run in one batched recurrence on the
    closure of all start states.  Returns (g host complex128, info dict: sector size, runs,
    Krylov sizes, the sector object for reuse)."""
    from .spectra import Sector

    ne, no = len(es), len(t_dops)
    t_outs = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t], t_dops, restr, slaterWeightMin)
    states, amps, runs = [], [], []
    for o, outs in enumerate(t_outs):
        for i, (s_, a_) in enumerate(outs):
            if s_.shape[0]:
                states.append(s_)
                amps.append(a_)
                runs.append((i, o))
    g = np.zeros((ne, no, len(w)), dtype=np.complex128)
    if not runs:
        return g, {"runs": 0}
    if sector is None:
        sector = Sector(eng, dop, restr, torch.cat(states, 0))
    n = sector.n
    R = len(runs)
    v0 = torch.zeros((n, R), dtype=torch.complex128, device=eng.device)
    scale = np.zeros(R)
    for r, (s_, a_) in enumerate(zip(states, amps)):
        rows = eng.lookup(sector.basis, s_)
        vals = torch.complex(a_[:, 0], a_[:, 1])
        nrm = float(torch.linalg.vector_norm(vals).item())
        scale[r] = nrm * nrm
        v0[rows, r] = vals / nrm
    e_runs = [es[i] for i, _ in runs]
    gr, a, b, k_len = green_large(eng, dop, mop, restr, sector, v0, scale, e_runs, w, delta, K, precision, matfree)
    for r, (i, o) in enumerate(runs):
        g[i, o] = gr[r]
    return g, {"runs": R, "sector": int(n), "k_len": [int(x) for x in k_len], "sector_obj": sector}
