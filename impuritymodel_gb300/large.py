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
import time

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


LEAD_RATIO = 4.0  # an orbital moved by this many times the median count of terms is a lead orbital


def locality_order(basis, dop, ratio=LEAD_RATIO):
    """Row order of a sector in which states linked by the Hamiltonian sit near each other.

    The lead orbitals (those that far more off-diagonal terms move than the median orbital:
    the impurity's, in these models, where a 3d spin-orbital appears in hundreds of Coulomb
    and hybridisation terms and a bath spin-orbital in its hybridisation pair) become the
    least significant part of the sort key.  States that agree on every other orbital (one
    bath configuration) then form one contiguous block of rows; a term that moves only lead
    orbitals links rows of the same block, and a hybridisation term links two blocks whose
    rows it pairs up in order.  The product H·x then gathers each x row for many entries of
    nearby rows (cache reuse) instead of once per entry from far apart.

    ``basis`` [n, W] int64 sorted product states.  Returns the permutation (new position ->
    sorted index, int64 on the basis' device) or None when no orbital stands out (the sorted
    order is kept)."""
    moves = np.asarray(dop.moves)
    nz = moves[moves > 0]
    if nz.size == 0:
        return None
    lead = np.nonzero(moves > ratio * np.median(nz))[0]
    if lead.size == 0 or lead.size == nz.size:
        return None
    n, W = basis.shape
    mask = np.zeros(W, dtype=np.uint64)
    for o in lead:
        if o // 64 < W:
            mask[o // 64] |= np.uint64(1) << np.uint64(63 - o % 64)
    m = torch.from_numpy(mask.view(np.int64)).to(basis.device)
    top = torch.tensor(-(1 << 63), dtype=torch.int64, device=basis.device)  # unsigned order as signed
    major = torch.bitwise_xor(torch.bitwise_and(basis, torch.bitwise_not(m)), top)
    minor = torch.bitwise_xor(torch.bitwise_and(basis, m), top)
    order = torch.arange(n, dtype=torch.int64, device=basis.device)
    # lexicographic on (major words, minor words): stable sorts from the least significant word
    for key, skip in ((minor, mask == 0), (major, mask == np.uint64(0xFFFFFFFFFFFFFFFF))):
        for q in reversed(range(W)):
            if skip[q]:
                continue
            order = order[torch.sort(key[order, q], stable=True).indices]
    return order


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


def lanczos_reorth_batched(eng, apply_h, v0, K, precision=1, shift=0.0, reorth="dgks", stats=None):
    """Batched Lanczos with full reorthogonalisation against the whole basis, for R runs at
    once.

    ``reorth="dgks"`` (default): each step first takes the three-term recurrence (alpha'_j =
    v_j^H w, w -= alpha'_j v_j + beta_{j-1} v_{j-1}), then one classical Gram-Schmidt pass
    against every basis vector, and a second pass only for a step where the first removed
    more than half of |w|^2 (the criterion of Daniel, Gragg, Kaufman and Stewart, 1976, with
    eta = 1/sqrt(2); by Pythagoras |w_before|^2 = beta^2 + |h|^2, so the test is |h|^2 >
    beta^2 for some run); the basis is read twice per step.  ``reorth="cgs2"``: two full
    classical Gram-Schmidt passes every step (the basis read four times per step).

    ``v0`` [n, R] complex128, each column normalised; ``apply_h(x, y)`` writes y = (H - shift)
    x for [n, R] vectors of the run dtype (complex64 for ``precision=1``, complex128 for 0).
    ``stats`` (a dict, optional) accumulates ``second_passes``: the steps that took a second
    Gram-Schmidt pass.  Returns (alpha [R, K], beta [R, K] host float64 with ``shift`` added
    back to alpha, k_len [R]: the Krylov size of each run, cut at its first zero beta)."""
    if reorth not in ("dgks", "cgs2"):
        raise ValueError("reorth must be 'dgks' or 'cgs2'")
    n, R = v0.shape
    dt = torch.complex64 if precision else torch.complex128
    K = int(min(K, n))
    V = torch.zeros((K, n, R), dtype=dt, device=eng.device)
    V[0] = v0.to(dt)
    w = torch.empty((n, R), dtype=dt, device=eng.device)
    h1 = torch.zeros((K, K, R), dtype=torch.complex128, device=eng.device)
    h2 = torch.zeros((K, K, R), dtype=torch.complex128, device=eng.device)
    ha = torch.zeros((K, R), dtype=torch.complex128, device=eng.device)  # three-term alpha'
    h3 = torch.zeros((2, R), dtype=torch.complex128, device=eng.device)  # [beta_{j-1}, alpha'_j]
    beta = torch.zeros((K, R), dtype=torch.float64, device=eng.device)
    scratch = torch.empty((n, R), dtype=dt, device=eng.device)
    ws, wsn = eng.workspace(eng.lib.edgpu_krylov_workspace(n, R, K))
    eng.reset_status()
    stride = n * R
    lib = eng.lib
    wr = _ptr(torch.view_as_real(w))

    def vp(k):
        return _ptr(torch.view_as_real(V[k]))

    def dot(k0, m, hrow):
        L.check(lib.edgpu_krylov_dot(precision, vp(k0), stride, m, n, R, wr, _ptr(torch.view_as_real(hrow)), ws, wsn,
                                     eng.stream), "krylov_dot")

    def project(k0, m, hrows, with_norm):
        L.check(lib.edgpu_krylov_project(precision, vp(k0), stride, m, n, R, _ptr(torch.view_as_real(hrows)), wr,
                                         with_norm, ws, wsn, eng.stream), "krylov_project")

    def normalize(dst, j):
        L.check(lib.edgpu_krylov_normalize(precision, n, R, wr, _ptr(torch.view_as_real(dst)), _ptr(beta[j]),
                                           _ptr(eng.status), ws, wsn, eng.stream), "krylov_normalize")

    second = 0
    for j in range(K):
        apply_h(V[j], w)
        m = j + 1
        dst = V[j + 1] if j + 1 < K else scratch
        if reorth == "cgs2":
            for hbuf, last in ((h1, 0), (h2, 1)):
                dot(0, m, hbuf[j])
                project(0, m, hbuf[j], last)
            normalize(dst, j)
            continue
        dot(j, 1, ha[j])
        if j == 0:
            project(0, 1, ha[0:1], 0)
        else:
            h3[0].copy_(beta[j - 1])
            h3[1].copy_(ha[j])
            project(j - 1, 2, h3, 0)
        dot(0, m, h1[j])
        project(0, m, h1[j], 1)
        normalize(dst, j)
        if bool(((h1[j].real ** 2 + h1[j].imag ** 2).sum(0) > beta[j] ** 2).any()):
            dot(0, m, h2[j])
            project(0, m, h2[j], 1)
            normalize(dst, j)
            second += 1
    idx = torch.arange(K, device=eng.device)
    alpha = (ha.real + h1[idx, idx].real + h2[idx, idx].real).t().contiguous() + shift
    a = alpha.cpu().numpy()
    b = beta.t().contiguous().cpu().numpy()
    k_len = np.full(R, K, dtype=np.int32)
    for r in range(R):
        z = np.nonzero(b[r] == 0.0)[0]
        if z.size:
            k_len[r] = int(z[0]) + 1
    if stats is not None:
        stats["second_passes"] = stats.get("second_passes", 0) + second
    return a, b, k_len


def ordered_sector(eng, sector, dop, order=True):
    """(basis [n, W] in the row order the recurrence runs in, the permutation new -> sorted
    index or None) of a sector; the locality order of :func:`locality_order` when ``order``,
    else the sorted order.  Cached on the sector."""
    cache = sector.__dict__.setdefault("_large", {})
    key = ("order", bool(order))
    if key not in cache:
        perm = locality_order(sector.basis, dop) if order else None
        basis = sector.basis if perm is None else sector.basis[perm].contiguous()
        cache[key] = (basis, perm)
    return cache[key]


def _sector_operator(eng, sector, dop, mop, order, precision, matfree):
    """apply_h(x, y) writing (H - shift) x in the sector's run order, and the shift; the
    pieces (diagonal, hash table, reordered CSR and its float copies) are cached on the
    sector."""
    basis, perm = ordered_sector(eng, sector, dop, order)
    cache = sector.__dict__["_large"]
    if precision and matfree:
        key = ("matfree", perm is not None, id(mop))
        if key not in cache:
            diag = hv_diag(eng, basis, mop)
            cache[key] = (diag, float(diag.mean().item()), state_hash(eng, basis))
        diag, shift, table = cache[key]
        restr = cache.get("restr")

        def apply_h(x, y):
            hv_matfree_into(eng, basis, mop, restr, diag, x, y, shift, table)
        return apply_h, shift
    key = ("csr", perm is not None)
    if key not in cache:
        cache[key] = sector.csr if perm is None else sector.csr.permuted(perm, "locality")
    csr = cache[key]
    if precision:
        csr.mixed()

        def apply_h(x, y):
            eng.spmv_into(csr, torch.view_as_real(x), torch.view_as_real(y), x.shape[1], precision=1)
        return apply_h, csr.mixed_shift

    def apply_h(x, y):
        if eng.spmv_planned_ok(x.shape[1], 0):
            eng.spmv_into(csr, torch.view_as_real(x), torch.view_as_real(y), x.shape[1], precision=0)
        else:
            y.copy_(eng.spmv(csr, x))
    return apply_h, 0.0


def green_large(eng, dop, mop, restr, sector, v0, scale, e_runs, omega, delta, K=150, precision=1, matfree=False,
                order=False, stats=None):
    """Continued-fraction Green's functions of R normalised start vectors ``v0`` [n, R] on a
    large ``sector`` (its sorted basis and, for the CSR path, its Hamiltonian).

    ``precision=1``: complex64 vectors, H from the complex64 CSR copy (or matrix-free with
    ``matfree``, for sectors whose matrix is not to be stored), FP64 reductions;
    ``precision=0``: complex128 vectors on the FP64 CSR (the reference).
    ``order``: the recurrence runs on the rows in :func:`locality_order` (v0 is permuted in,
    the coefficients do not depend on the row order).  Returns (g [R, n_omega] complex128
    host, alpha, beta, k_len)."""
    sector.__dict__.setdefault("_large", {})["restr"] = restr
    apply_h, shift = _sector_operator(eng, sector, dop, mop, order, precision, matfree)
    _, perm = ordered_sector(eng, sector, dop, order)
    if perm is not None:
        v0 = v0[perm]
    return _green_ordered(eng, apply_h, shift, v0, scale, e_runs, omega, delta, K, precision, stats)


def _green_ordered(eng, apply_h, shift, v0, scale, e_runs, omega, delta, K, precision, stats=None):
    """green_large after the row order and the operator are fixed."""
    # the H.v kernels serve R / (complex numbers per 16 bytes) lanes per row, a divisor of
    # 32: the run count is padded with empty runs (they stop at their first step)
    R = v0.shape[1]
    runs16 = 2 if precision else 1
    if R > 32 * runs16:  # more runs than one H.v launch serves: in chunks
        parts = [_green_ordered(eng, apply_h, shift, v0[:, c:c + 32 * runs16], scale[c:c + 32 * runs16],
                                e_runs[c:c + 32 * runs16], omega, delta, K, precision, stats)
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
    a, b, k_len = lanczos_reorth_batched(eng, apply_h, v0, K, precision, shift, stats=stats)
    a, b, k_len = a[:R], b[:R], k_len[:R]
    at = torch.from_numpy(np.ascontiguousarray(a)).to(eng.device)
    bt = torch.from_numpy(np.ascontiguousarray(b)).to(eng.device)
    g = eng.cfrac(at, bt, k_len, omega, delta, np.asarray(e_runs, dtype=np.float64),
                  np.asarray(scale, dtype=np.float64))
    return eng.to_host(g), a, b, k_len


def spectra_large(eng, dop, mop, restr, t_dops, psi_t, es, w, delta, K=150, precision=1, matfree=False,
                  slaterWeightMin=1e-7, sector=None, order=False):
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
    sector_s = 0.0
    if sector is None:
        t0 = time.perf_counter()
        sector = Sector(eng, dop, restr, torch.cat(states, 0))
        torch.cuda.synchronize(eng.device)
        sector_s = time.perf_counter() - t0
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
    stats = {}
    gr, a, b, k_len = green_large(eng, dop, mop, restr, sector, v0, scale, e_runs, w, delta, K, precision, matfree,
                                  order, stats)
    for r, (i, o) in enumerate(runs):
        g[i, o] = gr[r]
    return g, {"runs": R, "sector": int(n), "k_len": [int(x) for x in k_len], "sector_obj": sector,
               "sector_s": sector_s, "second_passes": stats.get("second_passes", 0)}
