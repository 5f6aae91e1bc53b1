"""Ensembles of models (different bath sizes, seeds and Hamiltonians) solved as ragged batches.

Upstream solves one model per program run: ``finite.eigensystem`` (finite.py:58-118) for the
lowest eigenstates, then ``spectra.getSpectra`` (spectra.py:684-806) for XAS.  Here the
sectors of all models are concatenated into one CSR (column indices local to each sector) and
every solve phase is one launch over all models:

* ground states: Lanczos with full reorthogonalisation, one CTA per model
  (``edgpu_lanczos_reorth_ragged``), Ritz pairs of the tridiagonal matrices on the host,
  eigenvectors by one ragged combine launch; models whose lowest Ritz pairs have not
  converged are re-run with a doubled Krylov size;
* XAS: every (model, eigenstate, polarisation) run of upstream's Lanczos recurrence in one
  launch (``edgpu_lanczos_ragged``, vectors in shared memory) and all continued fractions in
  one more; this solve phase can be captured once in a CUDA graph and replayed.

Per-model sector construction (basis, operator application, expansion, CSR) runs the
single-model engine calls.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from . import _lib as L
from .engine import CsrMatrix, get_engine, make_restrictions
from .finite import _device_hamiltonian, _device_op, _SortedBasis, get_basis
from .spectra import green_setup


class RaggedBatch:
    """Concatenated sector CSRs and the run -> sector map of a ragged batch."""

    def __init__(self, eng, csrs, run_sec):
        self.eng = eng
        self.csrs = list(csrs)
        run_sec = np.asarray(run_sec, dtype=np.int32)
        sizes = np.array([c.n for c in self.csrs], dtype=np.int64)
        nnzs = np.array([c.nnz for c in self.csrs], dtype=np.int64)
        for c in self.csrs:
            if c.ncols != c.n:
                raise ValueError("ragged batch: square sector matrices required")
        if run_sec.size and (run_sec.min() < 0 or run_sec.max() >= len(self.csrs)):
            raise ValueError("ragged batch: run sector index out of range")
        dev = eng.device
        nnz_off = np.zeros(len(self.csrs) + 1, dtype=np.int64)
        np.cumsum(nnzs, out=nnz_off[1:])
        parts = [c.row_ptr[:-1] + int(o) for c, o in zip(self.csrs, nnz_off[:-1])]
        parts.append(torch.tensor([int(nnz_off[-1])], dtype=torch.int64, device=dev))
        row_ptr = torch.cat(parts)
        col = torch.cat([c.col for c in self.csrs]) if len(self.csrs) else torch.zeros(0, dtype=torch.int32)
        real = all(c.val_c is None for c in self.csrs)
        if real:
            vals = torch.cat([c.val_r for c in self.csrs])
            self.csr = CsrMatrix(row_ptr, col, val_r=vals)
        else:
            vals = torch.cat([c.val_c if c.val_c is not None else torch.stack([c.val_r, torch.zeros_like(c.val_r)], 1)
                              for c in self.csrs])
            self.csr = CsrMatrix(row_ptr, col, val_c=vals.contiguous())
        self.sec_row0_h = np.zeros(len(self.csrs) + 1, dtype=np.int64)
        np.cumsum(sizes, out=self.sec_row0_h[1:])
        self.run_sec_h = run_sec
        self.run_rows_h = sizes[run_sec] if run_sec.size else np.zeros(0, dtype=np.int64)
        self.run_vec0_h = np.zeros(run_sec.size + 1, dtype=np.int64)
        np.cumsum(self.run_rows_h, out=self.run_vec0_h[1:])
        self.n_runs = int(run_sec.size)
        self.max_rows = int(self.run_rows_h.max()) if run_sec.size else 1
        self.sec_row0 = torch.from_numpy(self.sec_row0_h).to(dev)
        self.run_sec = torch.from_numpy(run_sec).to(dev)
        self.run_vec0 = torch.from_numpy(self.run_vec0_h).to(dev)
        s = L.Ragged()
        s.n_sectors = len(self.csrs)
        s.n_runs = self.n_runs
        s.sec_row0 = self.sec_row0.data_ptr()
        s.run_sec = self.run_sec.data_ptr()
        s.run_vec0 = self.run_vec0.data_ptr()
        s.max_rows = self.max_rows
        self._struct = s

    def struct(self):
        return self._struct

    def run_slice(self, r):
        return slice(int(self.run_vec0_h[r]), int(self.run_vec0_h[r + 1]))


def _random_start(eng, n, seed):
    g = torch.Generator(device=eng.device)
    g.manual_seed(int(seed))
    v = torch.randn(n, dtype=torch.complex128, device=eng.device, generator=g)
    return v / torch.linalg.vector_norm(v)


class ModelSectors:
    """Per-model ground-state data: operator table, sorted basis and Hamiltonian."""

    def __init__(self, eng, model):
        self.model = model
        self.n_spin_orbitals = model.n_spin_orbitals
        self.dop = _device_op(model.hOp, eng)
        self.sb = _SortedBasis(eng, list(get_basis(*model.basis_args())), self.n_spin_orbitals)
        self.csr = _device_hamiltonian(eng, self.dop, self.sb)
        self.restr = make_restrictions(model.restrictions, self.n_spin_orbitals)


def ensemble_ground_states(eng, sectors, n_states=3, k_start=120, tol_rel=1e-12, seed=0, slaterWeightMin=1e-7):
    """Lowest ``n_states`` eigenpairs of every model, one ragged launch per round.

    A model's Ritz pairs are accepted when ``beta_K |s_{K,i}| <= tol_rel * max(1, |theta_i|)``
    for the wanted i (the criterion of the single-model eig_lowest) or the Krylov space spans
    its basis; the others are re-run with twice the Krylov size.  Returns (energies list of
    [q] arrays, psis list of lists of (states [m, W], amps [m, 2]) keeping
    ``|amp|^2 >= slaterWeightMin`` as upstream's eigensystem).
    """
    M = len(sectors)
    energies = [None] * M
    psis = [None] * M
    todo = list(range(M))
    k_cap = int(k_start)
    while todo:
        batch = RaggedBatch(eng, [sectors[i].csr for i in todo], np.arange(len(todo)))
        k = np.array([min(k_cap, sectors[i].csr.n) for i in todo], dtype=np.int32)
        v0 = torch.cat([_random_start(eng, sectors[i].csr.n, seed + i) for i in todo])
        V, run_V0, alpha, beta = eng.lanczos_reorth_ragged(batch, v0, k)
        a_h, b_h = alpha.cpu().numpy(), beta.cpu().numpy()
        Q = n_states
        S = np.zeros((len(todo), int(k.max()), Q))
        retry = []
        done = []
        for r, i in enumerate(todo):
            kr = int(k[r])
            if kr == 1:
                th, s = a_h[r, :1].copy(), np.ones((1, 1))
            else:
                th, s = scipy.linalg.eigh_tridiagonal(a_h[r, :kr], b_h[r, : kr - 1])
            q = min(Q, kr)
            res = np.abs(b_h[r, kr - 1] * s[kr - 1, :q])
            exact = kr >= sectors[i].csr.n
            if exact or bool(np.all(res <= tol_rel * np.maximum(1.0, np.abs(th[:q])))):
                S[r, :kr, :q] = s[:, :q]
                energies[i] = th[:q].copy()
                done.append((r, i, q))
            else:
                retry.append(i)
        if done:
            X = eng.combine_ragged(batch, V, run_V0, k, S)
            _ritz_states(eng, sectors, batch, X, Q, done, slaterWeightMin, psis)
        if retry and k_cap >= max(sectors[i].csr.n for i in retry):
            raise RuntimeError("ensemble ground states: no convergence at the full basis size")
        todo = retry
        k_cap *= 2
    return energies, psis


def _ritz_states(eng, sectors, batch, X, Q, done, slaterWeightMin, psis):
    """psis[i] = [(states, amps)] of the converged models' Ritz vectors, all at once: the
    vectors (segments of X) padded into one [segments, max rows] array, normalised, pruned at
    |amp|^2 < slaterWeightMin with one nonzero, then split per (model, state) with one host
    read of the segment counts."""
    dev = eng.device
    # models grouped by state width (words per state), each group's bases concatenated: the
    # segments of a group are then contiguous in the nonzero output and gather from one array
    done = sorted(done, key=lambda d: int(sectors[d[1]].sb.sorted.shape[1]))
    seg_model, seg_base, seg_n, seg_q, row0, seg_group = [], [], [], [], [], []
    groups = []  # (width, [bases])
    off = 0
    for r, i, q in done:
        b = sectors[i].sb.sorted
        if not groups or groups[-1][0] != int(b.shape[1]):
            groups.append((int(b.shape[1]), []))
            off = 0
        n = sectors[i].csr.n
        base = Q * int(batch.run_vec0_h[r])
        for qq in range(q):
            seg_model.append(i)
            seg_base.append(base + qq * n)
            seg_n.append(n)
            seg_q.append(qq)
            row0.append(off)
            seg_group.append(len(groups) - 1)
        groups[-1][1].append(b)
        off += n
    ns = len(seg_n)
    width = max(seg_n)
    n_h = np.asarray(seg_n, dtype=np.int64)
    cols = torch.arange(width, device=dev).view(1, -1)
    nt = torch.from_numpy(n_h).to(dev).view(-1, 1)
    valid = cols < nt
    src = torch.from_numpy(np.asarray(seg_base, dtype=np.int64)).to(dev).view(-1, 1) + cols
    P = torch.where(valid, X[src.clamp(max=X.numel() - 1)], torch.zeros((), dtype=X.dtype, device=dev))
    P = P / torch.linalg.vector_norm(P, dim=1, keepdim=True)
    keep = valid & ((P.real ** 2 + P.imag ** 2) >= slaterWeightMin)
    seg, col = torch.nonzero(keep, as_tuple=True)  # grouped by segment, rows in order
    counts = torch.bincount(seg, minlength=ns).cpu().numpy()
    rows = torch.from_numpy(np.asarray(row0, dtype=np.int64)).to(dev)[seg] + col
    am = torch.view_as_real(P[seg, col]).contiguous()
    am_parts = torch.split(am, counts.tolist())
    ends = np.cumsum(counts)
    gseg = np.asarray(seg_group)
    st_parts = []
    for g, (_, bs) in enumerate(groups):
        segs = np.nonzero(gseg == g)[0]
        lo = int(ends[segs[0]] - counts[segs[0]])
        hi = int(ends[segs[-1]])
        st_g = torch.cat(bs, 0)[rows[lo:hi]]
        st_parts += list(torch.split(st_g, counts[segs].tolist()))
    for t, i in enumerate(seg_model):
        if seg_q[t] == 0:
            psis[i] = []
        psis[i].append((st_parts[t].contiguous(), am_parts[t].contiguous()))


class RaggedSpectra:
    """Lanczos + continued fractions of a ragged batch with every input on the device.

    ``run()`` enqueues the two launches; ``capture()`` records them once in a CUDA graph and
    ``replay()`` re-issues the graph (inputs and outputs stay at the same addresses)."""

    def __init__(self, eng, batch, v0, k, omega, delta, e, scale):
        self.eng = eng
        self.batch = batch
        dev = eng.device
        self.v0 = v0
        k = np.asarray(k, dtype=np.int32)
        self.K = int(k.max()) if k.size else 1
        self.k = torch.from_numpy(k).to(dev)
        self.om = torch.from_numpy(np.ascontiguousarray(omega, dtype=np.float64)).to(dev)
        self.e = torch.from_numpy(np.ascontiguousarray(e, dtype=np.float64)).to(dev)
        self.scale = torch.from_numpy(np.ascontiguousarray(scale, dtype=np.float64)).to(dev)
        self.delta = float(delta)
        self.alpha = torch.zeros((batch.n_runs, self.K), dtype=torch.float64, device=dev)
        self.beta = torch.zeros((batch.n_runs, self.K), dtype=torch.float64, device=dev)
        self.g = torch.empty((batch.n_runs, self.om.numel()), dtype=torch.complex128, device=dev)
        self.graph = None

    def run(self, check=True):
        self.eng.lanczos_ragged(self.batch, self.v0, self.k, self.alpha, self.beta, check=False)
        self.eng.cfrac_device(self.alpha, self.beta, self.k, self.om, self.delta, self.e, self.scale, self.g)
        if check:
            self.eng.read_status("ragged spectra")
        return self.g

    def capture(self):
        self.run()  # warm-up outside the capture (kernel attributes, lazy module loading)
        side = torch.cuda.Stream(device=self.eng.device)
        side.wait_stream(torch.cuda.current_stream(self.eng.device))
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                self.run(check=False)
        torch.cuda.current_stream(self.eng.device).wait_stream(side)
        return self

    def replay(self, check=True):
        self.graph.replay()
        if check:
            self.eng.read_status("ragged spectra (graph)")
        return self.g


def ensemble_xas_setup(eng, sectors, energies, psis, omega, delta, krylovSize=150, slaterWeightMin=1e-7):
    """Start vectors and the ragged batch of the XAS runs of every model.

    Runs of model m are ordered (eigenstate q, polarisation t), as upstream's getSpectra
    result gs[q, t, w].  Returns (RaggedSpectra, run_map) with run_map[m] = (live run
    indices into the solve, number of (q, t) slots)."""
    csrs, run_sec, v0_parts, ks, es, scales, run_map = [], [], [], [], [], [], []
    n_live = 0
    for m, sec in enumerate(sectors):
        t_dops = [_device_op(t, eng) for t in sec.model.xas_ops()]
        ps = psis[m]
        run_states, run_amps, e_runs = [], [], []
        # every polarisation on every eigenstate in one pass (one scan, one sort, one unique)
        per_t = eng.apply_vectors_multi([p[0] for p in ps], [p[1] for p in ps], t_dops, sec.restr, slaterWeightMin)
        for q in range(len(ps)):
            for t in range(len(t_dops)):
                o_s, o_a = per_t[t][q]
                run_states.append(o_s)
                run_amps.append(o_a)
                e_runs.append(float(energies[m][q]))
        st = green_setup(eng, sec.dop, sec.restr, run_states, run_amps, krylovSize)
        slots = len(run_states)
        if st is None:
            run_map.append((np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64), slots))
            continue
        s_idx = len(csrs)
        csrs.append(st.sector.csr)
        L_m = st.live.size
        run_sec.extend([s_idx] * L_m)
        v0_parts.append(st.v0.t().contiguous().reshape(-1))
        ks.append(st.k)
        es.append(np.asarray(e_runs, dtype=np.float64)[st.live])
        scales.append(st.scale[st.live])
        run_map.append((np.arange(n_live, n_live + L_m), st.live, slots))
        n_live += L_m
    batch = RaggedBatch(eng, csrs, run_sec)
    v0 = torch.cat(v0_parts) if v0_parts else torch.zeros(0, dtype=torch.complex128, device=eng.device)
    solve = RaggedSpectra(eng, batch, v0, np.concatenate(ks) if ks else np.zeros(0, np.int32), omega, delta,
                          np.concatenate(es) if es else np.zeros(0), np.concatenate(scales) if scales else np.zeros(0))
    return solve, run_map


def scatter_xas(g, run_map, n_states, n_ops, n_omega):
    """Per-model host arrays gs[q, t, w] from the ragged solve's output rows."""
    g_h = g.cpu().numpy()
    out = []
    for rows, live, slots in run_map:
        a = np.zeros((slots, n_omega), dtype=np.complex128)
        if rows.size:
            a[live] = g_h[rows]
        out.append(a.reshape(-1, n_ops, n_omega))
    return out


def ensemble_gs_xas(models, omega, delta, n_states=3, krylovSize=150, slaterWeightMin=1e-7, graph=False):
    """Lowest eigenstates and their XAS Green's functions for every model of an ensemble.

    Returns (energies list, gs list with gs[m] [q, t, w] complex128 host arrays)."""
    eng = get_engine()
    sectors = [ModelSectors(eng, m) for m in models]
    energies, psis = ensemble_ground_states(eng, sectors, n_states, slaterWeightMin=slaterWeightMin)
    solve, run_map = ensemble_xas_setup(eng, sectors, energies, psis, omega, delta, krylovSize, slaterWeightMin)
    if graph:
        solve.capture()
        g = solve.replay()
    else:
        g = solve.run()
    n_ops = len(models[0].xas_ops()) if models else 0
    return energies, scatter_xas(g, run_map, n_states, n_ops, len(np.atleast_1d(omega)))
