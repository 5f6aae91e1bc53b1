"""Drop-in replacement of upstream ``impurityModel.ed.spectra`` Green's functions and RIXS.

``getGreen``, ``getSpectra`` and ``getRIXSmap`` keep upstream's signatures and results
(``impurityModel/ed/spectra.py:551-1130``).  Internally every Green's function of one call
is one run of a batched Lanczos on a single device sector:

* the sector is the closure under H (with restrictions) of the union of all runs' start
  states — the closure of a union is the union of the per-run closures upstream builds,
  and H has no entries leaving a closure, so each run's Krylov space is unchanged;
* each run keeps upstream's Krylov size ``min(krylovSize, dim of its own closure)``, from
  the connected components of the sector graph;
* continued fractions for all runs and frequencies run in one kernel.

RIXS solves ``(w_in + i delta1 + e - H) x = psi1`` for all incoming energies from one
Krylov space per (in-operator, eigenstate) (full reorthogonalisation, FP64, relative
residual ``solve_tol``) instead of one BiCGSTAB per energy at rtol 1e-5.

``precision=1`` selects the mixed form: complex64 Lanczos vectors and H values with
float32 SpMV accumulation, float64 alpha/beta reductions, float32 continued fractions.
``precision=2`` keeps the Krylov recurrences in FP64 and evaluates only the continued
fractions in float32 (after forming alpha - e in FP64).
``precision=3`` runs the Lanczos recurrences of real Hamiltonians in double-float
arithmetic (unevaluated float pairs, ~48 significand bits, FP64 alpha/beta reductions) and
the continued fractions in float32 as in ``precision=2``.
"""

from __future__ import annotations

import math

import numpy as np
import scipy.linalg
import torch

from . import _lib as L
from . import codec
from .engine import _restr_key, get_engine, make_restrictions, words_for
from .finite import _device_op
from .models import (  # noqa: F401  (upstream names re-exported)
    K_B,
    daggered_dipole_ops as getDaggeredDipoleOperators,
    dipole_op as getDipoleOperator,
    dipole_ops as getDipoleOperators,
    inverse_photoemission_ops as getInversePhotoEmissionOperators,
    nixs_op as getNIXSOperator,
    photoemission_ops as getPhotoEmissionOperators,
)


def getNIXSOperators(nBaths, qs, li, lj, Ri, Rj, r, kmin=1):
    """NIXS operators for each momentum transfer (upstream spectra.py:385-434)."""
    return [getNIXSOperator(nBaths, q, li, lj, Ri, Rj, r, kmin) for q in qs]


def thermal_average(energies, observable, T=300):
    """Boltzmann average over eigenstates (upstream impurityModel/ed/average.py:11-45)."""
    energies = np.asarray(energies)
    if len(energies) != np.shape(observable)[0]:
        raise ValueError("Passed array is not of the right shape")
    shift = np.min(energies)
    z = 0.0
    acc = 0
    for e, o in zip(energies, observable):
        wgt = np.exp(-(e - shift) / (K_B * T))
        z += wgt
        acc = acc + wgt * np.asarray(o)
    return acc / z


# ---------------------------------------------------------------------------------------
# Batched Green's functions on one sector
# ---------------------------------------------------------------------------------------


class Sector:
    """Sorted device basis + CSR Hamiltonian of a closure."""

    def __init__(self, eng, dop, restr, start_states, precision=0):
        self.basis, _ = eng.expand(eng.sort_unique(start_states), dop, restr)
        self.csr = eng.build_csr(self.basis, dop, restr)
        if precision == 1:
            self.csr.mixed()
        self.n = self.basis.shape[0]
        self._labels = None
        self._sizes = None

    @classmethod
    def from_parts(cls, basis, csr):
        """A sector from a sorted basis and its Hamiltonian built elsewhere."""
        s = cls.__new__(cls)
        s.basis, s.csr, s.n = basis, csr, basis.shape[0]
        s._labels = None
        s._sizes = None
        return s

    def components(self, eng):
        """Component label of every state (its smallest member) and the size of each component
        stored at its label's index (0 elsewhere); no host synchronisation."""
        if self._labels is None:
            labels = eng.components(self.csr)
            sizes = torch.zeros(self.n, dtype=torch.int64, device=eng.device)
            sizes.index_add_(0, labels, torch.ones_like(labels))
            self._labels, self._sizes = labels, sizes
        return self._labels, self._sizes

    def run_dims(self, eng, rows, run_of_row, runs):
        """Closure dimension of each run's support (upstream len(basis_index) per getGreen):
        the summed sizes of the distinct components its start states touch."""
        labels, sizes = self.components(eng)
        n = self.n
        comp = labels[rows]
        if runs * n <= (1 << 26):
            touched = torch.zeros((runs, n), dtype=torch.bool, device=eng.device)
            touched[run_of_row, comp] = True
            return (touched.to(torch.int64) * sizes.view(1, -1)).sum(1)
        pair = torch.unique(run_of_row * n + comp)
        dims = torch.zeros(runs, dtype=torch.int64, device=eng.device)
        dims.index_add_(0, pair // n, sizes[pair % n])
        return dims


def _popcount64(x):
    """Bit counts of a uint64 array (SWAR, no numpy version requirement)."""
    x = x.astype(np.uint64)
    x = x - ((x >> np.uint64(1)) & np.uint64(0x5555555555555555))
    x = (x & np.uint64(0x3333333333333333)) + ((x >> np.uint64(2)) & np.uint64(0x3333333333333333))
    x = (x + (x >> np.uint64(4))) & np.uint64(0x0F0F0F0F0F0F0F0F)
    return ((x * np.uint64(0x0101010101010101)) >> np.uint64(56)).astype(np.int64)


def closed_sector(eng, dop, restr, basis_sorted, csr, words_host):
    """The sector of ``basis_sorted`` (device, sorted) with its Hamiltonian ``csr`` when every
    basis state satisfies the restrictions and H (restricted) maps the basis into itself; else
    None.  Such a basis contains the closure of any of its states (upstream expand_basis,
    finite.py:1696-1803) as a union of its connected components, with the same Hamiltonian
    rows, so Green's-function runs that start inside it can use it instead of a fresh
    expansion.  ``words_host``: the basis as host uint64 words (any order)."""
    from . import _lib as L

    if restr is not None:
        w = np.asarray(words_host, dtype=np.uint64)
        for k in range(int(restr.n)):
            cnt = np.zeros(w.shape[0], dtype=np.int64)
            for q in range(w.shape[1]):
                cnt += _popcount64(w[:, q] & np.uint64(restr.mask[k][q] & 0xFFFFFFFFFFFFFFFF))
            if np.any(cnt < int(restr.lo[k])) or np.any(cnt > int(restr.hi[k])):
                return None
    offsets, _, _, _ = eng.apply_columns(basis_sorted, dop, restr, 1e-12, basis=basis_sorted,
                                         filt=L.FILTER_NOT_IN_BASIS)
    if int(offsets[-1].item()) != 0:
        return None
    return Sector.from_parts(basis_sorted, csr)


class GreenSetup:
    """Start vectors of a batch of Green's-function runs on one sector (see green_setup)."""

    def __init__(self, runs, live, sector, v0, k, scale):
        self.runs = runs  # runs requested
        self.live = live  # host indices of runs with a nonzero start state
        self.sector = sector
        self.v0 = v0  # [sector.n, len(live)] complex128
        self.k = k  # host Krylov sizes of the live runs
        self.scale = scale  # host scale of every run (normalisation**2 or the given scales)


def green_setup(eng, dop, restr, run_states, run_amps, krylovSize=150, precision=0, sector=None, normalize=True,
                scales=None, perturb=None, stages=None, sector_hint=None):
    """Sector, start vectors and Krylov sizes of a batch of Green's-function runs.

    ``run_states[r]`` [n_r, W] / ``run_amps[r]`` [n_r, 2] are the start states (lists), or
    ``run_states`` is a packed ``(states [M, W], amps [M, 2], run_of_row [M], n_runs)``
    tuple with ``run_amps`` None.  With ``normalize=True`` each start state is normalised
    and its squared norm becomes the run's scale (upstream
    ``normalization**2 * getGreen(psi / normalization)``, spectra.py:786-802).  With
    ``normalize=False`` the start states are used as given (upstream getGreen on an arbitrary
    psi) and ``scales[r]`` (default 1) is the scale.  Each run's Krylov size is upstream's
    ``min(krylovSize, dim of its own closure)``.  Returns a GreenSetup, or None when every
    start state is empty.
    """
    if run_amps is None:
        states, amps, run_of_row, runs = run_states
    else:
        runs = len(run_states)
        if runs == 0:
            return None
        sizes = torch.tensor([int(x.shape[0]) for x in run_states], device=eng.device)
        states = torch.cat(run_states, 0)
        amps = torch.cat(run_amps, 0)
        run_of_row = torch.repeat_interleave(torch.arange(runs, device=eng.device), sizes,
                                             output_size=int(states.shape[0]))
    n2 = torch.zeros(runs, dtype=torch.float64, device=eng.device)
    if amps.shape[0]:
        # per-run squared norms as segment sums in a fixed order (rows are grouped by run), so
        # reruns give identical bits (an atomic scatter-add would not)
        a2 = torch.stack([amps[:, 0] ** 2 + amps[:, 1] ** 2, torch.zeros_like(amps[:, 0])], 1).contiguous()
        rk, _, s2 = eng.unique_sorted(run_of_row.view(-1, 1).contiguous(), None, a2)
        n2[rk[:, 0]] = s2[:, 0]
    n2_h = n2.cpu().numpy()
    live = np.nonzero(n2_h > 0)[0]
    if live.size == 0:
        return None
    _mark(stages, "green:norms")
    hinted = sector is None and sector_hint is not None
    if hinted:
        sector = sector_hint  # used when it holds every start state (checked below)
    if sector is None:
        sector = Sector(eng, dop, restr, states[n2[run_of_row] > 0], precision)
    _mark(stages, "green:sector")
    rows = eng.lookup(sector.basis, states)
    missing = (rows < 0).any()  # checked with the run dimensions below (one synchronisation)
    # live runs renumbered 0..L-1
    remap = torch.full((runs,), -1, dtype=torch.int64, device=eng.device)
    live_t = torch.from_numpy(live).to(eng.device)
    remap[live_t] = torch.arange(live.size, device=eng.device)
    lr = remap[run_of_row]
    sel = lr >= 0
    vals = torch.complex(amps[:, 0], amps[:, 1])
    if normalize:
        norm = torch.sqrt(n2)
        vals = vals / torch.where(norm > 0, norm, torch.ones_like(norm))[run_of_row]
        scale_h = n2_h
    else:
        scale_h = np.ones(runs) if scales is None else np.asarray(scales, dtype=np.float64)
    v0 = torch.zeros((sector.n, live.size), dtype=torch.complex128, device=eng.device)
    # a run's start states are distinct (dict keys, or unique outputs of an operator
    # application), so every (row, run) pair is written once: a plain scatter
    v0[rows[sel].clamp_min(0), lr[sel]] = vals[sel]
    if perturb is not None:
        # verification only: relative start-vector perturbation (eps, seed) to measure how
        # much the unreorthogonalised recurrence amplifies rounding-level differences
        eps, seed = perturb
        gen = torch.Generator(device=eng.device)
        gen.manual_seed(int(seed))
        v0 = v0 * (1.0 + eps * torch.randn(v0.shape, dtype=torch.float64, device=eng.device, generator=gen))
    _mark(stages, "green:v0")
    dims = sector.run_dims(eng, rows[sel].clamp_min(0), lr[sel], int(live.size))
    dims_h = torch.cat([dims, missing.view(1).to(torch.int64)]).cpu().numpy()
    if dims_h[-1] and hinted:
        return green_setup(eng, dop, restr, run_states, run_amps, krylovSize, precision, None, normalize, scales,
                           perturb, stages)
    if dims_h[-1]:
        raise RuntimeError("start state outside the sector basis")
    k_h = np.minimum(dims_h[:-1], int(krylovSize)).astype(np.int32)
    _mark(stages, "green:run_dims")
    return GreenSetup(runs, live, sector, v0, k_h, scale_h)


def _drive(steps):
    """Run a pipeline step generator to completion and return its value."""
    while True:
        try:
            next(steps)
        except StopIteration as done:
            return done.value


def run_concurrently(eng, jobs):
    """Run pipeline step generators side by side on one GPU and return their values.

    Job 0 runs on the current stream, job k > 0 on the engine's k-th high-priority side
    stream, which first waits for the work already queued on the current stream (the jobs'
    inputs).  A job yields right after it enqueues a long GPU operation whose result it needs
    next; the host then advances the next job, whose launches and synchronisations stay on
    its own stream, instead of idling until the long operation ends.  The current stream
    waits for every side stream before this returns, and the returned device tensors are
    marked as used on it.
    """
    main = torch.cuda.current_stream(eng.device)
    streams = [main] + [eng.side_stream(k) for k in range(len(jobs) - 1)]
    for s in streams[1:]:
        s.wait_stream(main)
    results = [None] * len(jobs)
    pending = list(range(len(jobs)))
    # the persistent one-CTA-per-run Lanczos leaves a CTA slot per SM to the other jobs
    if len(jobs) > 1:
        eng.lib.edgpu_set_small_reserve(1)
    try:
        while pending:
            for k in list(pending):
                with torch.cuda.stream(streams[k]):
                    try:
                        next(jobs[k])
                    except StopIteration as done:
                        results[k] = done.value
                        pending.remove(k)
    finally:
        if len(jobs) > 1:
            eng.lib.edgpu_set_small_reserve(0)
    for s in streams[1:]:
        main.wait_stream(s)
    for k, r in enumerate(results):
        if k and torch.is_tensor(r):
            r.record_stream(main)
    return results


def green_batch(eng, dop, restr, run_states, run_amps, e_runs, omega, delta, krylovSize=150, precision=0,
                sector=None, return_coeffs=False, normalize=True, scales=None, timing=None, capture=None,
                perturb=None, stages=None):
    """Continued-fraction Green's functions of many start states on one sector.

    Arguments as :func:`green_setup`; ``e_runs[r]`` is the energy added to the frequency of
    run r.  Returns g [R, n_omega] complex128 (device).
    """
    return _drive(_green_batch_steps(eng, dop, restr, run_states, run_amps, e_runs, omega, delta, krylovSize,
                                     precision, sector, return_coeffs, normalize, scales, timing, capture, perturb,
                                     stages))


def _green_batch_steps(eng, dop, restr, run_states, run_amps, e_runs, omega, delta, krylovSize=150, precision=0,
                       sector=None, return_coeffs=False, normalize=True, scales=None, timing=None, capture=None,
                       perturb=None, stages=None, sector_hint=None, sector_out=None):
    """green_batch as a step generator: yields once, after the Lanczos launch.  ``sector_out``
    (a dict) receives the sector the runs used under "sector"."""
    omega = np.asarray(omega, dtype=np.float64)
    st = green_setup(eng, dop, restr, run_states, run_amps, krylovSize, precision, sector, normalize, scales,
                     perturb, stages, sector_hint)
    if sector_out is not None and st is not None:
        sector_out["sector"] = st.sector
    runs = len(run_states) if run_amps is not None else run_states[3]
    g = torch.zeros((runs, len(omega)), dtype=torch.complex128, device=eng.device)
    if st is None:
        return (g, None) if return_coeffs else g
    live, k_h = st.live, st.k
    alpha, beta = eng.lanczos(st.sector.csr, st.v0, k_h, precision=precision if precision in (1, 3) else 0,
                              timing=timing, check=False)
    yield
    eng.read_status("lanczos")
    _mark(stages, "green:lanczos")
    e_live = np.asarray(e_runs, dtype=np.float64)[live]
    live_t = torch.from_numpy(live).to(eng.device)
    g[live_t] = eng.cfrac(alpha, beta, k_h, omega, delta, e_live, st.scale[live], precision=1 if precision else 0)
    _mark(stages, "green:cfrac")
    if capture is not None:
        capture.append(dict(csr=st.sector.csr, v0=st.v0, k=k_h, e=e_live, scale=st.scale[live], live=live, g=g,
                            omega=omega, delta=delta))
    if return_coeffs:
        return g, (alpha, beta, k_h, live)
    return g


def green_runs_one_by_one(eng, dop, restr, run_states, run_amps, e_runs, omega, delta, krylovSize=150, precision=0,
                          normalize=True, scales=None):
    """Upstream's call structure on the GPU: one Green's function per Lanczos launch, each on
    the closure of its own start state (upstream getGreen per run, spectra.py:551-681).  The
    reference point of the batched forms; same arguments as green_batch."""
    if run_amps is None:
        states, amps, run_of_row, runs = run_states
        rr = run_of_row.cpu().numpy()
        bounds = np.searchsorted(rr, np.arange(runs + 1))
        run_states = [states[bounds[r]:bounds[r + 1]] for r in range(runs)]
        run_amps = [amps[bounds[r]:bounds[r + 1]] for r in range(runs)]
    runs = len(run_states)
    g = torch.zeros((runs, len(np.atleast_1d(omega))), dtype=torch.complex128, device=eng.device)
    for r in range(runs):
        sc = None if scales is None else [scales[r]]
        g[r] = green_batch(eng, dop, restr, [run_states[r]], [run_amps[r]], [e_runs[r]], omega, delta, krylovSize,
                           precision, normalize=normalize, scales=sc)[0]
    return g


class StageTimer:
    """Optional per-stage wall-clock timing (synchronises the device at each mark)."""

    def __init__(self):
        self.t = {}
        self._last = None

    def mark(self, label):
        torch.cuda.synchronize()
        import time

        now = time.perf_counter()
        if self._last is not None:
            self.t[label] = self.t.get(label, 0.0) + now - self._last
        self._last = now


def _mark(stages, label):
    if stages is not None:
        stages.mark(label)


def _psi_tensors(eng, psi, n):
    words, amps = codec.psi_to_arrays(psi, n)
    return eng.upload_states(words), eng.to_device(amps)


# ---------------------------------------------------------------------------------------
# Upstream API
# ---------------------------------------------------------------------------------------


def getGreen(n_spin_orbitals, e, psi, hOp, omega, delta, krylovSize, slaterWeightMin, restrictions=None,
             h_dict=None, mode="sparse", parallelization_mode="serial", precision=0):
    r"""``<psi|((omega + i delta + e) - H)^{-1}|psi>`` (upstream spectra.py:551-681).

    ``psi`` is used as given (upstream does not normalise inside getGreen).  ``h_dict`` is
    upstream's in/out memo ``{state: H|state>}``: as upstream's expand_basis_and_hamiltonian
    (finite.py:1806-1894) the closure reuses the outputs stored for states already in it,
    and every state of the closure without an entry gets one (``applyOp(hOp, {b: 1},
    restrictions=...)``, computed on the device), in breadth-first order.
    """
    omega = np.asarray(omega)
    if len(psi) == 0:
        return np.zeros(len(omega), dtype=complex)
    if mode not in ("sparse", "dense", "dict"):
        raise Exception("Value of variable 'mode' is incorrect.")
    from .finite import _expand_device, _fill_h_dict

    eng = get_engine()
    n = int(n_spin_orbitals)
    words_for(n)
    dop = _device_op(hOp, eng)
    restr = make_restrictions(restrictions, n)
    words, amps = codec.psi_to_arrays(psi, n)
    s_t, a_t = eng.upload_states(words), eng.to_device(amps)
    sector = None
    if h_dict is not None:
        s_sorted, order = _expand_device(eng, n, dop, restr, words, h_dict)
        sector = Sector.from_parts(s_sorted, eng.build_csr(s_sorted, dop, restr))
        _fill_h_dict(eng, n, dop, restr, order, h_dict)
    g = green_batch(eng, dop, restr, [s_t], [a_t], [e], omega, delta, krylovSize, precision, sector=sector,
                    normalize=False)
    return eng.to_host(g[0])


def spectra_device(eng, dop, restr, t_dops, psi_t, es, w, delta, krylovSize=150, slaterWeightMin=1e-7,
                   precision=0, capture=None, perturb=None, batched=True):
    """Device form of :func:`getSpectra`: ``psi_t`` is a list of (states, amps) device tensors.

    ``batched=False`` runs upstream's call structure (one Green's function at a time).
    Returns g [n_states, n_ops, n_w] complex128 on the device.
    """
    return _drive(spectra_steps(eng, dop, restr, t_dops, psi_t, es, w, delta, krylovSize, slaterWeightMin, precision,
                                capture, perturb, batched))


def spectra_steps(eng, dop, restr, t_dops, psi_t, es, w, delta, krylovSize=150, slaterWeightMin=1e-7, precision=0,
                  capture=None, perturb=None, batched=True, t_outs=None, sector_hint=None, sector_out=None):
    """spectra_device as a step generator for :func:`run_concurrently`.  ``t_outs``: the
    result of ``eng.apply_vectors_multi`` for these operators and states when the caller
    has it already; ``sector_hint``: a sector closed under the restricted H that may hold
    every start state (used when it does, as in :func:`green_setup`)."""
    ne = len(es)
    w = np.asarray(w, dtype=np.float64)
    run_states, run_amps, e_runs = [], [], []
    if t_outs is None:
        t_outs = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t], t_dops, restr,
                                         slaterWeightMin)
    for outs in t_outs:
        for i, (s_, a_) in enumerate(outs):
            run_states.append(s_)
            run_amps.append(a_)
            e_runs.append(es[i])
    if batched:
        g = yield from _green_batch_steps(eng, dop, restr, run_states, run_amps, e_runs, w, delta, krylovSize,
                                          precision, capture=capture, perturb=perturb, sector_hint=sector_hint,
                                          sector_out=sector_out)
    else:
        g = green_runs_one_by_one(eng, dop, restr, run_states, run_amps, e_runs, w, delta, krylovSize, precision)
    return g.view(len(t_dops), ne, len(w)).permute(1, 0, 2)


def getSpectra(n_spin_orbitals, hOp, tOps, psis, es, w, delta, restrictions=None, krylovSize=150,
               slaterWeightMin=1e-7, parallelization_mode="H_build", precision=0):
    r"""Green's functions ``<psi|T^+ ((w + i delta + e) - H)^{-1} T|psi>`` for every
    transition operator and eigenstate (upstream spectra.py:684-806).

    Returns ``gs[n_states, n_ops, n_w]`` complex128 on the host.
    """
    if parallelization_mode not in ("eigen_states", "H_build"):
        raise Exception("Incorrect value of variable parallelization_mode.")
    eng = get_engine()
    n = int(n_spin_orbitals)
    words_for(n)
    dop = _device_op(hOp, eng)
    restr = make_restrictions(restrictions, n)
    psi_t = [_psi_tensors(eng, psis[i], n) for i in range(len(es))]
    t_dops = [_device_op(top, eng) for top in tOps]
    # a closure kept from an earlier call of this session serves as the sector when it holds
    # every start state (the role of upstream's h_dict memo); the sector used is kept
    hints = eng.sectors_for("closure", dop, restr)
    used = {}
    g = _drive(spectra_steps(eng, dop, restr, t_dops, psi_t, es, w, delta, krylovSize, slaterWeightMin, precision,
                             sector_hint=hints[0] if hints else None, sector_out=used))
    if "sector" in used:
        eng.remember_sector("closure", dop, restr, used["sector"])
    return eng.to_host(g.contiguous())


def _shifted_solutions(eng, sector, y, zs, tol, k_cap):
    """x(z) = (z - H)^{-1} y for all z from one Krylov space (full reorthogonalisation).

    Returns X [len(zs), N] complex128 (device).  Converged when the Lanczos residual
    estimate ``beta_K |e_K^T (z - T_K)^{-1} e_1|`` is below ``tol`` for every z.
    """
    ynorm = float(torch.linalg.vector_norm(y).item())
    if ynorm == 0.0:
        return torch.zeros((len(zs), sector.n), dtype=torch.complex128, device=eng.device)
    v0 = (y / ynorm).contiguous()
    zs = np.asarray(zs, dtype=np.complex128)

    def solve_all(a, b, kk):
        # (z - T) x = e1 for every z: tridiagonal banded solves
        xs = np.empty((kk, len(zs)), dtype=np.complex128)
        off = -np.asarray(b[: kk - 1], dtype=np.complex128)
        e1 = np.zeros(kk, dtype=np.complex128)
        e1[0] = 1.0
        for m, z in enumerate(zs):
            ab = np.zeros((3, kk), dtype=np.complex128)
            ab[0, 1:] = off
            ab[1, :] = z - np.asarray(a[:kk])
            ab[2, :-1] = off
            xs[:, m] = scipy.linalg.solve_banded((1, 1), ab, e1)
        return xs

    def stop(a, bfull, j):
        if j < 2:
            return False
        xs = solve_all(a, bfull, j)
        return bool(np.all(np.abs(bfull[j - 1] * xs[-1, :]) <= tol * np.linalg.norm(xs, axis=0)))

    V, a, bfull = eng.krylov_reorth(sector.csr, v0, k_cap, stop=stop, chunk=16)
    kk = len(a)
    xs = solve_all(a, bfull, kk) * ynorm
    return eng.combine(V, xs)


def getRIXSmap(n_spin_orbitals, hOp, tOpsIn, tOpsOut, psis, es, wIns, wLoss, delta1, delta2, restrictions=None,
               krylovSize=150, slaterWeightMin=1e-7, h_dict_ground=None, parallelization_mode="H_build_wIn",
               precision=0, solve_tol=1e-10, share_out_memo=True, max_krylov=2000):
    r"""RIXS map ``gs[nE, n_in, n_out, n_wIn, n_wLoss]`` (upstream spectra.py:809-1130).

    ``share_out_memo=True`` reproduces upstream's single memo dict shared by all outgoing
    operators (``tOut_big = [{}] * len(tOpsOut)``): every product state's outgoing action
    is the one of ``tOpsOut[0]``, the first operator to meet it, so all outgoing slices are
    equal; their final-state Green's functions are computed once and copied.  ``False``
    applies each outgoing operator itself.
    """
    if parallelization_mode not in ("serial", "H_build", "wIn", "H_build_wIn"):
        raise Exception("Incorrect value of variable parallelization_mode.")
    eng = get_engine()
    n = int(n_spin_orbitals)
    words_for(n)
    dop = _device_op(hOp, eng)
    restr = make_restrictions(restrictions, n)
    psi_t = [_psi_tensors(eng, psis[i], n) for i in range(len(es))]
    # sectors kept from earlier calls of this session: a closure that holds T_in psi serves as
    # the core-hole sector, and an eigensystem basis closed under the restricted H as the
    # final-state sector (the roles of upstream's h_dict memos across calls)
    hints = eng.sectors_for("closure", dop, restr)
    final = None
    for sb, csr in eng.sectors_for("basis", dop, None):
        cache = sb.__dict__.setdefault("_closed", {})
        rkey = _restr_key(restr)
        if rkey not in cache:
            cache[rkey] = closed_sector(eng, dop, restr, sb.sorted, csr, sb.words)
        if cache[rkey] is not None:
            final = cache[rkey]
            break
    share = {}
    g = _drive(rixs_steps(eng, dop, restr, [_device_op(t, eng) for t in tOpsIn], [_device_op(t, eng) for t in tOpsOut],
                          psi_t, es, wIns, wLoss, delta1, delta2, krylovSize, slaterWeightMin, precision, solve_tol,
                          share_out_memo, max_krylov, final_sector=final, share=share,
                          core_hint=hints[0] if hints else None))
    if "sector" in share:
        eng.remember_sector("closure", dop, restr, share["sector"])
    return eng.to_host(g)


def rixs_device(eng, dop, restr, tin_dops, tout_dops, psi_t, es, wIns, wLoss, delta1, delta2, krylovSize=150,
                slaterWeightMin=1e-7, precision=0, solve_tol=1e-10, share_out_memo=True, max_krylov=2000,
                timing=None, capture=None, perturb=None, stages=None, batched=True, final_sector=None):
    """Device form of :func:`getRIXSmap`; returns gs [nE, n_in, n_out, n_wIn, n_wLoss] (device).

    ``batched=False`` runs upstream's call structure: one shifted solve per incoming energy
    and one final-state Green's function per (incoming energy, outgoing channel)."""
    return _drive(rixs_steps(eng, dop, restr, tin_dops, tout_dops, psi_t, es, wIns, wLoss, delta1, delta2, krylovSize,
                             slaterWeightMin, precision, solve_tol, share_out_memo, max_krylov, timing, capture,
                             perturb, stages, batched, final_sector))


def rixs_steps(eng, dop, restr, tin_dops, tout_dops, psi_t, es, wIns, wLoss, delta1, delta2, krylovSize=150,
               slaterWeightMin=1e-7, precision=0, solve_tol=1e-10, share_out_memo=True, max_krylov=2000,
               timing=None, capture=None, perturb=None, stages=None, batched=True, final_sector=None, share=None,
               core_hint=None):
    """rixs_device as a step generator for :func:`run_concurrently` (yields after the launch
    of the shifted solves and after the launch of the final-state Lanczos).  ``final_sector``:
    a sector from :func:`closed_sector` (the ground-state sector) used for the final states
    (``core_hint``: a closure under the restricted H used as the core-hole sector when it holds
    every T_in psi state)
    when it holds them all, instead of expanding their closure.  ``share``: a dict that
    receives ``t_outs`` (T_in applied to the eigenstates, as ``eng.apply_vectors_multi``
    returns it), ``sector`` (the core-hole sector, the closure of those states) and
    ``ready`` (an event on the current stream after both) before the first yield."""
    _mark(stages, "start")
    wIns = np.asarray(wIns, dtype=np.float64)
    wLoss = np.asarray(wLoss, dtype=np.float64)
    ne, nin, nout, nwi = len(es), len(tin_dops), len(tout_dops), len(wIns)
    gs = torch.zeros((ne, nin, nout, nwi, len(wLoss)), dtype=torch.complex128, device=eng.device)
    if ne == 0 or nin == 0 or nout == 0 or nwi == 0:
        return gs
    # 1. core-hole states psi1 = T_in psi
    psi1 = {}
    t_outs = eng.apply_vectors_multi([p[0] for p in psi_t], [p[1] for p in psi_t], tin_dops, restr, slaterWeightMin)
    for t_in, outs in enumerate(t_outs):
        for ie, o in enumerate(outs):
            psi1[(t_in, ie)] = o
    nonempty = [v[0] for v in psi1.values() if v[0].shape[0]]
    if not nonempty:
        return gs
    _mark(stages, "rixs:psi1")
    # 2. core-hole sector
    core = None
    if core_hint is not None:
        # a closure under the restricted H that holds every T_in psi state holds their closure
        rows = eng.lookup(core_hint.basis, torch.cat(nonempty, 0))
        if bool((rows >= 0).all().item()):
            core = core_hint
    if core is None:
        core = Sector(eng, dop, restr, torch.cat(nonempty, 0))
    if share is not None:
        share.update(t_outs=t_outs, sector=core, ready=torch.cuda.current_stream(eng.device).record_event())
    _mark(stages, "rixs:core_sector")
    # 3. outgoing operators as sparse maps core basis -> output states
    def build_out_maps():
        maps = []
        for k in range(nout):
            if share_out_memo and k > 0:
                maps.append(maps[0])
                continue
            maps.append(_transfer_matrix(eng, tout_dops[0] if share_out_memo else tout_dops[k], restr, core.basis))
        return maps

    # 4. shifted solves x(z) = (z - H)^{-1} psi1 for every incoming energy and every
    # (t_in, eigenstate) right-hand side
    keys = [k for k, (s1, _) in psi1.items() if s1.shape[0]]
    Y = torch.zeros((len(keys), core.n), dtype=torch.complex128, device=eng.device)
    # every right-hand side in one lookup and one scatter (each psi1 holds distinct states)
    s_all = torch.cat([psi1[k][0] for k in keys], 0)
    a_all = torch.cat([psi1[k][1] for k in keys], 0)
    r_all = torch.repeat_interleave(torch.arange(len(keys), device=eng.device),
                                    torch.tensor([int(psi1[k][0].shape[0]) for k in keys], device=eng.device),
                                    output_size=int(s_all.shape[0]))
    Y.view(-1)[r_all * core.n + eng.lookup(core.basis, s_all)] = torch.complex(a_all[:, 0], a_all[:, 1])
    zs = np.array([wIns + 1j * delta1 + es[ie] for (_, ie) in keys])
    # without reorthogonalisation the recurrence may need a few times the sector dimension
    k_solve = min(6 * core.n + 50, max_krylov)
    if batched:
        # the outgoing maps are built on a side stream while the solves (one CTA per
        # right-hand side, most SMs idle) run; the side stream waits only for the core basis.
        # Then the step yields, so that a pipeline running beside this one (run_concurrently)
        # does its host work while the solves occupy the GPU.
        main = torch.cuda.current_stream(eng.device)
        ready = main.record_event()
        solved = eng.shifted_solve(core.csr, Y, zs, solve_tol, k_solve, precision, check=False)
        side = eng.side_stream(1)
        side.wait_event(ready)
        with torch.cuda.stream(side):
            out_maps = build_out_maps()
        main.wait_stream(side)
        for tm in set(out_maps):
            tm.record_stream(main)
        _mark(stages, "rixs:transfer")
        yield
        if solved is not None:
            solved[2]()
    else:
        out_maps = build_out_maps()
        _mark(stages, "rixs:transfer")
        solved = None
        blocks = []
        for r in range(len(keys)):
            cols = []
            for iw in range(nwi):
                one = eng.shifted_solve(core.csr, Y[r:r + 1], zs[r:r + 1, iw:iw + 1], solve_tol, k_solve)
                if one is None:
                    break
                cols.append(one[0][0, 0])
            if len(cols) < nwi:
                blocks = None
                break
            blocks.append(torch.stack(cols))
        if blocks is not None:
            solved = (torch.stack(blocks), None)
    if solved is not None:
        x_blocks = list(solved[0])
    else:
        x_blocks = [_shifted_solutions(eng, core, Y[r], zs[r], solve_tol, min(core.n, max_krylov))
                    for r in range(len(keys))]
    _mark(stages, "rixs:shifted")
    # 5. psi3 = T_out psi2 for every (t_in, ie, w_in, t_out), pruned and normalised as upstream:
    # one SpMV over all (right-hand side, incoming energy) rows per distinct outgoing map
    X_all = torch.stack(x_blocks).reshape(len(keys) * nwi, core.n)
    st_l, am_l, run_l, e_runs, slots, scales = [], [], [], [], [], []
    run0 = 0
    pruned = {}
    alias = {}  # outgoing channel -> earlier channel with the same map (identical spectra)
    for k in range(nout):
        tm = out_maps[k]
        first = next(k0 for k0 in range(k + 1) if out_maps[k0] is tm)
        if first != k and batched:
            alias[k] = first
            continue
        if id(tm) not in pruned:
            P = tm.apply(eng, X_all)  # [n_rhs * n_wIn, n_out_states] complex128
            a2 = P.real ** 2 + P.imag ** 2
            P = torch.where(a2 >= slaterWeightMin, P, torch.zeros_like(P))
            nrm = torch.sqrt((P.real ** 2 + P.imag ** 2).sum(1, keepdim=True))
            Pn = P / torch.where(nrm > 0, nrm, torch.ones_like(nrm))
            keep = (Pn.real ** 2 + Pn.imag ** 2) >= slaterWeightMin
            row_idx, o_idx = torch.nonzero(keep, as_tuple=True)  # grouped by row
            amp = Pn[row_idx, o_idx]
            pruned[id(tm)] = (tm.out_states[o_idx], torch.stack([amp.real, amp.imag], 1), row_idx,
                              (nrm[:, 0] ** 2).cpu().numpy())
        st_k, am_k, row_k, sc_k = pruned[id(tm)]
        st_l.append(st_k)
        am_l.append(am_k)
        run_l.append(row_k + run0)
        scales.append(sc_k)
        for (t_in, ie) in keys:
            e_runs.extend([es[ie]] * nwi)
            slots.extend((ie, t_in, k, iw) for iw in range(nwi))
        run0 += len(keys) * nwi
    packed = (torch.cat(st_l, 0).contiguous(), torch.cat(am_l, 0).contiguous(), torch.cat(run_l, 0), run0)
    scales = np.concatenate(scales)
    _mark(stages, "rixs:psi3")
    # 6. ground-like sector Lanczos + continued fractions for all runs at once.  Upstream
    # runs getGreen on the normalised-then-pruned psi3 and scales by the squared norm taken
    # before the second pruning (spectra.py:1097-1124).
    if batched:
        g = yield from _green_batch_steps(eng, dop, restr, packed, None, e_runs, wLoss, delta2, krylovSize, precision,
                                          normalize=False, scales=scales, timing=timing, capture=capture,
                                          perturb=perturb, stages=stages, sector_hint=final_sector)
    else:
        g = green_runs_one_by_one(eng, dop, restr, packed, None, e_runs, wLoss, delta2, krylovSize, precision,
                                  normalize=False, scales=scales)
    idx = torch.tensor([((ie * nin + t_in) * nout + k) * nwi + iw for (ie, t_in, k, iw) in slots],
                       device=eng.device)
    gs.view(-1, len(wLoss))[idx] = g
    for k, k0 in alias.items():
        gs[:, :, k] = gs[:, :, k0]
    _mark(stages, "rixs:assemble")
    return gs


def xas_rixs_device(eng, dop, restr, xas_dops, tin_dops, tout_dops, psi_t, es, w, delta, wIns, wLoss, delta1, delta2,
                    krylovSize=150, slaterWeightMin=1e-7, precision=0, solve_tol=1e-10, share_out_memo=True,
                    max_krylov=2000, final_sector=None, stages=None):
    """XAS (:func:`spectra_device`) and the RIXS map (:func:`rixs_device`) of the same
    eigenstates, computed side by side: the RIXS pipeline on the current stream, the XAS one
    on a side stream.  When the XAS operators are the RIXS incoming ones (the same objects),
    the XAS job takes the RIXS job's T_in psi and core-hole sector, and its remaining host
    work (start vectors, Krylov sizes, Lanczos launch) runs while the RIXS shifted solves
    occupy the GPU; its continued fractions run beside the RIXS final-state Lanczos.  Same
    results as the two calls one after the other.  ``stages``: optional
    :class:`StageTimer`-like object marking the RIXS stages.  Returns (g_xas [n_states,
    n_ops, n_w], g_rixs) on the device."""
    share = {}
    same_ops = len(xas_dops) == len(tin_dops) and all(a is b for a, b in zip(xas_dops, tin_dops))

    def xas_steps():
        # first advanced after the RIXS job's first yield, by when it has shared T_in psi and
        # the core-hole sector: with the same operators these are the XAS start states and
        # their sector, so the XAS job neither applies the operators again nor rebuilds it
        if share:
            torch.cuda.current_stream(eng.device).wait_event(share["ready"])
        g = yield from spectra_steps(eng, dop, restr, xas_dops, psi_t, es, w, delta, krylovSize, slaterWeightMin,
                                     precision, t_outs=share.get("t_outs") if same_ops else None,
                                     sector_hint=share.get("sector"))
        return g

    g_rixs, g_xas = run_concurrently(eng, [
        rixs_steps(eng, dop, restr, tin_dops, tout_dops, psi_t, es, wIns, wLoss, delta1, delta2, krylovSize,
                   slaterWeightMin, precision, solve_tol, share_out_memo, max_krylov, stages=stages,
                   final_sector=final_sector, share=share),
        xas_steps()])
    return g_xas, g_rixs


class _TransferMatrix:
    """Sparse map core-sector basis -> output product states of one operator (CSR rows = outputs)."""

    def __init__(self, out_states, csr):
        self.out_states = out_states
        self.csr = csr

    def record_stream(self, stream):
        """Mark the tensors as used on ``stream`` (they were made on another one)."""
        for x in (self.out_states, self.csr.row_ptr, self.csr.col, self.csr.val_c, self.csr.val_r):
            if x is not None:
                x.record_stream(stream)

    def apply(self, eng, X):
        """P[m] = T X[m] for rows m of X [M, Nc]; returns [M, n_out] complex128."""
        xt = X.t().contiguous()
        y = eng.spmv(self.csr, xt)
        return y.t().contiguous()


def _transfer_matrix(eng, tdop, restr, core_basis):
    from .engine import CsrMatrix

    offsets, out_s, _, out_v = eng.apply_columns(core_basis, tdop, restr, 0.0, want_states=True, want_vals=True)
    m = out_s.shape[0]
    w = core_basis.shape[1]
    if m == 0:
        rp = torch.zeros(1, dtype=torch.int64, device=eng.device)
        return _TransferMatrix(out_s, CsrMatrix(rp, torch.zeros(0, dtype=torch.int32, device=eng.device),
                                                val_c=torch.zeros((0, 2), dtype=torch.float64, device=eng.device),
                                                ncols=core_basis.shape[0]))
    outs = eng.sort_unique(out_s)
    row = eng.lookup(outs, out_s)
    col = torch.repeat_interleave(torch.arange(core_basis.shape[0], device=eng.device), offsets[1:] - offsets[:-1],
                                  output_size=m)
    # entries sorted by (row, col) via a stable sort on row of col-ordered entries
    keys = row.view(-1, 1).contiguous()
    payload = torch.arange(m, dtype=torch.int32, device=eng.device)
    eng.sort_states(keys, payload)
    p = payload.to(torch.int64)
    rows_sorted = keys.view(-1)
    counts = torch.bincount(rows_sorted, minlength=outs.shape[0])
    rp = torch.zeros(outs.shape[0] + 1, dtype=torch.int64, device=eng.device)
    rp[1:] = torch.cumsum(counts, 0)
    csr = CsrMatrix(rp, col[p].to(torch.int32).contiguous(), val_c=out_v[p].contiguous(), ncols=core_basis.shape[0])
    del w
    return _TransferMatrix(outs, csr)


# ---------------------------------------------------------------------------------------
# Output formats and the spectra driver (upstream spectra.py:36-293)
# ---------------------------------------------------------------------------------------


class NpzStore:
    """Dataset store with the ``create_dataset(name, data=...)`` call of an h5py file, written
    as one ``.npz`` on ``close()`` (same dataset names and shapes as upstream's spectra.h5;
    h5py itself works as well when it is installed)."""

    def __init__(self, filename):
        self.filename = filename
        self.data = {}

    def create_dataset(self, name, data):
        self.data[name] = np.asarray(data)
        return self.data[name]

    def close(self):
        np.savez_compressed(self.filename, **self.data)


def save_spectra_dat(filename, w, a):
    """Upstream's text spectra (spectra.py:152-162): columns energy, sum over transition
    operators, then each operator's thermally averaged spectrum; ``%8.4f``, same header."""
    a = np.asarray(a)
    tmp = [np.asarray(w), np.sum(a, axis=0)]
    for i in range(a.shape[0]):
        tmp.append(a[i, :])
    np.savetxt(filename, np.array(tmp).T, fmt="%8.4f", header="E  sum  T1  T2  T3 ...")


def save_rixs_bin(filename, wIn, wLoss, a):
    """Upstream's RIXS.bin (spectra.py:276-285): float32 [n_wLoss + 1, n_wIn + 1], element
    [0, 0] = n_wIn, first row wIn, first column wLoss, the rest the thermally averaged map
    summed over in- and out-polarisations, transposed to [wLoss, wIn]."""
    a_sum = np.sum(np.asarray(a), axis=(0, 1))
    tmp = np.zeros((len(wLoss) + 1, len(wIn) + 1), dtype=np.float32)
    tmp[0, 0] = len(wIn)
    tmp[0, 1:] = wIn
    tmp[1:, 0] = wLoss
    tmp[1:, 1:] = a_sum.T
    tmp.tofile(filename)


def simulate_spectra(es, psis, hOp, T, w, delta, epsilons, wLoss, deltaNIXS, qsNIXS, liNIXS, ljNIXS, RiNIXS,
                     RjNIXS, radialMesh, wIn, deltaRIXS, epsilonsRIXSin, epsilonsRIXSout, restrictions, h5f, nBaths,
                     out_dir=".", precision=0):
    """PS+IPS, XPS, NIXS, XAS and RIXS spectra with upstream's outputs (spectra.py:36-293):
    datasets PS/PSthermal, XPS/XPSthermal, NIXS/NIXSthermal, XAS/XASthermal, RIXS/RIXSthermal
    in ``h5f`` (an h5py file or NpzStore), text files PS.dat, XPS.dat, NIXS.dat, XAS.dat and
    RIXS.bin in ``out_dir``.  Every spectrum family is one batched device computation."""
    import os

    from .models import dipole_ops, daggered_dipole_ops, inverse_photoemission_ops, photoemission_ops

    n = sum(2 * (2 * ang + 1) + nb for ang, nb in nBaths.items())
    es = np.asarray(es)
    path = lambda f: os.path.join(out_dir, f)  # noqa: E731

    def store(name, gs, mesh, fname):
        a = thermal_average(es[: gs.shape[0]], -gs.imag, T=T)
        h5f.create_dataset(name, data=-gs.imag)
        h5f.create_dataset(name + "thermal", data=a)
        save_spectra_dat(path(fname), mesh, a)

    gs_ips = getSpectra(n, hOp, inverse_photoemission_ops(nBaths, l=2), psis, es, w, delta, restrictions,
                        precision=precision)
    gs_ps = -getSpectra(n, hOp, photoemission_ops(nBaths, l=2), psis, es, -w, -delta, restrictions,
                        precision=precision)
    store("PS", gs_ps + gs_ips, w, "PS.dat")
    gs = -getSpectra(n, hOp, photoemission_ops(nBaths, l=1), psis, es, -w, -delta, restrictions,
                     precision=precision)
    store("XPS", gs, w, "XPS.dat")
    gs = getSpectra(n, hOp, getNIXSOperators(nBaths, qsNIXS, liNIXS, ljNIXS, RiNIXS, RjNIXS, radialMesh), psis, es,
                    wLoss, deltaNIXS, restrictions, precision=precision)
    store("NIXS", gs, wLoss, "NIXS.dat")
    gs = getSpectra(n, hOp, dipole_ops(nBaths, epsilons), psis, es, w, delta, restrictions, precision=precision)
    store("XAS", gs, w, "XAS.dat")
    gs = getRIXSmap(n, hOp, dipole_ops(nBaths, epsilonsRIXSin), daggered_dipole_ops(nBaths, epsilonsRIXSout), psis,
                    es, wIn, wLoss, delta, deltaRIXS, restrictions, precision=precision)
    a = thermal_average(es[: gs.shape[0]], -gs.imag, T=T)
    h5f.create_dataset("RIXS", data=-gs.imag)
    h5f.create_dataset("RIXSthermal", data=a)
    save_rixs_bin(path("RIXS.bin"), wIn, wLoss, a)
