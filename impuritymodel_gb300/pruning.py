"""Learned basis pruning: a small network over occupation bitstrings ranks basis states.

No counterpart in upstream impurityModel, whose bases keep every restricted configuration
(``get_basis``, finite.py:294-374) and every state of a closure (``expand_basis``,
finite.py:1696-1803).  The network (occupation bits of up to 320 spin-orbitals -> 256 -> 256
-> 1, ReLU) is trained on the GPU by the library's own kernels (tcgen05 BF16 GEMMs with
FP32 accumulation, FP32 Adam master weights) to predict log10 of the ground-state weight
``|<s|psi_0>|^2`` of each basis state, from plain exact diagonalisation of seeded models.
Pruning keeps the best-ranked fraction of a basis; the full basis stays the fallback and the
judge of the energy error (``pruned_ground_state`` reports both).
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as L
from . import codec
from .engine import _ptr, get_engine

N_IN = 320  # 316 spin-orbitals of the largest model, padded to a multiple of 64
N_H = 256
WORDS = N_IN // 64
ROWS = 128  # batch granularity of the tensor-core GEMMs
FLOOR = 1e-14  # weights below this count as 10^-14


def pad_words(states, words=WORDS):
    """[N, W] int64 state words -> [N, words] (extra words zero: spin-orbitals beyond W*64 empty)."""
    n, w = states.shape
    if w == words:
        return states.contiguous()
    out = torch.zeros((n, words), dtype=torch.int64, device=states.device)
    out[:, : min(w, words)] = states[:, :words]
    return out


class BasisNet:
    """Device parameters, Adam state and the forward/backward passes of the network."""

    def __init__(self, eng=None, seed=0, lr=1e-3):
        self.eng = eng or get_engine()
        dev = self.eng.device
        g = torch.Generator().manual_seed(int(seed))
        shapes = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("w3", (N_H,)),
                  ("b3", (1,))]
        sizes = [int(np.prod(s)) for _, s in shapes]
        self.P = torch.zeros(sum(sizes), dtype=torch.float32, device=dev)
        self.G = torch.zeros_like(self.P)
        self.m = torch.zeros_like(self.P)
        self.v = torch.zeros_like(self.P)
        self.p, self.g = {}, {}
        off = 0
        for (name, shape), sz in zip(shapes, sizes):
            self.p[name] = self.P[off: off + sz].view(shape)
            self.g[name] = self.G[off: off + sz].view(shape)
            off += sz
        self.p["W1"].copy_(torch.randn((N_H, N_IN), generator=g) * math.sqrt(2.0 / N_IN))
        self.p["W2"].copy_(torch.randn((N_H, N_H), generator=g) * math.sqrt(2.0 / N_H))
        self.p["w3"].copy_(torch.randn((N_H,), generator=g) * math.sqrt(1.0 / N_H))
        self.p["b3"].fill_(-7.0)  # middle of the log10 weight range
        self.W1b = torch.empty((N_H, N_IN), dtype=torch.bfloat16, device=dev)
        self.W2b = torch.empty((N_H, N_H), dtype=torch.bfloat16, device=dev)
        self.W2t = torch.empty((N_H, N_H), dtype=torch.bfloat16, device=dev)
        self.lr = lr
        self.t = 0
        self.refresh()

    # -- kernels -------------------------------------------------------------------------
    def _lib(self):
        return self.eng.lib

    def refresh(self):
        """BF16 operand copies of the FP32 master weights (W2 also transposed)."""
        e = self.eng
        L.check(self._lib().edgpu_mlp_to_bf16(_ptr(self.p["W1"]), N_H, N_IN, _ptr(self.W1b), None, e.stream),
                "mlp_to_bf16")
        L.check(self._lib().edgpu_mlp_to_bf16(_ptr(self.p["W2"]), N_H, N_H, _ptr(self.W2b), _ptr(self.W2t),
                                              e.stream), "mlp_to_bf16")

    def _gemm(self, epi, A, B, M, N, K, C=None, bias=None, mask=None, Y=None, Yt=None):
        e = self.eng
        L.check(self._lib().edgpu_gemm_bf16_epi(epi, _ptr(A), _ptr(B), M, N, K, _ptr(C) if C is not None else None,
                                                _ptr(bias) if bias is not None else None,
                                                _ptr(mask) if mask is not None else None,
                                                _ptr(Y) if Y is not None else None,
                                                _ptr(Yt) if Yt is not None else None, _ptr(e.status), e.stream),
                "gemm_bf16_epi")

    def inputs(self, states, transposed=False):
        """BF16 occupation matrix X [B, N_IN] (and X^T) of padded states [B, WORDS]."""
        B = states.shape[0]
        dev = self.eng.device
        X = torch.empty((B, N_IN), dtype=torch.bfloat16, device=dev)
        Xt = torch.empty((N_IN, B), dtype=torch.bfloat16, device=dev) if transposed else None
        L.check(self._lib().edgpu_mlp_bits(_ptr(states), states.shape[1], B, N_IN, _ptr(X),
                                           _ptr(Xt) if Xt is not None else None, self.eng.stream), "mlp_bits")
        return X, Xt

    def forward(self, X, keep=False):
        B = X.shape[0]
        dev = self.eng.device
        H1 = torch.empty((B, N_H), dtype=torch.bfloat16, device=dev)
        H2 = torch.empty((B, N_H), dtype=torch.bfloat16, device=dev)
        H1t = torch.empty((N_H, B), dtype=torch.bfloat16, device=dev) if keep else None
        H2t = torch.empty((N_H, B), dtype=torch.bfloat16, device=dev) if keep else None
        self._gemm(1, X, self.W1b, B, N_H, N_IN, bias=self.p["b1"], Y=H1, Yt=H1t)
        self._gemm(1, H1, self.W2b, B, N_H, N_H, bias=self.p["b2"], Y=H2, Yt=H2t)
        y = torch.empty(B, dtype=torch.float32, device=dev)
        L.check(self._lib().edgpu_mlp_head(_ptr(H2), _ptr(self.p["w3"]), _ptr(self.p["b3"]), B, N_H, _ptr(y),
                                           self.eng.stream), "mlp_head")
        return y, (H1, H1t, H2, H2t)

    def gradients(self, X, Xt, target):
        """Mean-squared-error loss (device scalar) and gradients into self.g."""
        B = X.shape[0]
        dev = self.eng.device
        lib, s = self._lib(), self.eng.stream
        y, (H1, H1t, H2, H2t) = self.forward(X, keep=True)
        dy = torch.empty(B, dtype=torch.float32, device=dev)
        dH2 = torch.empty((B, N_H), dtype=torch.bfloat16, device=dev)
        dH2t = torch.empty((N_H, B), dtype=torch.bfloat16, device=dev)
        L.check(lib.edgpu_mlp_head_backward(_ptr(H2), _ptr(y), _ptr(target), _ptr(self.p["w3"]), B, N_H, _ptr(dy),
                                            _ptr(dH2), _ptr(dH2t), s), "mlp_head_backward")
        L.check(lib.edgpu_mlp_row_dot(_ptr(H2t), N_H, B, _ptr(dy), _ptr(self.g["w3"]), s), "row_dot")
        self.g["b3"].copy_(dy.sum().view(1))
        self._gemm(0, dH2t, H1t, N_H, N_H, B, C=self.g["W2"])
        L.check(lib.edgpu_mlp_row_dot(_ptr(dH2t), N_H, B, None, _ptr(self.g["b2"]), s), "row_dot")
        dH1 = torch.empty((B, N_H), dtype=torch.bfloat16, device=dev)
        dH1t = torch.empty((N_H, B), dtype=torch.bfloat16, device=dev)
        self._gemm(2, dH2, self.W2t, B, N_H, N_H, mask=H1, Y=dH1, Yt=dH1t)
        self._gemm(0, dH1t, Xt, N_H, N_IN, B, C=self.g["W1"])
        L.check(lib.edgpu_mlp_row_dot(_ptr(dH1t), N_H, B, None, _ptr(self.g["b1"]), s), "row_dot")
        return ((y - target) ** 2).mean()

    def adam_step(self, beta1=0.9, beta2=0.999, eps=1e-8):
        self.t += 1
        lr_t = self.lr * math.sqrt(1.0 - beta2 ** self.t) / (1.0 - beta1 ** self.t)
        L.check(self._lib().edgpu_mlp_adam(_ptr(self.P), _ptr(self.G), _ptr(self.m), _ptr(self.v), self.P.numel(),
                                           lr_t, beta1, beta2, eps, self.eng.stream), "mlp_adam")
        self.refresh()

    # -- training and inference ----------------------------------------------------------
    def train(self, states, log_w, epochs=4, batch=4096, seed=0, log=None):
        """Fit log10 weights ``log_w`` [N] of padded states [N, WORDS] by Adam on shuffled batches."""
        batch = max(ROWS, (batch // ROWS) * ROWS)
        n = states.shape[0]
        gen = torch.Generator(device=self.eng.device)
        gen.manual_seed(int(seed))
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=self.eng.device, generator=gen)
            for b0 in range(0, n - batch + 1, batch):
                idx = perm[b0: b0 + batch]
                X, Xt = self.inputs(states[idx].contiguous(), transposed=True)
                loss = self.gradients(X, Xt, log_w[idx].contiguous())
                self.adam_step()
                losses.append(loss)
            if log is not None:
                log.append(float(torch.stack(losses[-max(1, n // batch):]).mean().item()))
        self.eng.read_status("mlp training")
        return losses

    def predict(self, states):
        """Predicted log10 weights of padded states [N, WORDS] (any N)."""
        n = states.shape[0]
        nb = ((n + ROWS - 1) // ROWS) * ROWS
        if nb != n:
            pad = torch.zeros((nb - n, states.shape[1]), dtype=states.dtype, device=states.device)
            states = torch.cat([states, pad], 0)
        X, _ = self.inputs(states.contiguous())
        y, _ = self.forward(X)
        self.eng.read_status("mlp inference")
        return y[:n]


def ground_state_samples(eng, models, n_states=1, k_start=120):
    """(padded states [N, WORDS], log10 weights [N] float32) of the basis states of ``models``
    from plain exact diagonalisation (one ragged launch per convergence round).  The weight of
    a state is its largest ``|<s|psi_q>|^2`` over the ``n_states`` lowest eigenstates."""
    from .ensemble import ModelSectors, ensemble_ground_states

    secs = [ModelSectors(eng, m) for m in models]
    _, psis = ensemble_ground_states(eng, secs, n_states, k_start=k_start, slaterWeightMin=0.0)
    st, lw = [], []
    for ps in psis:
        s = ps[0][0]
        w2 = None
        for _, a in ps:  # every eigenvector holds the whole sorted basis (no truncation)
            q = a[:, 0] ** 2 + a[:, 1] ** 2
            w2 = q if w2 is None else torch.maximum(w2, q)
        st.append(pad_words(s))
        lw.append(torch.log10(w2.clamp_min(FLOOR)).to(torch.float32))
    return torch.cat(st), torch.cat(lw)


def prune_basis(n_spin_orbitals, basis, net, keep):
    """The ``keep`` fraction of ``basis`` (upstream ``bytes`` states) with the highest
    predicted weights, in the caller's order; pass it to ``finite.eigensystem`` as the basis."""
    from .finite import _SortedBasis

    eng = net.eng
    basis = list(basis)
    sb = _SortedBasis(eng, basis, int(n_spin_orbitals))
    m = max(1, int(round(keep * len(basis))))
    score = net.predict(pad_words(sb.given))
    top = torch.sort(torch.topk(score.to(torch.float64), m).indices).values.cpu().numpy()
    return [basis[i] for i in top]


def _scores(eng, sb, csr, ranking):
    N = sb.sorted.shape[0]
    if isinstance(ranking, BasisNet):
        return ranking.predict(pad_words(sb.sorted)).to(torch.float64)
    if ranking == "diagonal":
        rows = torch.repeat_interleave(torch.arange(N, device=eng.device), csr.row_ptr[1:] - csr.row_ptr[:-1])
        diag = torch.zeros(N, dtype=torch.float64, device=eng.device)
        on = rows == csr.col.to(torch.int64)
        vals = csr.val_r if csr.val_r is not None else csr.val_c[:, 0]
        diag[rows[on]] = vals[on]
        return -diag
    if ranking == "random":
        gen = torch.Generator(device=eng.device)
        gen.manual_seed(0)
        return torch.rand(N, device=eng.device, generator=gen, dtype=torch.float64)
    raise ValueError("ranking must be a BasisNet, 'diagonal' or 'random'")


def evaluate_pruning(eng, model, keeps, rankings, n_states=1):
    """Lowest ``n_states`` energies on the best-ranked ``keep`` fraction of the model's basis for
    every keep in ``keeps`` and every ranking in ``rankings`` ({name: BasisNet | "diagonal" |
    "random"}; "diagonal" keeps the lowest diagonal energies, the ranking without a network),
    against the full basis (the fallback and the judge).

    Returns {name: {keep: dict(error (eV, largest over the states, >= 0 by the variational
    principle), n_pruned, nnz_pruned)}} and the full-basis record."""
    from .finite import _device_hamiltonian, _device_op, _SortedBasis, eig_lowest, get_basis

    n = model.n_spin_orbitals
    dop = _device_op(model.hOp, eng)
    sb = _SortedBasis(eng, list(get_basis(*model.basis_args())), n)
    csr = _device_hamiltonian(eng, dop, sb)
    e_full, _ = eig_lowest(eng, csr, n_states)
    N = sb.sorted.shape[0]
    out = {}
    for name, ranking in rankings.items():
        score = _scores(eng, sb, csr, ranking)
        out[name] = {}
        for keep in keeps:
            m = max(1, int(round(keep * N)))
            top = torch.sort(torch.topk(score, m).indices).values
            csr_p = eng.build_csr(sb.sorted[top].contiguous(), dop, None)
            e_p, _ = eig_lowest(eng, csr_p, n_states)
            q = min(len(e_full), len(e_p))
            out[name][keep] = dict(error=float(np.max(np.asarray(e_p[:q]) - np.asarray(e_full[:q]))), n_pruned=int(m),
                                   nnz_pruned=int(csr_p.nnz))
    full = dict(e=[float(x) for x in e_full], n=int(N), nnz=int(csr.nnz))
    return out, full


def pruned_ground_state(eng, model, keep, ranking, n_states=1):
    """``evaluate_pruning`` for one keep fraction and one ranking; returns a flat dict."""
    res, full = evaluate_pruning(eng, model, [keep], {"r": ranking}, n_states)
    r = res["r"][keep]
    return dict(error=r["error"], n_full=full["n"], n_pruned=r["n_pruned"], nnz_full=full["nnz"],
                nnz_pruned=r["nnz_pruned"], e_full=full["e"])


# ---------------------------------------------------------------------------------------
# Pruning inside basis expansion
# ---------------------------------------------------------------------------------------


def seed_basis(model):
    """The lowest configurations of a seeded model: the impurity at its nominal occupation
    and every valence bath orbital filled (upstream get_basis with no bath holes)."""
    from .finite import get_basis

    nb, nvb, dnv, dnc, dnt, n0 = model.basis_args()
    dnv0 = type(dnv)((k, 0) for k in dnv)
    dnt0 = type(dnt)((k, 0) for k in dnt)
    return get_basis(nb, nvb, dnv0, dnc, dnt0, n0)


def expand_pruned(eng, dop, restr, basis0, net=None, keep=1.0, weight_min=1e-12, min_keep=16, layers=None):
    """Breadth-first closure of ``basis0`` [N0, W] under the restricted operator (upstream
    expand_basis, finite.py:1696-1803) in which every layer's new states are ranked by the
    network and only the best ``keep`` fraction (at least ``min_keep``) joins the basis and
    the next frontier; the states it drops are remembered and not offered again by later
    layers.  ``keep=1`` (or no network) is the full expansion, the fallback and the judge.  Returns (sorted basis [N, W], layered order [N, W], per-layer (new, kept))."""
    s_sorted = eng.sort_unique(basis0)
    seen = s_sorted  # basis states and the states pruned so far (never offered again)
    order = [basis0]
    frontier = basis0
    stats = []
    while frontier.shape[0] > 0 and (layers is None or len(stats) < layers):
        _, cand, _, _ = eng.apply_columns(frontier, dop, restr, weight_min, basis=seen,
                                          filt=L.FILTER_NOT_IN_BASIS, want_states=True)
        if cand.shape[0] == 0:
            break
        new = eng.sort_unique(cand)
        n_new = int(new.shape[0])
        if net is not None and keep < 1.0:
            m = max(min_keep, int(math.ceil(keep * n_new)))
            if m < n_new:
                # a BasisNet, or any function of the states giving a score per state
                score = (net.predict(pad_words(new)) if isinstance(net, BasisNet) else net(new)).to(torch.float64)
                mask = torch.zeros(n_new, dtype=torch.bool, device=new.device)
                mask[torch.topk(score, m).indices] = True
                seen = eng.merge(seen, new[~mask].contiguous())
                new = new[mask].contiguous()
        stats.append((n_new, int(new.shape[0])))
        s_sorted = eng.merge(s_sorted, new)
        seen = eng.merge(seen, new)
        order.append(new)
        frontier = new
    return s_sorted, torch.cat(order, 0), stats


class ExpandedBasis:
    """A sorted device basis in the form the eigensystem routines take (caller order = sorted
    order)."""

    def __init__(self, sorted_states):
        self.sorted = sorted_states
        self.given = sorted_states
        self.perm = torch.arange(sorted_states.shape[0], dtype=torch.int64, device=sorted_states.device)
        self.words = sorted_states.cpu().numpy().view(np.uint64)


def evaluate_expansion_pruning(eng, model, net, keeps, n_states=1):
    """Lowest ``n_states`` energies on the pruned expansion of the model's seed basis for every
    keep fraction, against the full expansion (the judge).  Returns {keep: dict(error eV (>= 0,
    variational), n, layers)} and the full record."""
    from .engine import make_restrictions
    from .finite import _device_op, eig_lowest

    n = model.n_spin_orbitals
    dop = _device_op(model.hOp, eng)
    restr = make_restrictions(model.restrictions, n)
    b0 = eng.upload_states(codec.bytes_to_words(list(seed_basis(model)), n))
    full, _, st_full = expand_pruned(eng, dop, restr, b0)
    e_full, _ = eig_lowest(eng, eng.build_csr(full, dop, None), n_states)
    out = {}
    for keep in keeps:
        pr, _, st = expand_pruned(eng, dop, restr, b0, net, keep)
        e_p, _ = eig_lowest(eng, eng.build_csr(pr, dop, None), n_states)
        q = min(len(e_full), len(e_p))
        out[keep] = dict(error=float(np.max(np.asarray(e_p[:q]) - np.asarray(e_full[:q]))), n=int(pr.shape[0]),
                         layers=st)
    return out, dict(e=[float(x) for x in e_full], n=int(full.shape[0]), layers=st_full)
