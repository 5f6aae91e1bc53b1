"""Device engine: compiled operators, sorted sector bases, CSR Hamiltonians and Lanczos.

Host orchestration in Python over the C ABI of ``libedgpu.so`` (``include/edgpu.h``).  All
device memory is owned by torch tensors; the library only receives pointers, sizes, a
workspace and the current CUDA stream.  States live on the device as ``int64[N, W]``
tensors holding the bit patterns of the packed ``uint64`` words.
"""

from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np
import torch

from . import _lib as L
from .codec import n_words
from .tuner import bucket, get_tuner

_U64 = np.uint64


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else C.c_void_p(0)


# packed operators and flags by key sequence: operators of the same structure (an ensemble's
# models of one bath size differ only in their coefficients) are encoded once
_TERM_ENCODING = {}


class DeviceOp:
    """Operator dict compiled to the device term table of ``edgpu_terms``.

    Upstream format ``{((i, 'c'|'a'), ...): amplitude}`` (impurityModel/ed/finite.py:1301);
    term order is the dict order, which fixes the summation order of equal outputs.
    """

    def __init__(self, op, device):
        t = len(op)
        keys = tuple(op.keys())
        coeff = np.array(list(op.values()), dtype=np.complex128).reshape(t).view(np.float64).reshape(t, 2).copy()
        hit = _TERM_ENCODING.get(keys)
        if hit is None:
            ops, flags, max_orb = self._encode(keys)
            if len(_TERM_ENCODING) >= 64:
                _TERM_ENCODING.clear()
            _TERM_ENCODING[keys] = (ops, flags, max_orb)
        else:
            ops, flags, max_orb = hit
        self._finish(t, ops, flags, coeff, max_orb, device)

    @staticmethod
    def _encode(keys):
        """Packed operators and flags of a key sequence (validated)."""
        t = len(keys)
        ops = np.zeros(t, dtype=np.uint64)
        flags = np.zeros(t, dtype=np.uint32)
        enc = {}  # (index, 'c'|'a') -> (16-bit code, index, created); each pair validated once
        max_orb = -1
        for k, key in enumerate(keys):
            if len(key) > 4:
                raise ValueError("terms with more than four operators are not supported")
            packed = 0
            cre = []
            ann = []
            for j, pair in enumerate(key):
                e = enc.get(pair)
                if e is None:
                    i, a = pair
                    if a not in ("c", "a"):
                        raise ValueError("Operator type unknown: {}".format(a))
                    i = int(i)
                    if not 0 <= i < 1024:
                        raise ValueError("spin-orbital index out of range: %d" % i)
                    e = enc[pair] = (0x8000 | (0x4000 if a == "c" else 0) | i, i, a == "c")
                packed |= e[0] << (16 * j)
                (cre if e[2] else ann).append(e[1])
                if e[1] > max_orb:
                    max_orb = e[1]
            ops[k] = packed
            if len(cre) == 1 and len(ann) == 1:
                diag = cre[0] == ann[0]
            else:
                diag = sorted(cre) == sorted(ann)
            flags[k] = (1 if diag else 0) | (len(key) << 8)
        return ops, flags, max_orb

    def _finish(self, t, ops, flags, coeff, max_orb, device):
        self.n_terms = t
        self.max_orbital = max_orb
        self._ops_host = ops
        self._flags_host = flags
        self._moves = None
        self.is_real = bool(np.all(coeff[:, 1] == 0.0))
        self.nbytes = ops.nbytes + coeff.nbytes + flags.nbytes
        self.ops = torch.from_numpy(ops.view(np.int64)).to(device)
        self.coeff = torch.from_numpy(coeff).to(device)
        self.flags = torch.from_numpy(flags.view(np.int32)).to(device)
        self.terms = L.Terms(self.ops.data_ptr() if t else 0, self.coeff.data_ptr() if t else 0,
                             self.flags.data_ptr() if t else 0, t)

    @property
    def moves(self):
        """Off-diagonal terms moving each orbital (host array [max_orbital + 1]): orbitals in the
        symmetric difference of a term's created and annihilated sets (orders sector rows for
        locality)."""
        if self._moves is None:
            t = self.n_terms
            code = np.stack([(self._ops_host >> np.uint64(16 * j)) & np.uint64(0xFFFF) for j in range(4)], 1)
            code = code.astype(np.int64).reshape(t, 4)
            valid = (code & 0x8000) != 0
            orb = np.where(valid, code & 0x3FF, -1)
            cre = valid & ((code & 0x4000) != 0)
            ann = valid & ~cre
            same = orb[:, :, None] == orb[:, None, :]
            in_cre = (same & cre[:, None, :]).any(2)
            in_ann = (same & ann[:, None, :]).any(2)
            first = ~np.tril(same, -1).any(2)  # first slot holding this orbital
            off = (self._flags_host & 1) == 0
            moved = valid & (in_cre != in_ann) & first & off[:, None]
            self._moves = np.bincount(orb[moved], minlength=self.max_orbital + 1)
        return self._moves


def make_restrictions(restrictions, n_spin_orbitals):
    """``{frozenset(indices): (lo, hi)}`` -> ``edgpu_restrictions`` (None when absent)."""
    if not restrictions:
        return None
    r = L.Restrictions()
    items = list(restrictions.items())
    if len(items) > L.MAX_RESTRICTIONS:
        raise ValueError("at most %d restrictions are supported" % L.MAX_RESTRICTIONS)
    r.n = len(items)
    for k, (idx, (lo, hi)) in enumerate(items):
        r.lo[k] = int(lo)
        r.hi[k] = int(hi)
        for q in range(L.MAX_WORDS):
            r.mask[k][q] = 0
        for i in idx:
            i = int(i)
            if not 0 <= i < 64 * L.MAX_WORDS:
                raise ValueError("restriction index out of range: %d" % i)
            r.mask[k][i // 64] |= 1 << (63 - i % 64)
    return r


def _restr_key(restr):
    if restr is None:
        return None
    return tuple((int(restr.lo[k]), int(restr.hi[k]), tuple(int(x) for x in restr.mask[k])) for k in range(restr.n))


class CsrMatrix:
    """CSR Hamiltonian on the device (row j holds <j|H|k> for the sector basis)."""

    def __init__(self, row_ptr, col, val_c=None, val_r=None, ncols=None):
        self.row_ptr = row_ptr
        self.col = col
        self.val_c = val_c
        self.val_r = val_r
        self.val_cf = None
        self.val_rf = None
        self.val_df = None
        self.mixed_shift = 0.0
        self.n = row_ptr.numel() - 1
        self.ncols = self.n if ncols is None else int(ncols)
        self.nnz = col.numel()
        self._struct = None
        self.order_tag = "sorted"  # row order (autotuner bucket): "sorted" basis or a permutation's tag

    def mixed(self):
        """Add the float32 / complex64 copy of H - shift*I used by the mixed-precision form.

        The shift is the mean diagonal element: with diagonals near -800 eV a float32 copy
        of H itself would carry ~5e-5 eV absolute rounding; H - shift keeps the float32
        entries small.  Callers add ``mixed_shift`` back to the Lanczos alphas.
        """
        if self.val_rf is not None or self.val_cf is not None:
            return self
        rows = torch.repeat_interleave(torch.arange(self.n, device=self.row_ptr.device),
                                       self.row_ptr[1:] - self.row_ptr[:-1], output_size=int(self.col.shape[0]))
        diag = rows == self.col.to(torch.int64)
        # the shift needs a stored diagonal entry in every row (H - shift*I keeps H's pattern)
        full_diag = int(diag.sum().item()) == self.n
        if self.val_r is not None:
            d = self.val_r[diag]
            self.mixed_shift = float(d.mean().item()) if d.numel() and full_diag else 0.0
            v = self.val_r.clone()
            v[diag] -= self.mixed_shift
            self.val_rf = v.to(torch.float32)
        else:
            d = self.val_c[diag, 0]
            self.mixed_shift = float(d.mean().item()) if d.numel() and full_diag else 0.0
            v = self.val_c.clone()
            v[diag, 0] -= self.mixed_shift
            self.val_cf = v.to(torch.float32)
        self._struct = None
        return self

    def double_float(self):
        """Add the (hi, lo) float-pair copy of a real H used by the double-float Lanczos form.

        hi = fl32(h), lo = fl32(h - hi): hi + lo equals h to about 2^-48 relative, so no
        shift is needed.  Complex matrices keep no copy (the form then runs in FP64).
        """
        if self.val_df is not None or self.val_r is None:
            return self
        hi = self.val_r.to(torch.float32)
        lo = (self.val_r - hi.to(torch.float64)).to(torch.float32)
        self.val_df = torch.stack([hi, lo], dim=1).contiguous()
        self._struct = None
        return self

    def struct(self):
        if self._struct is None:
            s = L.CSR()
            s.n = self.n
            s.nnz = self.nnz
            s.row_ptr = self.row_ptr.data_ptr()
            s.col = self.col.data_ptr() if self.nnz else self.row_ptr.data_ptr()
            s.val_c = self.val_c.data_ptr() if self.val_c is not None and self.nnz else None
            s.val_r = self.val_r.data_ptr() if self.val_r is not None and self.nnz else None
            if self.nnz == 0:
                s.val_r = self.row_ptr.data_ptr()
            s.val_cf = self.val_cf.data_ptr() if self.val_cf is not None and self.nnz else None
            s.val_rf = self.val_rf.data_ptr() if self.val_rf is not None and self.nnz else None
            s.val_df = self.val_df.data_ptr() if self.val_df is not None and self.nnz else None
            self._struct = s
        return self._struct

    def value_bytes(self):
        return 16 if self.val_c is not None else 8

    def permuted(self, perm, tag="permuted"):
        """The same operator on the basis reordered by ``perm`` (new position -> old index):
        P H P^T, row k' = old row perm[k'] with its columns renumbered and its entries kept in
        their stored order (so every row sums its terms in the same order as before).  FP64
        values only; call ``mixed()`` / ``double_float()`` on the result for the copies."""
        n = self.n
        if perm.numel() != n or self.ncols != n:
            raise ValueError("permuted: square operator and a permutation of its rows needed")
        dev = self.row_ptr.device
        inv = torch.empty_like(perm)
        inv[perm] = torch.arange(n, dtype=perm.dtype, device=dev)
        lens = self.row_ptr[1:] - self.row_ptr[:-1]
        rows = torch.repeat_interleave(torch.arange(n, device=dev), lens, output_size=self.nnz)
        # entries grouped by new row; a stable sort keeps each row's stored order
        idx = torch.sort(inv[rows], stable=True).indices
        row_ptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        row_ptr[1:] = torch.cumsum(lens[perm], 0)
        col = inv[self.col.to(torch.int64)[idx]].to(torch.int32)
        out = CsrMatrix(row_ptr, col, val_c=None if self.val_c is None else self.val_c[idx].contiguous(),
                        val_r=None if self.val_r is None else self.val_r[idx].contiguous())
        out.order_tag = tag
        return out


COMPONENTS_KERNEL_MAX_ROWS = 1 << 16  # single-CTA label propagation of edgpu_components


def _df_to_c128(v):
    """complex128-sized buffer holding double-float elements (re.hi, re.lo, im.hi, im.lo as
    float32) -> the complex128 values."""
    f = torch.view_as_real(v).contiguous().view(torch.float32).view(*v.shape, 4).to(torch.float64)
    return torch.complex(f[..., 0] + f[..., 1], f[..., 2] + f[..., 3])

def _c128_to_df(v):
    """complex128 values -> a complex128-sized buffer of double-float elements (re.hi, re.lo,
    im.hi, im.lo as float32; hi + lo equals the value to about 2^-48 relative)."""
    r = torch.view_as_real(v.contiguous())
    hi = r.to(torch.float32)
    lo = (r - hi.to(torch.float64)).to(torch.float32)
    f = torch.stack([hi[..., 0], lo[..., 0], hi[..., 1], lo[..., 1]], -1).contiguous()
    return torch.view_as_complex(f.view(torch.float64).view(*v.shape, 2))


# raw handle of the current stream without building a torch Stream object (about 10 us less
# per library call); the public accessor is the fallback
_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


class Engine:
    """One engine per CUDA device.  Holds the library handle and, per CUDA stream that issues
    work, a status word and a workspace (so that pipelines on different streams never share
    either)."""

    def __init__(self, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("impuritymodel_gb300 needs a CUDA device (there is no CPU fallback)")
        self.lib = L.load()
        self.device = torch.device(device if device is not None else "cuda")
        self._dev_index = self.device.index if self.device.index is not None else torch.cuda.current_device()
        self._lanes = {}
        self._side = []
        self.scratch_entries = 256
        # time the CTA sizes of the batched double-float Lanczos once per problem bucket
        self.tune_lanczos = True
        # bytes moved across the host<->device boundary by the drop-in API (inputs/results)
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        # sectors built by the drop-in API calls of a session (see remember_sector)
        self.sectors = []

    # -- session sector cache (the role of upstream's h_dict memo across calls) ------------
    def remember_sector(self, kind, dop, restr, item, keep=8):
        """Keep a sector built by a drop-in call: ``kind`` "closure" (a Sector closed under the
        restricted operator) or "basis" (an eigensystem basis with its Hamiltonian)."""
        rkey = _restr_key(restr)
        self.sectors = [e for e in self.sectors if e[3] is not item][-(keep - 1):] + [(kind, dop, rkey, item)]

    def sectors_for(self, kind, dop, restr):
        """Sectors of this kind kept for the same operator object and restrictions, newest
        first."""
        rkey = _restr_key(restr)
        return [e[3] for e in reversed(self.sectors) if e[0] == kind and e[1] is dop and e[2] == rkey]

    def clear_sectors(self):
        self.sectors = []

    # -- plumbing -------------------------------------------------------------------------
    def _stream_handle(self):
        if _raw_stream is not None:
            return _raw_stream(self._dev_index)
        return torch.cuda.current_stream(self.device).cuda_stream

    @property
    def stream(self):
        return C.c_void_p(self._stream_handle())

    def _lane(self):
        h = self._stream_handle()
        lane = self._lanes.get(h)
        if lane is None:
            lane = self._lanes[h] = [torch.zeros(1, dtype=torch.int32, device=self.device),
                                     torch.empty(1 << 20, dtype=torch.uint8, device=self.device)]
        return lane

    @property
    def status(self):
        """Device status word of the current stream (edgpu_* error codes)."""
        return self._lane()[0]

    def side_stream(self, k=0):
        """The k-th high-priority side stream of this engine (created on first use)."""
        while len(self._side) <= k:
            self._side.append(torch.cuda.Stream(self.device, priority=-1))
        return self._side[k]

    def workspace(self, nbytes):
        nbytes = int(nbytes)
        lane = self._lane()
        if lane[1].numel() < nbytes:
            lane[1] = torch.empty(max(nbytes, 2 * lane[1].numel()), dtype=torch.uint8, device=self.device)
        return C.c_void_p(lane[1].data_ptr()), C.c_size_t(lane[1].numel())

    def reset_status(self):
        self.status.zero_()

    def read_status(self, where):
        st = int(self.status.item())
        if st != L.EDGPU_OK:
            raise L.EdgpuError(st, where)

    def upload_states(self, words):
        words = np.ascontiguousarray(words, dtype=np.uint64)
        self.h2d_bytes += words.nbytes
        return torch.from_numpy(words.view(np.int64)).to(self.device)

    def download_states(self, t):
        self.d2h_bytes += t.numel() * t.element_size()
        return t.cpu().numpy().view(np.uint64)

    def to_device(self, arr):
        """Host NumPy array -> device tensor (counted as API input traffic)."""
        arr = np.ascontiguousarray(arr)
        self.h2d_bytes += arr.nbytes
        return torch.from_numpy(arr).to(self.device)

    def to_host(self, t):
        """Device tensor -> host NumPy array (counted as API result traffic).  Results of more
        than 1 MiB go through page-locked memory (torch's host caching allocator): on the
        Grace host a 145 MB map copies in under 1 ms that way, against 6-20 ms pageable."""
        nbytes = t.numel() * t.element_size()
        self.d2h_bytes += nbytes
        if nbytes <= (1 << 20) or not t.is_cuda:
            return t.cpu().numpy()
        host = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        host.copy_(t)
        return host.numpy()

    # -- primitives -----------------------------------------------------------------------
    def scan(self, counts):
        n = counts.numel()
        out = torch.empty(n + 1, dtype=torch.int64, device=self.device)
        ws, wsn = self.workspace(self.lib.edgpu_scan_workspace(n))
        L.check(self.lib.edgpu_scan_i64(_ptr(counts), _ptr(out), n, ws, wsn, self.stream), "scan")
        return out

    def sort_states(self, keys, payload):
        """In-place stable sort of ``keys`` [M, W] with ``payload`` int32 [M]."""
        m, w = keys.shape
        if m <= 1:
            return keys, payload
        if m <= 8192 and (1 << (m - 1).bit_length()) * (8 * w + 4) <= 160 * 1024:
            # one-CTA bitonic sort in the library: no byte-variation pass and no host read
            L.check(self.lib.edgpu_sort_states(w, _ptr(keys), _ptr(payload), m, None, C.c_void_p(0), 0,
                                               self.stream), "sort")
            return keys, payload
        vary = torch.empty(w, dtype=torch.int64, device=self.device)
        L.check(self.lib.edgpu_vary_mask(w, _ptr(keys), m, _ptr(vary), self.stream), "vary_mask")
        vm = vary.cpu().numpy().view(np.uint64).copy()
        arr = (C.c_uint64 * w)(*[int(x) for x in vm])
        ws, wsn = self.workspace(self.lib.edgpu_sort_states_workspace(w, m))
        L.check(self.lib.edgpu_sort_states(w, _ptr(keys), _ptr(payload), m, arr, ws, wsn, self.stream), "sort")
        return keys, payload

    def unique_sorted(self, keys, payload=None, vals=None):
        """Unique rows of sorted keys.  Returns (keys, first_payload, summed vals or None)."""
        m, w = keys.shape
        if m == 0:
            return keys, payload, vals
        head = torch.empty(m, dtype=torch.int64, device=self.device)
        L.check(self.lib.edgpu_segment_heads(w, _ptr(keys), m, _ptr(head), self.stream), "segment_heads")
        hs = self.scan(head)
        nu = int(hs[-1].item())
        out_keys = torch.empty((nu, w), dtype=torch.int64, device=self.device)
        if payload is None:
            payload = torch.arange(m, dtype=torch.int32, device=self.device)
        out_first = torch.empty(nu, dtype=torch.int32, device=self.device)
        out_vals = torch.empty((nu, 2), dtype=torch.float64, device=self.device) if vals is not None else None
        L.check(
            self.lib.edgpu_segment_reduce(w, _ptr(keys), _ptr(payload), m, _ptr(hs), _ptr(vals), _ptr(out_keys),
                                          _ptr(out_first), _ptr(out_vals), self.stream),
            "segment_reduce",
        )
        return out_keys, out_first, out_vals

    def merge(self, a, b):
        na, w = a.shape
        nb = b.shape[0]
        out = torch.empty((na + nb, w), dtype=torch.int64, device=self.device)
        L.check(self.lib.edgpu_merge_states(w, _ptr(a), na, _ptr(b), nb, _ptr(out), self.stream), "merge")
        return out

    def lookup(self, basis, query):
        nq, w = query.shape
        out = torch.empty(nq, dtype=torch.int64, device=self.device)
        L.check(self.lib.edgpu_lookup_states(w, _ptr(basis), basis.shape[0], _ptr(query), nq, _ptr(out), self.stream),
                "lookup")
        return out

    def sort_unique(self, keys):
        """Sorted unique rows of ``keys`` (copy)."""
        k = keys.clone()
        p = torch.arange(k.shape[0], dtype=torch.int32, device=self.device)
        self.sort_states(k, p)
        u, _, _ = self.unique_sorted(k, p)
        return u

    # -- operator application -------------------------------------------------------------
    def apply_columns(self, states, dop, restr, weight_min, basis=None, filt=L.FILTER_NONE, want_states=False,
                      want_index=False, want_vals=False, conj=False):
        """Per-state H|b> (see edgpu_apply_columns). Returns (offsets, states, index, vals)."""
        n, w = states.shape
        offsets = torch.zeros(n + 1, dtype=torch.int64, device=self.device)
        empty = torch.empty((0, w), dtype=torch.int64, device=self.device)
        if n == 0 or dop.n_terms == 0:
            return offsets, empty, torch.empty(0, dtype=torch.int64, device=self.device), torch.empty(
                (0, 2), dtype=torch.float64, device=self.device)
        counts = torch.empty(n, dtype=torch.int64, device=self.device)
        rp = C.byref(restr) if restr is not None else None
        bptr = _ptr(basis) if basis is not None else C.c_void_p(0)
        nb = basis.shape[0] if basis is not None else 0
        while True:
            self.reset_status()
            L.check(
                self.lib.edgpu_apply_columns(w, _ptr(states), n, C.byref(dop.terms), rp, weight_min, bptr, nb, filt,
                                             None, _ptr(counts), None, None, None, 0, self.scratch_entries,
                                             _ptr(self.status), self.stream),
                "apply_columns(count)",
            )
            offsets = self.scan(counts)
            # the status and the emission total in one read (the scan of an overflowed count
            # pass is discarded)
            st, total = (int(x) for x in torch.cat([self.status.to(torch.int64).view(1), offsets[-1:]]).cpu())
            if st == L.EDGPU_ERR_OVERFLOW and self.scratch_entries < 8192:
                self.scratch_entries *= 4
                continue
            if st != L.EDGPU_OK:
                raise L.EdgpuError(st, "apply_columns(count)")
            break
        out_s = torch.empty((total, w), dtype=torch.int64, device=self.device) if want_states else None
        out_i = torch.empty(total, dtype=torch.int64, device=self.device) if want_index else None
        out_v = torch.empty((total, 2), dtype=torch.float64, device=self.device) if want_vals else None
        if total:
            self.reset_status()
            L.check(
                self.lib.edgpu_apply_columns(w, _ptr(states), n, C.byref(dop.terms), rp, weight_min, bptr, nb, filt,
                                             _ptr(offsets), None, _ptr(out_s), _ptr(out_i), _ptr(out_v), int(conj),
                                             self.scratch_entries, _ptr(self.status), self.stream),
                "apply_columns(fill)",
            )
            self.read_status("apply_columns(fill)")
        return offsets, out_s, out_i, out_v

    def apply_vector_raw(self, states, amps, dop, restr):
        """Raw emissions (state, term) ordered.  Returns (offsets, out_states, out_vals)."""
        n, w = states.shape
        if n == 0 or dop.n_terms == 0:
            return (torch.zeros(n + 1, dtype=torch.int64, device=self.device),
                    torch.empty((0, w), dtype=torch.int64, device=self.device),
                    torch.empty((0, 2), dtype=torch.float64, device=self.device))
        counts = torch.empty(n, dtype=torch.int64, device=self.device)
        rp = C.byref(restr) if restr is not None else None
        L.check(self.lib.edgpu_apply_vector(w, _ptr(states), None, n, C.byref(dop.terms), rp, None, _ptr(counts), None,
                                            None, self.stream), "apply_vector(count)")
        offsets = self.scan(counts)
        total = int(offsets[-1].item())
        out_s = torch.empty((total, w), dtype=torch.int64, device=self.device)
        out_v = torch.empty((total, 2), dtype=torch.float64, device=self.device)
        if total:
            L.check(self.lib.edgpu_apply_vector(w, _ptr(states), _ptr(amps), n, C.byref(dop.terms), rp,
                                                _ptr(offsets), None, _ptr(out_s), _ptr(out_v), self.stream),
                    "apply_vector(fill)")
        return offsets, out_s, out_v

    def apply_vectors(self, run_states, run_amps, dop, restr, weight_min):
        """psi'_r = Op psi_r for several runs r (upstream applyOp per run, finite.py:1301-1511).

        ``run_states``/``run_amps``: lists of [n_r, W] int64 and [n_r, 2] float64 device
        tensors.  Returns per-run (states [m_r, W], amps [m_r, 2]) with outputs merged in
        upstream order (psi order, then term order), pruned at |a|^2 < weight_min, and listed
        in first-occurrence (dict insertion) order.
        """
        runs = len(run_states)
        w = run_states[0].shape[1] if runs else 1
        sizes = [int(s.shape[0]) for s in run_states]
        if sum(sizes) == 0 or dop.n_terms == 0:
            z = [(torch.empty((0, w), dtype=torch.int64, device=self.device),
                  torch.empty((0, 2), dtype=torch.float64, device=self.device)) for _ in range(runs)]
            return z
        states = torch.cat(run_states, 0)
        amps = torch.cat(run_amps, 0)
        offsets, out_s, out_v = self.apply_vector_raw(states, amps, dop, restr)
        total = out_s.shape[0]
        if total == 0:
            return [(out_s[:0], out_v[:0]) for _ in range(runs)]
        run_of_input = torch.repeat_interleave(torch.arange(runs, device=self.device),
                                               torch.tensor(sizes, device=self.device), output_size=sum(sizes))
        counts = offsets[1:] - offsets[:-1]
        run_of_emit = torch.repeat_interleave(run_of_input, counts, output_size=total)
        keys = torch.cat([run_of_emit.view(-1, 1), out_s], 1).contiguous()
        payload = torch.arange(total, dtype=torch.int32, device=self.device)
        self.sort_states(keys, payload)
        ukeys, first, sums = self.unique_sorted(keys, payload, out_v)
        a2 = torch.hypot(sums[:, 0], sums[:, 1]) ** 2
        keep = a2 >= weight_min
        ukeys, first, sums = ukeys[keep], first[keep], sums[keep]
        # dict insertion order: by first emission index within each run
        order = torch.argsort(first.to(torch.int64))
        ukeys, sums = ukeys[order], sums[order]
        run_id = ukeys[:, 0]
        out = []
        bounds = torch.searchsorted(torch.sort(run_id).values, torch.arange(runs + 1, device=self.device))
        # runs are interleaved after the first-occurrence ordering only if emissions of
        # run r all precede run r+1, which holds since inputs are concatenated by run.
        b = bounds.cpu().tolist()
        for r in range(runs):
            out.append((ukeys[b[r]:b[r + 1], 1:].contiguous(), sums[b[r]:b[r + 1]].contiguous()))
        return out

    def apply_vectors_multi(self, run_states, run_amps, dops, restr, weight_min):
        """``[op][run] -> (states, amps)``: every operator of ``dops`` applied to every run.

        The same results, bit for bit, as one ``apply_vectors`` call per operator, with one
        scan, one sort and one unique over all (operator, run) pairs instead of one each per
        operator (the count and fill passes still run per operator)."""
        runs, n_ops = len(run_states), len(dops)
        w = run_states[0].shape[1] if runs else 1
        empty = (torch.empty((0, w), dtype=torch.int64, device=self.device),
                 torch.empty((0, 2), dtype=torch.float64, device=self.device))
        if runs == 0 or n_ops == 0:
            return [[] for _ in range(n_ops)] if runs == 0 else []
        sizes = [int(x.shape[0]) for x in run_states]
        n = sum(sizes)
        if n == 0:
            return [[empty] * runs for _ in range(n_ops)]
        states = torch.cat(run_states, 0).contiguous()
        amps = torch.cat(run_amps, 0).contiguous()
        rp = C.byref(restr) if restr is not None else None
        counts = torch.zeros(n_ops * n, dtype=torch.int64, device=self.device)
        for o, dop in enumerate(dops):
            if dop.n_terms:
                L.check(self.lib.edgpu_apply_vector(w, _ptr(states), None, n, C.byref(dop.terms), rp, None,
                                                    _ptr(counts[o * n:]), None, None, self.stream),
                        "apply_vector(count)")
        offsets = self.scan(counts)
        total = int(offsets[-1].item())
        if total == 0:
            return [[empty] * runs for _ in range(n_ops)]
        out_s = torch.empty((total, w), dtype=torch.int64, device=self.device)
        out_v = torch.empty((total, 2), dtype=torch.float64, device=self.device)
        for o, dop in enumerate(dops):
            if dop.n_terms:
                L.check(self.lib.edgpu_apply_vector(w, _ptr(states), _ptr(amps), n, C.byref(dop.terms), rp,
                                                    _ptr(offsets[o * n:]), None, _ptr(out_s), _ptr(out_v),
                                                    self.stream), "apply_vector(fill)")
        run_of_input = torch.repeat_interleave(torch.arange(runs, device=self.device),
                                               torch.tensor(sizes, device=self.device), output_size=n)
        group = (torch.arange(n_ops, device=self.device).view(-1, 1) * runs + run_of_input.view(1, -1)).reshape(-1)
        group_of_emit = torch.repeat_interleave(group, offsets[1:] - offsets[:-1], output_size=total)
        keys = torch.cat([group_of_emit.view(-1, 1), out_s], 1).contiguous()
        payload = torch.arange(total, dtype=torch.int32, device=self.device)
        self.sort_states(keys, payload)
        ukeys, first, sums = self.unique_sorted(keys, payload, out_v)
        a2 = torch.hypot(sums[:, 0], sums[:, 1]) ** 2
        keep = a2 >= weight_min
        ukeys, first, sums = ukeys[keep], first[keep], sums[keep]
        order = torch.argsort(first.to(torch.int64))  # dict insertion order within each group
        ukeys, sums = ukeys[order], sums[order]
        bounds = torch.searchsorted(ukeys[:, 0].contiguous(),
                                    torch.arange(n_ops * runs + 1, device=self.device)).cpu().tolist()
        out = []
        for o in range(n_ops):
            row = []
            for r in range(runs):
                g = o * runs + r
                row.append((ukeys[bounds[g]:bounds[g + 1], 1:].contiguous(), sums[bounds[g]:bounds[g + 1]].contiguous()))
            out.append(row)
        return out

    # -- sectors --------------------------------------------------------------------------
    def expand(self, basis0, dop, restr, weight_min=1e-12):
        """Closure of ``basis0`` under the operator (upstream expand_basis, finite.py:1696-1803).

        Returns (sorted basis [N, W], layered order [N, W]); the layered order is upstream's
        basis order: ``basis0`` as given, then each breadth-first layer sorted.
        """
        s_sorted = self.sort_unique(basis0)
        layers = [basis0]
        frontier = basis0
        while frontier.shape[0] > 0:
            _, cand, _, _ = self.apply_columns(frontier, dop, restr, weight_min, basis=s_sorted,
                                               filt=L.FILTER_NOT_IN_BASIS, want_states=True)
            if cand.shape[0] == 0:
                break
            new = self.sort_unique(cand)
            s_sorted = self.merge(s_sorted, new)
            layers.append(new)
            frontier = new
        return s_sorted, torch.cat(layers, 0)

    def build_csr(self, basis_sorted, dop, restr, weight_min=1e-12):
        """Sector Hamiltonian on a sorted basis (upstream get_hamiltonian_matrix_from_h_dict).

        Column j of H (= H|b_j>) becomes row j with conjugated values, which for the
        Hermitian H is row j of H.  Real operators store float64 values.
        """
        offsets, _, idx, vals = self.apply_columns(basis_sorted, dop, restr, weight_min, basis=basis_sorted,
                                                   filt=L.FILTER_IN_BASIS, want_index=True, want_vals=True, conj=True)
        col = idx.to(torch.int32)
        if dop.is_real:
            return CsrMatrix(offsets, col, val_r=vals[:, 0].contiguous())
        return CsrMatrix(offsets, col, val_c=vals.contiguous())

    def components(self, csr):
        """Connected-component label (smallest member index) of every sector state."""
        n = csr.n
        if 0 < n <= COMPONENTS_KERNEL_MAX_ROWS:
            labels = torch.empty(n, dtype=torch.int64, device=self.device)
            L.check(self.lib.edgpu_components(C.byref(csr.struct()), _ptr(labels), None, self.stream), "components")
            return labels
        labels = torch.arange(n, dtype=torch.int64, device=self.device)
        if csr.nnz == 0:
            return labels
        rows = torch.repeat_interleave(torch.arange(n, device=self.device), csr.row_ptr[1:] - csr.row_ptr[:-1],
                                       output_size=int(csr.col.shape[0]))
        cols = csr.col.to(torch.int64)
        for _ in range(10 * n + 10):
            m = torch.minimum(labels[rows], labels[cols])
            new = labels.clone()
            new.scatter_reduce_(0, rows, m, reduce="amin")
            new.scatter_reduce_(0, cols, m, reduce="amin")
            new = new[new]
            if torch.equal(new, labels):
                break
            labels = new
        return labels

    def run_dims(self, csr, v0_nonzero_rows, run_of_row, runs):
        """Dimension of the closure of each run's support (upstream len(basis_index))."""
        labels = self.components(csr)
        uniq, inv = torch.unique(labels, return_inverse=True)
        sizes = torch.bincount(inv, minlength=uniq.numel())
        comp = inv[v0_nonzero_rows]
        pair = torch.unique(run_of_row * uniq.numel() + comp)
        dims = torch.zeros(runs, dtype=torch.int64, device=self.device)
        dims.index_add_(0, pair // uniq.numel(), sizes[pair % uniq.numel()])
        return dims

    # -- Krylov ---------------------------------------------------------------------------
    def lanczos(self, csr, v0, k_max, precision=0, timing=None, check=True):
        """Batched Lanczos on R start vectors v0 [N, R] complex128 (normalised).

        ``check=False`` only enqueues the work: the caller reads the status later on the same
        stream (``read_status``) before it relies on alpha and beta."""
        n, r = v0.shape
        if n != csr.n or csr.ncols != csr.n:
            raise ValueError("lanczos: square matrix of size %d required for vectors of size %d" % (csr.n, n))
        k_h = np.asarray(k_max.cpu() if torch.is_tensor(k_max) else k_max, dtype=np.int32)
        kmax = torch.from_numpy(k_h).to(self.device)
        K = int(k_h.max())
        alpha = torch.zeros((r, K), dtype=torch.float64, device=self.device)
        beta = torch.zeros((r, K), dtype=torch.float64, device=self.device)
        if precision == 1:
            csr.mixed()
        elif precision == 3:
            csr.double_float()
        elif precision != 0:
            raise ValueError("lanczos: precision must be 0, 1 or 3")
        v0r = torch.view_as_real(v0.contiguous()) if v0.is_complex() else v0
        ws, wsn = self.workspace(self.lib.edgpu_lanczos_workspace(n, r, K, precision))
        cta = self._lanczos_cta(csr, v0r, r, kmax, K, precision, ws, wsn) if self.tune_lanczos else -1
        self.reset_status()
        if timing is None:
            self.lib.edgpu_set_lanczos_cta(cta)
            try:
                L.check(self.lib.edgpu_lanczos(C.byref(csr.struct()), _ptr(v0r), r, _ptr(kmax), K, precision,
                                               _ptr(alpha), _ptr(beta), _ptr(self.status), ws, wsn, self.stream),
                        "lanczos")
            finally:
                self.lib.edgpu_set_lanczos_cta(-1)
        else:
            ms = (C.c_double * 3)()
            L.check(self.lib.edgpu_lanczos_timed(C.byref(csr.struct()), _ptr(v0r), r, _ptr(kmax), K, precision,
                                                 _ptr(alpha), _ptr(beta), _ptr(self.status), ws, wsn, self.stream,
                                                 ms), "lanczos_timed")
            vb = 8 if precision == 1 else 16
            sb = (4 if precision == 1 else 8) * (2 if csr.val_c is not None else 1)
            timing.append(dict(n=csr.n, nnz=csr.nnz, R=r, K=K, precision=precision, spmm_ms=ms[0], axpy_ms=ms[1],
                               normalize_ms=ms[2], spmm_launches=K, vec_bytes=vb, val_bytes=sb))
        if check:
            self.read_status("lanczos")
        if precision == 1 and csr.mixed_shift:
            alpha += csr.mixed_shift  # Lanczos ran on H - shift*I
        return alpha, beta

    # CTA sizes of the double-float one-CTA-per-run Lanczos (index into the library's list)
    LANCZOS_CTAS = (-1, 0, 1, 2, 3, 4)
    LANCZOS_SMALL_ROWS = 32767  # sectors served by that kernel

    def _lanczos_cta(self, csr, v0r, r, kmax, K, precision, ws, wsn):
        """The CTA size the autotuner picked for the double-float one-CTA-per-run Lanczos in
        this (n, R, K) bucket, timed on this call's own inputs on first use; -1 (the built-in
        rule) for every other form."""
        if precision != 3 or csr.val_df is None or csr.n > self.LANCZOS_SMALL_ROWS or r < 64:
            return -1
        key = (bucket(csr.n), bucket(r), bucket(K))
        tuner = get_tuner()
        hit = tuner.lookup("lanczos_cta", key)
        if hit is not None:
            return int(hit[0])
        a_s = torch.empty((r, K), dtype=torch.float64, device=self.device)
        b_s = torch.empty_like(a_s)
        st = torch.zeros(1, dtype=torch.int32, device=self.device)

        def run(c):
            self.lib.edgpu_set_lanczos_cta(c[0])
            try:
                L.check(self.lib.edgpu_lanczos(C.byref(csr.struct()), _ptr(v0r), r, _ptr(kmax), K, precision,
                                               _ptr(a_s), _ptr(b_s), _ptr(st), ws, wsn, self.stream), "lanczos")
            finally:
                self.lib.edgpu_set_lanczos_cta(-1)

        return int(tuner.pick("lanczos_cta", key, [(c,) for c in self.LANCZOS_CTAS], run, reps=2, warmup=1)[0])

    def spmv(self, csr, x, precision=0, mapping=None):
        """y [csr.n, R] = csr @ x for x [csr.ncols, R].

        For R with R / (complex numbers per 16 bytes) dividing 32 the row-scheduled kernel
        runs with the launch mapping the autotuner picked for this matrix's shape bucket (or
        ``mapping`` = (window, heavy_min, unroll, block)); other R use the row kernel."""
        nx, r = x.shape
        if nx != csr.ncols:
            raise ValueError("spmv: x has %d rows, matrix has %d columns" % (nx, csr.ncols))
        n = csr.n
        if precision:
            csr.mixed()
            xr = torch.view_as_real(x.to(torch.complex64).contiguous())
            y = torch.empty((n, r), dtype=torch.complex64, device=self.device)
            if self.spmv_planned_ok(r, precision) and csr.nnz:
                self.spmv_into(csr, xr, torch.view_as_real(y), r, precision, mapping)
            else:
                L.check(self.lib.edgpu_spmv_c64(C.byref(csr.struct()), _ptr(xr), _ptr(torch.view_as_real(y)), r,
                                                self.stream), "spmv_c64")
            if csr.mixed_shift:
                y += csr.mixed_shift * x.to(torch.complex64)  # float32 copy holds H - shift*I
            return y
        xr = torch.view_as_real(x.contiguous())
        y = torch.empty((n, r), dtype=torch.complex128, device=self.device)
        if self.spmv_planned_ok(r, precision) and csr.nnz:
            self.spmv_into(csr, xr, torch.view_as_real(y), r, precision, mapping)
        else:
            L.check(self.lib.edgpu_spmv(C.byref(csr.struct()), _ptr(xr), _ptr(torch.view_as_real(y)), r,
                                        self.stream), "spmv")
        return y

    # -- H.v with a row schedule (edgpu_spmv_plan / edgpu_spmv_planned / edgpu_spmv_paged) -
    SPMV_WINDOWS = (256, 4096, 0)
    SPMV_HEAVY = (16, 32, 64)
    SPMV_UNROLL = (4, 8)
    SPMV_BLOCK = (128, 256)
    SPMV_PAGES = (256, 512, 1024)
    SPMV_SLOTS = (8, 16, 32)  # columns in flight per warp of the tensor-memory-accelerator form
    # The tensor-memory-accelerator form is not among the autotuner's candidates: on the
    # 462 120-state PS sector (R = 16, 128-byte x rows) it took 196-508 us against 51-53 us for
    # the per-lane gathers (one bulk-tensor operation per four 128-byte rows).
    SPMV_TMA = False

    @staticmethod
    def spmv_planned_ok(R, precision):
        runs = 2 if precision else 1
        if R % runs:
            return False
        lanes = R // runs
        return lanes <= 32 and 32 % lanes == 0

    def spmv_candidates(self, csr, R, precision):
        """Launch mappings of H.v that the autotuner chooses from, as tuples:
        ("sched", window, heavy_min, unroll, block, 0): every row through the CSR, heavy rows
        one warp each, light rows in length-sorted windows;
        ("pages", window, heavy_min, unroll, page_entries, flags): the same schedule packed
        into pages that one warp each copies into shared memory (real values, or complex64);
        flags bit 0 keeps two batches of gathers in flight, bit 1 adds L2 eviction hints;
        ("tma", window, heavy_min, slots, page_entries, 0): the same pages with the x rows
        gathered into shared memory by bulk-tensor gathers, `slots` columns in flight per warp
        (complex64 vectors)."""
        out = [("sched", w, hm, u, b, 0) for w in self.SPMV_WINDOWS for hm in self.SPMV_HEAVY
               for u in self.SPMV_UNROLL for b in self.SPMV_BLOCK]
        lanes = R // (2 if precision else 1)
        kind = self._pages_kind(csr, precision)
        if kind is not None and lanes in (2, 4, 8, 16):
            # a slice must fit a page: light rows are shorter than heavy_min, a heavy row is
            # dealt to the row groups (its page share is about len / groups columns)
            groups = 32 // lanes
            max_len = self._max_row_len(csr)
            for w in self.SPMV_WINDOWS:
                for hm in self.SPMV_HEAVY:
                    need = groups * (max(hm, -(-max_len // groups)) + 2)
                    out += [("pages", w, hm, u, ch, f) for u in self.SPMV_UNROLL for ch in self.SPMV_PAGES
                            for f in (0, 1, 2, 3) if need <= ch]
                    if precision and self.SPMV_TMA:  # complex64: x rows by bulk-tensor gathers
                        out += [("tma", w, hm, sl, ch, 0) for sl in self.SPMV_SLOTS for ch in self.SPMV_PAGES
                                if need <= ch]
        return out

    @staticmethod
    def _max_row_len(csr):
        if "_max_len" not in csr.__dict__:
            csr._max_len = int((csr.row_ptr[1:] - csr.row_ptr[:-1]).max().item()) if csr.n else 0
        return csr._max_len

    @staticmethod
    def _pages_kind(csr, precision):
        if precision:
            return 2 if csr.val_cf is not None else (0 if csr.val_rf is not None else None)
        return 1 if (csr.val_c is None and csr.val_r is not None) else None

    def spmv_plan(self, csr, window, heavy_min):
        """Row schedule (sched int32 [n], heavy-row count) of ``csr``, built once per
        (window, heavy_min) and kept with the matrix."""
        key = (int(window), int(heavy_min))
        plans = csr.__dict__.setdefault("_plans", {})
        if key not in plans:
            sched = torch.empty(csr.n, dtype=torch.int32, device=self.device)
            nh = C.c_int64(0)
            ws, wsn = self.workspace(self.lib.edgpu_spmv_plan_workspace(csr.n))
            L.check(self.lib.edgpu_spmv_plan(C.byref(csr.struct()), key[0], key[1], _ptr(sched), C.byref(nh), ws, wsn,
                                             self.stream), "spmv_plan")
            plans[key] = (sched, int(nh.value))
        return plans[key]

    def spmv_pages(self, csr, window, heavy_min, lanes, page_entries, kind):
        """Paged copy of the light rows (uint8 device buffer, page count), built once per
        (schedule, lanes, page size, value kind) and kept with the matrix."""
        key = (int(window), int(heavy_min), int(lanes), int(page_entries), int(kind))
        pages = csr.__dict__.setdefault("_pages", {})
        if key not in pages:
            sched, nh = self.spmv_plan(csr, window, heavy_min)
            ws, wsn = self.workspace(self.lib.edgpu_spmv_pages_workspace(csr.n, lanes))
            npg = C.c_int64(0)
            rc = self.lib.edgpu_spmv_pages_build(C.byref(csr.struct()), _ptr(sched), nh, lanes, page_entries, kind,
                                                 None, 0, C.byref(npg), ws, wsn, self.stream)
            if rc not in (L.EDGPU_OK, L.EDGPU_ERR_OVERFLOW):
                raise L.EdgpuError(rc, "spmv_pages_build")
            ebytes = 8 if kind == 0 else 16
            buf = torch.empty(max(1, npg.value) * page_entries * ebytes, dtype=torch.uint8, device=self.device)
            if npg.value:
                ws, wsn = self.workspace(self.lib.edgpu_spmv_pages_workspace(csr.n, lanes))
                L.check(self.lib.edgpu_spmv_pages_build(C.byref(csr.struct()), _ptr(sched), nh, lanes, page_entries,
                                                        kind, _ptr(buf), npg.value, C.byref(npg), ws, wsn, self.stream),
                        "spmv_pages_build")
            pages[key] = (buf, int(npg.value))
        return pages[key]

    def spmv_key(self, csr, R, precision):
        """Autotuner bucket of an H.v launch: sizes as powers of two, vector width, types."""
        key = (bucket(csr.n), bucket(max(1, csr.nnz // max(csr.n, 1))), int(R), "c64" if precision else "c128",
               "c" if (csr.val_c is not None or csr.val_cf is not None) else "r")
        tag = getattr(csr, "order_tag", "sorted")
        return key if tag == "sorted" else key + (tag,)

    def spmv_mapping(self, csr, xr, yr, R, precision):
        """The launch mapping the autotuner picked for this shape bucket, measured on this
        matrix and these vectors on first use."""
        return get_tuner().pick("spmv", self.spmv_key(csr, R, precision), self.spmv_candidates(csr, R, precision),
                                lambda c: self._spmv_planned(csr, xr, yr, R, precision, c))

    def _spmv_planned(self, csr, xr, yr, R, precision, mapping):
        kernel, w, hm, u, last, flags = mapping
        sched, nh = self.spmv_plan(csr, w, hm)
        if kernel == "tma":
            buf, npg = self.spmv_pages(csr, w, hm, R // 2, last, self._pages_kind(csr, precision))
            L.check(self.lib.edgpu_spmv_paged_tma_c64(C.byref(csr.struct()), _ptr(buf), npg, int(last), int(u),
                                                      _ptr(xr), _ptr(yr), int(R), _ptr(self.status), self.stream),
                    "spmv_paged_tma")
            return
        if kernel == "pages":
            lanes = R // (2 if precision else 1)
            buf, npg = self.spmv_pages(csr, w, hm, lanes, last, self._pages_kind(csr, precision))
            fn = self.lib.edgpu_spmv_paged_c64 if precision else self.lib.edgpu_spmv_paged
            L.check(fn(C.byref(csr.struct()), _ptr(buf), npg, int(last), int(u), int(flags), _ptr(xr), _ptr(yr),
                       int(R), self.stream), "spmv_paged")
            return
        fn = self.lib.edgpu_spmv_planned_c64 if precision else self.lib.edgpu_spmv_planned
        L.check(fn(C.byref(csr.struct()), _ptr(sched), nh, int(u), int(last), _ptr(xr), _ptr(yr), int(R), self.stream),
                "spmv_planned")

    def spmv_into(self, csr, xr, yr, R, precision=0, mapping=None):
        """yr = csr @ xr on real views of complex [rows][R] buffers (no allocation once the
        plan exists): the launch the H.v roofline times.  Returns the mapping used."""
        if mapping is None:
            mapping = self.spmv_mapping(csr, xr, yr, R, precision)
        self._spmv_planned(csr, xr, yr, R, precision, tuple(mapping))
        return tuple(mapping)

    def cfrac(self, alpha, beta, k_len, omega, delta, e, scale, precision=0):
        r, K = alpha.shape
        om = torch.as_tensor(np.asarray(omega, dtype=np.float64)).to(self.device)
        e_t = torch.as_tensor(np.asarray(e, dtype=np.float64)).to(self.device)
        sc = torch.as_tensor(np.asarray(scale, dtype=np.float64)).to(self.device)
        kl = torch.as_tensor(k_len, dtype=torch.int32).to(self.device)
        g = torch.empty((r, om.numel()), dtype=torch.complex128, device=self.device)
        if precision:
            ws, wsn = self.workspace(self.lib.edgpu_cfrac_f32_workspace(K, r))
            L.check(self.lib.edgpu_cfrac_f32(_ptr(alpha), _ptr(beta), _ptr(kl), K, r, _ptr(om), om.numel(),
                                             float(delta), _ptr(e_t), _ptr(sc), _ptr(torch.view_as_real(g)), ws, wsn,
                                             self.stream), "cfrac_f32")
            return g
        L.check(self.lib.edgpu_cfrac(_ptr(alpha), _ptr(beta), _ptr(kl), K, r, _ptr(om), om.numel(), float(delta),
                                     _ptr(e_t), _ptr(sc), _ptr(torch.view_as_real(g)), self.stream), "cfrac")
        return g

    def krylov_reorth(self, csr, v0, k_cap, stop=None, chunk=16, precision=0, remaining=None, locked=None):
        """Lanczos with full reorthogonalisation from v0 (normalised, [N] complex128).

        ``stop(alpha, beta, j)`` (host arrays of length j) returns True when converged.
        Returns (V [K, N], alpha [K], beta [K]) with K the number of steps taken;
        ``beta[:K-1]`` is the tridiagonal's off-diagonal and ``beta[K-1]`` the coupling to
        the next Krylov vector (0 when the space is exhausted).  ``precision=3`` runs the
        recurrence in double-float arithmetic (real H up to 65536 rows; otherwise FP64); V is
        returned in complex128 either way.  ``remaining(j)`` (optional) estimates the steps
        still needed after step j; the chunk queued ahead of each convergence test is cut
        to that estimate (at least 8 steps), so little work runs past convergence.

        ``locked`` ([m, N] complex128, orthonormal, optional): vectors every new Krylov vector
        is orthogonalised against (deflation).  They are placed ahead of v0 in the Krylov
        basis with a negligible coupling, so the Gram-Schmidt passes of every step remove
        their components and the recurrence runs on the orthogonal complement; v0 must be
        orthogonal to them.
        """
        n = csr.n
        if csr.ncols != n or v0.numel() != n:
            raise ValueError("krylov_reorth: square matrix and start vector of matching size required")
        m = 0 if locked is None else int(locked.shape[0])
        k_cap = int(min(k_cap, n - m))
        if k_cap < 1:
            raise ValueError("krylov_reorth: no room for a Krylov vector beside the locked ones")
        K_tot = m + k_cap
        df = precision == 3 and csr.val_c is None and csr.val_r is not None and n <= (1 << 16)
        if df:
            csr.double_float()
        launch = self.lib.edgpu_lanczos_reorth_df if df else self.lib.edgpu_lanczos_reorth
        V = torch.zeros((K_tot, n), dtype=torch.complex128, device=self.device)
        w = torch.zeros(n, dtype=torch.complex128, device=self.device)
        alpha = torch.zeros(K_tot, dtype=torch.float64, device=self.device)
        beta = torch.zeros(K_tot, dtype=torch.float64, device=self.device)
        if m and not df:
            # step m reads v_m = V[m]; beta_{m-1} = 0 leaves the locked vectors out of the
            # three-term update (the Gram-Schmidt passes remove their components)
            V[:m] = locked
            V[m] = v0
        elif m:
            # the double-float step m forms v_m = w / beta_{m-1} itself: w = 2^-60 v0 with
            # beta_{m-1} = 2^-60 gives v0 exactly (powers of two), and the three-term update
            # then subtracts only 2^-60 of V[m-1]
            tiny = 2.0 ** -60
            V[:m] = _c128_to_df(locked)
            w.copy_(_c128_to_df(v0 * tiny))
            beta[m - 1] = tiny
        ws, wsn = self.workspace(self.lib.edgpu_lanczos_reorth_workspace(n, K_tot))
        v0r = torch.view_as_real(v0.contiguous())
        # one pinned device-to-host copy per chunk (status, alpha and beta together), read
        # through an event, so the next chunk is already queued while the host tests this
        # one (a chunk past convergence only writes beyond the returned steps)
        host_t = torch.empty(1 + 2 * k_cap, dtype=torch.float64, pin_memory=True)

        def enqueue(j0, j1):
            # j0, j1 count the run's own steps; the kernel sees them after the locked vectors
            self.reset_status()
            L.check(launch(C.byref(csr.struct()), _ptr(v0r), m + j0, m + j1, K_tot, _ptr(torch.view_as_real(V)),
                           _ptr(torch.view_as_real(w)), _ptr(alpha), _ptr(beta), _ptr(self.status), ws, wsn,
                           self.stream), "lanczos_reorth")
            host_t[: 1 + 2 * j1].copy_(torch.cat([self.status.to(torch.float64), alpha[m:m + j1], beta[m:m + j1]]),
                                       non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            return ev

        j = 0
        j1 = min(k_cap, chunk)
        ev = enqueue(0, j1)
        while True:
            ev.synchronize()
            host = host_t[: 1 + 2 * j1].numpy().copy()
            size = chunk
            if remaining is not None:
                est = remaining(j1)
                if est is not None:
                    size = int(min(chunk, max(8, np.ceil(est) + 4)))
            jn = min(k_cap, j1 + size)
            ev_next = enqueue(j1, jn) if jn > j1 else None  # speculative next chunk
            st = int(host[0])
            ah, bh = host[1:1 + j1], host[1 + j1:]
            if st == L.EDGPU_ERR_BREAKDOWN:
                # invariant subspace: the Krylov space is exact at the first zero beta
                kb = int(np.argmax(bh == 0.0)) + 1
                return (_df_to_c128(V[m:m + kb]) if df else V[m:m + kb]), ah[:kb], bh[:kb]
            if st != L.EDGPU_OK:
                raise L.EdgpuError(st, "lanczos_reorth")
            j = j1
            if ev_next is None or (stop is not None and stop(ah, bh, j)):
                break
            j1, ev = jn, ev_next
        return (_df_to_c128(V[m:m + j]) if df else V[m:m + j]), ah[:j], bh[:j]

    def shifted_solve(self, csr, Y, zs, tol, k_cap, precision=0, check=True):
        """X[r, z] = (zs[r, z] - H)^{-1} Y[r] for all right-hand sides (one launch set).

        ``precision=3`` runs the Krylov recurrence in double-float arithmetic when H is real
        (complex H stays FP64).  Returns (X [R, nz, N] complex128, krylov sizes [R]) or None
        when the sector or the shift count exceeds the single-CTA kernel's limits.  With
        ``check=False`` the work is only enqueued and a third value, a function that reads the
        status (on the same stream), is returned."""
        r, n = Y.shape
        nz = zs.shape[1]
        k_cap = int(k_cap)
        if nz > 512 or 48 * n + 300 > 200 * 1024 or 16 * k_cap > 200 * 1024:
            return None
        df = precision == 3 and csr.val_c is None and csr.val_r is not None
        if df:
            csr.double_float()
        solve = self.lib.edgpu_shifted_solve_df if df else self.lib.edgpu_shifted_solve
        zt = torch.as_tensor(np.ascontiguousarray(zs, dtype=np.complex128)).to(self.device)
        X = torch.empty((r, nz, n), dtype=torch.complex128, device=self.device)
        m = torch.empty(r, dtype=torch.int32, device=self.device)
        ws, wsn = self.workspace(self.lib.edgpu_shifted_solve_workspace(n, r, nz, k_cap))
        self.reset_status()
        L.check(solve(C.byref(csr.struct()), _ptr(torch.view_as_real(Y.contiguous())), r, _ptr(torch.view_as_real(zt)),
                      nz, k_cap, float(tol), _ptr(torch.view_as_real(X)), _ptr(m), _ptr(self.status), ws, wsn,
                      self.stream), "shifted_solve")
        status = self.status

        def finish():
            st = int(status.item())
            if st == L.EDGPU_ERR_NOCONV:
                # upstream only prints when BiCGSTAB misses its tolerance (spectra.py:963-971)
                warnings.warn("shifted solve: residual tolerance %g not reached in %d Krylov steps" % (tol, k_cap))
            elif st != L.EDGPU_OK:
                raise L.EdgpuError(st, "shifted_solve")

        if not check:
            return X, m, finish
        finish()
        return X, m

    def combine(self, V, coeffs):
        """X[m] = sum_k coeffs[k, m] V[k] (complex128)."""
        k, n = V.shape
        cm = torch.as_tensor(np.ascontiguousarray(coeffs, dtype=np.complex128)).to(self.device)
        m = cm.shape[1]
        X = torch.empty((m, n), dtype=torch.complex128, device=self.device)
        L.check(self.lib.edgpu_combine(_ptr(torch.view_as_real(V)), k, n, _ptr(torch.view_as_real(cm)), m,
                                       _ptr(torch.view_as_real(X)), self.stream), "combine")
        return X

    # -- ragged batches (sectors of many models, one launch per solve) ---------------------
    def lanczos_ragged(self, batch, v0, k_max, alpha=None, beta=None, check=True):
        """Upstream's Lanczos for every run of a RaggedBatch; v0 packed complex128 [sum n_r].

        ``k_max`` is a host array or a device int32 tensor; with preallocated ``alpha``/
        ``beta`` and ``check=False`` the call enqueues work only (no host synchronisation),
        so it can be captured in a CUDA graph."""
        if torch.is_tensor(k_max):
            kmax = k_max
            K = alpha.shape[1]
        else:
            k_h = np.asarray(k_max, dtype=np.int32)
            K = int(k_h.max()) if k_h.size else 1
            kmax = torch.from_numpy(k_h).to(self.device)
        if alpha is None:
            alpha = torch.zeros((batch.n_runs, K), dtype=torch.float64, device=self.device)
            beta = torch.zeros((batch.n_runs, K), dtype=torch.float64, device=self.device)
        self.reset_status()
        L.check(self.lib.edgpu_lanczos_ragged(C.byref(batch.csr.struct()), C.byref(batch.struct()),
                                              _ptr(torch.view_as_real(v0)), _ptr(kmax), K, _ptr(alpha), _ptr(beta),
                                              _ptr(self.status), self.stream), "lanczos_ragged")
        if check:
            self.read_status("lanczos_ragged")
        return alpha, beta

    def lanczos_reorth_ragged(self, batch, v0, k_max):
        """Reorthogonalised Lanczos for every run of a RaggedBatch (one launch).

        Returns (V packed complex128, run_V0 host offsets, alpha, beta) with run r's basis
        ``V[run_V0[r] : run_V0[r] + k_max[r] * n_r]`` as [k_max[r], n_r]."""
        k_h = np.asarray(k_max, dtype=np.int32)
        K = int(k_h.max()) if k_h.size else 1
        sizes = batch.run_rows_h
        run_V0 = np.zeros(batch.n_runs + 1, dtype=np.int64)
        np.cumsum(k_h.astype(np.int64) * sizes, out=run_V0[1:])
        V = torch.empty(int(run_V0[-1]), dtype=torch.complex128, device=self.device)
        rv = torch.from_numpy(run_V0).to(self.device)
        kmax = torch.from_numpy(k_h).to(self.device)
        alpha = torch.zeros((batch.n_runs, K), dtype=torch.float64, device=self.device)
        beta = torch.zeros((batch.n_runs, K), dtype=torch.float64, device=self.device)
        self.reset_status()
        L.check(self.lib.edgpu_lanczos_reorth_ragged(C.byref(batch.csr.struct()), C.byref(batch.struct()),
                                                     _ptr(torch.view_as_real(v0)), _ptr(kmax), K, _ptr(rv),
                                                     _ptr(torch.view_as_real(V)), _ptr(alpha), _ptr(beta),
                                                     _ptr(self.status), self.stream), "lanczos_reorth_ragged")
        self.read_status("lanczos_reorth_ragged")
        return V, run_V0, alpha, beta

    def combine_ragged(self, batch, V, run_V0, k_len, S):
        """Ritz vectors X[r][q] = sum_k S[r, k, q] V_r[k]; returns packed [Q * sum n_r]."""
        S = np.ascontiguousarray(S, dtype=np.float64)
        R, K, Q = S.shape
        s_t = torch.from_numpy(S).to(self.device)
        rv = torch.from_numpy(np.asarray(run_V0, dtype=np.int64)).to(self.device)
        kl = torch.from_numpy(np.asarray(k_len, dtype=np.int32)).to(self.device)
        X = torch.empty(Q * int(batch.run_vec0_h[-1]), dtype=torch.complex128, device=self.device)
        L.check(self.lib.edgpu_combine_ragged(_ptr(torch.view_as_real(V)), C.byref(batch.struct()), _ptr(rv),
                                              _ptr(kl), _ptr(s_t), K, Q, _ptr(torch.view_as_real(X)), self.stream),
                "combine_ragged")
        return X

    def cfrac_device(self, alpha, beta, kl, om, delta, e, sc, g):
        """Continued fractions with every input already on the device (capturable)."""
        r, K = alpha.shape
        L.check(self.lib.edgpu_cfrac(_ptr(alpha), _ptr(beta), _ptr(kl), K, r, _ptr(om), om.numel(), float(delta),
                                     _ptr(e), _ptr(sc), _ptr(torch.view_as_real(g)), self.stream), "cfrac")
        return g


_ENGINES = {}


def get_engine(device=None):
    dev = torch.device(device if device is not None else "cuda")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    key = str(dev)
    if key not in _ENGINES:
        _ENGINES[key] = Engine(dev)
    return _ENGINES[key]


def words_for(n_spin_orbitals):
    w = n_words(n_spin_orbitals)
    if w > L.MAX_WORDS:
        raise ValueError("at most %d spin-orbitals are supported" % (64 * L.MAX_WORDS))
    return w


def sqrt_norm2(amps):
    return math.sqrt(float((amps[:, 0] ** 2 + amps[:, 1] ** 2).sum().item())) if amps.numel() else 0.0
