"""3d-shell observables of many-body states on the device (upstream finite.py:843-1298).

Upstream evaluates every observable by dict loops over the states of ``psi``: the density
matrix by one ``a(i)``, ``c(j)`` and inner product per (i, j) pair (finite.py:967-1012), the
occupations by bit scans (finite.py:843-964, 1063-1112) and <L^2>, <S^2> by norms of ladder-
and z-operators applied to ``psi`` (finite.py:895-934, 1115-1298).  Here the whole spherical
3d density matrix ``n[a][b] = <psi| c_b^dagger c_a |psi>`` (a, b = spin * 5 + m + 2) of every
state comes from one kernel launch (``edgpu_density_matrix``); N(3d), Lz, Sz, the cubic
density matrix and the eg/t2g occupations are linear functions of it, and <L^2>, <S^2> are
norms of the one-body operators applied to all states at once by the operator kernel.

The upstream-named functions take ``nBaths`` and dict states like upstream and return the
same types (OrderedDicts in upstream's key order, floats, lists).
"""

from __future__ import annotations

from collections import OrderedDict
from math import sqrt

import numpy as np
import torch

from . import _lib as L
from . import codec
from .engine import DeviceOp, _ptr, get_engine, words_for
from .models import K_B, c2i, spherical_to_cubic


def _n_spin_orbitals(nBaths):
    return sum(2 * (2 * l + 1) + nb for l, nb in nBaths.items())


def _shell(nBaths, l=2):
    return [c2i(nBaths, (l, s, m)) for s in range(2) for m in range(-l, l + 1)]


def _pack(create, annihilate):
    return (0x8000 | 0x4000 | int(create)) | ((0x8000 | int(annihilate)) << 16)


def one_body_op(nBaths, kind):
    """Operator dict of upstream's applySz3d / applyLz3d / applySplus3d / applyLplus3d /
    applySminus3d / applyLminus3d (finite.py:1115-1298), terms in upstream's loop order."""
    c = lambda s, m: c2i(nBaths, (2, s, m))  # noqa: E731
    op = OrderedDict()
    if kind in ("Sz", "Lz"):
        for s in range(2):
            for m in range(-2, 3):
                op[((c(s, m), "c"), (c(s, m), "a"))] = (0.5 if s == 1 else -0.5) if kind == "Sz" else float(m)
    elif kind == "S+":
        for m in range(-2, 3):
            op[((c(1, m), "c"), (c(0, m), "a"))] = 1.0
    elif kind == "S-":
        for m in range(-2, 3):
            op[((c(0, m), "c"), (c(1, m), "a"))] = 1.0
    elif kind == "L+":
        for s in range(2):
            for m in range(-2, 2):
                op[((c(s, m + 1), "c"), (c(s, m), "a"))] = sqrt((2 - m) * (2 + m + 1))
    elif kind == "L-":
        for s in range(2):
            for m in range(-1, 3):
                op[((c(s, m - 1), "c"), (c(s, m), "a"))] = sqrt((2 + m) * (2 - m + 1))
    else:
        raise ValueError("unknown one-body operator %r" % (kind,))
    return op


def density_matrices(eng, psi_t, nBaths, l=2):
    """Spherical l-shell density matrices of device states ``psi_t`` (list of (states [m, W]
    int64, amps [m, 2] float64)): D[r, a, b] = <psi_r| c_b^dagger c_a |psi_r>, a and b
    running over (spin, m) as spin * (2l + 1) + m + l.  One launch for all states."""
    orbs = _shell(nBaths, l)
    k = len(orbs)
    R = len(psi_t)
    if R == 0:
        return torch.zeros((0, k, k), dtype=torch.complex128, device=eng.device)
    ops = np.array([_pack(orbs[b], orbs[a]) for a in range(k) for b in range(k)], dtype=np.uint64)
    words, amps, sizes = [], [], []
    for st, am in psi_t:
        keys = st.clone().contiguous()
        payload = torch.arange(keys.shape[0], dtype=torch.int32, device=eng.device)
        if keys.shape[0]:
            eng.sort_states(keys, payload)
        words.append(keys)
        amps.append(am[payload.to(torch.int64)])
        sizes.append(keys.shape[0])
    W = words[0].shape[1]
    st_all = torch.cat(words).contiguous()
    am_all = torch.cat(amps).contiguous()
    off = np.zeros(R + 1, dtype=np.int64)
    np.cumsum(sizes, out=off[1:])
    off_t = torch.from_numpy(off).to(eng.device)
    ops_t = torch.from_numpy(ops.view(np.int64)).to(eng.device)
    out = torch.empty((R, k * k), dtype=torch.complex128, device=eng.device)
    L.check(eng.lib.edgpu_density_matrix(W, _ptr(st_all), _ptr(am_all), _ptr(off_t), R, _ptr(ops_t), k * k,
                                         _ptr(torch.view_as_real(out)), eng.stream), "density_matrix")
    return out.view(R, k, k)


def _ladder_norms(eng, psi_t, nBaths, restr=None):
    """|X psi_r|^2 for X in Lz, L+, L-, Sz, S+, S- (upstream norm2(applyX3d(psi)))."""
    n = _n_spin_orbitals(nBaths)
    out = {}
    for kind in ("Lz", "L+", "L-", "Sz", "S+", "S-"):
        dop = DeviceOp(one_body_op(nBaths, kind), eng.device)
        res = eng.apply_vectors([p[0] for p in psi_t], [p[1] for p in psi_t], dop, restr, 0.0)
        out[kind] = np.array([float((a ** 2).sum().item()) if a.numel() else 0.0 for _, a in res])
    del n
    return out


def expectation_values(eng, psi_t, nBaths):
    """Per-state arrays of upstream's printed observables (finite.py:121-148): N(3d),
    N(eg_dn), N(eg_up), N(t2g_dn), N(t2g_up), Lz, Sz, L^2, S^2, plus the spherical and cubic
    density matrices."""
    D = density_matrices(eng, psi_t, nBaths).cpu().numpy()
    u = spherical_to_cubic(2)
    R = D.shape[0]
    m_of = np.tile(np.arange(-2, 3), 2)
    s_of = np.repeat([-0.5, 0.5], 5)
    res = {"n3d": np.real(np.einsum("raa->r", D)), "lz": np.real(np.einsum("raa,a->r", D, m_of)),
           "sz": np.real(np.einsum("raa,a->r", D, s_of)), "dm": D}
    # cubic blocks per spin: n_cub[(si,i),(sj,j)] = sum_{m,k} conj(u[m,i]) n[(si,m),(sj,k)] u[k,j]
    U = np.zeros((10, 10), dtype=complex)
    U[:5, :5] = u
    U[5:, 5:] = u
    res["dm_cubic"] = np.einsum("mi,rmk,kj->rij", np.conj(U), D, U)
    occ = np.zeros((R, 4))
    for s in range(2):
        blk = D[:, s * 5:(s + 1) * 5, s * 5:(s + 1) * 5]
        # <c_{ic,s}^dagger c_{ic,s}> = sum_{j,k} u[j,ic] conj(u[k,ic]) <c_j^dagger c_k>, and
        # <c_j^dagger c_k> = D[k][j]
        diag = np.real(np.einsum("ji,ki,rkj->ri", u, np.conj(u), blk))
        occ[:, s] = diag[:, :2].sum(1)
        occ[:, 2 + s] = diag[:, 2:].sum(1)
    res["eg_dn"], res["eg_up"], res["t2g_dn"], res["t2g_up"] = occ.T
    nrm = _ladder_norms(eng, psi_t, nBaths)
    res["l2"] = nrm["Lz"] + 0.5 * (nrm["L+"] + nrm["L-"])
    res["s2"] = nrm["Sz"] + 0.5 * (nrm["S+"] + nrm["S-"])
    return res


# ---------------------------------------------------------------------------------------
# Upstream API (dict states)
# ---------------------------------------------------------------------------------------


def _dev(psi, nBaths):
    eng = get_engine()
    n = _n_spin_orbitals(nBaths)
    words_for(n)
    words, amps = codec.psi_to_arrays(psi, n)
    return eng, [(eng.upload_states(words), eng.to_device(amps))]


def getDensityMatrix(nBaths, psi, l=2):
    """Density matrix in spherical harmonics (upstream finite.py:967-1012): keys
    ((l,si,mi),(l,sj,mj)), values <psi| c_j^dagger c_i |psi>, nonzero entries only."""
    eng, pt = _dev(psi, nBaths)
    D = density_matrices(eng, pt, nBaths, l).cpu().numpy()[0]
    k = 2 * l + 1
    out = OrderedDict()
    for si in range(2):
        for sj in range(2):
            for mi in range(-l, l + 1):
                for mj in range(-l, l + 1):
                    v = complex(D[si * k + mi + l, sj * k + mj + l])
                    if v != 0:
                        out[((l, si, mi), (l, sj, mj))] = v
    return out


def getDensityMatrixCubic(nBaths, psi):
    """Density matrix in cubic harmonics (upstream finite.py:1015-1060), keys ((si,i),(sj,j))
    in upstream's insertion order."""
    nsph = getDensityMatrix(nBaths, psi)
    u = spherical_to_cubic(2)
    out = OrderedDict()
    for i in range(5):
        for j in range(5):
            for si in range(2):
                for sj in range(2):
                    for k, mk in enumerate(range(-2, 3)):
                        for m, mm in enumerate(range(-2, 3)):
                            e = ((2, si, mm), (2, sj, mk))
                            if e in nsph:
                                t = np.conj(u[m, i]) * nsph[e] * u[k, j]
                                if t != 0:
                                    key = ((si, i), (sj, j))
                                    out[key] = out[key] + t if key in out else t
    return out


def getEgT2gOccupation(nBaths, psi):
    """[eg_dn, eg_up, t2g_dn, t2g_up] occupations (upstream finite.py:1063-1112)."""
    eng, pt = _dev(psi, nBaths)
    r = expectation_values(eng, pt, nBaths)
    return [float(r[k][0]) for k in ("eg_dn", "eg_up", "t2g_dn", "t2g_up")]


def getTraceDensityMatrix(nBaths, psi, l=2):
    """<psi| sum_i c_i^dagger c_i |psi> over the l shell (upstream finite.py:937-964)."""
    eng, pt = _dev(psi, nBaths)
    return float(np.real(np.trace(density_matrices(eng, pt, nBaths, l).cpu().numpy()[0])))


def getLz3d(nBaths, psi):
    """<Lz> of the 3d shell (upstream finite.py:843-866)."""
    eng, pt = _dev(psi, nBaths)
    return float(expectation_values(eng, pt, nBaths)["lz"][0])


def getSz3d(nBaths, psi):
    """<Sz> of the 3d shell (upstream finite.py:869-892)."""
    eng, pt = _dev(psi, nBaths)
    return float(expectation_values(eng, pt, nBaths)["sz"][0])


def getLsqr3d(nBaths, psi, tol=1e-8):
    """<L^2> of the 3d shell (upstream finite.py:916-934)."""
    eng, pt = _dev(psi, nBaths)
    return float(expectation_values(eng, pt, nBaths)["l2"][0])


def getSsqr3d(nBaths, psi, tol=1e-8):
    """<S^2> of the 3d shell (upstream finite.py:895-913)."""
    eng, pt = _dev(psi, nBaths)
    return float(expectation_values(eng, pt, nBaths)["s2"][0])


def _apply(nBaths, psi, kind):
    from .finite import applyOp

    return applyOp(_n_spin_orbitals(nBaths), one_body_op(nBaths, kind), psi, slaterWeightMin=0.0)


def applySz3d(nBaths, psi):
    """S^z_3d |psi> (upstream finite.py:1115-1142)."""
    return _apply(nBaths, psi, "Sz")


def applyLz3d(nBaths, psi):
    """L^z_3d |psi> (upstream finite.py:1145-1172)."""
    return _apply(nBaths, psi, "Lz")


def applySplus3d(nBaths, psi):
    """S^+_3d |psi> (upstream finite.py:1175-1204)."""
    return _apply(nBaths, psi, "S+")


def applyLplus3d(nBaths, psi):
    """L^+_3d |psi> (upstream finite.py:1207-1235)."""
    return _apply(nBaths, psi, "L+")


def applySminus3d(nBaths, psi):
    """S^-_3d |psi> (upstream finite.py:1238-1267)."""
    return _apply(nBaths, psi, "S-")


def applyLminus3d(nBaths, psi):
    """L^-_3d |psi> (upstream finite.py:1270-1298)."""
    return _apply(nBaths, psi, "L-")


def _table(nBaths, psis):
    eng = get_engine()
    n = _n_spin_orbitals(nBaths)
    words_for(n)
    pt = []
    for psi in psis:
        words, amps = codec.psi_to_arrays(psi, n)
        pt.append((eng.upload_states(words), eng.to_device(amps)))
    return expectation_values(eng, pt, nBaths)


def printExpValues(nBaths, es, psis, n=None):
    """Print E, N(3d), eg/t2g occupations, Lz, Sz, L^2, S^2 per state (upstream finite.py:121-148)."""
    if n is None:
        n = len(es)
    es = np.asarray(es)
    r = _table(nBaths, list(psis[:n]))
    print("E0 = {:7.4f}".format(es[0]))
    print(("  i  E-E0  N(3d) N(egDn) N(egUp) N(t2gDn) " "N(t2gUp) Lz(3d) Sz(3d) L^2(3d) S^2(3d)"))
    for i, e in enumerate(es[:n] - es[0]):
        print(("{:3d} {:6.3f} {:5.2f} {:6.3f} {:7.3f} {:8.3f} {:7.3f}" " {:7.2f} {:6.2f} {:7.2f} {:7.2f}").format(
            i, e, r["n3d"][i], r["eg_dn"][i], r["eg_up"][i], r["t2g_dn"][i], r["t2g_up"][i], r["lz"][i], r["sz"][i],
            r["l2"][i], r["s2"][i]))
    print("\n")


def thermal_expectation_values(nBaths, es, psis, T=300, cutOff=10):
    """Boltzmann averages over the states within cutOff * k_B * T of the lowest (the values
    upstream's printThermalExpValues prints, finite.py:151-174)."""
    from .spectra import thermal_average

    e = np.asarray(es) - es[0]
    mask = e < cutOff * K_B * T
    e = e[mask]
    r = _table(nBaths, [p for p, k in zip(psis, mask) if k])
    keys = ("n3d", "eg_dn", "eg_up", "t2g_dn", "t2g_up", "lz", "sz", "l2", "s2")
    out = {"e": thermal_average(e, e, T=T)}
    out.update({k: thermal_average(e, r[k], T=T) for k in keys})
    return out


def printThermalExpValues(nBaths, es, psis, T=300, cutOff=10):
    """Print thermal averages of E - E0 and the 3d observables (upstream finite.py:151-174)."""
    t = thermal_expectation_values(nBaths, es, psis, T, cutOff)
    print("<E-E0> = {:4.3f}".format(t["e"]))
    for label, k in (("N(3d)", "n3d"), ("N(egDn)", "eg_dn"), ("N(egUp)", "eg_up"), ("N(t2gDn)", "t2g_dn"),
                     ("N(t2gUp)", "t2g_up"), ("Lz(3d)", "lz"), ("Sz(3d)", "sz"), ("L^2(3d)", "l2"),
                     ("S^2(3d)", "s2")):
        print("<{}> = {:4.3f}".format(label, t[k]))
