"""Host-side operator assembly and seeded synthetic Anderson-impurity models.

The engine consumes operators in the upstream dict format
``{((i, 'c'|'a'), ...): amplitude}`` unchanged.  This module builds such operators the
way upstream does (``impurityModel/ed/finite.py:476-728`` Slater-Condon/SOC/B-field
terms, ``finite.py:177-268`` double counting and cubic harmonics,
``impurityModel/ed/get_spectra.py:335-418`` assembly order and index remap,
``impurityModel/ed/get_spectra_using_CF.py:433-563`` crystal-field h0) without sympy:
Gaunt coefficients come from an exact rational Racah formula for Wigner 3j symbols.

It also defines the seeded synthetic models used for benchmarking and parity:

* ``config1``: 26 spin-orbitals (6 2p + 10 3d + 10 bath), one bath level per 3d
  spin-orbital, bath energies U(-3,-1), V U(1,2.5), seed 0.
* ``config2``: 66 spin-orbitals (5 bath levels per 3d spin-orbital), energies U(-5,0),
  V U(0.3,1.5), seed 1, at most 3 bath holes.
* ``config4``: 316 spin-orbitals (30 bath levels), energies U(-8,2), V U(0.1,0.8), seed 3,
  at most 2 bath holes.

Random draws use ``numpy.random.default_rng(seed)``: all bath energies first (level-major,
cubic orbital minor), then all hoppings in the same order; both spins share a draw.
"""

from __future__ import annotations

import functools
import math
from collections import OrderedDict
from fractions import Fraction

import numpy as np

K_B = 8.617333262e-05  # Boltzmann constant in eV/K (CODATA 2018, as scipy.constants)

# ----------------------------------------------------------------------------------------
# Angular-momentum algebra
# ----------------------------------------------------------------------------------------


@functools.lru_cache(maxsize=None)
def _racah_3j_parts(j1, j2, j3, m1, m2, m3):
    """Return (sign, A, S) with 3j = sign * sqrt(A) * S, A and S rational (integer j)."""
    if m1 + m2 + m3 != 0:
        return 0, Fraction(0), Fraction(0)
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return 0, Fraction(0), Fraction(0)
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0, Fraction(0), Fraction(0)
    f = math.factorial
    delta = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    a = delta * (f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3))
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        den = f(k) * f(j3 - j2 + k + m1) * f(j3 - j1 + k - m2) * f(j1 + j2 - j3 - k) * f(j1 - k - m1) * f(j2 - k + m2)
        s += Fraction((-1) ** k, den)
    sign = -1 if (j1 - j2 - m3) % 2 else 1
    return sign, a, s


def wigner3j(j1, j2, j3, m1, m2, m3):
    sign, a, s = _racah_3j_parts(j1, j2, j3, m1, m2, m3)
    if sign == 0 or s == 0:
        return 0.0
    return sign * math.sqrt(float(a)) * float(s)


@functools.lru_cache(maxsize=None)
def gaunt_c(k, l, m, lp, mp):
    r"""Coulomb-expansion Gaunt coefficient :math:`c^k(l m; l' m')`.

    Equals ``sqrt(4 pi/(2k+1)) (-1)^m gaunt(l, k, lp, -m, m-mp, mp)``
    (``impurityModel/ed/finite.py:476-488``), evaluated exactly as
    ``(-1)^m sqrt((2l+1)(2lp+1)) (l k lp; 0 0 0)(l k lp; -m, m-mp, mp)``.
    """
    s1, a1, r1 = _racah_3j_parts(l, k, lp, 0, 0, 0)
    s2, a2, r2 = _racah_3j_parts(l, k, lp, -m, m - mp, mp)
    if s1 == 0 or s2 == 0 or r1 == 0 or r2 == 0:
        return 0.0
    x = (2 * l + 1) * (2 * lp + 1) * a1 * a2 * (r1 * r2) ** 2
    sign = s1 * s2 * (1 if (r1 * r2) > 0 else -1) * (-1 if m % 2 else 1)
    return sign * math.sqrt(float(x))


def get_u(l1, m1, l2, m2, l3, m3, l4, m4, R):
    """Slater-Condon matrix element (``finite.py:491-543``)."""
    if m1 + m2 != m3 + m4:
        return 0
    u = 0
    for k, rk in enumerate(R):
        u += rk * gaunt_c(k, l1, m1, l4, m4) * gaunt_c(k, l3, m3, l2, m2)
    return u


def get_uop(l1, l2, l3, l4, R):
    """Spin-resolved two-body operator ``1/2 sum u c+ c+ c c`` (``finite.py:588-629``)."""
    out = {}
    for m1 in range(-l1, l1 + 1):
        for m2 in range(-l2, l2 + 1):
            for m3 in range(-l3, l3 + 1):
                for m4 in range(-l4, l4 + 1):
                    u = get_u(l1, m1, l2, m2, l3, m3, l4, m4, R)
                    if u != 0:
                        for s in range(2):
                            for sp in range(2):
                                proc = (
                                    ((l1, s, m1), "c"),
                                    ((l2, sp, m2), "c"),
                                    ((l3, sp, m3), "a"),
                                    ((l4, s, m4), "a"),
                                )
                                if not (s == sp and ((l1, m1) == (l2, m2) or (l3, m3) == (l4, m4))):
                                    out[proc] = u / 2.0
    return out


def add_ops(ops):
    """Sum operators, skipping zero amplitudes (``finite.py:632-651``)."""
    total = {}
    for op in ops:
        for key, value in op.items():
            if value != 0:
                if key in total:
                    total[key] += value
                else:
                    total[key] = value
    return total


def slater_condon_2p3d_uop(Fdd=(9, 0, 8, 0, 6), Fpp=(20, 0, 8), Fpd=(10, 0, 8), Gpd=(0, 3, 0, 2)):
    """2p-3d Coulomb operator (``finite.py:654-681``)."""
    fdd = get_uop(2, 2, 2, 2, Fdd)
    fpp = get_uop(1, 1, 1, 1, Fpp)
    fpd = add_ops([get_uop(1, 2, 2, 1, Fpd), get_uop(2, 1, 1, 2, Fpd)])
    gpd = add_ops([get_uop(1, 2, 1, 2, Gpd), get_uop(2, 1, 2, 1, Gpd)])
    return add_ops([fdd, fpp, fpd, gpd])


def soc_op(xi, l=2):
    """Spin-orbit operator of one shell (``finite.py:684-705``)."""
    op = {}
    for m in range(-l, l + 1):
        for s in range(2):
            op[(((l, s, m), "c"), ((l, s, m), "a"))] = xi * m * (1 / 2.0 if s == 1 else -1 / 2.0)
    for m in range(-l, l):
        value = xi / 2.0 * math.sqrt((l - m) * (l + m + 1))
        op[(((l, 1, m), "c"), ((l, 0, m + 1), "a"))] = value
        op[(((l, 0, m + 1), "c"), ((l, 1, m), "a"))] = value
    return op


def hfield_op(hx, hy, hz, l=2):
    """Zeeman operator of one shell (``finite.py:708-728``)."""
    op = {}
    for m in range(-l, l + 1):
        op[(((l, 1, m), "c"), ((l, 0, m), "a"))] = hx / 2
        op[(((l, 0, m), "c"), ((l, 1, m), "a"))] = hx / 2
        op[(((l, 1, m), "c"), ((l, 0, m), "a"))] += -hy * 1j / 2
        op[(((l, 0, m), "c"), ((l, 1, m), "a"))] += hy * 1j / 2
        for s in range(2):
            op[(((l, s, m), "c"), ((l, s, m), "a"))] = hz / 2 if s == 1 else -hz / 2
    return op


def dc_mlft(n3d_i, c, Fdd, n2p_i=None, Fpd=None, Gpd=None):
    """MLFT double counting (``finite.py:177-213``)."""
    udd = Fdd[0] - 14.0 / 441 * (Fdd[2] + Fdd[4])
    if n2p_i is None and Fpd is None and Gpd is None:
        return udd * n3d_i - c
    upd = Fpd[0] - (1 / 15.0) * Gpd[1] - (3 / 70.0) * Gpd[3]
    return [udd * n3d_i + upd * n2p_i - c, upd * (n3d_i + 1) - c]


def spherical_to_cubic(l=2):
    """Unitary spherical -> cubic harmonics matrix (``finite.py:216-268``), no spin."""
    if l == 1:
        u = np.zeros((3, 3), dtype=complex)
        u[0, 0] = 1j / np.sqrt(2)
        u[2, 0] = 1j / np.sqrt(2)
        u[0, 1] = 1 / np.sqrt(2)
        u[2, 1] = -1 / np.sqrt(2)
        u[1, 2] = 1
        return u
    u = np.zeros((5, 5), dtype=complex)
    u[2, 0] = 1
    u[[0, -1], 1] = 1 / np.sqrt(2)
    u[1, 2] = -1j / np.sqrt(2)
    u[-2, 2] = -1j / np.sqrt(2)
    u[1, 3] = 1 / np.sqrt(2)
    u[-2, 3] = -1 / np.sqrt(2)
    u[0, 4] = 1j / np.sqrt(2)
    u[-1, 4] = -1j / np.sqrt(2)
    return u


def c2i(nBaths, spin_orb):
    """Spin-orbital tuple -> index: impurity (l, s, m) first, then baths (``finite.py:731-782``)."""
    i = 0
    for lp in nBaths.keys():
        for sp in range(2):
            for mp in range(-lp, lp + 1):
                if (lp, sp, mp) == spin_orb:
                    return i
                i += 1
    for lp, nb in nBaths.items():
        for b in range(nb):
            if (lp, b) == spin_orb:
                return i
            i += 1
    raise KeyError("no index for spin-orbital %r" % (spin_orb,))


def n_spin_orbitals_of(nBaths):
    return sum(2 * (2 * ang + 1) + nb for ang, nb in nBaths.items())


def dagger_op(op):
    """Hermitian conjugate of an operator (``finite.py:271-287``)."""
    out = {}
    for process, value in op.items():
        new = []
        for orb, act in process[::-1]:
            if act == "a":
                new.append((orb, "c"))
            elif act == "c":
                new.append((orb, "a"))
            else:
                raise ValueError("Operator type unknown: {}".format(act))
        out[tuple(new)] = value.conjugate()
    return out


# ----------------------------------------------------------------------------------------
# Hamiltonian assembly
# ----------------------------------------------------------------------------------------


def _hermitian_clean(m, tiny=1e-14):
    """Exactly Hermitian copy of ``m`` with rounding noise below ``tiny`` set to zero."""
    m = (m + m.conj().T) / 2
    re = np.where(np.abs(m.real) < tiny, 0.0, m.real)
    im = np.where(np.abs(m.imag) < tiny, 0.0, m.imag)
    return re + 1j * im


def _clean(m, tiny=1e-14):
    re = np.where(np.abs(m.real) < tiny, 0.0, m.real)
    im = np.where(np.abs(m.imag) < tiny, 0.0, m.imag)
    return re + 1j * im


def crystal_field_h0(n_levels, e_bath, v_bath, ten_dq, e_imp=0.0):
    """Non-interacting 3d + bath operator in spherical-harmonic labels.

    ``e_bath[b, c]``/``v_bath[b, c]``: energy / hopping of bath level ``b`` coupled to
    cubic orbital ``c`` (z2, x2-y2, yz, xz, xy), diagonal in cubic harmonics and shared by
    both spins.  Bath spin-orbital ``(2, b*10 + s*5 + i)`` carries spherical label ``i``,
    following ``get_spectra_using_CF.py:481-548`` with a spherical bath basis.
    """
    l = 2
    u = spherical_to_cubic(l)
    h_imp = np.diag([e_imp + 0.6 * ten_dq] * 2 + [e_imp - 0.4 * ten_dq] * 3).astype(complex)
    h_imp = _hermitian_clean(u @ h_imp @ u.conj().T)
    op = {}
    for i, mi in enumerate(range(-l, l + 1)):
        for j, mj in enumerate(range(-l, l + 1)):
            if h_imp[i, j] != 0:
                for s in range(2):
                    op[(((l, s, mi), "c"), ((l, s, mj), "a"))] = complex(h_imp[i, j])
    hopp = {}
    ebath = {}
    for b in range(n_levels):
        vmat = _clean(u @ np.diag(v_bath[b]).astype(complex) @ u.conj().T)
        emat = _hermitian_clean(u @ np.diag(e_bath[b]).astype(complex) @ u.conj().T)
        for s in range(2):
            for i in range(2 * l + 1):
                bi = b * 10 + s * (2 * l + 1) + i
                for j, mj in enumerate(range(-l, l + 1)):
                    bj = b * 10 + s * (2 * l + 1) + j
                    vh = vmat[i, j]
                    eb = emat[i, j]
                    if vh != 0:
                        hopp[(((l, bi), "c"), ((l, s, mj), "a"))] = complex(vh)
                        hopp[(((l, s, mj), "c"), ((l, bi), "a"))] = complex(np.conj(vh))
                    if eb != 0:
                        ebath[(((l, bi), "c"), ((l, bj), "a"))] = complex(eb)
    return add_ops([op, hopp, ebath])


def assemble_hamiltonian(nBaths, slater, socs, n0imps, charge_transfer_correction, hfield, h0_operator):
    """Full impurity Hamiltonian in index notation (``get_spectra.py:335-418``)."""
    Fdd, Fpp, Fpd, Gpd = slater
    xi_2p, xi_3d = socs
    hx, hy, hz = hfield
    u_op = slater_condon_2p3d_uop(Fdd=Fdd, Fpp=Fpp, Fpd=Fpd, Gpd=Gpd)
    soc2p = soc_op(xi_2p, l=1)
    soc3d = soc_op(xi_3d, l=2)
    dc = dc_mlft(n3d_i=n0imps[2], c=charge_transfer_correction, Fdd=Fdd, n2p_i=n0imps[1], Fpd=Fpd, Gpd=Gpd)
    e_dc = {}
    for il, l in enumerate([2, 1]):
        for s in range(2):
            for m in range(-l, l + 1):
                e_dc[(((l, s, m), "c"), ((l, s, m), "a"))] = -dc[il]
    hf = hfield_op(hx, hy, hz, l=2)
    total = add_ops([u_op, hf, soc2p, soc3d, e_dc, h0_operator])
    hop = {}
    for process, value in total.items():
        hop[tuple((c2i(nBaths, so), act) for so, act in process)] = value
    return hop


def get_restrictions(nBaths, nValBaths, n0imps, dnTols, dnValBaths, dnConBaths, core_holes=None):
    """Occupation restrictions of ``get_spectra.py:155-169``.

    With ``core_holes`` set, the 2p shell is additionally limited to at most that many holes.
    """
    l = 2
    r = {}
    idx = frozenset(c2i(nBaths, (l, s, m)) for s in range(2) for m in range(-l, l + 1))
    r[idx] = (n0imps[l] - 1, n0imps[l] + dnTols[l] + 1)
    r[frozenset(c2i(nBaths, (l, b)) for b in range(nValBaths[l]))] = (nValBaths[l] - dnValBaths[l], nValBaths[l])
    r[frozenset(c2i(nBaths, (l, b)) for b in range(nValBaths[l], nBaths[l]))] = (0, dnConBaths[l])
    if core_holes is not None:
        idx = frozenset(c2i(nBaths, (1, s, m)) for s in range(2) for m in range(-1, 2))
        r[idx] = (6 - core_holes, 6)
    return r


# ----------------------------------------------------------------------------------------
# Transition operators (``impurityModel/ed/spectra.py:302-548``)
# ----------------------------------------------------------------------------------------


def dipole_op(nBaths, n):
    """2p -> 3d dipole operator for polarisation ``n`` (``spectra.py:341-382``)."""
    op = {}
    nd = {-1: (n[0] + 1j * n[1]) / math.sqrt(2), 0: n[2], 1: (-n[0] + 1j * n[1]) / math.sqrt(2)}
    l1, l2 = nBaths.keys()
    for m in range(-l2, l2 + 1):
        for mp in range(-l1, l1 + 1):
            for s in range(2):
                if abs(m - mp) <= 1:
                    tij = gaunt_c(1, l2, m, l1, mp)
                    tij *= nd[m - mp]
                    if tij != 0:
                        op[((c2i(nBaths, (l2, s, m)), "c"), (c2i(nBaths, (l1, s, mp)), "a"))] = tij
    return op


def dipole_ops(nBaths, ns):
    return [dipole_op(nBaths, n) for n in ns]


def daggered_dipole_ops(nBaths, ns):
    return [dagger_op(dipole_op(nBaths, n)) for n in ns]


def photoemission_ops(nBaths, l=2):
    """``{c_i}`` over the shell (``spectra.py:530-548``)."""
    return [{((c2i(nBaths, (l, s, m)), "a"),): 1} for s in range(2) for m in range(-l, l + 1)]


def inverse_photoemission_ops(nBaths, l=2):
    """``{c_i^dagger}`` over the shell (``spectra.py:511-527``)."""
    return [{((c2i(nBaths, (l, s, m)), "c"),): 1} for s in range(2) for m in range(-l, l + 1)]


def _assoc_legendre(l, m, x):
    """P_l^m(x), m >= 0, with the Condon-Shortley phase."""
    pmm = 1.0
    if m > 0:
        somx2 = math.sqrt((1.0 - x) * (1.0 + x))
        fact = 1.0
        for _ in range(m):
            pmm *= -fact * somx2
            fact += 2.0
    if l == m:
        return pmm
    pmmp1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmmp1
    pll = 0.0
    for ll in range(m + 2, l + 1):
        pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pmmp1 = pmmp1, pll
    return pll


def sph_harm_y(l, m, theta, phi):
    """Y_l^m(theta polar, phi azimuth) with the Condon-Shortley phase."""
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    y = norm * _assoc_legendre(l, am, math.cos(theta)) * complex(math.cos(am * phi), math.sin(am * phi))
    if m < 0:
        y = (-1) ** am * y.conjugate()
    return y


def hydrogenic_3d_radial(z_eff=8.0, n_points=3000, r_max=6.0):
    """Radial mesh and a normalised hydrogen-like 3d radial function R(r) ~ r^2 exp(-Z r/3)."""
    r = np.linspace(1e-5, r_max, n_points)
    R = r**2 * np.exp(-z_eff * r / 3.0)
    R /= math.sqrt(np.trapezoid(R**2 * r**2, r))
    return r, R


def nixs_op(nBaths, q, li, lj, Ri, Rj, r, kmin=1):
    """NIXS operator ``<i|exp(iq.r)|j>`` in multipoles (``spectra.py:437-508``)."""
    from scipy.special import spherical_jn

    q = np.array(q, dtype=float)
    qn = np.linalg.norm(q)
    theta = np.arccos(q[2] / qn)
    phi = np.arccos(q[0] / (qn * np.sin(theta)))
    op = {}
    for k in range(kmin, abs(li + lj) + 1):
        if (li + lj + k) % 2 == 0:
            rint = np.trapezoid(np.conj(Ri) * spherical_jn(k, qn * r) * Rj * r**2, r)
            for mi in range(-li, li + 1):
                for mj in range(-lj, lj + 1):
                    m = mi - mj
                    if abs(m) <= k:
                        tij = rint
                        tij *= 1j**k * math.sqrt(2 * k + 1)
                        tij *= np.conj(sph_harm_y(k, m, theta, phi))
                        tij *= gaunt_c(k, li, mi, lj, mj)
                        if tij != 0:
                            for s in range(2):
                                key = ((c2i(nBaths, (li, s, mi)), "c"), (c2i(nBaths, (lj, s, mj)), "a"))
                                op[key] = op.get(key, 0) + complex(tij)
    return op


# ----------------------------------------------------------------------------------------
# Seeded synthetic models
# ----------------------------------------------------------------------------------------

CONFIGS = {
    "config1": dict(levels=1, e_range=(-3.0, -1.0), v_range=(1.0, 2.5), seed=0, bath_holes=2),
    "config2": dict(levels=5, e_range=(-5.0, 0.0), v_range=(0.3, 1.5), seed=1, bath_holes=3),
    "config4": dict(levels=30, e_range=(-8.0, 2.0), v_range=(0.1, 0.8), seed=3, bath_holes=2),
}

SLATER = dict(Fdd=(8.0, 0.0, 10.0, 0.0, 6.5), Fpp=(0.0, 0.0, 0.0), Fpd=(8.5, 0.0, 6.0), Gpd=(0.0, 4.5, 0.0, 2.5))


class Model:
    """A seeded Anderson-impurity model: operator, basis parameters, restrictions."""

    def __init__(self, levels, e_range, v_range, seed, bath_holes, ten_dq=0.6, xi_2p=11.5, xi_3d=0.08,
                 charge_transfer_correction=1.5, hfield=(0.0, 0.0, 1e-4), name=None, dn_tol=2):
        rng = np.random.default_rng(seed)
        e_bath = rng.uniform(e_range[0], e_range[1], size=(levels, 5))
        v_bath = rng.uniform(v_range[0], v_range[1], size=(levels, 5))
        self.name = name or "model_seed%d_%dbath" % (seed, 10 * levels)
        self.seed = seed
        self.levels = levels
        self.e_bath = e_bath
        self.v_bath = v_bath
        nb = 10 * levels
        self.nBaths = OrderedDict([(1, 0), (2, nb)])
        self.nValBaths = OrderedDict([(1, 0), (2, nb)])
        self.n0imps = OrderedDict([(1, 6), (2, 8)])
        self.dnTols = OrderedDict([(1, 0), (2, dn_tol)])
        self.dnValBaths = OrderedDict([(1, 0), (2, bath_holes)])
        self.dnConBaths = OrderedDict([(1, 0), (2, 0)])
        self.n_spin_orbitals = n_spin_orbitals_of(self.nBaths)
        h0 = crystal_field_h0(levels, e_bath, v_bath, ten_dq)
        self.hOp = assemble_hamiltonian(
            self.nBaths,
            (SLATER["Fdd"], SLATER["Fpp"], SLATER["Fpd"], SLATER["Gpd"]),
            (xi_2p, xi_3d),
            self.n0imps,
            charge_transfer_correction,
            hfield,
            h0,
        )
        self.restrictions = get_restrictions(
            self.nBaths, self.nValBaths, self.n0imps, self.dnTols, self.dnValBaths, self.dnConBaths, core_holes=1
        )

    def basis_args(self):
        return (self.nBaths, self.nValBaths, self.dnValBaths, self.dnConBaths, self.dnTols, self.n0imps)

    def xas_ops(self, eps=((1, 0, 0), (0, 1, 0), (0, 0, 1))):
        return dipole_ops(self.nBaths, eps)

    def rixs_out_ops(self, eps=((1, 0, 0), (0, 1, 0), (0, 0, 1))):
        return daggered_dipole_ops(self.nBaths, eps)

    def ps_ops(self, l=2):
        return photoemission_ops(self.nBaths, l=l)

    def ips_ops(self, l=2):
        return inverse_photoemission_ops(self.nBaths, l=l)

    def nixs_ops(self, qs=None):
        if qs is None:
            qs = [1.0 * np.array([1, 1, 1]) / np.sqrt(3), 2.0 * np.array([1, 1, 1]) / np.sqrt(3)]
        r, R = hydrogenic_3d_radial()
        return [nixs_op(self.nBaths, q, 2, 2, R, R, r) for q in qs]


def make_model(config="config1", **overrides):
    params = dict(CONFIGS[config])
    params.update(overrides)
    return Model(name=config, **params)


def random_model(seed, n_bath_levels, e_range=(-5.0, 0.0), v_range=(0.3, 1.5), bath_holes=2):
    """Ensemble member: ``n_bath_levels`` bath levels per 3d spin-orbital."""
    return Model(n_bath_levels, e_range, v_range, seed, bath_holes, name="ens_seed%d" % seed)
