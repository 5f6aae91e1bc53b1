"""Spectroscopy driver with upstream's command line (impurityModel/ed/get_spectra.py).

``python -m impuritymodel_gb300.get_spectra h0.pickle radial.dat [flags]`` takes the flags and
defaults of upstream's ``python -m impurityModel.ed.get_spectra`` (get_spectra.py:427-618),
builds the same Hamiltonian operator (get_spectra.py:335-418), finds the lowest eigenstates,
prints the same expectation values and writes the same files into the working directory:
``data.npz``, the datasets of ``spectra.h5`` (``spectra.npz`` when h5py is not installed) and
PS.dat, XPS.dat, NIXS.dat, XAS.dat, RIXS.bin.  MPI is not used: one process drives one GPU.

The h0 pickle is read with a restricted unpickler (containers, complex numbers and NumPy
scalars only), not with ``pickle.load``.
"""

from __future__ import annotations

import argparse
import os
import pickle
import time
from collections import OrderedDict

import numpy as np

from . import finite, spectra
from .models import K_B as k_B
from .models import assemble_hamiltonian, c2i


class _SafeUnpickler(pickle.Unpickler):
    """Only dicts, tuples, lists, sets, complex numbers and NumPy scalars/arrays."""

    _ALLOWED = {("collections", "OrderedDict"), ("builtins", "complex"), ("builtins", "frozenset"),
                ("builtins", "set"), ("builtins", "dict"), ("builtins", "tuple"), ("builtins", "list")}

    def find_class(self, module, name):
        if (module, name) in self._ALLOWED:
            import builtins
            import collections

            return getattr(collections if module == "collections" else builtins, name)
        if module in ("numpy.core.multiarray", "numpy._core.multiarray") and name in ("scalar", "_reconstruct"):
            try:
                from numpy._core import multiarray
            except ImportError:  # older NumPy
                from numpy.core import multiarray
            return getattr(multiarray, name)
        if module == "numpy" and name in ("dtype", "ndarray"):
            return getattr(np, name)
        raise pickle.UnpicklingError("refusing to load %s.%s from the h0 file" % (module, name))


def read_pickled_file(filename):
    """The operator dict of an h0 pickle (upstream get_spectra.py:421-424), restricted load."""
    with open(filename, "rb") as handle:
        return _SafeUnpickler(handle).load()


def get_hamiltonian_operator(nBaths, nValBaths, slaterCondon, SOCs, DCinfo, hField, h0_filename):
    """Hamiltonian in index notation (upstream get_spectra.py:335-418): Slater-Condon U,
    Zeeman field, 2p and 3d spin-orbit coupling, MLFT double counting and the h0 read from
    file, added in upstream's order and mapped to spin-orbital indices; checked Hermitian."""
    n0imps, charge_transfer_correction = DCinfo
    h0 = read_pickled_file(h0_filename)
    hOp = assemble_hamiltonian(nBaths, slaterCondon, SOCs, n0imps, charge_transfer_correction, hField, h0)
    finite.assert_hermitian(hOp)
    return hOp


def _restrictions(nBaths, nValBaths, n0imps, dnTols, dnValBaths, dnConBaths, l=2):
    """Occupation restrictions of the spectra (upstream get_spectra.py:158-170)."""
    restrictions = {}
    idx = frozenset(c2i(nBaths, (l, s, m)) for s in range(2) for m in range(-l, l + 1))
    restrictions[idx] = (n0imps[l] - 1, n0imps[l] + dnTols[l] + 1)
    idx = [c2i(nBaths, (l, b)) for b in range(nValBaths[l])]
    restrictions[frozenset(idx)] = (nValBaths[l] - dnValBaths[l], nValBaths[l])
    idx = [c2i(nBaths, (l, b)) for b in range(nValBaths[l], nBaths[l])]
    restrictions[frozenset(idx)] = (0, dnConBaths[l])
    return restrictions


def _open_store():
    try:
        import h5py

        return h5py.File("spectra.h5", "w")
    except ImportError:
        return spectra.NpzStore("spectra.npz")


def main(h0_filename, radial_filename, ls, nBaths, nValBaths, n0imps, dnTols, dnValBaths, dnConBaths, Fdd, Fpp, Fpd,
         Gpd, xi_2p, xi_3d, chargeTransferCorrection, hField, nPsiMax, nPrintSlaterWeights, tolPrintOccupation, T,
         energy_cut, delta, deltaRIXS, deltaNIXS):
    """Lowest eigenstates, expectation values and spectra (upstream get_spectra.py:20-332)."""
    t0 = time.time()
    nBaths = OrderedDict(zip(ls, nBaths))
    nValBaths = OrderedDict(zip(ls, nValBaths))
    n0imps = OrderedDict(zip(ls, n0imps))
    dnTols = OrderedDict(zip(ls, dnTols))
    dnValBaths = OrderedDict(zip(ls, dnValBaths))
    dnConBaths = OrderedDict(zip(ls, dnConBaths))
    energy_cut *= k_B * T
    # meshes and polarisations of upstream's driver
    w = np.linspace(-25, 25, 3000)
    epsilons = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    epsilonsRIXSin = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    epsilonsRIXSout = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    wIn = np.linspace(-10, 20, 50)
    wLoss = np.linspace(-2, 12, 4000)
    qsNIXS = [2 * np.array([1, 1, 1]) / np.sqrt(3), 7 * np.array([1, 1, 1]) / np.sqrt(3)]
    liNIXS, ljNIXS = 2, 2
    restrictions = _restrictions(nBaths, nValBaths, n0imps, dnTols, dnValBaths, dnConBaths)
    radialMesh, RiNIXS = np.loadtxt(radial_filename).T
    RjNIXS = np.copy(RiNIXS)
    n_spin_orbitals = sum(2 * (2 * ang + 1) + nb for ang, nb in nBaths.items())
    print("#spin-orbitals:", n_spin_orbitals)
    print("Construct the Hamiltonian operator...")
    hOp = get_hamiltonian_operator(nBaths, nValBaths, [Fdd, Fpp, Fpd, Gpd], [xi_2p, xi_3d],
                                   [n0imps, chargeTransferCorrection], hField, h0_filename)
    print("{:d} processes in the Hamiltonian.".format(len(hOp)))
    print("Create basis...")
    basis = finite.get_basis(nBaths, nValBaths, dnValBaths, dnConBaths, dnTols, n0imps)
    print("#basis states = {:d}".format(len(basis)))
    es, psis = finite.eigensystem(n_spin_orbitals, hOp, basis, nPsiMax)
    print("time(ground_state) = {:.2f} seconds \n".format(time.time() - t0))
    t0 = time.time()
    finite.printThermalExpValues(nBaths, es, psis)
    finite.printExpValues(nBaths, es, psis)
    print("Slater determinants/product states and correspoinding weights")
    for i, psi in enumerate(psis):
        print("Eigenstate {:d}.".format(i))
        print("Consists of {:d} product states.".format(len(psi)))
        ws = np.array([abs(a) ** 2 for a in psi.values()])
        s = np.array(list(psi.keys()))
        j = np.argsort(ws)[::-1]
        if nPrintSlaterWeights > 0:
            print("Highest (product state) weights:")
            print(ws[j][:nPrintSlaterWeights])
            print("Corresponding product states:")
            print(s[j][:nPrintSlaterWeights])
            print("")
    print("Density matrix (in cubic harmonics basis):")
    for i, psi in enumerate(psis):
        print("Eigenstate {:d}".format(i))
        n = finite.getDensityMatrixCubic(nBaths, psi)
        print("#density matrix elements: {:d}".format(len(n)))
        for e, ne in n.items():
            if abs(ne) > tolPrintOccupation:
                if e[0] == e[1]:
                    print("Diagonal: (i,s) =", e[0], ", occupation = {:7.2f}".format(ne))
                else:
                    print("Off-diagonal: (i,si), (j,sj) =", e, ", {:7.2f}".format(ne))
        print("")
    np.savez_compressed(
        "data", ls=ls, nBaths=nBaths, nValBaths=nValBaths, n0imps=n0imps, dnTols=dnTols, dnValBaths=dnValBaths,
        dnConBaths=dnConBaths, Fdd=Fdd, Fpp=Fpp, Fpd=Fpd, Gpd=Gpd, xi_2p=xi_2p, xi_3d=xi_3d,
        chargeTransferCorrection=chargeTransferCorrection, hField=hField, h0_filename=h0_filename, nPsiMax=nPsiMax,
        T=T, energy_cut=energy_cut, delta=delta, restrictions=restrictions, epsilons=epsilons,
        epsilonsRIXSin=epsilonsRIXSin, epsilonsRIXSout=epsilonsRIXSout, deltaRIXS=deltaRIXS, deltaNIXS=deltaNIXS,
        n_spin_orbitals=n_spin_orbitals, hOp=hOp)
    h5f = _open_store()
    for name, data in (("E", es), ("w", w), ("wIn", wIn), ("wLoss", wLoss), ("qsNIXS", qsNIXS), ("r", radialMesh),
                       ("RiNIXS", RiNIXS), ("RjNIXS", RjNIXS)):
        h5f.create_dataset(name, data=data)
    print("time(expectation values) = {:.2f} seconds \n".format(time.time() - t0))
    es = tuple(e for e in es if e - es[0] < energy_cut)
    psis = tuple(psis[i] for i in range(len(es)))
    print("Consider {:d} eigenstates for the spectra \n".format(len(es)))
    spectra.simulate_spectra(es, psis, hOp, T, w, delta, epsilons, wLoss, deltaNIXS, qsNIXS, liNIXS, ljNIXS, RiNIXS,
                             RjNIXS, radialMesh, wIn, deltaRIXS, epsilonsRIXSin, epsilonsRIXSout, restrictions, h5f,
                             nBaths, out_dir=os.getcwd())
    h5f.close()
    print("Script finished.")
    return es, hOp


def parser():
    """Upstream's argument parser (get_spectra.py:427-618): same positional arguments, flags
    and defaults."""
    p = argparse.ArgumentParser(description="Spectroscopy simulations")
    p.add_argument("h0_filename", type=str, help="Filename of non-interacting Hamiltonian, in pickle-format.")
    p.add_argument("radial_filename", type=str, help="Filename of radial part of correlated orbitals.")
    p.add_argument("--ls", type=int, nargs="+", default=[1, 2], help="Angular momenta of correlated orbitals.")
    p.add_argument("--nBaths", type=int, nargs="+", default=[0, 10],
                   help="Number of bath states, for each angular momentum.")
    p.add_argument("--nValBaths", type=int, nargs="+", default=[0, 10],
                   help="Number of valence bath states, for each angular momentum.")
    p.add_argument("--n0imps", type=int, nargs="+", default=[6, 8],
                   help="Initial impurity occupation, for each angular momentum.")
    p.add_argument("--dnTols", type=int, nargs="+", default=[0, 2],
                   help="Max devation from initial impurity occupation, for each angular momentum.")
    p.add_argument("--dnValBaths", type=int, nargs="+", default=[0, 2],
                   help="Max number of electrons to leave valence bath orbitals, for each angular momentum.")
    p.add_argument("--dnConBaths", type=int, nargs="+", default=[0, 0],
                   help="Max number of electrons to enter conduction bath orbitals, for each angular momentum.")
    p.add_argument("--Fdd", type=float, nargs="+", default=[7.5, 0, 9.9, 0, 6.6],
                   help="Slater-Condon parameters Fdd. d-orbitals are assumed.")
    p.add_argument("--Fpp", type=float, nargs="+", default=[0.0, 0.0, 0.0],
                   help="Slater-Condon parameters Fpp. p-orbitals are assumed.")
    p.add_argument("--Fpd", type=float, nargs="+", default=[8.9, 0, 6.8],
                   help="Slater-Condon parameters Fpd. p- and d-orbitals are assumed.")
    p.add_argument("--Gpd", type=float, nargs="+", default=[0.0, 5.0, 0, 2.8],
                   help="Slater-Condon parameters Gpd. p- and d-orbitals are assumed.")
    p.add_argument("--xi_2p", type=float, default=11.629, help="SOC value for p-orbitals. p-orbitals are assumed.")
    p.add_argument("--xi_3d", type=float, default=0.096, help="SOC value for d-orbitals. d-orbitals are assumed.")
    p.add_argument("--chargeTransferCorrection", type=float, default=1.5, help="Double counting parameter.")
    p.add_argument("--hField", type=float, nargs="+", default=[0, 0, 0.0001], help="Magnetic field. (h_x, h_y, h_z)")
    p.add_argument("--nPsiMax", type=int, default=5, help="Maximum number of eigenstates to consider.")
    p.add_argument("--nPrintSlaterWeights", type=int, default=3, help="Printing parameter.")
    p.add_argument("--tolPrintOccupation", type=float, default=0.5, help="Printing parameter.")
    p.add_argument("--T", type=float, default=300, help="Temperature (Kelvin).")
    p.add_argument("--energy_cut", type=float, default=10, help="How many k_B*T above lowest eigenenergy to consider.")
    p.add_argument("--delta", type=float, default=0.2,
                   help="Smearing, half width half maximum (HWHM). Due to short core-hole lifetime.")
    p.add_argument("--deltaRIXS", type=float, default=0.050,
                   help="Smearing, half width half maximum (HWHM). Due to finite lifetime of excited states.")
    p.add_argument("--deltaNIXS", type=float, default=0.100,
                   help="Smearing, half width half maximum (HWHM). Due to finite lifetime of excited states.")
    return p


def run(argv=None):
    """Parse ``argv`` like upstream (with its input checks) and run :func:`main`."""
    args = parser().parse_args(argv)
    if len(args.ls) != len(args.nBaths) or len(args.ls) != len(args.nValBaths):
        raise SystemExit("--ls, --nBaths and --nValBaths need one value per angular momentum")
    for nb, nvb in zip(args.nBaths, args.nValBaths):
        if nb < nvb:
            raise SystemExit("more valence bath states than bath states")
    for ang, n0 in zip(args.ls, args.n0imps):
        if not 0 <= n0 <= 2 * (2 * ang + 1):
            raise SystemExit("impurity occupation out of range")
    if len(args.Fdd) != 5 or len(args.Fpp) != 3 or len(args.Fpd) != 3 or len(args.Gpd) != 4 or len(args.hField) != 3:
        raise SystemExit("wrong number of Slater-Condon or field parameters")
    return main(h0_filename=args.h0_filename, radial_filename=args.radial_filename, ls=tuple(args.ls),
                nBaths=tuple(args.nBaths), nValBaths=tuple(args.nValBaths), n0imps=tuple(args.n0imps),
                dnTols=tuple(args.dnTols), dnValBaths=tuple(args.dnValBaths), dnConBaths=tuple(args.dnConBaths),
                Fdd=tuple(args.Fdd), Fpp=tuple(args.Fpp), Fpd=tuple(args.Fpd), Gpd=tuple(args.Gpd), xi_2p=args.xi_2p,
                xi_3d=args.xi_3d, chargeTransferCorrection=args.chargeTransferCorrection, hField=tuple(args.hField),
                nPsiMax=args.nPsiMax, nPrintSlaterWeights=args.nPrintSlaterWeights,
                tolPrintOccupation=args.tolPrintOccupation, T=args.T, energy_cut=args.energy_cut, delta=args.delta,
                deltaRIXS=args.deltaRIXS, deltaNIXS=args.deltaNIXS)


if __name__ == "__main__":
    run()
