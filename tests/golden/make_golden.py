"""Generate golden fixtures by running the upstream impurityModel implementation.

Run in a container that has the upstream checkout (read-only) at
``$IMPURITYMODEL_REFERENCE`` (default ``/root/reference``)::

    python tests/golden/make_golden.py

Writes small ``.npz`` files next to this script.  Upstream runs behind the stand-ins of
``_standins/`` (see ``refenv.py``).  Inputs are the seeded synthetic models of
``impuritymodel_gb300.models`` plus upstream's own shipped NiO 50-bath inputs
(``impurityModel/test/referenceOutput/Ni_NiO_50bath/data.npz``, read with a restricted
unpickler) and its shipped thermal spectra (``XAS.dat``).
"""

import io
import os
import pickle
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refenv  # noqa: E402

from impuritymodel_gb300 import models as M  # noqa: E402
from tests.golden.fixtures import encode_op, encode_psi, encode_restrictions, encode_states  # noqa: E402


class _SafeUnpickler(pickle.Unpickler):
    """Only containers, complex numbers and NumPy scalar/array reconstruction."""

    _ALLOWED = {
        ("collections", "OrderedDict"),
        ("builtins", "complex"),
        ("builtins", "frozenset"),
        ("builtins", "set"),
        ("builtins", "dict"),
        ("builtins", "tuple"),
        ("builtins", "list"),
    }

    def find_class(self, module, name):
        if (module, name) in self._ALLOWED:
            import builtins
            import collections

            return getattr(collections if module == "collections" else builtins, name)
        if module in ("numpy.core.multiarray", "numpy._core.multiarray") and name in ("scalar", "_reconstruct"):
            from numpy._core import multiarray

            return getattr(multiarray, name)
        if module == "numpy" and name in ("dtype", "ndarray"):
            return getattr(np, name)
        raise pickle.UnpicklingError("blocked %s.%s" % (module, name))


def _load_npz_object(npz, key):
    arr = npz[key]
    return arr.item() if arr.dtype == object and arr.shape == () else arr


def load_nio_data(ref_root):
    path = os.path.join(ref_root, "impurityModel/test/referenceOutput/Ni_NiO_50bath/data.npz")
    import zipfile

    out = {}
    with zipfile.ZipFile(path) as z:
        for name in z.namelist():
            with z.open(name) as fh:
                raw = fh.read()
            key = name[:-4]
            try:
                arr = np.load(io.BytesIO(raw), allow_pickle=False)
            except ValueError:
                # object array: parse the .npy header, then unpickle the payload safely
                buf = io.BytesIO(raw)
                version = np.lib.format.read_magic(buf)
                if version == (1, 0):
                    np.lib.format.read_array_header_1_0(buf)
                else:
                    np.lib.format.read_array_header_2_0(buf)
                arr = _SafeUnpickler(buf).load()
            out[key] = arr
    return out


def main():
    finite, spectra, psr, create, remove = refenv.load()
    import contextlib

    quiet = contextlib.redirect_stdout(io.StringIO())
    t0 = time.time()

    # ---------------- config1: full small pipeline -------------------------------------
    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    with quiet:
        basis = finite.get_basis(*mod.basis_args())
        h = finite.get_hamiltonian_matrix(n, mod.hOp, basis)
        es, psis = finite.eigensystem(n, mod.hOp, basis, 3)
    tops = mod.xas_ops()
    w = np.linspace(-25, 25, 2000)
    with quiet:
        gs_xas = spectra.getSpectra(n, mod.hOp, tops, psis, es, w, 0.1, mod.restrictions)
    psi1 = finite.applyOp(n, tops[0], psis[0], 1e-7, mod.restrictions)
    with quiet:
        exp_basis = finite.expand_basis(n, {}, mod.hOp, tuple(psi1.keys()), mod.restrictions)
        hx, bidx = finite.get_hamiltonian_matrix_from_h_dict(
            {b: finite.applyOp(n, mod.hOp, {b: 1}, restrictions=mod.restrictions) for b in exp_basis}, exp_basis)
    # Lanczos coefficients for the normalised psi1
    nrm = np.sqrt(finite.norm2(psi1))
    psi0 = np.zeros(len(exp_basis), dtype=complex)
    for s, a in psi1.items():
        psi0[bidx[s]] = a / nrm
    with quiet:
        alpha, beta = finite.get_tridiagonal_krylov_vectors(hx, psi0, 150)
    # PS / IPS single-operator spectra for state 0..2
    with quiet:
        gs_ps = spectra.getSpectra(n, mod.hOp, mod.ps_ops()[:3], psis, es, -w, -0.1, mod.restrictions)
        gs_ips = spectra.getSpectra(n, mod.hOp, mod.ips_ops()[:3], psis, es, w, 0.1, mod.restrictions)
    # small RIXS map with upstream's BiCGSTAB
    w_in = np.linspace(-5, 10, 4)
    w_loss = np.linspace(-2, 12, 300)
    with quiet:
        gs_rixs = spectra.getRIXSmap(n, mod.hOp, tops, mod.rixs_out_ops(), psis[:1], es[:1], w_in, w_loss,
                                     0.2, 0.05, mod.restrictions)
    hcoo = h.tocoo()
    np.savez_compressed(
        os.path.join(HERE, "config1.npz"),
        n_spin_orbitals=n,
        **encode_op("hop", mod.hOp),
        **encode_restrictions("restr", mod.restrictions),
        basis=encode_states(basis, n),
        h_row=hcoo.row, h_col=hcoo.col, h_val=hcoo.data,
        es=es,
        **{k: v for i, p in enumerate(psis) for k, v in encode_psi("eig%d" % i, p, n).items()},
        w=w, gs_xas=gs_xas,
        **encode_psi("psi1", psi1, n),
        exp_basis=encode_states(exp_basis, n),
        alpha=alpha, beta=beta,
        gs_ps=gs_ps, gs_ips=gs_ips,
        w_in=w_in, w_loss=w_loss, gs_rixs=gs_rixs,
    )
    print("config1 done %.1fs basis=%d exp=%d" % (time.time() - t0, len(basis), len(exp_basis)))

    # ---------------- applyOp semantics on config1 inputs (memo + restrictions) ----------
    cases = {}
    t_big = {}
    rng = np.random.default_rng(7)
    for k, i in enumerate([0, 1, 2, 0]):
        psi = {s: complex(a) for s, a in psis[i].items()}
        out = finite.applyOp(n, tops[k % 3], psi, 1e-7, mod.restrictions, t_big)
        cases.update(encode_psi("memo%d" % k, out, n))
    big = {b: complex(rng.normal(), rng.normal()) for b in basis}
    out = finite.applyOp(n, mod.hOp, big, 1e-12, None, None)
    cases.update(encode_psi("hpsi_in", big, n))
    cases.update(encode_psi("hpsi_out", out, n))
    out = finite.applyOp(n, mod.hOp, big, 1e-12, mod.restrictions, None)
    cases.update(encode_psi("hpsi_restr_out", out, n))
    np.savez_compressed(os.path.join(HERE, "applyop_config1.npz"), **cases)
    print("applyop done %.1fs" % (time.time() - t0))

    # ---------------- config2: 50-bath ground state + XAS --------------------------------
    mod2 = M.make_model("config2")
    n2 = mod2.n_spin_orbitals
    with quiet:
        basis2 = finite.get_basis(*mod2.basis_args())
        es2, psis2 = finite.eigensystem(n2, mod2.hOp, basis2, 5)
    cut = 10 * M.K_B * 300
    keep = [i for i in range(len(es2)) if es2[i] - es2[0] < cut]
    w2 = np.linspace(-25, 25, 3000)
    with quiet:
        gs2 = spectra.getSpectra(n2, mod2.hOp, mod2.xas_ops(), psis2[: len(keep)], es2[: len(keep)], w2, 0.2,
                                 mod2.restrictions)
    np.savez_compressed(
        os.path.join(HERE, "config2.npz"),
        n_spin_orbitals=n2,
        es=es2,
        n_basis=len(basis2),
        n_keep=len(keep),
        w=w2,
        xas_thermal=spectra.thermal_average(es2[: len(keep)], -gs2.imag, T=300),
        **{k: v for i, p in enumerate(psis2[: len(keep)]) for k, v in encode_psi("eig%d" % i, p, n2).items()},
    )
    print("config2 done %.1fs basis=%d keep=%d" % (time.time() - t0, len(basis2), len(keep)))

    # ---------------- upstream's NiO 50-bath inputs ---------------------------------------
    data = load_nio_data(refenv.REFERENCE_ROOT)
    hop = data["hOp"].item() if isinstance(data["hOp"], np.ndarray) else data["hOp"]
    restr = data["restrictions"].item() if isinstance(data["restrictions"], np.ndarray) else data["restrictions"]
    xas_dat = np.loadtxt(os.path.join(refenv.REFERENCE_ROOT,
                                      "impurityModel/test/referenceOutput/Ni_NiO_50bath/XAS.dat"))
    np.savez_compressed(
        os.path.join(HERE, "nio50.npz"),
        n_spin_orbitals=int(data["n_spin_orbitals"]),
        **encode_op("hop", hop),
        **encode_restrictions("restr", restr),
        xas_dat=xas_dat,
        es_log=np.array([-903.8237]),
    )
    print("nio done %.1fs" % (time.time() - t0))


def observables():
    """Upstream's 3d observables (finite.py:843-1298) on the stored eigenstates of the 26- and
    66-spin-orbital models: density matrices (spherical, cubic), N(3d), eg/t2g occupations,
    Lz, Sz, L^2, S^2, and the S/L ladder- and z-operator results on the lowest state."""
    finite, spectra, psr, create, remove = refenv.load()
    from tests.golden.fixtures import decode_psi, load

    out = {}
    for tag, cfg, fname in (("c1", "config1", "config1.npz"), ("c2", "config2", "config2.npz")):
        mod = M.make_model(cfg)
        z = load(fname)
        n = int(z["n_spin_orbitals"])
        nb = mod.nBaths
        k = 0
        while ("eig%d" % k + "_states") in z.files:
            k += 1
        psis = [decode_psi(z, "eig%d" % i, n) for i in range(k)]
        dm = np.zeros((k, 10, 10), dtype=complex)
        dmc = np.zeros((k, 10, 10), dtype=complex)
        vals = np.zeros((k, 9))
        for i, psi in enumerate(psis):
            for ((l, si, mi), (l2, sj, mj)), v in finite.getDensityMatrix(nb, psi).items():
                dm[i, si * 5 + mi + 2, sj * 5 + mj + 2] = v
            for ((si, ii), (sj, jj)), v in finite.getDensityMatrixCubic(nb, psi).items():
                dmc[i, si * 5 + ii, sj * 5 + jj] = v
            occ = finite.getEgT2gOccupation(nb, psi)
            vals[i] = [finite.getTraceDensityMatrix(nb, psi), *np.real(occ), finite.getLz3d(nb, psi),
                       finite.getSz3d(nb, psi), finite.getLsqr3d(nb, psi), finite.getSsqr3d(nb, psi)]
        out[tag + "_n_states"] = k
        out[tag + "_dm"] = dm
        out[tag + "_dm_cubic"] = dmc
        out[tag + "_values"] = vals
        for name in ("applySz3d", "applyLz3d", "applySplus3d", "applyLplus3d", "applySminus3d", "applyLminus3d"):
            out.update(encode_psi(tag + "_" + name, getattr(finite, name)(nb, psis[0]), n))
    np.savez_compressed(os.path.join(HERE, "observables.npz"), **out)
    print("observables done")


def simulate():
    """Upstream's spectra driver simulate_spectra (spectra.py:36-293) on the stored
    eigenstates of the 26-orbital model: every dataset and output file it writes."""
    import contextlib
    import tempfile

    finite, spectra, psr, create, remove = refenv.load()
    import h5py  # the in-memory stand-in of _standins/

    from tests.golden.fixtures import decode_psi, load

    z = load("config1.npz")
    n = int(z["n_spin_orbitals"])
    psis = [decode_psi(z, "eig%d" % i, n) for i in range(len(z["es"]))]
    from tests.golden.fixtures import simulate_inputs

    a = simulate_inputs()
    mod = a.pop("mod")
    h5f = h5py.File("spectra.h5", "w")
    out = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                spectra.simulate_spectra(z["es"], psis, mod.hOp, a["T"], a["w"], a["delta"], a["epsilons"], a["wLoss"],
                                         a["deltaNIXS"], a["qsNIXS"], a["liNIXS"], a["ljNIXS"], a["RiNIXS"],
                                         a["RjNIXS"], a["radialMesh"], a["wIn"], a["deltaRIXS"], a["epsilonsRIXSin"],
                                         a["epsilonsRIXSout"], mod.restrictions, h5f, mod.nBaths)
            for f in ("PS.dat", "XPS.dat", "NIXS.dat", "XAS.dat", "RIXS.bin"):
                with open(f, "rb") as fh:
                    out["file_" + f.replace(".", "_")] = np.frombuffer(fh.read(), dtype=np.uint8)
        finally:
            os.chdir(cwd)
    for k, v in h5f.data.items():
        out["ds_" + k] = v
    np.savez_compressed(os.path.join(HERE, "simulate_config1.npz"), **out)
    print("simulate done")


def nio_cli():
    """Upstream's shipped NiO 50-bath run (scripts/run_Ni_NiO_Xbath.sh 50: get_spectra.py with
    --nBaths 0 50 --nValBaths 0 50, other flags at their defaults): its inputs (the h0 operator
    read with the restricted unpickler, the Ni 3d radial orbital) and its output files."""
    root = refenv.REFERENCE_ROOT
    with open(os.path.join(root, "h0/h0_NiO_50bath.pickle"), "rb") as fh:
        h0 = _SafeUnpickler(fh).load()
    keys = [repr(k) for k in h0.keys()]
    vals = np.array([complex(v) for v in h0.values()])
    radial = np.loadtxt(os.path.join(root, "radialOrbitals/Ni3d.dat"))
    ref = os.path.join(root, "impurityModel/test/referenceOutput/Ni_NiO_50bath")
    out = dict(h0_keys=np.array(keys), h0_vals=vals, radial=radial)
    for f in ("PS.dat", "XPS.dat", "NIXS.dat", "XAS.dat", "RIXS.bin"):
        with open(os.path.join(ref, f), "rb") as fh:
            out["file_" + f.replace(".", "_")] = np.frombuffer(fh.read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "nio50_cli.npz"), **out)
    print("nio cli done: %d h0 terms" % len(keys))


def dropin():
    """Upstream's drop-in functions on the seeded models, for the parity tests of the same
    functions here: get_basis of the 66-spin-orbital model (finite.py:294-374),
    get_hamiltonian_matrix_from_h_dict on an h_dict that expand_basis filled
    (finite.py:1613-1693, 1696-1803), getGreen with the h_dict it fills (spectra.py:551-681),
    and eigensystem of the 26-spin-orbital model without a magnetic field and without 3d
    spin-orbit coupling, whose ground multiplet is an exactly degenerate spin triplet
    (finite.py:58-118, eigsh k=nPsiMax)."""
    import contextlib

    finite, spectra, psr, create, remove = refenv.load()
    from tests.golden.fixtures import decode_psi, load

    quiet = contextlib.redirect_stdout(io.StringIO())
    out = {}
    mod2 = M.make_model("config2")
    n2 = mod2.n_spin_orbitals
    with quiet:
        basis2 = finite.get_basis(*mod2.basis_args())
    out["basis2"] = encode_states(list(basis2), n2)
    # h_dict from expand_basis, then the matrix built from it
    mod = M.make_model("config1")
    n = mod.n_spin_orbitals
    z = load("config1.npz")
    psi1 = decode_psi(z, "psi1", n)
    h_dict = {}
    with quiet:
        exp_basis = finite.expand_basis(n, h_dict, mod.hOp, tuple(psi1.keys()), mod.restrictions)
        hx, bidx = finite.get_hamiltonian_matrix_from_h_dict(h_dict, exp_basis)
    keys = list(h_dict.keys())
    out["hd_keys"] = encode_states(keys, n)
    out["hd_ptr"] = np.cumsum([0] + [len(h_dict[k]) for k in keys])
    out["hd_out"] = encode_states([s for k in keys for s in h_dict[k]], n)
    out["hd_val"] = np.array([complex(v) for k in keys for v in h_dict[k].values()], dtype=np.complex128)
    out["hd_basis"] = encode_states(list(exp_basis), n)
    hc = hx.tocoo()
    out["hd_row"], out["hd_col"], out["hd_h"] = hc.row, hc.col, hc.data
    # getGreen on the normalised psi1 with a fresh h_dict (filled by upstream)
    nrm = np.sqrt(finite.norm2(psi1))
    psin = {s_: a / nrm for s_, a in psi1.items()}
    w = np.linspace(-25, 25, 500)
    g_dict = {}
    with quiet:
        g = spectra.getGreen(n, float(z["es"][0]), psin, mod.hOp, w, 0.1, 150, 1e-7, mod.restrictions, g_dict)
    out["green_w"] = w
    out["green_g"] = g
    out["green_keys"] = encode_states(list(g_dict.keys()), n)
    out["green_nout"] = np.array([len(v) for v in g_dict.values()])
    # exactly degenerate ground multiplet: no magnetic field and no 3d spin-orbit coupling,
    # so the d8 ground state is a spin triplet (three equal energies)
    mod0 = M.make_model("config1", hfield=(0.0, 0.0, 0.0), xi_3d=0.0)
    with quiet:
        basis0 = finite.get_basis(*mod0.basis_args())
        es0, psis0 = finite.eigensystem(n, mod0.hOp, basis0, 6)
    out["deg_es"] = np.asarray(es0)
    np.savez_compressed(os.path.join(HERE, "dropin.npz"), **out)
    print("dropin done: basis2 %d, h_dict %d, deg es %s" % (len(basis2), len(keys), np.round(es0, 6)))


if __name__ == "__main__":
    if sys.argv[1:] == ["dropin"]:
        dropin()
    elif sys.argv[1:] == ["nio_cli"]:
        nio_cli()
    elif sys.argv[1:] == ["observables"]:
        observables()
    elif sys.argv[1:] == ["simulate"]:
        simulate()
    else:
        main()
        observables()
        simulate()
        nio_cli()
        dropin()
