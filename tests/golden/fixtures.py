"""Encode/decode operators, states and restrictions to plain NumPy arrays for ``.npz`` fixtures."""

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _n_words(n):
    return (n + 63) // 64


def encode_states(states, n_spin_orbitals):
    w = _n_words(n_spin_orbitals)
    nb = 8 * w
    if not states:
        return np.zeros((0, w), dtype=np.uint64)
    buf = b"".join(s + b"\x00" * (nb - len(s)) for s in states)
    return np.frombuffer(buf, dtype=">u8").astype(np.uint64).reshape(len(states), w)


def decode_states(words, n_spin_orbitals):
    nbytes = (n_spin_orbitals + 7) // 8
    arr = np.ascontiguousarray(np.asarray(words, dtype=np.uint64).astype(">u8"))
    raw = arr.tobytes()
    stride = arr.shape[1] * 8
    return [raw[k * stride : k * stride + nbytes] for k in range(arr.shape[0])]


def encode_op(prefix, op):
    keys = list(op.keys())
    t = len(keys)
    n_ops = np.zeros(t, np.int32)
    orb = np.zeros((t, 4), np.int32)
    cre = np.zeros((t, 4), bool)
    val = np.zeros(t, np.complex128)
    for k, key in enumerate(keys):
        n_ops[k] = len(key)
        for j, (i, a) in enumerate(key):
            orb[k, j] = i
            cre[k, j] = a == "c"
        val[k] = complex(op[key])
    return {prefix + "_nops": n_ops, prefix + "_orb": orb, prefix + "_cre": cre, prefix + "_val": val}


def decode_op(z, prefix):
    n_ops, orb, cre, val = (z[prefix + s] for s in ("_nops", "_orb", "_cre", "_val"))
    op = {}
    for k in range(len(n_ops)):
        key = tuple((int(orb[k, j]), "c" if cre[k, j] else "a") for j in range(int(n_ops[k])))
        op[key] = complex(val[k])
    return op


def encode_psi(prefix, psi, n_spin_orbitals):
    states = list(psi.keys())
    return {prefix + "_states": encode_states(states, n_spin_orbitals),
            prefix + "_amps": np.array([complex(psi[s]) for s in states], dtype=np.complex128)}


def decode_psi(z, prefix, n_spin_orbitals):
    states = decode_states(z[prefix + "_states"], n_spin_orbitals)
    return dict(zip(states, (complex(a) for a in z[prefix + "_amps"])))


def encode_restrictions(prefix, restrictions):
    idx, lo, hi = [], [], []
    for k, (orbs, (a, b)) in enumerate(restrictions.items()):
        idx.append(sorted(orbs))
        lo.append(a)
        hi.append(b)
    width = max([len(x) for x in idx] + [1])
    arr = np.full((len(idx), width), -1, np.int32)
    for k, x in enumerate(idx):
        arr[k, : len(x)] = x
    return {prefix + "_idx": arr, prefix + "_lo": np.array(lo, np.int32), prefix + "_hi": np.array(hi, np.int32)}


def decode_restrictions(z, prefix):
    out = {}
    for row, a, b in zip(z[prefix + "_idx"], z[prefix + "_lo"], z[prefix + "_hi"]):
        out[frozenset(int(i) for i in row if i >= 0)] = (int(a), int(b))
    return out


def load(name):
    return np.load(os.path.join(HERE, name), allow_pickle=False)


def simulate_inputs():
    """Inputs of the small spectra-driver case (26-orbital model, short meshes) shared by the
    fixture generator and the GPU test of simulate_spectra."""
    from impuritymodel_gb300 import models as M

    mod = M.make_model("config1")
    r, R = M.hydrogenic_3d_radial()
    eps = [np.array(v, dtype=float) for v in ((1, 0, 0), (0, 1, 0), (0, 0, 1))]
    qs = [1.0 * np.array([1, 1, 1]) / np.sqrt(3), 2.0 * np.array([1, 1, 1]) / np.sqrt(3)]
    return dict(mod=mod, T=300.0, w=np.linspace(-25, 25, 400), delta=0.2, epsilons=eps,
                wLoss=np.linspace(-2, 12, 200), deltaNIXS=0.1, qsNIXS=qs, liNIXS=2, ljNIXS=2, RiNIXS=R, RjNIXS=R,
                radialMesh=r, wIn=np.linspace(-5, 10, 3), deltaRIXS=0.05, epsilonsRIXSin=eps, epsilonsRIXSout=eps)
