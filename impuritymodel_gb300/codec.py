"""Product-state codec: upstream ``bytes`` states <-> packed ``uint64`` words.

Upstream (impurityModel/ed/product_state_representation.py:131-161, 246-273) stores a
product state as the ``bytes`` of an MSB-first bitarray: spin-orbital ``i`` is bit
``7 - i % 8`` of byte ``i // 8``.  Here spin-orbital ``i`` is bit ``63 - i % 64`` of word
``i // 64``; reading the zero-padded bytes as big-endian 64-bit words gives exactly this
layout, and lexicographic order of the word tuples equals the order of the ``bytes``.
"""

from __future__ import annotations

import numpy as np


def n_words(n_spin_orbitals):
    return (int(n_spin_orbitals) + 63) // 64


def n_bytes(n_spin_orbitals):
    return (int(n_spin_orbitals) + 7) // 8


def bytes_to_words(states, n_spin_orbitals):
    """Iterable of ``bytes`` -> ``uint64[N, W]``."""
    w = n_words(n_spin_orbitals)
    nb = 8 * w
    states = list(states)
    if not states:
        return np.zeros((0, w), dtype=np.uint64)
    want = n_bytes(n_spin_orbitals)
    if set(map(len, states)) != {want}:
        raise ValueError("product states must all be %d bytes long" % want)
    raw = np.frombuffer(b"".join(states), dtype=np.uint8).reshape(len(states), want)
    if want != nb:  # zero-pad each state to whole words
        padded = np.zeros((len(states), nb), dtype=np.uint8)
        padded[:, :want] = raw
        raw = padded
    return raw.view(">u8").astype(np.uint64).reshape(len(states), w)


def words_to_bytes(words, n_spin_orbitals):
    """``uint64[N, W]`` -> list of ``bytes``."""
    nb = n_bytes(n_spin_orbitals)
    arr = np.ascontiguousarray(np.asarray(words, dtype=np.uint64).astype(">u8"))
    if arr.ndim != 2 or arr.shape[0] == 0:
        return []
    raw = arr.tobytes()
    stride = arr.shape[1] * 8
    return [raw[k * stride : k * stride + nb] for k in range(arr.shape[0])]


def tuple_to_bytes(t, n_spin_orbitals):
    """Occupied spin-orbital indices -> ``bytes`` (upstream ``psr.tuple2bytes``)."""
    nb = n_bytes(n_spin_orbitals)
    v = 0
    for i in t:
        v |= 1 << (8 * nb - 1 - int(i))
    return v.to_bytes(nb, "big")


def bytes_to_tuple(b, n_spin_orbitals):
    nb = len(b)
    v = int.from_bytes(b, "big")
    return tuple(i for i in range(n_spin_orbitals) if (v >> (8 * nb - 1 - i)) & 1)


def psi_to_arrays(psi, n_spin_orbitals):
    """dict {bytes: amplitude} -> (uint64[N, W], float64[N, 2])."""
    states = list(psi.keys())
    words = bytes_to_words(states, n_spin_orbitals)
    amps = np.fromiter(psi.values(), dtype=np.complex128, count=len(states))
    return words, np.ascontiguousarray(amps.view(np.float64).reshape(-1, 2))


def arrays_to_psi(words, amps, n_spin_orbitals):
    """(uint64[N, W], float64[N, 2]) -> dict {bytes: complex} in row order."""
    states = words_to_bytes(words, n_spin_orbitals)
    a = np.ascontiguousarray(np.asarray(amps, dtype=np.float64).reshape(-1, 2))
    return dict(zip(states, a.view(np.complex128).ravel().tolist()))
