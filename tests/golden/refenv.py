"""Import the upstream impurityModel package in this container (fixture generation only).

The upstream package needs ``bitarray``, ``mpi4py`` and ``h5py`` (absent here) and two
names that newer NumPy/SciPy removed (``np.trapz``, ``scipy.special.sph_harm``).  This
module puts the stand-ins of ``_standins/`` on ``sys.path`` and restores the two names,
then imports ``impurityModel.ed.finite`` / ``spectra`` from the read-only upstream checkout.

Nothing under ``impuritymodel_gb300/`` imports this; the GPU machine never runs it.
"""

import os
import sys

REFERENCE_ROOT = os.environ.get("IMPURITYMODEL_REFERENCE", "/root/reference")
_HERE = os.path.dirname(os.path.abspath(__file__))


def available():
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "impurityModel", "ed"))


def load():
    """Return the upstream ``(finite, spectra, psr, create, remove)`` modules."""
    if not available():
        raise RuntimeError("upstream impurityModel checkout not found at %s" % REFERENCE_ROOT)
    standins = os.path.join(_HERE, "_standins")
    if standins not in sys.path:
        sys.path.insert(0, standins)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import numpy as np
    import scipy.special

    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    if not hasattr(scipy.special, "sph_harm"):

        def sph_harm(m, n, azimuth, polar):
            return scipy.special.sph_harm_y(n, m, polar, azimuth)

        scipy.special.sph_harm = sph_harm
    from impurityModel.ed import create, finite, remove, spectra
    from impurityModel.ed import product_state_representation as psr

    return finite, spectra, psr, create, remove
