"""GB300-native exact diagonalization for Anderson impurity models.

Drop-in for the hot path of impurityModel: ``impuritymodel_gb300.finite`` mirrors
``impurityModel.ed.finite`` (applyOp, get_basis, Hamiltonian builders, expand_basis,
eigensystem, Lanczos) and ``impuritymodel_gb300.spectra`` mirrors
``impurityModel.ed.spectra`` (getGreen, getSpectra, getRIXSmap).  The compute runs in
hand-written sm_103a kernels of ``libedgpu.so`` (C ABI in ``include/edgpu.h``); the
device entry points are also PyTorch operators, ``torch.ops.edgpu.*`` (module ``ops``).
"""

__version__ = "0.1.0"


def build(verbose=False, force=False):
    from .nvcc_build import build as _build

    return _build(verbose=verbose, force=force)


from . import ops  # noqa: E402,F401  (registers torch.ops.edgpu.*)
