"""The CPU reference of bench.py (the oracle port of upstream's algorithm), on CPU: one whole
step on one core (the GPU line's cpu_baseline) and whole steps divided among spawned oracle
processes (``bench.py --impl reference``), on a reduced mesh so that the test stays short.
Both divisions of the work must give the same spectra."""

import copy
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _small_work():
    work = copy.deepcopy(bench.WORKLOAD)
    work["xas"]["n_w"] = 200
    work["rixs"]["n_w_in"] = 3
    work["rixs"]["n_w_loss"] = 100
    return work


def test_cpu_baseline_is_one_whole_step():
    line = bench.cpu_baseline(_small_work())
    assert line["cores"] == 1 and line["kind"] == "port" and line["unit"] == "s" and line["steps"] == 1
    assert line["value"] > 0
    assert line["parts_s"]["gs_s"] > 0 and line["parts_s"]["spectra_s"] > 0
    assert "1 core" in line["sample"] and "whole step" in line["sample"]


@pytest.mark.timeout(600)
def test_reference_steps_split_matches_one_process():
    """The work split over two processes gives the spectra of the one-process step (the
    split only changes which process computes each Green's function)."""
    import multiprocessing

    import oracle.ed_oracle as O
    from impuritymodel_gb300 import models

    work = _small_work()
    mod = models.make_model("config2")
    es1, gx1, gr1, _ = bench.ref_step(O, mod, work)
    with multiprocessing.get_context("spawn").Pool(2, initializer=bench._ref_worker_init, initargs=(work,)) as pool:
        es2, gx2, gr2, _ = bench.ref_step(O, mod, work, pool=pool, procs=2)
    # ARPACK starts from a random vector: energies agree to its tolerance, spectra closely
    assert np.abs(es1 - es2).max() < 1e-8
    assert np.abs(gx1).max() > 0 and np.abs(gr1).max() > 0
    assert np.abs(gx1 - gx2).max() <= 1e-5 * np.abs(gx1).max()
    # RIXS: BiCGSTAB (rtol 1e-5) and the unreorthogonalised final-state Lanczos amplify the
    # eigenvector differences; a missing unit would leave a whole slice at zero
    assert np.abs(gr1 - gr2).sum() <= 2e-2 * np.abs(gr1).sum()
    assert np.all(np.abs(gr2).reshape(-1, gr2.shape[-1]).max(1) > 0)
    times = bench.reference_steps(1, 0, 2, work)
    assert len(times) == 1 and times[0] > 0
