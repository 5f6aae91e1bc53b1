"""The row-scheduled H.v kernel (edgpu_spmv_plan / edgpu_spmv_planned[_c64]) and its autotuner.

Numerics against a plain FP64 product of the same matrix (SciPy on the host): complex128
vectors at 1e-13 relative, complex64 vectors with float32 accumulation at 2e-6 relative
(scale of the row sums), for every launch mapping the autotuner chooses from, real and
complex values, vector widths R from 1 to 64, empty rows and rows long enough to be served
by whole warps.  The schedule must be a permutation with the heavy rows first, longest first.
"""

import numpy as np
import pytest
import scipy.sparse
import torch

pytestmark = pytest.mark.gpu


def _matrix(n, seed, complex_vals):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, n)
    lens[rng.choice(n, 40, replace=False)] = rng.integers(64, 300, 40)  # heavy rows
    lens[rng.choice(n, 25, replace=False)] = 0  # empty rows
    rows = np.repeat(np.arange(n), lens)
    cols = rng.integers(0, n, rows.size)
    vals = rng.standard_normal(rows.size)
    if complex_vals:
        vals = vals + 1j * rng.standard_normal(rows.size)
    h = scipy.sparse.csr_matrix((vals, (rows, cols)), shape=(n, n))
    h.sum_duplicates()
    h.sort_indices()
    return h


@pytest.mark.parametrize("complex_vals", [False, True])
def test_planned_spmv_matches_fp64_for_every_mapping(eng, complex_vals):
    from impuritymodel_gb300 import finite

    n = 6000
    h = _matrix(n, 3 + complex_vals, complex_vals)
    csr = finite._scipy_to_device_csr(eng, h)
    rng = np.random.default_rng(9)
    for precision, widths in ((0, (1, 2, 4, 8, 16, 32)), (1, (2, 4, 8, 16, 32, 64))):
        if precision:
            csr.mixed()
        for R in widths:
            mappings = eng.spmv_candidates(csr, R, precision)
            assert any(m[0] == "pages" for m in mappings) == (
                (precision or not complex_vals) and R // (2 if precision else 1) in (2, 4, 8, 16))
            x = rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))
            ref = h @ x
            xt = torch.from_numpy(x).to(eng.device)
            scale = np.abs(h).dot(np.abs(x)).max()
            tol = 1e-13 if precision == 0 else 2e-6
            for m in (mappings if R in (2, 16) else mappings[::5]):
                y = eng.spmv(csr, xt, precision=precision, mapping=m).cpu().numpy()
                err = np.abs(y - ref).max() / scale
                assert err < tol, (precision, R, m, err)


def test_plan_is_a_heavy_first_length_schedule(eng):
    from impuritymodel_gb300 import finite

    n = 6000
    h = _matrix(n, 1, False)
    csr = finite._scipy_to_device_csr(eng, h)
    lens = np.diff(h.indptr)
    for window in (256, 4096, 0):
        for heavy_min in (16, 64):
            sched, nh = eng.spmv_plan(csr, window, heavy_min)
            s = sched.cpu().numpy()
            assert np.array_equal(np.sort(s), np.arange(n))
            assert nh == int(np.sum(lens >= heavy_min))
            heavy = s[:nh]
            assert np.all(lens[heavy] >= heavy_min)
            assert np.all(np.diff(lens[heavy]) <= 0)
            light = s[nh:]
            w = window or n
            win = light // w
            assert np.all(np.diff(win) >= 0)  # windows in order
            for k in np.unique(win):
                seg = light[win == k]
                assert np.all(np.diff(lens[seg]) <= 0)  # longest first within a window
                same = np.diff(lens[seg]) == 0
                assert np.all(np.diff(seg)[same] > 0)  # stable


def test_autotuner_picks_and_caches_a_mapping(eng, tmp_path):
    from impuritymodel_gb300 import finite
    from impuritymodel_gb300.tuner import Autotuner

    h = _matrix(4000, 5, False)
    csr = finite._scipy_to_device_csr(eng, h)
    R = 8
    x = torch.randn((4000, R), dtype=torch.complex128, device=eng.device)
    y = torch.empty_like(x)
    xr, yr = torch.view_as_real(x), torch.view_as_real(y)
    path = str(tmp_path / "tune.json")
    t = Autotuner(path)
    cands = eng.spmv_candidates(csr, R, 0)
    key = eng.spmv_key(csr, R, 0)
    calls = []

    def run(c):
        calls.append(c)
        eng._spmv_planned(csr, xr, yr, R, 0, c)

    best = t.pick("spmv", key, cands, run)
    assert best in cands and len(calls) >= len(cands)
    assert any(c[0] == "pages" for c in cands) and any(c[0] == "sched" for c in cands)
    n_calls = len(calls)
    assert t.pick("spmv", key, cands, run) == best and len(calls) == n_calls  # cached
    t2 = Autotuner(path)  # reloaded from the file
    assert t2.lookup("spmv", key) == best
    times = t2.report("spmv")["spmv|" + ",".join(str(k) for k in key)]["times_us"]
    assert len(times) == len(cands) and all(v > 0 for v in times.values())


@pytest.mark.parametrize("complex_vals", [False, True])
def test_tma_gather_form_equals_paged_form(eng, complex_vals):
    """The tensor-memory-accelerator form (x rows by bulk-tensor gathers into shared memory)
    gives the paged form's product bit for bit, for every ring size and page size, on a matrix
    with heavy and empty rows; no wait runs out."""
    from impuritymodel_gb300 import finite

    n = 6000
    h = _matrix(n, 5 + complex_vals, complex_vals)
    csr = finite._scipy_to_device_csr(eng, h)
    csr.mixed()
    rng = np.random.default_rng(11)
    eng.reset_status()
    for R in (4, 8, 16, 32):
        x = torch.from_numpy(rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))).to(eng.device)
        pages = [m for m in eng.spmv_candidates(csr, R, 1) if m[0] == "pages" and m[3] == 4 and m[5] == 0]
        tma = [("tma", m[1], m[2], sl, m[4], 0) for m in pages[::3] for sl in eng.SPMV_SLOTS]
        assert tma
        for m in tma:
            paged = ("pages", m[1], m[2], 4, m[4], 0)
            y_t = eng.spmv(csr, x, precision=1, mapping=m)
            y_p = eng.spmv(csr, x, precision=1, mapping=paged)
            assert torch.equal(y_t, y_p), (R, m)
    assert int(eng.status.item()) == 0
