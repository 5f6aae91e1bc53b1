#!/usr/bin/env python
"""Benchmark: ground state + XAS + RIXS map of the 50-bath model on one GB300.

One step = the whole pipeline on the seeded 66-spin-orbital model (5 bath levels per 3d
spin-orbital, seed 1, at most 3 bath holes and 1 core hole):

* ground state: 5 lowest eigenpairs of H on the 1770-state restricted basis;
* XAS: 3 dipole polarisations x the eigenstates within 10 k_B T (T = 300 K), 3000 points
  on [-25, 25] eV, broadening 0.2 eV, Krylov size 150;
* RIXS: 3 x 3 polarisations x 50 incoming energies on [-10, 20] eV x 4000 loss points on
  [-2, 12] eV, broadenings 0.2 / 0.05 eV (upstream get_spectra.py defaults).

``value`` is the device-resident time per step (operator tables and basis already in HBM)
of the fastest form whose spectra stay within 1e-3 relative L1 of the plain FP64 form;
``e2e`` is the same pipeline through the drop-in dict API (finite.eigensystem,
spectra.getSpectra, spectra.getRIXSmap) with host inputs and outputs.

``roofline`` reports the H·v kernel (the batched complex SpMV at the heart of every
Lanczos step) on a sector larger than L2: the photoemission sector of the seeded
316-spin-orbital model (30 bath levels, seed 3, at most 2 bath holes), complex64 vectors
and float32 values, 16 vectors per launch, timed with CUDA events on its stream.

``--impl reference`` times whole steps of the CPU oracle (NumPy/SciPy restatement of
upstream) on every host core; ``cpu_baseline`` is one whole step of it on one core.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

K_B = 8.617333262e-05
T_KELVIN = 300.0
WORKLOAD = dict(
    workload="gs_xas_rixs_50bath",
    model="66 spin-orbitals: 6 2p + 10 3d + 50 bath, seed 1, <=3 bath holes, <=1 core hole",
    n_psi=5,
    energy_cut_kT=10,
    xas=dict(polarisations=3, n_w=3000, w=[-25.0, 25.0], delta=0.2),
    rixs=dict(pol_in=3, pol_out=3, n_w_in=50, w_in=[-10.0, 20.0], n_w_loss=4000, w_loss=[-2.0, 12.0],
              delta_in=0.2, delta_loss=0.05),
    krylov=150,
    slater_weight_min=1e-7,
)
METRIC = "time to GS+XAS+RIXS at 50 bath"
# Arithmetic forms of the Green's-function pipeline (the ``precision`` argument of the
# spectra functions).  Each is judged by the same equal-error test against the exact
# resolvent before its time can become the headline.
FORMS = {"plain_fp64": 0, "fp64_krylov_fp32_cfrac": 2, "df64_krylov_fp32_cfrac": 3, "mixed_c64": 1}
FORM_DTYPES = {"plain_fp64": "c128", "fp64_krylov_fp32_cfrac": "c128+f32", "df64_krylov_fp32_cfrac": "df64+f32",
               "mixed_c64": "c64+f64"}
MIXED_L1_TOL = 1e-3


def meshes():
    x = WORKLOAD["xas"]
    r = WORKLOAD["rixs"]
    return (np.linspace(x["w"][0], x["w"][1], x["n_w"]), np.linspace(r["w_in"][0], r["w_in"][1], r["n_w_in"]),
            np.linspace(r["w_loss"][0], r["w_loss"][1], r["n_w_loss"]))


def rel_l1(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


# ---------------------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------------------


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = str(gpu_index)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------


class Pipeline:
    def __init__(self, eng):
        from impuritymodel_gb300 import finite, models
        from impuritymodel_gb300.engine import DeviceOp, make_restrictions

        self.eng = eng
        self.mod = models.make_model("config2")
        m = self.mod
        self.n = m.n_spin_orbitals
        self.basis = finite.get_basis(*m.basis_args())
        self.dop = DeviceOp(m.hOp, eng.device)
        self.restr = make_restrictions(m.restrictions, self.n)
        self.xas_dops = [DeviceOp(t, eng.device) for t in m.xas_ops()]
        self.out_dops = [DeviceOp(t, eng.device) for t in m.rixs_out_ops()]
        self.sb = finite._SortedBasis(eng, list(self.basis), self.n)
        self.w, self.w_in, self.w_loss = meshes()
        # the host operator dicts a caller of the dict API holds (built once, outside any step)
        self.xas_ops_host = m.xas_ops()
        self.out_ops_host = m.rixs_out_ops()

    def step(self, precision=0, timing=None, capture=None, perturb=None, batched=True, gs_basis=None):
        """One pipeline step; ``gs_basis`` (a pruned ground-state basis, pruning.ExpandedBasis)
        replaces the full restricted basis for the ground state."""
        from impuritymodel_gb300 import finite, spectra

        W = WORKLOAD
        sb = gs_basis if gs_basis is not None else self.sb
        es, psi_t, h_gs = finite.eigensystem_device(self.eng, self.dop, sb, W["n_psi"],
                                                    precision=3 if precision == 3 else 0, with_hamiltonian=True)
        ne = int(np.sum(es - es[0] < W["energy_cut_kT"] * K_B * T_KELVIN))
        es, psi_t = es[:ne], psi_t[:ne]
        # the ground-state sector serves the RIXS final states when it is closed
        gs_sector = spectra.closed_sector(self.eng, self.dop, self.restr, sb.sorted, h_gs,
                                          sb.words) if batched else None
        if capture is None and perturb is None and timing is None and batched:
            # XAS on a side stream while the RIXS pipeline runs on the current one
            g_xas, g_rixs = spectra.xas_rixs_device(
                self.eng, self.dop, self.restr, self.xas_dops, self.xas_dops, self.out_dops, psi_t, es, self.w,
                W["xas"]["delta"], self.w_in, self.w_loss, W["rixs"]["delta_in"], W["rixs"]["delta_loss"],
                W["krylov"], W["slater_weight_min"], precision, final_sector=gs_sector)
            return es, g_xas, g_rixs
        g_xas = spectra.spectra_device(self.eng, self.dop, self.restr, self.xas_dops, psi_t, es, self.w,
                                       W["xas"]["delta"], W["krylov"], W["slater_weight_min"], precision,
                                       capture=capture, perturb=perturb, batched=batched)
        g_rixs = spectra.rixs_device(self.eng, self.dop, self.restr, self.xas_dops, self.out_dops, psi_t, es,
                                     self.w_in, self.w_loss, W["rixs"]["delta_in"], W["rixs"]["delta_loss"],
                                     W["krylov"], W["slater_weight_min"], precision, timing=timing,
                                     capture=capture, perturb=perturb, batched=batched, final_sector=gs_sector)
        return es, g_xas, g_rixs

    def e2e_step(self, precision=0):
        """The same pipeline through the drop-in dict API (host inputs, host outputs).  Each
        step starts a fresh session: no sector kept by an earlier step is reused."""
        from impuritymodel_gb300 import finite, spectra

        W = WORKLOAD
        m = self.mod
        finite.clear_sector_cache()
        es, psis = finite.eigensystem(self.n, m.hOp, self.basis, W["n_psi"], precision=precision)
        ne = int(np.sum(es - es[0] < W["energy_cut_kT"] * K_B * T_KELVIN))
        es, psis = es[:ne], psis[:ne]
        g_xas = spectra.getSpectra(self.n, m.hOp, self.xas_ops_host, psis, es, self.w, W["xas"]["delta"],
                                   m.restrictions, W["krylov"], W["slater_weight_min"], precision=precision)
        g_rixs = spectra.getRIXSmap(self.n, m.hOp, self.xas_ops_host, self.out_ops_host, psis, es, self.w_in,
                                    self.w_loss, W["rixs"]["delta_in"], W["rixs"]["delta_loss"], m.restrictions,
                                    W["krylov"], W["slater_weight_min"], precision=precision)
        return es, g_xas, g_rixs


def exact_runs(cap):
    """Exact resolvents of a captured Lanczos batch: dense eigendecomposition of the sector
    H (verification only), G_r(w) = scale_r sum_k |<u_k|v0_r>|^2 / (w + i delta + e_r - l_k)."""
    import torch

    csr = cap["csr"]
    n = csr.n
    dev = csr.row_ptr.device
    rows = torch.repeat_interleave(torch.arange(n, device=dev), csr.row_ptr[1:] - csr.row_ptr[:-1])
    H = torch.zeros((n, n), dtype=torch.complex128, device=dev)
    if csr.val_c is not None:
        vals = torch.complex(csr.val_c[:, 0], csr.val_c[:, 1])
    else:
        vals = csr.val_r.to(torch.complex128)
    H[rows, csr.col.to(torch.int64)] = vals
    lam, U = torch.linalg.eigh(H)
    wgt = (U.conj().t() @ cap["v0"]).abs() ** 2  # [n, R]
    om = torch.as_tensor(cap["omega"], device=dev)
    out = torch.empty((wgt.shape[1], om.numel()), dtype=torch.complex128, device=dev)
    e = np.asarray(cap["e"])
    sc = torch.as_tensor(np.asarray(cap["scale"], dtype=np.float64), device=dev)
    for ev in np.unique(e):
        idx = torch.as_tensor(np.nonzero(e == ev)[0], device=dev)
        z = om + 1j * cap["delta"] + float(ev)
        D = 1.0 / (z[None, :] - lam[:, None].to(torch.complex128))  # [n, n_w]
        out[idx] = (wgt[:, idx].t().to(torch.complex128) @ D) * sc[idx, None]
    return out


def run_level(cap):
    return cap["g"][torch_index(cap["live"], cap["g"].device)]


def torch_index(live, dev):
    import torch

    return torch.as_tensor(live, device=dev)


def rel_l1_t(a, b):
    return float((a.imag - b.imag).abs().sum() / b.imag.abs().sum().clamp_min(1e-300))


def flush_l2(buf):
    buf.add_(1.0)


def time_steps(fn, steps, warmup, flush_buf):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush_l2(flush_buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return times, out


def hv_roofline(eng, peaks, R=16, launches=30, warmup=3, orders=("sorted", "locality")):
    """H·v on the 316-orbital model's photoemission sector (complex64, R vectors), in the
    sorted row order and in the locality order; the faster one is the roofline's launch."""
    import torch

    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions
    from impuritymodel_gb300.spectra import Sector

    mod = models.make_model("config4")
    n = mod.n_spin_orbitals
    basis = finite.get_basis(*mod.basis_args())
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    sb = finite._SortedBasis(eng, list(basis), n)
    # photoemission starts: c_i on every ground-basis state, i = first 3d spin-orbital
    ps = DeviceOp(mod.ps_ops()[0], eng.device)
    amps = torch.zeros((sb.sorted.shape[0], 2), dtype=torch.float64, device=eng.device)
    amps[:, 0] = 1.0
    (st, _), = eng.apply_vectors([sb.sorted], [amps], ps, restr, 0.0)
    t0 = time.perf_counter()
    sec = Sector(eng, dop, restr, st, precision=1)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    from impuritymodel_gb300.large import locality_order

    # the sector in its sorted order and in the locality order (bath configuration major,
    # impurity orbitals minor): the same operator with its rows and columns relabelled
    t0 = time.perf_counter()
    perm = locality_order(sec.basis, dop)
    mats = {}
    if "sorted" in orders:
        mats["sorted"] = sec.csr
    if perm is not None and "locality" in orders:
        mats["locality"] = sec.csr.permuted(perm, "locality").mixed()
    torch.cuda.synchronize()
    order_s = time.perf_counter() - t0
    g = torch.Generator(device=eng.device)
    g.manual_seed(0)
    x_sorted = torch.randn((sec.csr.n, R), dtype=torch.complex64, device=eng.device, generator=g)
    import ctypes

    from impuritymodel_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream()
    st = ctypes.c_void_p(stream.cuda_stream)

    def timed(fn, count):
        """Mean device time per launch: the launches are queued back to back between one
        pair of events, behind warm-up launches, so host launch overhead stays hidden."""
        for _ in range(warmup):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(count):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / count

    runs = {}
    for name, c in mats.items():
        x = x_sorted if name == "sorted" else x_sorted[perm].contiguous()
        y = torch.empty_like(x)
        xr, yr = torch.view_as_real(x), torch.view_as_real(y)
        # the autotuner measures every launch mapping on this matrix once (first call), then
        # the chosen one is timed
        t0 = time.perf_counter()
        mp = eng.spmv_into(c, xr, yr, R, precision=1)
        torch.cuda.synchronize()
        tune_s = time.perf_counter() - t0
        avg = timed(lambda: eng.spmv_into(c, xr, yr, R, precision=1, mapping=mp), launches)
        runs[name] = dict(csr=c, x=x, y=y, mapping=mp, avg=avg, tune_s=tune_s)
    best = min(runs, key=lambda k: runs[k]["avg"])
    csr, x, y, mapping, avg_s, tune_s = (runs[best][k] for k in ("csr", "x", "y", "mapping", "avg", "tune_s"))
    # both orders compute the same product (rows relabelled, each row's terms in one order)
    order_agree = None
    if "locality" in runs and "sorted" in runs:
        ys, yl = runs["sorted"]["y"], runs["locality"]["y"]
        order_agree = float((yl - ys[perm]).abs().max() / ys.abs().max().clamp_min(1e-30))
    xr, yr = torch.view_as_real(x), torch.view_as_real(y)

    def launch_rows():
        _lib.check(lib.edgpu_spmv_c64(ctypes.byref(csr.struct()), ctypes.c_void_p(xr.data_ptr()),
                                      ctypes.c_void_p(yr.data_ptr()), R, st), "spmv_c64")

    rows_s = timed(launch_rows, 10)
    # the same product from the row kernel: the schedule changes only the addition order
    y_rows = torch.empty_like(y)
    _lib.check(lib.edgpu_spmv_c64(ctypes.byref(csr.struct()), ctypes.c_void_p(xr.data_ptr()),
                                  ctypes.c_void_p(torch.view_as_real(y_rows).data_ptr()), R, st), "spmv_c64")
    eng.spmv_into(csr, xr, yr, R, precision=1, mapping=mapping)
    torch.cuda.synchronize()
    agree = float((y - y_rows).abs().max() / y_rows.abs().max().clamp_min(1e-30))
    val_b = 4 if csr.val_cf is None else 8
    alg = csr.nnz * (val_b + 4) + (csr.n + 1) * 8 + 2 * csr.n * R * 8
    achieved = alg / avg_s / 1e9
    # FP64 complex128 variant of the same kernel, for the plain form
    x64 = x.to(torch.complex128)
    y64 = torch.empty_like(x64)
    x64r, y64r = torch.view_as_real(x64), torch.view_as_real(y64)
    map64 = eng.spmv_into(csr, x64r, y64r, R, precision=0)
    avg64 = timed(lambda: eng.spmv_into(csr, x64r, y64r, R, precision=0, mapping=map64), 10)
    val64 = 8 if csr.val_c is None else 16
    alg64 = csr.nnz * (val64 + 4) + (csr.n + 1) * 8 + 2 * csr.n * R * 16
    del y64, y_rows
    peak = peaks.get("hbm_gbs")
    _, n_heavy = eng.spmv_plan(csr, mapping[1], mapping[2])
    return {
        "bound": "hbm",
        "kernel": {"pages": "spmv_pages_kernel<float> (edgpu_spmv_paged_c64)",
                   "tma": "spmv_pages_tma_kernel (edgpu_spmv_paged_tma_c64)"}.get(
                       mapping[0], "spmv_sched_kernel<float> (edgpu_spmv_planned_c64)"),
        "achieved": round(achieved, 1),
        "peak": peak,
        "unit": "GB/s",
        "frac": round(achieved / peak, 3) if peak else None,
        "traffic": None,
        "algorithmic_bytes_per_launch": int(alg),
        "avg_launch_us": round(avg_s * 1e6, 2),
        "launches": launches,
        "mapping": {"kernel": mapping[0], "window": mapping[1], "heavy_min": mapping[2],
                    ("slots" if mapping[0] == "tma" else "unroll"): mapping[3],
                    ("page_entries" if mapping[0] == "pages" else "block"): mapping[4], "flags": mapping[5],
                    "heavy_rows": int(n_heavy), "tune_s": round(tune_s, 3),
                    "candidates_us": get_tuner_report("spmv", eng.spmv_key(csr, R, 1))},
        "row_kernel_us": round(rows_s * 1e6, 2),
        "vs_row_kernel_max_rel": agree,
        "row_order": {"timed": best, "order_s": round(order_s, 3), "vs_sorted_max_rel": order_agree,
                      "avg_launch_us": {k: round(v["avg"] * 1e6, 2) for k, v in runs.items()},
                      "mapping": {k: list(v["mapping"]) for k, v in runs.items()},
                      "note": ("locality: rows ordered by bath configuration, impurity spin-orbitals last; "
                               "sorted: upstream's basis order")},
        "sector": {"n": int(csr.n), "nnz": int(csr.nnz), "R": R, "build_s": round(build_s, 3),
                   "model": "316 spin-orbitals, 30 bath levels, seed 3, <=2 bath holes; PS sector"},
        "fp64": {"achieved": round(alg64 / avg64 / 1e9, 1), "avg_launch_us": round(avg64 * 1e6, 2),
                 "algorithmic_bytes_per_launch": int(alg64), "mapping": list(map64)},
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
        "note": ("x (59 MB) stays in L2; every nonzero gathers one 128-byte x row from it (604 MB from L2 to the "
                 "SMs per launch)"),
    }


def get_tuner_report(kind, key, top=6):
    """The autotuner's measurements for this bucket: the fastest ``top`` mappings and the
    number of mappings timed."""
    from impuritymodel_gb300.tuner import get_tuner

    rep = get_tuner().report(kind)
    name = "%s|%s" % (kind, ",".join(str(k) for k in key))
    times = rep.get(name, {}).get("times_us") or {}
    best = sorted(times.items(), key=lambda t: t[1])[:top]
    return {"timed": len(times), "fastest_us": dict(best)}


def pruning_setup(eng, n_train=1000, n_held=200, keeps=(0.5, 0.75), epochs=10):
    """The basis-pruning network: trained on the ground-state weights of 1000 seeded models
    (seeds 1000-1999, 10-50 bath spin-orbitals), judged on 200 held-out models (seeds
    2000-2199; even seeds 50, odd seeds 100 bath spin-orbitals) by the ground-state energy on
    the best-ranked fraction of each basis, against the full basis and against keeping the
    lowest diagonal energies (the ranking without the network)."""
    import torch

    from impuritymodel_gb300 import models, pruning

    train = [models.random_model(s, 1 + s % 5) for s in range(1000, 1000 + n_train)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, lw = pruning.ground_state_samples(eng, train)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net = pruning.BasisNet(eng, seed=0, lr=2e-3)
    log = []
    n0 = eng.lib.edgpu_launch_count()
    net.train(st, lw, epochs=epochs, batch=4096, log=log)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    steps = net.t
    flop_fwd = 2.0 * (pruning.N_IN * pruning.N_H + pruning.N_H * pruning.N_H + pruning.N_H)
    rows = {"net": {}, "lowest_diagonal": {}}
    split = {}
    for s in range(2000, 2000 + n_held):
        levels = 5 if s % 2 == 0 else 10
        res, full = pruning.evaluate_pruning(eng, models.random_model(s, levels), keeps,
                                             {"net": net, "lowest_diagonal": "diagonal"})
        key = "%d_bath" % (10 * levels)
        split.setdefault(key, [0, full["n"]])[0] += 1
        for name in rows:
            for k in keeps:
                rows[name].setdefault((key, k), []).append(res[name][k]["error"])
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    held = {}
    for name, d in rows.items():
        for (key, k), errs in d.items():
            e = np.asarray(errs)
            held.setdefault(key, {}).setdefault("keep_%g" % k, {})[name] = {
                "median_error_eV": float(np.median(e)), "max_error_eV": float(e.max()),
                "within_1e-4_eV": int(np.sum(e <= 1e-4))}
    expansion = pruned_expansion_record(eng, net)
    return net, {
        "pruned_expansion": expansion,
        "train_models": n_train, "train_samples": int(st.shape[0]), "target": "log10 |<s|psi_0>|^2",
        "sample_gen_s": round(t1 - t0, 3), "epochs": epochs, "adam_steps": int(steps), "batch": 4096,
        "train_s": round(t2 - t1, 3), "train_launches": int(eng.lib.edgpu_launch_count() - n0),
        "train_loss_first_last": [round(log[0], 4), round(log[-1], 4)],
        "train_tflops": round(3.0 * flop_fwd * steps * 4096 / (t2 - t1) / 1e12, 3),
        "held_out": {k: {"models": v[0], "rows": v[1]} for k, v in split.items()}, "held_out_errors": held,
        "eval_s": round(t3 - t2, 3)}


def pruned_expansion_record(eng, net, keeps=(0.5, 0.75, 0.9), steps=3):
    """Pruning inside basis expansion on the headline model (66 spin-orbitals): the ground-state
    basis grown from the lowest configurations layer by layer, each layer's new states ranked
    by the network and only the best fraction kept; energies against the full expansion (the
    judge and fallback), then the whole pipeline (double-float form) on the pruned basis: its
    time and its XAS / RIXS distance (relative L1) to the pipeline on the full basis."""
    import torch

    from impuritymodel_gb300 import codec, pruning
    from impuritymodel_gb300.engine import make_restrictions

    pipe = Pipeline(eng)
    mod = pipe.mod
    b0 = eng.upload_states(codec.bytes_to_words(list(pruning.seed_basis(mod)), pipe.n))
    restr = make_restrictions(mod.restrictions, pipe.n)
    res, full = pruning.evaluate_expansion_pruning(eng, mod, net, keeps, n_states=WORKLOAD["n_psi"])
    full_basis, _, _ = pruning.expand_pruned(eng, pipe.dop, restr, b0)
    out = {"seed_states": int(b0.shape[0]), "full": full, "keeps": {}}
    ref = pipe.step(3, gs_basis=pruning.ExpandedBasis(full_basis))
    t_full, _ = time_steps(lambda: pipe.step(3, gs_basis=pruning.ExpandedBasis(full_basis)), steps, 2,
                           torch.zeros(1, device=eng.device))
    out["full_step_s"] = round(statistics.mean(t_full), 5)
    for keep in keeps:
        pr, _, _ = pruning.expand_pruned(eng, pipe.dop, restr, b0, net, keep)
        eb = pruning.ExpandedBasis(pr)
        got = pipe.step(3, gs_basis=eb)
        t, _ = time_steps(lambda: pipe.step(3, gs_basis=eb), steps, 2, torch.zeros(1, device=eng.device))
        rec = dict(res[keep])
        rec.update(step_s=round(statistics.mean(t), 5), states_kept=len(got[0]),
                   xas_rel_l1=rel_l1_t(got[1][: len(ref[0])], ref[1][: len(got[0])]) if len(got[0]) == len(
                       ref[0]) else None,
                   rixs_rel_l1=rel_l1_t(got[2], ref[2]) if len(got[0]) == len(ref[0]) else None)
        out["keeps"]["%g" % keep] = rec
    return out


def batched_configs(eng, n_models=256):
    """The batched workloads: an ensemble of seeded models (10-50 bath spin-orbitals) solved
    for their 3 lowest eigenstates + XAS as ragged batches, and the RIXS map of the 26-orbital
    model at 300 incoming x 2000 loss energies.  Each is timed once after a warm-up run."""
    import torch

    from impuritymodel_gb300 import ensemble, finite, models, spectra
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    out = {}
    members = [models.random_model(seed, 1 + seed % 5) for seed in range(n_models)]
    w = np.linspace(-10.0, 20.0, 2000)

    def ens_run(ms, graph):
        t0 = time.perf_counter()
        secs = [ensemble.ModelSectors(eng, m) for m in ms]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        es, psis = ensemble.ensemble_ground_states(eng, secs, 3)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        solve, run_map = ensemble.ensemble_xas_setup(eng, secs, es, psis, w, 0.2)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        if graph:
            solve.capture()
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            solve.replay()
        else:
            solve.run()
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        return dict(sectors_s=t1 - t0, gs_s=t2 - t1, xas_setup_s=t3 - t2, xas_solve_s=t4 - t3,
                    total_s=(t4 - t0)), secs, solve

    ens_run(members[:8], True)  # warm-up (module loading, graph machinery)
    n0 = eng.lib.edgpu_launch_count()
    t, secs, solve = ens_run(members, True)
    sizes = [s.csr.n for s in secs]
    xs = [int(c.n) for c in solve.batch.csrs]
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(5):
        solve.replay(check=False)
    b.record()
    torch.cuda.synchronize()
    eng.read_status("ensemble replay")
    out["ensemble_gs_xas"] = dict(
        models=n_models, bath_spin_orbitals="10 * (1 + (seed mod 5)), seeds 0..%d" % (n_models - 1), states=3,
        xas_points=int(w.size), gs_sector_rows=[min(sizes), max(sizes)], xas_sector_rows=[min(xs), max(xs)],
        xas_runs=int(solve.batch.n_runs), library_launches=int(eng.lib.edgpu_launch_count() - n0),
        graph_replay_ms=round(a.elapsed_time(b) / 5, 3), **{k: round(v, 4) for k, v in t.items()})
    # RIXS map of the 26-orbital model, 300 x 2000
    m1 = models.make_model("config1")
    n = m1.n_spin_orbitals
    dop = DeviceOp(m1.hOp, eng.device)
    restr = make_restrictions(m1.restrictions, n)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*m1.basis_args())), n)
    tin = [DeviceOp(x, eng.device) for x in m1.xas_ops()]
    tout = [DeviceOp(x, eng.device) for x in m1.rixs_out_ops()]
    w_in, w_loss = np.linspace(-10.0, 20.0, 300), np.linspace(-2.0, 12.0, 2000)
    es, psi_t = finite.eigensystem_device(eng, dop, sb, 3)
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        spectra.rixs_device(eng, dop, restr, tin, tout, psi_t, es, w_in, w_loss, 0.2, 0.05, 150, 1e-7, 3)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    out["rixs_26orb_300win"] = dict(states=len(es), w_in=int(w_in.size), w_loss=int(w_loss.size), pol_in=3,
                                    pol_out=3, form="df64_krylov_fp32_cfrac", s=round(dt, 4))
    return out


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "note": "fallback"}


def pipeline_kernel_stats(timing):
    if not timing:
        return None
    t = timing[-1]
    alg = t["nnz"] * (t["val_bytes"] + 4) + (t["n"] + 1) * 8 + 2 * t["n"] * t["R"] * t["vec_bytes"]
    avg = t["spmm_ms"] / max(t["spmm_launches"], 1) / 1e3
    kern = ("df_slices_kernel + lanczos_sliced_df_kernel (RIXS final-state Lanczos, one persistent launch; "
            "avg_launch_us is its time per Lanczos step)" if t["precision"] == 3
            else "spmm_alpha_kernel (RIXS final-state Lanczos)")
    return {"kernel": kern, "n": t["n"], "nnz": t["nnz"], "R": t["R"],
            "K": t["K"], "precision": {0: "c128", 1: "c64", 3: "df64"}.get(t["precision"], "c128"), "avg_launch_us": round(avg * 1e6, 2),
            "achieved_gbs": round(alg / avg / 1e9, 1) if avg > 0 else None,
            "note": "working set resident in L2; kernel times summed over the Lanczos call",
            "spmm_ms": round(t["spmm_ms"], 3), "axpy_ms": round(t["axpy_ms"], 3),
            "normalize_ms": round(t["normalize_ms"], 3)}


# relative start-vector perturbations of the plain FP64 runs that measure the spread of
# upstream's recurrence: FP64 rounding (1e-15) and the double-float unit (2^-48)
PERTURB_EPS = (1e-15, 2.0 ** -48)


def equal_error(pipe, forms, members=3, eps_list=PERTURB_EPS):
    """The equal-error test of every arithmetic form on the pipeline's XAS and RIXS runs.

    Each run's spectrum is compared with its exact resolvent (dense eigendecomposition of the
    sector, ``exact_runs``).  The spread of upstream's recurrence itself is measured by
    ``members`` plain FP64 runs per ``eps`` whose start vectors carry relative perturbations
    of that size: their distances to the exact resolvent and to the unperturbed plain run
    (``..._eps<k>`` keys per size; the unsuffixed keys hold all of them).  A form passes
    when its relative-L1 distance to the exact resolvent exceeds the worst plain one (plain or
    perturbed) by at most ``MIXED_L1_TOL``.  Returns (accuracy dict per spectrum kind, pass
    flag per form)."""
    caps = {name: [] for name in forms}
    for name, prec in forms.items():
        pipe.step(prec, capture=caps[name])
    caps_e = []  # (eps index, captures)
    for ke, eps in enumerate(eps_list):
        for k in range(members):
            ce = []
            pipe.step(0, capture=ce, perturb=(eps, 100 * ke + k + 1))
            caps_e.append((ke, ce))
    acc = {}
    for idx, kind in enumerate(("xas", "rixs")):
        cp = caps["plain_fp64"][idx]
        ex = exact_runs(cp)
        plain = run_level(cp)
        a = {"runs": len(cp["live"]), "sector": int(cp["csr"].n), "perturbation_eps": list(eps_list),
             "plain_ensemble_vs_exact_rel_l1": [round(rel_l1_t(run_level(ce[idx]), ex), 6) for _, ce in caps_e],
             "plain_ensemble_vs_plain_rel_l1": [round(rel_l1_t(run_level(ce[idx]), plain), 6) for _, ce in caps_e]}
        for ke in range(len(eps_list)):
            a["plain_ensemble_vs_plain_rel_l1_eps%d" % ke] = [
                round(rel_l1_t(run_level(ce[idx]), plain), 6) for kk, ce in caps_e if kk == ke]
        for name in forms:
            g = run_level(caps[name][idx])
            a[name + "_vs_exact_rel_l1"] = rel_l1_t(g, ex)
            a[name + "_vs_plain_rel_l1"] = rel_l1_t(g, plain)
        acc[kind] = a
    ok = {name: all(a[name + "_vs_exact_rel_l1"] <= max([a["plain_fp64_vs_exact_rel_l1"]] +
                                                         a["plain_ensemble_vs_exact_rel_l1"]) + MIXED_L1_TOL
                    for a in acc.values()) for name in forms}
    return acc, ok


def large_config(eng, K=150, n_states=1):
    """The 316-spin-orbital model (30 bath levels per 3d spin-orbital, seed 3, at most two
    bath holes): ground state on its 47 895-state sector, then PS (10 photoemission operators
    on 3d), XPS (6 on 2p) and XAS (3 dipole polarisations) of the lowest eigenstate, each family one batched
    reorthogonalised Lanczos (K steps) on its sector: complex64 vectors, matrix-free H·v and
    FP64 reductions, against the complex128 recurrence on the FP64 CSR Hamiltonian; the
    per-spectrum relative L1 error is reported."""
    import torch

    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions
    from impuritymodel_gb300.large import MatfreeOp, hv_diag, hv_matfree_into, spectra_large, state_hash

    mod = models.make_model("config4")
    n = mod.n_spin_orbitals
    out = {"model": "316 spin-orbitals (6 2p + 10 3d + 300 bath), seed 3, <=2 bath holes", "krylov": K,
           "states": n_states}
    # the ground state twice: the first call also pays the process's first use of these
    # shapes (the Lanczos CTA autotuner for this size, library module loading), the second is
    # the steady state; each from the model dict (basis enumeration included)
    gs_times = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        basis = finite.get_basis(*mod.basis_args())
        dop = DeviceOp(mod.hOp, eng.device)
        restr = make_restrictions(mod.restrictions, n)
        sb = finite._SortedBasis(eng, list(basis), n)
        es, psi_t = finite.eigensystem_device(eng, dop, sb, n_states, precision=3)
        torch.cuda.synchronize()
        gs_times.append(time.perf_counter() - t0)
    mop = MatfreeOp(mod.hOp, n, eng.device)
    out["gs"] = {"sector": len(basis), "s": round(gs_times[1], 3), "first_call_s": round(gs_times[0], 3),
                 "e0": float(es[0])}
    w = np.linspace(-25.0, 25.0, 2000)
    fams = {"PS": ([DeviceOp(t, eng.device) for t in mod.ps_ops()], -w, -0.2),
            "XPS": ([DeviceOp(t, eng.device) for t in mod.ps_ops(l=1)], -w, -0.2),
            "XAS": ([DeviceOp(t, eng.device) for t in mod.xas_ops()], w, 0.2)}
    for name, (tops, mesh, delta) in fams.items():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g64, info = spectra_large(eng, dop, mop, restr, tops, psi_t, es, mesh, delta, K=K, precision=1, matfree=True)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        sector = info.pop("sector_obj")
        # the complex64 CSR form twice: the first call also runs the H.v autotuner for this
        # shape (timed apart), the second is the steady state
        t64c_first = None
        for _ in range(2):
            t0 = time.perf_counter()
            g64c, _ = spectra_large(eng, dop, mop, restr, tops, psi_t, es, mesh, delta, K=K, precision=1,
                                    matfree=False, sector=sector)
            torch.cuda.synchronize()
            t64c = time.perf_counter() - t0
            t64c_first = t64c if t64c_first is None else t64c_first
        t0 = time.perf_counter()
        g128, _ = spectra_large(eng, dop, mop, restr, tops, psi_t, es, mesh, delta, K=K, precision=0, sector=sector)
        torch.cuda.synchronize()
        t128 = time.perf_counter() - t0
        errs, errs_c = [], []
        for i in range(g128.shape[0]):
            for o in range(g128.shape[1]):
                ref = g128[i, o].imag
                if np.abs(ref).sum() > 0:
                    errs.append(float(np.abs(g64[i, o].imag - ref).sum() / np.abs(ref).sum()))
                    errs_c.append(float(np.abs(g64c[i, o].imag - ref).sum() / np.abs(ref).sum()))
        # matrix-free H.v on this sector, R = the family's runs padded to a width the kernel
        # serves (as the recurrence does), complex64
        R = 2
        while R < info["runs"]:
            R *= 2
        d = hv_diag(eng, sector.basis, mop)
        table = state_hash(eng, sector.basis)
        x = torch.randn((sector.n, R), dtype=torch.complex64, device=eng.device)
        y = torch.empty_like(x)
        hv_matfree_into(eng, sector.basis, mop, restr, d, x, y, 0.0, table)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(5):
            hv_matfree_into(eng, sector.basis, mop, restr, d, x, y, 0.0, table)
        b.record()
        torch.cuda.synchronize()
        hv_us = a.elapsed_time(b) * 1e3 / 5
        out[name] = {"sector": info["sector"], "runs": info["runs"], "hv_width": R, "k_len_min": min(info["k_len"]),
                     "sector_build_s": round(info["sector_s"], 3), "dgks_second_passes": info["second_passes"],
                     "c64_matfree_s": round(t64 - info["sector_s"], 3), "c64_csr_s": round(t64c, 3),
                     "c64_csr_first_call_s": round(t64c_first, 3),
                     "c128_csr_s": round(t128, 3),
                     "rel_l1_vs_c128": {"max": max(errs), "median": float(np.median(errs))},
                     "csr_rel_l1_vs_c128": {"max": max(errs_c), "median": float(np.median(errs_c))},
                     "matfree_hv_us": round(hv_us, 1), "csr_nnz": int(sector.csr.nnz)}
        del sector, g64, g64c, g128
        torch.cuda.empty_cache()
    return out


def krylov_roofline(eng, peaks, n=462120, R=16, K=150, ms=(1, 16, 75, 150), precision=1, reps=5):
    """The large-sector Krylov kernels (edgpu_krylov_dot / _project / _normalize) on random
    complex64 (or complex128) vectors of the 316-orbital PS sector's shape: n rows, R runs, a
    basis of K vectors; per m (vectors in the pass) the mean CUDA-event time of back-to-back
    calls and the algorithmic bytes over it (dot: m + 1 vectors read; projection: m read, w
    read and written; normalisation: w read, v written), against the measured HBM copy peak."""
    import ctypes as C

    import torch

    from impuritymodel_gb300 import _lib as L
    from impuritymodel_gb300.engine import _ptr

    lib = eng.lib
    dt = torch.complex64 if precision else torch.complex128
    esz = 8 if precision else 16
    g = torch.Generator(device=eng.device).manual_seed(0)
    V = torch.randn((K, n, R), dtype=dt, device=eng.device, generator=g)
    w = torch.randn((n, R), dtype=dt, device=eng.device, generator=g)
    h = torch.zeros((K, R), dtype=torch.complex128, device=eng.device)
    beta = torch.zeros(R, dtype=torch.float64, device=eng.device)
    out = torch.empty_like(w)
    wsn = lib.edgpu_krylov_workspace(n, R, K)
    ws = torch.empty(wsn, dtype=torch.uint8, device=eng.device)
    wsp = C.c_void_p(ws.data_ptr())
    Vp, wp, hp = _ptr(torch.view_as_real(V)), _ptr(torch.view_as_real(w)), _ptr(torch.view_as_real(h))
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(3):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps * 1e3

    peak = peaks.get("hbm_gbs")
    vb = n * R * esz
    res = {}
    for m in ms:
        d = timed(lambda: L.check(lib.edgpu_krylov_dot(precision, Vp, n * R, m, n, R, wp, hp, wsp, wsn, eng.stream),
                                  "krylov_dot"))
        p = timed(lambda: L.check(lib.edgpu_krylov_project(precision, Vp, n * R, m, n, R, hp, wp, 1, wsp, wsn,
                                                           eng.stream), "krylov_project"))
        z = timed(lambda: L.check(lib.edgpu_krylov_normalize(precision, n, R, wp, _ptr(torch.view_as_real(out)),
                                                             _ptr(beta), _ptr(eng.status), wsp, wsn, eng.stream),
                                  "krylov_normalize"))
        row = {}
        for name, us, nbytes in (("dot", d, (m + 1) * vb), ("project", p, (m + 2) * vb), ("normalize", z, 2 * vb)):
            gbs = nbytes / us / 1e3
            row[name] = {"us": round(us, 1), "gbs": round(gbs, 1), "frac": round(gbs / peak, 3) if peak else None}
        res[str(m)] = row
    del V
    torch.cuda.empty_cache()
    return {"n": n, "R": R, "K": K, "dtype": "c64" if precision else "c128", "by_m": res,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}


def sector_build_timing(eng, reps=2):
    """Expansion and CSR of the 316-spin-orbital model's photoemission sector (462 120 states
    from the c_i images of its 47 895-state ground basis): wall time of each, device
    synchronised, the second of ``reps`` builds reported (the first also loads modules)."""
    import torch

    from impuritymodel_gb300 import finite, models
    from impuritymodel_gb300.engine import DeviceOp, make_restrictions

    mod = models.make_model("config4")
    n = mod.n_spin_orbitals
    dop = DeviceOp(mod.hOp, eng.device)
    restr = make_restrictions(mod.restrictions, n)
    sb = finite._SortedBasis(eng, list(finite.get_basis(*mod.basis_args())), n)
    ps = DeviceOp(mod.ps_ops()[0], eng.device)
    amps = torch.zeros((sb.sorted.shape[0], 2), dtype=torch.float64, device=eng.device)
    amps[:, 0] = 1.0
    (st, _), = eng.apply_vectors([sb.sorted], [amps], ps, restr, 0.0)
    out = {}
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        basis, _ = eng.expand(eng.sort_unique(st), dop, restr)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        csr = eng.build_csr(basis, dop, restr)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out = {"states": int(basis.shape[0]), "nnz": int(csr.nnz), "expand_s": round(t1 - t0, 4),
               "csr_s": round(t2 - t1, 4), "terms": int(dop.n_terms)}
    return out


def gemm_timing(eng, peaks, batch=4096, wide=65536, reps=20):
    """The tcgen05 GEMMs of the basis-pruning network: the five of one training step at batch
    ``batch`` (forward layers 1 and 2 with the bias + ReLU epilogue, the weight gradients dW2
    and dW1 with K = batch, the ReLU-mask backward dH1) and the first forward layer on
    ``wide`` rows (ranking a large candidate set); per GEMM the mean CUDA-event time of
    back-to-back calls and 2 M N K flops over it, against the measured bf16 burst peak (the
    operands, a few MB, stay in L2); and one whole training step (gradients + Adam)."""
    import numpy as np
    import torch

    from impuritymodel_gb300 import pruning
    from impuritymodel_gb300.engine import _ptr

    dev = eng.device
    g = torch.Generator(device=dev).manual_seed(0)
    net = pruning.BasisNet(eng, seed=0)
    B = batch
    bf = torch.bfloat16
    X = (torch.rand((B, pruning.N_IN), device=dev, generator=g) < 0.2).to(bf)
    Xt = X.t().contiguous()
    H1, H2, dH2, dH1 = (torch.rand((B, pruning.N_H), device=dev, generator=g).to(bf) for _ in range(4))
    H1t, dH2t, dH1t = (torch.rand((pruning.N_H, B), device=dev, generator=g).to(bf) for _ in range(3))
    Yt = torch.empty((pruning.N_H, B), dtype=bf, device=dev)
    Xw = (torch.rand((wide, pruning.N_IN), device=dev, generator=g) < 0.2).to(bf)
    Yw = torch.empty((wide, pruning.N_H), dtype=bf, device=dev)
    Y = torch.empty((B, pruning.N_H), dtype=bf, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(3):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps * 1e3

    nh, ni = pruning.N_H, pruning.N_IN
    cases = [
        ("forward1", (B, nh, ni), lambda: net._gemm(1, X, net.W1b, B, nh, ni, bias=net.p["b1"], Y=Y, Yt=Yt)),
        ("forward2", (B, nh, nh), lambda: net._gemm(1, H1, net.W2b, B, nh, nh, bias=net.p["b2"], Y=Y, Yt=Yt)),
        ("dW2", (nh, nh, B), lambda: net._gemm(0, dH2t, H1t, nh, nh, B, C=net.g["W2"])),
        ("dH1", (B, nh, nh), lambda: net._gemm(2, dH2, net.W2t, B, nh, nh, mask=H1, Y=dH1, Yt=Yt)),
        ("dW1", (nh, ni, B), lambda: net._gemm(0, dH1t, Xt, nh, ni, B, C=net.g["W1"])),
        ("forward1_wide", (wide, nh, ni), lambda: net._gemm(1, Xw, net.W1b, wide, nh, ni, bias=net.p["b1"], Y=Yw)),
    ]
    peak = peaks.get("bf16_tflops")
    out = {}
    for name, (M, N, K), fn in cases:
        us = timed(fn)
        tf = 2.0 * M * N * K / us / 1e6
        bn = int(eng.lib.edgpu_gemm_tile_width(M, N))
        out[name] = {"M": M, "N": N, "K": K, "tile": [128, bn], "ctas": (M // 128) * (N // bn), "us": round(us, 2),
                     "tflops": round(tf, 2), "frac": round(tf / peak, 4) if peak else None}
    target = torch.randn(B, device=dev, generator=g)

    def train_step():
        net.gradients(X, Xt, target)
        net.adam_step()

    step_us = timed(train_step)
    eng.read_status("gemm timing")
    flops = 2.0 * B * (nh * ni + nh * nh) * 3
    return {"gemms": out, "train_step_us": round(step_us, 1),
            "train_tflops": round(flops / step_us / 1e6, 2), "batch": B,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst, of measured)", "inputs": "L2-resident"}


def run_gemm_only(args):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps({"gemm": gemm_timing(get_engine(), read_peaks())}))


def run_sector_only(args):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps({"sector_build": sector_build_timing(get_engine())}))


def run_krylov_only(args):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ms = tuple(int(x) for x in args.krylov_m.split(","))
    print(json.dumps({"krylov_kernels": krylov_roofline(get_engine(), read_peaks(), K=args.krylov_k, ms=ms)}))


def run_large_only():
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    eng = get_engine()
    out = large_config(eng)
    out["krylov_kernels"] = krylov_roofline(eng, read_peaks())
    print(json.dumps({"large_316orb": out}))


def run_gpu(args):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300 import _lib
    from impuritymodel_gb300.engine import get_engine

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    eng = get_engine()
    lib = _lib.load()
    pipe = Pipeline(eng)
    flush_buf = torch.zeros(256 * 1024 * 1024 // 4, dtype=torch.float32, device=eng.device)
    peaks = read_peaks()

    # accuracy against exact resolvents (untimed): plain form, an ensemble of plain runs
    # with 1e-15 start-vector perturbations (the spread of upstream's recurrence), and the
    # faster forms
    forms = dict(FORMS)
    acc, ok = equal_error(pipe, forms)

    # time every form; the headline is the fastest form that keeps the error
    form_times = {}
    outs = {}
    for name, prec in forms.items():
        if name == "plain_fp64":
            continue
        t, o = time_steps(lambda p=prec: pipe.step(p), max(1, args.steps // 2), args.warmup, flush_buf)
        form_times[name] = statistics.mean(t)
        outs[name] = o
    plain_times, plain_out = time_steps(lambda: pipe.step(0), max(1, args.steps // 2), args.warmup, flush_buf)
    form_times["plain_fp64"] = statistics.mean(plain_times)
    # upstream's call structure on the GPU (one Green's function / one shifted solve per
    # launch, FP64): the reference point of the batched forms
    unb_times, unb_out = time_steps(lambda: pipe.step(0, batched=False), 1, 1, flush_buf)
    t_unbatched = statistics.mean(unb_times)
    unb_err = {k: rel_l1_t(a, b) for k, a, b in (("xas", unb_out[1], plain_out[1]), ("rixs", unb_out[2], plain_out[2]))}
    best_name = min((n for n in forms if ok[n]), key=lambda n: form_times[n])
    best_prec = forms[best_name]
    # production form: timed region for `value`, clocks and launch counts
    timing = []
    clocks = ClockSampler(local)
    for _ in range(args.warmup):
        pipe.step(best_prec)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    n0 = lib.edgpu_launch_count()
    best_times, best_out = time_steps(lambda: pipe.step(best_prec), args.steps, 0, flush_buf)
    launches = lib.edgpu_launch_count() - n0
    clk = clocks.stop()
    pipe.step(best_prec, timing)  # kernel times of the Lanczos calls (untimed step)
    es_p = plain_out[0]
    es_b = best_out[0]
    err = {"gs_energy_max_abs_eV": float(np.abs(es_b - es_p).max()), "vs_exact": acc, "forms_pass": ok,
           "form_s": {k: round(v, 5) for k, v in form_times.items()},
           # the headline form's distance to plain FP64 beside the spread of plain FP64 itself
           # under 1e-15 start-vector perturbations (upstream's recurrence amplifies rounding)
           "headline_vs_plain_rel_l1": {k: dict({"headline": round(a[best_name + "_vs_plain_rel_l1"], 6)},
                                                **{"plain_perturbed_%g_max" % e: max(
                                                    a["plain_ensemble_vs_plain_rel_l1_eps%d" % ke])
                                                   for ke, e in enumerate(a["perturbation_eps"])})
                                        for k, a in acc.items()}}
    t_plain = form_times["plain_fp64"]
    best = statistics.mean(best_times)
    # end to end through the dict API
    for _ in range(1):
        pipe.e2e_step(best_prec)
    torch.cuda.synchronize()
    eng.h2d_bytes = eng.d2h_bytes = 0
    e2e_times = []
    for _ in range(max(1, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pipe.e2e_step(best_prec)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    h2d = eng.h2d_bytes // len(e2e_times)
    d2h = eng.d2h_bytes // len(e2e_times)
    # times: max over ranks
    if world > 1:
        t = torch.tensor([best, statistics.mean(e2e_times)], dtype=torch.float64, device=eng.device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        best, e2e_t = float(t[0]), float(t[1])
    else:
        e2e_t = statistics.mean(e2e_times)
    roof = hv_roofline(eng, peaks) if rank == 0 else None
    if roof is not None:
        roof["traffic"] = traffic_scaled(roof)
        roof["traffic_source"] = "ncu DRAM bytes of this kernel on this sector, as a ratio, scaled to this launch"
    batched = batched_configs(eng) if (rank == 0 and not args.skip_batched) else None
    prune_info = pruning_setup(eng)[1] if (rank == 0 and not args.skip_batched) else None
    if prune_info is not None:
        prune_info["gemm_kernels"] = gemm_timing(eng, peaks)
    large = large_config(eng) if (rank == 0 and not args.skip_batched) else None
    if large is not None:
        large["krylov_kernels"] = krylov_roofline(eng, peaks)
    cpu = cpu_baseline() if (rank == 0 and not args.skip_cpu) else None
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(best, 5),
            "unit": "s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(best * 1e3, 3),
            "higher_is_better": False,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": FORM_DTYPES[best_name],
            "data": "synthetic seeded model (numpy default_rng), no dataset",
            "config": dict(WORKLOAD, form=best_name, l2="flushed between steps",
                           parallelism="replicas" if world > 1 else "single GPU"),
            "plain_fp64_s": round(t_plain, 5),
            "speedup_vs_plain": round(t_plain / best, 3),
            "plain_fp64_unbatched_s": round(t_unbatched, 4),
            "speedup_vs_plain_unbatched": round(t_unbatched / best, 1),
            "unbatched_vs_plain_rel_l1": unb_err,
            "forms": err,
            "e2e": {"value": round(e2e_t, 5), "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clk,
            "roofline": roof,
            "pipeline_kernel": pipeline_kernel_stats(timing),
            "cpu_baseline": cpu,
            "batched": batched,
            "basis_pruning": prune_info,
            "large_316orb": large,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_hv_only(args):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    orders = ("sorted", "locality") if args.hv_order == "both" else (args.hv_order,)
    roof = hv_roofline(get_engine(), read_peaks(), launches=5, warmup=3, orders=orders)
    roof["traffic"] = traffic_scaled(roof)
    print(json.dumps({"roofline": roof}))


def run_profile_step(args):
    """One pipeline step of the chosen form inside NVTX range 'pipeline_step' (for ncu)."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from impuritymodel_gb300 import _lib
    from impuritymodel_gb300.engine import get_engine

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    eng = get_engine()
    lib = _lib.load()
    pipe = Pipeline(eng)
    prec = FORMS[args.form]
    for _ in range(args.warmup):
        pipe.step(prec)
    torch.cuda.synchronize()
    n0 = lib.edgpu_launch_count()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("pipeline_step")
    pipe.step(prec)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    dt = time.perf_counter() - t0
    print(json.dumps({"form": args.form, "step_s": round(dt, 5), "library_launches": lib.edgpu_launch_count() - n0}))


# DRAM bytes (read + write) per launch of the H.v kernel over its algorithmic bytes, from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernel on the same
# 462 120-state sector in each row order; the bench line scales it to the launch it times.
HV_DRAM_OVER_ALGORITHMIC = {"sorted": 1.095, "locality": None}


def traffic_scaled(roof):
    ratio = HV_DRAM_OVER_ALGORITHMIC.get(roof.get("row_order", {}).get("timed", "sorted"))
    return int(ratio * roof["algorithmic_bytes_per_launch"]) if ratio else None


# ---------------------------------------------------------------------------------------
# CPU reference (oracle port of upstream): whole pipeline steps, timed end to end
# ---------------------------------------------------------------------------------------


def ref_meshes(work):
    x, r = work["xas"], work["rixs"]
    return (np.linspace(x["w"][0], x["w"][1], x["n_w"]), np.linspace(r["w_in"][0], r["w_in"][1], r["n_w_in"]),
            np.linspace(r["w_loss"][0], r["w_loss"][1], r["n_w_loss"]))


def ref_ground_state(O, mod, work):
    """Upstream's eigensystem (finite.py:58-118, ARPACK) on the restricted basis, then the
    eigenstates within ``energy_cut_kT`` of the lowest."""
    n = mod.n_spin_orbitals
    basis = O.get_basis(*mod.basis_args())
    es, psis = O.eigensystem(n, mod.hOp, basis, work["n_psi"])
    ne = int(np.sum(es - es[0] < work["energy_cut_kT"] * K_B * T_KELVIN))
    return np.asarray(es[:ne]), list(psis[:ne])


def ref_share(O, mod, es, psis, rank, procs, work):
    """One process's share of a step's spectra, as upstream's parallel modes divide them
    (getSpectra ``eigen_states``, spectra.py:746-777; getRIXSmap ``wIn``, spectra.py:1012-1129):

    * XAS Green's functions (operator t, eigenstate i), run k = t * n_states + i, for
      k % procs == rank: T psi, normalisation, getGreen on the closure (spectra.py:684-806);
    * RIXS: unit u = (setup, iw), setup = (t_in, eigenstate), goes to process u % procs;
      a process builds the core-hole sector of every setup it has units of, then per unit: BiCGSTAB (rtol 1e-5) at w_in, then for each
      outgoing operator T_out psi2 (one memo shared by the outgoing operators, as upstream's
      ``tOut_big = [{}] * n``), normalisation, pruning and getGreen (spectra.py:809-1130).

    Memos are fresh for every call (upstream builds them per getSpectra / getRIXSmap call).
    Returns ({(i, t): g}, {(t_in, i, iw): [n_out, n_loss]})."""
    import scipy.sparse
    import scipy.sparse.linalg

    n = mod.n_spin_orbitals
    w, w_in, w_loss = ref_meshes(work)
    ne = len(es)
    swm = work["slater_weight_min"]
    restr = mod.restrictions
    tins, touts = mod.xas_ops(), mod.rixs_out_ops()
    xas = {}
    memo_x = O._ColumnMemo(n, mod.hOp, restr)
    for k in range(rank, len(tins) * ne, procs):
        t, i = divmod(k, ne)
        pr = O.apply_op(n, tins[t], psis[i], swm, restr)
        nrm = np.sqrt(O.norm2(pr))
        pr = {s_: a / nrm for s_, a in pr.items()}
        xas[(i, t)] = nrm ** 2 * O.get_green(n, es[i], pr, mod.hOp, w, work["xas"]["delta"], work["krylov"], swm,
                                            restr, memo=memo_x)
    rixs = {}
    memo_exc = O._ColumnMemo(n, mod.hOp, restr)
    memo_gnd = O._ColumnMemo(n, mod.hOp, restr)
    shared_out = {}
    d_in, d_loss = work["rixs"]["delta_in"], work["rixs"]["delta_loss"]
    for t_in, top in enumerate(tins):
        t_in_big = {}
        for i in range(ne):
            # unit u = (setup, iw) goes to process u % procs: balanced over all setups
            u0 = (t_in * ne + i) * len(w_in)
            my_w = [iw for iw in range(len(w_in)) if (u0 + iw) % procs == rank]
            psi1 = O.apply_op(n, top, psis[i], swm, restr, t_in_big)
            if not my_w or not psi1:
                continue
            h, idx = O.expand_basis_and_hamiltonian(n, None, mod.hOp, list(psi1.keys()), restr, memo=memo_exc)
            m = len(idx)
            y = np.zeros(m, dtype=complex)
            for s_, a in psi1.items():
                y[idx[s_]] = a
            basis_state = {k: s_ for s_, k in idx.items()}
            for iw in my_w:
                a = scipy.sparse.csr_matrix(([w_in[iw] + 1j * d_in + es[i]] * m, (range(m), range(m))),
                                            shape=h.shape) - h
                x, _ = scipy.sparse.linalg.bicgstab(a, y, rtol=1e-5)
                psi2 = {basis_state[q]: amp for q, amp in enumerate(x) if amp != 0}
                out = np.zeros((len(touts), len(w_loss)), dtype=complex)
                for t_out, tout in enumerate(touts):
                    psi3 = O.apply_op(n, tout, psi2, swm, restr, shared_out)
                    nrm = np.sqrt(O.norm2(psi3))
                    psi3 = {s_: a_ / nrm for s_, a_ in psi3.items()}
                    psi3 = {s_: a_ for s_, a_ in psi3.items() if abs(a_) ** 2 >= swm}
                    out[t_out] = nrm ** 2 * O.get_green(n, es[i], psi3, mod.hOp, w_loss, d_loss, work["krylov"], swm,
                                                        restr, memo=memo_gnd)
                rixs[(t_in, i, iw)] = out
    return xas, rixs


_REF_WORKER = None


def _ref_worker_init(work):
    """Pool initialiser (spawned process, no CUDA state): the oracle module and the model
    (operator dicts), the inputs a caller of upstream holds before its first call."""
    global _REF_WORKER
    import oracle.ed_oracle as O

    from impuritymodel_gb300 import models

    _REF_WORKER = (O, models.make_model("config2"), work)


def _ref_worker_share(args):
    es, psis, rank, procs = args
    O, mod, work = _REF_WORKER
    return ref_share(O, mod, es, psis, rank, procs, work)


def ref_step(O, mod, work, pool=None, procs=1):
    """One whole step of upstream's algorithm: ground state (serial), then the XAS and RIXS
    work divided among ``procs`` processes (or run in this process when ``pool`` is None),
    and the spectra gathered into upstream's arrays gs_xas [n_states, 3, n_w] and
    gs_rixs [n_states, 3, 3, n_w_in, n_w_loss].  Returns (es, gs_xas, gs_rixs, parts_s)."""
    t0 = time.perf_counter()
    es, psis = ref_ground_state(O, mod, work)
    t1 = time.perf_counter()
    if pool is None:
        shares = [ref_share(O, mod, es, psis, 0, 1, work)]
    else:
        shares = pool.map(_ref_worker_share, [(es, psis, r, procs) for r in range(procs)])
    w, w_in, w_loss = ref_meshes(work)
    ne = len(es)
    gx = np.zeros((ne, 3, len(w)), dtype=complex)
    gr = np.zeros((ne, 3, 3, len(w_in), len(w_loss)), dtype=complex)
    for xas, rixs in shares:
        for (i, t), g in xas.items():
            gx[i, t] = g
        for (t_in, i, iw), g in rixs.items():
            gr[i, t_in, :, iw] = g
    t2 = time.perf_counter()
    return es, gx, gr, {"gs_s": t1 - t0, "spectra_s": t2 - t1}


def cpu_baseline(work=None):
    """The oracle port of upstream on one host core: one whole step, timed end to end."""
    import oracle.ed_oracle as O

    from impuritymodel_gb300 import models

    work = work or WORKLOAD
    mod = models.make_model("config2")
    t0 = time.perf_counter()
    _, _, gr, parts = ref_step(O, mod, work)
    total = time.perf_counter() - t0
    r = work["rixs"]
    sample = ("one whole step of upstream's algorithm (NumPy/SciPy oracle port) on 1 core: ground state, "
              "%d XAS Green's functions, %d RIXS (t_in, state, w_in) units with %d outgoing Green's functions each"
              % (3 * gr.shape[0], 3 * gr.shape[0] * r["n_w_in"], r["pol_out"]))
    return {"value": round(total, 3), "unit": "s", "cores": 1, "kind": "port", "sample": sample, "steps": 1,
            "parts_s": {k: round(v, 3) for k, v in parts.items()}}


def reference_steps(steps, warmup, procs, work=None):
    """Whole steps of upstream's algorithm on ``procs`` spawned oracle processes; returns the
    wall time of each timed step (the warm-up steps are run and discarded)."""
    import multiprocessing

    import oracle.ed_oracle as O

    from impuritymodel_gb300 import models

    work = work or WORKLOAD
    mod = models.make_model("config2")
    times = []
    with multiprocessing.get_context("spawn").Pool(procs, initializer=_ref_worker_init, initargs=(work,)) as pool:
        for k in range(warmup + steps):
            t0 = time.perf_counter()
            ref_step(O, mod, work, pool=pool, procs=procs)
            dt = time.perf_counter() - t0
            if k >= warmup:
                times.append(dt)
    return times


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # every host core: one oracle process each (spawned: no CUDA state is inherited)
    procs = max(1, os.cpu_count() or 1)
    t0 = time.perf_counter()
    times = reference_steps(args.steps, args.warmup, procs)
    wall = time.perf_counter() - t0
    value = statistics.mean(times)
    sample = ("whole steps of upstream's algorithm (NumPy/SciPy oracle port): ground state serial, then the XAS "
              "runs and the RIXS incoming energies divided among %d processes (upstream's eigen_states / wIn "
              "modes), spectra gathered; wall clock per step" % procs)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(value * 1e3, 1),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic seeded model (numpy default_rng), no dataset",
        "config": dict(WORKLOAD, form="upstream algorithm (NumPy/SciPy oracle port)"),
        "step_s": {"min": round(min(times), 4), "max": round(max(times), 4)},
        "timed_region_s": round(sum(times), 3),
        "run_s": round(wall, 3),
        "cpu_baseline": {"value": round(value, 4), "unit": "s", "cores": procs, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batched", action="store_true", help="skip the ensemble / 300-w_in RIXS lines")
    ap.add_argument("--large-only", action="store_true", help="only the 316-spin-orbital large-sector line")
    ap.add_argument("--hv-only", action="store_true",
                    help="only the H.v roofline measurement (the case profiled under ncu)")
    ap.add_argument("--sector-only", action="store_true",
                    help="only the 316-orbital PS sector construction (the case profiled under ncu)")
    ap.add_argument("--krylov-only", action="store_true",
                    help="only the large-sector Krylov kernel timings (the case profiled under ncu)")
    ap.add_argument("--gemm-only", action="store_true",
                    help="only the tensor-core GEMM timings of the pruning network (the case profiled under ncu)")
    ap.add_argument("--krylov-k", type=int, default=150, help="basis vectors held by --krylov-only")
    ap.add_argument("--krylov-m", default="1,16,75,150", help="vectors per pass timed by --krylov-only")
    ap.add_argument("--hv-order", choices=["both", "sorted", "locality"], default="both",
                    help="row orders of the sector timed by --hv-only")
    ap.add_argument("--profile-step", action="store_true",
                    help="warm up, then run one pipeline step inside the NVTX range 'pipeline_step'")
    ap.add_argument("--form", choices=list(FORMS),
                    default="df64_krylov_fp32_cfrac", help="form used by --profile-step")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.hv_only:
        run_hv_only(args)
    elif args.krylov_only:
        run_krylov_only(args)
    elif args.sector_only:
        run_sector_only(args)
    elif args.gemm_only:
        run_gemm_only(args)
    elif args.large_only:
        run_large_only()
    elif args.profile_step:
        run_profile_step(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
