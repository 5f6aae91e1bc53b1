"""Autotuner for the launch mappings of the engine's kernels.

A kernel with several correct launch mappings (threads per block, gathers in flight, row
schedules, runs per CTA ...) registers a *kind*; for a shape *bucket* (sizes rounded to a
power of two, so nearby problems share one measurement) the tuner times every candidate on
the caller's own data with CUDA events on the current stream, keeps the fastest, and
returns it for every later call in the same bucket.  The table of measurements is kept in
memory and, when ``EDGPU_TUNE_CACHE`` names a JSON file, reloaded from and saved to it, so a
later process skips the timing.  Every candidate must compute the same result (the tuner
only chooses how the work is laid out), which the engine's tests check per kind.
"""

from __future__ import annotations

import json
import math
import os
import threading

import torch


def bucket(x):
    """Power-of-two bucket of a positive size (0 stays 0)."""
    x = int(x)
    return 0 if x <= 0 else 1 << int(math.ceil(math.log2(x)))


class Autotuner:
    def __init__(self, path=None):
        self.path = path if path is not None else os.environ.get("EDGPU_TUNE_CACHE")
        self._lock = threading.Lock()
        self.table = {}  # "kind|key" -> {"best": candidate, "times_us": {candidate: us}}
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as fh:
                    self.table = json.load(fh)
            except (OSError, ValueError):
                self.table = {}

    @staticmethod
    def _name(kind, key):
        return "%s|%s" % (kind, ",".join(str(k) for k in key))

    def lookup(self, kind, key):
        hit = self.table.get(self._name(kind, key))
        return None if hit is None else tuple(hit["best"])

    def pick(self, kind, key, candidates, run, reps=5, warmup=2):
        """The fastest of ``candidates`` (tuples) for this kind and bucket key.

        ``run(candidate)`` enqueues one launch of the kernel with that mapping on the current
        stream.  Measured once per (kind, key); later calls return the cached choice."""
        name = self._name(kind, key)
        hit = self.table.get(name)
        if hit is not None:
            return tuple(hit["best"])
        times = {}
        stream = torch.cuda.current_stream()
        for cand in candidates:
            for _ in range(warmup):
                run(cand)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                run(cand)
            b.record(stream)
            b.synchronize()
            times[cand] = a.elapsed_time(b) * 1e3 / reps
        best = min(times, key=times.get)
        with self._lock:
            self.table[name] = {"best": list(best),
                                "times_us": {",".join(str(c) for c in k): round(v, 2) for k, v in times.items()}}
            self._save()
        return best

    def _save(self):
        if not self.path:
            return
        tmp = self.path + ".tmp"
        try:
            with open(tmp, "w") as fh:
                json.dump(self.table, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass

    def report(self, kind=None):
        """The measurements so far (optionally of one kind), for logs and the bench line."""
        return {k: v for k, v in self.table.items() if kind is None or k.startswith(kind + "|")}


_TUNER = None


def get_tuner():
    global _TUNER
    if _TUNER is None:
        _TUNER = Autotuner()
    return _TUNER
