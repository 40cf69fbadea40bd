"""Autotuner for grouped contractions.

For each shape class of a group (members that share a plan signature) it
times the candidate schedules - arithmetic form (the emulated form of the
element type, or the native one; both meet the precision target) and the
rasterisation band of the tensor-core kernel - on the group's own data, keeps
the fastest, and caches the decision in a JSON file keyed by device name,
element type and shape. Later groups with the same classes reuse the cached
choice without timing.
"""
from __future__ import annotations

import json
import os
import threading

import torch

from .grouped import Group

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "muscle_gb300", "autotune.json")
BANDS = (1, 2, 4)  # 2, 3, 8 row tiles per band


def _class_key(c, a, b) -> str:
    dev = torch.cuda.get_device_name(c.data.device)
    sig = lambda t: f"{tuple(t.data.shape)}:{tuple(t.data.stride())}:{[str(i.tag) for i in t.inds]}"
    return f"{dev}|{a.dtype}x{b.dtype}|{sig(a)}|{sig(b)}|{sig(c)}"


class Autotuner:
    def __init__(self, cache_path: str | None = None, reps: int = 3):
        self.path = cache_path or os.environ.get("MUSCLE_GB300_AUTOTUNE", DEFAULT_CACHE)
        self.reps = reps
        self.lock = threading.Lock()
        self.cache = {}
        if os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.cache = json.load(f)
            except (OSError, ValueError):
                self.cache = {}

    def _save(self):
        os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    @staticmethod
    def candidates(dtype):
        emulated = "ozaki" if dtype in (torch.float64, torch.complex128) else "bf16x3"
        return [(emulated, band) for band in BANDS] + [("plain", 0)]

    def _time(self, items, form, band) -> float:
        g = Group(items, form, bands=[band] * len(items))
        g.execute()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(self.reps):
            g.execute()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / self.reps

    def tune(self, items):
        """Returns (forms, bands) per item, timing classes not yet cached."""
        classes = {}
        for idx, (c, a, b) in enumerate(items):
            classes.setdefault(_class_key(c, a, b), []).append(idx)
        changed = False
        for key, idxs in classes.items():
            with self.lock:
                if key in self.cache:
                    continue
            sub = [items[i] for i in idxs]
            dt = torch.promote_types(sub[0][1].dtype, sub[0][2].dtype)
            best = None
            for form, band in self.candidates(dt):
                ms = self._time(sub, form, band)
                if best is None or ms < best[2]:
                    best = (form, band, ms)
            with self.lock:
                self.cache[key] = {"form": best[0], "band": best[1], "ms": best[2], "members": len(idxs)}
            changed = True
        if changed:
            with self.lock:
                self._save()
        forms, bands = [None] * len(items), [0] * len(items)
        for key, idxs in classes.items():
            d = self.cache[key]
            for i in idxs:
                forms[i] = d["form"]
                bands[i] = d["band"]
        return forms, bands

    def group(self, items) -> Group:
        forms, bands = self.tune(items)
        return Group(items, forms, bands=bands)
