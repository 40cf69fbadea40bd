"""Autotuner for grouped contractions.

Two decisions, each timed on the group's own data and cached in a JSON file
keyed by device name, element types and shapes (later groups with the same
classes reuse the cached choice without timing):
  * per shape class (members that share a plan signature): the arithmetic
    form (the emulated form of the element type, or the native one; both
    meet the precision target) and the rasterisation band of the
    tensor-core kernel;
  * per group: the schedule of the whole group as a CUDA graph - one
    persistent tensor-core launch per kernel variant after every pre-pass,
    or every bucket's own launches, on 1, 4 or 8 parallel branches.
"""
from __future__ import annotations

import hashlib
import json
import os
import threading

import torch

from .grouped import Group

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "muscle_gb300", "autotune.json")
BANDS = (1, 2, 4)  # 2, 3, 8 row tiles per band
# (parallel graph branches, one persistent launch per kernel variant)
SCHEDULES = ((1, True), (4, True), (4, False), (8, False))


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

    @staticmethod
    def time_schedule(group: Group, parts: int, persistent: bool, reps: int) -> float:
        """Milliseconds per replay of the group captured with this schedule."""
        graph = group.capture(parts, persistent)
        for _ in range(2):
            graph.replay()
        torch.cuda.synchronize(group.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            graph.replay()
        e1.record()
        torch.cuda.synchronize(group.device)
        del graph
        return e0.elapsed_time(e1) / reps

    def schedule(self, group: Group):
        """Chooses (parts, persistent) for the group, sets it as the group's
        default schedule and returns it with the time of every candidate
        (milliseconds per replay; empty when the choice came from the cache)."""
        counts = {}
        for c, a, b in group.items:
            k = _class_key(c, a, b)
            counts[k] = counts.get(k, 0) + 1
        sig = "\n".join(f"{k}#{n}" for k, n in sorted(counts.items()))
        key = "schedule|" + hashlib.sha1((sig + "|" + "|".join(group.forms)).encode()).hexdigest()
        with self.lock:
            hit = self.cache.get(key)
        times = {}
        if hit is None:
            for parts, pers in SCHEDULES:
                times[(parts, pers)] = self.time_schedule(group, parts, pers, self.reps)
            parts, pers = min(times, key=times.get)
            with self.lock:
                self.cache[key] = {"parts": parts, "persistent": pers, "ms": times[(parts, pers)],
                                   "members": len(group.items)}
                self._save()
        else:
            parts, pers = hit["parts"], hit["persistent"]
        group.schedule = (parts, pers)
        return (parts, pers), times
