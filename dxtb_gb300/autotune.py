"""
Autotuner of the SCF launch policy: the orbital-count thresholds of the size
classes (``dxtb_scf_set_size_classes``), i.e. which molecules run as one CTA
of 256 threads two per SM, one CTA of 512 threads per SM, or a thread-block
cluster of 2, 4, 8 or 16 CTAs.

``tune(pb)`` times the packed batch ``pb`` (energy + forces, CUDA events on
the current stream, the median of ``reps`` runs after one warm-up) under each
candidate threshold set, keeps the fastest, applies it process-wide and
caches it on disk, keyed by the GPU (name, SM count), the library build and
a signature of the batch's size distribution. ``ensure(pb)`` applies a
cached choice or tunes once per process and device. Setting
``DXTB_AUTOTUNE=0`` keeps the library's defaults. The choice changes only
the team each molecule runs on, so results agree to rounding.

The reference has no counterpart: its batched SCF is a padded tensor
program whose shapes PyTorch dispatches.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import time
from pathlib import Path

import numpy as np
import torch

from . import _lib, build

DEFAULT = (112, 136, 160, 320, 640)
# thresholds of classes 1..5 (one-SM CTA, clusters of 2, 4, 8, 16)
CANDIDATES = [
    DEFAULT,
    (100, 136, 160, 320, 640),
    (124, 136, 160, 320, 640),
    (112, 144, 176, 320, 640),
    (112, 128, 160, 320, 640),
    (112, 136, 192, 384, 768),
]
_applied: dict = {}


def cache_path() -> Path:
    root = os.environ.get("DXTB_CACHE_DIR") or os.path.join(
        os.environ.get("XDG_CACHE_HOME") or os.path.expanduser("~/.cache"), "dxtb_gb300")
    return Path(root) / "autotune.json"


def _device_key(dev: torch.device) -> str:
    p = torch.cuda.get_device_properties(dev)
    lib = build.LIB
    stamp = str(int(lib.stat().st_mtime)) if lib.exists() else "nolib"
    return f"{p.name}|{p.multi_processor_count}|{stamp}"


def _batch_key(pb) -> str:
    # the size distribution decides the policy: a histogram of orbital counts
    h, _ = np.histogram(pb.nao, bins=[0, 64, 96, 112, 128, 136, 144, 160, 192, 256, 320, 384, 640, 768,
                                      1 << 20])
    frac = np.round(h / max(1, pb.nmol), 2)
    return hashlib.sha1(f"{pb.tables.method}|{pb.nmol // 64}|{frac.tolist()}".encode()).hexdigest()[:16]


def set_classes(thr) -> None:
    arr = (C.c_int32 * 5)(*[int(v) for v in thr])
    _lib.check(_lib.lib().dxtb_scf_set_size_classes(arr), "size classes")


def get_classes() -> tuple:
    arr = (C.c_int32 * 5)()
    _lib.check(_lib.lib().dxtb_scf_get_size_classes(arr), "size classes")
    return tuple(int(v) for v in arr)


def _time(pb, state: dict, reps: int) -> float:
    from .engine import run

    run(pb, forces=True, state=state)
    times = []
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        run(pb, forces=True, state=state)
        e.record()
        e.synchronize()
        times.append(s.elapsed_time(e))
    return float(np.median(times))


def tune(pb, candidates=None, reps: int = 3, save: bool = True) -> dict:
    """Times every candidate on ``pb``, applies and returns the fastest:
    {"thresholds": [...], "ms": {candidate: median ms}, "source": "tuned"}."""
    cands = [tuple(c) for c in (candidates or CANDIDATES)]
    state: dict = {}
    ms = {}
    for c in cands:
        set_classes(c)
        ms[c] = _time(pb, state, reps)
    best = min(ms, key=ms.get)
    set_classes(best)
    out = {"thresholds": list(best), "ms": {",".join(map(str, c)): v for c, v in ms.items()},
           "source": "tuned", "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
    if save:
        path = cache_path()
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            data = json.loads(path.read_text()) if path.exists() else {}
            data.setdefault(_device_key(pb.device), {})[_batch_key(pb)] = out
            path.write_text(json.dumps(data, indent=1))
        except OSError:
            pass  # a read-only cache location only costs a re-tune
    return out


def ensure(pb, min_molecules: int = 32) -> dict:
    """Applies the cached policy for this GPU and batch shape, tuning once if
    none is cached. Batches below ``min_molecules`` keep the current policy."""
    if os.environ.get("DXTB_AUTOTUNE", "1") == "0" or pb.nmol < min_molecules:
        return {"thresholds": list(get_classes()), "source": "default"}
    dkey, bkey = _device_key(pb.device), _batch_key(pb)
    if (dkey, bkey) in _applied:
        set_classes(_applied[(dkey, bkey)]["thresholds"])
        return _applied[(dkey, bkey)]
    try:
        data = json.loads(cache_path().read_text())
        hit = data[dkey][bkey]
        set_classes(hit["thresholds"])
        res = dict(hit, source="cache")
    except (OSError, KeyError, ValueError):
        res = tune(pb)
    _applied[(dkey, bkey)] = res
    return res
