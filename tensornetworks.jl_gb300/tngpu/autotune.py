"""Launch-width autotuner of the trajectory engine (tn_qjmc_ensemble).

The engine's one schedule knob is its width: how many 128-thread blocks
(each running whole trajectories) share an SM.  Wider launches hide one
block's latency-bound phases behind the others' FP64 work but cut the
registers and cache per block and, for ensembles smaller than the slots,
leave SMs idle.  The best width depends on the bond dimension, the local
dimension and the ensemble size, so it is picked per bucket of
(maxdim, d, ntraj, N) -- each rounded up to a power of two -- by timing a
short probe of the caller's own workload at every candidate width with
the engine's CUDA-event launch time, and kept in a JSON cache.
"""

import json
import os
import tempfile
import warnings

WIDTHS = (1, 2, 4, 8)


def _p2(x):
    x = max(int(x), 1)
    return 1 << (x - 1).bit_length()


def bucket(maxdim, d, ntraj, nsites):
    """Cache key of a workload: maxdim, d, ensemble size and chain length,
    each rounded up to a power of two."""
    return f"chi{_p2(maxdim)}-d{int(d)}-traj{_p2(ntraj)}-N{_p2(nsites)}"


def default_cache_path():
    p = os.environ.get("TNGPU_TUNE_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "tngpu", "engine_widths.json")


class WidthCache:
    """bucket -> {"width": w, "seconds_per_traj_step": {w: s, ...}} in one
    JSON file, read at construction and rewritten atomically on put."""

    def __init__(self, path=None):
        self.path = path or default_cache_path()
        self.entries = {}
        try:
            with open(self.path) as f:
                data = json.load(f)
            if isinstance(data, dict):
                self.entries = {k: v for k, v in data.items()
                                if isinstance(v, dict) and v.get("width") in WIDTHS}
        except (OSError, ValueError):
            self.entries = {}

    def get(self, key):
        e = self.entries.get(key)
        return None if e is None else int(e["width"])

    def put(self, key, width, timings):
        self.entries[key] = {"width": int(width),
                             "seconds_per_traj_step": {str(w): float(t) for w, t in timings.items()}}
        d = os.path.dirname(self.path) or "."
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".engine_widths", dir=d)
        with os.fdopen(fd, "w") as f:
            json.dump(self.entries, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def tune(key, probe, widths=WIDTHS, cache=None):
    """The width for ``key``: from ``cache`` when present, else the one
    whose ``probe(width)`` (seconds per trajectory-step) is smallest, the
    narrower on a tie, stored in ``cache``.  Returns (width, timings), the
    timings empty on a cache hit."""
    widths = tuple(int(w) for w in widths)
    if not widths or any(w not in WIDTHS for w in widths):
        raise ValueError(f"widths must be drawn from {WIDTHS}")
    if cache is not None:
        w = cache.get(key)
        if w is not None:
            return w, {}
    timings = {}
    for w in widths:
        t = float(probe(w))
        if not t > 0.0:
            raise RuntimeError(f"probe at width {w} returned no time")
        timings[w] = t
    best = min(widths, key=lambda w: (timings[w], w))
    if cache is not None:
        try:
            cache.put(key, best, timings)
        except OSError as e:  # an unwritable cache costs a re-tune, not the run
            warnings.warn(f"autotune cache {cache.path} not written: {e}")
    return best, timings
