"""Launch-configuration autotuner for the batched dGN engine.

A batch of small CPDs (``cpd_batch``) is one engine launch; two choices shape
its speed and depend on the batch's size distribution:

* the engine's register tile (``tfx_dgn_options.tile``: 1, 2 or 4, i.e.
  16, 32 or 64 rows and columns per tile of its small contractions).  Smaller
  tiles need less shared memory and registers, so more problems run per SM
  (tiles 1 and 2 use the variant built for two resident CTAs per SM), but
  cost more loop trips on the larger problems;
* the order the problems are handed to the CTAs: as given, or largest first
  (the longest solves start in the first wave instead of forming a tail).

``BatchTuner.choose`` times every candidate with CUDA events on a sample of
the batch (every k-th problem, at least one full wave of CTAs) and keeps the
fastest.  Decisions are cached per batch signature (precision, order of the
tensors, largest core dimension, largest rank, a size class of the batch) in
memory and, unless ``TFX_TUNE_CACHE`` is set to an empty string, in a JSON file
(``TFX_TUNE_CACHE`` or ``~/.cache/tensorfox_gb300/batch_tune.json``), so a
signature is tuned once per machine.
"""
import json
import os

import numpy as np

TILES = (1, 2, 4)
ORDERS = ("given", "largest_first")


def signature(prec, L, max_core, max_rank, n):
    """Cache key of a batch: precision, order, bucketed largest core dimension
    and rank, and the batch size class (powers of four)."""
    def bucket(v):
        return int(2 ** int(np.ceil(np.log2(max(1, v)))))
    size_class = int(4 ** int(np.ceil(np.log(max(1, n)) / np.log(4))))
    return "%s|L%d|d%d|R%d|n%d" % (prec, L, bucket(max_core), bucket(max_rank), size_class)


def candidates(max_core, max_rank):
    """Every (tile, order) pair; tiles larger than needed by the batch's
    largest dimension or rank are left out (they only add padding)."""
    need = max(max_core, max_rank)
    tiles = [t for t in TILES if t == 1 or 16 * (t // 2) < need]
    return [(t, o) for t in tiles for o in ORDERS]


def sample_indices(n, waves_slots, max_sample=1024):
    """Every k-th problem, about one wave of CTAs (at least ``waves_slots``
    problems when the batch has them), at most ``max_sample``."""
    m = int(min(n, max(waves_slots, min(max_sample, n // 8))))
    if m >= n:
        return np.arange(n)
    step = n / m
    return np.unique((np.arange(m) * step).astype(np.int64))


def order_largest_first(work):
    """Problem order by decreasing work estimate (stable)."""
    return np.argsort(-np.asarray(work, dtype=np.float64), kind="stable")


class BatchTuner:
    def __init__(self, path=None):
        env = os.environ.get("TFX_TUNE_CACHE")
        if env is not None:
            path = env or None
        elif path is None:
            path = os.path.join(os.path.expanduser("~"), ".cache", "tensorfox_gb300", "batch_tune.json")
        self.path = path
        self.mem = {}
        self.log = []
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.mem.update(json.load(f))
            except (OSError, ValueError):
                pass

    def lookup(self, key):
        v = self.mem.get(key)
        return (int(v[0]), str(v[1])) if v is not None else None

    def choose(self, key, cands, run):
        """``run(candidate) -> seconds``; returns the fastest candidate (cached)."""
        hit = self.lookup(key)
        if hit is not None and hit in cands:
            return hit
        times = {}
        for c in cands:
            times[c] = float(run(c))
        best = min(cands, key=lambda c: times[c])
        self.mem[key] = [best[0], best[1]]
        self.log.append((key, {"%d/%s" % c: t for c, t in times.items()}, best))
        if self.path:
            try:
                os.makedirs(os.path.dirname(self.path), exist_ok=True)
                tmp = self.path + ".tmp%d" % os.getpid()
                with open(tmp, "w") as f:
                    json.dump(self.mem, f)
                os.replace(tmp, self.path)
            except OSError:
                pass
        return best


_TUNER = None


def tuner():
    global _TUNER
    if _TUNER is None:
        _TUNER = BatchTuner()
    return _TUNER
