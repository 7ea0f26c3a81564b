"""Launch-schedule autotuner: times candidate schedules of a kernel on the device and keeps
the fastest.

A choice is keyed by (device, knob, problem signature).  It is cached in memory and in a JSON
file (``FH_TUNE_CACHE``, default ``~/.cache/fh_gb300/tune.json``; set but empty: memory only),
so a shape is tuned once per machine and later processes reuse the result; ``FH_AUTOTUNE=0``
turns tuning off and every
knob keeps its built-in heuristic.  Each candidate runs once untimed, then ``reps`` times
between CUDA events on the current stream; the smallest time wins and ties keep the earlier
candidate (callers list the heuristic first).  Tuning launches kernels, so it must not run
while a stream is being captured into a graph: the engine tunes during its first, eager pass.

Knobs in use (fh_gb300.engine):
  xg_splits   split count of the split-K pass SVD_term^T = X G^T (fh_xg_f32 / fh_xg_bf16):
              more splits fill more SMs, fewer splits cut the partial-sum traffic and the
              reduction; candidates: the heuristic (fh_xg_splits / fh_xg_bf16_splits), half,
              twice and four times it.
  rwr_form    the form of the tensor-core walk (fh_rwr_tiles_tc): P in shared memory with
              one product group per epoch (1, the default), or P in tensor memory with the
              epochs pipelined by 64-column blocks and bulk output copies (2, tiles up to 192
              columns); timed as one full walk of the engine's tiles.
  cp_chunk_rows  bin rows per CTA of the CP-ALS row kernels (fh_cp_als chunk table): more
              rows per chunk mean fewer partial sums for the per-chromosome kernel and fewer
              CTAs; candidates 8 (the default), 4 and 16, timed as one sweep on the live
              factors, which are restored after every run.
"""
from __future__ import annotations

import json
import os
import tempfile
import threading


def _default_path():
    """FH_TUNE_CACHE when set (an empty value keeps choices in memory only), else the file
    under ~/.cache."""
    v = os.environ.get("FH_TUNE_CACHE")
    if v is not None:
        return v
    return os.path.join(os.path.expanduser("~"), ".cache", "fh_gb300", "tune.json")


class Tuner:
    def __init__(self, path=None, enabled=None, timer=None):
        """path: JSON cache file (None: the default; "" : memory only).  timer(fn, reps) ->
        milliseconds overrides the CUDA-event timer (tests)."""
        self.path = _default_path() if path is None else path
        if enabled is None:
            enabled = os.environ.get("FH_AUTOTUNE", "1") not in ("0", "false", "no")
        self.enabled = enabled
        self.timer = timer or _cuda_time
        self._lock = threading.Lock()
        self._mem = {}
        self._loaded = False
        self.log = []          # (key, {candidate: ms}, choice) of the tunings this process ran

    # ------------------------------------------------------------------ cache
    def _load(self):
        if self._loaded:
            return
        self._loaded = True
        if not self.path:
            return
        try:
            with open(self.path) as f:
                data = json.load(f)
            if isinstance(data, dict):
                self._mem.update(data)
        except (OSError, ValueError):
            pass

    def _save(self):
        if not self.path:
            return
        try:
            d = os.path.dirname(self.path)
            if d:
                os.makedirs(d, exist_ok=True)
            fd, tmp = tempfile.mkstemp(dir=d or ".", prefix=".tune", suffix=".json")
            with os.fdopen(fd, "w") as f:
                json.dump(self._mem, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass                     # a read-only home keeps the in-memory cache only

    @staticmethod
    def key(device, knob, signature):
        return "%s|%s|%s" % (device, knob, ",".join(str(s) for s in signature))

    # ------------------------------------------------------------------ choose
    def lookup(self, device, knob, signature):
        """The cached choice for this key, or None (no tuning)."""
        if not self.enabled:
            return None
        k = self.key(device, knob, signature)
        with self._lock:
            self._load()
            return self._mem.get(k)

    def choose(self, device, knob, signature, candidates, run, reps=3):
        """The fastest of candidates for run(candidate); candidates[0] when tuning is off."""
        cands = []
        for c in candidates:
            if c not in cands:
                cands.append(c)
        if not cands:
            raise ValueError("no candidates")
        if not self.enabled or len(cands) == 1:
            return cands[0]
        k = self.key(device, knob, signature)
        with self._lock:
            self._load()
            if k in self._mem and self._mem[k] in cands:
                return self._mem[k]
            times = {}
            for c in cands:
                times[c] = self.timer(lambda c=c: run(c), reps)
            best = min(cands, key=lambda c: (times[c], cands.index(c)))
            self._mem[k] = best
            self.log.append((k, times, best))
            self._save()
            return best


def _cuda_time(fn, reps):
    import torch
    fn()                                         # untimed: caches, lazy setup
    best = float("inf")
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return best


_default = None


def default_tuner():
    global _default
    if _default is None:
        _default = Tuner()
    return _default
