"""Autotuner for the tracking kernel's shape on a given workload.

Candidates: tracking-kernel block size (128 / 256 threads), the pool kernel's
collision-step threshold (24 / 32 pooled collisions) and refill threshold
(8 / 16 / 32 empty slots), and flux-tally replication (1 / 2 privatised
copies).  (The one-history-per-lane kernel's knobs -- collisions batched per
warp step, particles claimed per queue atomic -- can be searched the same way
by naming them in `space`.)  Each candidate
runs whole cycles (CUDA-graph replays, as production does) on a *scratch*
batch built from the same decks -- so tuning never advances the random
streams of the run that is being tuned -- optionally with the particle counts
scaled down, and the fastest in segments per second wins.  Results are cached
in a JSON file keyed by the workload's shape.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
import time
from pathlib import Path

from .monte_carlo import BatchMonteCarlo
from .problem import Deck

DEFAULT_CACHE = Path(os.environ.get("QSG_TUNE_CACHE", Path.home() / ".cache" / "quicksilver_gb300" / "autotune.json"))

CANDIDATES = {
    "block_size": (128, 256),
    "pool_collision_step": (24, 32),
    "pool_refill": (8, 16, 32),
    "flux_replicas": (1, 2),
}
DEFAULT = {"block_size": 128, "pool_collision_step": 32, "pool_refill": 16, "flux_replicas": 1}
KNOBS = ("block_size", "collision_batch", "queue_chunk", "pool_collision_step", "pool_refill")


def signature(decks: list) -> str:
    shape = []
    for d in decks:
        s = d.simulation
        shape.append((s.nx, s.ny, s.nz, s.n_groups, int(s.n_particles)))
    return hashlib.sha256(json.dumps(sorted(shape)).encode()).hexdigest()[:16]


def _time_candidate(deck_texts, scale, cand, cycles, warmup, max_passes, problems=None):
    decks = [Deck.from_string(t, {"nParticles": max(1000, int(Deck.from_string(t).simulation.n_particles * scale))})
             for t in deck_texts]
    bmc = BatchMonteCarlo(decks, flux_replicas=cand.get("flux_replicas", 1), max_passes=max_passes, problems=problems)
    try:
        bmc.tune(**{k: cand[k] for k in KNOBS if k in cand})
        bmc.run(warmup, use_graph=True)
        t0 = time.perf_counter()
        hist = bmc.run(cycles, use_graph=True)   # history read synchronises
        secs = time.perf_counter() - t0
        return hist.segments() / secs
    finally:
        bmc.close()


def autotune(deck_texts: list, scale: float = 0.25, cycles: int = 2, warmup: int = 1, max_passes: int = 16,
             cache_path: Path | None = DEFAULT_CACHE, space: dict | None = None, refresh: bool = False,
             problems: list | None = None) -> dict:
    """Return the fastest candidate for these decks (dict with the searched knobs
    plus `segments_per_s` and `trials`).  `deck_texts` are Quicksilver deck strings;
    `problems` (optional) are their already-built tables, reused by every
    candidate (the tables do not depend on the particle count)."""
    decks = [Deck.from_string(t) for t in deck_texts]
    key = signature(decks)
    cache = {}
    if cache_path is not None and Path(cache_path).exists():
        try:
            cache = json.loads(Path(cache_path).read_text())
        except (OSError, ValueError):
            cache = {}
    if not refresh and key in cache:
        return cache[key]
    space = space or CANDIDATES
    names = list(space)
    trials = []
    best = None
    for values in itertools.product(*(space[n] for n in names)):
        cand = dict(zip(names, values))
        rate = _time_candidate(deck_texts, scale, cand, cycles, warmup, max_passes, problems)
        trials.append({**cand, "segments_per_s": rate})
        if best is None or rate > best["segments_per_s"]:
            best = {**cand, "segments_per_s": rate}
    best["trials"] = trials
    if cache_path is not None:
        cache[key] = best
        Path(cache_path).parent.mkdir(parents=True, exist_ok=True)
        Path(cache_path).write_text(json.dumps(cache, indent=1))
    return best
