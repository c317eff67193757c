"""RNG known-answer vectors from the reference's rngSample / rngSpawn_Random_Number_Seed."""
import numpy as np

import oracle_py as O
from helpers import DECKS

GOLDEN = DECKS.parent.parent / "tests" / "golden"


def test_oracle_rng_known_answers():
    g = np.load(GOLDEN / "t_homog.npz")
    seeds = g["rng_seeds"]
    samples = g["rng_samples"].reshape(len(seeds), 8)
    states = g["rng_states"].reshape(len(seeds), 8)
    for i, s0 in enumerate(seeds):
        s = int(s0)
        for k in range(8):
            v, s = O.rng_sample(s)
            assert v == samples[i, k] and s == states[i, k]
        child, parent = O.rng_spawn(int(s0))
        assert child == g["rng_spawned"][i] and parent == g["rng_parent_after"][i]
