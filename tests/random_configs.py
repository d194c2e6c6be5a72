"""Random trainer configurations and power-law walk corpora, shared by the oracle's
differential test against the reference and the GPU engines' parity test.

The reference's model-sync thread (include/dsgl.hpp:641-711) draws one row per block of
equal counts and compares it with sync_ind[i - 1] before anything has been pushed when the
first block (the largest count) holds more than one vertex and the draw is not row 0: it
reads an empty vector and dies with SIGSEGV.  The reference harness lets that thread run
a final round after training, so a corpus whose largest count is shared crashes it (5 of
40 seeds of this generator, all with exactly that tie).  The generator breaks such a tie
with one more occurrence of a top vertex.
"""
import numpy as np


def random_case(seed):
    """(configuration, corpus): V in [1001, 2500) (the reference asserts V > 1000), d up to
    64, window 1-11, 0-10 negatives, 1-2 passes, sample 0 to 1e-2; walks of 1-89 tokens
    drawn from a power law, -1 after each."""
    rng = np.random.default_rng(seed)
    V = int(rng.integers(1001, 2500))
    w = (np.arange(V) + rng.uniform(2, 30)) ** -rng.uniform(0.6, 1.2)
    w /= w.sum()
    toks = []
    for _ in range(int(rng.integers(50, 250))):
        toks.extend(rng.choice(V, size=int(rng.integers(1, 90)), p=w).tolist())
        toks.append(-1)
    counts = np.bincount([t for t in toks if t >= 0], minlength=V)
    top = np.flatnonzero(counts == counts.max())
    if len(top) > 1:  # a shared largest count crashes the reference's sync round (see above)
        toks.extend([int(top[0]), -1])
    cfg = dict(V=V, d=int(rng.choice([4, 8, 12, 16, 20, 32, 36, 64])), window=int(rng.integers(1, 12)),
               negative=int(rng.integers(0, 11)), iter=int(rng.integers(1, 3)),
               sample=float(rng.choice([0.0, 1e-4, 1e-3, 1e-2])), alpha=float(rng.choice([0.01, 0.025, 0.05])))
    return cfg, np.array(toks, dtype=np.int32)
