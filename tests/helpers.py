"""Shared helpers of the test suite."""
import numpy as np

from dmdgb import systems


def first_mismatch(a: np.ndarray, b: np.ndarray) -> int:
    n = min(len(a), len(b))
    neq = np.nonzero(a[:n] != b[:n])[0]
    if len(neq):
        return int(neq[0])
    return n if len(a) != len(b) else -1


def describe(a, b, k):
    lo = max(0, k - 2)
    return "\n".join([f"gpu {a[q]}\ncpu {b[q]}" for q in range(lo, min(k + 2, len(a), len(b)))])


def dense_system(n_chains=6, L=12, box=60.0, tstar=0.25, seed=3, rng_seed=11, gly_pro=True):
    """A crowded system of random sequences (glycine and proline included)
    so that H-bond, shoulder and hydrophobic events all occur early."""
    rng = np.random.default_rng(rng_seed)
    res = []
    for _ in range(n_chains):
        seq = systems.random_sequence(rng, L)
        if gly_pro:
            seq[2] = 9      # glycine: no side chain
            seq[L - 3] = 17  # proline
        res += seq
    spec = systems.SystemSpec([L] * n_chains, res, box, tstar, seed, name="dense")
    return systems.generate(spec, min_sep=4.0)
