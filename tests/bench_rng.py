"""bench_rng_next of the reference's tests (src/tests/bench_common.h:31-37), vectorised with numpy.

splitmix64: the state advances by 0x9E3779B97F4A7C15 before each draw and the draw is the state
mixed. Draw k (k = 1, 2, ...) from a generator seeded s is therefore mix(s + k * gamma).
"""
import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)


def mix(z):
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def draws(seed, count, first=1):
    """Draws first .. first + count - 1 of the generator seeded `seed`."""
    with np.errstate(over="ignore"):
        k = np.arange(first, first + count, dtype=np.uint64)
        return mix(np.uint64(seed) + k * GAMMA)


def rows(seed, n, per_row):
    """n rows of per_row consecutive draws each -> array [n, per_row]."""
    return draws(seed, n * per_row).reshape(n, per_row)
