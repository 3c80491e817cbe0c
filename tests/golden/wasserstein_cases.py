"""Seeded transport-cost cases for the Wasserstein distance's solver.

A small xorshift64* stream (no library generator, so every machine builds the
same values) gives, for each size pair n1, n2 = 1..8, a few cost matrices of
the shapes the distance produces: sums of absolute differences at scales
1e-3..1e3, with ties (repeated rows and columns) in some of them.  Used by
make_wasserstein_goldens.py and tests/test_oracle_wasserstein.py.
"""

MASK = (1 << 64) - 1


def _stream(seed):
    s = (seed * 0x9E3779B97F4A7C15 + 1) & MASK
    while True:
        s ^= s >> 12
        s ^= (s << 25) & MASK
        s ^= s >> 27
        yield ((s * 0x2545F4914F6CDD1D) & MASK) >> 11  # 53 random bits


def cases(per_size=5, seed=20260):
    """[(n1, n2, D row-major list)] in a fixed order; the last case of each
    size pair with n1 > 1 has two equal rows (see tied())."""
    r = _stream(seed)
    out = []
    for n1 in range(1, 9):
        for n2 in range(1, 9):
            for c in range(per_size):
                scale = 10.0 ** ((next(r) % 7) - 3)
                D = [next(r) * 2.0 ** -53 * scale for _ in range(n1 * n2)]
                if c == per_size - 1 and n1 > 1:
                    D[n2:2 * n2] = D[0:n2]  # two equal rows: tied plans
                out.append((n1, n2, D))
    return out


def tied(index, per_size=5):
    """Whether case `index` of cases() has two equal rows, so that several
    plans are optimal and solvers may sum the same cost in another order."""
    n1 = index // (8 * per_size) + 1
    return index % per_size == per_size - 1 and n1 > 1
