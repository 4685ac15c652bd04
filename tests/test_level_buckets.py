"""Host check of the level-bucket bounds the tensor-core analyses walk.

Each column's candidates are sorted by obs level bucket b(o) = floor(level)
clamped to [0, nlev - 1] (non-finite levels to 0), and an analysis at level
l walks buckets floor(l - v) .. floor(l + v), clamped to the grid, for the
vertical support v.  A candidate can be kept only if |l - level| <= v (its
Gaspari-Cohn weight is zero beyond), so every such candidate must lie in a
walked bucket, whatever the level (inside or outside the grid, exact
integers) and the support (integer or not)."""
import numpy as np


def _bucket(level, nlev):
    b = np.zeros(level.shape, dtype=np.int64)
    fin = np.isfinite(level)
    f = np.floor(level[fin])
    b[fin] = np.where(f <= 0.0, 0, np.where(f >= nlev - 1, nlev - 1, f)).astype(np.int64)
    return b


def _range(lev, v, nlev):
    fl, fh = np.floor(lev - v), np.floor(lev + v)
    lo = 0 if fl <= 0.0 else int(fl)
    hi = nlev - 1 if fh >= nlev - 1 else int(fh)
    return lo, hi


def test_every_candidate_within_the_support_lies_in_a_walked_bucket():
    rng = np.random.default_rng(0)
    for nlev in (2, 3, 6, 10, 30, 64):
        levels = np.concatenate([
            rng.uniform(-3.0, nlev + 2.0, 20_000),             # inside and outside the grid
            rng.integers(-2, nlev + 2, 2_000).astype(float),   # exact integers
            np.array([-0.0, np.nextafter(0.0, -1.0), nlev - 1.0, np.nextafter(nlev - 1.0, nlev)]),
        ])
        b = _bucket(levels, nlev)
        for v in (0.0, 0.5, 1.0, 1.5, 2.0, 2.25, 3.0, float(nlev)):
            for lev in range(nlev):
                lo, hi = _range(lev, v, nlev)
                assert 0 <= lo <= lev <= hi <= nlev - 1
                inside = np.abs(lev - levels) <= v
                walked = (b >= lo) & (b <= hi)
                assert not np.any(inside & ~walked), (nlev, v, lev)


def test_walked_buckets_shrink_the_candidate_walk():
    # about (2 v + 1) / nlev of a column's uniformly spread candidates are walked
    rng = np.random.default_rng(1)
    nlev, v = 30, 2.0
    levels = rng.uniform(0.0, nlev - 1.0, 100_000)
    b = _bucket(levels, nlev)
    walked = np.mean([np.mean((b >= lo) & (b <= hi)) for lo, hi in (_range(l, v, nlev) for l in range(nlev))])
    assert walked < 0.2
