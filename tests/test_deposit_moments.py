"""The push's shared-memory deposit keeps, per cell, five 32-bit sums of its
particles (count, sum fx, sum fy, and the low 16 and the high bits of sum
fx*fy, fx = rint(ox 2^16)) and forms the four node weights from them when
the block flushes.  This restates that arithmetic in numpy and checks it
against the per-particle CIC weights of the reference's chargeAssignment
(thesisCode/collisionless/double/src/grid.cc:46-76, in 2^-32 charge units):
exact, and every 32-bit sum at most 2^31 (inside its unsigned word) for
the largest push chunk."""
import numpy as np

MAX_CHUNK = 32768


def node_weights_per_particle(fx, fy):
    fx, fy = fx.astype(np.uint64), fy.astype(np.uint64)
    one = np.uint64(65536)
    return ((one - fx) * (one - fy)).sum(), (fx * (one - fy)).sum(), \
        ((one - fx) * fy).sum(), (fx * fy).sum()


def moments(groups):
    """Per-cell sums as the window accumulates them: one add per group of
    particles (a lane's particles in one cell), each sum a 32-bit word."""
    cnt = sfx = sfy = lo = hi = 0
    for fx, fy in groups:
        xy = int((fx.astype(np.uint64) * fy.astype(np.uint64)).sum())
        cnt += len(fx)
        sfx += int(fx.sum())
        sfy += int(fy.sum())
        lo += xy & 0xFFFF
        hi += xy >> 16
    return cnt, sfx, sfy, lo, hi


def weights_from_moments(cnt, sfx, sfy, lo, hi):
    m = (1 << 64) - 1
    sxy = (hi << 16) + lo
    w00 = ((cnt << 32) - ((sfx + sfy) << 16) + sxy) & m
    w10 = ((sfx << 16) - sxy) & m
    w01 = ((sfy << 16) - sxy) & m
    return w00, w10, w01, sxy & m


def test_moment_weights_equal_particle_weights():
    rng = np.random.default_rng(3)
    for trial in range(200):
        n = int(rng.integers(1, 300))
        fx = rng.integers(0, 65537, n)  # rint(ox 2^16) reaches 2^16 for ox just below 1
        fy = rng.integers(0, 65537, n)
        if trial % 7 == 0:
            fx[: n // 2] = 65536
            fy[n // 3:] = 0
        cuts = np.sort(rng.choice(np.arange(1, n), size=min(n - 1, int(rng.integers(0, 8))),
                                  replace=False)) if n > 1 else []
        groups = [(a, b) for a, b in zip(np.split(fx, cuts), np.split(fy, cuts))]
        got = weights_from_moments(*moments(groups))
        want = tuple(int(v) for v in node_weights_per_particle(fx, fy))
        assert got == want
        assert sum(want) == n << 32  # the four weights of a particle sum to 2^32


def test_moment_sums_fit_their_32_bit_words_at_the_largest_chunk():
    # worst case: a whole chunk in one cell with the largest fx, fy, deposited
    # one particle per group (the most low-word adds)
    n = MAX_CHUNK
    fx = np.full(n, 65536)
    fy = np.full(n, 65536)
    cnt, sfx, sfy, lo, hi = moments([(fx[i:i + 1], fy[i:i + 1]) for i in range(0, n, 1)])
    assert max(cnt, sfx, sfy, lo, hi) <= 2**31
    fx = np.full(n, 65535)
    fy = np.full(n, 65535)
    cnt, sfx, sfy, lo, hi = moments([(fx[i:i + 1], fy[i:i + 1]) for i in range(0, n, 1)])
    assert max(cnt, sfx, sfy, lo, hi) <= 2**31
