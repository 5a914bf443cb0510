"""The mesher's cube case needs only the sign of Voxel::Distance = sum /
weight (Mesher.cpp:191-199).  The kernel takes that sign from the operands
where the IEEE quotient is a normal non-zero float -- 2^-100 <= |sum| and
2^-100 <= |weight| <= 2^24 -- and divides otherwise.  This checks the rule
against float32 division (correctly rounded, as on the GPU) over random,
boundary and special operands."""
import numpy as np


def rule(x, w):
    x = np.asarray(x, np.float32)
    w = np.asarray(w, np.float32)
    ax, aw = np.abs(x), np.abs(w)
    fast = (ax >= np.float32(2.0 ** -100)) & (aw >= np.float32(2.0 ** -100)) & (aw <= np.float32(2.0 ** 24))
    with np.errstate(all="ignore"):
        slow = (x / w) < 0
    return np.where(fast, (x < 0) != (w < 0), slow)


def test_sign_rule_equals_division():
    rng = np.random.default_rng(0)
    n = 2_000_000
    # magnitudes spread over the whole float range, both signs
    ex = rng.uniform(-149, 128, n)
    ew = rng.uniform(-149, 128, n)
    x = (np.sign(rng.uniform(-1, 1, n)) * 2.0 ** ex).astype(np.float32)
    w = (np.sign(rng.uniform(-1, 1, n)) * 2.0 ** ew).astype(np.float32)
    # TSDF-like values: sums of truncated distances and whole weights
    x2 = rng.uniform(-6, 6, n).astype(np.float32) * np.float32(0.02)
    w2 = rng.integers(1, 400, n).astype(np.float32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2.0 ** -149, -(2.0 ** -149), 2.0 ** -100,
                         -(2.0 ** -100), 2.0 ** -101, 2.0 ** 24, 2.0 ** 25, 1.0, -1.0, 3.4e38], np.float32)
    sx, sw = np.meshgrid(specials, specials)
    for xs, ws in ((x, w), (x2, w2), (sx.ravel(), sw.ravel()), (x, w2), (x2, w)):
        with np.errstate(all="ignore"):
            want = (xs / ws) < 0
        assert np.array_equal(rule(xs, ws), want)
