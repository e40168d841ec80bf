"""The packed cell-code arithmetic of the mixed-form list sweep
(fluidsim_gb300/csrc/fsim_kernels.cu: pack_cell, cells_adjacent, cell_codes),
restated with numpy in 32-bit unsigned arithmetic and checked against the
plain per-axis rule over every coordinate pair near the ends and the middle
of the largest grid the packing allows (2047 x 1023 x 2047 cells).

cell_codes(c_j, kCellBias - c_i) must give the codes (d + 1 per axis, d the
cell difference) exactly when every |d| <= 1, and fail otherwise: a field
below -1 wraps to at least 3 in its own bits and any borrow it passes up only
shows where a field has already failed."""
import itertools

import numpy as np

BIAS = np.uint32(1 | (1 << 11) | (1 << 21))
LIMITS = (2047, 1023, 2047)  # cells per axis the packing holds (x, y: 11, 10 bits; z: 11 bits)


def pack(x, y, z):
    return (np.uint32(x) | (np.uint32(y) << np.uint32(11)) | (np.uint32(z) << np.uint32(21))).astype(np.uint32)


def codes(cj, ci):
    with np.errstate(over="ignore"):
        d = (cj + (BIAS - ci)).astype(np.uint32)
    bx = d & np.uint32(0x7FF)
    by = (d >> np.uint32(11)) & np.uint32(0x3FF)
    bz = d >> np.uint32(21)
    ok = (bx <= 2) & (by <= 2) & (bz <= 2)
    return ok, bx.astype(np.int64), by.astype(np.int64), bz.astype(np.int64)


def _axis_values(n):
    # both ends, the middle and their neighbours
    return sorted({v for c in (0, 1, 2, 3, n // 2 - 1, n // 2, n // 2 + 1, n - 4, n - 3, n - 2, n - 1)
                   for v in (c,) if 0 <= v < n})


def test_codes_equal_the_per_axis_rule():
    vals = [np.array(_axis_values(n)) for n in LIMITS]
    gi = np.array(list(itertools.product(*vals)))  # own cells
    for xj, yj, zj in itertools.product(*vals):    # every neighbour cell from the same set
        ci = pack(gi[:, 0], gi[:, 1], gi[:, 2])
        cj = pack(np.full(len(gi), xj), np.full(len(gi), yj), np.full(len(gi), zj))
        ok, bx, by, bz = codes(cj, ci)
        d = np.stack([xj - gi[:, 0], yj - gi[:, 1], zj - gi[:, 2]], axis=1)
        adjacent = (np.abs(d) <= 1).all(axis=1)
        assert np.array_equal(ok, adjacent)
        assert np.array_equal(bx[ok], d[ok, 0] + 1)
        assert np.array_equal(by[ok], d[ok, 1] + 1)
        assert np.array_equal(bz[ok], d[ok, 2] + 1)


def test_codes_random_pairs():
    rng = np.random.default_rng(7)
    n = 200_000
    own = np.stack([rng.integers(0, m, n) for m in LIMITS], axis=1)
    step = rng.integers(-3, 4, (n, 3))
    other = np.clip(own + step, 0, np.array(LIMITS) - 1)
    ok, bx, by, bz = codes(pack(*other.T), pack(*own.T))
    d = other - own
    adjacent = (np.abs(d) <= 1).all(axis=1)
    assert np.array_equal(ok, adjacent)
    assert np.array_equal(np.stack([bx, by, bz], 1)[ok], d[ok] + 1)
