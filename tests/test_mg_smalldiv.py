"""The multigrid kernel's cell coordinates on the levels block 0 runs alone.

fl_mg.cu (SmallDiv) splits a cell index c of a level of at most 4096 cells
into (i, j, k) with multiply-high by rounded-up reciprocals ceil(2^32 / d)
instead of integer division; a divisor of 1 is stored as 0.  The claim is
exactness whenever c * d < 2^32, which holds there (c < 4096, d <= 4096).
This restates the arithmetic in numpy (uint64 products, high 32 bits) and
checks it against integer division for every level shape up to 4096 cells
with extents up to 64, and for the elongated extremes.
"""
import numpy as np


def recip(d):
    return (0xFFFFFFFF // d + 1) if d > 1 else 0


def ijk(c, nx, ny):
    c = c.astype(np.uint64)
    nxy = nx * ny
    mx, mxy = recip(nx), recip(nxy)
    k = (c * np.uint64(mxy)) >> np.uint64(32) if mxy else c
    rem = c - k * np.uint64(nxy)
    j = (rem * np.uint64(mx)) >> np.uint64(32) if mx else rem
    return rem - j * np.uint64(nx), j, k


def check(nx, ny, nz):
    c = np.arange(nx * ny * nz, dtype=np.uint64)
    i, j, k = ijk(c, nx, ny)
    assert np.array_equal(i, c % np.uint64(nx))
    assert np.array_equal(j, (c // np.uint64(nx)) % np.uint64(ny))
    assert np.array_equal(k, c // np.uint64(nx * ny))


def test_every_small_level_shape():
    n = 0
    for nx in range(1, 65):
        for ny in range(1, 65):
            nzmax = 4096 // (nx * ny)
            if nzmax < 1:
                continue
            for nz in sorted({1, max(1, nzmax // 2), nzmax}):
                check(nx, ny, nz)
                n += 1
    assert n > 5000


def test_elongated_levels():
    for shape in [(4096, 1, 1), (1, 4096, 1), (1, 1, 4096), (2048, 2, 1), (1, 2048, 2), (3, 1365, 1), (4095, 1, 1),
                  (17, 15, 16), (1, 1, 1)]:
        check(*shape)
