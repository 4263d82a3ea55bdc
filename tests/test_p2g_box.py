"""The shared-memory box of the P2G tile kernel (k_p2g_own, fl_grid.cu).

A particle that is not a stray has floor(q) == its bin cell kc along every
axis (q = (p - o) * inv_h in f32, the multiply form of scatter.wgsl:94).  Its
taps then start at floor(q) along the face axis and at floor(f32(q - 0.5))
along the other two; the kernel's face box holds them only if the latter is
kc - 1 or kc.  This checks that property of f32 arithmetic at every cell
coordinate a grid of up to 1024 cells per axis has, on the edge values of q
in [kc, kc + 1) and on random ones."""
import numpy as np


def first_taps(q):
    g = (q - np.float32(0.5)).astype(np.float32)  # __fadd_rn(q, -0.5f)
    return np.floor(g).astype(np.int64)


def test_off_axis_first_tap_is_kc_minus_one_or_kc():
    rng = np.random.default_rng(7)
    for kc in range(0, 1024):
        lo = np.float32(kc)
        hi = np.nextafter(np.float32(kc + 1), np.float32(0.0))  # largest f32 below kc + 1
        mid = np.float32(kc + 0.5)
        edge = np.array([lo, np.nextafter(lo, np.float32(2e9)), np.nextafter(mid, np.float32(0.0)), mid,
                         np.nextafter(mid, np.float32(2e9)), hi], dtype=np.float32)
        rnd = (np.float32(kc) + rng.random(64, dtype=np.float32)).astype(np.float32)
        q = np.concatenate([edge, rnd])
        q = q[np.floor(q) == kc]  # the non-stray condition
        b = first_taps(q)
        assert np.all((b == kc - 1) | (b == kc)), kc
