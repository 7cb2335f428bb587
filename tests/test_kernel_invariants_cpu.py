"""Host-side checks of two index and rounding invariants that device kernels
rely on (no GPU):

* the element spread's padded stencil bitmap (csrc/ggem_spread_elem.cu):
  for every element of a brick and every cell of the brick's frame, each
  5-bit field of (packed frame coordinates - per-element value) lies in
  [0, dim + 2B - 2), so one subtraction indexes the bitmap without bounds
  checks whenever dim + 2B - 2 <= 32 (the frame rule restated from
  brick_frame);
* the pair list's bounding-box cull (csrc/ggem_cells.cu): the FP32 distance
  of a candidate from the targets' box, formed with the same subtractions,
  squares and fused adds as a target's r2, never exceeds that r2, so a
  culled candidate would have been rejected for every target.
"""
import numpy as np


def brick_frame(nc, periodic, b0, b1, lo, hi):
    ext = (b1 - b0) + (hi - lo)
    if periodic and ext >= nc:
        return 0, nc, True
    if periodic:
        return b0 + lo, ext, False
    a, z = max(0, b0 + lo), min(nc - 1, b1 - 1 + hi)
    return a, z - a + 1, False


def test_padded_spread_bitmap_fields_stay_in_range():
    checked = 0
    for nc in (5, 9, 16, 29, 40, 72):
        for periodic in (False, True):
            for R in (1, 3, 6, 7, 9, 13, 15):
                lo, hi, dim = -R, R, 2 * R + 1
                for B in (1, 2, 3, 4, 6, 8):
                    if dim + 2 * B - 2 > 32:
                        continue  # the compact bitmap is used instead
                    for bi in range((nc + B - 1) // B):
                        b0, b1 = bi * B, min(bi * B + B, nc)
                        F, E, full = brick_frame(nc, periodic, b0, b1, lo, hi)
                        if full or E > 32:
                            continue  # whole-axis frames wrap; wider frames are refused
                        ex = np.arange(b0, b1)[:, None]
                        ux = np.arange(E)[None, :]
                        field = ux - (ex - F + lo - B + 1)
                        assert field.min() >= 0
                        assert field.max() <= dim + 2 * B - 3
                        checked += field.size
    assert checked > 100000


def _fma32(a, b, c):
    # fused multiply-add rounded to FP32 (the product of two FP32 values is
    # exact in FP64; the sum rounds once or twice, monotonically)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def _r2(dx, dy, dz):
    return _fma32(dz, dz, _fma32(dy, dy, (dx * dx).astype(np.float32)))


def test_box_distance_never_exceeds_a_targets_r2():
    rng = np.random.default_rng(7)
    for trial in range(40):
        nt = int(rng.integers(1, 33))
        h = np.float32(7.0)
        targets = (rng.uniform(-0.5, 0.5, (nt, 3)) * h).astype(np.float32)
        lo, hi = targets.min(axis=0), targets.max(axis=0)
        q = (rng.uniform(-2.0, 2.0, (4096, 3)) * h).astype(np.float32)
        # box distance per axis as the kernel forms it
        b = np.where(q > hi, q - hi, np.where(q < lo, lo - q, np.float32(0))).astype(np.float32)
        box = _r2(b[:, 0], b[:, 1], b[:, 2])
        for t in targets:
            d = (q - t).astype(np.float32)
            r2 = _r2(d[:, 0], d[:, 1], d[:, 2])
            assert np.all(box <= r2), trial
