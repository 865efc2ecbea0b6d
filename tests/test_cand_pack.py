"""The FP32K candidate entry (cand_pack in csrc/state.cuh) keeps a record's cell
offsets (xr, yr) for the candidate test with the flags in the low mantissa
bits: xr's two lowest bits the blanked / non-finite marks, yr's three lowest
bits the cell row modulo 8.  This restates the packing and the row difference
of the candidate scan (cand_row_diff, csrc/interact32.cuh) in numpy and checks
that the row difference is exact for every row pair the stencil can hold and
that each coordinate moves by at most 7 units in the last place."""
import numpy as np

K_CAND_BLANKED, K_CAND_NONFINITE = 1, 2
K_FLAG_BLANKED, K_FLAG_NONFINITE = 1 << 30, 1 << 28


def cand_pack(xr, yr, flags):
    bx = (xr.astype(np.float32).view(np.int32) & ~np.int32(3)) \
        | np.where(flags & K_FLAG_BLANKED, K_CAND_BLANKED, 0).astype(np.int32) \
        | np.where(flags & K_FLAG_NONFINITE, K_CAND_NONFINITE, 0).astype(np.int32)
    by = (yr.astype(np.float32).view(np.int32) & ~np.int32(7)) | (flags & 7).astype(np.int32)
    return bx.view(np.float32), by.view(np.float32)


def cand_row_diff(gj, cy):
    d = (gj.astype(np.uint32) - cy.view(np.int32).astype(np.uint32)) << np.uint32(29)
    return d.astype(np.uint32).view(np.int32) >> 29


def test_row_difference_is_exact_within_the_stencil():
    rng = np.random.default_rng(0)
    n = 1_000_000
    row = rng.integers(0, (1 << 28) - 1, n)
    gj = np.clip(row + rng.integers(-3, 4, n), 0, (1 << 28) - 1)
    cell = 8.5e-4
    yr = rng.uniform(-1e-3 * cell, 1.001 * cell, n)
    yr[::7] = -yr[::7]            # negative offsets (a predicted position below its cell)
    yr[::11] = 0.0
    yr[::13] = -0.0
    flags = (row & ((1 << 28) - 1)) | np.where(rng.random(n) < 0.1, K_FLAG_BLANKED, 0)
    _, cy = cand_pack(np.zeros(n), yr, flags)
    assert np.array_equal(cand_row_diff(gj, cy), gj - row)


def test_offsets_move_by_at_most_seven_ulp_and_flags_survive():
    rng = np.random.default_rng(1)
    n = 1_000_000
    cell = 8.5e-4
    xr = rng.uniform(-0.01 * cell, 1.01 * cell, n).astype(np.float32)
    yr = rng.uniform(-0.01 * cell, 1.01 * cell, n).astype(np.float32)
    flags = rng.integers(0, 1 << 28, n) | np.where(rng.random(n) < 0.2, K_FLAG_BLANKED, 0) \
        | np.where(rng.random(n) < 0.1, K_FLAG_NONFINITE, 0)
    cx, cy = cand_pack(xr, yr, flags)
    ulp_x = np.spacing(np.abs(xr))
    ulp_y = np.spacing(np.abs(yr))
    assert np.all(np.abs(cx - xr) <= 3 * ulp_x)
    assert np.all(np.abs(cy - yr) <= 7 * ulp_y)
    bx = cx.view(np.int32)
    assert np.array_equal((bx & K_CAND_BLANKED) != 0, (flags & K_FLAG_BLANKED) != 0)
    assert np.array_equal((bx & K_CAND_NONFINITE) != 0, (flags & K_FLAG_NONFINITE) != 0)
    # the support boundary moves by at most 2^-20 of a cell
    assert np.max(np.abs(cx - xr)) <= cell * 2.0 ** -20 and np.max(np.abs(cy - yr)) <= cell * 2.0 ** -20
