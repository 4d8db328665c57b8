"""The closed-form selection rule of the search kernels against the reference's
loop (CPU only).

The reference scans a window row by row and keeps the running minimum of
err_diff over valid candidates; the first err_diff <= 0 pins the minimum to 0
and ends that row only (codec/dxt_image.cpp:699-707 intra, :759-767 inter):

    if (e < m) { m = e; sel = pos; if (e <= 0) { m = 0; break; } }

The kernels (warp_select, cta_select) apply it in closed form from three
running values per lane: the first position with e <= 0, the largest key
row * 2^16 + (0xFFFF - col) over positions with e < 0 (the last row holding
one, its first such position), and the first position of the minimum. This
test restates that closed form and checks it against the loop on random
windows with many ties, zeros and invalid positions.
"""
import numpy as np

INVALID = None


def reference_loop(rows):
    """rows: list of rows, each a list of err_diff values or INVALID."""
    m, sel = 2**31 - 1, None
    for r, row in enumerate(rows):
        for c, e in enumerate(row):
            if e is INVALID:
                continue
            if e < m:
                m, sel = e, (r, c)
                if e <= 0:
                    m = 0
                    break
    return sel, m


def closed_form(rows):
    first_le0 = None       # first (row, col) in scan order with e <= 0
    best_key = -1          # max over e < 0 of row * 2^16 + (0xFFFF - col)
    first_min = None       # (e, row, col) of the first minimum
    for r, row in enumerate(rows):
        for c, e in enumerate(row):
            if e is INVALID:
                continue
            if e <= 0 and first_le0 is None:
                first_le0 = (r, c)
            if e < 0:
                best_key = max(best_key, (r << 16) + (0xFFFF - c))
            if first_min is None or e < first_min[0]:
                first_min = (e, r, c)
    if first_le0 is not None:
        r0 = first_le0[0]
        # a row after r0 holding an e < 0 replaces the selection with its first one
        if best_key >= 0 and (best_key >> 16) > r0:
            return ((best_key >> 16), 0xFFFF - (best_key & 0xFFFF)), 0
        return first_le0, 0
    if first_min is None:
        return None, 2**31 - 1
    return (first_min[1], first_min[2]), first_min[0]


def random_window(rng, n_rows, n_cols):
    lo, hi = rng.integers(-4, 1), rng.integers(1, 6)
    p_invalid = rng.choice([0.0, 0.3, 0.8])
    return [[INVALID if rng.random() < p_invalid else int(rng.integers(lo, hi)) for _ in range(n_cols)]
            for _ in range(n_rows)]


def test_closed_form_equals_reference_loop():
    rng = np.random.default_rng(1234)
    for _ in range(20000):
        rows = random_window(rng, int(rng.integers(1, 7)), int(rng.integers(1, 9)))
        assert closed_form(rows) == reference_loop(rows), rows


def test_later_row_negative_replaces_an_earlier_zero():
    # row 0 pins m = 0 at its first zero; row 2's first negative then wins
    rows = [[3, 0, -5], [1, 2, 0], [4, -1, -2]]
    assert reference_loop(rows) == ((2, 1), 0) == closed_form(rows)
    # without a negative after row 0, the first e <= 0 stays selected
    rows = [[3, 0, -5], [1, 2, 0], [4, 0, 1]]
    assert reference_loop(rows) == ((0, 1), 0) == closed_form(rows)
    # a negative in the same row after the first zero is never reached
    rows = [[2, 0, -7]]
    assert reference_loop(rows) == ((0, 1), 0) == closed_form(rows)


def test_first_minimum_when_nothing_is_at_most_zero():
    rows = [[5, 3, INVALID], [3, 4, 9]]
    assert reference_loop(rows) == ((0, 1), 3) == closed_form(rows)
    assert reference_loop([[INVALID, INVALID]]) == (None, 2**31 - 1) == closed_form([[INVALID, INVALID]])
