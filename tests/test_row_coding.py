"""The group coding of the row-blocked X^T u copy (severo.jl_gb300/csrc/sv_scale.cu,
k_rb_count / k_rb_copy / rb_seg_dot), restated in NumPy: a run's rows (sorted,
within a 16,384-row block) are stored in groups of 8 entries, one 64-bit word
per group holding the first row (16 bits) and seven 6-bit steps; a step longer
than 63 is bridged by value-0 padding entries and the run is filled with value-0
entries to a whole number of groups.  The tests check that decoding returns
every row with its value, that the padding carries value 0 at rows inside the
block, and that the padding count is what the counting pass predicts."""
import numpy as np

GROUP = 8


def pads_of(step):
    return (step - 1) // 63 if step > 63 else 0


def encode(rows, vals):
    out_rows, out_vals = [], []
    prev = None
    for r, v in zip(rows, vals):
        if prev is not None:
            for u in range(1, pads_of(r - prev) + 1):
                out_rows.append(prev + 63 * u)
                out_vals.append(0.0)
        out_rows.append(r)
        out_vals.append(v)
        prev = r
    last = out_rows[-1] if out_rows else 0
    while len(out_rows) % GROUP:
        out_rows.append(last)
        out_vals.append(0.0)
    codes = []
    for g in range(0, len(out_rows), GROUP):
        w = out_rows[g]
        for t in range(1, GROUP):
            step = out_rows[g + t] - out_rows[g + t - 1]
            assert 0 <= step <= 63
            w |= step << (16 + 6 * (t - 1))
        assert w < 2 ** 64
        codes.append(w)
    return np.array(codes, dtype=np.uint64), np.array(out_vals), out_rows


def decode(codes):
    rows = []
    for w in codes.tolist():
        r = w & 0xFFFF
        st = w >> 16
        for t in range(GROUP):
            if t:
                r += st & 63
                st >>= 6
            rows.append(r)
    return rows


def count_pass(rows):
    """Entries + padding of a run, whole groups (the counting kernel)."""
    n = len(rows) + sum(pads_of(b - a) for a, b in zip(rows[:-1], rows[1:]))
    return (n + GROUP - 1) // GROUP * GROUP


def test_round_trip_random_runs():
    rng = np.random.default_rng(5)
    for density in (0.35, 0.05, 0.004):
        for _ in range(20):
            mask = rng.random(16384) < density
            rows = np.flatnonzero(mask).tolist()
            if not rows:
                continue
            vals = rng.random(len(rows)) + 0.1
            codes, v, padded = encode(rows, vals)
            dec = decode(codes)
            assert dec == padded
            assert len(dec) == count_pass(rows)
            # the real entries come back in order with their values; padding is 0
            real = [(r, x) for r, x in zip(dec, v) if x != 0.0]
            assert [r for r, _ in real] == rows
            assert np.allclose([x for _, x in real], vals)
            assert all(0 <= r < 16384 for r in dec)


def test_long_steps_and_edges():
    rows = [0, 63, 64, 200, 16383]
    vals = [1.0, 2.0, 3.0, 4.0, 5.0]
    codes, v, padded = encode(rows, vals)
    assert decode(codes) == padded
    assert len(padded) == count_pass(rows)
    assert sum(1 for x in v if x != 0.0) == len(rows)
    # a dot product over the coded run equals the one over the run
    u = np.arange(16384, dtype=np.float64)
    dot = sum(x * u[r] for r, x in zip(decode(codes), v))
    assert dot == sum(x * u[r] for r, x in zip(rows, vals))
