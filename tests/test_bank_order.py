"""The bank-aware order of the X v copy (severo.jl_gb300/csrc/sv_scale.cu,
k_bankorder), restated in NumPy.

A segment's entries are permuted so that slot p (counted from the segment start
rounded down to EPL) holds an entry of class c(p) = (p div EPL + (NC/EPL)(p mod
EPL)) mod NC (class = column index mod NC) where possible: the 32 lanes of a
gather (slot EPL l + t of a group, lane l) then see each class 32/NC times.
Entries of a class fill that class's slots in order of appearance; the surplus
of over-full classes fills the empty slots in slot order.  The kernel finds the
slots through two tables (per class the sorted offsets within a period of EPL NC
slots, and per position the number of the class's offsets below it); these tests
check the tables against direct enumeration, that the placement is a
permutation that keeps each class's order, and the balance of the gathers, for
both instantiations (NC 16 with EPL 4 and 8).
"""
import numpy as np
import pytest

BO_EMPTY = 1024


def bo_class(p, NC, EPL):
    return ((p // EPL) + (NC // EPL) * (p % EPL)) & (NC - 1)


def tables(NC, EPL):
    """The kernel's soff and sbelow, built as it builds them."""
    PER = EPL * NC
    sbelow = np.zeros((NC, PER + 1), np.int64)
    soff = np.zeros((NC, EPL), np.int64)
    for c in range(NC):
        o = [EPL * ((c - (NC // EPL) * t) & (NC - 1)) + t for t in range(EPL)]
        for x in range(PER + 1):
            sbelow[c, x] = sum(v < x for v in o)
        soff[c] = sorted(o)
    return soff, sbelow


def place(cols, s, NC, EPL):
    """Output position (relative to s) of every entry of the segment, or None
    when the kernel copies the segment unchanged."""
    soff, sbelow = tables(NC, EPL)
    PER = EPL * NC
    L = len(cols)
    count = lambda c, X: EPL * (X // PER) + sbelow[c, X % PER]
    slot = lambda c, idx: PER * (idx // EPL) + soff[c, idx % EPL]
    P0 = s & (EPL - 1)
    P1 = P0 + L
    cls = np.asarray(cols) & (NC - 1)
    cnt = np.bincount(cls, minlength=NC)
    empty = [p - P0 for p in range(P0, P1)
             if count(bo_class(p, NC, EPL), p) - count(bo_class(p, NC, EPL), P0) >= cnt[bo_class(p, NC, EPL)]]
    if len(empty) > BO_EMPTY or L > 65535:
        return None
    slots = np.array([count(c, P1) - count(c, P0) for c in range(NC)])
    sur = np.maximum(0, cnt - slots)
    excl = np.concatenate([[0], np.cumsum(sur)[:-1]])
    rank = np.zeros(NC, np.int64)
    q = np.empty(L, np.int64)
    for i, c in enumerate(cls):
        rk = rank[c]
        rank[c] += 1
        q[i] = slot(c, count(c, P0) + rk) - P0 if rk < slots[c] else empty[excl[c] + (rk - slots[c])]
    return q


@pytest.mark.parametrize("NC,EPL", [(16, 4), (16, 8)])
def test_tables_match_enumeration(NC, EPL):
    soff, sbelow = tables(NC, EPL)
    PER = EPL * NC
    p = np.arange(5 * PER)
    cls = bo_class(p, NC, EPL)
    for c in range(NC):
        where = np.flatnonzero(cls == c)
        # the idx-th slot of class c, and the slots of class c before X
        for idx in range(len(where)):
            assert PER * (idx // EPL) + soff[c, idx % EPL] == where[idx]
        for X in range(len(p)):
            assert EPL * (X // PER) + sbelow[c, X % PER] == np.count_nonzero(where < X)


@pytest.mark.parametrize("NC,EPL", [(16, 4), (16, 8)])
def test_gathers_see_each_class_equally(NC, EPL):
    for g in range(3):
        for t in range(EPL):
            p = g * 32 * EPL + EPL * np.arange(32) + t
            assert np.all(np.bincount(bo_class(p, NC, EPL), minlength=NC) == 32 // NC)


@pytest.mark.parametrize("NC,EPL", [(16, 4), (16, 8)])
def test_placement_is_a_permutation_keeping_class_order(NC, EPL):
    rng = np.random.default_rng(NC * EPL)
    checked = skewed = 0
    for trial in range(60):
        L = int(rng.integers(1, 3000))
        s = int(rng.integers(0, 64))
        if trial % 3 == 0:      # skewed: a few features dominate
            cols = np.sort(rng.choice(rng.integers(0, 3000, 6), L))
        else:
            cols = np.sort(rng.integers(0, 3000, L))
        q = place(cols, s, NC, EPL)
        if q is None:           # too many empty slots: copied unchanged
            continue
        checked += 1
        skewed += trial % 3 == 0
        assert np.array_equal(np.sort(q), np.arange(L))
        cls = cols & (NC - 1)
        P0 = s & (EPL - 1)
        for c in range(NC):
            qc = q[cls == c]
            own = bo_class(qc + P0, NC, EPL) == c
            # the class's own slots come first, in order; the surplus afterwards
            k = int(own.sum())
            assert own[:k].all() and not own[k:].any()
            assert np.all(np.diff(qc[:k]) > 0)
    assert checked >= 40 and skewed >= 5
    # a segment with every class equally often lands on its own classes' slots
    cols = np.arange(4096) + 7
    q = place(cols, 3, NC, EPL)
    assert np.all(bo_class(q + (3 & (EPL - 1)), NC, EPL) == (cols & (NC - 1)))
