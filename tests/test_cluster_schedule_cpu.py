"""The streamed cluster wavefront's staging schedule (csrc/lscs.cuh), checked
on the CPU with the kernel's own step arithmetic.

Block r's loader issues the copies of diagonal e at step
t_w(e) = e - lead + m r (lead = 2m + 6; steps t < 0 are the pre-fill, waited
for before the first cluster barrier) into ring row e mod R, R = (2m+3)K + 8.
One copy group per barrier interval (steps [I(m+1), I(m+1) + m]) is waited
for before the barrier that ends the next interval, so a row issued in
interval I is readable from interval I + 2. Sweep k of block r updates
diagonal d = t + 2 - L k - m r at step t (L = 2m + 3) and reads the staged
rows of diagonals d - 1 .. d + 2; the last sweep writes its values of
diagonal d to x at that step. The test checks, for every diagonal and block:
- a staged row is readable before its first read;
- its last read happens in an earlier interval than the issue of the copy
  that overwrites its ring row;
- the last sweep's write of a cell to x happens after the copies of that
  cell that are read have landed (the owner's own, and the lower neighbour's
  of the owner's first position).
"""
import pytest


def interval(t, m):
    return t // (m + 1)


def readable_from(t_w, m):
    """First step at which a row issued at step t_w may be read."""
    if t_w < 0:  # pre-fill: waited for before the first barrier
        return 0
    return (interval(t_w, m) + 2) * (m + 1)


def check(N, K, C, m):
    S = N + 2
    L = 2 * m + 3
    lead = 2 * m + 6
    R = (2 * m + 3) * K + 8
    nd = 2 * S - 1
    J = (N + C - 1) // C
    for r in range(C):
        jb = 1 + r * J
        je = min(N, jb + J - 1)
        dlo, dhi = jb + 1, je + N  # diagonals holding this block's interior cells
        for e in range(nd):
            t_w = e - lead + m * r
            # diagonal e is read by the updates of diagonals d = e - 2 .. e + 1
            lo, hi = max(e - 2, dlo), min(e + 1, dhi)
            if lo <= hi:
                # first read: sweep 0 at the lowest such d; last: sweep K-1 at the highest
                t_first = lo - 2 + m * r
                assert t_first >= readable_from(t_w, m), (N, K, C, m, r, e)
                t_last = hi - 2 + L * (K - 1) + m * r
                # the copy of diagonal e + R reuses the row
                t_over = (e + R) - lead + m * r
                assert interval(t_last, m) < interval(t_over, m), (N, K, C, m, r, e)
            # the staged x cells the kernel reads: its own positions and je + 1 (the
            # upper neighbour's first; every other staged position it reads is on
            # the frame, never written), each written by its owner's last sweep at
            # step e - 2 + L (K-1) + m r'
            for j in range(jb, min(N, je + 1) + 1):
                i = e - j
                if not 1 <= i <= N:
                    continue
                owner = (j - 1) // J
                t_x = e - 2 + L * (K - 1) + m * owner
                # the copy lands before the barrier ending the interval after its issue
                lands_by = (interval(t_w, m) + 1) * (m + 1) + m if t_w >= 0 else -1
                assert interval(t_x, m) > interval(lands_by, m), (N, K, C, m, r, e, j)


@pytest.mark.parametrize("m", [0, 1, 2, 3])
@pytest.mark.parametrize("N,K,C", [(128, 20, 4), (398, 31, 13), (512, 20, 16), (698, 13, 16),
                                   (1024, 20, 16), (1024, 2, 16), (512, 1, 16)])
def test_streamed_staging_schedule(N, K, C, m):
    check(N, K, C, m)


def test_schedule_check_catches_a_short_ring():
    """The check fails when the ring is too short for the sweeps in flight."""
    N, K, C, m = 256, 20, 8, 2
    S = N + 2
    L = 2 * m + 3
    lead = 2 * m + 6
    short = L * (K - 1) + 2  # far below (2m + 3) K + 8
    failed = False
    for r in range(C):
        for e in range(2 * S - 1):
            t_last = (e + 1) - 2 + L * (K - 1) + m * r
            t_over = (e + short) - lead + m * r
            if not interval(t_last, m) < interval(t_over, m):
                failed = True
    assert failed
