"""The FP64 free-flight pass streams a free particle through n substeps along one axis
(kernels_fp64.cu, free_stream): runs of integer steps and, between them, the one addition
that crosses a binade or the box edge.  While the partial sums x + j k u stay at least one
unit u inside the binade of x and inside [2^-30 L, L), where the reference's mod is the
identity, and w / u is not halfway between two integers, the round-to-nearest additions
x = mod(x + w, L) give x + j k u with k = round(w / u).  This restates free_stream (its
integer runs, its crossing steps and its fallback to the additions one by one) in Python
and checks it bit for bit against n sequential IEEE double additions with the reference's
mod (numpy float64) on random and adversarial inputs: ties, binade edges, both box edges
(with the wrap), negative, tiny and subnormal displacements."""
import math
import struct

import numpy as np
import pytest


def bits(x):
    return struct.unpack("<q", struct.pack("<d", float(x)))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def lround(q):
    """C lround: to the nearest integer, halfway cases away from zero."""
    t = math.trunc(q)
    if abs(q - t) >= 0.5:
        t += 1 if q > 0 else -1
    return t


def ref_mod(a, L):
    """The reference's mod(a, L) = a - L lround((a - L/2) / L) in double arithmetic."""
    a, L = np.float64(a), np.float64(L)
    q = np.float64(np.float64(a - L * 0.5) / L)
    return float(np.float64(a - np.float64(L * lround(float(q)))))


def sequential(x, w, n, L):
    """n streaming additions as the per-substep passes do them."""
    for _ in range(n):
        x = ref_mod(np.float64(np.float64(x) + np.float64(w)), L)
    return x


MANT, HIDDEN = 0xFFFFFFFFFFFFF, 0x10000000000000


def seg_steps(room, step, left):
    if room < step:
        return 0
    return min(left, room // step)


def free_run(x, w, left, L):
    """The device's integer run: (j steps taken, new x), or None where it does not apply."""
    lo_bits, L_bits = bits(np.ldexp(float(L), -30)), bits(float(L))
    bx, bw = bits(x), bits(w)
    aw = bw & 0x7FFFFFFFFFFFFFFF
    ex, ew = (bx >> 52) & 0x7FF, (aw >> 52) & 0x7FF
    if not (lo_bits <= bx < L_bits and ex > 0 and (aw == 0 or ew > 0)):
        return None
    k = 0
    if aw != 0:
        mw = (aw & MANT) | HIDDEN
        sh = ex - ew
        if sh <= 0:
            if sh <= -8:
                return None
            k = mw << -sh
        elif sh <= 53:
            k = mw >> sh
            rem, half = mw & ((1 << sh) - 1), 1 << (sh - 1)
            if rem == half:
                return None
            k += 1 if rem > half else 0
        if bw < 0:
            k = -k
    if left < 1 or left > 1024:
        return None
    mx = (bx & MANT) | HIDDEN
    lo, hi = HIDDEN + 1, 2 * HIDDEN - 1
    if k == 0:
        n = left
    elif k > 0:
        room = hi - mx
        if (L_bits >> 52) & 0x7FF == ex:
            room = min(room, ((L_bits & MANT) | HIDDEN) - 1 - mx)
        n = seg_steps(room, k, left)
    else:
        room = mx - lo
        if (lo_bits >> 52) & 0x7FF == ex:
            room = min(room, mx - ((lo_bits & MANT) | HIDDEN))
        n = seg_steps(room, -k, left)
    if n > 0:
        x = from_bits((ex << 52) | ((mx + n * k) & MANT))
    return n, x


def free_stream(x, w, n, L, stats=None):
    """The device function: up to three runs with a crossing step after each, then the loop."""
    crossings = 0
    for _ in range(3):
        if n <= 0:
            break
        r = free_run(x, w, n, L)
        if r is None:
            break
        j, x = r
        n -= j
        if n == 0:
            break
        x = ref_mod(np.float64(np.float64(x) + np.float64(w)), L)
        n -= 1
        crossings += 1
    looped = n
    for _ in range(n):
        x = ref_mod(np.float64(np.float64(x) + np.float64(w)), L)
    if stats is not None:
        stats["crossings"] += crossings
        stats["looped"] += looped > 0
    return x


def check(x, w, n=10, L=64.0, stats=None):
    got = free_stream(x, w, n, L, stats)
    ref = sequential(x, w, n, L)
    assert bits(got) == bits(ref), (x, w, n, got, ref)


def test_random_positions_and_displacements():
    rng = np.random.default_rng(5)
    x = rng.uniform(0.0, 64.0, 200000)
    w = rng.normal(0.0, 1.0, x.size) * 0.01  # v dt at kT = m = 1, dt = 0.01
    stats = {"crossings": 0, "looped": 0}
    for a, b in zip(x, w):
        check(a, b, stats=stats)
    # a few per cent of the axis moves cross a binade or the box edge (one addition each);
    # the additions one by one are rare
    assert stats["crossings"] < 0.05 * x.size, stats
    assert stats["looped"] < 0.003 * x.size, stats


def test_binade_and_box_edges():
    n, L = 10, 64.0
    for edge in (0.125, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0, 32.0):
        for d in (1e-12, 1e-6, 0.01, 0.05, 0.2):
            for w in (0.02, -0.02, 0.004, -0.004, 0.3, -0.3):
                check(edge - d, w, n, L)
                check(edge + d, w, n, L)
    for d in (1e-9, 0.01, 0.1, 0.3):
        for w in (0.02, 0.05, -0.02, 0.3):
            check(L - d, w, n, L)  # across the upper edge: the wrap
            check(d, -w, n, L)     # across zero: the wrap
    check(np.nextafter(L, 0.0), 1e-15, n, L)
    check(np.nextafter(L, 0.0), 0.01, n, L)
    check(5e-324, -0.01, n, L)
    check(1e-300, 0.01, n, L)


def test_ties_take_the_loop_and_agree():
    # w exactly half a unit (and odd multiples of it) of x's binade: the integer run refuses
    for x in (33.25, 40.0, 17.5, 3.0):
        u = np.spacing(np.float64(x))
        for m in (0.5, 1.5, 2.5, 1e6 + 0.5):
            assert free_run(x, m * u, 10, 64.0) is None
            assert free_run(x, -m * u, 10, 64.0) is None
            check(x, m * u)
            check(x, -m * u)
        for m in (1.0, 3.0, 1e9):
            check(x, m * u)
            check(x, -m * u)
        check(x, u * 0.25)  # rounds back to x every time
        check(x, 0.0)


def test_tiny_and_subnormal_displacements():
    assert free_run(20.0, 5e-324, 10, 64.0) is None  # subnormal w: the loop
    check(20.0, 5e-324)
    check(20.0, 1e-300)
    check(0.75, 1e-17)


@pytest.mark.parametrize("n", [1, 7, 10, 20])
def test_substep_counts(n):
    rng = np.random.default_rng(n)
    for a, b in zip(rng.uniform(0.0, 64.0, 20000), rng.normal(0.0, 0.02, 20000)):
        check(a, b, n)


@pytest.mark.parametrize("L", [16.0, 48.0, 128.0])
def test_other_box_sizes(L):
    rng = np.random.default_rng(int(L))
    for a, b in zip(rng.uniform(0.0, L, 20000), rng.normal(0.0, 0.02, 20000)):
        check(a, b, 10, L)
