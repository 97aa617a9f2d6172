"""The FP64 free-flight pass streams a free particle through n substeps along one axis
with an exact shortcut (kernels_fp64.cu, free_stream): when every partial sum x + j k u
stays at least one unit u inside the binade of x and inside [2^-30 L, L), where the
reference's mod is the identity, and w / u is not halfway between two integers, the n
round-to-nearest additions x = mod(x + w, L) give x + n k u with k = round(w / u).  This
restates the shortcut's integer steps in Python and checks them against n sequential
IEEE double additions (numpy float64) on random and adversarial inputs: ties, binade
edges, the box edge, negative and tiny displacements."""
import struct

import numpy as np
import pytest


def bits(x):
    return struct.unpack("<q", struct.pack("<d", float(x)))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def ref_mod_identity_range(L):
    return bits(np.ldexp(float(L), -30)), bits(float(L))


def shortcut(x, w, n, L):
    """The device function's integer steps; None where it takes the additions one by one."""
    lo_bits, L_bits = ref_mod_identity_range(L)
    bx, bw = bits(x), bits(w)
    aw = bw & 0x7FFFFFFFFFFFFFFF
    ex, ew = (bx >> 52) & 0x7FF, (aw >> 52) & 0x7FF
    if not (lo_bits <= bx < L_bits and ex > 0 and (aw == 0 or ew > 0)):
        return None
    k = 0
    if aw != 0:
        mw = (aw & 0xFFFFFFFFFFFFF) | 0x10000000000000
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
    if not (n > 0 and abs(k) < 0x10000000000000 // n):
        return None
    mx = (bx & 0xFFFFFFFFFFFFF) | 0x10000000000000
    mn = mx + n * k
    lo, hi = 0x10000000000000 + 1, 0x20000000000000 - 1
    if not (lo <= mx <= hi and lo <= mn <= hi):
        return None
    bn = (ex << 52) | (mn & 0xFFFFFFFFFFFFF)
    if not (lo_bits <= bn < L_bits):
        return None
    return from_bits(bn)


def sequential(x, w, n, L):
    """n additions as the streaming passes do them (mod is the identity in the fast range)."""
    x = np.float64(x)
    for _ in range(n):
        x = np.float64(x + np.float64(w))
        if not (0 < x < L):  # outside the identity range: the shortcut must not have applied
            return None
    return float(x)


def check(x, w, n=10, L=64.0):
    fast = shortcut(x, w, n, L)
    if fast is None:
        return False
    ref = sequential(x, w, n, L)
    assert ref is not None, (x, w)
    assert bits(fast) == bits(ref), (x, w, fast, ref)
    return True


def test_random_positions_and_displacements():
    rng = np.random.default_rng(5)
    x = rng.uniform(0.0, 64.0, 200000)
    w = rng.normal(0.0, 1.0, x.size) * 0.01  # v dt at kT = m = 1, dt = 0.01
    used = sum(check(a, b) for a, b in zip(x, w))
    assert used > 0.8 * x.size  # most free particles take the shortcut


def test_binade_and_box_edges():
    n, L = 10, 64.0
    for edge in (1.0, 2.0, 4.0, 8.0, 16.0, 32.0):
        for d in (1e-12, 1e-6, 0.01, 0.05, 0.2):
            for w in (0.02, -0.02, 0.004, -0.004):
                check(edge - d, w, n, L)
                check(edge + d, w, n, L)
    for d in (1e-9, 0.01, 0.1, 0.3):
        for w in (0.02, 0.05, -0.02):
            check(L - d, w, n, L)
    check(np.nextafter(L, 0.0), 1e-15, n, L)


def test_ties_and_exact_multiples_take_the_loop_or_agree():
    # w exactly half a unit (and odd multiples of it) of x's binade: the shortcut refuses
    for x in (33.25, 40.0, 17.5, 3.0):
        u = np.spacing(np.float64(x))
        for m in (0.5, 1.5, 2.5, 1e6 + 0.5):
            w = m * u
            assert shortcut(x, w, 10, 64.0) is None
            assert shortcut(x, -w, 10, 64.0) is None
        # exact multiples of the unit, and tiny ones, are exact
        for m in (1.0, 3.0, 1e9):
            assert check(x, m * u)
            assert check(x, -m * u)
        assert check(x, u * 0.25)  # rounds back to x every time
        assert check(x, 0.0)


def test_tiny_and_subnormal_displacements():
    assert shortcut(20.0, 5e-324, 10, 64.0) is None  # subnormal w: the loop
    assert check(20.0, 1e-300)
    assert check(0.75, 1e-17)


@pytest.mark.parametrize("n", [1, 7, 10, 20])
def test_substep_counts(n):
    rng = np.random.default_rng(n)
    for a, b in zip(rng.uniform(0.5, 64.0, 20000), rng.normal(0.0, 0.02, 20000)):
        check(a, b, n)
