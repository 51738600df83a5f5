"""The exact collision sums (quids_gb300/csrc/qd_common.cuh: to_fix,
fix_add, from_fix, fix_scale), compiled for the host from the same source the
kernels use: a group's sum is the exact sum of its members rounded once to
the nearest double (ties to even), whatever the order of the members, and
the scale leaves room for the step's whole child count."""
import ctypes as C
import random
from fractions import Fraction

import numpy as np
import pytest

from tests.test_rules_host import shim  # noqa: F401  (the host build of the device headers)


def fix_sum(shim, xs, maxabs=None, n_scale=None):
    a = np.ascontiguousarray(xs, dtype=np.float64)
    if maxabs is None:
        maxabs = float(np.max(np.abs(a))) if len(a) else 0.0
    F = C.c_int()
    shim.shim_fix_sum.restype = C.c_double
    shim.shim_fix_sum.argtypes = [C.c_void_p, C.c_uint64, C.c_double, C.c_uint64, C.POINTER(C.c_int)]
    return shim.shim_fix_sum(a.ctypes.data, len(a), maxabs, n_scale or max(len(a), 1), C.byref(F)), F.value


def exact(xs):
    return float(sum(Fraction(x) for x in xs))


def random_terms(rng, n, span=40):
    top = rng.randint(-30, 30)
    return [rng.choice((-1.0, 1.0)) * rng.random() * 2.0 ** (top - rng.randint(0, span)) for _ in range(n)]


def test_sum_is_the_correctly_rounded_exact_sum(shim):
    rng = random.Random(7)
    for trial in range(400):
        xs = random_terms(rng, rng.randint(2, 64))
        if trial % 4 == 0:  # near cancellation
            xs.append(-sum(xs[:-1]))
        got, _ = fix_sum(shim, xs)
        want = exact(xs)
        assert got == want or (got == 0.0 and want == 0.0), (trial, got, want)


def test_sum_does_not_depend_on_the_order(shim):
    rng = random.Random(11)
    for _ in range(100):
        xs = random_terms(rng, 48)
        ref = fix_sum(shim, xs)[0]
        for _ in range(5):
            rng.shuffle(xs)
            assert fix_sum(shim, xs)[0] == ref


@pytest.mark.parametrize("xs,want", [
    ([1.0, 2.0 ** -53], 1.0),                               # halfway: down to the even neighbour
    ([1.0, 3 * 2.0 ** -53], 1.0 + 2.0 ** -51),              # halfway: up to the even neighbour
    ([1.0, 2.0 ** -53, 2.0 ** -60], 1.0 + 2.0 ** -52),      # above halfway by the sticky bits
    ([0.5, -0.5], 0.0),
    ([-1.0, -2.0 ** -53], -1.0),
])
def test_rounding_of_ties_and_cancellation(shim, xs, want):
    assert fix_sum(shim, xs)[0] == want


def test_scale_leaves_room_for_every_child_of_the_step(shim):
    """F comes from the largest component and the step's child count, so n
    terms of the largest magnitude sum without overflow."""
    x = np.nextafter(0.75, 0.0)
    n = 1 << 20
    got, F = fix_sum(shim, np.full(n, x), maxabs=x, n_scale=n)
    assert got == x * n
    got_neg, _ = fix_sum(shim, np.full(n, -x), maxabs=x, n_scale=n)
    assert got_neg == -x * n
    # a group of a few members in a large step uses the step's scale: still exact here
    xs = [0.25, 2.0 ** -30, -2.0 ** -31]
    assert fix_sum(shim, xs, maxabs=0.75, n_scale=1 << 32)[0] == exact(xs)
