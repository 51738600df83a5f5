"""Hash-range passes: a rule step run as K passes over hash ranges of its
children (the path of steps beyond one pass: 2^32 children or the device
memory) must give the one-pass step bit for bit -- the same objects in the
same order (bytes, padding included), the same magnitudes, the same total
probability and counters -- with and without truncation, under exact norm
ties at the cutoff (ties keep the lower child index), under probabilistic
truncation, and with modifiers fused after the rule (run())."""
import math

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
U64_MAX = capi.U64_MAX


@pytest.fixture(scope="module")
def ctx():
    c = quids.Context(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def knobs():
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = 1e-18, 8, True
    quids.truncation_seed, quids.hash_ranges = 0, 0
    yield
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = 1e-18, 8, True
    quids.truncation_seed, quids.hash_ranges = 0, 0


def ops_of(gates):
    out = []
    for g in gates:
        if g.kind == "mod":
            out.append(quids.rule_from(False, g.code, g.params))
        else:
            out.append(quids.rule_from(True, g.code, g.params))
    return out


def one_step(ctx, packed, rule, maxn, k):
    quids.hash_ranges = k
    a, b = quids.it_t(ctx, packed), quids.it_t(ctx)
    st = quids.simulate(a, rule, b, quids.sy_it_t(), maxn)
    quids.hash_ranges = 0
    return b.download(), b.total_proba, st


def assert_same(one, ranged, what):
    (p1, t1, s1), (p2, t2, s2) = one, ranged
    for name, x, y in zip(("objects", "begin", "size", "mag"), p1, p2):
        assert x.shape == y.shape and np.array_equal(x, y), f"{what}: {name} differs"
    assert t1 == t2, f"{what}: total_proba {t1!r} != {t2!r}"
    for key in ("num_object", "num_object_after_interferences", "num_object_out", "num_parents_kept"):
        assert s1[key] == s2[key], f"{what}: {key} {s1[key]} != {s2[key]}"


def qcgd_state(ctx, nodes, seed, n_steps, maxn):
    a, b = quids.it_t(ctx, W.qcgd_single_state(nodes, seed=seed)), quids.it_t(ctx)
    fin, _ = quids.run(a, b, ops_of(W.qcgd_step_rules()) * n_steps, maxn)
    return fin.download()


@pytest.mark.parametrize("k", [2, 3, 8])
@pytest.mark.parametrize("maxn", [U64_MAX, 3000, 257])
def test_qcgd_rules_ranges_equal_one_pass(ctx, k, maxn):
    start = qcgd_state(ctx, 8, 5, 1, 20000)
    gates = W.qcgd_step_rules()
    quids.simulate(s := quids.it_t(ctx, start), quids.rules.step)
    packed = s.download()
    for g in gates[1:]:
        rule = quids.rule_from(True, g.code, g.params)
        one = one_step(ctx, packed, rule, maxn, 0)
        ranged = one_step(ctx, packed, rule, maxn, k)
        assert one[2]["hash_ranges"] == 0 and ranged[2]["hash_ranges"] == k
        assert_same(one, ranged, f"rule {g.code}, k={k}, max_num_object={maxn}")
        packed = one_step(ctx, packed, rule, 20000, 0)[0]  # the next rule's input, bounded


@pytest.mark.parametrize("k", [2, 5])
def test_probabilistic_truncation_ranges_equal_one_pass(ctx, k):
    quids.simple_truncation, quids.truncation_seed = False, 1234
    packed = qcgd_state(ctx, 8, 2, 1, 20000)
    rule = quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, (math.pi / 4, 0.0, -math.pi / 2))
    for maxn in (5000, 611):
        assert_same(one_step(ctx, packed, rule, maxn, 0), one_step(ctx, packed, rule, maxn, k),
                    f"probabilistic, k={k}, max_num_object={maxn}")


@pytest.mark.parametrize("k", [2, 4, 16])
def test_exact_ties_at_the_cutoff(ctx, k):
    """Hadamard on every qubit of |0...0>: 2^n children of equal norm, so a
    cap keeps the lowest child indices among exact ties, spread over all
    ranges."""
    n = 11
    packed = W.qc_zero_state(n)
    for q in range(n):
        h = quids.rules.hadamard(q)
        maxn = U64_MAX if q < n - 1 else 700
        one = one_step(ctx, packed, h, maxn, 0)
        assert_same(one, one_step(ctx, packed, h, maxn, k), f"hadamard({q}), k={k}")
        packed = one[0]


def test_zero_elimination_and_interference(ctx):
    """H twice on one qubit of a superposition: every child pair interferes,
    half the groups cancel to zero and are dropped, in every range."""
    packed = W.qc_zero_state(8)
    for q in range(8):
        packed = one_step(ctx, packed, quids.rules.hadamard(q), U64_MAX, 0)[0]
    for q in (3, 3, 5):
        h = quids.rules.hadamard(q)
        one = one_step(ctx, packed, h, U64_MAX, 0)
        assert_same(one, one_step(ctx, packed, h, U64_MAX, 3), f"hadamard({q}) interference")
        packed = one[0]


def test_run_with_fused_modifiers(ctx):
    """run() with the QCGD step's modifier fused after erase_create: ranges
    on every rule give the same final state and per-rule counters."""
    ops = ops_of(W.qcgd_step_rules()) * 3
    res = []
    for k in (0, 3):
        quids.hash_ranges = k
        a, b = quids.it_t(ctx, W.qcgd_single_state(7, seed=9)), quids.it_t(ctx)
        fin, stats = quids.run(a, b, ops, 2000)
        res.append((fin.download(), fin.total_proba, stats))
        quids.hash_ranges = 0
    (p1, t1, s1), (p2, t2, s2) = res
    for x, y in zip(p1, p2):
        assert np.array_equal(x, y)
    assert t1 == t2
    assert [(s["num_object"], s["num_object_after_interferences"], s["num_object_out"]) for s in s1] == \
        [(s["num_object"], s["num_object_after_interferences"], s["num_object_out"]) for s in s2]


def test_automatic_truncation_stays_one_pass(ctx):
    """The automatic truncation (max_num_object = 0) keeps fewer parents
    until one pass fits, so it ignores a request for range passes."""
    packed = W.qc_zero_state(6)
    h = quids.rules.hadamard(2)
    assert_same(one_step(ctx, packed, h, 0, 0), one_step(ctx, packed, h, 0, 4), "automatic truncation")
