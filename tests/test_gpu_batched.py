"""GPU batched form: many independent instances stepped in one pipeline.

Each instance of a batched step must give what the plain GPU step gives on
that instance alone (set parity keyed on bytes, magnitudes within 1e-12
relative) and what the oracle gives; the per-instance totals before
normalisation must match the plain steps' total_proba within 1e-12."""
import math

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W
from tests.parity import assert_state_parity, canon

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
    yield
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = 1e-18, 8, True


def instances(n_inst, seed, lo=4, hi=9):
    """(packed state, split_merge angles, erase_create angles) per instance"""
    out = []
    for g, sm, ec in W.qcgd_batch_instances(n_inst, seed, lo, hi):
        out.append((W.pack([g], [1.0 + 0j], 8), sm, ec))
    return out


def step_ops(sm, ec):
    """the four operations of one QCGD step for one instance"""
    return [quids.rules.step,
            quids.rule_from(True, W.RULE_QCGD_COIN, W.COIN_DEFAULT),
            quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm),
            quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec)]


def plain_steps(ctx, p, sm, ec, n_steps, maxn):
    """one instance through the plain GPU path: packed states after each rule, totals"""
    a = quids.it_t(ctx, p)
    states, totals = [], []
    for _ in range(n_steps):
        for op in step_ops(sm, ec):
            if not op.is_rule:
                quids.simulate(a, op)
                continue
            b = quids.it_t(ctx)
            quids.simulate(a, op, b, quids.sy_it_t(), maxn)
            totals.append(b.total_proba)
            states.append(b.download())
            a = b
    return states, totals


def batched_steps(ctx, insts, n_steps, maxn):
    """all instances through the batched path, rule by rule"""
    a = quids.it_t(ctx)
    a.upload_batched([p for p, _, _ in insts])
    per_rule = []
    for _ in range(n_steps):
        for k, op in enumerate(step_ops((0, 0, 0), (0, 0, 0))):
            if not op.is_rule:
                quids.simulate(a, op)
                continue
            if k == 1:
                rs = [op] * len(insts)
            elif k == 2:
                rs = [quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm) for _, sm, _ in insts]
            else:
                rs = [quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec) for _, _, ec in insts]
            b = quids.it_t(ctx)
            stats, inst_stats = quids.simulate_batched(a, rs, b, maxn)
            ib, tot = b.instances()
            assert b.num_instances == len(insts)
            assert int(ib[-1]) == b.num_object == stats["num_object_out"]
            assert (np.diff(ib.astype(np.int64)) == inst_stats[:, 2].astype(np.int64)).all()
            per_rule.append((b.download_instances(), tot, inst_stats))
            a = b
    return per_rule


# QCGD states grow by orders of magnitude per step without a cap: one
# uncapped step, three capped ones
@pytest.mark.parametrize("maxn,n_steps", [(U64_MAX, 1), (60, 3), (500, 3)])
def test_batched_equals_plain_per_instance(ctx, maxn, n_steps):
    insts = instances(24, seed=2)
    got = batched_steps(ctx, insts, n_steps, maxn)
    for g, (p, sm, ec) in enumerate(insts):
        states, totals = plain_steps(ctx, p, sm, ec, n_steps, maxn)
        assert len(states) == len(got)
        for r, (exp, tot) in enumerate(zip(states, totals)):
            inst_states, inst_tot, inst_stats = got[r]
            what = f"instance {g} rule {r} max {maxn}"
            assert len(exp[2]) == int(inst_stats[g, 2]), what
            assert_state_parity(inst_states[g], exp, True, truncated=maxn != U64_MAX, what=what)
            assert inst_tot[g] == pytest.approx(tot, rel=1e-12, abs=1e-300), what


@pytest.mark.parametrize("maxn,n_steps", [(U64_MAX, 1), (40, 2)])
def test_batched_against_oracle(ctx, port, maxn, n_steps):
    """every rule of every instance against the oracle, from the same input
    (the batched state before that rule)"""
    insts = instances(6, seed=5, lo=4, hi=7)
    got = batched_steps(ctx, insts, n_steps, maxn)
    for g, (p, sm, ec) in enumerate(insts):
        ops = [op for op in step_ops(sm, ec) if op.is_rule] * n_steps
        for r, op in enumerate(ops):
            a = port.new_state(p if r == 0 else got[r - 1][0][g])
            if r % 3 == 0:
                port.modifier(a, W.MOD_QCGD_STEP, ())
            b = port.new_state()
            nc, nu = port.simulate(a, op.kind, (op.theta, op.phi, op.xi), b, maxn)
            inst_states, _, inst_stats = got[r]
            assert (int(inst_stats[g, 0]), int(inst_stats[g, 1])) == (nc, nu), f"instance {g} rule {r}"
            assert_state_parity(inst_states[g], b.store(), True, truncated=maxn != U64_MAX,
                                what=f"oracle instance {g} rule {r}")


def test_batched_hadamard_and_modifiers(ctx):
    """qubit instances with a different Hadamard bit per instance; a modifier
    acts on every instance; an empty instance stays empty."""
    quids.align_byte_length = 8
    states = [W.qc_zero_state(6), W.pack([], [], 8), W.qc_zero_state(6), W.qc_zero_state(6)]
    a = quids.it_t(ctx)
    a.upload_batched(states)
    quids.simulate(a, quids.rules.Xgate(1))
    bits = [0, 0, 3, 5]
    for step in range(3):
        b = quids.it_t(ctx)
        quids.simulate_batched(a, [quids.rules.hadamard((bi + step) % 6) for bi in bits], b)
        a = b
    inst = a.download_instances()
    assert len(inst[1][2]) == 0
    for g in (0, 2, 3):
        p = quids.it_t(ctx, W.qc_zero_state(6))
        quids.simulate(p, quids.rules.Xgate(1))
        for step in range(3):
            q = quids.it_t(ctx)
            quids.simulate(p, quids.rules.hadamard((bits[g] + step) % 6), q, quids.sy_it_t())
            p = q
        assert_state_parity(inst[g], p.download(), False, what=f"hadamard instance {g}")


def test_batched_single_instance_and_plain_output(ctx):
    """one instance equals the plain step; a plain step of a batched state
    gives a plain state"""
    p = W.qcgd_single_state(8, seed=4)
    a = quids.it_t(ctx)
    a.upload_batched([p])
    quids.simulate(a, quids.rule_from(False, W.MOD_QCGD_STEP, ()))
    b = quids.it_t(ctx)
    quids.simulate_batched(a, [quids.rules.split_merge(math.pi / 4, 0.0, -math.pi / 2)], b)
    c = quids.it_t(ctx, p)
    quids.simulate(c, quids.rule_from(False, W.MOD_QCGD_STEP, ()))
    d = quids.it_t(ctx)
    quids.simulate(c, quids.rules.split_merge(math.pi / 4, 0.0, -math.pi / 2), d, quids.sy_it_t())
    assert_state_parity(b.download_instances()[0], d.download(), True, what="single instance")
    e = quids.it_t(ctx)
    quids.simulate(b, quids.rules.coin(math.pi / 4), e, quids.sy_it_t())
    assert e.num_instances == 0


def test_batched_run_equals_rule_by_rule(ctx):
    insts = instances(10, seed=7)
    a = quids.it_t(ctx)
    a.upload_batched([p for p, _, _ in insts])
    ops = []
    for _ in range(2):
        ops += [quids.rule_from(False, W.MOD_QCGD_STEP, ()),
                quids.rule_from(True, W.RULE_QCGD_COIN, W.COIN_DEFAULT),
                [quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm) for _, sm, _ in insts],
                [quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec) for _, _, ec in insts]]
    fin, stats = quids.run_batched(a, quids.it_t(ctx), ops, 80)
    assert len(stats) == 6
    ref = batched_steps(ctx, insts, 2, 80)
    got = fin.download_instances()
    for g in range(len(insts)):
        assert_state_parity(got[g], ref[-1][0][g], True, what=f"run_batched instance {g}")


def test_batched_bad_arguments(ctx):
    lib = capi.load()
    p = W.qcgd_single_state(5, seed=1)
    objects, begin, size, mag = p
    st = quids.it_t(ctx)
    ib = np.array([0, 2], np.uint64)  # ends beyond the one object
    rc = lib.quids_gpu_state_upload_batched(st.h, 1, objects.ctypes.data, begin.ctypes.data, size.ctypes.data,
                                            np.ascontiguousarray(mag).ctypes.data, len(objects), 1,
                                            ib.ctypes.data)
    assert rc == -1  # QUIDS_ERR_BAD_ARG
    plain = quids.it_t(ctx, p)
    with pytest.raises(quids.QuidsError):
        quids.simulate_batched(plain, [], quids.it_t(ctx))
    a = quids.it_t(ctx)
    a.upload_batched([p, p])
    with pytest.raises(quids.QuidsError) as e:
        quids.simulate_batched(a, [quids.rules.coin(1.0)] * 2, quids.it_t(ctx), 0)
    assert e.value.code == -9  # QUIDS_ERR_UNSUPPORTED


def test_batched_bit_identical_to_plain(ctx):
    """Normalisation is exact in both paths with the same fixed-point scale
    per instance, so each instance's survivors and magnitudes are the plain
    step's, bit for bit (and so are the trajectories under truncation)."""
    insts = instances(12, seed=9)
    got = batched_steps(ctx, insts, 3, 100)
    for g, (p, sm, ec) in enumerate(insts):
        states, totals = plain_steps(ctx, p, sm, ec, 3, 100)
        for r, (exp, tot) in enumerate(zip(states, totals)):
            inst_states, inst_tot, _ = got[r]
            a, b = canon(inst_states[g], True), canon(exp, True)
            assert a == b, f"instance {g} rule {r}: not bit-identical"
            assert inst_tot[g] == tot, f"instance {g} rule {r}: total {inst_tot[g]!r} vs {tot!r}"
