"""Planned runs of quids_gpu_run: a repeated gate list runs without host
waits (planned) and then as a replayed CUDA graph.  Every planned or replayed
run must give the synchronous steps' result bit for bit (bytes, magnitudes,
total probability, counters), fall back to the synchronous steps where a step
exceeds its plan, and stop with the synchronous steps' error status."""
import itertools

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
U64_MAX = capi.U64_MAX
COUNTERS = ("num_parents", "num_object", "num_object_after_interferences", "num_object_out", "out_bytes")


@pytest.fixture(scope="module")
def ctx():
    c = quids.Context(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def knobs():
    quids.tolerance, quids.align_byte_length = 1e-18, 8
    yield
    quids.tolerance, quids.align_byte_length = 1e-18, 8


def ops_of(gates):
    return [quids.rule_from(g.kind == "rule", g.code, g.params) for g in gates]


def sync_result(ctx, init, ops, maxn):
    a, b = quids.it_t(ctx, init), quids.it_t(ctx)
    fin, stats = quids.run(a, b, ops, maxn, capi.FLAG_NO_PLAN)
    return fin.download(), fin.total_proba, [{k: s[k] for k in COUNTERS} for s in stats]


def assert_same(got, want, what):
    (gp, gt, gs), (wp, wt, ws) = got, want
    for u, v, name in zip(gp, wp, ("objects", "begin", "size", "magnitude")):
        assert np.array_equal(u, v), f"{what}: {name} differ"
    assert gt == wt, f"{what}: total {gt} != {wt}"
    assert gs == ws, f"{what}: counters differ"


def run_repeated(ctx, inputs, ops, maxn):
    """Runs ops from each input in turn on the same two handles."""
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    out = []
    for init in inputs:
        a.upload(init)
        fin, stats = quids.run(a, b, ops, maxn)
        out.append((fin.download(), fin.total_proba, [{k: s[k] for k in COUNTERS} for s in stats]))
    return out


def counts_delta(ctx, before):
    now = ctx.run_counts()
    return {k: now[k] - before[k] for k in now}


def test_planned_circuit_bit_identical(ctx):
    """The 12-qubit 40-gate circuit, four times: synchronous, planned,
    captured, replayed -- all equal to the synchronous steps."""
    ops = ops_of(W.circuit_small(0))
    init = W.qc_zero_state(12)
    want = sync_result(ctx, init, ops, U64_MAX)
    c0 = ctx.run_counts()
    got = run_repeated(ctx, [init] * 4, ops, U64_MAX)
    for k, g in enumerate(got):
        assert_same(g, want, f"run {k}")
    d = counts_delta(ctx, c0)
    assert d == {"sync": 1, "planned": 3, "graph": 2}, d


def test_planned_truncated_layers(ctx):
    """16 qubits, 4 layers of H on a random half plus CNOT/Z, truncated to
    2^10 objects (the truncation path, exact ties at the cutoff)."""
    gates = [g for layer in W.circuit_layers(5, n_qubits=16, n_layers=4, n_mods=16) for g in layer]
    ops = ops_of(gates)
    init = W.qc_zero_state(16)
    want = sync_result(ctx, init, ops, 1 << 10)
    c0 = ctx.run_counts()
    for k, g in enumerate(run_repeated(ctx, [init] * 4, ops, 1 << 10)):
        assert_same(g, want, f"run {k}")
    assert counts_delta(ctx, c0)["graph"] == 2


@pytest.mark.parametrize("maxn", [U64_MAX, 3000])
def test_planned_qcgd(ctx, maxn):
    """Two QCGD steps (step, coin, split_merge, erase_create) of a 6-node
    graph: the grouped symbolic pass, variable-size children, truncation."""
    ops = ops_of(W.qcgd_step_rules() * 2)
    init = W.qcgd_single_state(6, seed=1)
    want = sync_result(ctx, init, ops, maxn)
    for k, g in enumerate(run_repeated(ctx, [init] * 4, ops, maxn)):
        assert_same(g, want, f"run {k}")


def basis_state(rows, n_qubits=12, mags=None):
    objs = [bytes(int(b) for b in r) for r in rows]
    if mags is None:
        mags = np.full(len(objs), 1 / np.sqrt(len(objs)), np.complex128)
    return W.pack(objs, list(mags), 8)


def two_inputs():
    """Two 1024-object inputs that the ops below take through the same sizes
    for two rule steps, then apart: H0 collapses B's qubit-0 pairs (512
    survivors) but spreads A (2048)."""
    free = [q for q in range(12) if q not in (0, 5)]
    rows_a = []
    for bits in itertools.product((0, 1), repeat=len(free)):
        r = [0] * 12
        for q, v in zip(free, bits):
            r[q] = v
        rows_a.append(r)
    rows_b = []
    for bits in itertools.product((0, 1), repeat=len(free) - 1):
        for q0 in (0, 1):
            r = [0] * 12
            r[0] = q0
            for q, v in zip(free[1:], bits):
                r[q] = v
            rows_b.append(r)
    return basis_state(rows_a), basis_state(rows_b)


def test_replan_resumes_synchronously(ctx):
    """A plan made from input B, then input A, whose third rule step exceeds
    B's bounds: the planned run stops there and resumes synchronously from
    that step's intact input; the result equals the synchronous run.  Later
    runs of A and B use the new plan."""
    a_in, b_in = two_inputs()
    ops = [quids.rules.hadamard(5), quids.rules.hadamard(5), quids.rules.hadamard(0), quids.rules.Xgate(3),
           quids.rules.hadamard(1)]
    want_a = sync_result(ctx, a_in, ops, U64_MAX)
    want_b = sync_result(ctx, b_in, ops, U64_MAX)
    assert want_a[2][2]["num_object_out"] == 2048 and want_b[2][2]["num_object_out"] == 512
    c0 = ctx.run_counts()
    got = run_repeated(ctx, [b_in, b_in, a_in, a_in, a_in, a_in, b_in], ops, U64_MAX)
    for k, (g, w) in enumerate(zip(got, [want_b, want_b, want_a, want_a, want_a, want_a, want_b])):
        assert_same(g, w, f"run {k}")
    d = counts_delta(ctx, c0)
    # sync: the first run and the resumed tail of the third; planned: runs 2-7
    assert d["sync"] == 2 and d["planned"] == 6, d


def test_planned_error_matches_synchronous(ctx):
    """A Hadamard on qubit 12 fits the 13-byte objects of the first input but
    not the 12-byte objects of the second: the planned run returns the
    synchronous steps' error."""
    ops = [quids.rules.hadamard(0), quids.rules.hadamard(12), quids.rules.hadamard(1)]
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    for _ in range(3):
        a.upload(W.qc_zero_state(13))
        quids.run(a, b, ops)
    a.upload(W.qc_zero_state(12))
    with pytest.raises(quids.QuidsError) as planned_err:
        quids.run(a, b, ops)
    x, y = quids.it_t(ctx, W.qc_zero_state(12)), quids.it_t(ctx)
    with pytest.raises(quids.QuidsError) as sync_err:
        quids.run(x, y, ops, U64_MAX, capi.FLAG_NO_PLAN)
    assert planned_err.value.code == sync_err.value.code == -1
    # the context stays usable: the valid input runs again, planned
    a.upload(W.qc_zero_state(13))
    fin, _ = quids.run(a, b, ops)
    x.upload(W.qc_zero_state(13))
    want, _ = quids.run(x, y, ops, U64_MAX, capi.FLAG_NO_PLAN)
    for u, v in zip(fin.download(), want.download()):
        assert np.array_equal(u, v)


# ------------------------------------------------------------ batched form
def batch_case(n_inst, seed, lo=4, hi=8):
    insts = W.qcgd_batch_instances(n_inst, seed, lo, hi)
    packed = [W.pack([g], [1.0 + 0j], 8) for g, _, _ in insts]
    ops = [quids.rules.step, quids.rule_from(True, W.RULE_QCGD_COIN, W.COIN_DEFAULT),
           [quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm) for _, sm, _ in insts],
           [quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec) for _, _, ec in insts]]
    return packed, ops * 2


def batched_result(fin, stats):
    ib, tot = fin.instances()
    return fin.download(), ib, tot, [{k: s[k] for k in COUNTERS} for s in stats]


def test_planned_batched_bit_identical(ctx):
    """Two QCGD steps of 24 instances with per-instance angles, under a
    per-instance cap: planned and replayed batched runs give the synchronous
    batched steps' states, instance offsets and per-instance totals."""
    packed, ops = batch_case(24, 5)
    maxn = 200
    x, y = quids.it_t(ctx), quids.it_t(ctx)
    x.upload_batched(packed)
    want = batched_result(*quids.run_batched(x, y, ops, maxn, capi.FLAG_NO_PLAN))
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    c0 = ctx.run_counts()
    for k in range(4):
        a.upload_batched(packed)
        got = batched_result(*quids.run_batched(a, b, ops, maxn))
        for u, v in zip(got[0], want[0]):
            assert np.array_equal(u, v), f"run {k}: state differs"
        assert np.array_equal(got[1], want[1]), f"run {k}: instance offsets differ"
        assert np.array_equal(got[2], want[2]), f"run {k}: instance totals differ"
        assert got[3] == want[3], f"run {k}: counters differ"
    d = counts_delta(ctx, c0)
    assert d == {"sync": 1, "planned": 3, "graph": 2}, d


def test_planned_batched_replan(ctx):
    """A batched plan made on 4-node graphs, then run on 8-node graphs of the
    same instance count: the bounds are exceeded, the run resumes
    synchronously and equals the synchronous batched run."""
    small, ops_s = batch_case(16, 6, 4, 4)
    big, _ = batch_case(16, 6, 8, 8)
    ops = ops_s
    want = {}
    for name, packed in (("small", small), ("big", big)):
        x, y = quids.it_t(ctx), quids.it_t(ctx)
        x.upload_batched(packed)
        want[name] = batched_result(*quids.run_batched(x, y, ops, U64_MAX, capi.FLAG_NO_PLAN))
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    for k, name in enumerate(["small", "small", "small", "big", "big", "big", "small"]):
        a.upload_batched(small if name == "small" else big)
        got = batched_result(*quids.run_batched(a, b, ops, U64_MAX))
        w = want[name]
        for u, v in zip(got[0], w[0]):
            assert np.array_equal(u, v), f"run {k} ({name}): state differs"
        assert np.array_equal(got[1], w[1]) and np.array_equal(got[2], w[2]), f"run {k} ({name})"
        assert got[3] == w[3], f"run {k} ({name}): counters differ"


# ------------------------------------------------------------ autotuning
def check_tuning(t):
    assert t["trials"] >= 7, t
    assert t["table_load_factor"] in (0.3, 0.5, 0.7) and t["table_block"] in (128, 256, 512), t
    assert t["blocks_per_sm"] in (4, 8, 16) and 0 < t["ms_tuned"] <= t["ms_default"], t


@pytest.mark.parametrize("case", ["circuit", "layers"])
def test_autotuned_runs_bit_identical(ctx, case):
    """QUIDS_FLAG_AUTOTUNE times the planned run under several launch
    configurations before its first capture; every configuration, and so the
    chosen one, gives the synchronous steps' result bit for bit."""
    if case == "circuit":
        ops, init, maxn = ops_of(W.circuit_small(0)), W.qc_zero_state(12), U64_MAX
    else:
        gates = [g for layer in W.circuit_layers(5, n_qubits=16, n_layers=4, n_mods=16) for g in layer]
        ops, init, maxn = ops_of(gates), W.qc_zero_state(16), 1 << 10
    want = sync_result(ctx, init, ops, maxn)
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    c0 = ctx.run_counts()
    for k in range(4):
        a.upload(init)
        fin, stats = quids.run(a, b, ops, maxn, capi.FLAG_AUTOTUNE)
        assert_same((fin.download(), fin.total_proba, [{c: s[c] for c in COUNTERS} for s in stats]), want,
                    f"run {k}")
    check_tuning(ctx.last_tuning())
    assert counts_delta(ctx, c0) == {"sync": 1, "planned": 3, "graph": 2}


def test_autotuned_batched_bit_identical(ctx):
    packed, ops = batch_case(24, 7)
    maxn = 150
    x, y = quids.it_t(ctx), quids.it_t(ctx)
    x.upload_batched(packed)
    want = batched_result(*quids.run_batched(x, y, ops, maxn, capi.FLAG_NO_PLAN))
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    for k in range(4):
        a.upload_batched(packed)
        got = batched_result(*quids.run_batched(a, b, ops, maxn, capi.FLAG_AUTOTUNE))
        for u, v in zip(got[0], want[0]):
            assert np.array_equal(u, v), f"run {k}: state differs"
        assert np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2]), f"run {k}"
        assert got[3] == want[3], f"run {k}: counters differ"
    check_tuning(ctx.last_tuning())
