"""Every error status of the rule step, forced without faulting the GPU, and
the context stepping on normally afterwards.

The reference's own failure modes these statuses replace: the allocation
throw (src/utils/vector.hpp:127), the `uint num_child` that wraps to 0 at 32
doubling sites and silently drops the parent's children
(src/rules/qcgd.hpp:480-485, :555-560).  A probe limit, an allocation limit
and a stalled look-back tile are injected through the step's parameters; the
size-bound status comes from a user rule that breaks its contract
(tests/test_gpu_cpp_api.py)."""
import time

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
    saved = (quids.max_probes, quids.max_alloc_bytes, quids.debug_flags, quids.table_load_factor)
    quids.tolerance, quids.align_byte_length = 1e-18, 8
    yield
    quids.max_probes, quids.max_alloc_bytes, quids.debug_flags, quids.table_load_factor = saved


def qubit_state(n_objects, n_qubits=24, seed=5):
    rng = W.Rng(seed)
    objs = list(dict.fromkeys(bytes(rng.below(2) for _ in range(n_qubits)) for _ in range(n_objects + n_objects // 4)))
    objs = objs[:n_objects]
    mags = np.array([complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs])
    return W.pack(objs, mags / np.linalg.norm(mags), 8)


def step(ctx, p, kind=W.RULE_HADAMARD, params=(3,), maxn=U64_MAX):
    a, b, sy = quids.it_t(ctx, p), quids.it_t(ctx), quids.sy_it_t()
    quids.simulate(a, quids.rule_from(True, kind, params), b, sy, maxn)
    return b, sy


def expect_status(code, fn):
    with pytest.raises(capi.QuidsError) as e:
        fn()
    assert e.value.code == code, str(e.value)


def reference_step(ctx, p):
    """the same step with default knobs: the context still works"""
    quids.max_probes = quids.max_alloc_bytes = quids.debug_flags = 0
    quids.table_load_factor = 0.5
    b, sy = step(ctx, p)
    assert sy.num_object == 2 * len(p[2]) and b.num_object > 0
    return b


def test_table_full(ctx):
    """A probe sequence that reaches the limit stops the step with
    QUIDS_ERR_TABLE_FULL: with one probe per child and a table at 90 % load,
    some child's home slot is always taken by another key."""
    p = qubit_state(20000)
    quids.max_probes, quids.table_load_factor = 1, 0.9
    expect_status(capi.ERR_TABLE_FULL, lambda: step(ctx, p))
    # a bounded planned run stops the same way
    ops = [quids.rules.hadamard(3)]
    expect_status(capi.ERR_TABLE_FULL, lambda: quids.run(quids.it_t(ctx, p), quids.it_t(ctx), ops))
    reference_step(ctx, p)


def test_allocation_failure(ctx):
    """A device allocation beyond max_alloc_bytes fails with QUIDS_ERR_OOM
    before cudaMalloc (the reference throws from its allocator); the
    context keeps what it held and steps on once the limit is lifted."""
    p = qubit_state(50000)
    fresh = quids.Context(0)  # no scratch yet: the step's first buffer already exceeds the limit
    try:
        quids.max_alloc_bytes = 4096
        expect_status(capi.ERR_OOM, lambda: step(fresh, p))
        quids.max_alloc_bytes = 0
        b, sy = step(fresh, p)
        assert sy.num_object == 2 * len(p[2])
    finally:
        fresh.close()
    # in a context that has scratch already, only a step needing more fails
    reference_step(ctx, p)
    quids.max_alloc_bytes = 1 << 20
    expect_status(capi.ERR_OOM, lambda: step(ctx, qubit_state(120000, seed=6)))
    reference_step(ctx, p)


def test_child_count_overflow(ctx, port):
    """A parent with 32 doubling sites has 2^32 children, beyond the u32
    child count: the reference's count wraps to 0 and loses the parent's
    children; this library returns QUIDS_ERR_CHILD_COUNT_OVERFLOW."""
    n = 32
    g_ec = W.make_graph(n, [0] * n, [0] * n)   # erase_create: every node has left == right
    g_coin = W.make_graph(n, [1] * n, [0] * n)  # coin: every node has left != right
    for g, kind in ((g_ec, W.RULE_QCGD_ERASE_CREATE), (g_coin, W.RULE_QCGD_COIN)):
        params = (0.3, 0.1, 0.2)
        assert port.num_child(kind, params, g)[0] == 0  # the reference's wrap
        p = W.pack([W.make_graph(4, [1, 0, 0, 1], [0, 0, 1, 1]), g], [0.6, 0.8], 8)
        expect_status(capi.ERR_CHILD_COUNT_OVERFLOW, lambda: step(ctx, p, kind, params))
        # 31 sites is 2^31 children: fine by the count (not run here)
        g31 = W.make_graph(31, [0] * 31, [0] * 31) if kind == W.RULE_QCGD_ERASE_CREATE else \
            W.make_graph(31, [1] * 31, [0] * 31)
        assert port.num_child(kind, params, g31)[0] == 1 << 31
    ok = W.pack([W.make_graph(6, [1, 0, 1, 0, 0, 1], [0, 0, 1, 1, 0, 1])], [1.0], 8)
    b, sy = step(ctx, ok, W.RULE_QCGD_ERASE_CREATE, (0.3, 0.1, 0.2))
    assert sy.num_object == port.num_child(W.RULE_QCGD_ERASE_CREATE, (0.3, 0.1, 0.2), W.unpack(ok)[0][0])[0]
    reference_step(ctx, qubit_state(1000))


def test_bounded_wait_timeout(ctx):
    """A look-back tile whose predecessor never publishes gives up after its
    poll limit: QUIDS_ERR_TIMEOUT, in well under the call's time, with the
    context usable.  (QUIDS_DEBUG_STALL_LOOKBACK makes tile 1 of the
    child-offset scan withhold its prefix; the scan needs 3 tiles or more.)"""
    p = qubit_state(3 * 2048 + 100)
    quids.debug_flags = capi.DEBUG_STALL_LOOKBACK
    t0 = time.perf_counter()
    expect_status(capi.ERR_TIMEOUT, lambda: step(ctx, p))
    waited = time.perf_counter() - t0
    assert waited < 30, f"the bounded wait took {waited:.1f} s"
    print(f"bounded look-back wait gave up after {waited:.2f} s")
    b = reference_step(ctx, p)
    c, _ = step(ctx, p)
    for u, v in zip(b.download(), c.download()):
        assert np.array_equal(u, v)
