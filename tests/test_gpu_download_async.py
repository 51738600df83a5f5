"""Asynchronous downloads (quids_gpu_state_download_async / _wait): the
copies run on the context's copy stream while later work runs, give the
synchronous download's bytes, and are never overwritten by work issued after
them on the same state (that work waits for the copies on the device)."""
import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu


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


def host_buffers(st, pinned=True):
    import torch
    n, nb = st.num_object, st.num_bytes
    mk = (lambda k, t: torch.empty(k, dtype=t).pin_memory()) if pinned else (lambda k, t: torch.empty(k, dtype=t))
    return (mk(max(nb, 1), torch.uint8), mk(n + 1, torch.int64), mk(max(n, 1), torch.int32),
            mk(max(n, 1), torch.complex128))


def as_packed(bufs, st):
    n, nb = st.num_object, st.num_bytes
    o, b, s, m = (t.numpy() for t in bufs)
    return o[:nb], b.view(np.uint64)[: n + 1], s.view(np.uint32)[:n], m[:n]


def assert_same(got, exp):
    for g, e in zip(got, exp):
        assert np.array_equal(np.asarray(g), np.asarray(e))


def qcgd_state(ctx, nodes, seed):
    it = quids.it_t(ctx, W.qcgd_single_state(nodes, seed=seed))
    nxt, sy = quids.it_t(ctx), quids.sy_it_t()
    quids.simulate(it, quids.rules.step)
    quids.simulate(it, quids.rules.coin(np.pi / 4), nxt, sy)
    out = quids.it_t(ctx)
    quids.simulate(nxt, quids.rules.split_merge(np.pi / 4, 0.0, -np.pi / 2), out, sy)
    return out


@pytest.mark.parametrize("pinned", [True, False])
def test_async_download_equals_sync(ctx, pinned):
    st = qcgd_state(ctx, 8, 2)
    exp = st.download()
    bufs = host_buffers(st, pinned)
    st.download_async(*bufs)
    st.download_wait()
    assert_same(as_packed(bufs, st), exp)


def test_work_after_an_async_download_waits_for_it(ctx):
    """Overwriting the state right after download_async (an upload of other
    objects, then a rule step into it) must not change what the copies read."""
    st = qcgd_state(ctx, 10, 3)
    n, nb = st.num_object, st.num_bytes
    exp = st.download()
    bufs = host_buffers(st)
    st.download_async(*bufs)
    other = W.qcgd_single_state(6, seed=9)
    st.upload(other)  # waits for the copies on the device, then overwrites
    tmp = quids.it_t(ctx, other)
    quids.simulate(tmp, quids.rules.coin(np.pi / 3), st, quids.sy_it_t())
    st.download_wait()
    o, b, s, m = (t.numpy() for t in bufs)
    assert_same((o[:nb], b.view(np.uint64)[: n + 1], s.view(np.uint32)[:n], m[:n]), exp)


def test_pipelined_steps(ctx):
    """Two state pairs: each step's result downloads while the next step runs;
    every result equals the synchronous step's."""
    wl_gates = W.qcgd_step_rules()
    ops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in wl_gates]
    inputs = [W.qcgd_single_state(9, seed=s) for s in (4, 5, 6, 7, 8)]
    expected = []
    for inp in inputs:
        a, b = quids.it_t(ctx, inp), quids.it_t(ctx)
        fin, _ = quids.run(a, b, ops, 1 << 16, capi.FLAG_NO_PLAN)
        expected.append(fin.download())
    pairs = [(quids.it_t(ctx), quids.it_t(ctx)) for _ in range(2)]
    pending = [None, None]
    got = [None] * len(inputs)
    for i, inp in enumerate(inputs):
        k = i % 2
        if pending[k] is not None:
            j, fin, bufs = pending[k]
            fin.download_wait()
            got[j] = as_packed(bufs, fin)
        a, b = pairs[k]
        a.upload(inp)
        fin, _ = quids.run(a, b, ops, 1 << 16)
        bufs = host_buffers(fin)
        fin.download_async(*bufs)
        pending[k] = (i, fin, bufs)
    for p in pending:
        if p is not None:
            j, fin, bufs = p
            fin.download_wait()
            got[j] = as_packed(bufs, fin)
    for g, e in zip(got, expected):
        assert_same(g, e)


def test_small_buffers_are_refused(ctx):
    st = qcgd_state(ctx, 6, 1)
    import torch
    bufs = list(host_buffers(st))
    bufs[0] = torch.empty(1, dtype=torch.uint8)
    with pytest.raises(ValueError):
        st.download_async(*bufs)
