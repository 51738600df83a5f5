"""The allocation-free children enumeration (quids_gpu_rule_children_noalloc).

Some callers cannot allocate device memory: processes whose device memory is
all owned by another allocator (a pool or a fixed budget that a stray
cudaMalloc would break) and code that cannot pay the implicit device
synchronisation of cudaMalloc/cudaFree.  For them the library offers one
entry point whose scratch is a static device array.  This test calls it
through the C ABI, twice in a row on different states (so the second call
runs on the array the first one left behind), and checks every child against
the allocating entry point quids_gpu_rule_children.  The test file is
collected last and builds its own context, so it runs the same alone in a
fresh process and after the other tests.
"""
import ctypes as C
import math

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, rules, workloads as W
from tests.parity import mag_close

pytestmark = pytest.mark.gpu

NOALLOC_MAX_PARENTS = 1 << 18
ERR_NOALLOC_LIMIT = -10


def _device_arrays(it):
    o, b, s, m = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    capi.check(it.lib.quids_gpu_state_device_arrays(it.h, C.byref(o), C.byref(b), C.byref(s), C.byref(m)))
    return o, b, s, m


def _children_noalloc(ctx, it, rule):
    import torch

    L = ctx.lib
    o, b, s, m = _device_arrays(it)
    p = rule.params()
    n = it.num_object
    nc, stride = C.c_uint64(), C.c_uint64()
    capi.check(L.quids_gpu_rule_children_noalloc(ctx.stream, n, o, b, s, m, rule.kind, C.byref(p), 0,
                                                 C.byref(nc), C.byref(stride), None, None, None, None), "query")
    k, st = nc.value, stride.value
    dev = torch.device("cuda", ctx.device)
    d_bytes = torch.zeros(max(k * st, 1), dtype=torch.uint8, device=dev)
    d_hash = torch.zeros(max(k, 1), dtype=torch.int64, device=dev)
    d_size = torch.zeros(max(k, 1), dtype=torch.int32, device=dev)
    d_mag = torch.zeros(max(2 * k, 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    capi.check(L.quids_gpu_rule_children_noalloc(ctx.stream, n, o, b, s, m, rule.kind, C.byref(p), k,
                                                 C.byref(nc), C.byref(stride), d_bytes.data_ptr(),
                                                 d_hash.data_ptr(), d_size.data_ptr(), d_mag.data_ptr()),
               "enumerate")
    raw = d_bytes.cpu().numpy()
    sizes = d_size.cpu().numpy().view(np.uint32)[:k]
    hashes = d_hash.cpu().numpy().view(np.uint64)[:k]
    mags = d_mag.cpu().numpy().view(np.complex128)[:k]
    children = [raw[i * st: i * st + int(sizes[i])].tobytes() for i in range(k)]
    return children, hashes, mags


def _states():
    rng = W.Rng(31)
    qubits = [bytes(rng.below(2) for _ in range(10)) for _ in range(3000)]
    q_mags = [complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in qubits]
    graphs = [W.random_graph(2 + i % 9, rng) for i in range(30)]
    return [
        # more parents than one scan tile, then far fewer: the second call
        # runs on what the first left in the shared array
        (W.pack(qubits, q_mags, 8), rules.hadamard(3)),
        (W.pack(graphs, [0.6 - 0.8j] * len(graphs), 8), rules.split_merge(math.pi / 4, 0.0, -math.pi / 2)),
    ]


def test_noalloc_children_match_the_allocating_entry_point():
    ctx = quids.Context(0)
    try:
        for packed, rule in _states():
            it = quids.it_t(ctx, packed)
            exp_children, exp_hash, exp_mag = quids.rule_children(it, rule)
            got_children, got_hash, got_mag = _children_noalloc(ctx, it, rule)
            assert len(got_children) == len(exp_children) > 0
            assert got_children == exp_children
            assert np.array_equal(got_hash, exp_hash)
            assert all(mag_close(complex(a), complex(b)) for a, b in zip(got_mag, exp_mag))
    finally:
        ctx.close()


def test_noalloc_rejects_states_beyond_its_scratch():
    ctx = quids.Context(0)
    try:
        n = NOALLOC_MAX_PARENTS + 1
        packed = (np.zeros(8 * n, np.uint8), np.arange(n + 1, dtype=np.uint64) * 8, np.ones(n, np.uint32),
                  np.ones(n, np.complex128))
        it = quids.it_t(ctx, packed)
        o, b, s, m = _device_arrays(it)
        p = rules.hadamard(0).params()
        nc, stride = C.c_uint64(), C.c_uint64()
        rc = ctx.lib.quids_gpu_rule_children_noalloc(ctx.stream, n, o, b, s, m, 1, C.byref(p), 0, C.byref(nc),
                                                     C.byref(stride), None, None, None, None)
        assert rc == ERR_NOALLOC_LIMIT
    finally:
        ctx.close()
