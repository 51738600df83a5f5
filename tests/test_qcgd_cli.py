"""The QCGD simulation string (src/rules/qcgd.hpp:1038-1177): the restated
C library rand(), the state and rule parsing against the reference's own
flags::read_state / flags::read_rule (compiled in place, where the
reference tree is present), and one driven simulation on the GPU against
the oracle."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from quids_gb300 import qcgd_cli as Q
from quids_gb300 import workloads as W
from tests.parity import canon


def test_crand_is_the_c_library_rand():
    try:
        libc = C.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no libc.so.6")
    for seed in (0, 1, 7, 12345, 2**31 + 5):
        libc.srand(C.c_uint(seed))
        r = Q.CRand(seed)
        assert [r.rand() for _ in range(3000)] == [libc.rand() for _ in range(3000)], seed


def test_parse_settings_and_defaults():
    s = Q.read_n_iter("12,seed=3,reversed_n_iter=2,tolerance=1e-15,align=4,simple_truncate=0,max_num_object=500")
    assert (s.n_iter, s.seed, s.reversed_n_iter, s.align, s.simple_truncation, s.max_num_object) == \
        (12, 3, 2, 4, False, 500)
    assert s.tolerance == float(np.float32(1e-15))
    d = Q.read_n_iter("5")
    assert (d.n_iter, d.seed, d.reversed_n_iter, d.align, d.simple_truncation, d.max_num_object) == \
        (5, None, 0, 8, True, 0)
    rules = Q.read_rule("step;coin;split_merge,theta=0.3,xi=0.5,n_iter=3;bogus;reversed_step")
    assert [(r.name, r.n_iter, r.is_rule) for r in rules] == \
        [("step", 1, False), ("coin", 1, True), ("split_merge", 3, True), ("reversed_step", 1, False)]
    assert rules[1].theta == float(np.float32(math.pi * np.float32(0.25)))
    assert rules[2].xi == float(np.float32(math.pi * np.float32(0.5)))


@pytest.fixture(scope="module")
def ref_lib():
    from oracle import oracle as orc
    if not os.path.isdir(os.path.join(orc.REFERENCE_TREE, "src")):
        pytest.skip("reference tree not present")
    o = orc.Oracle("ref")
    L = o.lib
    L.qo_ref_read_state.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p]
    L.qo_ref_read_rules.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
    return o


@pytest.mark.parametrize("settings,state", [
    ("2,seed=7", "6"),
    ("1,seed=1,align=8", "6;4,n_graphs=3,real=0.5,imag=0.25;9,n_graphs=2"),
    ("3,seed=99", "12,n_graphs=5,imag=1"),
])
def test_read_state_matches_reference(ref_lib, settings, state):
    st = ref_lib.new_state()
    ref_lib.lib.qo_ref_read_state(settings.encode(), state.encode(), st.h)
    exp = st.store()
    s = Q.read_n_iter(settings)
    got = Q.read_state(state, Q.CRand(s.seed), s.align)
    assert len(got[2]) == len(exp[2])
    g, e = canon(got, True), canon(exp, True)
    assert g == e   # bytes (padding masked) and magnitudes, exactly


def test_read_rules_matches_reference(ref_lib, port):
    arg = "step;coin;split_merge,theta=0.3,phi=0.1,xi=0.7,n_iter=2;erase_create,xi=-0.2,theta=0.4;reversed_step"
    probe = W.make_graph(6, [1, 0, 1, 1, 0, 0], [1, 1, 0, 1, 0, 1])
    buf = (C.c_uint8 * len(probe)).from_buffer_copy(probe)
    n_iter = np.zeros(8, np.int32)
    is_rule = np.zeros(8, np.int32)
    out = np.zeros(8 * 8 * 2, np.float64)
    n = ref_lib.lib.qo_ref_read_rules(arg.encode(), buf, len(probe), 8, n_iter.ctypes.data, is_rule.ctypes.data,
                                      out.ctypes.data)
    rules = Q.read_rule(arg)
    assert n == len(rules)
    codes = {"erase_create": W.RULE_QCGD_ERASE_CREATE, "coin": W.RULE_QCGD_COIN,
             "split_merge": W.RULE_QCGD_SPLIT_MERGE}
    for k, r in enumerate(rules):
        assert (int(n_iter[k]), bool(is_rule[k])) == (r.n_iter, r.is_rule)
        if not r.is_rule:
            continue
        for v, xi in enumerate((r.xi, -r.xi)):
            nc, _ = port.num_child(codes[r.name], (r.theta, r.phi, xi), probe)
            for c in range(min(nc, 4)):
                _, m = port.populate_child(codes[r.name], (r.theta, r.phi, xi), probe, c, mag=(1.0, 0.0))
                e = complex(out[((k * 8) + v * 4 + c) * 2], out[((k * 8) + v * 4 + c) * 2 + 1])
                assert m == e, (r.name, v, c)


@pytest.mark.gpu
def test_driven_simulation_matches_oracle(port):
    import quids_gb300 as quids
    arg = "2,seed=5,reversed_n_iter=1,tolerance=1e-18,max_num_object=100000|5;4,n_graphs=2|" \
          "step;coin;split_merge,theta=0.3,xi=0.2;erase_create,theta=0.3333"
    sim = Q.parse_simulation(arg)
    ctx = quids.Context(0)
    try:
        fin, results = Q.run(sim, ctx, report=lambda r: None)
        assert len(results) == 3
        got = fin.download()
        port.set_globals(sim.settings.tolerance, True, sim.settings.align)
        s = port.new_state(sim.state)
        for it in range(3):
            for op in Q.iteration_ops(sim, it >= 2):
                if not op.is_rule:
                    port.modifier(s, op.kind, ())
                else:
                    t = port.new_state()
                    port.simulate(s, op.kind, (op.theta, op.phi, op.xi), t, 100000)
                    s = t
        from tests.parity import assert_state_parity
        assert_state_parity(got, s.store(), True, what="driven simulation")
        assert results[-1]["total_proba"] == pytest.approx(s.total_proba, rel=1e-12)
    finally:
        ctx.close()
        port.set_globals(1e-18, True, 8)
