"""Pins the CPU oracle (oracle/quids_port.cpp) to the reference.

* against the golden fixtures made by the reference itself
  (tests/golden/make_golden.py runs the reference headers compiled in place);
* live against the compiled reference where its tree is present.
"""
import math
import os

import numpy as np
import pytest

from oracle.oracle import U64_MAX
from quids_gb300 import workloads as W
from tests.parity import assert_state_parity, is_qcgd_kind, load_golden, packed


@pytest.fixture(scope="module")
def golden():
    return load_golden()


def test_port_default_hasher_matches_reference(port, golden):
    z, _ = golden
    data, lens, vals = z["hash_bytes_data"], z["hash_bytes_len"], z["hash_bytes_value"]
    off = 0
    for L, v in zip(lens, vals):
        b = data[off: off + int(L)].tobytes()
        off += int(L)
        assert port.hash_bytes(b) == int(v)


def test_port_qcgd_hash_matches_reference(port, golden):
    z, _ = golden
    objs, _ = W.unpack(packed(z, "graphs"))
    for o, h in zip(objs, z["graphs_hash"]):
        assert port.qcgd_hash_graph(o) == int(h)


def test_port_rule_children_match_reference(port, golden):
    z, man = golden
    for ri, c in enumerate(man["children"]):
        parents, _ = W.unpack(packed(z, f"children{ri}_parents"))
        outs, mags = W.unpack(packed(z, f"children{ri}_out"))
        for o, m, pi, cid in zip(outs, mags, z[f"children{ri}_pid"], z[f"children{ri}_cid"]):
            got, gm = port.populate_child(c["kind"], c["params"], parents[int(pi)], int(cid), mag=(0.6, -0.8))
            if c["kind"] == W.RULE_HADAMARD:
                assert got == o
            else:
                mk = W.graph_padding_mask(o)
                assert len(got) == len(o)
                assert (np.frombuffer(got, np.uint8)[mk] == np.frombuffer(o, np.uint8)[mk]).all()
            assert gm == m


def test_port_steps_match_reference(port, golden):
    z, man = golden
    port.set_threads(1)
    for k, case in enumerate(man["steps"]):
        port.set_globals(case["tolerance"], True, case["align"])
        a = port.new_state(packed(z, f"step{k}_in"))
        b = port.new_state()
        nc, nu = port.simulate(a, case["kind"], case["params"], b, int(case["max"]))
        assert (nc, nu) == (case["num_object"], case["num_object_after_interferences"]), case["name"]
        assert b.total_proba == pytest.approx(case["total_proba"], rel=1e-12, abs=1e-300)
        # one thread: the port restates the reference's exact order, so compare packed layouts too
        got = b.store()
        exp = packed(z, f"step{k}_out")
        assert_state_parity(got, exp, is_qcgd_kind(case["kind"]), truncated=False, what=case["name"])
        assert np.array_equal(got[1], exp[1]), case["name"]
    port.set_globals(1e-18, True, 8)
    port.set_threads(os.cpu_count() or 1)


def _run(o, p, gates, maxn=U64_MAX):
    s = o.new_state(p)
    out = []
    for g in gates:
        if g.kind == "mod":
            o.modifier(s, g.code, g.params)
        else:
            t = o.new_state()
            c = o.simulate(s, g.code, g.params, t, maxn)
            s = t
            out.append(c)
    return s, out


def test_port_matches_live_reference_multithreaded(port, ref):
    """Untruncated trajectories are set-exact across implementations and thread counts."""
    for o in (port, ref):
        o.set_threads(4)
    s1, c1 = _run(ref, W.qcgd_single_state(6, seed=11), W.qcgd_step_rules() * 2)
    s2, c2 = _run(port, W.qcgd_single_state(6, seed=11), W.qcgd_step_rules() * 2)
    assert c1 == c2
    assert_state_parity(s2.store(), s1.store(), True, what="qcgd6 x2")
    layers = W.circuit_layers(0)[:4]
    gates = [g for layer in layers for g in layer]
    s1, c1 = _run(ref, W.qc_zero_state(24), gates, 1 << 22)
    s2, c2 = _run(port, W.qc_zero_state(24), gates, 1 << 22)
    assert c1 == c2
    assert_state_parity(s2.store(), s1.store(), False, what="circuit layers 0-3")
