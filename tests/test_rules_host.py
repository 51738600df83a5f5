"""The device rule headers (quids_gb300/csrc/rules_*.cuh) compiled for the
host by g++ and compared with the oracle and the golden fixtures: every
callback (get_num_child, populate_child, populate_child_simple, hash_child,
hasher, modifiers) on the CPU, bit for bit."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from quids_gb300 import workloads as W
from tests.parity import load_golden, packed

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM_SRC = os.path.join(HERE, "shim", "rules_shim.cpp")
SHIM_SO = os.path.join(HERE, "shim", "librules_shim.so")


@pytest.fixture(scope="module")
def shim():
    deps = [SHIM_SRC] + [os.path.join(HERE, "..", "quids_gb300", "csrc", f)
                         for f in ("qd_common.cuh", "rules_qc.cuh", "rules_qcgd.cuh")]
    if not os.path.exists(SHIM_SO) or any(os.path.getmtime(d) > os.path.getmtime(SHIM_SO) for d in deps):
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", SHIM_SO, SHIM_SRC], check=True)
    S = C.CDLL(SHIM_SO)
    for f in ("shim_hash_child", "shim_hash_graph", "shim_murmur"):
        getattr(S, f).restype = C.c_uint64
    S.shim_expand_group.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                    C.c_void_p, C.c_void_p, C.c_void_p]
    S.shim_murmur.argtypes = [C.c_void_p, C.c_uint64]
    return S


def _buf(b: bytes):
    return (C.c_uint8 * max(len(b), 1)).from_buffer_copy(b if b else b"\0")


def _dp(p):
    a = np.asarray(list(p) + [0.0, 0.0, 0.0], dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def test_murmur_is_std_hash(shim):
    z, _ = load_golden()
    data, lens, vals = z["hash_bytes_data"], z["hash_bytes_len"], z["hash_bytes_value"]
    off = 0
    for L, v in zip(lens, vals):
        b = data[off: off + int(L)].tobytes()
        off += int(L)
        assert shim.shim_murmur(_buf(b), len(b)) == int(v)


def test_hash_graph_matches_reference(shim):
    z, _ = load_golden()
    objs, _ = W.unpack(packed(z, "graphs"))
    for o, h in zip(objs, z["graphs_hash"]):
        assert shim.shim_hash_graph(_buf(o)) == int(h)


def _child(shim, kind, params, parent, cid, mag, cap):
    keep, p = _dp(params)
    out = (C.c_uint8 * (cap + 64))()
    sz = C.c_uint32()
    m = (C.c_double * 2)(mag.real, mag.imag)
    shim.shim_populate_child(kind, p, _buf(parent), len(parent), cid, out, C.byref(sz), m)
    return bytes(out)[: sz.value], complex(m[0], m[1])


def test_children_match_golden(shim):
    z, man = load_golden()
    for ri, c in enumerate(man["children"]):
        parents, _ = W.unpack(packed(z, f"children{ri}_parents"))
        outs, mags = W.unpack(packed(z, f"children{ri}_out"))
        for o, m, pi, cid in zip(outs, mags, z[f"children{ri}_pid"], z[f"children{ri}_cid"]):
            par = parents[int(pi)]
            got, gm = _child(shim, c["kind"], c["params"], par, int(cid), 0.6 - 0.8j, 4 * len(par))
            mk = W.graph_padding_mask(o) if c["kind"] != 1 else np.ones(len(o), bool)
            assert len(got) == len(o)
            assert (np.frombuffer(got, np.uint8)[mk] == np.frombuffer(o, np.uint8)[mk]).all()
            assert gm == m
            # fast path: hash, size and magnitude without the bytes
            keep, p = _dp(c["params"])
            sz = C.c_uint32()
            mm = (C.c_double * 2)(0.6, -0.8)
            h = shim.shim_hash_child(c["kind"], p, _buf(par), len(par), int(cid), C.byref(sz), mm)
            if c["kind"] == 1:
                assert h == shim.shim_murmur(_buf(o), len(o))
            else:
                assert h == shim.shim_hash_graph(_buf(o))
            assert sz.value == len(o) and complex(mm[0], mm[1]) == m


@pytest.mark.parametrize("kind", [2, 3, 4])
def test_qcgd_rules_against_oracle_random(shim, port, kind):
    rng = W.Rng(77 + kind)
    graphs = [W.random_graph(n, rng) for n in range(1, 11) for _ in range(4)]
    sm = (math.pi / 4, 0.0, -math.pi / 2)
    for g in graphs[:16]:
        nc, _ = port.num_child(4, sm, g)
        graphs += [port.populate_child(4, sm, g, cid)[0] for cid in range(min(nc, 6))]
    params = [(math.pi / 3, math.pi / 5, 0.0), (0.3, 1.1, 2.2), (2.9, 5.0, 0.7)]
    for gi, g in enumerate(graphs):
        p = params[gi % 3]
        nc, mcs = port.num_child(kind, p, g)
        keep, pp = _dp(p)
        a, b = C.c_uint32(), C.c_uint32()
        shim.shim_num_child(kind, pp, _buf(g), len(g), C.byref(a), C.byref(b))
        assert (a.value, b.value) == (nc, mcs)
        for cid in range(min(nc, 40)):
            exp, em = port.populate_child(kind, p, g, cid, mag=(0.28, 0.96))
            got, gm = _child(shim, kind, p, g, cid, 0.28 + 0.96j, mcs)
            mk = W.graph_padding_mask(exp)
            assert len(got) == len(exp)
            assert (np.frombuffer(got, np.uint8)[mk] == np.frombuffer(exp, np.uint8)[mk]).all()
            assert gm == em


def test_modifiers_match_oracle(shim, port):
    rng = W.Rng(5)
    objs = [bytes(rng.below(2) for _ in range(9)) for _ in range(40)]
    mags = [complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs]
    for kind, params in [(1, (2, 5)), (2, (3,)), (3, (4,)), (4, (0,)), (4, (8,))]:
        st = port.new_state(W.pack(objs, mags, 8))
        port.modifier(st, kind, params)
        eo, em = W.unpack(st.store())
        for o, m, xo, xm in zip(objs, mags, eo, em):
            keep, p = _dp(params)
            b = _buf(o)
            mm = (C.c_double * 2)(m.real, m.imag)
            shim.shim_modifier(kind, p, b, len(o), mm)
            assert bytes(b)[: len(o)] == xo and complex(mm[0], mm[1]) == xm
    graphs = [W.random_graph(n, rng) for n in range(1, 9)]
    for kind in (5, 6):
        st = port.new_state(W.pack(graphs, [1.0] * len(graphs), 8))
        port.modifier(st, kind, ())
        eo, _ = W.unpack(st.store())
        for o, xo in zip(graphs, eo):
            b = _buf(o)
            mm = (C.c_double * 2)(1.0, 0.0)
            keep, p = _dp(())
            shim.shim_modifier(kind, p, b, len(o), mm)
            assert bytes(b)[: len(o)] == xo


@pytest.mark.parametrize("h", [2, 3])
@pytest.mark.parametrize("kind", [W.RULE_QCGD_ERASE_CREATE, W.RULE_QCGD_COIN])
def test_grouped_expansion_is_hash_child_bit_for_bit(shim, kind, h):
    """The grouped symbolic pass (children sharing factor prefixes share
    their products) gives every child's hash and magnitude bit for bit as
    hash_child does, child by child."""
    rng = W.Rng(11)
    keep, pp = _dp((1.1, 0.7, 2.3))
    checked = 0
    for trial in range(60):
        n = 4 + rng.below(13)
        g = W.random_graph(n, rng)
        a, b = C.c_uint32(), C.c_uint32()
        shim.shim_num_child(kind, pp, _buf(g), len(g), C.byref(a), C.byref(b))
        nc = a.value
        if nc < (1 << h):
            continue
        s = nc.bit_length() - 1
        pm = np.array([0.3 + 0.01 * trial, -0.2], np.float64)
        pmp = pm.ctypes.data_as(C.POINTER(C.c_double))
        for e in range(0, 1 << (s - h), max(1, (1 << (s - h)) // 5)):
            hs = np.zeros(1 << h, np.uint64)
            ms = np.zeros(2 << h, np.float64)
            assert shim.shim_expand_group(kind, h, pp, _buf(g), len(g), e, pmp, hs.ctypes.data,
                                          ms.ctypes.data) == s
            for j in range(1 << h):
                cid = e + (j << (s - h))
                mm = (C.c_double * 2)(pm[0], pm[1])
                sz = C.c_uint32()
                hv = shim.shim_hash_child(kind, pp, _buf(g), len(g), cid, C.byref(sz), mm)
                assert hv == int(hs[j]), (trial, e, j)
                assert (mm[0], mm[1]) == (ms[2 * j], ms[2 * j + 1]), (trial, e, j)
                checked += 1
    assert checked > 500


@pytest.mark.parametrize("h", [2, 3])
@pytest.mark.parametrize("params", [(math.pi / 4, 0.0, -math.pi / 2), (0.7, 2.1, 4.4)])
def test_split_merge_grouped_expansion_is_hash_child_bit_for_bit(shim, params, h):
    """split_merge's grouped expansion (siblings share the wrap decisions and
    the walk up to the last H middle sites, which form a tree) gives every
    child's hash, size and magnitude as hash_child does, on graphs whose
    names were split and merged, with and without the wrap sites."""
    rng = W.Rng(77)
    graphs = [W.random_graph(n, rng) for n in range(1, 21) for _ in range(12)]
    for g in graphs[:120]:
        for cid in range(4):
            graphs.append(_child(shim, 4, params, g, cid, 1.0 + 0j, 4 * len(g))[0])
    keep, pp = _dp(params)
    checked, grouped = 0, 0
    for trial, g in enumerate(graphs):
        a, b = C.c_uint32(), C.c_uint32()
        shim.shim_num_child(4, pp, _buf(g), len(g), C.byref(a), C.byref(b))
        nc = a.value
        if nc < (1 << h):
            continue
        s = nc.bit_length() - 1
        pm = np.array([0.3 + 0.001 * trial, -0.2], np.float64)
        pmp = pm.ctypes.data_as(C.POINTER(C.c_double))
        for e in range(0, 1 << (s - h), max(1, (1 << (s - h)) // 7)):
            hs = np.zeros(1 << h, np.uint64)
            ms = np.zeros(2 << h, np.float64)
            assert shim.shim_expand_group(4, h, pp, _buf(g), len(g), e, pmp, hs.ctypes.data, ms.ctypes.data) == s
            for j in range(1 << h):
                cid = e + (j << (s - h))
                mm = (C.c_double * 2)(pm[0], pm[1])
                sz = C.c_uint32()
                hv = shim.shim_hash_child(4, pp, _buf(g), len(g), cid, C.byref(sz), mm)
                assert hv == int(hs[j]), (trial, e, j)
                assert (mm[0], mm[1]) == (ms[2 * j], ms[2 * j + 1]), (trial, e, j)
                checked += 1
            grouped += 1
    print(f"{checked} children in {grouped} groups")
    assert checked > 3000 and grouped > 700


@pytest.mark.parametrize("params", [(math.pi / 4, 0.0, -math.pi / 2), (0.7, 2.1, 4.4)])
def test_split_merge_hash_child_is_populate_then_hash(shim, params):
    """split_merge's hash_child (one pass: wrap decisions, then the walk with
    the site factors applied on the way) gives, for every child of many
    graphs, the hash_graph of populate_child's bytes, its size and its
    magnitude, bit for bit."""
    rng = W.Rng(2024)
    graphs = [W.random_graph(n, rng) for n in range(1, 15) for _ in range(6)]
    for g in graphs[:30]:  # graphs with split and merged names
        for cid in range(3):
            graphs.append(_child(shim, 4, params, g, cid, 1.0 + 0j, 4 * len(g))[0])
    keep, pp = _dp(params)
    checked = 0
    for g in graphs:
        a, b = C.c_uint32(), C.c_uint32()
        shim.shim_num_child(4, pp, _buf(g), len(g), C.byref(a), C.byref(b))
        for cid in range(min(a.value, 64)):
            child, cm = _child(shim, 4, params, g, cid, 0.28 + 0.96j, b.value)
            sz = C.c_uint32()
            mm = (C.c_double * 2)(0.28, 0.96)
            h = shim.shim_hash_child(4, pp, _buf(g), len(g), cid, C.byref(sz), mm)
            assert h == shim.shim_hash_graph(_buf(child))
            assert sz.value == len(child)
            assert complex(mm[0], mm[1]) == cm
            checked += 1
    assert checked > 500
