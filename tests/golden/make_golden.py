"""Generates tests/golden/golden.npz from the reference itself.

Runs the reference headers compiled in place (oracle/_ref/libquids_ref.so,
built by ``make -C oracle ref`` from the reference tree) with one OpenMP
thread, on seeded inputs from quids_gb300.workloads, and stores inputs,
outputs and counters.  Re-run with:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, U64_MAX  # noqa: E402
from quids_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "golden.npz")


class Store:
    def __init__(self):
        self.arrays = {}
        self.manifest = {"steps": [], "hash_bytes": None, "qcgd_hash": None, "children": []}

    def packed(self, prefix, packed):
        objects, begin, size, mag = packed
        self.arrays[prefix + "_objects"] = np.asarray(objects, np.uint8)
        self.arrays[prefix + "_begin"] = np.asarray(begin, np.uint64)
        self.arrays[prefix + "_size"] = np.asarray(size, np.uint32)
        self.arrays[prefix + "_mag"] = np.asarray(mag, np.complex128)


def step_case(st: Store, ref: Oracle, name, packed, kind, params, maxn=U64_MAX, tol=1e-18, align=8):
    ref.set_globals(tol, True, align)
    a = ref.new_state(packed)
    b = ref.new_state()
    nc, nu = ref.simulate(a, kind, params, b, maxn)
    out = b.store()
    k = len(st.manifest["steps"])
    st.packed(f"step{k}_in", packed)
    st.packed(f"step{k}_out", out)
    st.manifest["steps"].append({"name": name, "kind": kind, "params": list(params), "max": str(maxn),
                                 "tolerance": tol, "align": align, "num_object": nc,
                                 "num_object_after_interferences": nu, "total_proba": b.total_proba})
    ref.set_globals(1e-18, True, 8)
    return out


def main():
    ref = Oracle("ref")
    ref.set_threads(1)
    ref.set_globals(1e-18, True, 8)
    st = Store()
    rng = W.Rng(20240601)

    # 1. default hasher (std::hash<std::string_view>) known answers
    blobs = [bytes(rng.below(256) for _ in range(L)) for L in list(range(0, 40)) + [63, 64, 65, 127, 255]]
    st.arrays["hash_bytes_data"] = np.frombuffer(b"".join(blobs), np.uint8).copy() if blobs else np.zeros(0, np.uint8)
    st.arrays["hash_bytes_len"] = np.array([len(b) for b in blobs], np.uint64)
    st.arrays["hash_bytes_value"] = np.array([ref.hash_bytes(b) for b in blobs], np.uint64)

    # 2. QCGD graph hash known answers, on graphs grown by split_merge
    graphs = [W.random_graph(n, rng) for n in range(1, 13)]
    sm = (math.pi / 4, 0.0, -math.pi / 2)
    for g in list(graphs[:8]):
        nc, _ = ref.num_child(4, sm, g)
        for cid in range(min(nc, 4)):
            graphs.append(ref.populate_child(4, sm, g, cid)[0])
    gp = W.pack(graphs, [1.0] * len(graphs), 8)
    st.packed("graphs", gp)
    st.arrays["graphs_hash"] = np.array([ref.qcgd_hash_graph(g) for g in graphs], np.uint64)

    # 3. rule callbacks: every child of a few parents
    rules = [(1, (2.0,)), (2, (math.pi / 3, math.pi / 5, 0.0)), (3, W.COIN_DEFAULT), (4, sm),
             (4, (0.3, 1.1, 2.2)), (2, (2.0, 4.0, 5.5))]
    for ri, (kind, params) in enumerate(rules):
        parents = [bytes([0, 1, 1, 0, 1])] if kind == 1 else graphs[3:12]
        objs, mags, pid, cids = [], [], [], []
        for pi, g in enumerate(parents):
            nc, _ = ref.num_child(kind, params, g)
            for cid in range(min(nc, 32)):
                c, m = ref.populate_child(kind, params, g, cid, mag=(0.6, -0.8))
                objs.append(c)
                mags.append(m)
                pid.append(pi)
                cids.append(cid)
        st.packed(f"children{ri}_parents", W.pack(parents, [0.6 - 0.8j] * len(parents), 8))
        st.packed(f"children{ri}_out", W.pack(objs, mags, 8))
        st.arrays[f"children{ri}_pid"] = np.array(pid, np.uint32)
        st.arrays[f"children{ri}_cid"] = np.array(cids, np.uint32)
        st.manifest["children"].append({"kind": kind, "params": list(params)})

    # 4. rule steps
    # 4a. the small circuit, gate by gate (no truncation)
    gates = W.circuit_small(0)
    state = W.qc_zero_state(12)
    ref.set_globals(1e-18, True, 8)
    s = ref.new_state(state)
    for gi, g in enumerate(gates):
        if g.kind == "mod":
            ref.modifier(s, g.code, g.params)
            continue
        step_case(st, ref, f"circuit_small_gate{gi}", s.store(), g.code, g.params)
        t = ref.new_state()
        ref.simulate(s, g.code, g.params, t)
        s = t
    # 4b. a uniform superposition truncated: exact ties at the cutoff
    s = ref.new_state(W.qc_zero_state(12))
    for q in range(11):
        t = ref.new_state()
        ref.simulate(s, 1, (q,), t)
        s = t
    step_case(st, ref, "hadamard_ties_truncated", s.store(), 1, (11,), maxn=1000)
    # 4c. a state with unequal norms, truncated
    objs = [bytes(rng.below(2) for _ in range(10)) for _ in range(300)]
    objs = list(dict.fromkeys(objs))
    mags = np.array([complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs])
    mags /= np.linalg.norm(mags)
    step_case(st, ref, "hadamard_random_truncated", W.pack(objs, mags, 8), 1, (4,), maxn=150)
    step_case(st, ref, "hadamard_random_parent_truncation", W.pack(objs, mags, 8), 1, (4,), maxn=100)
    # 4d. QCGD steps on small graphs, no truncation
    qs = W.qcgd_single_state(5, seed=1)
    ref.set_globals(1e-18, True, 8)
    s = ref.new_state(qs)
    for rep in range(2):
        for g in W.qcgd_step_rules():
            if g.kind == "mod":
                ref.modifier(s, g.code, g.params)
                continue
            step_case(st, ref, f"qcgd5_step{rep}_{g.code}", s.store(), g.code, g.params)
            t = ref.new_state()
            ref.simulate(s, g.code, g.params, t)
            s = t
    # 4e. QCGD truncated, and with other alignments
    qs = W.qcgd_single_state(7, seed=3)
    s = ref.new_state(qs)
    for g in W.qcgd_step_rules():
        if g.kind == "mod":
            ref.modifier(s, g.code, g.params)
            continue
        t = ref.new_state()
        ref.simulate(s, g.code, g.params, t)
        s = t
    base = s.store()
    step_case(st, ref, "qcgd7_split_merge_truncated", base, 4, (math.pi / 4, 0.0, -math.pi / 2), maxn=500)
    for al in (0, 1, 4, 16):
        objs_, mags_ = W.unpack(base)
        step_case(st, ref, f"qcgd7_coin_align{al}", W.pack(objs_, mags_, al), 3, W.COIN_DEFAULT, align=al)
    # 4f. interference to zero: |0> and |1> halves that cancel under H
    p = W.pack([bytes([0, 0, 1]), bytes([1, 0, 1])], [1 / math.sqrt(2), 1 / math.sqrt(2)], 8)
    step_case(st, ref, "hadamard_cancel", p, 1, (0,))
    # 4g. empty state
    step_case(st, ref, "empty", W.pack([], [], 8), 1, (0,))

    st.arrays["manifest"] = np.frombuffer(json.dumps(st.manifest).encode(), np.uint8).copy()
    np.savez_compressed(OUT, **st.arrays)
    print(OUT, os.path.getsize(OUT), "bytes,", len(st.manifest["steps"]), "step cases")


if __name__ == "__main__":
    main()
