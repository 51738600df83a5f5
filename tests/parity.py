"""Parity helpers: golden fixture access and state comparison.

A state is compared as a set keyed on object bytes (the reference's output
order and collision representative depend on its thread count), with QCGD
name-sub-node padding masked (never initialised by the reference,
src/rules/qcgd.hpp:35-61).  Magnitudes must agree within
|d| <= 1e-12 * max(|m|, 1e-9) (relative 1e-12, floored at sqrt(tolerance)).
Under truncation, objects whose norm lies within 1e-12 (relative) of the
cutoff norm form a tie band: outside the band the sets must be equal, inside
only the counts.
"""
from __future__ import annotations

import json
import os

import numpy as np

from quids_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")
REL = 1e-12
FLOOR = 1e-9


def load_golden():
    z = np.load(GOLDEN)
    manifest = json.loads(bytes(z["manifest"]).decode())
    return z, manifest


def packed(z, prefix):
    return (z[prefix + "_objects"], z[prefix + "_begin"], z[prefix + "_size"], z[prefix + "_mag"])


def is_qcgd_kind(kind: int) -> bool:
    return kind in (W.RULE_QCGD_ERASE_CREATE, W.RULE_QCGD_COIN, W.RULE_QCGD_SPLIT_MERGE)


def canon(p, qcgd: bool):
    objs, mags = W.unpack(p)
    out = {}
    for o, m in zip(objs, mags):
        key = o
        if qcgd and len(o) >= 2:
            key = bytes(np.frombuffer(o, np.uint8)[W.graph_padding_mask(o)])
        if key in out:
            raise AssertionError("duplicate object in a state")
        out[key] = complex(m)
    return out


def mag_close(a: complex, b: complex) -> bool:
    return abs(a - b) <= REL * max(abs(a), abs(b), FLOOR)


def assert_state_parity(got, exp, qcgd: bool, truncated: bool = False, what: str = ""):
    g = canon(got, qcgd)
    e = canon(exp, qcgd)
    assert len(g) == len(e), f"{what}: {len(g)} objects, expected {len(e)}"
    if not truncated:
        missing = set(e) - set(g)
        assert not missing, f"{what}: {len(missing)} expected objects missing"
        keys = e.keys()
    else:
        if not e:
            return
        tau = min(abs(m) ** 2 for m in e.values())
        band = lambda m: abs(abs(m) ** 2 - tau) <= REL * tau * 4  # noqa: E731
        eo = {k for k, m in e.items() if not band(m)}
        go = {k for k, m in g.items() if not band(m)}
        assert eo == go, f"{what}: {len(eo ^ go)} objects differ outside the tie band"
        keys = eo
    bad = [k for k in keys if not mag_close(g[k], e[k])]
    assert not bad, f"{what}: {len(bad)} magnitudes differ, e.g. {g[bad[0]]} vs {e[bad[0]]}"
