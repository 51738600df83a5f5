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


def _rows(p):
    """fixed-size objects as a (n, size) uint8 matrix, plus magnitudes"""
    objects, begin, size, mag = p
    n = len(size)
    if n == 0:
        return np.zeros((0, 0), np.uint8), np.zeros(0, np.complex128)
    sz = int(size[0])
    assert (np.asarray(size) == sz).all(), "fixed-size comparison on variable-size objects"
    idx = np.asarray(begin[:n], dtype=np.int64)[:, None] + np.arange(sz, dtype=np.int64)[None, :]
    return np.asarray(objects)[idx], np.asarray(mag, dtype=np.complex128)


def assert_fixed_state_parity(got, exp, truncated=False, what=""):
    """Vectorised assert_state_parity for states of equal-size objects (large states)."""
    g_rows, g_mag = _rows(got)
    e_rows, e_mag = _rows(exp)
    assert g_rows.shape == e_rows.shape, f"{what}: shapes {g_rows.shape} vs {e_rows.shape}"
    if len(g_mag) == 0:
        return
    gk = np.ascontiguousarray(g_rows).view(np.dtype((np.void, g_rows.shape[1]))).ravel()
    ek = np.ascontiguousarray(e_rows).view(np.dtype((np.void, e_rows.shape[1]))).ravel()
    go, eo = np.argsort(gk), np.argsort(ek)
    gk, ek, g_mag, e_mag = gk[go], ek[eo], g_mag[go], e_mag[eo]
    if not truncated:
        assert (gk == ek).all(), f"{what}: object sets differ"
        keep_g = keep_e = np.ones(len(gk), bool)
    else:
        en = np.abs(e_mag) ** 2
        tau = en.min()
        band_e = np.abs(en - tau) <= REL * tau * 4
        band_g = np.abs(np.abs(g_mag) ** 2 - tau) <= REL * tau * 4
        assert (gk[~band_g] == ek[~band_e]).all() if (~band_g).sum() == (~band_e).sum() else False, \
            f"{what}: objects outside the tie band differ"
        keep_g, keep_e = ~band_g, ~band_e
    a, b = g_mag[keep_g], e_mag[keep_e]
    tol = REL * np.maximum(np.maximum(np.abs(a), np.abs(b)), FLOOR)
    bad = np.abs(a - b) > tol
    assert not bad.any(), f"{what}: {int(bad.sum())} magnitudes differ"


def assert_hashed_state_parity(ctx, got_it, exp_packed, hash_rule, qcgd=True, truncated=False, what="",
                               sample=2000):
    """Large-state parity through hashes: both states are hashed on the GPU
    with the rule's hasher (pinned to the reference's by the golden vectors)
    and compared as (hash -> magnitude) maps with the tie band; then, paired
    by hash, every object's bytes are compared on the host (QCGD padding
    masked), and a random sample once more object by object."""
    import quids_gb300 as quids
    exp_it = quids.it_t(ctx, exp_packed)
    gh = quids.state_hash(got_it, hash_rule)
    eh = quids.state_hash(exp_it, hash_rule)
    got = got_it.download()
    gm, em = np.asarray(got[3]), np.asarray(exp_packed[3])
    assert len(gh) == len(eh), f"{what}: {len(gh)} objects, expected {len(eh)}"
    go, eo = np.argsort(gh, kind="stable"), np.argsort(eh, kind="stable")
    gh, eh, gm, em = gh[go], eh[eo], gm[go], em[eo]
    assert (np.diff(gh.astype(np.uint64)) != 0).all(), f"{what}: duplicate hashes in the result"
    if truncated and len(em):
        en = np.abs(em) ** 2
        tau = en.min()
        kg = np.abs(np.abs(gm) ** 2 - tau) > REL * tau * 4
        ke = np.abs(en - tau) > REL * tau * 4
        assert kg.sum() == ke.sum() and (gh[kg] == eh[ke]).all(), f"{what}: sets differ outside the tie band"
        gm, em = gm[kg], em[ke]
        gsel, esel = go[kg], eo[ke]
    else:
        assert (gh == eh).all(), f"{what}: object sets differ"
        gsel, esel = go, eo
    tol = REL * np.maximum(np.maximum(np.abs(gm), np.abs(em)), FLOOR)
    bad = np.abs(gm - em) > tol
    assert not bad.any(), f"{what}: {int(bad.sum())} magnitudes differ"
    # every object's bytes (padding masked), in hash order on both sides
    assert_all_bytes_equal(got, exp_packed, gsel, esel, qcgd, what)
    # and a random sample object by object, through the scalar mask
    rng = np.random.default_rng(0)
    pick = rng.choice(len(gsel), size=min(sample, len(gsel)), replace=False) if len(gsel) else []
    gobj, gbeg, gsz = got[0], got[1], got[2]
    eobj, ebeg, esz = exp_packed[0], exp_packed[1], exp_packed[2]
    for k in pick:
        a, b = int(gsel[k]), int(esel[k])
        x = gobj[int(gbeg[a]): int(gbeg[a]) + int(gsz[a])].tobytes()
        y = eobj[int(ebeg[b]): int(ebeg[b]) + int(esz[b])].tobytes()
        assert len(x) == len(y), f"{what}: object sizes differ"
        if qcgd:
            mk = W.graph_padding_mask(y)
            assert (np.frombuffer(x, np.uint8)[mk] == np.frombuffer(y, np.uint8)[mk]).all(), f"{what}: bytes differ"
        else:
            assert x == y, f"{what}: bytes differ"


def assert_all_bytes_equal(got, exp, gsel, esel, qcgd: bool, what: str = "", chunk_bytes: int = 1 << 27):
    """Object gsel[k] of `got` has the bytes of object esel[k] of `exp`, for
    every k: sizes equal, and every byte equal except, for QCGD graphs, the 4
    padding bytes of each 16-byte name sub-node (never initialised by the
    reference, src/rules/qcgd.hpp:35-61; the layout is that of
    graph_padding_mask).  Vectorised on the host in chunks of about
    chunk_bytes bytes, so states of 2^24 objects compare in full."""
    gobj, eobj = np.asarray(got[0]), np.asarray(exp[0])
    gbeg, ebeg = np.asarray(got[1], np.int64), np.asarray(exp[1], np.int64)
    gsel, esel = np.asarray(gsel, np.int64), np.asarray(esel, np.int64)
    gsz = np.asarray(got[2], np.int64)[gsel]
    esz = np.asarray(exp[2], np.int64)[esel]
    assert len(gsel) == len(esel), f"{what}: {len(gsel)} objects paired with {len(esel)}"
    bad = np.nonzero(gsz != esz)[0]
    assert not len(bad), f"{what}: {len(bad)} object sizes differ"
    ends = np.cumsum(gsz)
    lo = 0
    while lo < len(gsel):
        start_bytes = int(ends[lo - 1]) if lo else 0
        hi = int(np.searchsorted(ends, start_bytes + chunk_bytes, side="right"))
        hi = max(hi, lo + 1)
        sz = gsz[lo:hi]
        tot = int(sz.sum())
        rel = np.arange(tot, dtype=np.int64) - np.repeat(np.cumsum(sz) - sz, sz)
        gb = gobj[np.repeat(gbeg[gsel[lo:hi]], sz) + rel]
        eb = eobj[np.repeat(ebeg[esel[lo:hi]], sz) + rel]
        diff = gb != eb
        if qcgd:
            e0 = ebeg[esel[lo:hi]]
            n = eobj[e0].astype(np.int64) | (eobj[e0 + 1].astype(np.int64) << 8)
            q = rel - np.repeat(4 + 4 * n, sz)
            r = q & 15
            pad = (q >= 0) & (r >= 4) & (r < 8) & (q - r + 8 <= np.repeat(sz, sz) - np.repeat(4 + 4 * n, sz))
            diff &= ~pad
        if diff.any():
            first = int(np.searchsorted(np.cumsum(sz), int(np.argmax(diff)), side="right")) + lo
            raise AssertionError(f"{what}: bytes differ (first at paired object {first}, "
                                 f"{int(diff.sum())} bytes in this chunk)")
        lo = hi
