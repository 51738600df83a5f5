"""The QCGD simulation string and its driver (src/rules/qcgd.hpp:1038-1177),
on the GPU rule step.

A simulation string has three '|'-separated parts, as the reference's
flags::parse_simulation reads it:

  "<n_iter>[,seed=S][,reversed_n_iter=R][,tolerance=T][,align=A]
   [,simple_truncate=0|1][,max_num_object=M]
   | <n_node>[,n_graphs=G][,real=x][,imag=y] [; <n_node>...]
   | <rule>[,theta=t][,phi=p][,xi=x][,n_iter=k] [; <rule>...]"

Rules are step, reversed_step, coin, erase_create, split_merge; angles are
in units of pi (theta defaults to 0.25) and, as in the reference, pass
through single precision.  Each rule entry also has its reversed form
(xi -> -xi for the rules, step <-> reversed_step for the modifiers).  The
initial state holds, for every state entry, G cycle graphs of n_node nodes
with magnitude (x, y)/sqrt(G) (single precision), whose left/right bits are
then drawn with the C library's rand() seeded by srand(S): rand() is
restated here (glibc's additive feedback generator, degree 31,
separation 3), so a seed gives the reference's graphs.

The driver runs n_iter iterations of the rule list, each entry k times,
then reversed_n_iter iterations of the reversed list in reverse order, and
reports the statistics of qcgd::utils::serialize (src/rules/qcgd.hpp:309-366)
after every iteration.

  python -m quids_gb300.qcgd_cli "3,seed=1,max_num_object=100000|6|step;coin;split_merge;erase_create,theta=0.3333"
"""
from __future__ import annotations

import json
import math
import sys
from dataclasses import dataclass, field

import numpy as np

from . import workloads as W

F32 = np.float32


# ------------------------------------------------------------- C library rand()
class CRand:
    """glibc's rand()/srand(): the TYPE_3 additive feedback generator
    r[i] = r[i-31] + r[i-3] (mod 2^32) over a table seeded by the
    Park-Miller step 16807 r (mod 2^31 - 1); the first 310 values are
    discarded and each output is r >> 1."""

    def __init__(self, seed: int = 1):
        self.srand(seed)

    def srand(self, seed: int):
        seed &= 0xFFFFFFFF
        if seed == 0:
            seed = 1
        r = [0] * 34
        r[0] = seed
        for i in range(1, 31):
            # 16807 * r[i-1] mod (2^31 - 1) with signed 32-bit arithmetic (Schrage)
            prev = r[i - 1] - (1 << 32) if r[i - 1] >= (1 << 31) else r[i - 1]
            q = abs(prev) // 127773
            hi = q if prev >= 0 else -q  # C division truncates towards zero
            lo = prev - hi * 127773
            word = 16807 * lo - 2836 * hi
            if word < 0:
                word += 2147483647
            r[i] = word & 0xFFFFFFFF
        for i in range(31, 34):
            r[i] = r[i - 31]
        self.r = r
        for _ in range(310):
            self._next()

    def _next(self) -> int:
        r = self.r
        v = (r[-31] + r[-3]) & 0xFFFFFFFF
        r.append(v)
        if len(r) > 64:
            del r[:-34]
        return v

    def rand(self) -> int:
        return self._next() >> 1


# ------------------------------------------------------------------ parsing
def _strip(s: str, sep: str):
    """flags::strip: the text before the first sep, and the rest after it."""
    i = s.find(sep)
    return (s, "") if i < 0 else (s[:i], s[i + len(sep):])


def _number_after(s: str, key: str):
    """flags::parse: the numeric prefix after the first occurrence of key,
    or None (atoi/atof stop at the first character that is not part of the
    number)."""
    i = s.find(key)
    if i < 0:
        return None
    rest = s[i + len(key):]
    j = 0
    while j < len(rest) and (rest[j].isdigit() or rest[j] in "+-.eE"):
        j += 1
    return rest[:j]


def _int(s, key, default):
    v = _number_after(s, key)
    if v is None or v == "":
        return default
    try:
        return int(float(v)) if any(c in v for c in ".eE") else int(v)
    except ValueError:
        return 0


def _float(s, key, default):
    v = _number_after(s, key)
    if v is None or v == "":
        return float(F32(default))
    try:
        return float(F32(float(v)))
    except ValueError:
        return 0.0


@dataclass
class Settings:
    n_iter: int = 1
    reversed_n_iter: int = 0
    seed: int | None = None
    tolerance: float = 1e-30
    align: int = 8
    simple_truncation: bool = True
    max_num_object: int = 0


@dataclass
class RuleEntry:
    name: str
    n_iter: int
    theta: float = 0.0
    phi: float = 0.0
    xi: float = 0.0
    is_rule: bool = True

    def ops(self, reversed_: bool = False):
        """the rule or modifier of this entry (its reversed form)"""
        from . import rules, rule_from
        if not self.is_rule:
            step = (self.name == "step") != reversed_
            return rules.step if step else rules.reversed_step
        code = {"erase_create": W.RULE_QCGD_ERASE_CREATE, "coin": W.RULE_QCGD_COIN,
                "split_merge": W.RULE_QCGD_SPLIT_MERGE}[self.name]
        return rule_from(True, code, (self.theta, self.phi, -self.xi if reversed_ else self.xi))


@dataclass
class Simulation:
    settings: Settings
    state: tuple                       # packed initial state
    rules: list = field(default_factory=list)


def read_n_iter(arg: str) -> Settings:
    """flags::read_n_iter (src/rules/qcgd.hpp:1086-1117)"""
    first, rest = _strip(arg, ",")
    s = Settings()
    s.n_iter = _int(first, "", 0) if first else 0
    seed = _number_after(rest, "seed=")
    s.seed = int(seed) if seed else None
    s.reversed_n_iter = _int(rest, "reversed_n_iter=", 0)
    s.tolerance = _float(rest, "tolerance=", 1e-30) if "tolerance=" in rest else 1e-30
    s.align = _int(rest, "align=", 8)
    s.simple_truncation = bool(_int(rest, "simple_truncate=", 1))
    s.max_num_object = _int(rest, "max_num_object=", 0)
    return s


def read_state(arg: str, rng: CRand, align: int = 8):
    """flags::read_state (src/rules/qcgd.hpp:1119-1137): the graphs of every
    entry, then their bits drawn in order (utils::randomize)."""
    graphs, mags = [], []
    rest = arg
    while True:
        entry, rest = _strip(rest, ";")
        if entry == "":
            break
        n_str, opts = _strip(entry, ",")
        n_node = _int(n_str, "", 0)
        n_graphs = _int(opts, "n_graphs=", 1)
        scale = F32(math.sqrt(float(F32(n_graphs))))
        real = float(F32(F32(_float(opts, "real=", 1.0)) / scale))
        imag = float(F32(F32(_float(opts, "imag=", 0.0)) / scale))
        for _ in range(n_graphs):
            graphs.append(n_node)
            mags.append(complex(real, imag))
    objs = []
    for n in graphs:
        left, right = [], []
        for _ in range(n):
            left.append(rng.rand() & 1)
            right.append(rng.rand() & 1)
        objs.append(W.make_graph(n, left, right))
    return W.pack(objs, mags, align)


def read_rule(arg: str):
    """flags::read_rule (src/rules/qcgd.hpp:1139-1166)"""
    out = []
    rest = arg
    while True:
        entry, rest = _strip(rest, ";")
        if entry == "":
            break
        name, opts = _strip(entry, ",")
        angle = lambda key, d: float(F32(math.pi * _float(opts, key, d)))  # noqa: E731
        theta, phi, xi = angle("theta=", 0.25), angle("phi=", 0.0), angle("xi=", 0.0)
        n_iter = _int(opts, "n_iter=", 1)
        if name in ("split_merge", "erase_create", "coin"):
            out.append(RuleEntry(name, n_iter, theta, phi, xi, True))
        elif name in ("step", "reversed_step"):
            out.append(RuleEntry(name, n_iter, is_rule=False))
    return out


def parse_simulation(arg: str) -> Simulation:
    """flags::parse_simulation (src/rules/qcgd.hpp:1168-1176)"""
    first, rest = _strip(arg, "|")
    settings = read_n_iter(first)
    state_arg, rule_arg = _strip(rest, "|")
    import time
    rng = CRand(settings.seed if settings.seed is not None else int(time.time()))
    state = read_state(state_arg, rng, settings.align)
    return Simulation(settings, state, read_rule(rule_arg))


# ------------------------------------------------------------------- driver
def iteration_ops(sim: Simulation, reversed_: bool = False):
    entries = list(reversed(sim.rules)) if reversed_ else sim.rules
    ops = []
    for e in entries:
        ops += [e.ops(reversed_)] * max(e.n_iter, 0)
    return ops


def run(sim: Simulation, ctx=None, report=print):
    """Runs the simulation on the GPU; report(dict) after every iteration."""
    import quids_gb300 as quids
    s = sim.settings
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = s.tolerance, s.align, s.simple_truncation
    ctx = ctx or quids.default_context()
    cur, other = quids.it_t(ctx, sim.state), quids.it_t(ctx)
    maxn = s.max_num_object if s.max_num_object else 0
    results = []
    for it in range(s.n_iter + s.reversed_n_iter):
        rev = it >= s.n_iter
        fin, stats = quids.run(cur, other, iteration_ops(sim, rev), maxn)
        if fin is other:
            cur, other = other, cur
        sy = quids.sy_it_t()
        if stats:
            sy.num_object = stats[-1]["num_object"]
            sy.num_object_after_interferences = stats[-1]["num_object_after_interferences"]
        r = {"iteration": it, "reversed": rev, **quids.qcgd_statistics(cur, sy)}
        results.append(r)
        report(r)
    return cur, results


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print(__doc__)
        return 2
    sim = parse_simulation(argv[0])
    run(sim, report=lambda r: print(json.dumps(r), flush=True))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
