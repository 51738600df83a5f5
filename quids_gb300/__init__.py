"""quids_gb300 -- the QuIDS rule step on one GB300 GPU.

A host-side mirror of the reference's public interface (src/quids.hpp):

    import quids_gb300 as quids
    from quids_gb300 import rules
    quids.tolerance = 1e-18                      # quids::tolerance (src/quids.hpp:62)
    ctx = quids.Context()                        # one GPU, one CUDA stream
    it, nxt, sy = quids.it_t(ctx), quids.it_t(ctx), quids.sy_it_t()
    it.append(bytes(12), 1 + 0j)                 # iteration::append (:174-188)
    quids.simulate(it, rules.hadamard(3), nxt, sy, max_num_object)   # (:448-543)
    quids.simulate(nxt, rules.Zgate(3))          # modifier (:436-438)
    nxt.num_object, nxt.total_proba, sy.num_object, sy.num_object_after_interferences

Every call goes through the C ABI of include/quids_gpu.h into the in-tree
CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import QuidsError, U64_MAX

# reference globals (src/quids.hpp:59-75); read at every simulate() call
tolerance: float = 1e-30          # TOLERANCE default (src/quids.hpp:30-32)
align_byte_length: int = 8        # ALIGNMENT_BYTE_LENGTH (src/quids.hpp:27-29)
simple_truncation: bool = True    # False: probabilistic truncation (src/quids.hpp:69-75)
truncation_seed: int = 0          # generator seed of probabilistic truncation
memory_budget: int = 0            # automatic truncation (max_num_object = 0): bytes per step, 0 = device
table_load_factor: float = 0.5    # collision table maximum load
hash_ranges: int = 0              # 0: one pass while the children fit; k >= 2: k hash-range passes
max_probes: int = 0               # collision-table probe limit (0: the library's default)
max_alloc_bytes: int = 0          # largest device allocation a call may make (0: no limit)
debug_flags: int = 0              # capi.DEBUG_*: failure injection for tests of the error paths


class rules:
    """Rule and modifier constructors (src/rules/quantum_computer.hpp, src/rules/qcgd.hpp)."""

    @dataclass(frozen=True)
    class _R:
        kind: int
        is_rule: bool
        bit: int = 0
        control: int = 0
        theta: float = 0.0
        phi: float = 0.0
        xi: float = 0.0

        def params(self) -> capi.RuleParams:
            return capi.RuleParams(self.bit, self.control, self.theta, self.phi, self.xi)

    @staticmethod
    def hadamard(bit):
        return rules._R(1, True, bit=int(bit))

    @staticmethod
    def erase_create(theta, phi=0.0, xi=0.0):
        return rules._R(2, True, theta=float(theta), phi=float(phi), xi=float(xi))

    @staticmethod
    def coin(theta, phi=0.0, xi=0.0):
        return rules._R(3, True, theta=float(theta), phi=float(phi), xi=float(xi))

    @staticmethod
    def split_merge(theta, phi=0.0, xi=0.0):
        return rules._R(4, True, theta=float(theta), phi=float(phi), xi=float(xi))

    @staticmethod
    def cnot(control_bit, bit):
        return rules._R(1, False, bit=int(bit), control=int(control_bit))

    @staticmethod
    def Xgate(bit):
        return rules._R(2, False, bit=int(bit))

    @staticmethod
    def Ygate(bit):
        return rules._R(3, False, bit=int(bit))

    @staticmethod
    def Zgate(bit):
        return rules._R(4, False, bit=int(bit))

    step = None            # set below (QCGD modifiers take no parameters)
    reversed_step = None


rules.step = rules._R(5, False)
rules.reversed_step = rules._R(6, False)


def rule_from(kind_is_rule: bool, code: int, params=()):
    """Build a rule/modifier from the numeric codes used by quids_gb300.workloads."""
    p = list(params)
    if kind_is_rule:
        if code == 1:
            return rules.hadamard(p[0])
        return rules._R(code, True, theta=float(p[0]), phi=float(p[1]) if len(p) > 1 else 0.0,
                        xi=float(p[2]) if len(p) > 2 else 0.0)
    if code == 1:
        return rules.cnot(p[0], p[1])
    if code in (2, 3, 4):
        return rules._R(code, False, bit=int(p[0]))
    return rules._R(code, False)


class Context:
    """A device context: one GPU, one CUDA stream, the step's scratch memory."""

    def __init__(self, device: int = 0):
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.quids_gpu_ctx_create(int(device), C.byref(h)), "quids_gpu_ctx_create")
        self.h = h
        self.device = device

    def close(self):
        """Destroys the context; its states are released with it (their
        handles stay safe to drop afterwards)."""
        if getattr(self, "h", None):
            self.lib.quids_gpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.quids_gpu_ctx_stream(self.h) or 0)

    def synchronize(self):
        capi.check(self.lib.quids_gpu_ctx_synchronize(self.h), "synchronize")

    @property
    def scratch_bytes(self) -> int:
        return int(self.lib.quids_gpu_ctx_scratch_bytes(self.h))

    def trim(self):
        capi.check(self.lib.quids_gpu_ctx_trim(self.h), "trim")

    def run_counts(self) -> dict:
        """How this context's run() calls ran: "sync" (two host waits per
        rule step), "planned" (one host wait per run) and "graph" (planned
        runs replayed from a captured CUDA graph)."""
        v = [C.c_uint64() for _ in range(3)]
        capi.check(self.lib.quids_gpu_ctx_run_counts(self.h, *[C.byref(x) for x in v]), "run_counts")
        return {"sync": int(v[0].value), "planned": int(v[1].value), "graph": int(v[2].value)}

    def last_tuning(self) -> dict:
        """The most recent autotuning of a planned run in this context
        (run(..., flags=capi.FLAG_AUTOTUNE)): the chosen collision-table load
        factor, table-pass block size and blocks per SM, the run time under
        the default and the chosen configuration, and the configurations
        timed."""
        t = capi.Tuning()
        capi.check(self.lib.quids_gpu_ctx_last_tuning(self.h, C.byref(t)), "last_tuning")
        return {k: getattr(t, k) for k, _ in t._fields_ if k != "pad"}


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class sy_it_t:
    """symbolic_iteration (src/quids.hpp:338-429): the step's public counters."""

    def __init__(self):
        self.num_object = 0
        self.num_object_after_interferences = 0
        self.stats = {}


class it_t:
    """iteration (src/quids.hpp:149-335) held in device memory."""

    def __init__(self, ctx: Context | None = None, packed=None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        h = C.c_void_p()
        capi.check(self.lib.quids_gpu_state_create(self.ctx.h, C.byref(h)), "state_create")
        self.h = h
        self._pending = []
        if packed is not None:
            self.upload(packed)

    def __del__(self):
        try:
            if self.h:
                self.lib.quids_gpu_state_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- host <-> device
    def upload(self, packed):
        """packed = (objects u8, begin u64[n+1], size u32[n], mag complex128[n])"""
        objects, begin, size, mag = packed
        objects = np.ascontiguousarray(objects, dtype=np.uint8)
        begin = np.ascontiguousarray(begin, dtype=np.uint64)
        size = np.ascontiguousarray(size, dtype=np.uint32)
        mag = np.ascontiguousarray(mag, dtype=np.complex128)
        n = int(size.shape[0])
        nbytes = int(objects.shape[0])
        capi.check(self.lib.quids_gpu_state_upload(
            self.h, n, objects.ctypes.data if nbytes else None, begin.ctypes.data, size.ctypes.data,
            mag.ctypes.data, nbytes), "state_upload")
        self._pending = []

    def download(self):
        self._flush()
        n, nb = self.num_object, self.num_bytes
        objects = np.zeros(max(nb, 1), dtype=np.uint8)
        begin = np.zeros(n + 1, dtype=np.uint64)
        size = np.zeros(max(n, 1), dtype=np.uint32)
        mag = np.zeros(max(n, 1), dtype=np.complex128)
        capi.check(self.lib.quids_gpu_state_download(self.h, objects.ctypes.data, begin.ctypes.data,
                                                     size.ctypes.data, mag.ctypes.data), "state_download")
        return objects[:nb], begin, size[:n], mag[:n]

    def download_async(self, objects, begin, size, mag):
        """Starts the device -> host copies of the state into the given arrays
        (objects >= num_bytes bytes, begin >= num_object + 1 u64, size >=
        num_object u32, mag >= num_object complex128; pinned memory lets the
        copies overlap later steps) and returns; download_wait() completes
        them.  Later writes to the state wait for the copies on the device."""
        self._flush()
        n, nb = self.num_object, self.num_bytes
        arrays = ((objects, nb, 1), (begin, n + 1, 8), (size, n, 4), (mag, n, 16))
        for a, count, item in arrays:
            if _nbytes(a) < count * item:
                raise ValueError("download_async: a host buffer is too small for the state")
        capi.check(self.lib.quids_gpu_state_download_async(self.h, *(_address(a) for a, _, _ in arrays)),
                   "state_download_async")

    def download_wait(self):
        capi.check(self.lib.quids_gpu_state_download_wait(self.h), "state_download_wait")

    def _flush(self):
        if not self._pending:
            return
        pend, self._pending = self._pending, []
        from .workloads import pack, unpack
        objs, mags = unpack(self.download()) if self._n_device() else ([], np.zeros(0, np.complex128))
        objs = list(objs) + [o for o, _ in pend]
        mags = list(mags) + [m for _, m in pend]
        self.upload(pack(objs, mags, align_byte_length))

    def _n_device(self) -> int:
        v = C.c_uint64()
        capi.check(self.lib.quids_gpu_state_num_object(self.h, C.byref(v)))
        return int(v.value)

    # ---- reference interface
    def append(self, obj: bytes, mag: complex = 1.0):
        """iteration::append (src/quids.hpp:174-188)"""
        self._pending.append((bytes(obj), complex(mag)))

    @property
    def num_object(self) -> int:
        return self._n_device() + len(self._pending)

    @property
    def num_bytes(self) -> int:
        v = C.c_uint64()
        capi.check(self.lib.quids_gpu_state_num_bytes(self.h, C.byref(v)))
        return int(v.value)

    @property
    def total_proba(self) -> float:
        v = C.c_double()
        capi.check(self.lib.quids_gpu_state_total_proba(self.h, C.byref(v)))
        return float(v.value)

    def get_object(self, oid: int):
        """iteration::get_object (src/quids.hpp:254-258): (bytes, magnitude)"""
        objects, begin, size, mag = self.download()
        b = int(begin[oid])
        return objects[b: b + int(size[oid])].tobytes(), complex(mag[oid])

    # ---- batched states (no counterpart in the reference)
    def upload_batched(self, states):
        """Uploads independent states (a list of packed tuples) as the
        instances of one batched state; each instance's bytes are padded to a
        multiple of 8 so every object keeps its alignment."""
        objs, begins, sizes, mags, inst_begin = [], [], [], [], [0]
        off = 0
        for objects, begin, size, mag in states:
            objects = np.asarray(objects, dtype=np.uint8)
            n = len(size)
            nb = int(objects.shape[0])
            pad = (-nb) % 8
            objs.append(objects)
            if pad:
                objs.append(np.zeros(pad, np.uint8))
            begins.append(np.asarray(begin[:n], dtype=np.uint64) + np.uint64(off))
            sizes.append(np.asarray(size, dtype=np.uint32))
            mags.append(np.asarray(mag, dtype=np.complex128))
            off += nb + pad
            inst_begin.append(inst_begin[-1] + n)
        n = inst_begin[-1]
        objects = np.ascontiguousarray(np.concatenate(objs) if objs else np.zeros(0, np.uint8))
        begin = np.ascontiguousarray(np.concatenate(begins + [np.array([off], np.uint64)]))
        size = np.ascontiguousarray(np.concatenate(sizes) if sizes else np.zeros(0, np.uint32))
        mag = np.ascontiguousarray(np.concatenate(mags) if mags else np.zeros(0, np.complex128))
        ib = np.ascontiguousarray(np.asarray(inst_begin, dtype=np.uint64))
        capi.check(self.lib.quids_gpu_state_upload_batched(
            self.h, n, objects.ctypes.data if off else None, begin.ctypes.data, size.ctypes.data,
            mag.ctypes.data, off, len(states), ib.ctypes.data), "state_upload_batched")
        self._pending = []

    @property
    def num_instances(self) -> int:
        g = C.c_uint32()
        capi.check(self.lib.quids_gpu_state_instances(self.h, C.byref(g), None, None), "state_instances")
        return int(g.value)

    def instances(self):
        """(inst_begin u64[n_inst + 1], inst_total f64[n_inst]): instance
        offsets, and each instance's total probability before the last
        step normalised it."""
        g = self.num_instances
        ib = np.zeros(g + 1, np.uint64)
        tot = np.zeros(max(g, 1), np.float64)
        n = C.c_uint32()
        capi.check(self.lib.quids_gpu_state_instances(self.h, C.byref(n), ib.ctypes.data, tot.ctypes.data),
                   "state_instances")
        return ib, tot[:g]

    def download_instances(self):
        """The instances as a list of packed tuples (begin rebased per instance)."""
        objects, begin, size, mag = self.download()
        ib, _ = self.instances()
        out = []
        for g in range(len(ib) - 1):
            a, b = int(ib[g]), int(ib[g + 1])
            if a == b:
                out.append((np.zeros(0, np.uint8), np.zeros(1, np.uint64), np.zeros(0, np.uint32),
                            np.zeros(0, np.complex128)))
                continue
            lo = int(begin[a])
            hi = int(begin[b]) if b < len(size) else int(begin[len(size)])
            out.append((objects[lo:hi].copy(), (begin[a:b + 1] - np.uint64(lo)).astype(np.uint64),
                        size[a:b].copy(), mag[a:b].copy()))
        return out

    def average_value(self, observable) -> float:
        """iteration::average_value (src/quids.hpp:208-234), evaluated on the host."""
        objects, begin, size, mag = self.download()
        tot = 0.0
        for i in range(len(size)):
            b = int(begin[i])
            tot += observable(objects[b: b + int(size[i])].tobytes()) * abs(mag[i]) ** 2
        return tot


def _nbytes(a) -> int:
    """Bytes of a host buffer: a numpy array or a (pinned) torch tensor."""
    return int(a.nbytes) if isinstance(a, np.ndarray) else int(a.numel() * a.element_size())


def _address(a) -> int:
    return int(a.ctypes.data) if isinstance(a, np.ndarray) else int(a.data_ptr())


def _params(max_num_object, flags=0):
    return capi.Params(float(tolerance), int(max_num_object) & U64_MAX, int(bool(simple_truncation)),
                       int(align_byte_length), float(table_load_factor), int(hash_ranges), int(flags),
                       int(truncation_seed) & U64_MAX, int(memory_budget), int(max_probes), int(debug_flags),
                       int(max_alloc_bytes))


def simulate(iteration: it_t, rule, next_iteration: it_t | None = None, symbolic_iteration: sy_it_t | None = None,
             max_num_object: int = U64_MAX, flags: int = 0):
    """quids::simulate.  With a rule: (iteration, rule, next_iteration, sy_it, max_num_object)
    (src/quids.hpp:448-543); with a modifier: (iteration, modifier) (:436-438).
    max_num_object = U64_MAX means no truncation (the reference's -1)."""
    iteration._flush()
    lib = iteration.lib
    p = rule.params()
    if not rule.is_rule:
        capi.check(lib.quids_gpu_apply_modifier(iteration.ctx.h, iteration.h, rule.kind, C.byref(p)),
                   "apply_modifier")
        return None
    if next_iteration is None or next_iteration is iteration:
        raise QuidsError(-1, "simulate: next_iteration must be a distinct it_t")
    next_iteration._pending = []
    stats = capi.StepStats()
    prm = _params(max_num_object, flags)
    capi.check(lib.quids_gpu_simulate(iteration.ctx.h, iteration.h, rule.kind, C.byref(p), next_iteration.h,
                                      C.byref(prm), C.byref(stats)), "simulate")
    d = stats.as_dict()
    if symbolic_iteration is not None:
        symbolic_iteration.num_object = d["num_object"]
        symbolic_iteration.num_object_after_interferences = d["num_object_after_interferences"]
        symbolic_iteration.stats = d
    return d


def run(a: it_t, b: it_t, ops, max_num_object: int = U64_MAX, flags: int = 0):
    """Applies a list of rules and modifiers in one library call (the loop of
    simulate() calls of the reference's examples, ping-ponging between two
    iterations).  ops: rules/modifiers from ``rules``.  Returns
    (final it_t, list of per-rule stats).

    Repeating a run (same ops, knobs and handles, new input uploaded into
    ``a``) makes it a planned run: the library sizes every step from the
    earlier run, launches the whole list without host waits and, from the
    third run on, replays it as a captured CUDA graph.  The results are the
    synchronous steps' bit for bit; a step beyond its plan falls back to the
    synchronous steps from there.  flags |= capi.FLAG_NO_PLAN turns this off."""
    a._flush()
    arr = (capi.Op * max(len(ops), 1))()
    n_rules = 0
    for i, r in enumerate(ops):
        arr[i].is_rule = int(r.is_rule)
        arr[i].kind = r.kind
        arr[i].params = r.params()
        n_rules += int(r.is_rule)
    stats = (capi.StepStats * max(n_rules, 1))()
    fin = C.c_int(0)
    prm = _params(max_num_object, flags)
    b._pending = []
    rc = a.lib.quids_gpu_run(a.ctx.h, a.h, b.h, arr, len(ops), C.byref(prm), stats, C.byref(fin))
    capi.check(rc, "run")
    return (a if fin.value == 0 else b), [stats[i].as_dict() for i in range(n_rules)]


def simulate_batched(iteration: it_t, rules_per_instance, next_iteration: it_t, max_num_object: int = U64_MAX,
                     flags: int = 0):
    """One rule step of every instance of a batched state: instance g steps
    with rules_per_instance[g] (all of one kind).  Returns (step stats,
    per-instance u64[n_inst, 3] {num_object, num_object_after_interferences,
    survivors})."""
    iteration._flush()
    g = iteration.num_instances
    if len(rules_per_instance) != g:
        raise QuidsError(-1, f"simulate_batched: {len(rules_per_instance)} rules for {g} instances")
    kinds = {r.kind for r in rules_per_instance}
    if len(kinds) != 1 or not rules_per_instance[0].is_rule:
        raise QuidsError(-1, "simulate_batched: one rule kind for every instance")
    arr = (capi.RuleParams * g)(*[r.params() for r in rules_per_instance])
    inst = np.zeros((g, 3), np.uint64)
    stats = capi.StepStats()
    prm = _params(max_num_object, flags)
    next_iteration._pending = []
    capi.check(iteration.lib.quids_gpu_simulate_batched(iteration.ctx.h, iteration.h, kinds.pop(), arr,
                                                        next_iteration.h, C.byref(prm), inst.ctypes.data,
                                                        C.byref(stats)), "simulate_batched")
    return stats.as_dict(), inst


def run_batched(a: it_t, b: it_t, ops, max_num_object: int = U64_MAX, flags: int = 0):
    """run() over a batched state.  A rule op is one rule (every instance) or
    a list of rules of one kind, one per instance; modifiers act on every
    object.  Returns (final it_t, per-rule stats)."""
    a._flush()
    g = a.num_instances
    arr = (capi.Op * max(len(ops), 1))()
    per = []
    n_rules = 0
    for i, r in enumerate(ops):
        if isinstance(r, (list, tuple)):
            if len(r) != g or len({x.kind for x in r}) != 1:
                raise QuidsError(-1, "run_batched: a per-instance op needs one rule of one kind per instance")
            head = r[0]
            per.extend(x.params() for x in r)
        else:
            head = r
            if r.is_rule:
                per.extend(r.params() for _ in range(g))
        arr[i].is_rule = int(head.is_rule)
        arr[i].kind = head.kind
        arr[i].params = head.params()
        n_rules += int(head.is_rule)
    inst = (capi.RuleParams * max(len(per), 1))(*per)
    stats = (capi.StepStats * max(n_rules, 1))()
    fin = C.c_int(0)
    prm = _params(max_num_object, flags)
    b._pending = []
    capi.check(a.lib.quids_gpu_run_batched(a.ctx.h, a.h, b.h, arr, len(ops), inst, C.byref(prm), stats,
                                           C.byref(fin)), "run_batched")
    return (a if fin.value == 0 else b), [stats[i].as_dict() for i in range(n_rules)]


class Tape:
    """A forward run of rules and modifiers recorded for simulate_backward
    (no counterpart in the reference): reverse mode with respect to the rule
    angles, each step's structure (children, collisions, truncation) held
    fixed.  Checkpoints every `checkpoint_every` rule applications."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        h = C.c_void_p()
        capi.check(self.lib.quids_gpu_tape_create(self.ctx.h, C.byref(h)), "tape_create")
        self.h = h
        self.n_ops = 0

    def __del__(self):
        try:
            if self.h:
                self.lib.quids_gpu_tape_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def forward(self, initial: it_t, ops, max_num_object: int = U64_MAX, checkpoint_every: int = 1, flags: int = 0):
        """Runs ops from `initial`; returns (final it_t, per-rule stats)."""
        initial._flush()
        arr = (capi.Op * max(len(ops), 1))()
        n_rules = 0
        for i, r in enumerate(ops):
            arr[i].is_rule = int(r.is_rule)
            arr[i].kind = r.kind
            arr[i].params = r.params()
            n_rules += int(r.is_rule)
        stats = (capi.StepStats * max(n_rules, 1))()
        out = it_t(self.ctx)
        prm = _params(max_num_object, flags)
        capi.check(self.lib.quids_gpu_forward(self.ctx.h, self.h, initial.h, arr, len(ops), C.byref(prm),
                                              int(checkpoint_every), out.h, stats), "forward")
        self.n_ops = len(ops)
        return out, [stats[i].as_dict() for i in range(n_rules)]

    def backward(self, loss_adjoint):
        """loss_adjoint: complex array a = 2 dL/d(conj m) over the final
        state's objects.  Returns dL/d(theta, phi, xi) per op, shape (n_ops, 3)."""
        a = np.ascontiguousarray(loss_adjoint, dtype=np.complex128)
        g = np.zeros((max(self.n_ops, 1), 3), np.float64)
        capi.check(self.lib.quids_gpu_simulate_backward(self.ctx.h, self.h, a.ctypes.data if len(a) else None,
                                                        g.ctypes.data), "simulate_backward")
        return g[: self.n_ops]

    def backward_observable(self, observable: int, bit: int = 0):
        """L = the final state's average_value of a built-in observable;
        returns (L, dL/d(theta, phi, xi) per op)."""
        g = np.zeros((max(self.n_ops, 1), 3), np.float64)
        loss = C.c_double()
        p = capi.RuleParams(int(bit), 0, 0.0, 0.0, 0.0)
        capi.check(self.lib.quids_gpu_simulate_backward_observable(self.ctx.h, self.h, int(observable), C.byref(p),
                                                                   C.byref(loss), g.ctypes.data),
                   "simulate_backward_observable")
        return float(loss.value), g[: self.n_ops]


def observable_adjoint(iteration: it_t, observable: int, bit: int = 0):
    """(L, a): L = average_value of a built-in observable and its adjoint
    a = 2 dL/d(conj m) over the state's objects."""
    iteration._flush()
    n = iteration.num_object
    a = np.zeros(max(n, 1), np.complex128)
    v = C.c_double()
    p = capi.RuleParams(int(bit), 0, 0.0, 0.0, 0.0)
    capi.check(iteration.lib.quids_gpu_observable_adjoint(iteration.ctx.h, iteration.h, int(observable), C.byref(p),
                                                          C.byref(v), a.ctypes.data), "observable_adjoint")
    return float(v.value), a[:n]


def rule_children(iteration: it_t, rule):
    """Every child of every parent with its bytes, hash, size and magnitude
    (the symbolic iteration with the child bytes kept)."""
    iteration._flush()
    lib = iteration.lib
    p = rule.params()
    nc = C.c_uint64()
    stride = C.c_uint64()
    capi.check(lib.quids_gpu_rule_children(iteration.ctx.h, iteration.h, rule.kind, C.byref(p), C.byref(nc),
                                           C.byref(stride), None, None, None, None), "rule_children")
    n, s = int(nc.value), int(stride.value)
    bytes_ = np.zeros(max(n * s, 1), dtype=np.uint8)
    hashes = np.zeros(max(n, 1), dtype=np.uint64)
    sizes = np.zeros(max(n, 1), dtype=np.uint32)
    mags = np.zeros(max(n, 1), dtype=np.complex128)
    if n:
        capi.check(lib.quids_gpu_rule_children(iteration.ctx.h, iteration.h, rule.kind, C.byref(p), C.byref(nc),
                                               C.byref(stride), bytes_.ctypes.data, hashes.ctypes.data,
                                               sizes.ctypes.data, mags.ctypes.data), "rule_children")
    children = [bytes_[i * s: i * s + int(sizes[i])].tobytes() for i in range(n)]
    return children, hashes[:n], mags[:n]


OBS_QCGD_NUM_NODES, OBS_QCGD_NUM_NODES_SQ, OBS_QCGD_DENSITY, OBS_QCGD_DENSITY_SQ, OBS_QC_BIT = 1, 2, 3, 4, 5


def average_value(iteration: it_t, observable: int, bit: int = 0) -> float:
    """iteration::average_value (src/quids.hpp:208-234) for a built-in
    observable (OBS_*), reduced on the GPU."""
    iteration._flush()
    v = C.c_double()
    p = capi.RuleParams(int(bit), 0, 0.0, 0.0, 0.0)
    capi.check(iteration.lib.quids_gpu_average_value(iteration.ctx.h, iteration.h, int(observable), C.byref(p),
                                                     C.byref(v)), "average_value")
    return v.value


def qcgd_statistics(iteration: it_t, sy: sy_it_t) -> dict:
    """The statistics of qcgd::utils::serialize (src/rules/qcgd.hpp:309-366)."""
    iteration._flush()
    r = capi.QcgdStats()
    capi.check(iteration.lib.quids_gpu_qcgd_statistics(iteration.ctx.h, iteration.h, int(sy.num_object),
                                                       int(sy.num_object_after_interferences), float(tolerance),
                                                       C.byref(r)), "qcgd_statistics")
    return r.as_dict()


def state_hash(iteration: it_t, rule):
    """The rule's hasher over every object of a state, computed on the GPU."""
    iteration._flush()
    n = iteration.num_object
    out = np.zeros(max(n, 1), dtype=np.uint64)
    p = rule.params()
    capi.check(iteration.lib.quids_gpu_state_hash(iteration.ctx.h, iteration.h, rule.kind, C.byref(p),
                                                  out.ctypes.data), "state_hash")
    return out[:n]
