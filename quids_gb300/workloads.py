"""Seeded workload generators for the QuIDS rule step.

The reference seeds its QCGD inputs with ``rand()``
(``src/rules/qcgd.hpp:114-120``, ``:1093-1095``), so the inputs here come from
a project-owned generator (splitmix64) and both the GPU path and the CPU
oracle receive identical bytes.

Object formats follow the reference:

* quantum_computer: one byte per qubit (``src/rules/quantum_computer.hpp``).
* QCGD graph (``src/rules/qcgd.hpp:63-112``, ``make_graph`` ``:214-230``)::

      [u16 n][u8 left[n]][u8 right[n]][u16 name_begin[n+1]][name sub-nodes ...]

  a name sub-node is 16 bytes: i16 hmlz_and_element, i16 right_or_type,
  4 padding bytes, u64 hash.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

# rule / modifier kinds (same numbering as include/quids_gpu.h)
RULE_HADAMARD = 1
RULE_QCGD_ERASE_CREATE = 2
RULE_QCGD_COIN = 3
RULE_QCGD_SPLIT_MERGE = 4

MOD_CNOT = 1
MOD_X = 2
MOD_Y = 3
MOD_Z = 4
MOD_QCGD_STEP = 5
MOD_QCGD_REVERSED_STEP = 6

U64_MAX = (1 << 64) - 1
M64 = (1 << 64) - 1


class Rng:
    """splitmix64: a tiny, portable, seeded generator."""

    def __init__(self, seed: int):
        self.s = seed & M64

    def u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def below(self, n: int) -> int:
        return self.u64() % n

    def bit(self) -> int:
        return self.u64() >> 63

    def uniform(self, a: float, b: float) -> float:
        return a + (b - a) * ((self.u64() >> 11) * (1.0 / (1 << 53)))


# --------------------------------------------------------------- packing
def align_pad(size: int, align: int) -> int:
    """get_alignment_offset, src/quids.hpp:93-102"""
    if align <= 1:
        return 0
    off = align - size % align
    return 0 if off == align else off


def pack(objs, mags, align: int = 8):
    """list of bytes + magnitudes -> (objects u8, begin u64[n+1], size u32, mag c128)"""
    n = len(objs)
    size = np.array([len(o) for o in objs], dtype=np.uint32)
    begin = np.zeros(n + 1, dtype=np.uint64)
    buf = bytearray()
    for i, o in enumerate(objs):
        begin[i] = len(buf)
        buf += o
        buf += b"\0" * align_pad(len(o), align)
    begin[n] = len(buf)
    objects = np.frombuffer(bytes(buf), dtype=np.uint8).copy() if buf else np.zeros(0, np.uint8)
    return objects, begin, size, np.asarray(mags, dtype=np.complex128)


def unpack(packed):
    objects, begin, size, mag = packed
    return [objects[int(begin[i]): int(begin[i]) + int(size[i])].tobytes() for i in range(len(size))], np.asarray(mag)


# --------------------------------------------------------------- quantum computer
def qc_zero_state(n_qubits: int, align: int = 8):
    return pack([bytes(n_qubits)], [1.0 + 0j], align)


@dataclass
class Gate:
    kind: str                  # "rule" | "mod"
    code: int
    params: tuple = field(default_factory=tuple)


def circuit_small(seed: int = 0, n_qubits: int = 12, n_gates: int = 40):
    """Plain quantum_computer circuit, CPU-runnable size: a Hadamard rule on
    every qubit, then n_gates drawn uniformly from {H rule, X, Y, Z, CNOT} on
    uniformly random qubits (control != target)."""
    rng = Rng(seed)
    gates = [Gate("rule", RULE_HADAMARD, (q,)) for q in range(n_qubits)]
    for _ in range(n_gates):
        k = rng.below(5)
        if k == 0:
            gates.append(Gate("rule", RULE_HADAMARD, (rng.below(n_qubits),)))
        elif k in (1, 2, 3):
            gates.append(Gate("mod", (MOD_X, MOD_Y, MOD_Z)[k - 1], (rng.below(n_qubits),)))
        else:
            c = rng.below(n_qubits)
            t = rng.below(n_qubits - 1)
            t = t + 1 if t >= c else t
            gates.append(Gate("mod", MOD_CNOT, (c, t)))
    return gates


def circuit_layers(seed: int = 1, n_qubits: int = 24, n_layers: int = 6, n_mods: int = 24):
    """Plain quantum_computer circuit at scale: each layer is a Hadamard rule
    on a seeded random half of the qubits followed by n_mods seeded random
    CNOT / Z modifiers.  Returns a list of layers (lists of Gate)."""
    rng = Rng(seed)
    layers = []
    for _ in range(n_layers):
        perm = list(range(n_qubits))
        for i in range(n_qubits - 1, 0, -1):
            j = rng.below(i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        layer = [Gate("rule", RULE_HADAMARD, (q,)) for q in sorted(perm[: n_qubits // 2])]
        for _ in range(n_mods):
            if rng.bit():
                c = rng.below(n_qubits)
                t = rng.below(n_qubits - 1)
                t = t + 1 if t >= c else t
                layer.append(Gate("mod", MOD_CNOT, (c, t)))
            else:
                layer.append(Gate("mod", MOD_Z, (rng.below(n_qubits),)))
        layers.append(layer)
    return layers


# --------------------------------------------------------------- QCGD
def make_graph(n: int, left=None, right=None) -> bytes:
    """make_graph (src/rules/qcgd.hpp:214-230): cycle graph of n nodes named
    0..n-1, one element sub-node per node; padding bytes are zero here."""
    left = left if left is not None else [0] * n
    right = right if right is not None else [0] * n
    out = bytearray(struct.pack("<H", n))
    out += bytes(int(bool(x)) for x in left)
    out += bytes(int(bool(x)) for x in right)
    out += struct.pack(f"<{n + 1}H", *range(n + 1))
    for i in range(n):
        hmlz = -1 if i == 0 else i + 1
        out += struct.pack("<hhIQ", hmlz, -1, 0, i)
    return bytes(out)


def random_graph(n: int, rng: Rng) -> bytes:
    bits = [(rng.bit(), rng.bit()) for _ in range(n)]   # left then right per node
    return make_graph(n, [b[0] for b in bits], [b[1] for b in bits])


def graph_num_nodes(obj: bytes) -> int:
    return struct.unpack_from("<H", obj, 0)[0]


def graph_padding_mask(obj: bytes) -> np.ndarray:
    """bool mask over obj's bytes: False on the 4 padding bytes of every name
    sub-node (never initialised by the reference, src/rules/qcgd.hpp:35-61)."""
    n = graph_num_nodes(obj)
    mask = np.ones(len(obj), dtype=bool)
    base = 4 + 4 * n
    k = 0
    while base + 16 * k + 8 <= len(obj):
        mask[base + 16 * k + 4: base + 16 * k + 8] = False
        k += 1
    return mask


COIN_DEFAULT = (math.pi * 0.25, 0.0, 0.0)   # read_rule defaults, src/rules/qcgd.hpp:1147-1149


def qcgd_step_rules(split_merge=(math.pi / 4, 0.0, -math.pi / 2), erase_create=(math.pi / 3, math.pi / 5, 0.0),
                    coin=COIN_DEFAULT):
    """One QCGD step: step modifier, coin, split_merge, erase_create."""
    return [
        Gate("mod", MOD_QCGD_STEP, ()),
        Gate("rule", RULE_QCGD_COIN, tuple(coin)),
        Gate("rule", RULE_QCGD_SPLIT_MERGE, tuple(split_merge)),
        Gate("rule", RULE_QCGD_ERASE_CREATE, tuple(erase_create)),
    ]


def qcgd_single_state(n_nodes: int = 12, seed: int = 1, align: int = 8):
    rng = Rng(seed)
    return pack([random_graph(n_nodes, rng)], [1.0 + 0j], align)


def qcgd_batch_instances(n_inst: int = 256, seed: int = 2, lo: int = 4, hi: int = 16):
    """Batched QCGD instances: node count U[lo, hi], bits Bernoulli(0.5),
    split_merge / erase_create theta ~ U(0, pi), phi, xi ~ U(0, 2 pi)."""
    rng = Rng(seed)
    out = []
    for _ in range(n_inst):
        n = lo + rng.below(hi - lo + 1)
        g = random_graph(n, rng)
        sm = (rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi), rng.uniform(0, 2 * math.pi))
        ec = (rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi), rng.uniform(0, 2 * math.pi))
        out.append((g, sm, ec))
    return out


def qcgd_adjoint_workload(n_nodes: int = 10, seed: int = 3):
    """Adjoint workload: a cycle graph of n_nodes with Bernoulli(0.5) bits and
    six angles U(0, pi) -- split_merge (theta1, phi1, xi1) and erase_create
    (theta2, phi2, xi2) -- drawn from one generator of `seed`, bits first."""
    rng = Rng(seed)
    g = random_graph(n_nodes, rng)
    angles = [rng.uniform(0, math.pi) for _ in range(6)]
    return pack([g], [1.0 + 0j], 8), angles


def qcgd_adjoint_ops(angles, n_steps: int):
    """(ops, slots): n_steps of step, coin, split_merge(angles[0:3]),
    erase_create(angles[3:6]) as Gate tuples; slots maps (op index,
    component 0..2) -> angle index for the rule ops carrying the angles."""
    ops, slots = [], []
    for _ in range(n_steps):
        base = len(ops)
        ops += [Gate("mod", MOD_QCGD_STEP, ()), Gate("rule", RULE_QCGD_COIN, tuple(COIN_DEFAULT)),
                Gate("rule", RULE_QCGD_SPLIT_MERGE, tuple(angles[0:3])),
                Gate("rule", RULE_QCGD_ERASE_CREATE, tuple(angles[3:6]))]
        slots += [(base + 2, k, k) for k in range(3)] + [(base + 3, k, 3 + k) for k in range(3)]
    return ops, slots
