"""ctypes loader for the CPU oracles of the QuIDS rule step.

TEST INFRASTRUCTURE.  Only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import this module,
and only as the checker or the timed CPU baseline.

Two libraries share one C interface (``oracle/oracle_api.h``):

* ``port``: ``oracle/libquids_port.so``, this project's restatement of the
  reference algorithm (``oracle/quids_port.cpp``); it builds on any host.
* ``ref``:  ``oracle/_ref/libquids_ref.so``, the reference headers compiled in
  place (``make -C oracle ref``); only where the reference tree exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libquids_port.so")
REF_SO = os.path.join(HERE, "_ref", "libquids_ref.so")
REFERENCE_TREE = os.environ.get("QUIDS_REFERENCE_TREE", "/root/reference")

U64_MAX = (1 << 64) - 1

_u8p = C.POINTER(C.c_uint8)
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)


def build(which: str = "port") -> str:
    """Compile one oracle with oracle/Makefile and return the .so path."""
    target = {"port": "port", "ref": "ref"}[which]
    if which == "ref" and not os.path.isdir(os.path.join(REFERENCE_TREE, "src")):
        raise FileNotFoundError("reference tree not present; the ref oracle cannot be built")
    subprocess.run(["make", "-s", "-C", HERE, target, f"REF={REFERENCE_TREE}"], check=True)
    return PORT_SO if which == "port" else REF_SO


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class Oracle:
    """One loaded oracle library (``kind`` = "port" or "ref")."""

    def __init__(self, kind: str = "port", autobuild: bool = True):
        path = PORT_SO if kind == "port" else REF_SO
        if autobuild and not os.path.exists(path):
            build(kind)
        self.kind = kind
        self.lib = L = C.CDLL(path)
        L.qo_state_new.restype = C.c_void_p
        L.qo_state_free.argtypes = [C.c_void_p]
        L.qo_state_load.argtypes = [C.c_void_p, C.c_uint64, _u8p, _u64p, _u32p, _dp]
        L.qo_state_num_object.argtypes = [C.c_void_p]
        L.qo_state_num_object.restype = C.c_uint64
        L.qo_state_num_bytes.argtypes = [C.c_void_p]
        L.qo_state_num_bytes.restype = C.c_uint64
        L.qo_state_store.argtypes = [C.c_void_p, _u8p, _u64p, _u32p, _dp]
        L.qo_state_total_proba.argtypes = [C.c_void_p]
        L.qo_state_total_proba.restype = C.c_double
        L.qo_set_globals.argtypes = [C.c_double, C.c_int, C.c_uint32]
        L.qo_set_threads.argtypes = [C.c_int]
        L.qo_get_threads.restype = C.c_int
        L.qo_simulate.argtypes = [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_uint64, _u64p]
        L.qo_modifier.argtypes = [C.c_void_p, C.c_int, _dp]
        L.qo_hash_bytes.argtypes = [_u8p, C.c_uint64]
        L.qo_hash_bytes.restype = C.c_uint64
        L.qo_qcgd_hash_graph.argtypes = [_u8p]
        L.qo_qcgd_hash_graph.restype = C.c_uint64
        L.qo_num_child.argtypes = [C.c_int, _dp, _u8p, C.c_uint32, _u32p, _u32p]
        L.qo_populate_child.argtypes = [C.c_int, _dp, _u8p, C.c_uint32, C.c_uint32, _u8p, _u32p, _dp]
        L.qo_rule_hash.argtypes = [C.c_int, _dp, _u8p, C.c_uint32]
        L.qo_rule_hash.restype = C.c_uint64

    # ---- globals
    def set_globals(self, tolerance=1e-18, simple_truncation=True, align=8):
        self.lib.qo_set_globals(float(tolerance), int(bool(simple_truncation)), int(align))

    def set_threads(self, n: int):
        self.lib.qo_set_threads(int(n))

    def threads(self) -> int:
        return self.lib.qo_get_threads()

    # ---- states
    def new_state(self, packed=None) -> "OracleState":
        st = OracleState(self)
        if packed is not None:
            st.load(packed)
        return st

    def simulate(self, st_in, rule_kind, params, st_out, max_num_object=U64_MAX):
        p = np.asarray(params, dtype=np.float64)
        counters = np.zeros(2, dtype=np.uint64)
        rc = self.lib.qo_simulate(st_in.h, int(rule_kind), _ptr(p, _dp), st_out.h,
                                  int(max_num_object), _ptr(counters, _u64p))
        if rc != 0:
            raise RuntimeError(f"oracle simulate failed ({rc})")
        return int(counters[0]), int(counters[1])

    def modifier(self, st, kind, params=()):
        p = np.asarray(list(params) + [0.0], dtype=np.float64)
        if self.lib.qo_modifier(st.h, int(kind), _ptr(p, _dp)) != 0:
            raise RuntimeError("oracle modifier failed")

    # ---- rule-level callbacks
    def hash_bytes(self, b: bytes) -> int:
        a = np.frombuffer(b, dtype=np.uint8).copy() if len(b) else np.zeros(1, np.uint8)
        return int(self.lib.qo_hash_bytes(_ptr(a, _u8p), len(b)))

    def qcgd_hash_graph(self, b: bytes) -> int:
        a = np.frombuffer(b, dtype=np.uint8).copy()
        return int(self.lib.qo_qcgd_hash_graph(_ptr(a, _u8p)))

    def rule_hash(self, kind, params, b: bytes) -> int:
        p = np.asarray(params, dtype=np.float64)
        a = np.frombuffer(b, dtype=np.uint8).copy()
        return int(self.lib.qo_rule_hash(int(kind), _ptr(p, _dp), _ptr(a, _u8p), len(b)))

    def num_child(self, kind, params, b: bytes):
        p = np.asarray(params, dtype=np.float64)
        a = np.frombuffer(b, dtype=np.uint8).copy()
        nc = C.c_uint32()
        mcs = C.c_uint32()
        self.lib.qo_num_child(int(kind), _ptr(p, _dp), _ptr(a, _u8p), len(b), C.byref(nc), C.byref(mcs))
        return nc.value, mcs.value

    def populate_child(self, kind, params, b: bytes, child_id: int, mag=(1.0, 0.0), cap=None):
        p = np.asarray(params, dtype=np.float64)
        a = np.frombuffer(b, dtype=np.uint8).copy()
        _, mcs = self.num_child(kind, params, b)
        out = np.zeros(max(cap or 0, mcs, 1) + 64, dtype=np.uint8)
        sz = C.c_uint32()
        m = np.asarray(mag, dtype=np.float64).copy()
        self.lib.qo_populate_child(int(kind), _ptr(p, _dp), _ptr(a, _u8p), len(b), int(child_id),
                                   _ptr(out, _u8p), C.byref(sz), _ptr(m, _dp))
        return out[: sz.value].tobytes(), complex(m[0], m[1])


class OracleState:
    def __init__(self, oracle: Oracle):
        self.o = oracle
        self.h = oracle.lib.qo_state_new()

    def __del__(self):
        try:
            self.o.lib.qo_state_free(self.h)
        except Exception:
            pass

    def load(self, packed):
        """packed = (objects u8[], begin u64[n+1], size u32[n], mag complex128[n])"""
        objects, begin, size, mag = packed
        objects = np.ascontiguousarray(objects, dtype=np.uint8)
        if objects.size == 0:
            objects = np.zeros(1, np.uint8)
        begin = np.ascontiguousarray(begin, dtype=np.uint64)
        size = np.ascontiguousarray(size, dtype=np.uint32)
        m = np.ascontiguousarray(np.asarray(mag, dtype=np.complex128).view(np.float64))
        n = size.shape[0]
        self.o.lib.qo_state_load(self.h, n, _ptr(objects, _u8p), _ptr(begin, _u64p),
                                 _ptr(size, _u32p), _ptr(m, _dp))

    @property
    def num_object(self) -> int:
        return int(self.o.lib.qo_state_num_object(self.h))

    @property
    def total_proba(self) -> float:
        return float(self.o.lib.qo_state_total_proba(self.h))

    def store(self):
        n = self.num_object
        nb = int(self.o.lib.qo_state_num_bytes(self.h))
        objects = np.zeros(max(nb, 1), dtype=np.uint8)
        begin = np.zeros(n + 1, dtype=np.uint64)
        size = np.zeros(max(n, 1), dtype=np.uint32)
        mag = np.zeros(max(n, 1), dtype=np.complex128)
        self.o.lib.qo_state_store(self.h, _ptr(objects, _u8p), _ptr(begin, _u64p),
                                  _ptr(size, _u32p), _ptr(mag.view(np.float64), _dp))
        return objects[:nb], begin, size[:n], mag[:n]
