"""ctypes binding of the C ABI in ``include/quids_gpu.h``.

Loads the in-tree ``quids_gb300/_lib/libquids_gb300.so``; there is no CPU
fallback: if the library is missing, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

U64_MAX = (1 << 64) - 1

QUIDS_OK = 0
STATUS = {
    0: "ok", -1: "bad argument", -2: "device out of memory", -3: "collision table full",
    -4: "child count overflow", -5: "child larger than max_child_size bound",
    -6: "bounded device wait expired", -7: "CUDA runtime error", -8: "no CUDA device",
    -9: "unsupported request", -10: "beyond the static scratch of the no-allocation entry point",
}
ERR_BAD_ARG, ERR_OOM, ERR_TABLE_FULL, ERR_CHILD_COUNT_OVERFLOW, ERR_SIZE_BOUND, ERR_TIMEOUT = -1, -2, -3, -4, -5, -6
ERR_CUDA, ERR_NO_DEVICE, ERR_UNSUPPORTED, ERR_NOALLOC_LIMIT = -7, -8, -9, -10
FLAG_NO_FAST_HASH = 1
FLAG_STAGE_TIMING = 2
FLAG_TABLE = 4
FLAG_PARTITION = 8
FLAG_NO_PLAN = 16
FLAG_AUTOTUNE = 32
DEBUG_STALL_LOOKBACK = 1


class QuidsError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {STATUS.get(code, 'unknown status')} ({code})")


class RuleParams(C.Structure):
    _fields_ = [("bit", C.c_uint64), ("control", C.c_uint64), ("theta", C.c_double),
                ("phi", C.c_double), ("xi", C.c_double)]


class Params(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("max_num_object", C.c_uint64), ("simple_truncation", C.c_int32),
                ("align_byte_length", C.c_uint32), ("table_load_factor", C.c_double),
                ("hash_ranges", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint64),
                ("memory_budget", C.c_uint64), ("max_probes", C.c_uint32), ("debug_flags", C.c_uint32),
                ("max_alloc_bytes", C.c_uint64)]


class Op(C.Structure):
    _fields_ = [("is_rule", C.c_int32), ("kind", C.c_int32), ("params", RuleParams)]


class QcgdStats(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("total_proba", "num_graphs", "avg_size", "std_dev_size", "avg_density",
                                          "std_dev_density", "interference_ratio", "deletion_ratio")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepStats(C.Structure):
    _fields_ = [("num_parents", C.c_uint64), ("num_parents_kept", C.c_uint64), ("num_object", C.c_uint64),
                ("num_object_after_interferences", C.c_uint64), ("num_object_out", C.c_uint64),
                ("max_child_size", C.c_uint64), ("table_capacity", C.c_uint64), ("out_bytes", C.c_uint64),
                ("total_proba", C.c_double), ("algorithmic_bytes", C.c_double), ("ms_total", C.c_float),
                ("stage_ms", C.c_float * 8), ("kernel_launches", C.c_uint64),
                ("hash_ranges", C.c_uint64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stage_ms"}
        d["stage_ms"] = list(self.stage_ms)
        return d


class Tuning(C.Structure):
    _fields_ = [("table_load_factor", C.c_double), ("table_block", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("ms_default", C.c_float), ("ms_tuned", C.c_float), ("trials", C.c_uint32), ("pad", C.c_uint32)]


EXPORTS = [
    "quids_gpu_ctx_create", "quids_gpu_ctx_destroy", "quids_gpu_ctx_stream", "quids_gpu_ctx_synchronize",
    "quids_gpu_ctx_scratch_bytes", "quids_gpu_ctx_trim", "quids_gpu_status_string", "quids_gpu_ctx_launch_count",
    "quids_gpu_ctx_run_counts", "quids_gpu_ctx_last_tuning",
    "quids_gpu_state_create", "quids_gpu_state_destroy", "quids_gpu_state_upload", "quids_gpu_state_num_object",
    "quids_gpu_state_num_bytes", "quids_gpu_state_total_proba", "quids_gpu_state_download",
    "quids_gpu_state_download_async", "quids_gpu_state_download_wait",
    "quids_gpu_state_device_arrays", "quids_gpu_simulate", "quids_gpu_apply_modifier",
    "quids_gpu_rule_children", "quids_gpu_state_hash", "quids_gpu_rule_children_noalloc", "quids_gpu_run",
    "quids_gpu_average_value", "quids_gpu_qcgd_statistics", "quids_gpu_state_upload_batched",
    "quids_gpu_state_instances", "quids_gpu_simulate_batched", "quids_gpu_run_batched", "quids_gpu_tape_create",
    "quids_gpu_tape_destroy", "quids_gpu_forward", "quids_gpu_tape_final_state", "quids_gpu_simulate_backward",
    "quids_gpu_simulate_backward_observable", "quids_gpu_observable_adjoint",
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first if absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"CUDA library not built: {path}")
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    u64p = C.POINTER(C.c_uint64)
    L.quids_gpu_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.quids_gpu_ctx_destroy.argtypes = [vp]
    L.quids_gpu_ctx_stream.argtypes = [vp]
    L.quids_gpu_ctx_stream.restype = vp
    L.quids_gpu_ctx_synchronize.argtypes = [vp]
    L.quids_gpu_ctx_scratch_bytes.argtypes = [vp]
    L.quids_gpu_ctx_scratch_bytes.restype = C.c_uint64
    L.quids_gpu_ctx_trim.argtypes = [vp]
    L.quids_gpu_status_string.argtypes = [C.c_int]
    L.quids_gpu_status_string.restype = C.c_char_p
    L.quids_gpu_ctx_launch_count.argtypes = [vp]
    L.quids_gpu_ctx_launch_count.restype = C.c_uint64
    L.quids_gpu_ctx_run_counts.argtypes = [vp, u64p, u64p, u64p]
    L.quids_gpu_ctx_last_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.quids_gpu_state_create.argtypes = [vp, C.POINTER(vp)]
    L.quids_gpu_state_destroy.argtypes = [vp]
    L.quids_gpu_state_upload.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, C.c_uint64]
    L.quids_gpu_state_num_object.argtypes = [vp, u64p]
    L.quids_gpu_state_num_bytes.argtypes = [vp, u64p]
    L.quids_gpu_state_total_proba.argtypes = [vp, C.POINTER(C.c_double)]
    L.quids_gpu_state_download.argtypes = [vp, vp, vp, vp, vp]
    L.quids_gpu_state_download_async.argtypes = [vp, vp, vp, vp, vp]
    L.quids_gpu_state_download_wait.argtypes = [vp]
    L.quids_gpu_state_device_arrays.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
    L.quids_gpu_simulate.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), vp, C.POINTER(Params),
                                     C.POINTER(StepStats)]
    L.quids_gpu_apply_modifier.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams)]
    L.quids_gpu_run.argtypes = [vp, vp, vp, C.POINTER(Op), C.c_uint64, C.POINTER(Params), C.POINTER(StepStats),
                                C.POINTER(C.c_int)]
    L.quids_gpu_rule_children.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), u64p, u64p, vp, vp, vp, vp]
    L.quids_gpu_state_hash.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), vp]
    L.quids_gpu_average_value.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), C.POINTER(C.c_double)]
    L.quids_gpu_qcgd_statistics.argtypes = [vp, vp, C.c_uint64, C.c_uint64, C.c_double, C.POINTER(QcgdStats)]
    L.quids_gpu_rule_children_noalloc.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, C.c_int, C.POINTER(RuleParams),
                                                  C.c_uint64, u64p, u64p, vp, vp, vp, vp]
    L.quids_gpu_state_upload_batched.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, C.c_uint64, C.c_uint32, vp]
    L.quids_gpu_state_instances.argtypes = [vp, C.POINTER(C.c_uint32), vp, vp]
    L.quids_gpu_simulate_batched.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), vp, C.POINTER(Params), vp,
                                             C.POINTER(StepStats)]
    L.quids_gpu_run_batched.argtypes = [vp, vp, vp, C.POINTER(Op), C.c_uint64, C.POINTER(RuleParams),
                                        C.POINTER(Params), C.POINTER(StepStats), C.POINTER(C.c_int)]
    L.quids_gpu_tape_create.argtypes = [vp, C.POINTER(vp)]
    L.quids_gpu_tape_destroy.argtypes = [vp]
    L.quids_gpu_forward.argtypes = [vp, vp, vp, C.POINTER(Op), C.c_uint64, C.POINTER(Params), C.c_uint64, vp,
                                    C.POINTER(StepStats)]
    L.quids_gpu_tape_final_state.argtypes = [vp, vp]
    L.quids_gpu_simulate_backward.argtypes = [vp, vp, vp, vp]
    L.quids_gpu_simulate_backward_observable.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams),
                                                         C.POINTER(C.c_double), vp]
    L.quids_gpu_observable_adjoint.argtypes = [vp, vp, C.c_int, C.POINTER(RuleParams), C.POINTER(C.c_double), vp]
    _lib = L
    return L


def check(rc: int, what: str = "quids_gpu"):
    if rc != QUIDS_OK:
        raise QuidsError(rc, what)
