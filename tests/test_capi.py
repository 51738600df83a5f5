"""The C ABI library: it builds for sm_103a, loads, and exports every
function include/quids_gpu.h declares.  No compute call is made here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from quids_gb300 import build as qbuild
from quids_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "quids_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(quids_gpu_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    return qbuild.build()


def test_header_declares_the_abi():
    names = declared_functions()
    assert "quids_gpu_simulate" in names and "quids_gpu_apply_modifier" in names
    assert set(names) == set(capi.EXPORTS)


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (quids_gpu_\w+)", out))
    missing = set(declared_functions()) - exported
    assert not missing, f"not exported: {sorted(missing)}"


def test_library_loads_with_ctypes(lib_path):
    L = capi.load()
    for name in declared_functions():
        assert getattr(L, name) is not None
    assert L.quids_gpu_status_string(-3) == b"collision table full"


def test_built_for_sm103a_only():
    assert qbuild.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_flags_match_the_header():
    """capi.py's QUIDS_FLAG_* values are the header's."""
    text = open(HEADER).read()
    flags = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define QUIDS_FLAG_(\w+) (\d+)u", text)}
    assert flags, "no QUIDS_FLAG_* in the header"
    for name, value in flags.items():
        assert getattr(capi, "FLAG_" + name) == value, name


def test_no_device_is_an_error_not_a_crash(lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = capi.load()
    h = C.c_void_p()
    assert L.quids_gpu_ctx_create(0, C.byref(h)) == -8


def test_null_handles_are_bad_arg_not_a_crash(lib_path):
    """Every status-returning entry point, called with null handles and
    pointers and zero sizes, returns QUIDS_ERR_BAD_ARG before any CUDA call
    (so here, with no GPU, not QUIDS_ERR_NO_DEVICE)."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    status_fns = sorted(set(re.findall(r"^int (quids_gpu_\w+)\s*\(", text, flags=re.M)))
    assert len(status_fns) > 30
    raw = C.CDLL(lib_path)  # a separate handle: no argtypes, every argument NULL / 0
    for name in status_fns:
        f = getattr(raw, name)
        f.restype = C.c_int
        assert f(*([None] * 20)) == -1, name


def test_params_struct_layout_matches_the_header(tmp_path):
    """ctypes' mirror of quids_gpu_params and quids_gpu_step_stats has the C
    layout (size and the offsets of the last fields)."""
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "quids_gpu.h"\nint main(void) {\n'
                   '  printf("%zu %zu %zu %zu %zu\\n", sizeof(quids_gpu_params), offsetof(quids_gpu_params, max_probes),'
                   ' offsetof(quids_gpu_params, max_alloc_bytes), sizeof(quids_gpu_step_stats),'
                   ' offsetof(quids_gpu_step_stats, hash_ranges));\n  return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [C.sizeof(capi.Params), capi.Params.max_probes.offset, capi.Params.max_alloc_bytes.offset,
                   C.sizeof(capi.StepStats), capi.StepStats.hash_ranges.offset]
