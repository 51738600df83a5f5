"""The integration surfaces build without a GPU: a program written against
the header-only C++ API (include/quids_gpu.hpp) with its own rule and
modifier (tests/cpp/user_rules.cu) compiles for sm_103a and links against the
library; the integration guide's Python example (tests/shim/python_example.py)
uses existing names and stops at the context with the no-device status."""
import os
import runpy
import shutil

import pytest

from quids_gb300 import capi
from tests.test_gpu_cpp_api import compile_user_program

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="no nvcc")
def test_user_rule_program_compiles_and_links(tmp_path):
    exe = compile_user_program(str(tmp_path))
    assert os.path.getsize(exe) > 0


def test_python_example_names_exist_and_no_device_is_an_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import quids_gb300 as quids
    with pytest.raises(capi.QuidsError, match="no CUDA device"):
        runpy.run_path(os.path.join(ROOT, "tests", "shim", "python_example.py"))
    for name in ("Context", "it_t", "sy_it_t", "simulate"):
        assert hasattr(quids, name), name
    assert hasattr(quids.it_t, "append")
