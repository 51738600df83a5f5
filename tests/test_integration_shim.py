"""The C++ shim shown for reference users (the ```cpp block of the
integration guide) compiles against include/quids_gpu.h, links against the
built library, and runs: without a context every call is rejected with
QUIDS_ERR_BAD_ARG.  No GPU is needed."""
import os
import re
import shutil
import subprocess

import pytest

from quids_gb300 import build as qbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MAIN = r"""
#include <cstdio>
int main() {
    quids::gpu::it_t a(nullptr), b(nullptr);
    quids::gpu::sy_it_t sy;
    quids_gpu_rule_params p{};
    std::printf("%d %zu\n", quids::gpu::simulate(nullptr, a, QUIDS_RULE_HADAMARD, p, b, sy), sy.num_object);
    return 0;
}
"""


def shim_source():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    assert len(blocks) == 1
    return blocks[0]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_cpp_shim_compiles_links_and_rejects_a_null_context(tmp_path):
    lib = qbuild.build()
    src = tmp_path / "shim.cpp"
    src.write_text(shim_source() + MAIN)
    exe = tmp_path / "shim"
    libdir = os.path.dirname(lib)
    cuda_lib = "/usr/local/cuda/lib64"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lquids_gb300", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{libdir}",
                    f"-Wl,-rpath,{cuda_lib}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["-1", "0"]


def test_python_example_names_exist_and_no_device_is_an_error():
    """The guide's Python example uses names the package has; without a GPU
    it stops at the context with the library's no-device status."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import quids_gb300 as quids
    from quids_gb300 import capi
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", text, flags=re.S)
    assert len(blocks) == 1
    with pytest.raises(capi.QuidsError, match="no CUDA device"):
        exec(blocks[0], {})
    for name in ("Context", "it_t", "sy_it_t", "simulate"):
        assert hasattr(quids, name), name
    assert hasattr(quids.it_t, "append")
