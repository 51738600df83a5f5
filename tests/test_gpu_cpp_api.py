"""The header-only C++ API (include/quids_gpu.hpp) on the GPU: a program that
defines its own rule and modifier as a reference user would
(tests/cpp/user_rules.cu) is compiled with nvcc, linked against the library
and run; its steps are checked against the oracle's Hadamard step
(src/rules/quantum_computer.hpp:31-50) on the same input, and against the
library's built-in rule bit for bit."""
import math
import os
import subprocess

import numpy as np
import pytest

from quids_gb300 import build as qbuild, capi, workloads as W
from tests.parity import assert_state_parity

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "user_rules.cu")
BIT = 5


def compile_user_program(out_dir):
    """nvcc for sm_103a against the public header; returns the executable"""
    lib = qbuild.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "user_rules")
    cmd = [qbuild.nvcc_path(), "-std=c++17", "-O2", *qbuild.ARCH, "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", libdir, "-lquids_gb300",
           "-Xlinker", f"-rpath={libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def write_state(path, p):
    objects, begin, size, mag = p
    n = len(size)
    with open(path, "wb") as f:
        f.write(np.array([n, int(begin[n])], np.uint64).tobytes())
        f.write(np.asarray(objects, np.uint8)[: int(begin[n])].tobytes())
        f.write(np.asarray(begin, np.uint64).tobytes())
        f.write(np.asarray(size, np.uint32).tobytes())
        f.write(np.asarray(mag, np.complex128).view(np.float64).tobytes())


def read_state(path):
    raw = open(path, "rb").read()
    n, nb = (int(x) for x in np.frombuffer(raw[:16], np.uint64))
    o = 16
    objects = np.frombuffer(raw[o: o + nb], np.uint8).copy()
    o += nb
    begin = np.frombuffer(raw[o: o + 8 * (n + 1)], np.uint64).copy()
    o += 8 * (n + 1)
    size = np.frombuffer(raw[o: o + 4 * n], np.uint32).copy()
    o += 4 * n
    mag = np.frombuffer(raw[o: o + 16 * n], np.float64).view(np.complex128).copy()
    return objects, begin, size, mag


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("cpp_api"))
    exe = compile_user_program(d)
    rng = W.Rng(23)
    objs = list(dict.fromkeys(bytes(rng.below(2) for _ in range(14)) for _ in range(3000)))
    mags = np.array([complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs])
    inp = W.pack(objs, mags / np.linalg.norm(mags), 8)
    write_state(os.path.join(d, "in.state"), inp)
    r = subprocess.run([exe, os.path.join(d, "in.state"), d, str(BIT)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    counts = [line.split() for line in open(os.path.join(d, "counts.txt"))]
    errors = [int(x) for x in open(os.path.join(d, "errors.txt")).read().split()]
    return d, inp, counts, errors


def test_user_rule_matches_the_oracle(run, port):
    d, inp, counts, _ = run
    port.set_globals(1e-18, True, 8)
    a, b = port.new_state(inp), port.new_state()
    nc, nu = port.simulate(a, W.RULE_HADAMARD, (BIT,), b)
    assert (int(counts[0][0]), int(counts[0][1])) == (nc, nu)
    assert float(counts[0][2]) == pytest.approx(b.total_proba, rel=1e-12)
    got = read_state(os.path.join(d, "user_hadamard.state"))
    assert_state_parity(got, b.store(), False, what="user hadamard")
    # the reference's rounding: every magnitude bit for bit when both sides
    # normalise by the same factor.  The oracle's total is an OpenMP sum (its
    # last bit depends on the thread count), the library's an exact one, so
    # the factors can differ by an ulp; then each magnitude is that ulp away.
    e_objs, e_mags = W.unpack(b.store())
    g_objs, g_mags = W.unpack(got)
    ref = dict(zip(e_objs, e_mags))
    exp = np.array([ref[o] for o in g_objs])
    if math.sqrt(float(counts[0][2])) == math.sqrt(b.total_proba):
        assert all(complex(m) == complex(r) for m, r in zip(g_mags, exp))
    else:
        assert np.allclose(g_mags, exp, rtol=1e-15, atol=0)


def test_user_rule_equals_the_builtin_rule(run):
    d, _, counts, _ = run
    assert counts[0] == counts[1]
    user = read_state(os.path.join(d, "user_hadamard.state"))
    builtin = read_state(os.path.join(d, "builtin_hadamard.state"))
    for u, v in zip(user, builtin):
        assert np.array_equal(u, v)


def test_user_modifier_then_user_rule(run, port):
    d, inp, counts, _ = run
    port.set_globals(1e-18, True, 8)
    a = port.new_state(inp)
    port.modifier(a, W.MOD_X, (BIT,))
    b = port.new_state()
    nc, nu = port.simulate(a, W.RULE_HADAMARD, (BIT,), b)
    assert (int(counts[2][0]), int(counts[2][1])) == (nc, nu)
    assert_state_parity(read_state(os.path.join(d, "user_x.state")), b.store(), False, what="user X then H")


def test_size_bound_lie_is_an_error(run):
    """A rule reporting children larger than the max_child_size it declared
    (the reference would overrun its scratch, src/quids.hpp:677) stops the
    step with QUIDS_ERR_SIZE_BOUND; the next step on the context runs."""
    _, _, counts, errors = run
    assert errors[0] == capi.ERR_SIZE_BOUND
    assert errors[1] > 0
