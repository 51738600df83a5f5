"""GPU parity: the CUDA rule step through the C ABI against the oracle and the
golden fixtures of the reference.  Every comparison is per step from an
identical input state (set parity keyed on bytes, magnitudes within 1e-12
relative floored at 1e-9, a tie band at truncation cutoffs)."""
import math

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W
from quids_gb300 import rules
from tests.parity import assert_state_parity, canon, is_qcgd_kind, load_golden, packed

pytestmark = pytest.mark.gpu
U64_MAX = capi.U64_MAX


@pytest.fixture(scope="module")
def ctx():
    c = quids.Context(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def knobs():
    quids.tolerance, quids.align_byte_length = 1e-18, 8
    yield
    quids.tolerance, quids.align_byte_length = 1e-18, 8


def gpu_step(ctx, p, kind, params, maxn=U64_MAX, flags=0):
    a, b = quids.it_t(ctx, p), quids.it_t(ctx)
    sy = quids.sy_it_t()
    quids.simulate(a, quids.rule_from(True, kind, params), b, sy, maxn, flags=flags)
    return b, sy


def test_golden_steps(ctx):
    z, man = load_golden()
    for k, case in enumerate(man["steps"]):
        quids.tolerance, quids.align_byte_length = case["tolerance"], case["align"]
        maxn = int(case["max"])
        for flags in (0, capi.FLAG_NO_FAST_HASH, capi.FLAG_PARTITION):
            b, sy = gpu_step(ctx, packed(z, f"step{k}_in"), case["kind"], case["params"], maxn, flags)
            what = f"{case['name']} flags={flags}"
            assert sy.num_object == case["num_object"], what
            assert sy.num_object_after_interferences == case["num_object_after_interferences"], what
            got = b.download()
            assert_state_parity(got, packed(z, f"step{k}_out"), is_qcgd_kind(case["kind"]),
                                truncated=maxn < case["num_object_after_interferences"], what=what)
            assert b.total_proba == pytest.approx(case["total_proba"], rel=1e-12, abs=1e-300), what
            # layout: offsets follow the requested alignment
            objects, begin, size, _ = got
            al = case["align"]
            if al > 1 and len(size):
                assert all(int(x) % al == 0 for x in begin), what


def test_golden_children_and_hashes(ctx, port):
    """Every child the GPU rule produces (bytes, magnitude, hash) against the
    reference's populate_child on the same parents."""
    z, man = load_golden()
    for ri, c in enumerate(man["children"]):
        pp = packed(z, f"children{ri}_parents")
        it = quids.it_t(ctx, pp)
        children, hashes, mags = quids.rule_children(it, quids.rule_from(True, c["kind"], c["params"]))
        parents, _ = W.unpack(pp)
        start = {}
        idx = 0
        for pi, g in enumerate(parents):
            start[pi] = idx
            idx += port.num_child(c["kind"], c["params"], g)[0]
        assert idx == len(children)
        outs, omags = W.unpack(packed(z, f"children{ri}_out"))
        for o, m, pi, cid in zip(outs, omags, z[f"children{ri}_pid"], z[f"children{ri}_cid"]):
            k = start[int(pi)] + int(cid)
            got = children[k]
            mk = W.graph_padding_mask(o) if c["kind"] != 1 else np.ones(len(o), bool)
            assert len(got) == len(o)
            assert (np.frombuffer(got, np.uint8)[mk] == np.frombuffer(o, np.uint8)[mk]).all()
            assert complex(mags[k]) == m  # same rounding as the reference: bit-exact
            href = port.hash_bytes(o) if c["kind"] == 1 else port.qcgd_hash_graph(o)
            assert int(hashes[k]) == href


def test_default_hasher_on_gpu_is_std_hash(ctx):
    z, _ = load_golden()
    data, lens, vals = z["hash_bytes_data"], z["hash_bytes_len"], z["hash_bytes_value"]
    objs, off = [], 0
    for L in lens:
        objs.append(data[off: off + int(L)].tobytes())
        off += int(L)
    for al in (8, 1):
        it = quids.it_t(ctx, W.pack(objs, [1.0] * len(objs), al))
        h = quids.state_hash(it, rules.hadamard(0))
        assert [int(x) for x in h] == [int(v) for v in vals]


def test_graph_hash_on_gpu(ctx):
    z, _ = load_golden()
    for al in (8, 0):
        objs, _ = W.unpack(packed(z, "graphs"))
        it = quids.it_t(ctx, W.pack(objs, [1.0] * len(objs), al))
        h = quids.state_hash(it, rules.coin(0.5))
        assert [int(x) for x in h] == [int(v) for v in z["graphs_hash"]]


def test_modifiers(ctx, port):
    rng = W.Rng(9)
    objs = list(dict.fromkeys(bytes(rng.below(2) for _ in range(11)) for _ in range(500)))
    mags = np.array([complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs])
    p = W.pack(objs, mags, 8)
    for kind, params in [(1, (2, 5)), (2, (3,)), (3, (4,)), (4, (0,)), (4, (10,))]:
        st = port.new_state(p)
        port.modifier(st, kind, params)
        it = quids.it_t(ctx, p)
        quids.simulate(it, quids.rule_from(False, kind, params))
        g, e = it.download(), st.store()
        assert np.array_equal(g[0], e[0]) and np.array_equal(g[1], e[1])
        assert np.array_equal(g[3], e[3])
    graphs = [W.random_graph(n, rng) for n in range(1, 20)]
    gp = W.pack(graphs, [1.0] * len(graphs), 8)
    for kind in (5, 6):
        st = port.new_state(gp)
        port.modifier(st, kind, ())
        it = quids.it_t(ctx, gp)
        quids.simulate(it, quids.rule_from(False, kind, ()))
        assert np.array_equal(it.download()[0], st.store()[0])


def _trajectory(ctx, port, p, gates, maxn, qcgd, check_every=True):
    a_gpu = quids.it_t(ctx, p)
    a_cpu = port.new_state(p)
    for gi, g in enumerate(gates):
        if g.kind == "mod":
            quids.simulate(a_gpu, quids.rule_from(False, g.code, g.params))
            port.modifier(a_cpu, g.code, g.params)
            continue
        # parity per step from an identical input: feed the GPU's input to the oracle
        inp = a_gpu.download()
        ref_in = port.new_state(inp)
        ref_out = port.new_state()
        nc, nu = port.simulate(ref_in, g.code, g.params, ref_out, maxn)
        b_gpu = quids.it_t(ctx)
        sy = quids.sy_it_t()
        quids.simulate(a_gpu, quids.rule_from(True, g.code, g.params), b_gpu, sy, maxn)
        assert (sy.num_object, sy.num_object_after_interferences) == (nc, nu), f"gate {gi}"
        if check_every or gi == len(gates) - 1:
            assert_state_parity(b_gpu.download(), ref_out.store(), qcgd, truncated=maxn < nu, what=f"gate {gi}")
        assert b_gpu.total_proba == pytest.approx(ref_out.total_proba, rel=1e-12)
        a_gpu = b_gpu
    return a_gpu


def test_circuit_small_full_trajectory(ctx, port):
    """12 qubits, Hadamard on each then 40 seeded gates, no truncation:
    set-exact after every gate against the oracle, and against the golden
    reference trajectory."""
    port.set_globals(1e-18, True, 8)
    _trajectory(ctx, port, W.qc_zero_state(12), W.circuit_small(0), U64_MAX, False)


def test_circuit_layers_truncated(ctx, port):
    """24 qubits, seeded layers, max_num_object 2^12 (truncation exercised)."""
    port.set_globals(1e-18, True, 8)
    gates = [g for layer in W.circuit_layers(0)[:4] for g in layer]
    _trajectory(ctx, port, W.qc_zero_state(24), gates, 1 << 12, False, check_every=False)


def test_qcgd_steps(ctx, port):
    """QCGD step/coin/split_merge/erase_create on an 8-node graph, 2 steps."""
    port.set_globals(1e-18, True, 8)
    _trajectory(ctx, port, W.qcgd_single_state(8, seed=1), W.qcgd_step_rules() * 2, U64_MAX, True)


def test_qcgd_truncated(ctx, port):
    port.set_globals(1e-18, True, 8)
    _trajectory(ctx, port, W.qcgd_single_state(9, seed=4), W.qcgd_step_rules() * 2, 2000, True)


def test_deterministic(ctx):
    p = W.qcgd_single_state(9, seed=2)
    outs = []
    for _ in range(2):
        it = quids.it_t(ctx, p)
        for g in W.qcgd_step_rules() * 2:
            if g.kind == "mod":
                quids.simulate(it, quids.rule_from(False, g.code, g.params))
            else:
                nxt = quids.it_t(ctx)
                quids.simulate(it, quids.rule_from(True, g.code, g.params), nxt, quids.sy_it_t(), 5000)
                it = nxt
        outs.append(it.download())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_empty_and_zero_children(ctx):
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    sy = quids.sy_it_t()
    quids.simulate(a, rules.hadamard(0), b, sy)
    assert b.num_object == 0 and sy.num_object == 0 and b.total_proba == 0
    # every child cancels: the state empties
    p = W.pack([bytes([0]), bytes([1])], [1 / math.sqrt(2), -1 / math.sqrt(2)], 8)
    # H|0> - H|1> = sqrt2 |1>: one survivor
    b2, sy2 = gpu_step(ctx, p, 1, (0,))
    assert sy2.num_object == 4 and sy2.num_object_after_interferences == 1 and b2.num_object == 1


def test_bad_arguments_are_errors(ctx):
    a = quids.it_t(ctx, W.qc_zero_state(4))
    with pytest.raises(capi.QuidsError):
        quids.simulate(a, rules.hadamard(0), a, quids.sy_it_t())
    b = quids.it_t(ctx)
    with pytest.raises(capi.QuidsError) as e:
        quids.simulate(a, rules._R(99, True), b, quids.sy_it_t())
    assert e.value.code == -1
    with pytest.raises(capi.QuidsError) as e:  # qubit beyond the object
        quids.simulate(a, rules.hadamard(9), b, quids.sy_it_t())
    assert e.value.code == -1
    # the context stays usable after an error
    quids.simulate(a, rules.hadamard(0), b, quids.sy_it_t())
    assert b.num_object == 2


def test_run_gate_list_equals_per_call(ctx):
    """quids_gpu_run (one call for a gate list) gives the same final state and
    counters as the same gates applied call by call."""
    gates = W.circuit_small(0)
    ops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in gates]
    a = quids.it_t(ctx, W.qc_zero_state(12))
    counts = []
    for r in ops:
        if not r.is_rule:
            quids.simulate(a, r)
            continue
        b, sy = quids.it_t(ctx), quids.sy_it_t()
        quids.simulate(a, r, b, sy)
        counts.append((sy.num_object, sy.num_object_after_interferences))
        a = b
    x, y = quids.it_t(ctx, W.qc_zero_state(12)), quids.it_t(ctx)
    final, stats = quids.run(x, y, ops)
    assert [(s["num_object"], s["num_object_after_interferences"]) for s in stats] == counts
    for u, v in zip(final.download(), a.download()):
        assert np.array_equal(u, v)
    assert final.total_proba == a.total_proba


def test_large_steps(ctx, port):
    """The 8.4M-child Hadamard applications of the 24-qubit circuit against the
    oracle from identical inputs, with truncation to 2^22 (exact ties at the
    cutoff); each with the collision table and with the partitioned stage."""
    from tests.parity import assert_fixed_state_parity
    port.set_globals(1e-18, True, 8)
    gates = [g for layer in W.circuit_layers(0) for g in layer]
    it = quids.it_t(ctx, W.qc_zero_state(24))
    checked = 0
    for g in gates:
        r = quids.rule_from(g.kind == "rule", g.code, g.params)
        if g.kind == "mod":
            quids.simulate(it, r)
            continue
        nxt, sy = quids.it_t(ctx), quids.sy_it_t()
        big = it.num_object >= (1 << 21)
        if big:
            inp = it.download()
        quids.simulate(it, r, nxt, sy, 1 << 22)
        if big:
            a, b = port.new_state(inp), port.new_state()
            nc, nu = port.simulate(a, g.code, g.params, b, 1 << 22)
            assert (sy.num_object, sy.num_object_after_interferences) == (nc, nu)
            assert_fixed_state_parity(nxt.download(), b.store(), truncated=nu > (1 << 22), what=f"H{g.params}")
            assert nxt.total_proba == pytest.approx(b.total_proba, rel=1e-12)
            # the collision table and the partitioned stage give the same state, bit for bit
            for fl in (capi.FLAG_TABLE, capi.FLAG_PARTITION):
                ra, rb, rsy = quids.it_t(ctx, inp), quids.it_t(ctx), quids.sy_it_t()
                quids.simulate(ra, r, rb, rsy, 1 << 22, flags=fl)
                assert (rsy.num_object, rsy.num_object_after_interferences) == (nc, nu)
                for u, v in zip(rb.download(), nxt.download()):
                    assert np.array_equal(u, v)
                assert rb.total_proba == nxt.total_proba
            checked += 1
            if checked == 3:
                break
        it = nxt
    assert checked == 3


def _qcgd_large(ctx, port, nodes, seed, cap, what):
    from tests.parity import assert_hashed_state_parity
    port.set_globals(1e-18, True, 8)
    it = quids.it_t(ctx, W.qcgd_single_state(nodes, seed=seed))
    for step in range(2):
        for g in W.qcgd_step_rules():
            r = quids.rule_from(g.kind == "rule", g.code, g.params)
            if g.kind == "mod":
                quids.simulate(it, r)
                continue
            nxt, sy = quids.it_t(ctx), quids.sy_it_t()
            if step == 1:
                inp = it.download()
            quids.simulate(it, r, nxt, sy, cap)
            if step == 1:
                a, b = port.new_state(inp), port.new_state()
                nc, nu = port.simulate(a, g.code, g.params, b, cap)
                assert (sy.num_object, sy.num_object_after_interferences) == (nc, nu), f"{what} rule {g.code}"
                assert_hashed_state_parity(ctx, nxt, b.store(), rules.coin(0.5), truncated=nu > cap,
                                           what=f"{what} rule {g.code}")
                assert nxt.total_proba == pytest.approx(b.total_proba, rel=1e-12)
            it = nxt


def test_qcgd_step1_10_nodes(ctx, port):
    """QCGD step 1 of a 10-node graph (6.4e7 children, 2^22 cap) per rule
    application against the oracle from identical inputs."""
    _qcgd_large(ctx, port, 10, 3, 1 << 22, "qcgd10")


def _host_ram_gb():
    with open("/proc/meminfo") as f:
        for line in f:
            if line.startswith("MemTotal:"):
                return int(line.split()[1]) / 2**20
    return 0.0


def test_qcgd_step1_12_nodes(ctx, port):
    """The 2^24-object QCGD step: step 1 of a 12-node graph (coin 1.0e7,
    split_merge 1.0e8, erase_create ~5.7e8 children, 2^24 cap) against the
    oracle from identical inputs.  The oracle needs ~60 GB of host memory."""
    if _host_ram_gb() < 150:
        pytest.skip("the CPU oracle of this step needs more host memory")
    _qcgd_large(ctx, port, 12, 1, 1 << 24, "qcgd12")


def test_probabilistic_truncation(ctx):
    """simple_truncation = false keeps the smallest u / norm (src/quids.hpp:594-608,
    :829-845).  A 1-node graph under erase_create has two children of norms
    2/3 and 1/3; keeping one, the first survives with probability
    1 - (1/3) / (2 * 2/3) = 3/4."""
    t = math.asin(math.sqrt(2 / 3))
    p = W.pack([W.make_graph(1, [0], [0])], [1.0], 8)
    quids.simple_truncation = False
    try:
        kept = []
        for seed in range(400):
            quids.truncation_seed = seed
            b, sy = gpu_step(ctx, p, W.RULE_QCGD_ERASE_CREATE, (t, 0.0, 0.0), 1)
            objs, mags = W.unpack(b.download())
            assert len(objs) == 1 and abs(abs(mags[0]) - 1) < 1e-12
            kept.append(objs[0][2])  # left bit: 1 for the flipped (2/3) child
        assert abs(sum(kept) / 400 - 0.75) < 0.07
        quids.truncation_seed = 7
        again = [W.unpack(gpu_step(ctx, p, 2, (t, 0.0, 0.0), 1)[0].download())[0][0][2] for _ in range(3)]
        assert len(set(again)) == 1 and again[0] == kept[7]
        # a cap above the number of survivors keeps everything, as simple truncation does
        c, _ = gpu_step(ctx, W.qcgd_single_state(6, seed=2), W.RULE_QCGD_COIN, W.COIN_DEFAULT, 1 << 20)
        quids.simple_truncation = True
        d, _ = gpu_step(ctx, W.qcgd_single_state(6, seed=2), W.RULE_QCGD_COIN, W.COIN_DEFAULT, 1 << 20)
        for u, v in zip(c.download(), d.download()):
            assert np.array_equal(u, v)
    finally:
        quids.simple_truncation = True
        quids.truncation_seed = 0


def test_automatic_truncation(ctx, port):
    """max_num_object = 0: as many top-norm parents as the memory budget
    allows (src/quids.hpp:459-485), then as many survivors as fit."""
    rng = W.Rng(17)
    objs = list(dict.fromkeys(bytes(rng.below(2) for _ in range(16)) for _ in range(5000)))[:4096]
    mags = np.array([complex(rng.uniform(-1, 1), rng.uniform(-1, 1)) for _ in objs])
    mags /= np.linalg.norm(mags)
    p = W.pack(objs, mags, 8)
    full, sy_full = gpu_step(ctx, p, 1, (5,), 0)  # default budget: everything fits
    ref, sy_ref = gpu_step(ctx, p, 1, (5,), U64_MAX)
    for u, v in zip(full.download(), ref.download()):
        assert np.array_equal(u, v)
    per_child = 38 + 96 + 32
    budget = 2000 * 2 * per_child
    quids.memory_budget = budget
    try:
        b, sy = gpu_step(ctx, p, 1, (5,), 0)
    finally:
        quids.memory_budget = 0
    kept = sy.stats["num_parents_kept"]
    assert 1900 <= kept <= 2000 and sy.num_object == 2 * kept
    assert sy.num_object * per_child <= budget
    assert 0 < b.num_object <= sy.num_object_after_interferences
    # The kept parents are the `kept` of largest norm (ties: lower index;
    # the random norms here have none), in their input order
    # (src/quids.hpp:613-642): the oracle's step on exactly those parents
    # has the GPU's child and group counts ...
    norms = np.abs(mags) ** 2
    top = np.sort(np.argsort(-norms, kind="stable")[:kept])
    sub = W.pack([objs[i] for i in top], mags[top], 8)
    port.set_globals(1e-18, True, 8)
    a, c = port.new_state(sub), port.new_state()
    nc, nu = port.simulate(a, 1, (5,), c, U64_MAX)
    assert (sy.num_object, sy.num_object_after_interferences) == (nc, nu)
    # ... and the survivors, cut to what the budget left for them
    # (src/quids.hpp:510-536), are the oracle's groups of largest norm,
    # renormalised (a tie band at the cutoff)
    e_objs, e_mags = W.unpack(c.store())
    assert b.num_object < len(e_objs), "the survivor budget binds in this case"
    pick = np.sort(np.argsort(-np.abs(e_mags) ** 2, kind="stable")[:b.num_object])
    kept_mags = e_mags[pick]
    exp = W.pack([e_objs[i] for i in pick], kept_mags / np.linalg.norm(kept_mags), 8)
    assert_state_parity(b.download(), exp, False, truncated=True, what="memory-driven truncation")
    # total_proba is the survivors' norm before normalising; the oracle's
    # magnitudes are normalised over all its groups
    assert b.total_proba == pytest.approx(float(np.sum(np.abs(kept_mags) ** 2)) * c.total_proba, rel=1e-12)


def test_observables(ctx):
    st = quids.it_t(ctx, W.qcgd_single_state(8, seed=5))
    a = st
    for g in W.qcgd_step_rules():
        r = quids.rule_from(g.kind == "rule", g.code, g.params)
        if g.kind == "mod":
            quids.simulate(a, r)
            continue
        nxt, sy = quids.it_t(ctx), quids.sy_it_t()
        quids.simulate(a, r, nxt, sy)
        a = nxt
    objs, mags = W.unpack(a.download())
    w = np.abs(mags) ** 2
    n = np.array([W.graph_num_nodes(o) for o in objs], dtype=float)
    dens = np.array([sum(o[2: 2 + 2 * int(k)]) / (2 * k) for o, k in zip(objs, n)])
    assert quids.average_value(a, quids.OBS_QCGD_NUM_NODES) == pytest.approx((w * n).sum(), rel=1e-12)
    assert quids.average_value(a, quids.OBS_QCGD_NUM_NODES_SQ) == pytest.approx((w * n * n).sum(), rel=1e-12)
    assert quids.average_value(a, quids.OBS_QCGD_DENSITY) == pytest.approx((w * dens).sum(), rel=1e-12)
    stats = quids.qcgd_statistics(a, sy)
    assert stats["num_graphs"] == len(objs)
    assert stats["interference_ratio"] == pytest.approx(sy.num_object_after_interferences / sy.num_object)
    assert stats["deletion_ratio"] == pytest.approx(len(objs) / sy.num_object_after_interferences)
    assert stats["avg_size"] == pytest.approx((w * n).sum(), rel=1e-12)
    q = quids.it_t(ctx, W.pack([bytes([1, 0, 1]), bytes([0, 1, 1])], [0.6, 0.8j], 8))
    assert quids.average_value(q, quids.OBS_QC_BIT, bit=0) == pytest.approx(0.36)
    assert quids.average_value(q, quids.OBS_QC_BIT, bit=2) == pytest.approx(1.0)


@pytest.mark.parametrize("simple", [True, False])
@pytest.mark.parametrize("maxn", [U64_MAX, 3000, 700])
def test_partitioned_collisions_equal_table(ctx, simple, maxn):
    """The partitioned collision stage (per-block shared-memory tables, a
    child-indexed bitmap for the order) and the open-addressing table give
    the same steps bit for bit: QCGD trajectories with and without
    truncation, simple and probabilistic, plus a Hadamard layer with massive
    exact ties at the cutoff."""
    quids.simple_truncation = simple
    quids.truncation_seed = 11
    try:
        ops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in W.qcgd_step_rules() * 2]
        runs = []
        for fl in (capi.FLAG_TABLE | capi.FLAG_NO_PLAN, capi.FLAG_PARTITION | capi.FLAG_NO_PLAN):
            fin, st = quids.run(quids.it_t(ctx, W.qcgd_single_state(9, seed=4)), quids.it_t(ctx), ops, maxn, fl)
            runs.append((fin.download(), [(x["num_object"], x["num_object_after_interferences"],
                                           x["num_object_out"]) for x in st], fin.total_proba))
        assert runs[0][1] == runs[1][1]
        for u, v in zip(runs[0][0], runs[1][0]):
            assert np.array_equal(u, v)
        assert runs[0][2] == runs[1][2]
        gates = [g for layer in W.circuit_layers(0)[:3] for g in layer]
        hops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in gates]
        outs = []
        for fl in (capi.FLAG_TABLE | capi.FLAG_NO_PLAN, capi.FLAG_PARTITION | capi.FLAG_NO_PLAN):
            fin, _ = quids.run(quids.it_t(ctx, W.qc_zero_state(24)), quids.it_t(ctx), hops, maxn, fl)
            outs.append(fin.download())
        for u, v in zip(*outs):
            assert np.array_equal(u, v)
    finally:
        quids.simple_truncation = True
        quids.truncation_seed = 0


def test_partitioned_collisions_in_planned_runs(ctx):
    """Repeated runs with the partitioned stage: synchronous, planned (sizes
    on the device) and replayed as a CUDA graph, all equal to the table's
    synchronous steps bit for bit."""
    ops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in W.qcgd_step_rules() * 2]
    init = W.qcgd_single_state(9, seed=4)
    ref, ref_st = quids.run(quids.it_t(ctx, init), quids.it_t(ctx), ops, 2000, capi.FLAG_TABLE | capi.FLAG_NO_PLAN)
    ref = ref.download()
    a, b = quids.it_t(ctx), quids.it_t(ctx)
    counts0 = ctx.run_counts()
    for _ in range(4):
        a.upload(init)
        fin, st = quids.run(a, b, ops, 2000, capi.FLAG_PARTITION)
        assert [x["num_object_out"] for x in st] == [x["num_object_out"] for x in ref_st]
        for u, v in zip(fin.download(), ref):
            assert np.array_equal(u, v)
    counts = {k: v - counts0[k] for k, v in ctx.run_counts().items()}
    assert counts["planned"] >= 2 and counts["graph"] >= 1, counts
