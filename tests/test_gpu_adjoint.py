"""GPU adjoint: gradients of the expected node count after T QCGD steps with
respect to the six rule angles (split_merge and erase_create theta, phi,
xi), from quids_gpu_simulate_backward, against central finite differences
(h = 1e-6) of the plain GPU forward and of the CPU oracle forward.
Tolerance, per component k: |adjoint_k - fd_k| <= 1e-6 |fd_k| + FD_FLOOR |L|,
where the absolute floor covers the central difference's own rounding."""
import math

import numpy as np
import pytest

import quids_gb300 as quids
from quids_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
U64_MAX = capi.U64_MAX
H = 1e-6
RTOL = 1e-6
# A central difference divides the rounding of the two losses by 2h: a loss
# L summed over up to ~1e6 objects carries a few 1e-15 |L| of rounding, so
# the difference quotient is only known to about 1e-15 |L| / 2e-6 = 5e-10 |L|.
# Components smaller than FD_FLOOR |L| / RTOL are checked to that floor.
FD_FLOOR = 2e-9


@pytest.fixture(scope="module")
def ctx():
    c = quids.Context(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def knobs():
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = 1e-18, 8, True
    yield
    quids.tolerance, quids.align_byte_length, quids.simple_truncation = 1e-18, 8, True


def rule_ops(angles, n_steps):
    gates, slots = W.qcgd_adjoint_ops(list(angles), n_steps)
    return [quids.rule_from(g.kind == "rule", g.code, g.params) for g in gates], slots, gates


def adjoint_grad(ctx, init, angles, n_steps, maxn, every=1):
    ops, slots, _ = rule_ops(angles, n_steps)
    tape = quids.Tape(ctx)
    tape.forward(quids.it_t(ctx, init), ops, maxn, every)
    loss, g = tape.backward_observable(quids.OBS_QCGD_NUM_NODES)
    grad = np.zeros(6)
    for oi, comp, ai in slots:
        grad[ai] += g[oi, comp]
    return loss, grad, g


def gpu_loss(ctx, init, angles, n_steps, maxn):
    ops, _, _ = rule_ops(angles, n_steps)
    fin, _ = quids.run(quids.it_t(ctx, init), quids.it_t(ctx), ops, maxn)
    return quids.average_value(fin, quids.OBS_QCGD_NUM_NODES)


def oracle_loss(port, init, angles, n_steps, maxn):
    _, _, gates = rule_ops(angles, n_steps)
    s = port.new_state(init)
    for g in gates:
        if g.kind == "mod":
            port.modifier(s, g.code, g.params)
        else:
            t = port.new_state()
            port.simulate(s, g.code, g.params, t, maxn)
            s = t
    return node_count(s.store())


def node_count(p):
    objs, mags = W.unpack(p)
    return float(sum(W.graph_num_nodes(o) * abs(m) ** 2 for o, m in zip(objs, mags)))


# A truncation keeps the top max_num_object norms; a finite difference that
# lets the kept set change measures the jumps of the set, not the
# derivative.  The adjoint holds every mask fixed, so under truncation it is
# checked against finite differences of a forward with the masks of the
# unperturbed run: each rule step runs without a cap, then keeps exactly the
# objects the unperturbed truncated step kept (by graph hash) and
# renormalises.
GRAPH_HASH = quids.rules.split_merge(0.0)


def subset(p, keep):
    objects, begin, size, mag = p
    objs = [objects[int(begin[i]): int(begin[i]) + int(size[i])].tobytes() for i in np.nonzero(keep)[0]]
    m = np.asarray(mag)[keep]
    m = m / math.sqrt(float(np.sum(np.abs(m) ** 2)))
    return W.pack(objs, list(m), 8)


def masks_of(ctx, init, angles, n_steps, maxn):
    """the hashes of the objects each truncated rule step keeps"""
    ops, _, _ = rule_ops(angles, n_steps)
    a = quids.it_t(ctx, init)
    masks = []
    for op in ops:
        if not op.is_rule:
            quids.simulate(a, op)
            continue
        b = quids.it_t(ctx)
        quids.simulate(a, op, b, quids.sy_it_t(), maxn)
        masks.append(np.sort(quids.state_hash(b, GRAPH_HASH)))
        a = b
    return masks


def masked_gpu_loss(ctx, init, angles, n_steps, masks):
    ops, _, _ = rule_ops(angles, n_steps)
    a = quids.it_t(ctx, init)
    r = 0
    for op in ops:
        if not op.is_rule:
            quids.simulate(a, op)
            continue
        b = quids.it_t(ctx)
        quids.simulate(a, op, b, quids.sy_it_t())
        keep = np.isin(quids.state_hash(b, GRAPH_HASH), masks[r])
        a = quids.it_t(ctx, subset(b.download(), keep))
        r += 1
    return quids.average_value(a, quids.OBS_QCGD_NUM_NODES)


def masked_oracle_loss(ctx, port, init, angles, n_steps, masks):
    _, _, gates = rule_ops(angles, n_steps)
    s = port.new_state(init)
    r = 0
    for g in gates:
        if g.kind == "mod":
            port.modifier(s, g.code, g.params)
            continue
        t = port.new_state()
        port.simulate(s, g.code, g.params, t)
        p = t.store()
        keep = np.isin(quids.state_hash(quids.it_t(ctx, p), GRAPH_HASH), masks[r])
        s = port.new_state(subset(p, keep))
        r += 1
    return node_count(s.store())


def fd_grad(loss_fn, angles):
    g = np.zeros(6)
    for k in range(6):
        up, dn = list(angles), list(angles)
        up[k] += H
        dn[k] -= H
        g[k] = (loss_fn(up) - loss_fn(dn)) / (2 * H)
    return g


def assert_grad_close(got, exp, what, loss):
    got, exp = np.asarray(got, np.float64), np.asarray(exp, np.float64)
    tol = RTOL * np.abs(exp) + FD_FLOOR * max(abs(loss), 1.0)
    err = np.abs(got - exp)
    rel = err / np.maximum(np.abs(exp), 1e-300)
    assert (err <= tol).all(), (f"{what}: components {np.nonzero(err > tol)[0].tolist()} off; relative errors "
                                f"{np.array2string(rel, precision=2)}; adjoint {got} fd {exp}")


@pytest.mark.parametrize("n_nodes,n_steps", [(6, 2), (4, 3)])
def test_adjoint_against_gpu_finite_differences(ctx, n_nodes, n_steps):
    init, angles = W.qcgd_adjoint_workload(n_nodes, seed=3)
    loss, grad, _ = adjoint_grad(ctx, init, angles, n_steps, U64_MAX, every=2)
    assert loss == pytest.approx(gpu_loss(ctx, init, angles, n_steps, U64_MAX), rel=1e-12)
    fd = fd_grad(lambda a: gpu_loss(ctx, init, a, n_steps, U64_MAX), angles)
    assert_grad_close(grad, fd, f"{n_nodes} nodes, {n_steps} steps", loss)


@pytest.mark.parametrize("n_nodes,n_steps,maxn", [(8, 3, 2000), (10, 3, 1024)])
def test_adjoint_truncated_against_gpu_finite_differences(ctx, n_nodes, n_steps, maxn):
    init, angles = W.qcgd_adjoint_workload(n_nodes, seed=3)
    loss, grad, _ = adjoint_grad(ctx, init, angles, n_steps, maxn, every=2)
    masks = masks_of(ctx, init, angles, n_steps, maxn)
    assert any(len(m) == maxn for m in masks), "the case truncates"
    assert masked_gpu_loss(ctx, init, angles, n_steps, masks) == pytest.approx(loss, rel=1e-12)
    fd = fd_grad(lambda a: masked_gpu_loss(ctx, init, a, n_steps, masks), angles)
    assert_grad_close(grad, fd, f"{n_nodes} nodes, {n_steps} steps, max {maxn}", loss)


def test_adjoint_against_oracle_finite_differences(ctx, port):
    init, angles = W.qcgd_adjoint_workload(5, seed=3)
    loss, grad, _ = adjoint_grad(ctx, init, angles, 2, U64_MAX)
    fd = fd_grad(lambda a: oracle_loss(port, init, a, 2, U64_MAX), angles)
    assert_grad_close(grad, fd, "oracle forward", loss)


def test_adjoint_truncated_against_oracle_finite_differences(ctx, port):
    init, angles = W.qcgd_adjoint_workload(7, seed=3)
    n_steps, maxn = 2, 400
    loss, grad, _ = adjoint_grad(ctx, init, angles, n_steps, maxn)
    masks = masks_of(ctx, init, angles, n_steps, maxn)
    assert any(len(m) == maxn for m in masks), "the case truncates"
    fd = fd_grad(lambda a: masked_oracle_loss(ctx, port, init, a, n_steps, masks), angles)
    assert_grad_close(grad, fd, "oracle forward, masks held", loss)


def test_checkpoint_interval_does_not_change_gradients(ctx):
    """Recomputed segments replay the forward bit for bit, so every
    checkpoint interval gives the same gradients."""
    init, angles = W.qcgd_adjoint_workload(7, seed=3)
    ref = adjoint_grad(ctx, init, angles, 4, 1500, every=1)[2]
    for every in (2, 5, 7, 1000):
        g = adjoint_grad(ctx, init, angles, 4, 1500, every=every)[2]
        assert np.array_equal(g, ref), f"checkpoint every {every}"


def test_backward_with_host_adjoint(ctx):
    init, angles = W.qcgd_adjoint_workload(6, seed=3)
    ops, _, _ = rule_ops(angles, 2)
    tape = quids.Tape(ctx)
    fin, _ = tape.forward(quids.it_t(ctx, init), ops, 1000, 3)
    loss, a = quids.observable_adjoint(fin, quids.OBS_QCGD_NUM_NODES)
    objs, mags = W.unpack(fin.download())
    w = np.array([W.graph_num_nodes(o) for o in objs], np.float64)
    assert np.allclose(a, 2 * w * np.asarray(mags), rtol=0, atol=1e-15)
    g_host = tape.backward(a)
    loss2, g_obs = tape.backward_observable(quids.OBS_QCGD_NUM_NODES)
    assert loss == pytest.approx(loss2, rel=1e-14)
    assert np.allclose(g_host, g_obs, rtol=1e-13, atol=1e-15)


def test_torch_autograd_function(ctx):
    torch = pytest.importorskip("torch")
    from quids_gb300.autograd import expected_value
    init, angles = W.qcgd_adjoint_workload(6, seed=3)

    def build(a):
        ops, slots, _ = rule_ops(a, 2)
        return ops, slots

    f = expected_value(init, build, quids.OBS_QCGD_NUM_NODES, U64_MAX, 2, ctx)
    x = torch.tensor(angles, dtype=torch.float64, requires_grad=True)
    loss = f(x)
    loss.backward()
    fd = fd_grad(lambda a: gpu_loss(ctx, init, a, 2, U64_MAX), angles)
    assert_grad_close(x.grad.numpy(), fd, "torch.autograd", float(loss))


def test_adjoint_unsupported_and_bad_arguments(ctx):
    init, angles = W.qcgd_adjoint_workload(5, seed=3)
    tape = quids.Tape(ctx)
    with pytest.raises(quids.QuidsError) as e:
        tape.forward(quids.it_t(ctx, init), [quids.rules.Zgate(0)], 100)
    assert e.value.code == -9  # a modifier that changes magnitudes
    ops, _, _ = rule_ops(angles, 1)
    with pytest.raises(quids.QuidsError) as e:
        tape.forward(quids.it_t(ctx, init), ops, 0)
    assert e.value.code == -9  # memory-driven cap
    fresh = quids.Tape(ctx)
    with pytest.raises(quids.QuidsError) as e:
        fresh.backward_observable(quids.OBS_QCGD_NUM_NODES)
    assert e.value.code == -1  # no forward run yet
