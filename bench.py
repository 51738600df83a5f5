"""Benchmark of the QuIDS rule step on GB300: child objects/s per simulate() step.

Workload (default "qcgd12"): the 2^24-object QCGD step -- one step of the
QCGD rule sequence (step, coin(pi/4), split_merge(pi/4, 0, -pi/2),
erase_create(pi/3, pi/5, 0)) on a 12-node cycle graph (Bernoulli(0.5) bits,
seed 1), from the 149,760-object state after the first step, max_num_object
2^24, simple truncation, tolerance 1e-18, align 8: 7.3e8 children, 2^24
survivors.  The metric is the sum of symbolic children over the step's rule
applications divided by the step time.  The line also carries the batched
form against the plain path run instance by instance ("batched_vs_plain",
the batch256 workload) and the adjoint's forward + backward against the
plain forward ("adjoint_vs_forward", the adjoint10 workload), measured after
the main line on the same GPU (--no-extras leaves them out).

"circuit24": the plain quantum_computer rule at scale -- 24 qubits at one
byte each, all |0>, 6 seeded layers (Hadamard rule on a random half of the
qubits, then 24 random CNOT/Z modifiers), max_num_object 2^22.  One bench
step is the whole circuit from |0...0> (72 rule applications, 144
modifiers).

"batch256": the batched form -- 256 independent QCGD instances (cycle
graphs of U[4,16] nodes, Bernoulli(0.5) bits, per-instance split_merge and
erase_create angles, seed 2), max_num_object 2^18 per instance; one bench
step is the first QCGD step of every instance in one pipeline per rule
(quids_gpu_run_batched).  The same step run instance by instance through
the plain path is timed beside it ("plain_instance_by_instance").  Later
steps do not fit one GPU: the coin rule of the second step has more than
2^32 children (about 4.7e10).

"adjoint10": the adjoint -- a 10-node cycle graph (seed 3), T = 20 QCGD
steps with split_merge / erase_create angles U(0, pi) from seed 3,
max_num_object 2^22; one bench step is the taped forward plus
simulate_backward of the expected node count (checkpoints every 5 QCGD
steps); the value counts the forward's children per second of the whole
forward + backward, and the plain forward is timed beside it.

Every bench step runs from the same two state handles, the input uploaded
before the step: the first warm-up step is the synchronous steps, the next
are planned runs (sizes from the first, no host waits), autotuned and
captured as a CUDA graph that the timed steps replay (quids_gpu_run with
QUIDS_FLAG_AUTOTUNE; config.runs_timed counts how the timed steps ran).  The
stage timing pass runs the synchronous steps with CUDA events per stage.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]

--impl reference times the reference's CPU algorithm on all host cores: the
reference compiled from its own headers (oracle/_ref) where it was built on
this host, else its restatement (oracle/quids_port.cpp, OpenMP + libstdc++
parallel mode).
Under torchrun each rank runs an independent replica (the step does not
shard across GPUs); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "child objects/s per simulate() step"
UNIT = "children/s"
MAX24 = 1 << 22
L2_BYTES = 129 * 1024 * 1024
# DRAM traffic of the dominant stage is not measured in this process (ncu
# cannot run inside it): a recorded ncu figure per workload, with the
# profile it comes from.  dram__bytes_read.sum + dram__bytes_write.sum over
# the stage's kernels, per rule application of the timed step.
#
# qcgd12 holds about 60 GB on the device, too much for ncu's replay, so its
# figure comes from a capture of qcgd10's erase_create application (whose
# table, like qcgd12's, is far larger than L2), scaled by qcgd12's units:
# the grouped symbolic pass with its fused table claim moved 10.98 GB for
# 6.06e7 children (181 B per child) and the table clear before it 16 B per
# slot; qcgd12's three applications have 7.26e8 children and 1.45e9 slots:
# 154.6 GB per step, 51.5 GB per application.
RECORDED_TRAFFIC = {
    ("qcgd12", "symbolic+table_claim", "table"): {
        "bytes_per_launch": 51.5e9,
        "source": "profiles/symbolic_table_claim_qcgd10.md (ncu capture of qcgd10's erase_create grouped pass "
                  "with its fused table claim and the table clear, scaled to qcgd12's children and slots)"},
}


# ------------------------------------------------------------------ workloads
def workload(name):
    from quids_gb300 import workloads as W
    if name == "circuit24":
        gates = [g for layer in W.circuit_layers(0) for g in layer]
        return {"name": name, "init": W.qc_zero_state(24), "gates": gates, "max": MAX24, "tolerance": 1e-18,
                "align": 8, "config": {"workload": "quantum_computer circuit, 24 qubits x 1 byte, 6 layers "
                                       "(H on a seeded random half + 24 CNOT/Z), max_num_object 2^22",
                                       "qubits": 24, "layers": 6, "max_num_object": MAX24, "seed": 0,
                                       "tolerance": 1e-18, "align_byte_length": 8}}
    if name in ("qcgd12", "qcgd10"):
        nodes, seed, cap = (12, 1, 1 << 24) if name == "qcgd12" else (10, 3, 1 << 22)
        # the reference arm's bounded sample: the first quarter of the
        # 149,760 objects of the input (about 3 s per step on 16 cores)
        ref_sample = 37440 if name == "qcgd12" else None
        return {"name": name, "init": None, "nodes": nodes, "seed": seed, "gates": W.qcgd_step_rules(), "max": cap,
                "tolerance": 1e-18, "align": 8, "ref_sample_objects": ref_sample,
                "config": {"workload": f"QCGD step 1 (step, coin(pi/4), split_merge(pi/4,0,-pi/2), "
                                       f"erase_create(pi/3,pi/5,0)) of a {nodes}-node cycle graph, from the "
                                       f"state after step 0, max_num_object 2^{cap.bit_length() - 1}",
                           "nodes": nodes, "seed": seed, "max_num_object": cap, "tolerance": 1e-18,
                           "align_byte_length": 8}}
    if name == "qcgd12s2":
        cap = 1 << 24
        return {"name": name, "init": None, "nodes": 12, "seed": 1, "gates": W.qcgd_step_rules(), "max": cap,
                "pre_steps": 2, "cpu_sample_objects": 1 << 20, "tolerance": 1e-18, "align": 8,
                "config": {"workload": "QCGD step 2 (step, coin(pi/4), split_merge(pi/4,0,-pi/2), "
                                       "erase_create(pi/3,pi/5,0)) of a 12-node cycle graph, from the 2^24-object "
                                       "state after steps 0-1, max_num_object 2^24: coin has 3.15e9 children "
                                       "(beyond 2^31 table slots: hash-range passes)",
                           "nodes": 12, "seed": 1, "max_num_object": cap, "tolerance": 1e-18,
                           "align_byte_length": 8}}
    if name == "batch256":
        insts = W.qcgd_batch_instances(256, 2, 4, 16)
        return {"name": name, "insts": insts, "max": 1 << 18, "tolerance": 1e-18, "align": 8,
                "config": {"workload": "batched QCGD: 256 instances (cycle graphs, U[4,16] nodes, per-instance "
                                       "split_merge/erase_create angles, seed 2), first step (step, coin, "
                                       "split_merge, erase_create) of all instances in one pipeline per rule, "
                                       "max_num_object 2^18 per instance",
                           "instances": 256, "seed": 2, "max_num_object": 1 << 18, "tolerance": 1e-18,
                           "align_byte_length": 8}}
    if name == "adjoint10":
        init, angles = W.qcgd_adjoint_workload(10, seed=3)
        return {"name": name, "init": init, "angles": angles, "T": 20, "every": 15, "max": 1 << 22,
                "tolerance": 1e-18, "align": 8,
                "config": {"workload": "adjoint: gradient of the expected node count after 20 QCGD steps (step, "
                                       "coin, split_merge, erase_create) of a 10-node cycle graph with respect to "
                                       "the 6 split_merge/erase_create angles, max_num_object 2^22, checkpoints "
                                       "every 5 steps", "nodes": 10, "seed": 3, "T": 20,
                           "max_num_object": 1 << 22, "tolerance": 1e-18, "align_byte_length": 8}}
    raise SystemExit(f"unknown config {name}")


def qcgd_initial_cpu(wl, o):
    """State after the QCGD steps before the timed one (computed by the CPU
    oracle, for its own timing), cut to the CPU sample."""
    from quids_gb300 import workloads as W
    s = o.new_state(W.qcgd_single_state(wl["nodes"], seed=wl["seed"]))
    for _ in range(wl.get("pre_steps", 1)):
        for g in wl["gates"]:
            if g.kind == "mod":
                o.modifier(s, g.code, g.params)
            else:
                t = o.new_state()
                o.simulate(s, g.code, g.params, t, wl["max"])
                s = t
    return cpu_sample(wl, s.store())


def cpu_sample(wl, packed):
    """The first cpu_sample_objects objects of a state (the CPU's bounded
    sample of a workload too large for it), else the state."""
    n = wl.get("cpu_sample_objects")
    objects, begin, size, mag = packed
    if not n or n >= len(size):
        return packed
    return (objects[:int(begin[n])].copy(), begin[:n + 1].copy(), size[:n].copy(), mag[:n].copy())


# ------------------------------------------------------------------ helpers
def max_over_ranks(x, dev=None):
    """The largest x over the ranks of the process group (NCCL: on the
    rank's GPU; gloo: on the CPU)."""
    import torch
    device = f"cuda:{dev}" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(children_per_rank, local_ms, world, dev=None):
    """Whole-job throughput of `world` replicas that each processed
    children_per_rank in local_ms: the children of all ranks over the
    slowest rank's time.  Returns (children/s, that time in ms)."""
    total_ms = max_over_ranks(local_ms, dev) if world > 1 else float(local_ms)
    return world * children_per_rank / (total_ms / 1e3), total_ms


def barrier(world):
    if world > 1:
        import torch
        torch.distributed.barrier()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def run_step_gpu(ctx, quids, wl, init_state, stats_acc=None, flags=0, spare=None):
    """One bench step on device-resident input, through quids_gpu_run (the
    gate list in one library call): returns (children, final it_t).  With the
    same two handles every step (init_state re-uploaded, `spare`), repeated
    steps are planned runs replayed as a CUDA graph."""
    if "_ops" not in wl:
        wl["_ops"] = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in wl["gates"]]
    if spare is None:
        if "_spare" not in wl:
            wl["_spare"] = quids.it_t(ctx)
        spare = wl["_spare"]
    in_bytes = init_state.num_bytes
    final, stats = quids.run(init_state, spare, wl["_ops"], wl["max"], flags)
    if final is spare and spare is wl.get("_spare"):  # keep a free handle for the next step
        wl["_spare"] = init_state
    children = 0
    for st in stats:
        st["_in_bytes"] = in_bytes
        in_bytes = st["out_bytes"]
        children += st["num_object"]
    if stats_acc is not None:
        stats_acc.extend(stats)
    return children, final


# per-stage algorithmic bytes (compulsory HBM traffic of each stage's kernels)
def stage_bytes(st, fused=False):
    NP, NC, NU, NS = st["num_parents_kept"], st["num_object"], st["num_object_after_interferences"], st["num_object_out"]
    sp = st.get("_in_bytes", 0)
    sbar_p = sp / NP if NP else 0
    sbar_c = st["out_bytes"] / NS if NS else 0
    M = st["table_capacity"]
    out_layout = 56.0 * NS  # gathered magnitude and size, written magnitude, size, offset, child index
    trunc = NU > NS
    base = {
        0: 12.0 * st["num_parents"] + 8.0 * NP + sp,                   # num_child: sizes/begins/bytes, offsets
        1: sp + 36.0 * NP + 28.0 * NC,                                  # symbolic: parents in, 28 B/child out
        5: 16.0 * NS,                                                   # exact total: survivor magnitudes
        6: NS * (sbar_p + sbar_c + 48.0),                               # populate + normalise magnitudes
        7: 0.0,
    }
    if M == 0 and NC:
        # partitioned stage (stages 2-4 in one): each child's hash and
        # magnitude read once, each group's record (key, representative,
        # magnitude) written and read once, the survivors laid out
        base.update({2: 24.0 * NC + 56.0 * NU + out_layout, 3: 0.0, 4: 0.0})
        return base
    if fused:
        # the grouped symbolic pass clears the table and claims the slots
        # (slot out per child; the hash stays in registers); stage 2 is the
        # accumulate: each child's slot, the joiners' magnitudes
        base[1] += 8.0 * M + 4.0 * NC
        base.update({
            2: 20.0 * NC,
            3: 8.0 * NC + 32.0 * NU + (40.0 * NU if trunc else out_layout),
            4: (8.0 * NU + 40.0 * NU + out_layout) if trunc else 0.0,
        })
        return base
    # collision table: insert (24 in, 4 out); per child slot + rep, per rep its sum
    base.update({
        2: 8.0 * M + 28.0 * NC,
        3: 8.0 * NC + 32.0 * NU + (40.0 * NU if trunc else out_layout),
        4: (8.0 * NU + 40.0 * NU + out_layout) if trunc else 0.0,       # select (first pass), keep + layout
    })
    return base


def ours(args, rank, world):
    import torch
    import quids_gb300 as quids
    from quids_gb300 import capi

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = workload(args.config)
    quids.tolerance, quids.align_byte_length = wl["tolerance"], wl["align"]
    ctx = quids.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=f"cuda:{dev}")
    xflags = capi.FLAG_PARTITION if args.collisions == "partition" else 0

    init_packed = wl["init"]
    if init_packed is None:  # QCGD: the state after step 0, computed on the GPU
        from quids_gb300 import workloads as W
        it = quids.it_t(ctx, W.qcgd_single_state(wl["nodes"], seed=wl["seed"]))
        for _ in range(wl.get("pre_steps", 1)):
            _, it = run_step_gpu(ctx, quids, wl, it)
        init_packed = it.download()
        del it
        wl.pop("_spare", None)
    # the two handles of every step: the input is uploaded into `src` before
    # each step (outside the timed region), `spare` takes the ping-pong
    src, spare = quids.it_t(ctx), quids.it_t(ctx)

    # warm-up (the first run records the steps' sizes, the next ones are
    # planned runs, captured as a CUDA graph from the third on)
    for _ in range(args.warmup):
        src.upload(init_packed)
        run_step_gpu(ctx, quids, wl, src, spare=spare, flags=capi.FLAG_AUTOTUNE | xflags)
    ctx.synchronize()

    # timed: device-resident input, L2 flushed before each step (outside the events)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ctx.synchronize()
    launches0 = ctx.lib.quids_gpu_ctx_launch_count(ctx.h)
    runs0 = ctx.run_counts()
    ms = []
    children = 0
    stats = []
    t_wall0 = time.perf_counter()
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            src.upload(init_packed)
            with torch.cuda.stream(stream):
                flush.fill_(1)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            torch.cuda.nvtx.range_push("timed_step")  # lets ncu --nvtx-include select the timed launches
            c, _ = run_step_gpu(ctx, quids, wl, src, spare=spare, flags=capi.FLAG_AUTOTUNE | xflags)
            torch.cuda.nvtx.range_pop()
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            children += c
    ctx.synchronize()
    barrier(world)
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.lib.quids_gpu_ctx_launch_count(ctx.h) - launches0
    runs = {k: v - runs0[k] for k, v in ctx.run_counts().items()}

    # stage timing: the same steps again with CUDA events around every stage
    # of every rule application (live, on the library's stream)
    for _ in range(args.steps):
        src.upload(init_packed)
        with torch.cuda.stream(stream):
            flush.fill_(1)
        run_step_gpu(ctx, quids, wl, src, stats, flags=capi.FLAG_STAGE_TIMING | xflags, spare=spare)
    ctx.synchronize()
    value, total_ms = job_value(children, sum(ms), world, dev)

    # dominant stage and its roofline (stage times are CUDA events on the library's stream);
    # the QCGD rules' grouped symbolic pass claims the collision-table slots itself
    fused = wl["name"].startswith("qcgd") and args.collisions == "table"
    stage_t = [0.0] * 8
    stage_b = [0.0] * 8
    for st in stats:
        sb = stage_bytes(st, fused)
        for k in range(8):
            stage_t[k] += st["stage_ms"][k]
            stage_b[k] += sb[k]
    dom = max(range(8), key=lambda k: stage_t[k])
    names = ["num_child+offsets", "symbolic+table_claim" if fused else "symbolic",
             "collision_accumulate" if fused else "collisions", "group_compaction+layout",
             "truncation+layout", "total_proba", "finalize_populate+normalize", "unused"]
    peak, peak_kind = peaks()
    achieved = stage_b[dom] / (stage_t[dom] / 1e3) / 1e9 if stage_t[dom] > 0 else 0.0
    step_bytes = sum(st["algorithmic_bytes"] for st in stats)
    # per launch of the dominant stage (one per rule application)
    n_apps = max(1, len(stats) // args.steps)
    alg_per_launch = stage_b[dom] / args.steps / n_apps
    rec = RECORDED_TRAFFIC.get((wl["name"], names[dom], args.collisions))
    traffic = rec["bytes_per_launch"] if rec else None

    # e2e through the public API with host buffers (pinned), copies inside the timed region
    e2e = None
    if rank == 0 or world > 1:
        objects, begin, size, mag = init_packed
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        h_in = tuple(pin(a) for a in (objects, begin, size, mag))
        h2d = sum(a.nbytes for a in h_in)
        final_n = stats[-1]["num_object_out"]
        final_b = stats[-1]["out_bytes"]
        h_out = (torch.empty(max(final_b, 1), dtype=torch.uint8).pin_memory(),
                 torch.empty(final_n + 1, dtype=torch.int64).pin_memory(),
                 torch.empty(max(final_n, 1), dtype=torch.int32).pin_memory(),
                 torch.empty(max(final_n, 1), dtype=torch.complex128).pin_memory())
        d2h = final_b + 8 * (final_n + 1) + 4 * final_n + 16 * final_n
        # two state pairs: each step's result downloads asynchronously (the
        # context's copy stream) while the next step runs on the other pair;
        # the second pair is planned and captured before the timed region
        src2, spare2 = quids.it_t(ctx), quids.it_t(ctx)
        for _ in range(3):
            src2.upload(h_in)
            run_step_gpu(ctx, quids, wl, src2, spare=spare2, flags=capi.FLAG_AUTOTUNE | xflags)
        pairs = [(src, spare), (src2, spare2)]
        h_outs = [h_out, tuple(torch.empty_like(t).pin_memory() for t in h_out)]
        pending = [None, None]
        ctx.synchronize()
        t0 = time.perf_counter()
        e2e_children = 0
        for i in range(args.steps):
            k = i % 2
            if pending[k] is not None:  # its host buffers are written again
                pending[k].download_wait()
            s_in, s_spare = pairs[k]
            s_in.upload(h_in)
            c, out = run_step_gpu(ctx, quids, wl, s_in, spare=s_spare, flags=capi.FLAG_AUTOTUNE | xflags)
            e2e_children += c
            out.download_async(*h_outs[k])
            pending[k] = out
        for out in pending:
            if out is not None:
                out.download_wait()
        ctx.synchronize()
        t_e2e = time.perf_counter() - t0
        e2e = {"value": e2e_children / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * t_e2e / args.steps,
               "copies": "every step uploads its input and downloads its whole result inside the timed "
                         "region; a step's download overlaps the next step (two state pairs, "
                         "quids_gpu_state_download_async)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, cpu_sample(wl, init_packed), samples=1, warm=wl["name"] == "circuit24")
        # the same work?  Both start from the same input; a truncation with
        # exact ties can send the two along different states afterwards
        cpu["gpu_children_per_step"] = children // args.steps
        cpu["same_trajectory"] = (cpu["children_per_step"] == children // args.steps
                                  and not wl.get("cpu_sample_objects"))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators; the reference publishes no dataset)",
            "config": dict(wl["config"], parallelism=f"replicas x{world}",
                           l2="flushed before every step (256 MiB write)",
                           children_per_step=children // args.steps, collisions=args.collisions,
                           runs_timed=runs, autotuned=ctx.last_tuning()),
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "achieved_source": "stage-timing pass: the timed steps run again synchronously with "
                                            "CUDA events around each stage on the library's stream; "
                                            "algorithmic bytes of the stage / its event time",
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg_per_launch,
                         "traffic_source": (f"recorded, not measured in this run: {rec['source']}" if rec
                                            else "not measured in this run"),
                         "stage_ms_per_step": [t / args.steps for t in stage_t],
                         "stage_share_of_timed_step": [t / args.steps / (total_ms / args.steps) for t in stage_t],
                         "step_algorithmic_GBps": step_bytes / (total_ms / 1e3) / 1e9,
                         "step_frac": step_bytes / (total_ms / 1e3) / 1e9 / peak},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
    ctx.close()
    del flush
    if rank == 0 and world == 1 and args.extras:
        line.update(extra_ratios(args, rank, world))
    if rank == 0:
        print(json.dumps(line), flush=True)


def extra_ratios(args, rank, world):
    """Two ratios on the same GPU, beside the default line: the batched form
    against the plain path instance by instance (batch256),
    and the adjoint's forward + backward against the plain forward
    (adjoint10).  Fewer steps than the main line (each is a full workload)."""
    import torch
    out = {}
    torch.cuda.empty_cache()
    b = ours_batched(argparse.Namespace(**dict(vars(args), config="batch256", steps=min(args.steps, 5),
                                               warmup=max(3, min(args.warmup, 3)))), rank, world, emit=False)
    pl = b["plain_instance_by_instance"]
    out["batched_vs_plain"] = {
        "workload": b["config"]["workload"], "unit": UNIT, "batched": b["value"], "batched_ms_per_step": b["ms_per_step"],
        "plain_instance_by_instance": pl["value"], "plain_ms_per_step": pl["ms_per_step"],
        "ratio": b["value"] / pl["value"], "steps": b["steps"], "clocks": b["clocks"]}
    torch.cuda.empty_cache()
    a = ours_adjoint(argparse.Namespace(**dict(vars(args), config="adjoint10", steps=1, warmup=1)), rank, world,
                     emit=False)
    out["adjoint_vs_forward"] = {
        "workload": a["config"]["workload"], "forward_plus_backward_ms": a["ms_per_step"],
        "plain_forward_ms": a["adjoint"]["plain_forward_ms"],
        "ratio": a["adjoint"]["forward_plus_backward_over_forward"], "loss": a["adjoint"]["loss"],
        "grad": a["adjoint"]["grad"], "steps": a["steps"], "clocks": a["clocks"]}
    return out


def batch_ops(quids, wl):
    from quids_gb300 import workloads as W
    insts = wl["insts"]
    return [quids.rules.step, quids.rule_from(True, W.RULE_QCGD_COIN, W.COIN_DEFAULT),
            [quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm) for _, sm, _ in insts],
            [quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec) for _, _, ec in insts]]


def instance_ops(quids, sm, ec):
    from quids_gb300 import workloads as W
    return [quids.rules.step, quids.rule_from(True, W.RULE_QCGD_COIN, W.COIN_DEFAULT),
            quids.rule_from(True, W.RULE_QCGD_SPLIT_MERGE, sm), quids.rule_from(True, W.RULE_QCGD_ERASE_CREATE, ec)]


def ours_batched(args, rank, world, emit=True):
    """The batched form: one QCGD step of 256 instances per bench step.
    emit=False: no end-to-end or CPU legs, the line is returned, not printed
    (the batched-vs-plain ratio of the default line)."""
    import torch
    import quids_gb300 as quids
    from quids_gb300 import capi, workloads as W

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = workload(args.config)
    quids.tolerance, quids.align_byte_length = wl["tolerance"], wl["align"]
    ctx = quids.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=f"cuda:{dev}")
    packed = [W.pack([g], [1.0 + 0j], 8) for g, _, _ in wl["insts"]]
    ops = batch_ops(quids, wl)
    # the same two handles every step: the instances are uploaded into `src`
    # before each step (outside the timed region); repeated steps are planned
    # runs, replayed as a CUDA graph from the third on
    src, spare = quids.it_t(ctx), quids.it_t(ctx)

    def step(a):
        fin, st = quids.run_batched(a, spare, ops, wl["max"], capi.FLAG_AUTOTUNE)
        return sum(x["num_object"] for x in st), sum(x["algorithmic_bytes"] for x in st), fin

    def fresh():
        src.upload_batched(packed)
        return src

    for _ in range(args.warmup):
        step(fresh())
    ctx.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.lib.quids_gpu_ctx_launch_count(ctx.h)
    runs0 = ctx.run_counts()
    ms, children, abytes = [], 0, 0.0
    t_wall0 = time.perf_counter()
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            src = fresh()
            with torch.cuda.stream(stream):
                flush.fill_(1)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            torch.cuda.nvtx.range_push("timed_step")
            c, b, _ = step(src)
            torch.cuda.nvtx.range_pop()
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            children += c
            abytes += b
    ctx.synchronize()
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.lib.quids_gpu_ctx_launch_count(ctx.h) - launches0
    runs = {k: v - runs0[k] for k, v in ctx.run_counts().items()}
    barrier(world)
    value, total_ms = job_value(children, sum(ms), world, dev)

    # the same step, instance by instance through the plain path (a fresh
    # pair of states per instance, as the reference's loop over instances
    # would: the synchronous steps)
    plain_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        pc = 0
        for (g, sm, ec), p in zip(wl["insts"], packed):
            fin, st = quids.run(quids.it_t(ctx, p), quids.it_t(ctx), instance_ops(quids, sm, ec), wl["max"])
            pc += sum(x["num_object"] for x in st)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    plain_value = pc / (statistics.mean(plain_ms) / 1e3)

    # e2e: host instances in, each instance's object count and total
    # probability out (the full final state is 7.9 GB), copies inside the
    # timed region
    e2e = None
    if emit and (rank == 0 or world > 1):
        ctx.synchronize()
        t0 = time.perf_counter()
        e2e_children, h2d, d2h = 0, 0, 0
        for _ in range(args.steps):
            src = fresh()
            h2d = sum(sum(a.nbytes for a in p) for p in packed)
            c, _, out = step(src)
            e2e_children += c
            ib, tot = out.instances()
            d2h = ib.nbytes + tot.nbytes
        ctx.synchronize()
        t_e2e = time.perf_counter() - t0
        e2e = {"value": e2e_children / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * t_e2e / args.steps}

    peak, peak_kind = peaks()
    achieved = abytes / (total_ms / 1e3) / 1e9
    cpu = None
    if emit and rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_batched(wl, packed)
    tuning = ctx.last_tuning()
    ctx.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators; the reference publishes no dataset)",
            "config": dict(wl["config"], parallelism=f"replicas x{world}",
                           l2="flushed before every step (256 MiB write)",
                           children_per_step=children // args.steps,
                           runs_timed=runs, autotuned=tuning),
            "plain_instance_by_instance": {"value": plain_value, "unit": UNIT,
                                           "ms_per_step": statistics.mean(plain_ms),
                                           "batched_over_plain": value / plain_value},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "whole batched step (all kernels)", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": None},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
        if emit:
            print(json.dumps(line), flush=True)
        return line


def ours_adjoint(args, rank, world, emit=True):
    """The adjoint: taped forward + simulate_backward per bench step.
    emit=False: no end-to-end leg, the line is returned, not printed (the
    adjoint-vs-forward ratio of the default line)."""
    import torch
    import quids_gb300 as quids
    from quids_gb300 import workloads as W

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = workload(args.config)
    quids.tolerance, quids.align_byte_length = wl["tolerance"], wl["align"]
    ctx = quids.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=f"cuda:{dev}")
    gates, slots = W.qcgd_adjoint_ops(wl["angles"], wl["T"])
    ops = [quids.rule_from(g.kind == "rule", g.code, g.params) for g in gates]
    tape = quids.Tape(ctx)

    def step():
        final, st = tape.forward(quids.it_t(ctx, wl["init"]), ops, wl["max"], wl["every"])
        loss, g = tape.backward_observable(quids.OBS_QCGD_NUM_NODES)
        grad = [0.0] * 6
        for oi, comp, ai in slots:
            grad[ai] += float(g[oi, comp])
        return sum(x["num_object"] for x in st), sum(x["algorithmic_bytes"] for x in st), loss, grad

    def timed(fn):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        r = fn()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), r

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    torch.cuda.synchronize()
    launches0 = ctx.lib.quids_gpu_ctx_launch_count(ctx.h)
    ms, children, abytes = [], 0, 0.0
    t_wall0 = time.perf_counter()
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            t, (c, b, loss, grad) = timed(step)
            ms.append(t)
            children += c
            abytes += b
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.lib.quids_gpu_ctx_launch_count(ctx.h) - launches0
    barrier(world)
    value, total_ms = job_value(children, sum(ms), world, dev)

    def plain():
        fin, st = quids.run(quids.it_t(ctx, wl["init"]), quids.it_t(ctx), ops, wl["max"])
        return sum(x["num_object"] for x in st)
    plain_ms = [timed(plain)[0] for _ in range(max(1, min(args.steps, 2)))]
    fwd_ms = statistics.mean(plain_ms)

    # e2e: initial state from pinned host memory, gradients back to the host
    objects, begin, size, mag = wl["init"]
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    h_in = tuple(pin(a) for a in (objects, begin, size, mag))
    t0 = time.perf_counter()
    e2e_children = 0
    for _ in range(args.steps if emit else 0):
        final, st = tape.forward(quids.it_t(ctx, h_in), ops, wl["max"], wl["every"])
        tape.backward_observable(quids.OBS_QCGD_NUM_NODES)
        e2e_children += sum(x["num_object"] for x in st)
    t_e2e = time.perf_counter() - t0
    peak, peak_kind = peaks()
    achieved = abytes / (total_ms / 1e3) / 1e9
    del tape
    ctx.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators; the reference publishes no dataset)",
            "config": dict(wl["config"], parallelism=f"replicas x{world}",
                           l2="flushed before every step (256 MiB write)",
                           children_per_step=children // args.steps),
            "adjoint": {"loss": loss, "grad": grad, "plain_forward_ms": fwd_ms,
                        "forward_plus_backward_over_forward": (total_ms / args.steps) / fwd_ms},
            "e2e": {"value": e2e_children / t_e2e, "unit": UNIT,
                    "h2d_bytes_per_step": int(sum(a.nbytes for a in h_in)), "d2h_bytes_per_step": 6 * 8 + 8,
                    "ms_per_step": 1e3 * t_e2e / args.steps} if emit else None,
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "whole forward (all kernels; backward not counted)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "traffic": None},
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
        if emit:
            print(json.dumps(line), flush=True)
        return line


def cpu_oracle():
    """The CPU implementation timed as the baseline: the reference compiled
    from its own headers (oracle/_ref) where it was built on this host, else
    the oracle port (the reference algorithm restated, built anywhere).
    Returns (oracle, kind) with kind "reference" or "port"."""
    from oracle.oracle import Oracle
    try:
        return Oracle("ref", autobuild=False), "reference"
    except OSError:  # not built here, or built for another architecture
        return Oracle("port"), "port"


def cpu_baseline_batched(wl, packed):
    """The CPU oracle on all host cores, instance after instance."""
    from quids_gb300 import workloads as W
    o, kind = cpu_oracle()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    o.set_globals(wl["tolerance"], True, wl["align"])
    t0 = time.perf_counter()
    ch = 0
    for (g, sm, ec), p in zip(wl["insts"], packed):
        s = o.new_state(p)
        o.modifier(s, W.MOD_QCGD_STEP, ())
        for rule_kind, prm in ((W.RULE_QCGD_COIN, W.COIN_DEFAULT), (W.RULE_QCGD_SPLIT_MERGE, sm),
                               (W.RULE_QCGD_ERASE_CREATE, ec)):
            t = o.new_state()
            ch += o.simulate(s, rule_kind, prm, t, wl["max"])[0]
            s = t
    dt = time.perf_counter() - t0
    return {"value": ch / dt, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"the first step of all {len(packed)} instances, one after another ({ch} children, "
                      f"{dt:.2f} s)"}


def cpu_baseline(wl, init_packed, samples=1, warm=True):
    """The CPU oracle (cpu_oracle) on all host cores."""
    o, kind = cpu_oracle()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    o.set_globals(wl["tolerance"], True, wl["align"])

    def one():
        s = o.new_state(init_packed)
        ch = 0
        for g in wl["gates"]:
            if g.kind == "mod":
                o.modifier(s, g.code, g.params)
            else:
                t = o.new_state()
                ch += o.simulate(s, g.code, g.params, t, wl["max"])[0]
                s = t
        return ch

    if warm:
        one()  # warm-up (skipped for the long QCGD steps)
    t0 = time.perf_counter()
    ch = sum(one() for _ in range(samples))
    dt = time.perf_counter() - t0
    part = (f"the first {wl['cpu_sample_objects']} objects of " if wl.get("cpu_sample_objects") else "")
    return {"value": ch / dt, "unit": UNIT, "cores": cores, "kind": kind, "children_per_step": ch // samples,
            "sample": f"{samples} step(s) of {part}the {wl['name']} workload from the GPU arm's input "
                      f"({ch} children, {dt:.2f} s)"}


def reference(args, rank, world):
    if rank != 0:
        return
    wl = workload(args.config)
    if wl["name"] == "batch256":  # the reference steps one state per call: instances one by one
        from quids_gb300 import workloads as W
        packed = [W.pack([g], [1.0 + 0j], 8) for g, _, _ in wl["insts"]]
        for _ in range(args.warmup):
            cpu_baseline_batched(wl, packed)
        vals = [cpu_baseline_batched(wl, packed) for _ in range(args.steps)]
        v = statistics.mean(x["value"] for x in vals)
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(wl["config"], parallelism="host cores, instances one after another"),
            "cpu_baseline": dict(vals[-1], value=v),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    o, kind = cpu_oracle()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    o.set_globals(wl["tolerance"], True, wl["align"])
    if wl["name"] == "adjoint10":  # no adjoint in the reference: its forward, first 2 of the 20 steps
        from quids_gb300 import workloads as W
        wl["gates"] = W.qcgd_adjoint_ops(wl["angles"], 2)[0]
        wl["config"] = dict(wl["config"], sample="reference forward only, first 2 of the 20 steps")
    if wl.get("ref_sample_objects"):  # a bounded sample of each step (children/s is per child)
        wl["cpu_sample_objects"] = wl["ref_sample_objects"]
    init_packed = wl["init"] if wl["init"] is not None else qcgd_initial_cpu(wl, o)

    def one():
        s = o.new_state(init_packed)
        ch = 0
        for g in wl["gates"]:
            if g.kind == "mod":
                o.modifier(s, g.code, g.params)
            else:
                t = o.new_state()
                ch += o.simulate(s, g.code, g.params, t, wl["max"])[0]
                s = t
        return ch

    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    ch = sum(one() for _ in range(args.steps))
    dt = time.perf_counter() - t0
    v = ch / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(wl["config"], parallelism="host cores"),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{args.steps} step(s) of "
                                   + (f"the first {wl['cpu_sample_objects']} objects of "
                                      if wl.get("cpu_sample_objects") else "")
                                   + wl["name"]},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="qcgd12", choices=["circuit24", "qcgd12", "qcgd10", "qcgd12s2", "batch256",
                                                              "adjoint10"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--collisions", default="table", choices=["table", "partition"],
                    help="collision elimination of the plain steps: the open-addressing table (default) or the "
                         "partitioned stage (QUIDS_FLAG_PARTITION)")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="qcgd12 line without the batched-vs-plain and adjoint-vs-forward ratios")
    args = ap.parse_args()
    if args.config != "qcgd12":
        args.extras = False
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    try:
        if args.impl == "reference":
            reference(args, rank, world)
        elif args.config == "batch256":
            ours_batched(args, rank, world)
        elif args.config == "adjoint10":
            ours_adjoint(args, rank, world)
        else:
            ours(args, rank, world)
    finally:
        if world > 1 and args.impl == "ours":
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
