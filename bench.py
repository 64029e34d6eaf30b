"""Benchmark of the batched MBQC statevector sweep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): one batched statevector sweep of mentpy's
``many_wires([8]*4)`` cluster (32 qubits, window 5, 28 trainable angles) over
4096 (angle vector, Haar-random 4-qubit input) pairs, complex64 amplitudes,
outputs in the reference's order with its global phase.  Synthetic seeded
inputs with the shapes of the configuration.

``value``  runs/s with inputs resident in HBM: K back-to-back steps on one
           stream, step i reading input set i of 128 distinct sets (184 MB,
           more than L2) after one 256 MiB L2 flush.  The sets are written
           before the timed region, so the steps declare their inputs ready
           (``inputs_ready=True``): a launch sweeps while the previous one
           finishes and waits for it only before writing.  ``ordered`` is the
           same without the declaration; ``isolated_step`` is one step alone
           with a flush before it (carries the event/launch floor).
``e2e``    runs/s through the drop-in simulator's batched call with host
           buffers: every step ``PatternSimulator(circuit,
           backend="cuda-sv").run_batch(angles, inputs, out=, status=,
           inputs_ready=True)`` reads that step's angles and inputs from pinned
           host memory and writes the output states there (host-filled
           buffers, bound on the first call; the kernel's uncached loads and
           its stores cross the CPU-GPU link; no staging copy).  Four batches
           are in flight, each on its own stream with its own host buffer set.
           Timed over max(K, 200) calls (a serving loop's steady state);
           ``e2e.k_steps`` is the same loop over K calls.
           ``e2e.prepared`` is the same through ``StatevectorSweep.prepare``,
           ``e2e.serial`` keeps one in flight; ``e2e.staged`` moves the same
           bytes with the copy engines instead (host->device copies, sweep,
           device->host copy in one graph per batch, four batches in flight).
Under torchrun every rank runs its own 4096-run batch (weak scaling, no
collective on the data path); time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BATCH = 4096
WIRES, COLS = 4, 8
SEED = 20261203
METRIC = "batched MBQC statevector runs/s (many_wires 4x8, w=5, complex64)"
UNIT = "runs/s"
E2E_RING = 4  # host buffer sets of the end-to-end loop
E2E_STREAMS = 4  # batches in flight in the end-to-end loop (each on its own stream)
E2E_STEADY = 200  # end-to-end calls timed at least (a serving loop's steady state; K-step figure kept beside)
VALUE_STREAMS = 4  # batches in flight in the concurrent device-resident figure
VALUE_SETS = 128  # device input sets of the timed loop (184 MB > L2)


def workload_config(world):
    """The workload both arms time (identical dict in both JSON lines)."""
    return {"workload": "many_wires([8]*4) statevector sweep, window 5, 28 angles",
            "batch_per_gpu": BATCH, "global_batch": world * BATCH,
            "l2": "inputs larger than L2 between timed steps",
            "parallelism": f"replicas x{world} (independent batches)"}


def workload_arrays(batch=BATCH, seed=SEED):
    from mentpy_gb300 import circuit as C

    circ = C.many_wires([COLS] * WIRES)
    rng = np.random.default_rng(seed)
    A = len(circ.trainable_nodes)
    angles = rng.uniform(0, 2 * np.pi, size=(batch, A))
    d = 2 ** len(circ.input_nodes)
    z = (rng.standard_normal((batch, d, d)) + 1j * rng.standard_normal((batch, d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    diag = np.diagonal(r, axis1=1, axis2=2)
    inputs = np.ascontiguousarray((q * (diag / np.abs(diag))[:, None, :])[:, :, 0])
    return circ, angles, inputs


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    n_runs, seed, budget_s = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle.dense import DenseSV

    circ, angles, inputs = workload_arrays(batch=max(n_runs, 1), seed=seed)
    sim = DenseSV(circ)
    t0 = time.perf_counter()
    done = 0
    for r in range(n_runs):
        sim.run(angles[r], inputs[r])
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return done, time.perf_counter() - t0


def cpu_baseline(budget_s=12.0, runs_per_proc=4000):
    """The reference algorithm (dense-operator port of the numpy statevector
    simulator, oracle/dense.py) on every host core: one spawned process per
    core, each running its own runs for at most ``budget_s`` seconds."""
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(runs_per_proc, SEED + i, budget_s) for i in range(cores)])
    runs = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return {
        "value": runs / wall,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": f"{runs} runs of the workload ({cores} processes x <= {budget_s:.0f} s), "
                  "dense 2^w x 2^w operators as in np_simulator_sv.py",
    }


# ------------------------------------------------------------ profile figures
def profile_traffic(key):
    """DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) recorded for
    ``key`` in a profiles/*.md summary, on a line of the form
    ``traffic[<key>] = <bytes> bytes ...`` next to the ncu command that
    measured it; None when no summary records it."""
    import glob
    import re

    pat = re.compile(r"^traffic\[" + re.escape(key) + r"\] = (\d+) bytes")
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for line in open(f):
            m = pat.match(line.strip())
            if m:
                return int(m.group(1))
    return None


# ------------------------------------------------------------ oracle checks
# Every benchmarked result is checked against the complex128 oracle outside
# the timed regions: the GPU outputs of the timed batches are handed to a
# spawned process pool (one process per host core), which recomputes them
# with oracle/sweep.py and returns the error figures stated in the line.

def _circuit(spec):
    from mentpy_gb300 import circuit as C

    kind, *a = spec
    if kind == "many_wires":
        return C.many_wires([a[1]] * a[0])
    if kind == "grid":
        return C.grid_cluster(a[0], a[1])
    raise ValueError(spec)


def _oracle_task(task):
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import gradients as G
    from oracle import sweep as O

    kind = task[0]
    if kind == "sv":  # (spec, angles, inputs, gpu states, gpu logprob or None)
        _, spec, ang, inp, got, lp = task
        ref, probs = O.run_sv_batch(_circuit(spec), ang, inp)
        got = np.asarray(got, dtype=np.complex128)
        a = got / np.linalg.norm(got, axis=1, keepdims=True)
        infid = 1.0 - np.abs(np.sum(ref.conj() * a, axis=1)) ** 2
        r = {"n": len(ang), "max_infidelity": float(infid.max()), "max_abs_amp_err": float(np.abs(got - ref).max())}
        if lp is not None:
            r["max_logprob_err"] = float(np.abs(lp - np.log(probs).sum(axis=1)).max())
        return r
    if kind == "loss":  # (spec, angle rows, inputs, targets, gpu losses)
        _, spec, ang, inp, tg, got = task
        ref = G.fidelity_losses(_circuit(spec), ang, inp, tg)
        return {"n": len(ang), "max_loss_err": float(np.abs(got - ref).max())}
    if kind == "fd":  # (spec, angles, angle indices, inputs, targets, h, gpu gradient entries)
        _, spec, x, idx, inp, tg, h, got = task
        circ = _circuit(spec)
        rows = np.repeat(np.asarray(x)[None], 2 * len(idx), axis=0)
        rows[np.arange(len(idx)), idx] += h
        rows[len(idx) + np.arange(len(idx)), idx] -= h
        f = G.fidelity_losses(circ, rows, inp, tg)
        ref = (f[: len(idx)] - f[len(idx):]) / (2 * h)
        return {"n": len(idx), "max_grad_err": float(np.abs(got - ref).max()), "max_abs_grad": float(np.abs(ref).max())}
    if kind == "dir":  # (spec, angles, gout, direction, h, gpu grad . direction, max |gpu grad|)
        _, spec, x, gout, d, h, got, gmax = task
        circ = _circuit(spec)
        f = lambda a: float(np.real(np.vdot(gout, G.canonical_sv(circ, a, None))))  # noqa: E731
        ref = (f(x + h * d) - f(x - h * d)) / (2 * h)
        return {"n": 1, "max_dir_grad_err": abs(got - ref), "max_abs_grad": gmax}
    if kind == "dm":  # (spec, angles, inputs, noise, gpu rho, gpu outcomes)
        _, spec, ang, inp, noise, rho, outc = task
        ref, ref_out, _ = O.run_dm_batch(_circuit(spec), ang, inp, noise_p=noise)
        return {"n": len(ang), "max_rho_err": float(np.abs(rho - ref).max()),
                "outcome_mismatches": int((outc != ref_out).any(axis=1).sum()),
                "outcomes_checked": int(outc.size)}
    raise ValueError(kind)


def _merge(results):
    """Combine the per-task error figures of one workload (max of the
    maxima, sums of the counts)."""
    out = {}
    for r in results:
        for k, v in r.items():
            if k in ("n", "outcome_mismatches", "outcomes_checked"):
                out[k] = out.get(k, 0) + v
            else:
                out[k] = max(out.get(k, 0.0), v)
    return out


def run_oracle_checks(tasks):
    """tasks: {workload: [task, ...]} -> {workload: merged error figures}."""
    flat = [(w, t) for w, ts in tasks.items() for t in ts]
    if not flat:
        return {}
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(os.cpu_count() or 1, len(flat))) as pool:
        res = pool.map(_oracle_task, [t for _, t in flat], chunksize=1)
    by = {}
    for (w, _), r in zip(flat, res):
        by.setdefault(w, []).append(r)
    return {w: _merge(rs) for w, rs in by.items()}


# ------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ GPU arm
def run_ours(args, rank, world, local_rank):
    import torch

    from mentpy_gb300 import _native
    from mentpy_gb300.replicas import reduce_max
    from mentpy_gb300.sweep import StatevectorSweep, gpu_hold

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    circ, angles, inputs = workload_arrays(seed=SEED + rank)
    sw = StatevectorSweep(circ, device=dev)
    plan = sw.plan
    B, A = angles.shape
    d_in, d_out = inputs.shape[1], 2 ** sw.n_out
    ang_d = torch.as_tensor(angles, device=dev)
    inp_d = torch.as_tensor(inputs.astype(np.complex64), device=dev)
    out_d = torch.empty((B, d_out), dtype=torch.complex64, device=dev)
    st_d = torch.empty((B,), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    # measured FP32 peak of this GPU (roofline denominator)
    import ctypes

    sink = torch.zeros(1, dtype=torch.float32, device=dev)
    tf = ctypes.c_double()
    _native.check(_native.lib().mbqc_probe_fp32_fma(20000, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(tf),
                                                    ctypes.c_void_p(stream.cuda_stream)))
    fp32_peak = tf.value

    # lanes per run of the register kernel: chosen below for the device-resident
    # steps by timing each variant on those steps, and separately for the
    # host-buffer (e2e) path; every number is re-measured after the choice
    head_v = sw.tune(ang_d, inp_d)

    def step():
        sw.forward(ang_d, inp_d, out=out_d, status=st_d, variant=head_v)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    assert int((st_d != 0).sum()) == 0, "kernel reported failed runs"

    # inputs larger than L2: VALUE_SETS distinct (angles, inputs, outputs) sets
    # of the workload, 1.44 MB in + 0.5 MB out each, read in turn by the
    # back-to-back timed steps after one L2 flush, so no step finds its inputs
    # on chip
    n_sets = VALUE_SETS
    ang_sets = torch.empty((n_sets, B, A), dtype=torch.float64, device=dev)
    ang_sets.copy_(ang_d.expand(n_sets, B, A))
    inp_sets = torch.empty((n_sets, B, d_in), dtype=torch.complex64, device=dev)
    inp_sets.copy_(inp_d.expand(n_sets, B, d_in))
    out_sets = torch.empty((n_sets, B, d_out), dtype=torch.complex64, device=dev)

    def set_step(i, ready=True, v=None):
        # every input set is written before the timed region, so the steps
        # may declare their inputs ready (MBQC_F_INPUTS_READY): a launch reads
        # them and sweeps while the previous one finishes, and waits for it
        # only before writing
        j = i % n_sets
        sw.forward(ang_sets[j], inp_sets[j], out=out_sets[j], status=st_d, inputs_ready=ready,
                   variant=head_v if v is None else v)

    # variant choice for the back-to-back steps: each variant timed on the same
    # loop the headline runs (untimed here; the headline below is a new run)
    head_tuning = {}
    for v in sw.variants():
        head_v = v
        for i in range(4):
            set_step(i)
        torch.cuda.synchronize()
        flush.fill_(-3.0)
        gpu_hold(1000.0 + 150.0 * args.steps)
        t0_, t1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0_.record(stream)
        for i in range(args.steps):
            set_step(i)
        t1_.record(stream)
        torch.cuda.synchronize()
        head_tuning[v] = t0_.elapsed_time(t1_) / args.steps
    head_v = min(head_tuning, key=head_tuning.get) if head_tuning else -1
    # and for launches that each wait for the previous one (the ordered and
    # isolated figures: latency rather than overlap)
    ord_tuning = {}
    for v in sw.variants():
        for i in range(4):
            set_step(i, ready=False, v=v)
        torch.cuda.synchronize()
        flush.fill_(-4.0)
        gpu_hold(1000.0 + 150.0 * args.steps)
        t0_, t1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0_.record(stream)
        for i in range(args.steps):
            set_step(i, ready=False, v=v)
        t1_.record(stream)
        torch.cuda.synchronize()
        ord_tuning[v] = t0_.elapsed_time(t1_) / args.steps
    ord_v = min(ord_tuning, key=ord_tuning.get) if ord_tuning else -1
    out_iso = torch.empty_like(out_d)

    def step_iso():
        sw.forward(ang_d, inp_d, out=out_iso, status=st_d, variant=ord_v)

    for _ in range(3):
        step()
        step_iso()
    torch.cuda.synchronize()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clk:
        # untimed soak so the clock samples see the GPU under this load
        t_end = time.perf_counter() + 1.0
        while time.perf_counter() < t_end:
            for _ in range(50):
                flush.fill_(0.0)
                step()
            torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        # queue every timed step behind a GPU hold so that the event intervals
        # measure device time, not host submission gaps
        gpu_hold(1000.0 + 150.0 * args.steps)
        for i in range(args.steps):
            flush.fill_(float(i))
            evs[i][0].record(stream)
            step_iso()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        # back-to-back steps over the input sets (the headline): one flush,
        # then the K launches queued behind a GPU hold run without host gaps
        flush.fill_(-1.0)
        torch.cuda.synchronize()
        barrier()
        gpu_hold(1000.0 + 150.0 * args.steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            set_step(i)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        # the same K steps without the declaration: each launch reads its
        # inputs only after the previous launch completes
        flush.fill_(-2.0)
        torch.cuda.synchronize()
        gpu_hold(1000.0 + 150.0 * args.steps)
        o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        o0.record(stream)
        for i in range(args.steps):
            set_step(i, ready=False, v=ord_v)
        o1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ordered_ms = reduce_max(o0.elapsed_time(o1) / args.steps)
    assert int((st_d != 0).sum()) == 0
    assert torch.equal(out_sets[(args.steps - 1) % n_sets], out_iso)
    # the same with VALUE_STREAMS independent batches in flight (a stream each)
    streams_v = [torch.cuda.Stream(device=dev) for _ in range(VALUE_STREAMS)]
    sts_v = [torch.zeros_like(st_d) for _ in range(VALUE_STREAMS)]

    def conc_step(i):
        j = i % n_sets
        with torch.cuda.stream(streams_v[i % VALUE_STREAMS]):
            sw.forward(ang_sets[j], inp_sets[j], out=out_sets[j], status=sts_v[i % VALUE_STREAMS], variant=head_v)

    for i in range(2 * VALUE_STREAMS):
        conc_step(i)
    flush.fill_(-2.0)
    torch.cuda.synchronize()
    barrier()
    gpu_hold(1000.0 + 150.0 * args.steps)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for s_ in streams_v:
        s_.wait_stream(stream)
    for i in range(args.steps):
        conc_step(i)
    for s_ in streams_v:
        stream.wait_stream(s_)
    c1.record(stream)
    torch.cuda.synchronize()
    conc_ms = reduce_max(c0.elapsed_time(c1) / args.steps)
    assert all(int((t != 0).sum()) == 0 for t in sts_v)
    kernel_ms = [a.elapsed_time(b) for a, b in evs]
    isolated_ms = reduce_max(float(np.mean(kernel_ms)))  # one step alone, L2 flushed before it
    ms = reduce_max(e0.elapsed_time(e1) / args.steps)  # max over ranks (timing only)

    # ---- end to end through the public API with pinned host buffers: a ring
    # of E2E_RING host buffer sets (double buffering, as a serving loop keeps
    # them), each bound once to a CUDA graph (StatevectorSweep.prepare)
    ang_h = torch.empty((E2E_RING, B, A), dtype=torch.float64).pin_memory()
    ang_h.copy_(torch.as_tensor(angles).expand(E2E_RING, B, A))
    inp_h = torch.empty((E2E_RING, B, d_in), dtype=torch.complex64).pin_memory()
    inp_h.copy_(torch.as_tensor(inputs.astype(np.complex64)).expand(E2E_RING, B, d_in))
    out_h = torch.empty((E2E_RING, B, d_out), dtype=torch.complex64).pin_memory()
    st_r = torch.zeros((E2E_RING, B), dtype=torch.int32, device=dev)
    # mapped (below): the kernel reads the angles and inputs (uncached loads, so
    # every step fetches them over the CPU-GPU link) and writes the states in place
    # staged: copy engines host -> device, sweep, device -> host, one graph per
    # set, each set with its own device buffers (so that sets run concurrently)
    ang_e = torch.empty((E2E_RING, B, A), dtype=torch.float64, device=dev)
    inp_e = torch.empty((E2E_RING, B, d_in), dtype=torch.complex64, device=dev)
    out_e = torch.empty((E2E_RING, B, d_out), dtype=torch.complex64, device=dev)
    st_e = torch.zeros((E2E_RING, B), dtype=torch.int32, device=dev)
    staged_graphs = []
    for j in range(E2E_RING):
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            sw.forward(ang_e[j], inp_e[j], out=out_e[j], status=st_e[j], variant=head_v)
        stream.wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            ang_e[j].copy_(ang_h[j], non_blocking=True)
            inp_e[j].copy_(inp_h[j], non_blocking=True)
            sw.forward(ang_e[j], inp_e[j], out=out_e[j], status=st_e[j], variant=head_v)
            out_h[j].copy_(out_e[j], non_blocking=True)
        staged_graphs.append(g)

    def time_e2e(fn, n_streams=1, steps=None):
        # step i runs on stream i % n_streams (independent batches in flight)
        steps = e2e_steps if steps is None else steps
        streams = [torch.cuda.Stream(device=dev) for _ in range(n_streams)]

        def on(i):
            fn(i, streams[i % n_streams])

        nw = max(3, E2E_RING)  # warm-up: every buffer set has been called (bound) once
        for i in range(nw):
            on(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for s in streams:
            s.wait_stream(stream)
        for i in range(steps):
            on(nw + i)
        for s in streams:
            stream.wait_stream(s)
        e1.record(stream)
        torch.cuda.synchronize()
        return reduce_max(e0.elapsed_time(e1) / steps)

    # the end-to-end loops run at least E2E_STEADY calls: over K = 20 calls
    # the first call's submission and the last batches' drain (~35 us) are a
    # fifth of the loop
    e2e_steps = max(args.steps, E2E_STEADY)

    def staged_step(i, s):
        with torch.cuda.stream(s):
            staged_graphs[i % E2E_RING].replay()

    e2e_staged_serial_ms = time_e2e(staged_step)
    e2e_staged_ms = time_e2e(staged_step, n_streams=E2E_STREAMS)
    assert all(torch.equal(out_h[j], out_d.cpu()) for j in range(E2E_RING))
    assert int((st_e != 0).sum()) == 0
    # variant choice for the host-buffer path (its loads cross the CPU-GPU
    # link, which can favour another lanes-per-run than the device steps)
    e2e_tuning = {}
    for v in sw.variants():
        pv = [sw.prepare(ang_h[j], inp_h[j], out_h[j], status=st_r[j], mapped_host=True, inputs_ready=True,
                         variant=v) for j in range(E2E_RING)]
        e2e_tuning[v] = time_e2e(lambda i, s: pv[i % E2E_RING](s), n_streams=E2E_STREAMS)
    e2e_v = min(e2e_tuning, key=e2e_tuning.get) if e2e_tuning else -1
    preps = [sw.prepare(ang_h[j], inp_h[j], out_h[j], status=st_r[j], mapped_host=True, inputs_ready=True,
                        variant=e2e_v) for j in range(E2E_RING)]
    out_h.zero_()
    e2e_serial_ms = time_e2e(lambda i, s: preps[i % E2E_RING](s))
    out_h.zero_()
    e2e_prep_ms = time_e2e(lambda i, s: preps[i % E2E_RING](s), n_streams=E2E_STREAMS)
    # the headline end-to-end figure: the drop-in simulator's batched call
    # (PatternSimulator(circuit, backend="cuda-sv").run_batch) on the same
    # pinned host buffer sets, each call returning states, outcomes and status
    from mentpy_gb300 import PatternSimulator

    psim = PatternSimulator(circ, backend="cuda-sv")
    # the serving loop's buffer sets, held as tensors (as a server keeps them)
    rb_sets = [(ang_h[j], inp_h[j], out_h[j], st_r[j]) for j in range(E2E_RING)]

    def rb_step(i, s):
        a_, p_, o_, t_ = rb_sets[i % E2E_RING]
        psim.run_batch(a_, p_, out=o_, status=t_, stream=s, inputs_ready=True, variant=e2e_v)

    out_h.zero_()
    e2e_ms = time_e2e(rb_step, n_streams=E2E_STREAMS)
    out_h.zero_()
    e2e_k_ms = time_e2e(rb_step, n_streams=E2E_STREAMS, steps=args.steps)
    # the states written to host memory are the sweep's (check against a
    # device-resident run of the same variant)
    out_v = torch.empty_like(out_d)
    sw.forward(ang_d, inp_d, out=out_v, status=st_d, variant=e2e_v)
    torch.cuda.synchronize()
    for j in range(E2E_RING):
        assert torch.equal(out_h[j], out_v.cpu())
    assert int((st_r != 0).sum()) == 0 and int((st_d != 0).sum()) == 0

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None

    # oracle check of the timed batch (every run; outside the timed regions):
    # the same call with the all-zero-branch log-probability gives the same
    # states bit for bit
    lp_d = torch.empty((B,), dtype=torch.float64, device=dev)
    out_chk, _, _ = sw.forward(ang_d, inp_d, logprob=lp_d, variant=head_v)
    assert torch.equal(out_chk, out_d)
    out_np, lp_np = out_d.cpu().numpy(), lp_d.cpu().numpy()
    inp_c64 = inputs.astype(np.complex64).astype(np.complex128)  # the inputs the kernel read
    tasks = {"headline": [("sv", ("many_wires", WIRES, COLS), angles[i:i + 256], inp_c64[i:i + 256],
                           out_np[i:i + 256], lp_np[i:i + 256]) for i in range(0, B, 256)]}

    w = plan.window
    flops_per_run = sum(12 * 2 ** min(w, plan.n_nodes - k) for k in range(plan.n_steps))
    achieved = flops_per_run * B / (ms * 1e-3) / 1e12
    traffic = profile_traffic("sv_fwd_reg_mw4x8")
    cpu = cpu_baseline()
    clocks = clk.summary()
    hbm_peak = 6765.7
    peaks_file = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_file):
        hbm_peak = float(json.load(open(peaks_file)).get("hbm_gbs", hbm_peak))
    extra = {}
    if not args.headline_only:
        for name, fn in (("adjoint_many_wires_6x12", lambda: bench_adjoint(dev, fp32_peak, flush)),
                         ("wide_window_grid_16x10", lambda: bench_wide(dev, hbm_peak, flush)),
                         ("uneven_dm_2048_circuits", lambda: bench_uneven_dm(dev, fp32_peak, flush))):
            extra[name], tasks[name] = fn()
        # the wide workload's adjoint checks are reported inside its "adjoint" object
        tasks["wide_window_grid_16x10/adjoint"] = [t for t in tasks["wide_window_grid_16x10"] if t[0] == "dir"]
        tasks["wide_window_grid_16x10"] = [t for t in tasks["wide_window_grid_16x10"] if t[0] != "dir"]
        extra["train_many_wires_6x12"] = bench_train(dev)
    t0 = time.perf_counter()
    checks = run_oracle_checks(tasks)
    check_s = time.perf_counter() - t0
    for name, r in checks.items():
        if name == "headline":
            continue
        if "/" in name:
            top, sub = name.split("/")
            extra[top][sub]["oracle_error"] = r
        else:
            extra[name]["oracle_error"] = r
    h2d = ang_h[0].numel() * 8 + inp_h[0].numel() * 8
    d2h = out_h[0].numel() * 8
    line = {
        "metric": METRIC,
        "value": world * B / (ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "complex64",
        "data": "synthetic: seeded uniform angles in [0, 2pi) and Haar-random 4-qubit inputs",
        "config": workload_config(world),
        "timing": "inputs larger than L2: 128 distinct input sets (184 MB) read in turn by back-to-back steps "
                  "after one flush",
        "e2e": {"value": world * B / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "k_steps": {"steps": args.steps, "ms_per_step": e2e_k_ms,
                            "value": world * B / (e2e_k_ms * 1e-3),
                            "note": "the same loop over the bench's K calls (pipeline fill and drain included)"},
                "path": f"PatternSimulator(circuit, backend='cuda-sv').run_batch(angles, inputs, out=, status=, "
                        f"inputs_ready=True) on pinned host buffers, {E2E_STREAMS} independent batches in flight "
                        f"on {E2E_STREAMS} streams: the kernel reads the pinned host angles/inputs with uncached "
                        f"loads (fetched over the CPU-GPU link every step) and writes the states to pinned host "
                        f"memory; {E2E_RING} host buffer sets",
                "prepared": {"value": world * B / (e2e_prep_ms * 1e-3), "ms_per_step": e2e_prep_ms,
                             "note": "the same through StatevectorSweep.prepare (one pre-bound C call per step)"},
                "streams": E2E_STREAMS,
                "lanes_per_run_log2": e2e_v,
                "variant_ms": {str(k): v for k, v in e2e_tuning.items()},
                "serial": {"value": world * B / (e2e_serial_ms * 1e-3), "ms_per_step": e2e_serial_ms,
                           "note": "the same with one batch in flight at a time"},
                "staged": {"value": world * B / (e2e_staged_ms * 1e-3), "ms_per_step": e2e_staged_ms,
                           "path": f"one CUDA graph per step (cudaMemcpyAsync host->device x2, sweep, "
                                   f"device->host), {E2E_STREAMS} batches in flight on {E2E_STREAMS} streams, "
                                   f"each with its own device buffers",
                           "serial_ms_per_step": e2e_staged_serial_ms}},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "frac_ordered": flops_per_run * B / (ordered_ms * 1e-3) / 1e12 / fp32_peak,
                     "frac_isolated": flops_per_run * B / (isolated_ms * 1e-3) / 1e12 / fp32_peak,
                     "note": "algorithmic 12*2^w flop per step per run; frac over the step interval of the "
                             "back-to-back loop (launches overlap: a sweep runs while the previous launch "
                             "finishes), frac_ordered over the interval of launches that read their inputs after "
                             "the previous one completes, frac_isolated over one launch alone between events "
                             "(includes the event/launch floor); peak = measured FP32 FMA throughput of this GPU "
                             "(mbqc_probe_fp32_fma); traffic = ncu DRAM read + write of one launch "
                             "(profiles/sv_fwd_reg_mw4x8.md)"},
        "concurrent": {"streams": VALUE_STREAMS, "runs_per_s": world * B / (conc_ms * 1e-3), "ms_per_step": conc_ms,
                       "note": "the same steps with independent batches in flight on separate streams; the "
                               "latency-bound kernel leaves most of the GPU free for a concurrent batch"},
        "ordered": {"ms_per_step": ordered_ms, "runs_per_s": world * B / (ordered_ms * 1e-3),
                    "lanes_per_run_log2": ord_v,
                    "variant_ms": {str(k): v for k, v in ord_tuning.items()},
                    "note": "the same back-to-back steps without MBQC_F_INPUTS_READY: each launch reads its "
                            "inputs after the previous launch completes (only the plan prologue overlaps); "
                            "lanes per run chosen for this mode"},
        "isolated_step": {"ms": isolated_ms, "runs_per_s": world * B / (isolated_ms * 1e-3),
                          "lanes_per_run_log2": ord_v,
                          "note": "one step alone between CUDA events, 256 MiB L2 flush before each; includes "
                                  "the ~4 us event/launch floor a trivial kernel shows"},
        "cpu_baseline": cpu,
        "oracle_error": dict(checks["headline"], reference="complex128 oracle (oracle/sweep.py run_sv_batch), "
                             "every run of the timed batch; infidelity 1 - |<ref|gpu>|^2, amplitude error includes "
                             "the reference's global phase", check_s=check_s),
        "clocks": clocks,
        "gpu_launches": args.steps,
        "kernel": f"sv_fwd_reg<float,5,{head_v}> (autotuned lanes-per-run 2^{head_v}; per-variant back-to-back "
                  f"ms: {', '.join(f'{k}: {v * 1e3:.2f} us' for k, v in head_tuning.items())})",
        "workloads": extra,
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return line


# ------------------------------------------------------------ secondary workloads
def _haar(rng, n, count):
    d = 2**n
    z = (rng.standard_normal((count, d, d)) + 1j * rng.standard_normal((count, d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    diag = np.diagonal(r, axis1=1, axis2=2)
    return np.ascontiguousarray((q * (diag / np.abs(diag))[:, None, :])[:, :, 0])


def _time_cuda(fn, reps, flush=None):
    import torch

    from mentpy_gb300.sweep import gpu_hold

    ts = []
    for i in range(reps):
        gpu_hold(1500.0)
        if flush is not None:
            flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def bench_adjoint(dev, fp32_peak, flush, reps=5):
    """Batched fused adjoint on many_wires([12]*6): 1024 angle vectors x 256
    Haar inputs per launch, loss = 1 - mean fidelity to a fixed random 6-qubit
    unitary's outputs; against the plain per-run GPU kernel with mentpy-style
    central finite differences (sampled) and a batched device FD."""
    import torch

    from mentpy_gb300 import circuit as C
    from mentpy_gb300.gradients import batched_fd_fidelity_grad
    from mentpy_gb300.simulators import PatternSimulator
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(SEED + 4)
    circ = C.many_wires([12] * 6)
    sw = StatevectorSweep(circ, device=dev)
    V, J, A = 1024, 256, sw.n_angles
    U = np.linalg.qr(rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64)))[0]
    inputs = _haar(rng, 6, J)
    targets = inputs @ U.T
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(V, A)), device=dev)
    inp = torch.as_tensor(inputs, dtype=torch.complex64, device=dev)
    tg = torch.as_tensor(targets, dtype=torch.complex64, device=dev)
    for _ in range(3):
        sw.fidelity_grad(ang, inp, tg)
    ms = _time_cuda(lambda: sw.fidelity_grad(ang, inp, tg), reps, flush)
    plan = sw.plan
    fwd = sum(12 * 2 ** min(plan.window, plan.n_nodes - k) for k in range(plan.n_steps))
    # forward + checkpointed recompute + backward (~2x forward): 4x forward flops per run
    alg_flops = 4.0 * fwd * V * J
    # batched device FD: (2A+1) x J runs in one forward launch per angle vector
    a1 = ang[:1].cpu().numpy()
    batched_fd_fidelity_grad(sw, a1, inputs, targets)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        batched_fd_fidelity_grad(sw, a1, inputs, targets)
    torch.cuda.synchronize()
    bfd = 3 / (time.perf_counter() - t0)
    # plain per-run GPU kernel: one PatternSimulator launch per run, sampled cost evaluation
    ps = PatternSimulator(circ, backend="cuda-sv", device=dev)
    theta = a1[0]

    def cost(th, n):
        f = 0.0
        for j in range(n):
            ps.reset(input_state=inputs[j])
            st = ps(th, output_form="sv")
            f += abs(np.vdot(targets[j], st)) ** 2
        return 1 - f / n

    cost(theta, 8)
    n_sample = 64
    t0 = time.perf_counter()
    cost(theta, n_sample)
    per_run = (time.perf_counter() - t0) / n_sample
    plain_grad_s = per_run * J * (2 * A + 1)
    grads_per_s = V / (ms * 1e-3)
    # oracle checks of the timed launch's results: the loss of 64 angle
    # vectors and the gradient of 4 against complex128 central differences
    # (h = 1e-4, mentpy's fd_gradient) of the oracle's loss
    loss_g, grad_g = sw.fidelity_grad(ang, inp, tg)
    loss_np, grad_np, ang_np = loss_g.cpu().numpy(), grad_g.cpu().numpy(), ang.cpu().numpy()
    inp64 = inp.cpu().numpy().astype(np.complex128)
    tg64 = tg.cpu().numpy().astype(np.complex128)
    spec = ("many_wires", 6, 12)
    pick = np.random.default_rng(SEED + 40).choice(V, 64, replace=False)
    tasks = [("loss", spec, ang_np[pick[i:i + 4]], inp64, tg64, loss_np[pick[i:i + 4]]) for i in range(0, 64, 4)]
    for v in pick[:4]:
        for i in range(0, A, 11):
            idx = np.arange(i, min(A, i + 11))
            tasks.append(("fd", spec, ang_np[v], idx, inp64, tg64, 1e-4, grad_np[v, idx]))
    return {
        "workload": "fused adjoint: many_wires([12]*6), w=7, 66 angles, 1024 angle vectors x 256 Haar inputs per launch",
        "grads_per_s": grads_per_s,
        "ms_per_launch": ms,
        "runs_per_launch": V * J,
        "plain_per_run_fd": {"grads_per_s": 1.0 / plain_grad_s, "sample": f"{n_sample} single-run launches "
                             f"({per_run * 1e3:.3f} ms each) x {J} inputs x {2 * A + 1} central-FD evaluations"},
        "batched_device_fd": {"grads_per_s": bfd},
        "speedup_vs_plain_per_run_fd": grads_per_s * plain_grad_s,
        "speedup_vs_batched_fd": grads_per_s / bfd,
        "roofline": {"bound": "fp32", "achieved": alg_flops / (ms * 1e-3) / 1e12, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": alg_flops / (ms * 1e-3) / 1e12 / fp32_peak,
                     "note": "4 x forward flops (forward, checkpointed recompute, reverse sweep ~2x)"},
        "workspace_mb": sw._ws.numel() / 1e6,
        "note": "speed-up against the batched device FD (one forward launch of (2A+1) x 256 runs per angle "
                "vector) is the meaningful comparator; the plain per-run figure is mostly host overhead of one "
                "PatternSimulator call per run",
    }, tasks


def bench_wide(dev, hbm_peak, flush, reps=7):
    """Streamed wide window: grid_cluster(16, 10), w=17, 64 runs, |+>^16 input."""
    import torch

    from mentpy_gb300 import circuit as C
    from mentpy_gb300.sweep import StatevectorSweep

    rng = np.random.default_rng(SEED + 3)
    circ = C.grid_cluster(16, 10)
    sw = StatevectorSweep(circ, device=dev)
    B = 64
    ang = torch.tensor(rng.uniform(0, 2 * np.pi, size=(B, sw.n_angles)), device=dev)
    out = torch.empty(B, 2**sw.n_out, dtype=torch.complex64, device=dev)
    st = torch.empty(B, dtype=torch.int32, device=dev)
    for _ in range(3):
        sw.forward(ang, None, out=out, status=st)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        sw.forward(ang, None, out=out, status=st)
    ms = _time_cuda(g.replay, reps, flush)
    w, M = sw.plan.window, sw.plan.n_steps
    alg = B * M * 16 * 2**w
    out_np, ang_np = out.cpu().numpy(), ang.cpu().numpy()
    pick = np.random.default_rng(SEED + 30).choice(B, 8, replace=False)
    tasks = [("sv", ("grid", 16, 10), ang_np[r:r + 1], None, out_np[r:r + 1], None) for r in pick]
    n_pass = 0
    k = 0
    while k < M:  # the kernel's mixed-pass grouping (windows >= 10): high* low* high*, <= 5 + 5 bits
        phase, nh, nl = 0, 0, 0
        while k < M:
            if (k % w) < 5:
                if phase == 2 or nl == 5:
                    break
                phase, nl = 1, nl + 1
            else:
                if nh == 5:
                    break
                phase, nh = (2 if phase == 1 else phase), nh + 1
            k += 1
        n_pass += 1
    moved = B * 2**w * 8 * (2 * n_pass + 2)
    dram = profile_traffic("stream_grid16x10_batch")
    roof = {"bound": "hbm", "peak": hbm_peak, "unit": "GB/s", "traffic": dram,
            "achieved": None if dram is None else dram / (ms * 1e-3) / 1e9,
            "frac": None if dram is None else dram / (ms * 1e-3) / 1e9 / hbm_peak,
            "note": "achieved = DRAM bytes of one batch (ncu dram__bytes_read.sum + dram__bytes_write.sum over "
                    "every launch of the batch, profiles/stream_pass_grid16x10.md) / batch time; the 64 MiB "
                    "state is partly L2-resident between passes",
            "l2_pass_bytes_per_batch": moved, "l2_pass_gbs": moved / (ms * 1e-3) / 1e9,
            "l2_pass_note": "one read + one write of every window per pass (what the SMs move; mostly served "
                            "by L2), not an HBM figure",
            "per_step_model_gbs": alg / (ms * 1e-3) / 1e9,
            "per_step_model_note": "16*2^w bytes per measurement step, the reference algorithm's traffic; the "
                                   "kernel fuses up to 10 steps per pass, so this is not a roofline fraction"}
    # adjoint of the same batch (a block per run, per-step history in the workspace)
    gout_np = (rng.standard_normal((B, 2**sw.n_out)) + 1j * rng.standard_normal((B, 2**sw.n_out))) / 2**sw.n_out
    gout = torch.tensor(gout_np.astype(np.complex64), device=dev)
    ast = torch.empty(B, dtype=torch.int32, device=dev)
    grad = sw.adjoint(ang, None, gout, status=ast)
    torch.cuda.synchronize()
    assert int((ast != 0).sum()) == 0
    adj_ms = _time_cuda(lambda: sw.adjoint(ang, None, gout, status=ast), reps, flush)
    hist = B * M * 2 * 2 ** (w - 1) * 8  # every step's half-state written once and read once
    grad_np = grad.cpu().numpy()
    drng = np.random.default_rng(SEED + 31)
    for r in pick[:4]:
        d = drng.standard_normal(sw.n_angles)
        d /= np.linalg.norm(d)
        tasks.append(("dir", ("grid", 16, 10), ang_np[r], gout_np[r].astype(np.complex64).astype(np.complex128), d,
                      1e-4, float(grad_np[r] @ d), float(np.abs(grad_np[r]).max())))
    fd_ms = ms * (2 * sw.n_angles + 1)  # batched device FD: (2A + 1) forward runs per gradient, same batch
    adjoint = {
        "workload": "generic adjoint (dL = Re <g|dz>) of the same 64 runs: a cluster of two 1024-thread "
                    "blocks per run (128 of the SMs), window and per-step half-states in the workspace",
        "grads_per_s": B / (adj_ms * 1e-3),
        "ms_per_launch": adj_ms,
        "speedup_vs_batched_device_fd": fd_ms / adj_ms,
        "batched_device_fd_note": "(2A+1) = 289 forward runs of the streamed kernel per gradient at the batch "
                                  "time above",
        "roofline": {"bound": "hbm", "peak": hbm_peak, "unit": "GB/s",
                     "achieved": hist / (adj_ms * 1e-3) / 1e9, "frac": hist / (adj_ms * 1e-3) / 1e9 / hbm_peak,
                     "traffic": (None if profile_traffic("sv_adj_wide_grid16x10_per_run") is None
                                 else profile_traffic("sv_adj_wide_grid16x10_per_run") * B),
                     "traffic_note": "ncu DRAM read + write per run (profiles/sv_adj_wide_grid16x10.md, a "
                                     "16-run capture) x the launch's runs",
                     "note": "algorithmic bytes = the history (2^(w-1) complex64 per step and run, written "
                             "forward, read backward) over the launch time; the 1 MB window per block stays "
                             "in L2"},
    }
    return {
        "workload": "streamed statevector: grid_cluster(16,10), w=17 (2^17 complex64 per run), 144 angles, 64 runs",
        "runs_per_s": B / (ms * 1e-3),
        "ms_per_batch": ms,
        "passes": n_pass,
        "roofline": roof,
        "adjoint": adjoint,
    }, tasks


def bench_uneven_dm(dev, fp32_peak, flush, reps=7):
    """2048 noisy density-matrix circuits: many_wires([D]*W), W ~ U{2..6},
    D ~ U{4..12}, depolarising p = 0.01, one CUDA graph per call."""
    import torch

    from mentpy_gb300 import circuit as C
    from mentpy_gb300.dm import UnevenDensityMatrixBatch
    from mentpy_gb300.plan import compile_plan

    from mentpy_gb300.native_plan import GraphBatch

    rng = np.random.default_rng(SEED + 5)
    n = 2048
    shapes = [(int(rng.integers(2, 7)), int(rng.integers(4, 13))) for _ in range(n)]
    # plan compilation: native batch compiler (flat graph arrays -> one device
    # plan table) against the Python compiler on MBQCircuit objects (sampled)
    t0 = time.perf_counter()
    ub = UnevenDensityMatrixBatch.from_graph_batch(GraphBatch.many_wires(shapes), device=dev)
    native_compile_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    for W_, D_ in shapes[:128]:
        compile_plan(C.many_wires([D_] * W_), "dm")
    python_compile_ms = (time.perf_counter() - t0) * 1e3 * n / 128
    plans = ub.plans
    buf = ub.allocate()
    angs, psis = [], []
    for c, p in enumerate(plans):
        angs.append(rng.uniform(0, 2 * np.pi, p.n_angles))
        psis.append(_haar(rng, p.n_in, 1)[0].astype(np.complex64))
        buf["angles"][c, : p.n_angles] = torch.as_tensor(angs[-1])
        buf["inputs"][c, : 2**p.n_in] = torch.as_tensor(psis[-1])
    # autotuned tile shapes of the persistent launch, then one CUDA graph
    tuned = ub.tune(buf, noise=0.01)
    ub.capture(buf, noise=0.01)
    ms = _time_cuda(lambda: ub.run(buf, noise=0.01), reps, flush)
    # the same batch as one launch per window size on its own stream (graph)
    per = UnevenDensityMatrixBatch(plans, device=dev, _dplan=ub.dplan, persistent=False)
    buf_p = {k: v.clone() for k, v in buf.items()}
    per.capture(buf_p, noise=0.01)
    per_ms = _time_cuda(lambda: per.run(buf_p, noise=0.01), reps, flush)
    assert torch.equal(buf_p["outcomes"], buf["outcomes"])
    # oracle check of every circuit of the timed batch (one vectorised call per shape)
    rho_np, outc_np = buf["rho"].cpu().numpy(), buf["outcomes"].cpu().numpy()
    by_shape = {}
    for c, sh in enumerate(shapes):
        by_shape.setdefault(sh, []).append(c)
    tasks = []
    for (W_, D_), idx in sorted(by_shape.items()):
        d = 2 ** plans[idx[0]].n_out
        M_ = plans[idx[0]].n_steps
        tasks.append(("dm", ("many_wires", W_, D_), np.stack([angs[c] for c in idx]),
                      np.stack([psis[c] for c in idx]).astype(np.complex128), 0.01,
                      np.stack([rho_np[c, : d * d].reshape(d, d) for c in idx]),
                      np.stack([outc_np[c, :M_] for c in idx])))
    flops = sum(sum(14 * 4 ** min(p.window, p.n_nodes - k) for k in range(p.n_steps)) for p in plans)
    # the factored sweep reads and writes the (w-1)-qubit matrix once per step
    smem_bytes = sum(16 * 4 ** (p.window - 1) * p.n_steps for p in plans)
    smem_peak = _smem_peak(dev)
    ok = int((buf["status"] == 0).sum())
    # adjoint through the noisy channel for every circuit (d Re<Gamma|rho>/d angles)
    buf["grad_out"] = torch.zeros_like(buf["rho"])
    for c, p in enumerate(plans):
        d = 2 ** p.n_out
        buf["grad_out"][c, : d * d] = torch.eye(d, dtype=torch.complex64).reshape(-1)[: d * d] * 0.5
    ub.adjoint(buf, noise=0.01)
    adj_ms = _time_cuda(lambda: ub.adjoint(buf, noise=0.01), reps, flush)
    adj_ok = int((buf["status"] == 0).sum())
    return {
        "workload": "uneven noisy density matrix: 2048 circuits many_wires([D]*W), W~U{2..6}, D~U{4..12}, "
                    "w=W+1<=7, depolarising 0.01, one persistent launch (tiles claimed longest first, tile shapes "
                    "autotuned) captured in a CUDA graph",
        "circuits_per_s": n / (ms * 1e-3),
        "ms_per_batch": ms,
        "tuned": {k: v for k, v in tuned.items() if k != "candidates"},
        "per_window_launches": {"ms_per_batch": per_ms, "circuits_per_s": n / (per_ms * 1e-3),
                                "note": "one launch per window size, each on its own stream, in one graph"},
        "status_ok": ok,
        "adjoint": {"circuits_per_s": n / (adj_ms * 1e-3), "ms_per_batch": adj_ms, "status_ok": adj_ok,
                    "note": "gradient of Re<Gamma|rho_out> for every circuit through the depolarising channel "
                            "(one launch per window size on its own stream)"},
        "plan_compile_ms": {"native_batch": native_compile_ms,
                            "python_mbqcircuit_estimate": python_compile_ms,
                            "note": "native: GraphBatch.many_wires + mbqc_plan_create_from_graphs (incl. upload); "
                                    "python: MBQCircuit + compile_plan per circuit, 128 timed, scaled to 2048"},
        "roofline": {"bound": "smem", "achieved": smem_bytes / (ms * 1e-3) / 1e9, "peak": smem_peak, "unit": "GB/s",
                     "frac": smem_bytes / (ms * 1e-3) / 1e9 / smem_peak, "traffic": None,
                     "note": "factored density matrix: one read and one write of the 4^(w-1)-entry complex64 "
                             "matrix per step and run (16*4^(w-1) B), over the batch time; peak = measured "
                             "shared-memory bandwidth of this GPU (mbqc_probe_smem_bw); the matrices never leave "
                             "shared memory, so DRAM carries only inputs and outputs",
                     "full_matrix_flop_model": {"achieved_tflops": flops / (ms * 1e-3) / 1e12,
                                                "frac_of_fp32": flops / (ms * 1e-3) / 1e12 / fp32_peak,
                                                "note": "14*4^w flop per step per run, the full-matrix algorithm's "
                                                        "work"}},
    }, tasks


def _smem_peak(dev):
    import ctypes

    import torch

    from mentpy_gb300 import _native

    sink = torch.zeros(1, dtype=torch.float32, device=dev)
    g = ctypes.c_double()
    _native.check(_native.lib().mbqc_probe_smem_bw(20000, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(g),
                                                   ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    return g.value


def bench_train(dev, iters=20):
    """Device training run: many_wires([12]*6), 1024 angle vectors trained at
    once on 256 (Haar input, target) pairs, fused fidelity adjoint + Adam per
    iteration, one CUDA graph replay per iteration."""
    import torch

    from mentpy_gb300 import circuit as C
    from mentpy_gb300.sweep import StatevectorSweep
    from mentpy_gb300.train import FidelityTrainer

    rng = np.random.default_rng(SEED + 7)
    sw = StatevectorSweep(C.many_wires([12] * 6), device=dev)
    V, J = 1024, 256
    x0 = rng.uniform(0, 2 * np.pi, size=(V, sw.n_angles))
    inp = _haar(rng, 6, J)
    u = np.linalg.qr(rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64)))[0]
    tr = FidelityTrainer(sw, inp, inp @ u.T, x0, step_size=0.02)
    tr.run(2)  # records the graph
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    tr.run(iters)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    return {"workload": "device training run: many_wires([12]*6), 1024 angle vectors x 256 inputs, fused fidelity "
                        "adjoint + Adam (mentpy's), one graph replay per iteration",
            "iterations_per_s": 1e3 / ms, "ms_per_iteration": ms, "grads_per_s": V * 1e3 / ms,
            "loss_first_last_mean": [float(tr.losses[0].mean()), float(tr.losses[-1].mean())]}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    per_step = []
    cb = None
    for _ in range(max(args.warmup, 3) // 3):
        cpu_baseline(budget_s=2.0, runs_per_proc=50)
    budget = max(1.0, min(8.0, 100.0 / max(args.steps, 1)))
    for _ in range(args.steps):
        cb = cpu_baseline(budget_s=budget, runs_per_proc=BATCH)
        per_step.append(cb["value"])
    v = float(np.mean(per_step))
    cb["value"] = v
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": BATCH / v * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "complex128",
        "data": "synthetic: seeded uniform angles in [0, 2pi) and Haar-random 4-qubit inputs",
        "config": workload_config(world),
        "timing": "each step times a bounded sample of the batch on every host core",
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_baseline": cb,
    }
    print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the secondary workloads (adjoint, wide window, uneven density matrix)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
