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
``e2e``    runs/s through the public API with host buffers: every step the
           sweep reads that step's angles and inputs from pinned host memory
           and writes the output states there (``prepare(mapped_host=True,
           inputs_ready=True)``, host-filled buffers: one pre-bound C call per
           step; the kernel's uncached loads and its stores cross the CPU-GPU
           link; no staging copy).  Four batches are in flight, each on its
           own stream with its own host buffer set.
           ``e2e.serial`` keeps one in flight; ``e2e.staged`` is one batch at
           a time with copy-engine transfers (host->device copies, sweep,
           device->host copy in one graph).
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
VALUE_STREAMS = 4  # batches in flight in the concurrent device-resident figure
VALUE_SETS = 128  # device input sets of the timed loop (184 MB > L2)


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

    def step():
        sw.forward(ang_d, inp_d, out=out_d, status=st_d)

    # autotuner: fastest lanes-per-run for this batch with ordered launches;
    # every path below uses the choice (timed with overlapping launches it
    # picks 1 lane per run: ~2 % faster back to back, but 5x slower through
    # host buffers and 2x alone)
    tuned_variant = sw.tune(ang_d, inp_d)
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

    def set_step(i, ready=True):
        # every input set is written before the timed region, so the steps
        # may declare their inputs ready (MBQC_F_INPUTS_READY): a launch reads
        # them and sweeps while the previous one finishes, and waits for it
        # only before writing
        j = i % n_sets
        sw.forward(ang_sets[j], inp_sets[j], out=out_sets[j], status=st_d, inputs_ready=ready)

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
            step()
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
            set_step(i, ready=False)
        o1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ordered_ms = reduce_max(o0.elapsed_time(o1) / args.steps)
    assert int((st_d != 0).sum()) == 0
    assert torch.equal(out_sets[(args.steps - 1) % n_sets], out_d)
    # the same with VALUE_STREAMS independent batches in flight (a stream each)
    streams_v = [torch.cuda.Stream(device=dev) for _ in range(VALUE_STREAMS)]
    sts_v = [torch.zeros_like(st_d) for _ in range(VALUE_STREAMS)]

    def conc_step(i):
        j = i % n_sets
        with torch.cuda.stream(streams_v[i % VALUE_STREAMS]):
            sw.forward(ang_sets[j], inp_sets[j], out=out_sets[j], status=sts_v[i % VALUE_STREAMS])

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
    # mapped: the kernel reads the angles and inputs (uncached loads, so every
    # step fetches them over the CPU-GPU link) and writes the states in place
    preps = [sw.prepare(ang_h[j], inp_h[j], out_h[j], status=st_r[j], mapped_host=True, inputs_ready=True)
             for j in range(E2E_RING)]
    # staged: copy engines host -> device, sweep, device -> host, one graph per set
    ang_e = torch.empty_like(ang_d)
    inp_e = torch.empty_like(inp_d)
    staged_graphs = []
    for j in range(E2E_RING):
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            sw.forward(ang_e, inp_e, out=out_d, status=st_d)
        stream.wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            ang_e.copy_(ang_h[j], non_blocking=True)
            inp_e.copy_(inp_h[j], non_blocking=True)
            sw.forward(ang_e, inp_e, out=out_d, status=st_d)
            out_h[j].copy_(out_d, non_blocking=True)
        staged_graphs.append(g)

    def time_e2e(fn, n_streams=1):
        # step i runs on stream i % n_streams (independent batches in flight)
        streams = [torch.cuda.Stream(device=dev) for _ in range(n_streams)]

        def on(i):
            fn(i, streams[i % n_streams])

        for i in range(3):
            on(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for s in streams:
            s.wait_stream(stream)
        for i in range(args.steps):
            on(3 + i)
        for s in streams:
            stream.wait_stream(s)
        e1.record(stream)
        torch.cuda.synchronize()
        return reduce_max(e0.elapsed_time(e1) / args.steps)

    def staged_step(i, s):
        with torch.cuda.stream(s):
            staged_graphs[i % E2E_RING].replay()

    e2e_staged_ms = time_e2e(staged_step)
    assert torch.equal(out_h[(2 + args.steps) % E2E_RING], out_d.cpu())
    out_h.zero_()
    e2e_serial_ms = time_e2e(lambda i, s: preps[i % E2E_RING](s))
    out_h.zero_()
    e2e_ms = time_e2e(lambda i, s: preps[i % E2E_RING](s), n_streams=E2E_STREAMS)
    # the states written to host memory are the sweep's (check against the resident run)
    for j in range(E2E_RING):
        assert torch.equal(out_h[j], out_d.cpu())
    assert int((st_r != 0).sum()) == 0 and int((st_d != 0).sum()) == 0

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None

    w = plan.window
    flops_per_run = sum(12 * 2 ** min(w, plan.n_nodes - k) for k in range(plan.n_steps))
    achieved = flops_per_run * B / (ms * 1e-3) / 1e12
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile)).get("sv_fwd_reg_mw4x8")
    cpu = cpu_baseline()
    clocks = clk.summary()
    hbm_peak = 6765.7
    peaks_file = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_file):
        hbm_peak = float(json.load(open(peaks_file)).get("hbm_gbs", hbm_peak))
    extra = {}
    if not args.headline_only:
        extra["adjoint_many_wires_6x12"] = bench_adjoint(dev, fp32_peak, flush)
        extra["wide_window_grid_16x10"] = bench_wide(dev, hbm_peak, flush)
        extra["uneven_dm_2048_circuits"] = bench_uneven_dm(dev, fp32_peak, flush)
        extra["train_many_wires_6x12"] = bench_train(dev)
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
        "config": {"workload": "many_wires([8]*4) statevector sweep, window 5, 28 angles",
                   "batch_per_gpu": B, "global_batch": world * B,
                   "l2": "inputs larger than L2: 128 distinct input sets (184 MB) read in turn by back-to-back "
                         "steps after one flush",
                   "parallelism": f"replicas x{world} (independent batches)"},
        "e2e": {"value": world * B / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "path": f"StatevectorSweep.prepare(mapped_host=True, inputs_ready=True), one pre-bound C call per step, "
                        f"{E2E_STREAMS} independent batches in flight on {E2E_STREAMS} streams: the kernel reads "
                        f"the pinned host angles/inputs with uncached loads (fetched over the CPU-GPU link every "
                        f"step) and writes the states to pinned host memory; {E2E_RING} host buffer sets",
                "streams": E2E_STREAMS,
                "serial": {"value": world * B / (e2e_serial_ms * 1e-3), "ms_per_step": e2e_serial_ms,
                           "note": "the same with one batch in flight at a time"},
                "staged": {"value": world * B / (e2e_staged_ms * 1e-3), "ms_per_step": e2e_staged_ms,
                           "path": "one CUDA graph per step, one batch in flight: cudaMemcpyAsync host->device "
                                   "x2, sweep, device->host"}},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "note": "algorithmic 12*2^w flop per step per run over the step interval of the "
                             "back-to-back loop; peak = measured FP32 FMA throughput of this GPU "
                             "(mbqc_probe_fp32_fma)"},
        "concurrent": {"streams": VALUE_STREAMS, "runs_per_s": world * B / (conc_ms * 1e-3), "ms_per_step": conc_ms,
                       "note": "the same steps with independent batches in flight on separate streams; the "
                               "latency-bound kernel leaves most of the GPU free for a concurrent batch"},
        "ordered": {"ms_per_step": ordered_ms, "runs_per_s": world * B / (ordered_ms * 1e-3),
                    "note": "the same back-to-back steps without MBQC_F_INPUTS_READY: each launch reads its "
                            "inputs after the previous launch completes (only the plan prologue overlaps)"},
        "isolated_step": {"ms": isolated_ms, "runs_per_s": world * B / (isolated_ms * 1e-3),
                          "note": "one step alone between CUDA events, 256 MiB L2 flush before each; includes "
                                  "the ~4 us event/launch floor a trivial kernel shows"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": args.steps,
        "kernel": f"sv_fwd_reg<float,5,{tuned_variant}> (autotuned lanes-per-run 2^{tuned_variant})",
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
    }


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
    return {
        "workload": "streamed statevector: grid_cluster(16,10), w=17 (2^17 complex64 per run), 144 angles, 64 runs",
        "runs_per_s": B / (ms * 1e-3),
        "ms_per_batch": ms,
        "passes": n_pass,
        "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                     "frac": alg / (ms * 1e-3) / 1e9 / hbm_peak, "traffic": None,
                     "note": "achieved counts one read + one write of the window per measurement (16*2^w B per "
                             "step); the kernel fuses up to 10 steps per pass",
                     "pass_bytes_per_batch": moved, "pass_gbs": moved / (ms * 1e-3) / 1e9,
                     "pass_frac": moved / (ms * 1e-3) / 1e9 / hbm_peak},
    }


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
    for c, p in enumerate(plans):
        buf["angles"][c, : p.n_angles] = torch.as_tensor(rng.uniform(0, 2 * np.pi, p.n_angles))
        buf["inputs"][c, : 2**p.n_in] = torch.as_tensor(_haar(rng, p.n_in, 1)[0], dtype=torch.complex64)
    ub.capture(buf, noise=0.01)
    ms = _time_cuda(lambda: ub.run(buf, noise=0.01), reps, flush)
    flops = sum(sum(14 * 4 ** min(p.window, p.n_nodes - k) for k in range(p.n_steps)) for p in plans)
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
                    "w=W+1<=7, depolarising 0.01, one CUDA graph (one launch per window size on its own stream)",
        "circuits_per_s": n / (ms * 1e-3),
        "ms_per_batch": ms,
        "status_ok": ok,
        "adjoint": {"circuits_per_s": n / (adj_ms * 1e-3), "ms_per_batch": adj_ms, "status_ok": adj_ok,
                    "note": "gradient of Re<Gamma|rho_out> for every circuit through the depolarising channel "
                            "(one launch per window size on its own stream)"},
        "plan_compile_ms": {"native_batch": native_compile_ms,
                            "python_mbqcircuit_estimate": python_compile_ms,
                            "note": "native: GraphBatch.many_wires + mbqc_plan_create_from_graphs (incl. upload); "
                                    "python: MBQCircuit + compile_plan per circuit, 128 timed, scaled to 2048"},
        "roofline": {"bound": "fp32", "achieved": flops / (ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": flops / (ms * 1e-3) / 1e12 / fp32_peak, "note": "14*4^w flop per step per run"},
    }


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
        "config": {"workload": "many_wires([8]*4) statevector sweep, window 5, 28 angles",
                   "batch_per_gpu": BATCH, "sampled": "each step times a bounded sample of the batch"},
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
