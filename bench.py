"""Benchmark of the GB300 NTT library (one JSON line on stdout).

Workload (one step): the batched radix-4 int16 forward NTT of 4096 polynomials
x 4 RNS moduli {7681, 10753, 12289, 12289}.  7681 and 10753 have no 1024-th
root of unity (their largest power-of-two root order is 512) and radix-4 needs
n = 4^k, so their lanes run at n = 256; the two 12289 lanes run at n = 1024.
Inputs are seeded uniform residues, resident in HBM; L2 is flushed (256 MiB
write) before every timed step.  A step is the whole batch (16384 NTTs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's algorithm on the host cores: the
reference's own kernels need AMD's AIE toolchain, so its CPU restatement in
oracle/ (the parity oracle) is run with all host threads instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

SEGMENTS = [  # (q, n, polynomials, generator of Z_q^*)
    (7681, 256, 4096, 17),
    (10753, 256, 4096, 11),
    (12289, 1024, 8192, 41),
]
SEED = 20261203
METRIC = "batched NTT/s & HBM GB/s vs plain per-NTT launch (bit-exact); p50/p99 serve latency"
WORKLOAD = ("batched radix-4 int16 forward NTT: 4096 polys x 4 moduli {7681,10753,12289,12289}; "
            "n=256 for 7681/10753 (no 1024-th root of unity), n=1024 for 12289")


OUTPUTS = {
    "canonical": "canonical residues in [0, q): the reference's outputs reduced mod q (its lanes do not wrap "
                 "on this workload), i.e. the forward DFT in bit-reversed order",
    "lanes": "the reference's partially reduced int16 outputs, bit for bit",
}


def workload_config(arith, gpus):
    """The JSON line's config: identical in both arms (same keys, same values)."""
    return {"workload": WORKLOAD, "outputs": OUTPUTS[arith], "polys_per_step": sum(cnt for _, _, cnt, _ in SEGMENTS),
            "coefficients_per_step": sum(n * cnt for _, n, cnt, _ in SEGMENTS),
            "algorithmic_bytes_per_step": sum(2 * n * 2 * cnt for _, n, cnt, _ in SEGMENTS),
            "l2": "flushed before every step (256 MiB write, untimed); the CPU arm times host memory",
            "parallelism": f"replicas{gpus}"}


def coeffs_per_poly():
    return sum(n * cnt for _, n, cnt, _ in SEGMENTS) / sum(cnt for _, _, cnt, _ in SEGMENTS)


def oracle_outputs(oracle, x, q, n, g, arith, threads=1):
    """The reference's algorithm (the oracle's restatement) on x; reduced mod q
    for canonical outputs."""
    return oracle.Plan(oracle.R4_I16_FWD, n, q, root_of(q, n, g))(x, threads=threads,
                                                                   canonical=arith == "canonical")


def max_over_ranks(x, dist=None, device="cpu"):
    """The slowest rank's value (every rank calls it; `dist` None on one process)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(polys_per_rank, world, ms_max):
    """Replicas: every rank transforms its own copy of the batch; the job's
    throughput is all ranks' polynomials over the slowest rank's step time."""
    return world * polys_per_rank / (ms_max / 1e3)


def root_of(q, n, g):
    if q == 12289:
        return pow(41, 4096 // n, q)
    return pow(g, (q - 1) // n, q)


def make_inputs():
    rng = np.random.default_rng(SEED)
    return [rng.integers(0, q, size=(cnt, n)).astype(np.int16) for q, n, cnt, _ in SEGMENTS]


def load_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def host_threads():
    """The host cores this process may run on (the cgroup / affinity set, not the machine's count)."""
    try:
        return len(os.sched_getaffinity(0)) or 1
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def load_traffic():
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.samples = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        inside = [s for t, s in self.samples if t0 <= t <= t1]
        note = "sampled during the timed region"
        if not inside:
            inside = [s for t, s in self.samples if t1 - 2.0 <= t <= t1 + 0.2]
            note = "timed region shorter than the sampling period: samples from the surrounding load"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "note": "nvidia-smi unavailable"}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[1]) for s in inside if num(s[1]) is not None]
        mx = [num(s[2]) for s in inside if num(s[2]) is not None]
        reasons = sorted({names[i] for s in inside for i in range(4) if s[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "note": note}


def cpu_baseline(inputs, seconds, threads, arith):
    """The oracle (CPU restatement of the reference's loops) over all host threads,
    whole batches until `seconds` have passed (reduced mod q for canonical outputs)."""
    from oracle import oracle
    done, t0 = 0, time.perf_counter()
    while True:
        for (q, n, _, g), x in zip(SEGMENTS, inputs):
            oracle_outputs(oracle, x, q, n, g, arith, threads)
        done += sum(x.shape[0] for x in inputs)
        el = time.perf_counter() - t0
        if el >= seconds:
            return done / el, done, el


def run_reference(args):
    """--impl reference: the reference's algorithm (oracle restatement) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = host_threads()
    inputs = make_inputs()
    from oracle import oracle

    def step(xs):
        for (q, n, _, g), x in zip(SEGMENTS, xs):
            oracle_outputs(oracle, x, q, n, g, args.arith, threads)
    # size each step so that warmup + steps stay within about two minutes
    t0 = time.perf_counter()
    step(inputs)
    full = time.perf_counter() - t0
    budget = 120.0
    frac = 1.0
    if full * (args.steps + args.warmup) > budget:
        frac = max(1e-3, budget / (full * (args.steps + args.warmup)))
    sample = [x[: max(1, int(x.shape[0] * frac))] for x in inputs]
    per_step = sum(s.shape[0] for s in sample)
    for _ in range(args.warmup):
        step(sample)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step(sample)
        times.append(time.perf_counter() - t)
    ms = 1e3 * sum(times) / len(times)
    value = per_step / (ms / 1e3)
    desc = f"{per_step} of the 16384 NTTs per step ({frac:.3f} of every segment)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "NTT/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16", "data": "synthetic",
        "config": workload_config(args.arith, args.gpus),
        "coefficients_per_s": value * coeffs_per_poly(),
        "cpu_baseline": {"value": value, "unit": "NTT/s", "cores": threads, "kind": "port",
                         "sample": desc + "; the reference's AIE kernels cannot be built here, so its CPU "
                                          "restatement (oracle/ntt_oracle.c, the parity oracle) is timed"
                                          + ("; outputs reduced mod q in the same threads" if args.arith == "canonical" else "")},
        "e2e": {"value": value, "unit": "NTT/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from oracle import oracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    inputs = make_inputs()
    flags = gb.FLAG_CANONICAL if args.arith == "canonical" else 0
    plans = [gb.Plan(gb.Kind.R4_I16_FWD, n, q, root_of(q, n, g), 0, flags) for (q, n, _, g) in SEGMENTS]
    d_in = [torch.from_numpy(x).to(dev) for x in inputs]
    d_out = [torch.empty_like(x) for x in d_in]
    batch = gb.Batch([(plans[i], d_in[i], d_out[i]) for i in range(len(SEGMENTS))])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    polys = sum(cnt for _, _, cnt, _ in SEGMENTS)
    algo_bytes = sum(2 * n * 2 * cnt for _, n, cnt, _ in SEGMENTS)

    # correctness gate on the timed data: every polynomial, bit-exact vs the oracle
    batch.execute(stream)
    torch.cuda.synchronize()
    batch.status()
    want_out = []
    for i, (q, n, _, g) in enumerate(SEGMENTS):
        want = oracle_outputs(oracle, inputs[i], q, n, g, args.arith, host_threads())
        assert np.array_equal(d_out[i].cpu().numpy(), want), "GPU output differs from the oracle"
        want_out.append(want)

    def timed(run, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            run()
            b.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    for _ in range(args.warmup):
        flush.zero_()
        batch.execute(stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = gb.launch_count()
    t_wall0 = time.time()
    # one plain launch of the persistent kernel per step (a CUDA graph replay of
    # the same single launch measured 0.9-1.2 us slower per step; see run)
    step_ms = timed(lambda: batch.execute(stream), args.steps)
    t_wall1 = time.time()
    launches = gb.launch_count() - launches0
    if dist:
        dist.barrier()
    sampler.stop()
    batch.status()
    ms = max_over_ranks(sum(step_ms) / len(step_ms), dist, dev)
    # the same step as a CUDA graph replay (gbntt_batch_graph_launch), untimed by the contract
    gsteps = min(args.steps, 500)
    graph_ms = sum(timed(lambda: batch.graph_launch(stream), gsteps)) / gsteps
    batch.status()
    value = whole_job_value(polys, world, ms)
    peak, peak_src = load_peaks()
    achieved = algo_bytes / (ms / 1e3) / 1e9
    traffic = load_traffic()

    extra = {}
    if rank == 0 and not args.skip_per_ntt:
        # the same batch as one launch per segment (plan path) ...
        pp = timed(lambda: [plans[i].execute(d_in[i], d_out[i], SEGMENTS[i][2], stream)
                            for i in range(len(SEGMENTS))], min(args.steps, 200))
        pms = sum(pp) / len(pp)
        extra["per_segment_launches"] = {"value": polys / (pms / 1e3), "unit": "NTT/s", "launches_per_step": 3}
        # ... and as plain per-NTT launches (one launch per polynomial)
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for i, (q, n, cnt, _) in enumerate(SEGMENTS):
            bs = n * 2
            base_in, base_out = d_in[i].data_ptr(), d_out[i].data_ptr()
            for j in range(cnt):
                plans[i].execute(base_in + j * bs, base_out + j * bs, 1, stream)
        b.record(stream)
        torch.cuda.synchronize()
        pm = a.elapsed_time(b)
        extra["per_ntt_launch"] = {"value": polys / (pm / 1e3), "unit": "NTT/s", "launches": polys,
                                   "batched_speedup": (polys / (ms / 1e3)) / (polys / (pm / 1e3))}

    e2e = None
    if not args.skip_e2e:
        # end to end through the C ABI: pinned host buffers in, results in host memory out
        h_in = [torch.from_numpy(x).pin_memory() for x in inputs]
        h_out = [torch.empty_like(x).pin_memory() for x in h_in]
        e2e_steps = max(3, min(args.steps, 100))
        for _ in range(min(args.warmup, 5)):
            batch.execute_host(h_in, h_out, stream)
        e2e_t = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            batch.execute_host(h_in, h_out, stream)
            e2e_t.append(time.perf_counter() - t0)
        e2e_ms = max_over_ranks(1e3 * sum(e2e_t) / len(e2e_t), dist, dev)   # whole job: slowest rank
        for i in range(len(SEGMENTS)):
            assert np.array_equal(h_out[i].numpy(), want_out[i]), "end-to-end output differs from the oracle"
        e2e = {"value": whole_job_value(polys, world, e2e_ms), "unit": "NTT/s",
               "h2d_bytes_per_step": world * algo_bytes // 2, "d2h_bytes_per_step": world * algo_bytes // 2,
               "ms_per_step": e2e_ms, "steps": e2e_steps,
               "api": "gbntt_batch_execute_host, wall clock; pinned host buffers, which the zero-copy persistent "
                      "kernel reads and writes directly over the host-device link (one launch per step)"}

    configs = None
    if rank == 0 and not args.skip_configs:
        configs = run_configs(gb, oracle, flush, stream, peak, args.arith)

    serving = None
    if rank == 0 and not args.skip_serve:
        serving = run_serving(gb, args.serve_seconds, args.arith)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    threads = host_threads()
    cpu = None
    if not args.skip_cpu:
        v, done, el = cpu_baseline(inputs, args.cpu_seconds, threads, args.arith)
        cpu = {"value": v, "unit": "NTT/s", "cores": threads, "kind": "port",
               "sample": f"{done} NTTs of the same workload in {el:.1f} s (whole batches), oracle/ntt_oracle.c "
                         f"with {threads} threads; the reference's AIE kernels cannot be built here"
                         + ("; outputs reduced mod q in the same threads" if args.arith == "canonical" else "")}
    tr = (traffic or {}).get("headline_" + args.arith) or {}
    line = {
        "metric": METRIC, "value": value, "unit": "NTT/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16", "data": "synthetic",
        "config": workload_config(args.arith, world),
        "coefficients_per_s": value * coeffs_per_poly(),
        "run": {"launch": "one persistent kernel launch per step (gbntt_batch_execute)", "arithmetic": args.arith,
                "graph_replay_ms_per_step": graph_ms,
                "autotuned_log2_coeffs_per_thread": batch.query(4), "autotuned_cta_threads": batch.query(6),
                "autotuned_ctas_per_sm_budget": batch.query(7)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src,
                     "kernel": f"k_batch<int16> persistent radix-4 ({args.arith} arithmetic, all 16384 polys "
                               "per launch)",
                     "algorithmic_bytes_per_launch": algo_bytes, "avg_launch_ms": ms,
                     "traffic": tr.get("bytes_per_launch"),
                     # the bound that holds: integer issue (ncu capture of the same kernel)
                     "issue": {k: tr.get(k) for k in
                               ("issue_active_frac", "alu_pipe_frac", "thread_instructions_per_coefficient")}},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": sampler.summary(t_wall0, t_wall1),
        "serving": serving,
        "other_configs": configs,
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_configs(gb, oracle, flush, stream, peak, arith):
    """The other workloads, measured beside the headline (device-resident
    inputs, L2 flushed before each timed launch, CUDA events on the stream,
    median of the timed launches), each checked against the oracle first (the
    reference's lanes) or the exact transform (canonical residues):
      C3 twin: the headline batch in the other arithmetic;
      C1: radix-2 int16 forward then inverse, n = 1024, one polynomial (latency);
      C2: radix-2 int32 forward + inverse, n = 4096, 1024 polynomials for each
          of four primes (one persistent launch per direction);
      C4a: ragged radix-8 int16 forward with the bit reversal fused, 2000
          polynomials of n = 2^U, U uniform in {8..12}, one persistent launch;
      C4b: int32 forward and inverse of 64 polynomials of n = 2^20, q = 998244353
          (canonical: the TMA-fed four-step; lanes: the two-pass schedule);
      C16k: int32 forward and inverse of 4096 polynomials of n = 2^14.
    Entries for n >= 2^14 carry a roofline object like the headline's."""
    import torch

    dev = torch.device("cuda")
    rng = np.random.default_rng(SEED + 2)
    traffic = load_traffic() or {}
    out = {}
    CAN = gb.FLAG_CANONICAL

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for _ in range(3):
            fn()
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return statistics.median([a.elapsed_time(b) for a, b in evs])

    def entry(ntts, coefs, nbytes, ms, launches, **kw):
        e = {"NTT_per_s": ntts / (ms / 1e3), "coefficients_per_s": coefs / (ms / 1e3),
             "GBps": nbytes / (ms / 1e3) / 1e9, "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / peak, "ms": ms,
             "launches": launches}
        e.update(kw)
        return e

    def roofline(key, nbytes, ms, kernel):
        achieved = nbytes / (ms / 1e3) / 1e9
        tr = traffic.get(key) or {}
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "kernel": kernel, "algorithmic_bytes_per_launch": nbytes, "avg_launch_ms": ms,
                "traffic": tr.get("bytes_per_launch"), "traffic_note": tr.get("note")}

    # C3 in the other arithmetic
    other = "lanes" if arith == "canonical" else "canonical"
    fl = CAN if other == "canonical" else 0
    xs = make_inputs()
    segs = []
    for (q, n, cnt, g), x in zip(SEGMENTS, xs):
        d = torch.from_numpy(x).to(dev)
        segs.append((gb.Plan(gb.Kind.R4_I16_FWD, n, q, root_of(q, n, g), 0, fl), d, torch.empty_like(d)))
    b3 = gb.Batch(segs)
    b3.execute(stream)
    torch.cuda.synchronize()
    for (q, n, _, g), x, (_, _, y) in zip(SEGMENTS, xs, segs):
        assert np.array_equal(y.cpu().numpy(), oracle_outputs(oracle, x, q, n, g, other, host_threads())), "C3"
    ms = timed(lambda: b3.execute(stream), 200)
    polys = sum(c for _, _, c, _ in SEGMENTS)
    coefs = sum(n * c for _, n, c, _ in SEGMENTS)
    out[f"C3_{other}"] = entry(polys, coefs, 4 * coefs, ms, b3.launches, outputs=OUTPUTS[other])
    del b3, segs

    # C1: latency of one forward + inverse pair
    q, n = 12289, 1024
    root = pow(41, 4, q)
    x = rng.integers(0, q, (1, n)).astype(np.int16)
    dx = torch.from_numpy(x).to(dev)
    for name, fl in (("lanes", 0), ("canonical", CAN)):
        f = gb.Plan(gb.Kind.R2_I16_FWD, n, q, root, 0, fl)
        i = gb.Plan(gb.Kind.R2_I16_INV, n, q, root, 0, fl)
        y, z = torch.empty_like(dx), torch.empty_like(dx)
        f.execute(dx, y, 1, stream)
        i.execute(y, z, 1, stream)
        torch.cuda.synchronize()
        want = oracle.Plan(oracle.R2_I16_FWD, n, q, root)(x)
        assert np.array_equal(y.cpu().numpy(), want % q if fl else want), "C1"
        assert np.array_equal(z.cpu().numpy().astype(np.int64) % q, (x.astype(np.int64) * n) % q), "C1"
        ms = timed(lambda: (f.execute(dx, y, 1, stream), i.execute(y, z, 1, stream)), 200)
        out[f"C1_r2_i16_fwd_inv_n1024_{name}"] = {"us_per_fwd_inv_pair": ms * 1e3, "launches": 2}

    # C2: the four primes' forward transforms as one persistent launch, then the inverses
    n, cnt = 4096, 1024
    for name, fl in (("canonical", CAN), ("lanes", 0)):
        fwd_segs, inv_segs, keep = [], [], []
        for qq, g in SERVE_Q32:
            root = pow(g, (qq - 1) // n, qq)
            x = rng.integers(0, qq, (cnt, n)).astype(np.int32)
            dx = torch.from_numpy(x).to(dev)
            y, z = torch.empty_like(dx), torch.empty_like(dx)
            fwd_segs.append((gb.Plan(gb.Kind.R2_I32_FWD, n, qq, root, 0, fl), dx, y))
            inv_segs.append((gb.Plan(gb.Kind.R2_I32_INV, n, qq, root, 0, fl), y, z))
            keep.append((x, qq, root))
        bf, bi = gb.Batch(fwd_segs), gb.Batch(inv_segs)
        bf.execute(stream)
        bi.execute(stream)
        torch.cuda.synchronize()
        for (x, qq, root), (_, _, y), (_, _, z) in zip(keep, fwd_segs, inv_segs):
            # every polynomial: the forward against the oracle, the round trip n x
            want = oracle.Plan(oracle.R2_I32_FWD, n, qq, root)(x, threads=host_threads())
            assert np.array_equal(y.cpu().numpy(), want % qq if fl else want), "C2"
            assert np.array_equal(z.cpu().numpy().astype(np.int64) % qq, (x.astype(np.int64) * n) % qq), "C2"
        ms = timed(lambda: (bf.execute(stream), bi.execute(stream)), 50)
        nb = 4 * 2 * cnt * 2 * n * 4
        out[f"C2_r2_i32_fwd_inv_n4096_4primes_{name}"] = entry(8 * cnt, 8 * cnt * n, nb, ms, 2)
        del bf, bi, fwd_segs, inv_segs

    # C4a: ragged radix-8, natural-order output, one persistent launch
    q = 12289
    U = rng.integers(8, 13, 2000)
    for name, fl in (("canonical", CAN), ("lanes", 0)):
        segs, keep, algo, coefs = [], [], 0, 0
        for L in range(8, 13):
            c = int((U == L).sum())
            n = 1 << L
            p = gb.Plan(gb.Kind.R8_I16_FWD, n, q, pow(41, 4096 // n, q), 0, gb.FLAG_NATURAL_ORDER | fl)
            x = rng.integers(0, q, (c, n)).astype(np.int16)
            dx = torch.from_numpy(x).to(dev)
            dy = torch.empty_like(dx)
            segs.append((p, dx, dy))
            keep.append((x, dy, n))
            algo += 2 * 2 * n * c
            coefs += n * c
        batch = gb.Batch(segs)
        batch.execute(stream)
        torch.cuda.synchronize()
        for x, dy, n in keep:
            # every polynomial against the oracle's radix-8 chain, bit reversal applied
            want = oracle.Plan(oracle.R8_I16_FWD, n, q, pow(41, 4096 // n, q), r8_exact=True)(x, threads=host_threads())
            want = want[:, oracle.bitrev_perm(n)]
            assert np.array_equal(dy.cpu().numpy(), want % q if fl else want), "C4a"
        ms = timed(lambda: batch.execute(stream), 200)
        out[f"C4a_ragged_r8_i16_natural_2000_{name}"] = entry(2000, coefs, algo, ms, batch.query(0), us=ms * 1e3)
        del batch, segs

    # C4b and C16k: int32 n >= 2^14, forward and inverse
    for tag, L, cnt in (("C4b", 20, 64), ("C16k", 14, 4096)):
        q = 998244353
        n = 1 << L
        root = pow(3, (q - 1) >> L, q)
        x = rng.integers(0, q, (cnt, n)).astype(np.int32)
        dx = torch.from_numpy(x).to(dev)
        y, z = torch.empty_like(dx), torch.empty_like(dx)
        nb = 2 * n * 4 * cnt
        for name, fl in (("canonical", CAN), ("lanes", 0)):
            f = gb.Plan(gb.Kind.R2_I32_FWD, n, q, root, 0, fl)
            i = gb.Plan(gb.Kind.R2_I32_INV, n, q, root, 0, fl)
            f.execute(dx, y, cnt, stream)
            i.execute(y, z, cnt, stream)
            torch.cuda.synchronize()
            f.status()
            i.status()
            # the first and last polynomials (different chunks of the two-pass
            # schedules) against the exact transform / the oracle; every
            # polynomial's round trip n x
            for k in (0, cnt - 1):
                if fl:
                    assert np.array_equal(y[k:k + 1].cpu().numpy().astype(np.int64),
                                          oracle.ntt_exact(x[k:k + 1], q, root)), tag
                else:
                    assert np.array_equal(y[k:k + 1].cpu().numpy(),
                                          oracle.Plan(oracle.R2_I32_FWD, n, q, root)(x[k:k + 1])), tag
            assert np.array_equal(z.cpu().numpy().astype(np.int64) % q, (x.astype(np.int64) * n) % q), tag
            for d, pl, src, dst in (("fwd", f, dx, y), ("inv", i, y, z)):
                c0 = gb.launch_count()
                pl.execute(src, dst, cnt, stream)
                launches = gb.launch_count() - c0
                ms = timed(lambda: pl.execute(src, dst, cnt, stream), 20)
                key = f"{tag}_r2_i32_{d}_n2^{L}_{cnt}_{name}"
                out[key] = entry(cnt, cnt * n, nb, ms, launches)
                if fl:
                    kern = ("four-step: k_ccols (TMA column pass) + k_crows (twist, row pass)" if L >= 16
                            else "k_ntt (one CTA per polynomial)")
                    out[key]["roofline"] = roofline(key, nb, ms, kern)
    return out


SERVE_Q32 = [(998244353, 3), (469762049, 3), (167772161, 3), (754974721, 11)]   # (q, generator)


def run_serving(gb, seconds, arith="canonical"):
    """Serving loop over a stream of single-polynomial requests.

    n = 2^U with U uniform in {8..16}, forward/inverse 50/50, int16 (q = 12289)
    or int32 (four NTT primes) 50/50.  q = 12289 has no root of unity of order
    above 4096 and no int16-storable prime below the lazy-reduction bound has
    one of order 8192, so int16 requests draw U again from {8..12}.  Host
    buffers are pinned.  A saturating burst measures the capacity; open-loop
    Poisson arrivals at 50%, 90% and 100% of it give p50/p99 latency (submit to
    result in host memory).  A sample of requests is checked against the same
    transform launched alone.  The plans compute the headline's arithmetic."""
    import torch

    rng = np.random.default_rng(SEED + 1)
    fl = gb.FLAG_CANONICAL if arith == "canonical" else 0
    plans, keys = [], {}
    for inv in (0, 1):
        for L in range(8, 13):
            n = 1 << L
            keys[(16, 12289, L, inv)] = len(plans)
            plans.append(gb.Plan(gb.Kind.R2_I16_INV if inv else gb.Kind.R2_I16_FWD, n, 12289, pow(41, 4096 // n, 12289),
                                 0, fl))
        for q, g in SERVE_Q32:
            for L in range(8, 17):
                n = 1 << L
                keys[(32, q, L, inv)] = len(plans)
                plans.append(gb.Plan(gb.Kind.R2_I32_INV if inv else gb.Kind.R2_I32_FWD, n, q, pow(g, (q - 1) // n, q),
                                     0, fl))
    pool = {}      # (dtype bits, q, L) -> pinned input polynomials
    for (bits, q, L, inv) in keys:
        if (bits, q, L) not in pool:
            dt = np.int16 if bits == 16 else np.int32
            pool[(bits, q, L)] = torch.from_numpy(rng.integers(0, q, (4, 1 << L)).astype(dt)).pin_memory()
    ring = 8
    outs = {k: torch.empty((ring,) + v.shape[1:], dtype=v.dtype).pin_memory() for k, v in pool.items()}

    def draw(nreq):
        bits = rng.integers(0, 2, nreq)
        U = rng.integers(8, 17, nreq)
        U16 = rng.integers(8, 13, nreq)
        inv = rng.integers(0, 2, nreq)
        qi = rng.integers(0, len(SERVE_Q32), nreq)
        idx, ins, outl, nbytes = [], [], [], 0
        for k in range(nreq):
            if bits[k] == 0:
                key = (16, 12289, int(U16[k]))
            else:
                key = (32, SERVE_Q32[qi[k]][0], int(U[k]))
            idx.append(keys[key + (int(inv[k]),)])
            ins.append(pool[key][k % 4])
            outl.append(outs[key][k % ring])
            nbytes += 2 * (1 << key[2]) * (key[0] // 8)
        return idx, ins, outl, nbytes

    srv = gb.Server(plans, slots=8)
    # alone-vs-mix: a mixed burst with distinct output buffers, each checked against a lone launch
    idx, ins, _, _ = draw(256)
    own = [torch.empty_like(x).pin_memory() for x in ins]
    for t in srv.submit_schedule(idx, ins, own, [1] * len(idx), [0.0] * len(idx)):
        srv.wait(t)
    for i, x, y in zip(idx, ins, own):
        assert torch.equal(plans[i](x.unsqueeze(0).cuda()).cpu()[0], y), "served result differs from a lone launch"

    def run(nreq, arrivals):
        srv.stats(reset=True)
        idx, ins, outl, nbytes = draw(nreq)
        srv.submit_schedule(idx, ins, outl, [1] * nreq, arrivals)
        srv.drain()
        st = srv.stats()
        assert st["completed"] == nreq and st["refused"] == 0
        # the server's own clock: first arrival to last completion (single-polynomial requests)
        el = nreq / st["polys_per_s"]
        return st, el, nbytes

    run(5000, [0.0] * 5000)                                         # warm-up
    nsat = 50000
    st, el, nbytes = run(nsat, [0.0] * nsat)
    cap = nsat / el
    out = {"workload": "single-polynomial requests: n=2^U, U~{8..16} (int16: {8..12}), fwd/inv 50/50, "
                       "int16 q=12289 / int32 q in {998244353,469762049,167772161,754974721} 50/50",
           "plans": len(plans), "slots": 8, "api": "gbntt_server_* (pinned host buffers)", "arithmetic": arith,
           "alone_vs_mix_checked": 256,
           "saturation": {"requests_per_s": cap, "NTT_per_s": cap, "algorithmic_GBps": nbytes / el / 1e9,
                          "requests": nsat, "microbatches": st["microbatches"], "launches": st["launches"],
                          "p50_us": st["p50_us"], "p99_us": st["p99_us"]}}
    for frac in (0.5, 0.9, 1.0):
        rate = frac * cap
        nreq = int(min(200000, max(1000, rate * seconds)))
        arrivals = np.cumsum(rng.exponential(1e6 / rate, nreq)).tolist()
        st, el, nbytes = run(nreq, arrivals)
        out[f"poisson_{int(frac * 100)}"] = {
            "offered_requests_per_s": rate, "achieved_requests_per_s": nreq / el, "requests": nreq,
            "p50_us": st["p50_us"], "p99_us": st["p99_us"], "max_us": st["max_us"],
            "microbatches": st["microbatches"], "launches": st["launches"],
            "peak_arena_bytes": st["peak_arena_bytes"]}
    srv.close()
    return out


PROFILE_CASES = {
    # name: (kind, n, q, root, polys) -- a few hundred MiB, inputs larger than L2
    "r4_1024": (2, 1024, 12289, 11580, 65536),
    "r2f16_1024": (0, 1024, 12289, 11580, 65536),
    "r2i16_1024": (1, 1024, 12289, 11580, 65536),
    "r2f32_4096": (4, 4096, 998244353, 63912897, 16384),
    "r2g32_4096": (5, 4096, 998244353, 63912897, 16384),
    "r8_4096": (8, 4096, 12289, 41, 16384),
    "r2f32_1m": (4, 1 << 20, 998244353, 565042129, 64),
    "r2g32_1m": (5, 1 << 20, 998244353, 565042129, 64),
    "r2f32_16k": (4, 1 << 14, 998244353, 666702199, 4096),
    # canonical families (GBNTT_FLAG_CANONICAL)
    "c_r4_1024": (2, 1024, 12289, 11580, 65536, 1),
    "c_r2f16_1024": (0, 1024, 12289, 11580, 65536, 1),
    "c_r2i16_1024": (1, 1024, 12289, 11580, 65536, 1),
    "c_r2f32_4096": (4, 4096, 998244353, 63912897, 16384, 1),
    "c_r2f16_256": (0, 256, 12289, pow(41, 16, 12289), 262144, 1),
    "c_r2i16_256": (1, 256, 12289, pow(41, 16, 12289), 262144, 1),
    "c_r2g32_4096": (5, 4096, 998244353, 63912897, 16384, 1),
    "c_r2f32_16k": (4, 1 << 14, 998244353, 666702199, 4096, 1),
    "c_r2g32_16k": (5, 1 << 14, 998244353, 666702199, 4096, 1),
    "c_r2f32_32k": (4, 1 << 15, 998244353, pow(3, (998244353 - 1) >> 15, 998244353), 2048, 1),
    "c_r2f32_1m": (4, 1 << 20, 998244353, 565042129, 64, 1),
    "c_r2g32_1m": (5, 1 << 20, 998244353, 565042129, 64, 1),
    "c_r2f32_64k": (4, 1 << 16, 998244353, pow(3, (998244353 - 1) >> 16, 998244353), 1024, 1),
    # the stand-alone units (HBM-bound): bit reversal, full Barrett multiplication by n^-1
    "bitrev_4096": (6, 4096, 12289, 0, 65536),
    "fullbarrett_4096": (7, 4096, 12289, 0, 65536),
    "r8stage_4096": (3, 4096, 12289, 41, 65536),
    "batch_r4": None,   # the benchmark batch, 4x larger, persistent kernel
    "c_batch_r4": None,  # the same with GBNTT_FLAG_CANONICAL
}


def run_profile_batch(scale=4, launches=3, flags=0):
    """The benchmark's batch with every segment `scale` times larger (inputs
    larger than L2), executed `launches` times as one persistent launch."""
    import torch

    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    rng = np.random.default_rng(SEED)
    plans, xs, ys = [], [], []
    for q, n, cnt, g in SEGMENTS:
        plans.append(gb.Plan(gb.Kind.R4_I16_FWD, n, q, root_of(q, n, g), 0, flags))
        xs.append(torch.from_numpy(rng.integers(0, q, (cnt * scale, n)).astype(np.int16)).cuda())
        ys.append(torch.empty_like(xs[-1]))
    batch = gb.Batch(list(zip(plans, xs, ys)))
    for _ in range(launches):
        batch.execute()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    batch.execute()
    b.record()
    torch.cuda.synchronize()
    batch.status()
    ms = a.elapsed_time(b)
    nbytes = sum(2 * x.numel() * 2 for x in xs)
    print(json.dumps({"case": f"batch_x{scale}", "flags": flags, "el": batch.query(4), "cta_per_sm_cfg": None,
                      "polys": sum(x.shape[0] for x in xs), "ms": ms,
                      "algorithmic_GBps": nbytes / (ms / 1e3) / 1e9}))


def run_profile_case(name, launches=3):
    """One design on one large batch, `launches` times (for ncu captures)."""
    import torch

    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    if name == "batch_r4":
        return run_profile_batch(4, launches)
    if name == "c_batch_r4":
        return run_profile_batch(4, launches, flags=1)
    kind, n, q, root, polys, *fl = PROFILE_CASES[name]
    factor = pow(n, -1, q) if kind == 7 else 0        # the full Barrett unit multiplies by n^-1
    plan = gb.Plan(kind, n, q, root, factor, fl[0] if fl else 0)
    dt = torch.int32 if plan.elem_bytes == 4 else torch.int16
    g = torch.Generator(device="cuda").manual_seed(SEED)
    x = torch.randint(0, q, (polys, n), dtype=torch.int64, device="cuda", generator=g).to(dt)
    y = torch.empty_like(x)
    for _ in range(launches):
        plan(x, out=y)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    plan(x, out=y)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    nbytes = 2 * x.numel() * x.element_size()
    print(json.dumps({"case": name, "kind": kind, "n": n, "q": q, "polys": polys, "ms": ms,
                      "algorithmic_GBps": nbytes / (ms / 1e3) / 1e9}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--arith", choices=["canonical", "lanes"], default="canonical",
                    help="outputs of the timed workload: canonical residues (default) or the reference's "
                         "partially reduced lanes")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-per-ntt", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--skip-configs", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=1.5)
    ap.add_argument("--profile", choices=sorted(PROFILE_CASES), default=None,
                    help="run one design on a large batch (for ncu captures) instead of the benchmark")
    args = ap.parse_args()
    if args.profile:
        run_profile_case(args.profile)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
