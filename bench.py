"""Benchmark: n=40 hafnians/s on one GB300 (or N GPUs as independent shards).

Workload: the plain Glynn hafnian of a 40x40 complex128 symmetric matrix A = (G + G^T)/2,
Re G, Im G ~ N(0, 1/2) iid, seed 0 (524,288 sieve terms).  One step = one hafnian.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|df|dd] [--impl gb300|reference]

value    : hafnians/s with the input resident in HBM (device time of the sieve + reduction
           launches, CUDA events on the launching stream, L2 flushed between steps), summed
           over ranks (each rank runs its own shard of hafnians: weak scaling).
e2e      : the same metric through the public API thewalrus_gb300.hafnian(A) from host NumPy
           input: host preparation, host->device upload, kernels, device->host result.
roofline : algorithmic flops of the sieve (thewalrus_gb300.costmodel) / mean device time,
           against the FP64 (or, for df, FP32) FMA-pipe peak measured in the same run.
cpu_baseline : the CPU oracle (a C restatement of the reference algorithm: mixed-radix term
           order, power traces by repeated matrix products) on all host cores, timed on a
           bounded sample of the same hafnian's terms and scaled to hafnians/s.
rel_err_vs_reference : the result against the value the reference's own code produced for the
           same input (committed fixture), and against the long-double oracle.
loop, batch, serve : (one GPU, default workload) the 40-photon loop hafnian of a 20-mode
           Gaussian state (FP64 rate, and the error of FP64, double-double and precision="auto"
           against its _Float128 value: loop_summary), the batched form on a stated subset of the
           4,096-instance workload and the served form at two arrival rates, each against one
           call per instance and checked against the oracle (see batch_summary, serve_summary).
--impl reference : that CPU restatement alone, as the reference arm (rank 0 only), on whole
           hafnians.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MATRIX = 40
METRIC = "n=40 hafnians/s (complex128, Glynn sieve)"
UNIT = "hafnians/s"
# The published wall time of one 40x40 complex hafnian (thewalrus hafnian tutorial, 4 threads of
# an AMD A12-9800, the library's earlier C++ implementation): vs_baseline = value x 41.32 s.
PUBLISHED_N40_SECONDS = 41.32


def workload(n=N_MATRIX, matrix="complex"):
    from thewalrus_gb300 import workloads as wl

    return wl.complex_symmetric(n, seed=0) if matrix == "complex" else wl.real_signed(n, seed=0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_sample(seconds=12.0, threads=None):
    """Time the CPU oracle on terms [0, S) of the n=40 sieve; returns (hafnians/s, info)."""
    import numpy as np

    import oracle

    threads = threads or os.cpu_count() or 1
    A = workload()
    x, reps, _ = oracle.matched_reps([1] * N_MATRIX)
    Ax = A[np.ix_(x, x)]
    total_terms = 2 ** (N_MATRIX // 2 - 1)
    probe = 4 * threads
    t0 = time.perf_counter()
    oracle.haf_term_range(Ax, reps, 0, probe, nthreads=threads)
    dt = time.perf_counter() - t0
    S = int(min(total_terms, max(probe, probe * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    oracle.haf_term_range(Ax, reps, 0, S, nthreads=threads)
    dt = time.perf_counter() - t0
    rate = S / dt / total_terms
    info = {"terms": S, "seconds": dt, "threads": threads, "total_terms": total_terms}
    return rate, info


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sms.append(float(parts[1]))
                    maxes.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if sms:
            out = {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes),
                   "reasons": sorted(reasons), "samples": len(sms)}
        return out


def run_reference(args, rank, world):
    """The reference arm: whole n=40 hafnians by the CPU restatement of the reference algorithm
    on all host cores.  One hafnian takes ~28 s on 16 cores, so at most ``BENCH_REF_STEPS``
    (default 3) whole hafnians are timed, whatever ``--steps`` asks, and no warm-up runs (a C
    library has no JIT to warm); the line states both."""
    if rank != 0:
        return
    import numpy as np

    import oracle

    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, int(os.environ.get("BENCH_REF_STEPS", "3"))))
    A = workload()
    secs = []
    result = None
    for _ in range(steps):
        t0 = time.perf_counter()
        result = complex(oracle.hafnian(A, nthreads=threads))
        secs.append(time.perf_counter() - t0)
    value = steps / sum(secs)
    sample = ("%d whole hafnians (all %d sieve terms each), C restatement of the reference algorithm "
              "(mixed-radix terms, matrix-power traces; double, %d threads)" % (steps, 2 ** (N_MATRIX // 2 - 1),
                                                                                 threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": 1e3 * sum(secs) / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": value * PUBLISHED_N40_SECONDS, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "hafnian 40x40 complex128 (G+G^T)/2, seed 0, 524288 sieve terms",
                   "precision": "fp64", "parallelism": "%d host threads" % threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "result": [result.real, result.imag],
    }
    ref = metric_reference("haf40_complex")
    if ref is not None:
        line["rel_err_vs_reference"] = abs(result - ref[0]) / abs(ref[0])
    print(json.dumps(line), flush=True)


def metric_reference(case):
    """(value the reference's own code produced, long-double oracle value) for a benchmark input,
    from the committed fixture tests/golden/metric_cases.npz; None when the fixture is absent."""
    import numpy as np

    path = os.path.join(ROOT, "tests", "golden", "metric_cases.npz")
    if not os.path.exists(path):
        return None
    data = np.load(path)
    if case + "/out" not in data.files:
        return None
    ld = data[case + "/oracle_ld"] if case + "/oracle_ld" in data.files else None
    return complex(data[case + "/out"]), (None if ld is None else complex(ld))


def run_gpu(args, rank, world, local):
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import thewalrus_gb300 as tw
    from thewalrus_gb300 import _native as nat
    from thewalrus_gb300 import costmodel

    nat.check(nat.load().wg_init(local))
    n = args.n
    A = workload(n, args.matrix)
    inst = tw.prepare_hafnian(A)
    plan = nat.Plan([inst], precision=args.precision)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    fp64_peak, fp32_peak = nat.measure_fp_peaks()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        plan.execute(sptr)
    torch.cuda.synchronize()
    result = plan.read(sptr)[0]

    clocks = ClockSampler(local)
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        plan.execute(sptr)
        e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms * 1e-3)

    # end to end through the public API: host prep + upload + kernels + result download
    for _ in range(min(args.warmup, 2)):
        tw.hafnian(A, precision=args.precision)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = tw.hafnian(A, precision=args.precision)
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * args.steps / e2e_s
    h2d, d2h = plan.transfer_bytes()

    flops = costmodel.plain_hafnian_flops(n, complex_input=args.matrix == "complex")
    mean_s = total_ms / args.steps * 1e-3
    achieved = flops / mean_s / 1e12
    peak = fp32_peak if args.precision == "df" else fp64_peak  # double-double runs on the FP64 pipe
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": (value * PUBLISHED_N40_SECONDS if n == N_MATRIX else None),
        "dtype": {"fp64": "f64", "df": "df32", "dd": "dd64"}[args.precision],
        "data": "synthetic",
        "config": {"workload": "hafnian %dx%d %s, seed 0, %d sieve terms"
                               % (n, n, "complex128 (G+G^T)/2" if args.matrix == "complex"
                                  else "float64 (G+G^T)/2, G ~ N(0,1)", 2 ** (n // 2 - 1)),
                   "precision": args.precision, "parallelism": "shard-per-gpu" if world > 1 else "1 gpu",
                   "l2": "flushed between steps (256 MiB write, outside the timed events)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "fp32" if args.precision == "df" else "fp64",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "traffic_note": "DRAM bytes need an ncu capture, not taken inside the bench",
                     "peak_source": "FMA-pipe microbenchmark (wg_measure_fp_peaks) in this run",
                     "flops_per_launch": flops},
        "gpu_launches": args.steps * plan.kernel_launches,
        "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
        "result": [float(np.real(result)), float(np.imag(result))],
        "e2e_result_matches": bool(abs(r - result) <= 1e-12 * abs(result)),
    }
    if n != N_MATRIX or args.matrix != "complex":
        line["metric"] = "n=%d hafnians/s (%s, Glynn sieve)" % (
            n, "complex128" if args.matrix == "complex" else "float64")
    ref = metric_reference("haf40_complex" if args.matrix == "complex" else "haf40_real") if n == N_MATRIX else None
    if ref is not None:
        line["rel_err_vs_reference"] = abs(complex(result) - ref[0]) / abs(ref[0])
        if ref[1] is not None:
            line["rel_err_vs_oracle_ld"] = abs(complex(result) - ref[1]) / abs(ref[1])
        line["e2e_rel_err_vs_reference"] = abs(complex(r) - ref[0]) / abs(ref[0])
    if not args.no_cpu_baseline and n == N_MATRIX and args.matrix == "complex":
        rate, info = cpu_sample(seconds=args.cpu_seconds)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": info["threads"], "kind": "port",
            "sample": "terms [0, %d) of the %d-term sieve in %.1f s, C restatement of the reference "
                      "algorithm in double on %d threads" % (info["terms"], info["total_terms"],
                                                             info["seconds"], info["threads"])}
    plan.close()
    if world == 1 and not args.no_extras and n == N_MATRIX and args.matrix == "complex":
        line["loop"] = loop_summary("fp64", 20, 3, extra_precisions=("dd", "auto"))
        line["batch"] = batch_summary(args)
        line["serve"] = serve_summary(args)
    print(json.dumps(line), flush=True)


def batch_summary(args):
    """Batching (a stated subset of the 4096-instance workload): every 16th of the 4096 uneven
    instances (n in 8..40, half real non-negative, half complex) plus the 16 loop_hafnian_batch
    calls (12 modes, cutoff 6), as one autotuned, graph-replayed plan against the same instances
    through the public API one call each; accuracy of the batched results against the
    long-double oracle on the members with n <= 20."""
    import numpy as np
    import torch

    import oracle
    import thewalrus_gb300 as tw
    from thewalrus_gb300 import _native as nat, autotune, workloads as wl

    mats = wl.batch_instances(count=4096, seed=2)[::16]
    calls = wl.batch_loop_calls(count=16, seed=3, modes=12, cutoff=6)
    insts = [tw.prepare_hafnian(A) for A in mats] + \
        [tw.prepare_loop_hafnian_batch(B, D, list(f), c) for B, D, f, c in calls]
    cands = [{"chunk_scale": cs, "max_warps_per_cta": 0, "merge_classes": mc, "serial_groups": False}
             for cs in (1.0, 2.0, 4.0) for mc in (False, True)]
    t0 = time.perf_counter()
    best, _ = autotune.tune(insts[::4], precision="fp64", candidates=cands, repeats=1, use_cache=False)
    tune_s = time.perf_counter() - t0
    plan = nat.Plan(insts, precision="fp64", use_graph=True, **best)
    s = torch.cuda.current_stream()
    plan.execute(s.cuda_stream)  # captures the graph
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        plan.execute(s.cuda_stream)
        e1.record(s)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    batched_s = statistics.median(times)
    got = plan.read(s.cuda_stream)
    plan.close()
    outputs = len(mats) + sum(int(c) + 1 for _, _, _, c in calls)
    t0 = time.perf_counter()
    per = [tw.hafnian(A, precision="fp64") for A in mats]
    per_b = [tw.loop_hafnian_batch(B, D, list(f), c, precision="fp64") for B, D, f, c in calls]
    per_call_s = time.perf_counter() - t0
    diff = max(abs(per[i] - got[i]) / abs(per[i]) for i in range(len(mats)))
    off = len(mats)
    for b in per_b:
        diff = max(diff, float(np.max(np.abs(b - got[off:off + len(b)])) / np.max(np.abs(b))))
        off += len(b)
    err = 0.0
    checked = 0
    for i, A in enumerate(mats):
        if len(A) <= 20:
            want = complex(oracle.hafnian(A, precision="long"))
            err = max(err, abs(got[i] - want) / abs(want))
            checked += 1
    return {"workload": "every 16th of the 4096 uneven hafnians (%d, n in 8..40) + 16 loop_hafnian_batch "
                        "(12 modes, cutoff 6; %d outputs): one autotuned plan, CUDA-graph replay" % (len(mats), outputs - len(mats)),
            "hafnians_per_s": outputs / batched_s, "seconds": batched_s,
            "per_call_hafnians_per_s": outputs / per_call_s, "per_call_seconds": per_call_s,
            "speedup_vs_per_call": per_call_s / batched_s,
            "max_rel_diff_vs_per_call": diff, "max_rel_err_vs_oracle_ld": err, "oracle_checked": checked,
            "autotuned": best, "autotune_seconds": tune_s, "kernel_launches": plan.kernel_launches}


def serve_summary(args):
    """Serving (Poisson streams of probability requests on four 64-mode Gaussian states, patterns
    of 8-44 photons, at most 2 per mode): p50/p99 latency and hafnians/s at two arrival rates with
    ``--serve-count`` requests each (the same requests, arrival times scaled), admitted cheapest
    first; the higher rate's requests also admitted oldest first, and one call each (matrices
    formed on the device, one plan per request, synchronous); loop hafnians of the requests with
    at most 24 photons against the long-double oracle."""
    import numpy as np

    import oracle
    from thewalrus_gb300 import _native as nat
    from thewalrus_gb300._hafnian import matched_reps
    from thewalrus_gb300.serving import GaussianState, ProbabilityServer, poisson_requests, summary

    states = [GaussianState.synthetic(modes=64, seed=s) for s in range(4)]
    srv = ProbabilityServer(states, precision="fp64", max_batch=256, streams=args.serve_streams)
    srv.serve(poisson_requests(states, 1e6, 16, photons=(8, 16), seed=99))  # warm-up
    rows = []
    err, checked = 0.0, 0
    for rate in args.serve_rates:
        # one seed for every rate: the same requests (states, patterns), arrival times scaled by 1/rate
        reqs = poisson_requests(states, rate, args.serve_count, photons=(8, 44), seed=7)
        t0 = time.perf_counter()
        res = srv.serve(reqs)
        span = time.perf_counter() - t0
        sm = summary(res, makespan=span)
        sm["rate"] = rate
        rows.append(sm)
        for (t, sidx, pat), r in zip(reqs, res):
            if np.sum(pat) <= 24 and checked < 64:
                st = states[sidx]
                want = complex(oracle.hafnian_repeated(st.B, list(pat), mu=st.gamma, loop=True, precision="long"))
                lhaf = r["amplitude"] / st.norm(pat)
                err = max(err, abs(lhaf - want) / abs(want))
                checked += 1
    # the same requests at the top rate, admitted oldest first (no cost ordering) for contrast
    fifo = ProbabilityServer(states, precision="fp64", max_batch=256, streams=args.serve_streams, order="arrival")
    t0 = time.perf_counter()
    res = fifo.serve(reqs)
    arrival = summary(res, makespan=time.perf_counter() - t0)
    arrival["rate"] = args.serve_rates[-1]
    done = 0
    t0 = time.perf_counter()
    for _, sidx, pat in reqs:
        if states[sidx].trivial_loop_hafnian(pat) is not None:
            continue
        plan = nat.Plan.from_requests(states[sidx].device, [matched_reps(pat)], "fp64")
        plan.execute()
        plan.read()
        plan.close()
        done += 1
    srv.torch.cuda.synchronize()
    per_call_s = time.perf_counter() - t0
    return {"workload": "%d requests per rate, Poisson arrivals, 4 synthetic 64-mode pure states, 8-44 photons"
                        % args.serve_count,
            "admission": "cheapest first, batches closed at ~25 ms of GPU work",
            "rates": rows, "arrival_order_at_top_rate": arrival,
            "per_call": {"requests": done, "seconds": per_call_s, "hafnians_per_s": done / per_call_s,
                                        "same_requests_as_rate": args.serve_rates[-1]},
            "max_rel_err_vs_oracle_ld": err, "oracle_checked": checked}


def _gpu_setup(local=0):
    import torch

    torch.cuda.set_device(local)
    from thewalrus_gb300 import _native as nat

    nat.check(nat.load().wg_init(local))
    return torch, nat


def loop_summary(precision, steps, warmup, extra_precisions=()):
    """Loop hafnian of the 20-mode Gaussian-state reduced matrix (40 photons, repeats <= 3):
    hafnian_repeated(A, rpt, mu=gamma, loop=True), device time per call and end to end, the error
    against the committed _Float128 value, the sum's condition number, and (extra_precisions) the
    error of one call in each further precision ("dd", "auto")."""
    import numpy as np
    import torch

    from thewalrus_gb300 import _native as nat
    import thewalrus_gb300 as tw
    from thewalrus_gb300 import costmodel, workloads as wl

    # the committed fixture holds this input as generated for the reference run (the Haar unitary
    # comes from a QR factorisation, whose last bits differ between LAPACK builds, and this sum
    # amplifies input differences ~1e10-fold); the generator is the fallback
    path = os.path.join(ROOT, "tests", "golden", "metric_cases.npz")
    truth = None
    if os.path.exists(path):
        fx = np.load(path)
        A, gamma, rpt = fx["lhaf_state20_40/A"], fx["lhaf_state20_40/mu"], fx["lhaf_state20_40/rpt"]
        truth = complex(fx["lhaf_state20_40/oracle_q"])
    else:
        A, gamma, rpt = wl.gaussian_state_loop(modes=20, seed=1, photons=40, max_rep=3)
    inst = tw.prepare_loop_hafnian(A, gamma, list(rpt))
    plan = nat.Plan([inst], precision=precision)
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        plan.execute(s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        plan.execute(s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    plan.close()
    dev_s = e0.elapsed_time(e1) / 1e3 / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        val = tw.hafnian_repeated(A, list(rpt), mu=gamma, loop=True, precision=precision)
    e2e_s = (time.perf_counter() - t0) / steps
    x, reps, odd = tw.matched_reps(list(rpt))
    flops = costmodel.instance_flops(reps, True, kind="loop", odd=odd is not None)
    line = {"metric": "loop hafnians/s (20-mode Gaussian state, 40 photons)", "value": 1 / dev_s,
            "unit": "hafnians/s", "ms_per_step": dev_s * 1e3, "e2e": {"value": 1 / e2e_s, "unit": "hafnians/s"},
            "edge_reps": [int(r) for r in reps], "terms": int(np.prod([r + 1 for r in reps]) // 1),
            "achieved_tflops": flops / dev_s / 1e12, "precision": precision,
            "result": [float(val.real), float(val.imag)]}
    # accuracy against the committed _Float128 value, and the sum's condition number
    if truth is not None:
        line["rel_err_vs_float128"] = abs(complex(val) - truth) / abs(truth)
    vals, mags = tw.run_with_magnitudes([inst], "fp64")
    line["sum_abs_terms_over_abs_sum"] = float(mags[0] / abs(vals[0]))
    for p in extra_precisions:
        t0 = time.perf_counter()
        v = complex(tw.hafnian_repeated(A, list(rpt), mu=gamma, loop=True, precision=p))
        sec = time.perf_counter() - t0
        line[p] = {"seconds": sec, "rel_err_vs_float128": abs(v - truth) / abs(truth) if truth is not None else None}
    return line


def run_loop(args):
    """The loop hafnian line on its own (``--workload loop``)."""
    _gpu_setup()
    print(json.dumps(loop_summary(args.precision, args.steps, args.warmup)), flush=True)


def run_batch(args):
    """4096 hafnians of uneven even n in {8..40} (half real non-negative, half complex) plus 16
    loop_hafnian_batch calls (12 modes, cutoff 6) in one autotuned, graph-replayed plan, against
    per-call launches of the same instances (a bounded sample of them)."""
    torch, nat = _gpu_setup()
    import thewalrus_gb300 as tw
    from thewalrus_gb300 import autotune, workloads as wl

    count = args.batch_count
    mats = wl.batch_instances(count=count, seed=2)
    calls = wl.batch_loop_calls(count=16, seed=3, modes=12, cutoff=6)
    insts = [tw.prepare_hafnian(A) for A in mats] + \
        [tw.prepare_loop_hafnian_batch(B, D, list(f), c) for B, D, f, c in calls]
    sub = insts[::16]
    cands = [{"chunk_scale": cs, "max_warps_per_cta": 0, "merge_classes": mc, "serial_groups": sg}
             for cs in (1.0, 2.0, 4.0) for mc in (False, True) for sg in (False, True)]
    best, table = autotune.tune(sub, precision=args.precision, candidates=cands, repeats=1, use_cache=False)
    plan = nat.Plan(insts, precision=args.precision, use_graph=True, **best)
    s = torch.cuda.current_stream()
    plan.execute(s.cuda_stream)  # first execution captures the graph
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    plan.execute(s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    batched_s = e0.elapsed_time(e1) / 1e3
    got = plan.read(s.cuda_stream)
    # per-call plain launches on a deterministic sample (every 32nd instance), same accuracy
    sample = list(range(0, len(mats), 32))
    t0 = time.perf_counter()
    per = [tw.hafnian(mats[i], precision=args.precision) for i in sample]
    per_call_s = time.perf_counter() - t0
    idx_sum = 0
    err = 0.0
    for k, i in enumerate(sample):
        err = max(err, abs(per[k] - got[i]) / abs(per[k]))
        idx_sum += 1
    # the same sample as one batched plan (same options), timed on the device
    pplan = nat.Plan([insts[i] for i in sample], precision=args.precision, use_graph=True, **best)
    pplan.execute(s.cuda_stream)
    torch.cuda.synchronize()
    e0.record(s)
    pplan.execute(s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    sample_batched_s = e0.elapsed_time(e1) / 1e3
    outputs = len(mats) + 16
    # contrast: many small instances (n in 8..20), where per-call launch and host overheads dominate
    small = wl.batch_instances(count=count, seed=4, n_min=8, n_max=20)
    splan = nat.Plan([tw.prepare_hafnian(A) for A in small], precision=args.precision, use_graph=True)
    splan.execute(s.cuda_stream)
    torch.cuda.synchronize()
    e0.record(s)
    splan.execute(s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    small_batched_s = e0.elapsed_time(e1) / 1e3
    sgot = splan.read(s.cuda_stream)
    ssample = list(range(0, len(small), 16))
    t0 = time.perf_counter()
    sper = [tw.hafnian(small[i], precision=args.precision) for i in ssample]
    small_per_call_s = (time.perf_counter() - t0) / len(ssample)
    small_err = max(abs(sper[k] - sgot[i]) / abs(sper[k]) for k, i in enumerate(ssample))
    print(json.dumps({
        "metric": "batched hafnians/s (4096 uneven n in 8..40 + 16 loop_hafnian_batch, one plan)",
        "value": outputs / batched_s, "unit": "hafnians/s", "seconds": batched_s,
        "per_call": {"hafnians_per_s": len(sample) / per_call_s, "sample": len(sample),
                     "batched_same_sample_hafnians_per_s": len(sample) / sample_batched_s},
        "max_rel_diff_batched_vs_per_call": err, "autotuned": best,
        "autotune_table": [[c, t] for c, t in table], "kernel_launches": plan.kernel_launches,
        "graph": True, "precision": args.precision,
        "small_n": {"instances": len(small), "n_range": [8, 20], "batched_hafnians_per_s": len(small) / small_batched_s,
                    "per_call_hafnians_per_s": 1.0 / small_per_call_s, "per_call_sample": len(ssample),
                    "max_rel_diff_batched_vs_per_call": small_err}}), flush=True)


def run_serve(args):
    """Poisson streams of probability requests on 64-mode synthetic pure Gaussian states; rates
    swept; p50/p99 latency and hafnians/s per rate."""
    _gpu_setup()
    from thewalrus_gb300.serving import GaussianState, ProbabilityServer, poisson_requests, summary

    states = [GaussianState.synthetic(modes=64, seed=s) for s in range(4)]
    srv = ProbabilityServer(states, precision=args.precision, max_batch=256, streams=args.serve_streams)
    lo, hi = args.photons
    srv.serve(poisson_requests(states, 1e6, 8, photons=(lo, min(hi, lo + 8)), seed=99))  # warm-up
    rows = []
    for rate in args.rates:
        reqs = poisson_requests(states, rate, args.serve_count, photons=(lo, hi), seed=7)
        t0 = time.perf_counter()
        res = srv.serve(reqs)
        span = time.perf_counter() - t0
        sm = summary(res, makespan=span)
        sm["rate"] = rate
        rows.append(sm)
    # per-call baseline: the last rate's requests one at a time (same device-formed matrices, one
    # plan each, synchronous), against the served makespan of the same set
    import numpy as np
    from thewalrus_gb300 import _native as nat
    from thewalrus_gb300._hafnian import matched_reps

    torch = srv.torch
    done = 0
    t0 = time.perf_counter()
    for _, sidx, pat in reqs:
        if states[sidx].trivial_loop_hafnian(pat) is not None:
            continue
        plan = nat.Plan.from_requests(states[sidx].device, [matched_reps(pat)], args.precision)
        plan.execute()
        plan.read()
        plan.close()
        done += 1
    torch.cuda.synchronize()
    per_call_s = time.perf_counter() - t0
    served = rows[-1]
    print(json.dumps({"metric": "served loop-hafnian probabilities (64-mode states, %d-%d photons)" % (lo, hi),
                      "unit": "hafnians/s", "precision": args.precision, "sweep": rows,
                      "per_call": {"requests": done, "seconds": per_call_s, "hafnians_per_s": done / per_call_s,
                                   "served_at_rate": served["rate"],
                                   "served_hafnians_per_s": served["hafnians_per_s"]}}), flush=True)


def run_precision(args):
    """Precision of the three term arithmetics: FP64, FP32 double-float and FP64 double-double.

    * n = 20 (``--precision-n``), ``--precision-seeds`` seeds per class: against the _Float128
      oracle.
    * n = 48, the large-size table: random 0/1 graphs (edge probability 0.5, ``--precision-seeds48``
      seeds) and integer non-negative matrices (floor(|G| + |G|^T), entries 0..5; a quarter as
      many seeds) against their exact hafnians (the exact sieve over residues, pinned against
      the CPU modular oracle); signed real and complex matrices against the double-double sieve (pinned against the
      _Float128 oracle to the last bits of complex128 at n <= 20), ``--precision-dd-seeds`` seeds (half that for the
      complex class, whose double-double run takes minutes).  Times per hafnian per mode."""
    import numpy as np

    torch, nat = _gpu_setup()
    import oracle
    import thewalrus_gb300 as tw
    from thewalrus_gb300 import workloads as wl

    def stats(v):
        return {"max": float(np.max(v)), "median": float(np.median(v)), "seeds": len(v)}

    gens = {"complex": wl.complex_symmetric, "real_signed": wl.real_signed, "real_nonneg": wl.real_nonneg,
            "adjacency01": wl.adjacency01}
    small = {}
    for name, gen in gens.items():
        errs = {"fp64": [], "df": [], "dd": []}
        for seed in range(args.precision_seeds):
            A = gen(args.precision_n, seed=seed)
            ref = complex(oracle.hafnian(A, precision="quad"))
            for p in errs:
                g = tw.hafnian(A, precision=p)
                errs[p].append(abs(g - ref) / abs(ref) if ref != 0 else abs(g))
        small[name] = {p: stats(v) for p, v in errs.items()}

    def timed(A, p):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        v = tw.hafnian(A, precision=p)
        return complex(v), time.perf_counter() - t0

    n = 48
    large = {}
    classes = [("adjacency01", lambda sd: wl.adjacency01(n, seed=sd), "exact", args.precision_seeds48),
               ("int_nonneg", lambda sd: np.floor(wl.real_nonneg(n, seed=sd)), "exact", args.precision_seeds48 // 4),
               ("real_signed", lambda sd: wl.real_signed(n, seed=sd), "dd", args.precision_dd_seeds),
               ("complex", lambda sd: wl.complex_symmetric(n, seed=sd), "dd", max(1, args.precision_dd_seeds // 2))]
    for name, gen, truth_mode, seeds in classes:
        errs = {"fp64": [], "df": []}
        secs = {"fp64": [], "df": [], truth_mode: []}
        rounds = 0
        for seed in range(seeds):
            A = gen(seed)
            truth, dt = timed(A, truth_mode)
            secs[truth_mode].append(dt)
            for p in errs:
                v, dt = timed(A, p)
                secs[p].append(dt)
                errs[p].append(abs(v - truth) / abs(truth))
                if truth_mode == "exact" and p == "fp64":
                    rounds += int(round(v.real) == truth.real)
        row = {"truth": truth_mode, **{p: stats(v) for p, v in errs.items()},
               "seconds_per_hafnian": {p: float(np.median(v)) for p, v in secs.items()}}
        if truth_mode == "exact":
            row["fp64_rounds_to_the_integer"] = rounds
        large[name] = row
    print(json.dumps({"metric": "relative error of FP64 / double-float / double-double sieve terms",
                      "n%d_vs_float128_oracle" % args.precision_n: small, "n48": large}), flush=True)


def run_sample(args):
    """Gaussian boson sampling by the chain rule on a synthetic 12-mode squeezed, displaced, lossy
    state: photon-number samples/s with all attempts in lockstep (one plan per mode), the same
    sampler one attempt at a time, threshold (click) samples/s, and the same chain on the CPU
    oracle for a bounded number of attempts."""
    import numpy as np

    _gpu_setup()
    from thewalrus_gb300 import samples as smp, workloads as wl

    M, cutoff = args.sample_modes, 5
    cov, mean = wl.gaussian_state_cov(M, seed=21)
    smp.hafnian_sample_state(cov, 4, mean=mean, cutoff=cutoff)  # warm-up
    np.random.seed(1)
    t0 = time.perf_counter()
    got = smp.hafnian_sample_state(cov, args.samples, mean=mean, cutoff=cutoff)
    lock_s = time.perf_counter() - t0
    photons = float(np.mean(np.sum(got, axis=1)))
    np.random.seed(2)
    seq = 16
    t0 = time.perf_counter()
    for _ in range(seq):
        smp.generate_hafnian_sample(cov, mean=mean, cutoff=cutoff, max_photons=30)
    seq_s = (time.perf_counter() - t0) / seq
    np.random.seed(3)
    t0 = time.perf_counter()
    thr = 16
    smp.torontonian_sample_state(cov, thr, mu=mean)
    thr_s = (time.perf_counter() - t0) / thr
    # CPU: the same chain with the oracle's loop_hafnian_batch, one attempt at a time
    import oracle
    chain = smp._Chain(cov, mean, 2)
    fac = np.array([math.factorial(k) for k in range(cutoff + 1)], dtype=float)
    np.random.seed(4)
    t0 = time.perf_counter()
    cpu_n = 0
    while time.perf_counter() - t0 < args.cpu_seconds:
        n_pure, n_het, u = chain.attempt_draws()
        het, gam = chain.start(n_pure, n_het)
        det = np.zeros(M, dtype=int)
        for mode in range(M):
            gam = gam - het[mode] * chain.B[:, mode]
            l = oracle.loop_hafnian_batch(chain.B[:mode + 1, :mode + 1], gam[:mode + 1], det[:mode], cutoff)
            p = (l * l.conj()).real / fac
            det[mode] = smp._choose(p / p.sum(), u[mode])
        cpu_n += 1
    cpu_s = (time.perf_counter() - t0) / cpu_n
    print(json.dumps({"metric": "GBS photon-number samples/s (%d-mode Gaussian state, cutoff %d)" % (M, cutoff),
                      "value": args.samples / lock_s, "unit": "samples/s", "samples": args.samples,
                      "mean_photons_per_sample": photons,
                      "one_attempt_at_a_time_samples_per_s": 1 / seq_s,
                      "threshold_samples_per_s": 1 / thr_s,
                      "cpu_baseline": {"value": 1 / cpu_s, "unit": "attempts/s", "kind": "port",
                                       "cores": int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1)),
                                       "sample": "%d attempts, oracle loop_hafnian_batch per mode" % cpu_n}}),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--n", type=int, default=N_MATRIX, help="matrix size (40 is the benchmark)")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", choices=["fp64", "df", "dd"], default="fp64")
    ap.add_argument("--matrix", choices=["complex", "real"], default="complex",
                    help="the n-x-n workload: complex symmetric (the benchmark) or real signed")
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batch and serve sub-objects of the default line")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[1000.0, 20000.0])
    ap.add_argument("--serve-streams", type=int, default=3, help="stream slots of the server")
    ap.add_argument("--workload", choices=["n40", "loop", "batch", "serve", "precision", "sample"], default="n40",
                    help="n40: the benchmark line; the others report the other configurations")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--rates", type=float, nargs="+", default=[100.0, 1000.0, 5000.0, 20000.0])
    ap.add_argument("--serve-count", type=int, default=512)
    ap.add_argument("--photons", type=int, nargs=2, default=[8, 44])
    ap.add_argument("--precision-n", type=int, default=20)
    ap.add_argument("--precision-seeds", type=int, default=8)
    ap.add_argument("--precision-seeds48", type=int, default=64)
    ap.add_argument("--precision-dd-seeds", type=int, default=8)
    ap.add_argument("--sample-modes", type=int, default=12)
    ap.add_argument("--samples", type=int, default=256)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload != "n40":
        if rank == 0:
            {"loop": run_loop, "batch": run_batch, "serve": run_serve, "precision": run_precision,
             "sample": run_sample}[args.workload](args)
        return
    run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
