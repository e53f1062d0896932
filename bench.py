#!/usr/bin/env python3
"""Throughput benchmark: PSD-filtered candidates/s on one GB300.

Workload (the synthetic PSD-filter throughput configuration): a seeded batch
of 2^28 length-45 sequences (order-90 Golay pairs, compression 2), entries
i.i.d. uniform over {-2, 0, 2}, conditioned by rejection on a row sum whose
square is in {a^2 : a^2 + b^2 = 180} = {36, 144}, stored int8 and resident
in HBM (12.08 GB, far larger than the 129 MB L2, so no flush is needed).

One step = one pass of the guarded-FP32 tensor-core PSD filter (tcgen05,
FP64 recheck of the guard band) over the whole batch, through the C ABI
(gp_psd_filter_device).  Reported beside it on the same data: the plain FP64
CUDA-core filter (the comparator), end-to-end throughput through the
host-buffer entry point gp_psd_filter (pinned host memory, copies inside the
timed region), the roofline of the filter kernel, and the oracle's FP64
filter timed on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

ORDER, COMPRESS, PAF = 90, 2, 0
L = ORDER // COMPRESS
ROWS = 1 << 28  # --rows overrides (profiling runs only)
REF_SLICE = 1 << 25  # rows per step of the reference arm
METRIC = "PSD-filtered candidates/s (guarded-FP32 tensor-core filter, verdicts exact vs FP64)"
UNIT = "candidates/s"
WORKLOAD = {"workload": "synthetic PSD-filter throughput: 2^28 x 45 int8, order 90, compress 2, paf 0",
            "rows": ROWS, "L": L, "order": ORDER, "compress": COMPRESS, "paf": PAF,
            "alphabet": [-2, 0, 2], "row_sums": [-12, -6, 6, 12], "seed": 0,
            "l2": "inputs (12.08 GB) larger than L2; no flush"}


def dist_env():
    from golaypair_gb300.replicas import dist_env as env
    return env()


def oracle_lib():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_build", "libgolay_oracle.so"))
    lib.gpo_psd_filter_batch.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int]
    lib.gpo_psd_filter_batch.restype = ctypes.c_int64
    return lib


def device_batch_to_host(rows, seed=0):
    """The bench batch itself (make_batch on the GPU with the same seed, so
    the very rows the GPU arm filters), copied to pinned host memory; the
    device copy is freed before anything is timed."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    d = make_batch(torch, rows, dev, seed=seed)
    h = torch.empty((rows, L), dtype=torch.int8, pin_memory=True)
    h.copy_(d)
    del d
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return h.numpy()


def cpu_baseline(host_rows, seconds=12.0):
    """The oracle's FP64 PSD filter (restating src/utils/fourier.cpp:25-52)
    on all host cores, over a bounded sample of the bench batch: its first
    rows (host_rows, copied from the device batch), cycled for ~12 s."""
    import numpy as np
    lib = oracle_lib()
    cores = os.cpu_count() or 1
    sample = np.ascontiguousarray(host_rows)
    verdict = np.zeros(len(sample), dtype=np.uint8)
    lib.gpo_psd_filter_batch(sample.ctypes.data, 1 << 16, L, ORDER, PAF, verdict.ctypes.data, cores)  # warm
    done, t0 = 0, time.perf_counter()
    while True:
        lib.gpo_psd_filter_batch(sample.ctypes.data, len(sample), L, ORDER, PAF, verdict.ctypes.data, cores)
        done += len(sample)
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return {"value": done / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{done} rows: the first {len(sample)} rows of the bench batch, cycled; FP64 direct DFT of "
                      f"bins 1..L/2 with early exit, {cores} threads, {el:.1f} s"}


def run_reference(args):
    """The reference's filter (the oracle's FP64 restatement of
    src/utils/fourier.cpp:25-52; the reference's own build needs FFTW and
    Boost, absent on the GPU machine) on the host cores, over the same rows as
    the GPU arm (same generator and seed).  A step filters one slice of
    REF_SLICE rows of that batch, the slices taken in turn (warm-up steps
    included), so that the default run stays within a few minutes of CPU
    time and a run of at least rows / REF_SLICE steps covers every row."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    lib = oracle_lib()
    cores = os.cpu_count() or 1
    rows = args.rows
    WORKLOAD["rows"] = rows
    seqs = device_batch_to_host(rows, seed=0)
    verdict = np.zeros(rows, dtype=np.uint8)
    sl = min(rows, REF_SLICE)
    nsl = (rows + sl - 1) // sl
    covered = [False] * nsl
    done = 0

    def step(g):
        i = g % nsl
        lo = i * sl
        n = min(sl, rows - lo)
        lib.gpo_psd_filter_batch(seqs[lo:].ctypes.data, n, L, ORDER, PAF, verdict[lo:].ctypes.data, cores)
        covered[i] = True
        return n

    for g in range(args.warmup):
        step(g)
    t0 = time.perf_counter()
    for g in range(args.warmup, args.warmup + args.steps):
        done += step(g)
    el = time.perf_counter() - t0
    v = done / el
    whole = all(covered)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, generated on device, copied to host before timing)", "config": WORKLOAD,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"one slice of {sl} rows of the {rows}-row batch per step, the {nsl} slices "
                                       f"in turn ({done} rows timed); the oracle's FP64 filter "
                                       f"(restating src/utils/fourier.cpp:25-52), {cores} threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if whole:
        line["passes"] = int(verdict.sum())
    print(json.dumps(line))
    return 0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sms, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sms.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for i, nm in enumerate(names):
                    if r[5 + i].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sms)}


def make_batch(torch, rows, device, seed=0):
    """2^28 x 45 int8 on the device: uniform {-2,0,2}, rejection on row sum."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.empty((rows, L), dtype=torch.int8, device=device)
    have = 0
    while have < rows:
        s = torch.randint(0, 3, (1 << 25, L), generator=g, device=device, dtype=torch.int8)
        s.sub_(1).mul_(2)
        rs = s.sum(1, dtype=torch.int32)
        keep = s[(rs == 6) | (rs == -6) | (rs == 12) | (rs == -12)]
        take = min(rows - have, keep.shape[0])
        out[have:have + take] = keep[:take]
        have += take
        del s, rs, keep
    return out


def read_profile_record(name):
    """A machine-readable ncu record under profiles/ (None when absent)."""
    p = os.path.join(REPO, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def read_profile_traffic():
    """DRAM bytes per row of the filter kernel, from the machine-readable
    record of its ncu capture (profiles/psd_tc_L45.json)."""
    p = os.path.join(REPO, "profiles", "psd_tc_L45.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return float(json.load(f)["dram_bytes_per_row"])


def run_gpu(args):
    import torch

    import golaypair_gb300 as gp
    from golaypair_gb300.replicas import max_over_ranks

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    ctx = gp.Context(local)
    # a dedicated (non-default) stream: the library enqueues on exactly this
    # stream, so CUDA events recorded on it bracket the kernels
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0

    global ROWS
    ROWS = args.rows
    WORKLOAD["rows"] = ROWS
    seqs = make_batch(torch, ROWS, dev, seed=rank)
    mask = torch.zeros((ROWS + 31) // 32, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    def step(mode):
        ctx.psd_filter_device(seqs.data_ptr(), ROWS, L, ORDER, PAF, mode, mask.data_ptr(), sptr)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(mode, steps, warmup):
        for _ in range(warmup):
            step(mode)
        barrier()
        ctx.kernel_timing(True)
        ctx.kernel_time()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(mode)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        kms, klaunch = ctx.kernel_time()
        ctx.kernel_timing(False)
        ms = max_over_ranks(ms, dev)
        return ms, kms, klaunch

    # exact-verdict spot check of this very batch against the FP64 kernel
    step(gp.GP_PSD_TC_GUARDED)
    tc_mask = mask.clone()
    st = ctx.psd_filter_device(seqs.data_ptr(), ROWS, L, ORDER, PAF, gp.GP_PSD_TC_GUARDED, mask.data_ptr(), sptr,
                               stats=True)
    step(gp.GP_PSD_FP64)
    torch.cuda.synchronize()
    verdicts_equal = bool(torch.equal(tc_mask, mask))

    clocks = ClockSampler(local)
    clocks.start()
    ms, kms, klaunch = timed(gp.GP_PSD_TC_GUARDED, args.steps, args.warmup)
    clk = clocks.stop()
    if args.profile:
        # profiling run: the tensor-core filter only (no comparator, no e2e)
        trace = None
        if args.trace:
            ctx.tc_trace(True)
            for _ in range(3):
                step(gp.GP_PSD_TC_GUARDED)
            torch.cuda.synchronize()
            tr = ctx.tc_trace(False)
            tiles = max(tr["tiles"], 1)
            # per tile: converter / epilogue counters cover 4 warps each
            trace = {k: round(v / tiles / (4 if k.startswith(("conv", "epi")) else 1), 1)
                     for k, v in tr.items() if k != "tiles"}
            trace["tiles"] = tr["tiles"]
        if rank == 0:
            print(json.dumps({"profile_run": True, "rows": ROWS, "ms_per_step": ms / args.steps,
                              "kernel_ms": kms / max(klaunch, 1), "verdicts_exact_vs_fp64_kernel": verdicts_equal,
                              "cycles_per_tile_per_role": trace}))
        ctx.close()
        return 0
    ms_step = ms / args.steps
    value = ROWS * ws / (ms_step / 1e3)

    # plain FP64 CUDA-core comparator, same data (fewer steps: it is slow)
    f_steps = max(1, min(3, args.steps))
    fms, fkms, _ = timed(gp.GP_PSD_FP64, f_steps, 1)
    fp64_value = ROWS * ws / (fms / f_steps / 1e3)

    # end to end through the host-buffer C ABI: pinned host input, H2D and the
    # D2H of the pass mask inside the timed region
    hseqs = torch.empty((ROWS, L), dtype=torch.int8, pin_memory=True)
    hseqs.copy_(seqs)
    cpu_rows = hseqs[:min(ROWS, 1 << 22)].numpy()  # the CPU baseline's sample: the batch's first rows
    hmask = torch.zeros((ROWS + 31) // 32, dtype=torch.int32, pin_memory=True)
    del seqs
    torch.cuda.empty_cache()
    e_steps = max(1, min(args.steps, 5))
    for _ in range(max(1, min(args.warmup, 2))):
        ctx.psd_filter_host_raw(hseqs.data_ptr(), ROWS, L, ORDER, PAF, gp.GP_PSD_TC_GUARDED, hmask.data_ptr())
    barrier()
    t0 = time.perf_counter()
    for _ in range(e_steps):
        ctx.psd_filter_host_raw(hseqs.data_ptr(), ROWS, L, ORDER, PAF, gp.GP_PSD_TC_GUARDED, hmask.data_ptr())
    barrier()
    e_el = time.perf_counter() - t0
    e_el = max_over_ranks(e_el, dev)
    e2e_value = ROWS * ws * e_steps / e_el
    e2e_equal = bool(torch.equal(hmask, tc_mask.cpu()))

    if rank == 0:
        peaks = {}
        pk = os.path.join(REPO, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            with open(pk) as f:
                peaks = json.load(f)
        peak = peaks.get("hbm_gbs")
        peak_src = "of measured" if peak else "of fallback"
        peak = peak or 6800.0
        alg_bytes = ROWS * L + ROWS / 8  # int8 rows read + 1-bit verdict written
        k_ms = kms / max(klaunch, 1)
        achieved = alg_bytes / (k_ms / 1e3) / 1e9
        traffic_row = read_profile_traffic()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp16 x fp16 -> fp32 (tcgen05) + f64 recheck; int8 input",
            "data": "synthetic (seeded, generated on device)", "config": WORKLOAD,
            "gpu_launches": 2 * args.steps,
            "verdicts_exact_vs_fp64_kernel": verdicts_equal and e2e_equal,
            "unsure_per_step": int(st.n_unsure), "pass_per_step": int(st.n_pass),
            "fp64_comparator": {"value": fp64_value, "unit": UNIT, "ms_per_step": fms / f_steps,
                                "kernel_ms": fkms / f_steps, "tc_speedup": value / fp64_value},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_src,
                         "traffic": traffic_row * ROWS if traffic_row else None,
                         "algorithmic_bytes_per_launch": alg_bytes, "kernel": "psd_tc_kernel<48>",
                         "kernel_ms": k_ms},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ROWS * L,
                    "d2h_bytes_per_step": ROWS // 8, "steps": e_steps},
            "clocks": clk,
        }
        line["cpu_baseline"] = cpu_baseline(cpu_rows)
        if ws == 1 and not args.no_extras:
            try:  # the headline stands even if a generation figure cannot be taken
                line["generation"] = generation_extras(gp, ctx, peaks)
            except Exception as e:  # noqa: BLE001 -- reported in the line, not raised
                line["generation"] = {"error": f"{type(e).__name__}: {e}"}
        print(json.dumps(line))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def tc_flops(L):
    """Algorithmic PSD flops per candidate: 4 L floor(L/2) + 3 floor(L/2)."""
    return 4 * L * (L // 2) + 3 * (L // 2)


class OracleGenStats(ctypes.Structure):
    """gpo_gen_stats of oracle/golay_oracle.h."""
    _fields_ = [("necklaces", ctypes.c_int64), ("psd_evals", ctypes.c_int64), ("psd_pass", ctypes.c_int64),
                ("written_a", ctypes.c_int64), ("written_b", ctypes.c_int64)]


def _oracle_gen_job(job):
    """One generation job through the oracle, in a spawned pool worker: a
    rank window ("window", order, c, paf, lo, hi) or one job of the
    reference's -n/-j split ("split", order, c, paf, j, n)."""
    import tempfile as _t
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_build", "libgolay_oracle.so"))
    i32, u64, cp, P = ctypes.c_int, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_void_p
    lib.gpo_generate.argtypes = [i32, i32, i32, cp, cp, i32, i32, P]
    lib.gpo_generate_window.argtypes = [i32, i32, i32, cp, cp, u64, u64, u64, u64, P]
    st = OracleGenStats()
    with _t.TemporaryDirectory() as d:
        a, b = os.path.join(d, "a").encode(), os.path.join(d, "b").encode()
        if job[0] == "window":
            _, order, comp, paf, lo, hi = job
            m = 2 ** 64 - 1
            lib.gpo_generate_window(order, comp, paf, a, b, lo >> 64, lo & m, hi >> 64, hi & m, ctypes.byref(st))
        else:
            _, order, comp, paf, j, n = job
            lib.gpo_generate(order, comp, paf, a, b, j, n, ctypes.byref(st))
    return st.necklaces, st.psd_evals


def generation_extras(gp, ctx, peaks):
    """The generation configurations, measured after the headline (one
    dict): the uneven batch (orders 34, 50, 58, 68 at compression 2 and 90
    at compression 5 over 2^32-word windows) in one tuned engine run; order
    57 (paf -2, compression 3 -> 1) through the golay driver: gen, sort,
    match over the whole word space, the uncompression of all 196,216 pairs
    to length 57 and the equivalence filter of the result; and the oracle's
    generation on the host cores over bounded samples of the same two
    workloads."""
    import multiprocessing as mp
    import tempfile

    from golaypair_gb300.workloads import batch_windows
    env = dict(os.environ, LC_ALL="C")
    bf16 = peaks.get("bf16_tflops") or 1887.2
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        wins = batch_windows()
        spec = [(o, c, p, lo, hi, os.path.join(tmp, f"{o}a"), os.path.join(tmp, f"{o}b")) for (o, c, p, lo, hi) in wins]
        ctx.generate_batch(spec, autotune=True)  # the tuner runs once; its choice is cached in the context
        t0 = time.perf_counter()
        stats, cfg = ctx.generate_batch(spec, autotune=True)
        el = time.perf_counter() - t0
        nk = sum(s.necklaces for s in stats)
        cand = sum(s.candidates for s in stats)
        flops = sum(s.candidates * tc_flops(o // c) for s, (o, c, _, _, _) in zip(stats, wins))
        out["uneven_batch"] = {
            "seconds": el, "necklaces": nk, "candidates": cand, "necklaces_per_s": nk / el,
            "candidates_per_s": cand / el, "iterations": cfg.iterations,
            "tuned": {k: getattr(cfg, k) for k in ("enum_variant", "windows_per_thread", "cand_cap", "tc_ctas_per_sm",
                                                   "multi_launch")},
            "tensor_pipe": {"algorithmic_tflops": flops / el / 1e12, "peak_tflops": bf16,
                            "frac": flops / el / 1e12 / bf16,
                            "note": "algorithmic PSD flops of the candidates over the whole engine run; the "
                                    "enumerator (integer issue) takes most of the device time"},
            "enumerator_issue": read_profile_record("enumerate_batch.json")}
        cli = gp.CLI_PATH
        d = os.path.join(tmp, "r57")
        base = [cli, "57", "-c", "3", "1", "--paf", "-2", "--dir", d]
        times = {}
        for stage in ("gen", "sort", "match", "uncompress", "filter"):
            t0 = time.perf_counter()
            subprocess.run(base + [stage], check=True, env=env, stdout=subprocess.DEVNULL)
            times[stage] = time.perf_counter() - t0
        wd = os.path.join(d, "order-57")
        with open(os.path.join(wd, "57-pairs-3")) as f:
            p3 = f.read().split("\n")[:-1]
        nlines = {fn: sum(1 for _ in open(os.path.join(wd, fn)))
                  for fn in ("57-filtered_sorted-a", "57-filtered_sorted-b", "57-pairs-1", "57-unique")}
        exps = 0
        for line in p3:
            v = line.split()
            for side in (v[:19], v[19:]):
                ones = sum(1 for x in side if x in ("1", "-1"))
                exps += 3 ** (ones - 1) if ones else 1
        out["order57"] = {
            "stage_seconds": times, "lines": nlines, "pairs_compression3": len(p3), "expansions": exps,
            "uncompress_pairs_per_s": len(p3) / times["uncompress"],
            "uncompress_expansions_per_s": exps / times["uncompress"],
            "match_pairs_per_s": len(p3) / times["match"],
            "filter_pairs_per_s": nlines["57-pairs-1"] / times["filter"],
            "note": "process wall times of the golay driver, context creation and file I/O included"}
        # the oracle on the host cores: the batch's windows cut to 2^28 words,
        # and 16 of 1000 jobs of the order-57 split, one process per item
        cores = os.cpu_count() or 1
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
        # each 2^28-word window cut into `cores` equal rank ranges, so that
        # every core has work
        sample = []
        for (o, c, p, lo, hi) in batch_windows(1 << 28):
            for k in range(cores):
                a, b = lo + (hi - lo) * k // cores, lo + (hi - lo) * (k + 1) // cores
                if a < b:
                    sample.append(("window", o, c, p, a, b))
        with mp.get_context("spawn").Pool(min(cores, len(sample))) as pool:
            t0 = time.perf_counter()
            res = pool.map(_oracle_gen_job, sample)
            wel = time.perf_counter() - t0
        shards = [("split", 57, 3, -2, j, 1000) for j in range(min(cores, 16))]
        with mp.get_context("spawn").Pool(len(shards)) as pool:
            t0 = time.perf_counter()
            res57 = pool.map(_oracle_gen_job, shards)
            sel = time.perf_counter() - t0
        out["cpu_pipeline"] = {
            "kind": "port", "cores": cores,
            "uneven_batch_2^28_windows": {"seconds": wel, "necklaces_per_s": sum(r[0] for r in res) / wel,
                                          "candidates_per_s": sum(r[1] for r in res) / wel,
                                          "jobs": len(sample), "processes": min(cores, len(sample))},
            "order57_16_of_1000_jobs": {"seconds": sel, "necklaces_per_s": sum(r[0] for r in res57) / sel,
                                        "candidates_per_s": sum(r[1] for r in res57) / sel,
                                        "processes": len(shards)},
            "note": "the oracle's generation (FP64 PSD filter, canonical check, files) on the same host's cores"}
    return out


def run_pipeline(args):
    """Times the search stages on the generation configurations (one JSON
    line each): the uneven batch (orders 34, 50, 58, 68 at compression 2 and
    90 at compression 5, 2^32-word windows) in one engine run and one order
    at a time, then full generation of order 57 (paf -2, compression 3), its
    sort and match, and uncompression of its first pairs."""
    import tempfile

    import golaypair_gb300 as gp
    from golaypair_gb300.workloads import batch_windows
    env = dict(os.environ, LC_ALL="C")
    with gp.Context(0) as ctx, tempfile.TemporaryDirectory() as tmp:
        def gen_window(order, comp, paf, lo, hi):
            t0 = time.perf_counter()
            st = ctx.generate_window(order, comp, paf, lo, hi, os.path.join(tmp, "a"), os.path.join(tmp, "b"))
            return st, time.perf_counter() - t0

        def stats_dict(st, el):
            return {"seconds": el, "necklaces": st.necklaces, "candidates": st.candidates, "psd_pass": st.psd_pass,
                    "written": st.written_a + st.written_b, "unsure": st.unsure,
                    "necklaces_per_s": st.necklaces / el, "candidates_per_s": st.candidates / el}

        gen_window(16, 2, 0, 0, 3 ** 8)  # warm-up (module load, twiddles)
        wins = batch_windows()
        # the uneven batch in one engine run: tuner first (its result is
        # cached in the context), then the timed run with the tuned settings
        spec = [(o, c, p, lo, hi, os.path.join(tmp, f"{o}a"), os.path.join(tmp, f"{o}b"))
                for (o, c, p, lo, hi) in wins]
        # --pipeline-no-graph: default settings with direct launches (for
        # per-kernel profiling, which does not follow graph replays)
        direct = gp.BatchConfig()
        direct.no_graph = 1 if args.pipeline_no_graph else 0
        direct.multi_launch = 1 if args.pipeline_multi_launch else 0
        tune = not (args.pipeline_no_graph or args.pipeline_multi_launch)
        t0 = time.perf_counter()
        _, cfg = ctx.generate_batch(spec, autotune=tune, config=None if tune else direct)
        tune_el = time.perf_counter() - t0
        t0 = time.perf_counter()
        stats, cfg = ctx.generate_batch(spec, autotune=tune, config=None if tune else direct)
        el = time.perf_counter() - t0
        tot_n = sum(s.necklaces for s in stats)
        tot_c = sum(s.candidates for s in stats)
        print(json.dumps({"pipeline": "batch", "jobs": [list(w) for w in wins], "seconds": el,
                          "necklaces_per_s": tot_n / el, "candidates_per_s": tot_c / el,
                          "necklaces": tot_n, "candidates": tot_c, "iterations": cfg.iterations,
                          "tuned": {k: getattr(cfg, k) for k in ("enum_variant", "windows_per_thread", "cand_cap",
                                                                 "tc_ctas_per_sm", "multi_launch")},
                          "tune_run_seconds": tune_el, "tuner_seconds": cfg.tune_seconds,
                          "per_job": [dict(order=w[0], compress=w[1], written=s.written_a + s.written_b,
                                           necklaces=s.necklaces, candidates=s.candidates, psd_pass=s.psd_pass,
                                           unsure=s.unsure) for w, s in zip(wins, stats)]}), flush=True)
        if args.pipeline_only == "batch":
            return 0
        # the same windows one order per call, for comparison
        for order, comp, paf, lo, hi in wins:
            st, el = gen_window(order, comp, paf, lo, hi)
            print(json.dumps(dict({"pipeline": "window", "order": order, "compress": comp, "paf": paf,
                                   "rank_window": [lo, hi]}, **stats_dict(st, el))), flush=True)
        cli = gp.CLI_PATH
        d = os.path.join(tmp, "r57")
        times = {}
        for stage in ("gen", "sort", "match"):
            t0 = time.perf_counter()
            subprocess.run([cli, "57", "-c", "3", "1", "--paf", "-2", "--dir", d, stage], check=True, env=env,
                           stdout=subprocess.DEVNULL)
            times[stage] = time.perf_counter() - t0
        wd = os.path.join(d, "order-57")
        with open(os.path.join(wd, "57-pairs-3")) as f:
            pairs = f.readlines()
        head = pairs[:args.pipeline_pairs]
        with open(os.path.join(wd, "57-head-3"), "w") as f:
            f.writelines(head)
        t0 = time.perf_counter()
        subprocess.run([cli, "57", "-c", "3", "1", "--paf", "-2", "--dir", d, "uncompress", "-i", "head", "-o",
                        "headout"], check=True, env=env, stdout=subprocess.DEVNULL)
        times["uncompress"] = time.perf_counter() - t0
        with open(os.path.join(wd, "57-headout-1")) as f:
            found = sum(1 for _ in f)
        lines = {fn: sum(1 for _ in open(os.path.join(wd, fn))) for fn in
                 ("57-filtered-a#0", "57-filtered-b#0", "57-pairs-3")}
        print(json.dumps({"pipeline": "order57", "order": 57, "compress": [3, 1], "paf": -2,
                          "seconds": times, "lines": lines, "uncompressed_pairs_of_first": [len(head), found],
                          "pairs_per_s_match": lines["57-pairs-3"] / times["match"],
                          "candidates_written_per_s_gen": (lines["57-filtered-a#0"] + lines["57-filtered-b#0"])
                          / times["gen"],
                          "note": "process wall times of the golay driver, including context creation"}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rows", type=int, default=1 << 28, help="batch rows (profiling runs only)")
    ap.add_argument("--profile", action="store_true", help="time the tensor-core filter only")
    ap.add_argument("--no-extras", action="store_true", help="skip the generation configurations after the headline")
    ap.add_argument("--trace", action="store_true", help="with --profile: per-role cycle counters")
    ap.add_argument("--pipeline", action="store_true", help="time the generation configurations instead")
    ap.add_argument("--pipeline-pairs", type=int, default=200, help="compressed pairs to uncompress (--pipeline)")
    ap.add_argument("--pipeline-only", choices=["all", "batch"], default="all",
                    help="--pipeline: everything, or only the uneven batch in one engine run")
    ap.add_argument("--pipeline-no-graph", action="store_true",
                    help="--pipeline: run the batch engine with direct launches and default settings")
    ap.add_argument("--pipeline-multi-launch", action="store_true",
                    help="--pipeline: run the batch engine untuned with one launch per kernel over all jobs")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.pipeline:
        return run_pipeline(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
