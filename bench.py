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


def host_sample(rows, seed=0):
    """The same distribution as the device batch, generated on the host."""
    import numpy as np
    rng = np.random.default_rng(seed + 1000)
    out, have = [], 0
    while have < rows:
        s = rng.choice(np.array([-2, 0, 2], dtype=np.int8), size=(1 << 20, L))
        rs = s.astype(np.int32).sum(1)
        s = s[np.isin(rs, [-12, -6, 6, 12])]
        out.append(s)
        have += len(s)
    return np.ascontiguousarray(np.concatenate(out)[:rows])


def cpu_baseline(seconds=12.0):
    """The oracle's FP64 PSD filter (restating src/utils/fourier.cpp:25-52)
    on all host cores, over a bounded sample of the workload."""
    import numpy as np
    lib = oracle_lib()
    cores = os.cpu_count() or 1
    sample = host_sample(1 << 21)
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
            "sample": f"{done} rows of the workload distribution (2^21 distinct, seeded), FP64 direct DFT of "
                      f"bins 1..L/2 with early exit, {cores} threads, {el:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    lib = oracle_lib()
    cores = os.cpu_count() or 1
    per_step = 1 << 22
    sample = host_sample(per_step)
    verdict = np.zeros(per_step, dtype=np.uint8)
    for _ in range(args.warmup):
        lib.gpo_psd_filter_batch(sample.ctypes.data, per_step, L, ORDER, PAF, verdict.ctypes.data, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.gpo_psd_filter_batch(sample.ctypes.data, per_step, L, ORDER, PAF, verdict.ctypes.data, cores)
    el = time.perf_counter() - t0
    v = per_step * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(WORKLOAD, step_rows=per_step),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per_step} rows per step of the workload distribution; the oracle's FP64 "
                                       f"filter (restating src/utils/fourier.cpp:25-52), {cores} threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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


def read_profile_traffic():
    """dram bytes per row of the filter kernel from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "psd_tc_L45.md")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("dram_bytes_per_row:"):
                return float(line.split(":")[1].split()[0])
    return None


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
        line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line))
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


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
        direct.no_graph = 1
        tune = not args.pipeline_no_graph
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
                                                                 "tc_ctas_per_sm")},
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
    ap.add_argument("--trace", action="store_true", help="with --profile: per-role cycle counters")
    ap.add_argument("--pipeline", action="store_true", help="time the generation configurations instead")
    ap.add_argument("--pipeline-pairs", type=int, default=200, help="compressed pairs to uncompress (--pipeline)")
    ap.add_argument("--pipeline-only", choices=["all", "batch"], default="all",
                    help="--pipeline: everything, or only the uneven batch in one engine run")
    ap.add_argument("--pipeline-no-graph", action="store_true",
                    help="--pipeline: run the batch engine with direct launches and default settings")
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
