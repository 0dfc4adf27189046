"""Benchmark of the int32 Floyd-Warshall APSP engine on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (default): the reference's maximum size, n = 32768 (a 4 GiB int32
matrix), density 0.5, integer weights uniform in [1, 100], missing edge = INF,
diagonal 0, seed 7, solved by the drop-in for the reference's
multi_layer_tiling_gpu (kappa = 8) in int32 arithmetic. Inputs are synthetic
(the reference's generator with the weight range as a parameter). Metric:
relaxations per second, n^3 per solve / solve time.

One step = restore the pristine input (device-to-device copy) + one full
solve. `value` is timed on the device with CUDA events over exactly K steps
(inputs resident in HBM, 4 GiB > L2 so nothing stays cached between steps);
`e2e` is the same metric through the C ABI with host buffers: every step
copies the input from pinned host memory, solves, and copies the distance
matrix back. `auto_path` is the same workload through FW_VARIANT_AUTO (the
exact packed 16-bit fast path, taken only when provably identical), with its
own roofline and e2e; `verified` compares its result with the int32 result
bit for bit and checks sampled full rows of the int32 result against the
oracle's Dijkstra, and 64 graphs of the batched result against the oracle's
sweep. With --gpus N (torchrun) every rank solves its own copy of
the workload (replicas; the path has no data-parallel exchange) and `value`
is the sum over ranks, timed by the slowest rank.

--impl reference times the reference's CPU implementation of the path
(baseline_cpu, src/fw_baseline_cpu.cpp:3-16, as restated by the oracle) on
all host cores over bounded samples of the same workload, and additionally
the reference's own GPU kernels (multi_layer_tiling_gpu, the run's kappa,
built for sm_103a from its sources) on the full workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "APSP relaxations/s (n^3/t)"
UNIT = "relax/s"
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
VARIANTS = {"baseline_gpu": 0, "tiling_gpu": 1, "multi_layer_tiling_gpu": 2, "auto": 3}


def parse() -> argparse.Namespace:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--density", type=float, default=0.5)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--wmin", type=int, default=1)
    ap.add_argument("--wmax", type=int, default=100)
    ap.add_argument("--algorithm", default="multi_layer_tiling_gpu", choices=list(VARIANTS),
                    help="the headline; auto = exact packed 16-bit sweep when provably identical, else "
                         "multi_layer_tiling_gpu")
    ap.add_argument("--kappa", type=int, default=8)
    ap.add_argument("--no-auto", action="store_true",
                    help="skip the sub-record of the exact packed fast path (FW_VARIANT_AUTO)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target length of the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-graphs measurement")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable fp32 measurement")
    ap.add_argument("--no-ooc", action="store_true", help="skip the out-of-core (host-resident matrix) measurement")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons, power = [], None, set(), []
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names[1:], parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "sm_mhz_min": min(sm) if sm else None, "power_w_median": statistics.median(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time (all ranks get it)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(world: int, steps: int, relax_per_step: float, elapsed_s: float) -> float:
    """Whole-job relaxations/s: every rank solves its own replica of the
    workload each step; the job takes as long as its slowest rank."""
    return world * steps * relax_per_step / elapsed_s


# Matrices smaller than this are L2-resident: the timed steps then flush L2
# (a write of L2_FLUSH_BYTES) before each step, outside the timed events.
L2_RESIDENT_BYTES = 256 << 20
L2_FLUSH_BYTES = 512 << 20


def l2_policy(n: int) -> str:
    if 4 * n * n >= L2_RESIDENT_BYTES:
        return f"inputs larger than L2 ({4 * n * n / 2**30:.2f} GiB matrix), restored from a pristine copy every step"
    return (f"L2 flushed before every step (a {L2_FLUSH_BYTES >> 20} MiB write outside the timed events; "
            f"{4 * n * n / 2**20:.1f} MiB matrix)")


def solve_steps(F, torch, stream, work, pristine, n, kappa, variant, steps, warmup, world, local=None):
    """`warmup` untimed then `steps` timed restore + solve steps of `variant`
    on `stream` (CUDA events, per-kernel profile over the timed steps). With
    `local` set, nvidia-smi clocks are sampled during the timed region. A
    matrix that fits L2 is timed step by step, with L2 flushed between steps
    outside the events."""
    def step():
        work.copy_(pristine, non_blocking=True)
        F.apsp_i32(work, n, 32, kappa, variant, stream)

    flush = None
    if 4 * n * n < L2_RESIDENT_BYTES:
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=work.device)
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local if local is not None else 0)
    if local is not None:
        clocks.__enter__()
    try:
        F.profile_begin()
        if flush is None:
            e0.record(stream)
            for _ in range(steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            secs = e0.elapsed_time(e1) / 1e3
        else:
            evs = []
            for _ in range(steps):
                flush.fill_(1)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                step()
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize()
            secs = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        prof = F.profile_end()
    finally:
        if local is not None:
            clocks.__exit__(None, None, None)
    barrier(world)
    F.check_faults(stream)
    elapsed = max_over_ranks(secs, world)
    return elapsed, prof, (clocks.summary() if local is not None else None)


E2E_MIN_STEPS = 10


def end_to_end(F, torch, stream, work, h_in, n, kappa, variant, steps, world, local, relax, serial_steps):
    """The metric through the C ABI with host buffers: every step copies its
    input from pinned host memory and its result back. Pipelined over two
    device buffers (as a user streaming matrices would run it): step k+1's
    host-to-device copy and step k-1's device-to-host copy run on their own
    streams while step k solves. The pipelined stream runs max(steps,
    E2E_MIN_STEPS) matrices, so that its fill and drain (the first input's
    copy in, the last result's copy out, which nothing overlaps) weigh as
    they would in a stream of matrices rather than in a handful. The serial
    form (copy, solve, copy) is timed too, over `serial_steps` steps. Returns
    the e2e record and the host copy of the last result."""
    h_out = torch.empty((n, n), dtype=torch.int32).pin_memory()
    bufs = [work, torch.empty_like(work)]
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()

    def serial_step():
        work.copy_(h_in, non_blocking=True)
        F.apsp_i32(work, n, 32, kappa, variant, stream)
        h_out.copy_(work, non_blocking=True)

    def pipelined(k_steps):
        ev_in = [torch.cuda.Event() for _ in bufs]
        ev_solved = [torch.cuda.Event() for _ in bufs]
        ev_out = [torch.cuda.Event() for _ in bufs]
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)

        def copy_in(k):  # step k's input into buffer k % 2, once its previous result is home
            i = k % 2
            if k >= 2:
                s_in.wait_event(ev_out[i])
            with torch.cuda.stream(s_in):
                bufs[i].copy_(h_in, non_blocking=True)
            ev_in[i].record(s_in)

        a.record(s_in)
        copy_in(0)
        for k in range(k_steps):
            i = k % 2
            # Enqueue the next input before this solve: the solve's ~2000
            # launches can block the host until the GPU has run most of them.
            if k + 1 < k_steps:
                copy_in(k + 1)
            stream.wait_event(ev_in[i])
            F.apsp_i32(bufs[i], n, 32, kappa, variant, stream)
            ev_solved[i].record(stream)
            s_out.wait_event(ev_solved[i])
            with torch.cuda.stream(s_out):
                h_out.copy_(bufs[i], non_blocking=True)
            ev_out[i].record(s_out)
        b.record(s_out)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    def copy_rate(fn):
        fn()
        torch.cuda.synchronize()
        x = torch.cuda.Event(enable_timing=True)
        y = torch.cuda.Event(enable_timing=True)
        x.record(stream)
        fn()
        y.record(stream)
        torch.cuda.synchronize()
        return 4.0 * n * n / (x.elapsed_time(y) / 1e3) / 1e9

    h2d_gbs = copy_rate(lambda: work.copy_(h_in, non_blocking=True))
    d2h_gbs = copy_rate(lambda: h_out.copy_(work, non_blocking=True))

    serial_step()
    pipelined(2)
    torch.cuda.synchronize()
    barrier(world)
    t1 = torch.cuda.Event(enable_timing=True)
    t2 = torch.cuda.Event(enable_timing=True)
    pipe_steps = max(steps, E2E_MIN_STEPS)
    with ClockSampler(local) as e2e_clocks:
        e2e_s = max_over_ranks(pipelined(pipe_steps), world)
        t1.record(stream)
        for _ in range(serial_steps):
            serial_step()
        t2.record(stream)
        torch.cuda.synchronize()
    F.check_faults(stream)
    serial_s = max_over_ranks(t1.elapsed_time(t2) / 1e3, world)
    rec = {"value": aggregate(world, pipe_steps, relax, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": 4 * n * n, "d2h_bytes_per_step": 4 * n * n,
           "ms_per_step": 1e3 * e2e_s / pipe_steps, "steps": pipe_steps, "pipelined": True,
           "serial_ms_per_step": 1e3 * serial_s / serial_steps, "serial_steps": serial_steps,
           "serial_value": aggregate(world, serial_steps, relax, serial_s),
           "copy_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs}, "clocks": e2e_clocks.summary()}
    # the two buffers solved the same input
    rec["buffers_agree"] = bool(torch.equal(bufs[0], bufs[1]))
    del bufs[1]
    return rec, h_out


def int32_ceiling(F, stream, sm_mhz):
    """The int32 relaxation ceiling of this GPU from register-only kernels:
    the best measured relaxation form (the roofline's peak) and a model from
    the measured instruction-class rates. A relaxation is either one DPX
    add-min (ALU pipe) or one multiply-add (FMA pipe) plus half of a DPX
    three-way min (ALU pipe); with a fraction x of the first kind the ALU
    needs (1 + x) / 2 lane operations per relaxation, the FMA pipe 1 - x, and
    both together (3 - x) / 2, bounded by the add-min rate, the multiply-add
    rate and the measured rate of the two classes alternating. The model's
    best x is the most any int32 instruction mix of these classes can give."""
    dpx_only, mixed = F.measure_relax_peak(stream)
    rates = F.measure_int32_rates(stream)
    forms = {"form_b_relax": rates["form_b_relax"], "form_a_relax": rates["form_a_relax"],
             "form_b_then_addmin_relax": rates["form_b_then_addmin_relax"], "mixed_probe": mixed,
             "dpx_only_probe": dpx_only}
    best_name = max(forms, key=forms.get)
    r_alu, r_fma, r_both = rates["dpx_addmin"], rates["imad"], rates["dpx_addmin_imad_alternating"]
    best_x, best_r = 0.0, 0.0
    for i in range(1001):
        x = i / 1000.0
        r = min(r_alu / ((1 + x) / 2), r_fma / (1 - x) if x < 1 else float("inf"), r_both / ((3 - x) / 2))
        if r > best_r:
            best_x, best_r = x, r
    out = {"peak": forms[best_name], "peak_form": best_name, "forms_relax_per_s": forms,
           "class_lane_ops_per_s": {k: rates[k] for k in ("dpx_addmin", "imad", "dpx_min3", "add", "min",
                                                          "dpx_addmin_imad_alternating")},
           "model_peak": best_r, "model_addmin_fraction": best_x}
    if sm_mhz:
        sms = torch_sm_count()
        per = 1.0 / (sm_mhz * 1e6 * sms)
        out["per_clock_per_sm"] = {"sm_mhz": sm_mhz, "sms": sms,
                                   "class_warp_instr": {k: v * per / 32 for k, v in out["class_lane_ops_per_s"].items()},
                                   "peak_relax": out["peak"] * per, "model_peak_relax": best_r * per}
    return out


def torch_sm_count() -> int:
    import torch

    return int(torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count)


def dijkstra_rows(W: np.ndarray, D_rows: dict, threads: int) -> dict:
    """Full rows of a solved matrix against the oracle's dense Dijkstra from the
    same sources (exact for non-negative weights), in parallel threads."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, min(threads, len(D_rows)))) as ex:
        refs = dict(zip(D_rows, ex.map(lambda src: O.sssp_row(W, src), list(D_rows))))
    ok = [int(src) for src in D_rows if np.array_equal(refs[src], D_rows[src])]
    return {"rows": sorted(int(s) for s in D_rows), "rows_vs_dijkstra": f"{len(ok)}/{len(D_rows)}",
            "all_rows_match": len(ok) == len(D_rows), "seconds": round(time.perf_counter() - t0, 2)}


def run_ours(args) -> None:
    import torch

    import fw_cuda_gb300 as F

    rank, world, local = dist_setup(args)
    n = args.n
    variant = VARIANTS[args.algorithm]
    F.lib()
    # All work goes to one non-blocking stream of our own rather than the
    # legacy default stream (which synchronises with every blocking stream).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    t0 = time.time()
    h_in = torch.empty((n, n), dtype=torch.int32).pin_memory()
    F.generate_graph(n, args.density, args.seed, args.wmin, args.wmax, out=h_in.numpy())
    gen_s = time.time() - t0
    pristine = h_in.cuda()
    work = torch.empty_like(pristine)
    relax = float(n) ** 3
    # The same matrix generated on the device (fw_generate_graph_device_i32).
    torch.cuda.synchronize()
    t0 = time.time()
    F.generate_graph_device(work, n, args.density, args.seed, args.wmin, args.wmax, stream)
    torch.cuda.synchronize()
    gen_dev_s = time.time() - t0
    gen_dev_same = bool(torch.equal(work, pristine))

    # ---- the headline: the named algorithm, timed over exactly `steps` steps
    elapsed, prof, clocks = solve_steps(F, torch, stream, work, pristine, n, args.kappa, variant, args.steps,
                                        args.warmup, world, local)
    value = aggregate(world, args.steps, relax, elapsed)
    head_out = work.clone()  # the timed solve's result, for the checks below
    head_packed = F.auto_used_packed(stream) if variant == VARIANTS["auto"] else False

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_measured = "hbm_gbs" in peaks
    ceiling = int32_ceiling(F, stream, clocks.get("sm_mhz") if clocks else None)
    torch.cuda.synchronize()
    roofline = head_roofline(F, stream, prof, n, args, variant, head_packed, ceiling, hbm_peak, hbm_measured)

    e2e = None
    if not args.no_e2e:
        e2e, h_out = end_to_end(F, torch, stream, work, h_in, n, args.kappa, variant, args.steps, world, local, relax,
                                max(1, min(args.steps, 5)))
        # the host copy of the last result equals the device-timed solve of the same input
        e2e["matches_device_result"] = bool(torch.equal(h_out, head_out.cpu())) and e2e.pop("buffers_agree")
        del h_out

    # ---- the exact packed fast path (FW_VARIANT_AUTO) as a labelled sub-record
    auto = None
    if variant != VARIANTS["auto"] and not args.no_auto:
        auto = run_auto(args, F, torch, stream, work, pristine, h_in, n, world, local, relax, head_out, hbm_peak,
                        hbm_measured)

    batched, batched_data = None, None
    if not args.no_batched:
        batched, batched_data = run_batched(args, F, torch, stream, world)

    diff = None
    if not args.no_diff:
        diff = run_diff(args, torch, stream, world)

    ooc = None
    if not args.no_ooc:
        ooc = run_out_of_core(args, F, torch, h_in, head_out, n, world, relax)

    verified = {"fault_status": "fw_check_faults clean after every timed region"}
    if auto is not None:
        verified["auto_equals_int32"] = auto.pop("equals_headline")
    if e2e is not None:
        verified["e2e_equals_device_result"] = e2e["matches_device_result"]
    if ooc is not None:
        verified["out_of_core_equals_in_core"] = ooc["matches_in_core"]
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # The CPU-baseline leg: the oracle's sweep timed on a sample, and the
        # oracle's Dijkstra rows as the checker of the timed solve's result.
        cpu = cpu_sample(h_in.numpy(), threads=1, seconds=args.cpu_seconds)
        rng = np.random.default_rng(2024)
        srcs = sorted({0, n - 1, *[int(x) for x in rng.choice(n, size=min(n, 6), replace=False)]})
        rows = {s: head_out[s].cpu().numpy() for s in srcs}
        verified.update(dijkstra_rows(h_in.numpy(), rows, os.cpu_count() or 1))
        if batched_data is not None:
            verified.update(batched_sample_check(batched_data, 64, os.cpu_count() or 1))

    launches = sum(v["launches"] for v in prof.values())
    if rank == 0:
        int32_arith = variant != VARIANTS["auto"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "int32" if int32_arith or not head_packed else "int32 result via exact packed u16x2 arithmetic",
            "data": "synthetic",
            "config": {"workload": f"APSP n={n} density={args.density} weights U[{args.wmin},{args.wmax}] "
                                   f"seed={args.seed}",
                       "n": n, "density": args.density, "seed": args.seed, "algorithm": args.algorithm,
                       "kappa": args.kappa, "parallelism": f"replicas{world}",
                       "l2": l2_policy(n),
                       "generate_s": round(gen_s, 2), "generate_device_s": round(gen_dev_s, 3),
                       "device_generator_matches": gen_dev_same},
            "gpu_launches": launches,
            "kernels": {k: {"launches": v["launches"], "total_ms": round(v["total_ms"], 3)} for k, v in prof.items()},
            "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
            "verified": verified, "auto_path": auto,
            "batched": batched, "differentiable": diff, "out_of_core": ooc,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def head_roofline(F, stream, prof, n, args, variant, packed, ceiling, hbm_peak, hbm_measured):
    """Roofline of the headline's dominant kernel."""
    if variant == VARIANTS["baseline_gpu"]:
        st = prof.get("fw_pivot_step")
        if not st or not st["launches"]:
            return None
        secs = st["total_ms"] / 1e3
        # algorithmic bytes of a pivot launch: the matrix read once (4 n^2);
        # writes are the entries that change, which the kernel alone stores
        gbs = 4.0 * n * n * st["launches"] / secs / 1e9
        return {"kernel": "fw_pivot_step_vec_kernel" if n % 4 == 0 else "fw_pivot_step_kernel",
                "bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm_measured else "fallback",
                "avg_launch_ms": st["total_ms"] / st["launches"],
                "traffic": (268.54e6 + 3.45e6) * (n / 8192.0) ** 2, "traffic_unit": "bytes per launch",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of pivot 4000 at "
                                  "n = 8192, scaled by n^2"}
    if packed:
        return packed_roofline(F, stream, prof, n, hbm_peak, hbm_measured)
    st = prof.get("fw_stripe")
    if st and st["launches"]:
        # n <= 2048: one cooperative launch whose time is its chain of
        # ceil(n / 8) stages (flag hand-over, stripe update, 8-pivot closure,
        # stripe panel), not its arithmetic: reported against the same int32
        # peak, with the time per stage beside it.
        secs = st["total_ms"] / 1e3 / st["launches"]
        stages = -(-n // 8)
        achieved = float(n) ** 3 / secs
        gbs = 8.0 * n * n / secs / 1e9  # the matrix read and written once
        return {"kernel": "fw_stripe_kernel", "bound": "latency", "achieved": achieved, "peak": ceiling["peak"],
                "unit": UNIT, "frac": achieved / ceiling["peak"],
                "peak_source": "measured live: best register-only int32 relaxation form "
                               f"({ceiling['peak_form']}, fw_measure_relax_peak / fw_measure_int32_rates)",
                "traffic": None, "avg_launch_ms": 1e3 * secs, "stages": stages,
                "us_per_stage": 1e6 * secs / stages,
                "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm_measured else "fallback"}}
    pair = variant == VARIANTS["multi_layer_tiling_gpu"] and args.kappa > 4 and n >= 24576
    # bulk launch: all tiles outside two pivot blocks (the two-block pass, or
    # the look-ahead of the one-block pass)
    r = roofline_of(prof.get("fw_remainder"), "fw_remainder_kernel", n, 256 if pair else 128, 4, 256,
                    ceiling["peak"], "measured live: best register-only int32 relaxation form "
                    f"({ceiling['peak_form']}, fw_measure_relax_peak / fw_measure_int32_rates)", hbm_peak,
                    hbm_measured, traffic_at_16384=(1.11e9 + 983.25e6) if pair else (1.07e9 + 979.55e6))
    if r:
        r["int32_ceiling"] = ceiling
        r["frac_of_model_peak"] = r["achieved"] / ceiling["model_peak"]
    return r


def packed_roofline(F, stream, prof, n, hbm_peak, hbm_measured):
    peak_packed_dpx, peak_packed = F.measure_relax_peak_packed(stream)
    r = roofline_of(prof.get("fw_p16_remainder"), "fw_p16_remainder_kernel", n, 256, 2, 512, peak_packed,
                    "measured live: register-only packed 16-bit relaxation kernels "
                    "(fw_measure_relax_peak_packed), best instruction mix", hbm_peak, hbm_measured,
                    traffic_at_16384=537.49e6 + 444.44e6)
    if r:
        r["dpx_only_peak"] = peak_packed_dpx
        r["frac_of_dpx_only"] = r["achieved"] / peak_packed_dpx
    return r


def run_auto(args, F, torch, stream, work, pristine, h_in, n, world, local, relax, head_out, hbm_peak, hbm_measured):
    """FW_VARIANT_AUTO on the same workload: the exact packed 16-bit sweep
    (two 15-bit lanes per DPX instruction) when the encode/decode proof
    holds, else the int32 sweep. Its result is compared bit for bit with the
    headline's int32 result."""
    steps = max(1, min(args.steps, 10))
    elapsed, prof, clocks = solve_steps(F, torch, stream, work, pristine, n, args.kappa, VARIANTS["auto"], steps,
                                        1, world, local)
    used = F.auto_used_packed(stream)
    same = bool(torch.equal(work, head_out))
    out = {"algorithm": "auto (FW_VARIANT_AUTO)", "kappa": args.kappa,
           "dtype": "int32 result via exact packed u16x2 arithmetic" if used else "int32",
           "used_packed": used, "value": aggregate(world, steps, relax, elapsed), "unit": UNIT, "steps": steps,
           "ms_per_step": 1e3 * elapsed / steps, "clocks": clocks, "equals_headline": same,
           "roofline": packed_roofline(F, stream, prof, n, hbm_peak, hbm_measured) if used else None,
           "kernels": {k: {"launches": v["launches"], "total_ms": round(v["total_ms"], 3)} for k, v in prof.items()}}
    if not args.no_e2e:
        e2e, h_out = end_to_end(F, torch, stream, work, h_in, n, args.kappa, VARIANTS["auto"], steps, world, local,
                                relax, 1)
        e2e["matches_device_result"] = bool(torch.equal(h_out, head_out.cpu())) and e2e.pop("buffers_agree")
        out["e2e"] = e2e
        del h_out
    return out


def roofline_of(stats, kernel, n, pivots, bytes_per_value, gap, peak, peak_source, hbm_peak, hbm_measured,
                traffic_at_16384=None):
    """Roofline of the dominant kernel from its event-timed launches.

    Work: relaxations. Algorithmic bytes: a launch with K pivots reads and
    writes each of its tiles once, so its tile bytes are relaxations * 2 *
    bytes_per_value / K (the panels it streams, K * n values, are left out:
    under 2 % at n = 32768). The bulk launch of a pass covers (n - gap)^2
    entries; `traffic_at_16384` is ncu's dram__bytes_read.sum +
    dram__bytes_write.sum for that launch at n = 16384 (one pass, the matrix
    well above L2), scaled by the entries a launch touches."""
    if not stats or not stats["launches"]:
        return None
    secs = stats["total_ms"] / 1e3
    achieved = stats["relaxations"] / secs
    tile_bytes = stats["relaxations"] * 2.0 * bytes_per_value / pivots
    hbm_gbs = tile_bytes / secs / 1e9
    bulk_bytes = 2.0 * bytes_per_value * (n - gap) ** 2
    out = {"kernel": kernel, "bound": "int_issue", "achieved": achieved, "peak": peak, "unit": UNIT,
           "frac": achieved / peak, "peak_source": peak_source, "traffic": None,
           "avg_launch_ms": stats["total_ms"] / stats["launches"],
           "relax_per_launch": stats["relaxations"] / stats["launches"],
           "bulk_launch": {"pivots": pivots, "entries": (n - gap) ** 2, "algorithmic_bytes": bulk_bytes},
           "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_gbs / hbm_peak,
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm_measured else "fallback"}}
    if traffic_at_16384:
        out["traffic"] = traffic_at_16384 * ((n - gap) / (16384.0 - gap)) ** 2
        out["traffic_unit"] = "bytes per bulk launch"
        out["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one bulk launch at "
                                 "n = 16384, scaled by (n - %d)^2" % gap)
    return out


def run_batched(args, F, torch, stream, world) -> dict:
    """4096 graphs, n log-uniform in [16, 512] (fw_cuda_gb300.workloads): one
    autotuned, graph-captured batched launch per step, against looping the
    single-graph entry point over the same graphs. Both time `steps` steps of
    restore (device copy of the packed input) + solve with CUDA events."""
    from fw_cuda_gb300 import workloads

    sizes, offsets, packed = workloads.batched_graphs(F)
    pristine = torch.from_numpy(packed).cuda()
    work = torch.empty_like(pristine)
    plan = F.BatchPlan(sizes, offsets)
    schedule = plan.autotune(pristine, stream)
    relax = plan.relaxations
    base = work.data_ptr()

    def timed(fn, steps):
        for _ in range(max(1, args.warmup)):
            work.copy_(pristine, non_blocking=True)
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            work.copy_(pristine, non_blocking=True)
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(a.elapsed_time(b) / 1e3, world) / steps

    def loop():
        for g in range(len(sizes)):
            F.apsp_i32(base + 4 * int(offsets[g]), int(sizes[g]), 32, args.kappa, 2, stream)

    t_batched = timed(lambda: plan.solve(work, stream), args.steps)
    result = work.cpu().numpy()  # the last timed solve's output, for the sampled check
    t_loop = timed(loop, max(1, min(args.steps, 2)))
    plan.close()
    count = len(sizes)
    rec = {"workload": "4096 graphs, n log-uniform [16, 512], density U(0.05, 1), weights U[1, 100], seed 1234",
           "graphs_per_s": world * count / t_batched, "relax_per_s": world * relax / t_batched,
           "ms_per_step": 1e3 * t_batched, "schedule": schedule,
           "loop_plain_graphs_per_s": world * count / t_loop, "loop_plain_ms_per_step": 1e3 * t_loop,
           "speedup_vs_loop": t_loop / t_batched, "relaxations_per_step": relax}
    return rec, (sizes, offsets, packed, result)


def batched_sample_check(data, count: int, threads: int) -> dict:
    """The 8 largest graphs and `count - 8` seeded random others of the
    batched result against the oracle's sweep of each graph (parallel host
    threads)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    sizes, offsets, packed, out = data
    rng = np.random.default_rng(4096)
    largest = np.argsort(-sizes, kind="stable")[:8]
    rest = np.setdiff1d(np.arange(len(sizes)), largest)
    pick = sorted(largest.tolist() + rng.choice(rest, min(len(rest), count - 8), replace=False).tolist())

    def ok(g):
        n, o = int(sizes[g]), int(offsets[g])
        return np.array_equal(out[o:o + n * n], O.fw_i32(packed[o:o + n * n].reshape(n, n)).ravel())

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        good = sum(ex.map(ok, pick))
    return {"batched_graphs_vs_oracle": f"{good}/{len(pick)}", "batched_all_match": good == len(pick),
            "batched_check_seconds": round(time.perf_counter() - t0, 2)}


def run_diff(args, torch, stream, world) -> dict:
    """256 graphs at n = 256 (one batched call) plus one graph at n = 4096,
    density 0.3, fp32 weights U(0.5, 10) tie-free, dL/dD ~ N(0, 1): forward
    (distances + next hops) alone, and forward + backward, per step."""
    from fw_cuda_gb300 import autograd as A
    from fw_cuda_gb300 import workloads

    rng = np.random.default_rng(5)
    Wb = torch.from_numpy(np.stack([workloads.diff_graph(256, rng) for _ in range(256)])).cuda()
    Wl = torch.from_numpy(workloads.diff_graph(4096, rng)).cuda()
    Gb = torch.randn(Wb.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    Gl = torch.randn(Wl.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(2))

    def fwd():
        A.forward_with_next_hops(Wb, stream)
        A.forward_with_next_hops(Wl, stream)

    def fwd_bwd():
        _, nhb = A.forward_with_next_hops(Wb, stream)
        _, nhl = A.forward_with_next_hops(Wl, stream)
        A.backward_from_next_hops(Gb, nhb, stream)
        A.backward_from_next_hops(Gl, nhl, stream)

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(a.elapsed_time(b) / 1e3, world) / args.steps

    t_f = timed(fwd)
    t_fb = timed(fwd_bwd)
    relax = 256 * 256.0 ** 3 + 4096.0 ** 3
    return {"workload": "256 graphs n=256 + 1 graph n=4096, density 0.3, fp32 U(0.5,10) tie-free, dL/dD ~ N(0,1)",
            "forward_ms": 1e3 * t_f, "forward_backward_ms": 1e3 * t_fb, "fwd_bwd_over_fwd": t_fb / t_f,
            "forward_relax_per_s": world * relax / t_f}


def run_out_of_core(args, F, torch, h_in, d_result, n, world, relax) -> dict:
    """The same matrix solved in place in pinned HOST memory by the
    out-of-core sweep (pass width 2048, stripes sized from free device
    memory): one warm-up and up to two timed calls (each returns when the host
    matrix holds the result; wall clock). The result is compared with the
    in-core solve of the same input (d_result)."""
    h = torch.empty_like(h_in).pin_memory()
    times = []
    for i in range(1 + max(1, min(args.steps, 2))):
        h.copy_(h_in)
        t0 = time.perf_counter()
        F.apsp_i32_host(h, n, 2048, 0)
        el = time.perf_counter() - t0
        if i > 0:
            times.append(el)
    el = max_over_ranks(sum(times) / len(times), world)
    same = bool(torch.equal(d_result.cpu(), h))
    return {"workload": "the APSP workload above, matrix in pinned host memory, pass width 2048",
            "value": world * relax / el, "unit": UNIT, "ms_per_solve": 1e3 * el,
            "host_link_bytes_per_solve": 8.0 * n * n * ((n + 2047) // 2048), "matches_in_core": same}


def cpu_sample(W: np.ndarray, threads: int, seconds: float) -> dict:
    """The oracle's baseline_cpu sweep over the first pivots of the full matrix
    until about `seconds` have passed; relaxations/s = pivots * n^2 / t."""
    from oracle import oracle as O

    n = W.shape[0]
    D = W.copy()
    done, t0 = 0, time.perf_counter()
    chunk = 1
    while True:
        O.fw_i32_pivots(D, done, done + chunk, threads)
        done += chunk
        el = time.perf_counter() - t0
        if el >= seconds or done >= n:
            break
        per = el / done
        chunk = max(1, min(n - done, int((seconds - el) / per / 2) or 1))
    return {"value": done * float(n) ** 2 / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"baseline_cpu k-i-j sweep (oracle restatement of src/fw_baseline_cpu.cpp:3-16), "
                      f"pivots 0..{done - 1} of the n={n} workload matrix, {done} * n^2 relaxations in {el:.2f} s"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    n = args.n
    threads = os.cpu_count() or 1
    t0 = time.time()
    W = np.empty((n, n), dtype=np.int32)
    O.lib().oracle_generate_graph(W, n, args.density, args.seed, args.wmin, args.wmax)
    gen_s = time.time() - t0
    D = W.copy()
    # Size one step to a few seconds of all-core work on this host.
    t0 = time.perf_counter()
    O.fw_i32_pivots(D, 0, 2, threads)
    per_pivot = (time.perf_counter() - t0) / 2
    pivots = max(1, min(n, int(4.0 / max(per_pivot, 1e-6))))
    k = 2
    for _ in range(args.warmup):
        kk = min(n, k + pivots)
        O.fw_i32_pivots(D, k, kk, threads)
        k = kk if kk < n else 0
    times = []
    for _ in range(args.steps):
        kk = min(n, k + pivots)
        t0 = time.perf_counter()
        O.fw_i32_pivots(D, k, kk, threads)
        times.append((time.perf_counter() - t0, kk - k))
        k = kk if kk < n else 0
    tot_t = sum(t for t, _ in times)
    tot_p = sum(p for _, p in times)
    value = tot_p * float(n) ** 2 / tot_t
    ref_gpu = reference_gpu(args, W)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"APSP n={n} density={args.density} weights U[{args.wmin},{args.wmax}] "
                               f"seed={args.seed}", "n": n, "generate_s": round(gen_s, 2),
                   "step": f"{pivots} pivots of the baseline_cpu k-i-j sweep over the full matrix"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps x {pivots} pivots (of {n}) of the baseline_cpu sweep "
                                   f"(oracle restatement of src/fw_baseline_cpu.cpp:3-16) over the full n={n} "
                                   f"matrix, rows split over {threads} host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)


def reference_gpu(args, W: np.ndarray, timed: int = 3):
    """The reference's kernels of the run's algorithm (`--algorithm`;
    multi_layer_tiling_gpu for "auto", with the run's kappa), built for
    sm_103a from its sources and launched by its own launch loop on the
    legacy default stream, on the full workload: one untimed full-size solve,
    then `timed` solves of a fresh copy of the input, each bracketed by CUDA
    events on that stream (the reference's Timer::measureGPU also times one
    solve with events after a warm-up, src/timer.cu:35-64)."""
    try:
        import torch

        from oracle import oracle as O

        if not torch.cuda.is_available() or not O.refgpu_available():
            return {"unavailable": "reference kernels not built (needs the reference sources at build time)"}
        n = W.shape[0]
        algo = args.algorithm if args.algorithm in ("baseline_gpu", "tiling_gpu") else "multi_layer_tiling_gpu"
        source = {"baseline_gpu": "src/fw_baseline_gpu.cu", "tiling_gpu": "src/fw_tiling_gpu.cu",
                  "multi_layer_tiling_gpu": "src/fw_multi_layer_tiling_gpu.cu"}[algo]
        legacy = torch.cuda.default_stream()
        pristine = torch.from_numpy(W).cuda()
        d = torch.empty_like(pristine)
        secs = []
        for i in range(1 + timed):
            d.copy_(pristine)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(legacy)
            O.refgpu_run(algo, d.data_ptr(), n, args.kappa)  # synchronises the context
            b.record(legacy)
            b.synchronize()
            if i > 0:
                secs.append(a.elapsed_time(b) / 1e3)
        mean = sum(secs) / len(secs)
        return {"algorithm": algo, "kappa": args.kappa, "value": float(n) ** 3 / mean,
                "unit": UNIT, "seconds_per_solve": mean, "seconds_min": min(secs), "seconds_max": max(secs),
                "solves_timed": len(secs),
                "how": f"reference kernels ({source}) compiled for sm_103a, launched by the "
                       "reference launch loop on the legacy default stream; one full-size warm-up solve, then "
                       "CUDA events around each timed solve of a fresh copy of the input"}
    except Exception as e:  # report, never fail the CPU line
        return {"unavailable": f"{type(e).__name__}: {e}"}


def main() -> None:
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
