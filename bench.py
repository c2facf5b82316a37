"""Benchmark: RAJA data-parallel primitives on GB300 (bandwidth-sweep config).

One step = one pass of every primitive of the bandwidth-sweep configuration
at N = 2^28 elements each (inputs resident in HBM, every input larger than
the 129 MB L2, so no flush is needed between steps):

  ReduceSum f32, ReduceSum f64       uniform[-1,1)
  ReduceMinLoc / ReduceMaxLoc        f32 and f64 uniform[-1,1)
  exclusive_scan int64               uniform{0..1023}
  radix sort u32, u64                uniform over the full range
  sort_pairs                         f32 normal(0,1) keys, int32 index values
  MultiReduceSum histogram           int32 Zipf(1.1) into 256 and 65536 bins

value = algorithmic bytes of all primitives / device time of the step
(GB/s); the per-primitive bytes follow the fixed convention: sum/min/max
sizeof(T) per element, scan 2 sizeof(T), LSD radix sort
N sizeof(K) (2P+1) with P = bits/8 digit passes (+ N sizeof(V) 2P for
values), histogram 4 bytes per element.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the oracle's OpenMP restatement of RAJA's
omp_parallel_for_exec path on the host cores, on the same workload.  RAJA's
own omp policies are compiled only where the RAJA sources are (they pin the
oracle bit for bit there, tests/golden/make_ref_fixtures.py); the GPU host
has no RAJA tree, so the timed arm is the pinned restatement.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "primitive GB/s (aggregate over the bandwidth-sweep primitives)"
UNIT = "GB/s"


# ----------------------------------------------------------------- workload
def primitive_table(n: int):
    """(name, algorithmic bytes) for one step at n elements per primitive."""
    return [
        ("reduce_sum_f32", 4 * n), ("reduce_sum_f64", 8 * n),
        ("minloc_f32", 4 * n), ("maxloc_f32", 4 * n),
        ("minloc_f64", 8 * n), ("maxloc_f64", 8 * n),
        ("exclusive_scan_i64", 16 * n),
        ("sort_u32", 4 * n * (2 * 4 + 1)), ("sort_u64", 8 * n * (2 * 8 + 1)),
        ("sort_pairs_f32_i32", 4 * n * (2 * 4 + 1) + 4 * n * 2 * 4),
        ("histogram_256", 4 * n), ("histogram_65536", 4 * n),
    ]


def zipf_cdf(nbins: int, s: float = 1.1):
    import numpy as np
    w = 1.0 / np.arange(1, nbins + 1, dtype=np.float64) ** s
    c = np.cumsum(w)
    return c / c[-1]


def make_inputs(n: int, seed: int, device: str):
    """Seeded synthetic inputs of the bandwidth-sweep configuration."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    t = {}
    t["f32"] = torch.rand(n, generator=g, device=device, dtype=torch.float32) * 2 - 1
    t["f64"] = torch.rand(n, generator=g, device=device, dtype=torch.float64) * 2 - 1
    t["scan_in"] = torch.randint(0, 1024, (n,), generator=g, device=device, dtype=torch.int64)
    t["u32"] = torch.randint(-2 ** 31, 2 ** 31, (n,), generator=g, device=device,
                             dtype=torch.int32).view(torch.uint32)
    t["u64"] = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), generator=g, device=device,
                             dtype=torch.int64).view(torch.uint64)
    t["pk"] = torch.randn(n, generator=g, device=device, dtype=torch.float32)
    t["pv"] = torch.arange(n, device=device, dtype=torch.int32)
    for nb in (256, 65536):
        cdf = torch.from_numpy(zipf_cdf(nb)).to(device)
        u = torch.rand(n, generator=g, device=device, dtype=torch.float64)
        t[f"z{nb}"] = torch.searchsorted(cdf, u, right=True).clamp_(0, nb - 1).to(torch.int32)
        del u
    return t


def make_outputs(n: int, device: str):
    import torch
    return {
        "scan_out": torch.empty(n, dtype=torch.int64, device=device),
        "u32_out": torch.empty(n, dtype=torch.int32, device=device).view(torch.uint32),
        "u64_out": torch.empty(n, dtype=torch.int64, device=device).view(torch.uint64),
        "pk_out": torch.empty(n, dtype=torch.float32, device=device),
        "pv_out": torch.empty(n, dtype=torch.int32, device=device),
        "sum": torch.empty(2, dtype=torch.float64, device=device),
        "loc_f32": torch.empty(4, dtype=torch.float32, device=device),
        "loc_f64": torch.empty(4, dtype=torch.float64, device=device),
        "idx": torch.empty(4, dtype=torch.int64, device=device),
        "h256": torch.zeros(256, dtype=torch.int64, device=device),
        "h65536": torch.zeros(65536, dtype=torch.int64, device=device),
    }


def step_calls(lib, t, o, n: int, stream: int):
    """The step as a list of (name, zero-arg callable) over the C ABI."""
    P = lambda x: x.data_ptr()  # noqa: E731
    s = stream
    o_sum, o_lf, o_ld, o_ix = P(o["sum"]), P(o["loc_f32"]), P(o["loc_f64"]), P(o["idx"])
    return [
        ("reduce_sum_f32", lambda: lib.b200_reduce_sum_f32(P(t["f32"]), n, 0, o_sum, s)),
        ("reduce_sum_f64", lambda: lib.b200_reduce_sum_f64(P(t["f64"]), n, 0, o_sum + 8, s)),
        ("minloc_f32", lambda: lib.b200_reduce_minloc_f32(P(t["f32"]), n, o_lf, o_ix, s)),
        ("maxloc_f32", lambda: lib.b200_reduce_maxloc_f32(P(t["f32"]), n, o_lf + 4, o_ix + 8, s)),
        ("minloc_f64", lambda: lib.b200_reduce_minloc_f64(P(t["f64"]), n, o_ld, o_ix + 16, s)),
        ("maxloc_f64", lambda: lib.b200_reduce_maxloc_f64(P(t["f64"]), n, o_ld + 8, o_ix + 24, s)),
        ("exclusive_scan_i64", lambda: lib.b200_scan_exclusive_i64(
            P(t["scan_in"]), P(o["scan_out"]), n, 0, 0, s)),
        ("sort_u32", lambda: lib.b200_sort_keys_copy_u32(P(t["u32"]), P(o["u32_out"]), n, 0, s)),
        ("sort_u64", lambda: lib.b200_sort_keys_copy_u64(P(t["u64"]), P(o["u64_out"]), n, 0, s)),
        ("sort_pairs_f32_i32", lambda: lib.b200_sort_pairs_copy_f32_i32(
            P(t["pk"]), P(t["pv"]), P(o["pk_out"]), P(o["pv_out"]), n, 0, s)),
        ("histogram_256", lambda: lib.b200_histogram_i32(P(t["z256"]), n, 256, P(o["h256"]), s)),
        ("histogram_65536", lambda: lib.b200_histogram_i32(P(t["z65536"]), n, 65536,
                                                           P(o["h65536"]), s)),
    ]


def run_step(calls):
    for name, fn in calls:
        rc = fn()
        if rc != 0:
            from raja_gb300 import _lib
            _lib.check(name, rc)


# ------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# -------------------------------------------------------------- cpu legs
class CpuSuite:
    """The oracle's OpenMP restatement of RAJA's omp_parallel_for_exec path
    over the bandwidth-sweep primitives at n elements per primitive.

    Inputs are generated once (seeded numpy, the same distributions as the
    device inputs) on first use of each primitive; output and sort work
    buffers are allocated and touched up front, so a timed call pays for the
    primitive only: sorts are timed in place on a fresh copy of the input
    (RAJA's sort is in place), made outside the timer."""

    def __init__(self, n: int, seed: int = 0):
        import numpy as np
        import oracle
        self.np, self.orc, self.n, self.seed = np, oracle, n, seed
        self.arrays: dict = {}
        self.table = dict(primitive_table(n))
        self.names = [p for p, _ in primitive_table(n)]

    def _get(self, key):
        np = self.np
        if key in self.arrays:
            return self.arrays[key]
        n = self.n
        rng = np.random.default_rng([self.seed, sorted(self._KEYS).index(key)])
        if key == "f32":
            a = rng.uniform(-1, 1, n).astype(np.float32)
        elif key == "f64":
            a = rng.uniform(-1, 1, n)
        elif key == "scan_in":
            a = rng.integers(0, 1024, n).astype(np.int64)
        elif key == "u32":
            a = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        elif key == "u64":
            a = rng.integers(0, 2 ** 64, n, dtype=np.uint64)
        elif key == "pk":
            a = rng.normal(0, 1, n).astype(np.float32)
        elif key == "pv":
            a = np.arange(n, dtype=np.int32)
        else:  # z256, z65536
            nb = int(key[1:])
            a = np.searchsorted(zipf_cdf(nb), rng.random(n), side="right").clip(0, nb - 1) \
                .astype(np.int32)
        self.arrays[key] = a
        return a

    _KEYS = ("f32", "f64", "scan_in", "u32", "u64", "pk", "pv", "z256", "z65536")

    def _work(self, key, like):
        w = self.arrays.get("w_" + key)
        if w is None:
            w = self.np.ones_like(like)       # touched: no page faults in the timed call
            self.arrays["w_" + key] = w
        return w

    def call(self, name: str):
        """(prepare, timed): inputs are generated here, outside the timed
        call; prepare() copies sort inputs into their work buffers."""
        o, g, w, np = self.orc, self._get, self._work, self.np
        if name == "reduce_sum_f32" or name == "reduce_sum_f64":
            x = g(name[-3:])
            return None, lambda: o.reduce_sum(x, parallel=True)
        if name in ("minloc_f32", "maxloc_f32", "minloc_f64", "maxloc_f64"):
            fn = o.reduce_minloc if name.startswith("min") else o.reduce_maxloc
            x = g(name[-3:])
            return None, lambda: fn(x, parallel=True)
        if name == "exclusive_scan_i64":
            x = g("scan_in")
            out = w("scan", x)
            return None, lambda: o.scan(x, "plus", exclusive=True, init=0, parallel=True, out=out)
        if name in ("sort_u32", "sort_u64"):
            src = g(name[-3:])
            buf = w(name, src)
            return (lambda: np.copyto(buf, src)), \
                (lambda: o.sort_inplace(buf, parallel=True, stable=False))
        if name == "sort_pairs_f32_i32":
            ks, vs = g("pk"), g("pv")
            kb, vb = w("pk", ks), w("pv", vs)
            return (lambda: (np.copyto(kb, ks), np.copyto(vb, vs))), \
                (lambda: o.sort_pairs_inplace(kb, vb, parallel=True, stable=False))
        if name.startswith("histogram_"):
            nb = int(name.split("_")[1])
            x = g(f"z{nb}")
            return None, lambda: o.histogram(x, nb, parallel=True)
        raise KeyError(name)

    def time(self, name: str) -> float:
        prep, fn = self.call(name)
        if prep:
            prep()
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0


def cpu_suite_rotation(suite: "CpuSuite", steps: int, warmup: int):
    """Time `steps` rotation steps after `warmup` untimed ones: step k runs
    primitive k mod 12 of the suite at the full n (a bounded sample of one
    step of the workload).  Primitives the rotation did not reach run once
    more, so every primitive has a time.  Returns per-primitive mean
    seconds and the seconds the timed steps took."""
    names = suite.names
    for k in range(warmup):
        suite.time(names[k % len(names)])
    acc: dict[str, list] = {}
    timed = 0.0
    for k in range(steps):
        nm = names[k % len(names)]
        dt = suite.time(nm)
        timed += dt
        acc.setdefault(nm, []).append(dt)
    for nm in names:
        if nm not in acc:
            acc[nm] = [suite.time(nm)]
    return {nm: sum(v) / len(v) for nm, v in acc.items()}, timed


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ------------------------------------------------------------- reference
def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over all ranks (x itself on one rank): every rank's
    timed region ends at the slowest rank."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gbs(world: int, bytes_per_step: float, steps: int, ms: float) -> float:
    """Whole-job GB/s: every rank processes its own step (weak scaling), so
    the job moves world x bytes per step in the slowest rank's time."""
    return world * bytes_per_step * steps / (ms / 1e3) / 1e9


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    import oracle
    oracle.build()
    os.environ.setdefault("OMP_PROC_BIND", "close")
    n = 1 << args.cpu_log2n
    suite = CpuSuite(n)
    per, _ = cpu_suite_rotation(suite, args.steps, args.warmup)
    table = suite.table
    step_s = sum(per.values())            # one full step: every primitive once
    value = sum(table.values()) / step_s / 1e9
    cores = oracle.max_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * step_s, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed (f32,f64,i32,i64,u32,u64)",
        "data": "synthetic (seeded, bandwidth-sweep shapes)",
        "config": config_block(args, n_override=n),
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each timed step runs one primitive of the suite at "
                                   f"N=2^{args.cpu_log2n} in rotation (all 12 covered); "
                                   f"ms_per_step = the sum of the per-primitive means "
                                   f"(oracle OpenMP restatement of omp_parallel_for_exec, "
                                   f"pinned to RAJA's own results; no RAJA sources on this "
                                   f"host), CPU {cpu_model()}"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "primitives": {nm: {"ms": round(1000 * per[nm], 2),
                            "gbs": round(table[nm] / per[nm] / 1e9, 3)} for nm in suite.names},
    }
    print(json.dumps(line), flush=True)


def config_block(args, n_override=None):
    n = n_override or (1 << args.log2n)
    return {"workload": "primitive bandwidth sweep (reductions, MinLoc/MaxLoc, int64 scan, sorts, "
                        "histograms) at N=2^%d per primitive"
                        % (n.bit_length() - 1),
            "n": n, "primitives": [p for p, _ in primitive_table(n)],
            "l2_flush": "none: every input is larger than the 129 MB L2",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--cpu-log2n", type=int, default=28)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cub", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import raja_gb300
    from raja_gb300 import _lib

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()
    n = 1 << args.log2n
    dev = "cuda"
    inputs = make_inputs(n, seed=rank, device=dev)
    outs = make_outputs(n, dev)
    stream = torch.cuda.current_stream()
    calls = step_calls(lib, inputs, outs, n, stream.cuda_stream)
    table = dict(primitive_table(n))
    step_bytes = sum(table.values())

    for _ in range(args.warmup):
        run_step(calls)
    raja_gb300.synchronize()

    # ---- timed region: K steps, barrier + sync on both sides
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        run_step(calls)
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    raja_gb300.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    ms_per_step = ms / args.steps
    value = aggregate_gbs(world, step_bytes, args.steps, ms)
    launches_per_step = None

    # ---- per-primitive breakdown and per-kernel times (CUDA events on the
    # launching stream, inside the library)
    per_prim = {}
    reps = max(3, min(10, args.steps))
    for name, fn in calls:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            rc = fn()
            _lib.check(name, rc)
        b.record(stream)
        torch.cuda.synchronize()
        t_ms = a.elapsed_time(b) / reps
        per_prim[name] = {"ms": round(t_ms, 4), "gbs": round(table[name] / t_ms / 1e6, 1)}
    raja_gb300.prof_reset()
    raja_gb300.prof_enable(True)
    for _ in range(reps):
        run_step(calls)
    torch.cuda.synchronize()
    kern = raja_gb300.prof_read()
    raja_gb300.prof_enable(False)
    launches_per_step = sum(v[0] for v in kern.values()) // reps
    kernels = {k: {"launches_per_step": v[0] // reps, "ms_per_step": round(v[1] / reps, 4)}
               for k, v in kern.items()}

    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    peak_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    for name, v in per_prim.items():
        v["frac_of_" + peak_src + "_hbm"] = round(v["gbs"] / hbm_peak, 3)
        if name.startswith("sort"):
            v["gkeys_per_s"] = round(n / v["ms"] / 1e6, 2)
    # the library's own run of each primitive left its outputs in `outs`:
    # CUB runs on the same inputs and its results are compared bit for bit
    if not args.no_cub:
        try:
            for name, c in bench_cub(inputs, outs, n, stream, reps).items():
                per_prim[name]["cub_ms"] = c["ms"]
                per_prim[name]["vs_cub"] = round(c["ms"] / per_prim[name]["ms"], 3)
                per_prim[name]["equal_to_cub"] = c["equal"]
        except Exception as e:  # report, do not lose the headline line
            per_prim["cub_error"] = f"{type(e).__name__}: {e}"
    roof = roofline(kernels, n, hbm_peak, peak_src)

    # ---- e2e through the public API with host buffers
    e2e = run_e2e(args, lib, inputs, outs, n, stream, table, dist)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = run_cpu_baseline(args)
    extras = {}
    if not args.no_extras:
        del inputs, outs
        torch.cuda.empty_cache()
        for nm, fn in (("forall_daxpy_dot", bench_forall_dot),
                       ("batched_workgroup_4096_loops", bench_batched), ("jacobi_256_meshes", bench_jacobi),
                       ("raja_api_indexset_workgroup", bench_raja_api),
                       ("accuracy_ill_conditioned", bench_accuracy)):
            try:
                extras[nm] = fn(lib)
            except Exception as e:  # report, do not lose the headline line
                extras[nm] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "mixed (f32,f64,i32,i64,u32,u64)",
            "data": "synthetic (seeded on device, bandwidth-sweep shapes)",
            "config": config_block(args),
            "frac_of_hbm_peak": round(value / world / hbm_peak, 3),
            "hbm_peak_gbs": hbm_peak, "hbm_peak_source": peak_src,
            "roofline": roof, "e2e": e2e, "cpu_baseline": cpu,
            "gpu_launches": launches_per_step * args.steps if launches_per_step else None,
            "gpu_launches_per_step": launches_per_step,
            "clocks": clk,
            "extras": extras, "kernels": kernels,
            # last, so that a record that keeps only the tail of the line
            # still carries every primitive's time, GB/s, fraction and CUB ratio
            "primitives": per_prim,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------------------ extra configs
def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _limbs(v):
    """Exact fixed-point form of a float64 CUDA tensor: (limbs, emin) with
    limbs[i, k] int64 such that v[i] = sum_k limbs[i, k] * 2^(32k + emin).
    Each mantissa (53 bits) is split in two halves that land in 32-bit
    limbs, so every limb entry stays below 2^32 in magnitude and sums of up
    to 2^30 entries are exact in int64."""
    import torch
    m, e = torch.frexp(v)
    mi = torch.ldexp(m, torch.full_like(e, 53)).to(torch.int64)   # exact, |mi| < 2^53
    e2 = e.to(torch.int64) - 53
    nz = mi != 0
    emin = int(e2[nz].min()) if bool(nz.any()) else 0
    sh = torch.where(nz, e2 - emin, torch.zeros_like(e2))
    mh = mi >> 26                       # floor division, also for negatives
    ml = mi - (mh << 26)                # 0 <= ml < 2^26
    nq = int(sh.max()) // 32 + 3
    limbs = torch.zeros(v.numel(), nq, dtype=torch.int64, device=v.device)
    for val, s_ in ((ml, sh), (mh, sh + 26)):
        q, r = s_ // 32, s_ % 32
        w = val << r                    # |w| < 2^58
        limbs.scatter_add_(1, q.unsqueeze(1), (w & 0xFFFFFFFF).unsqueeze(1))
        limbs.scatter_add_(1, (q + 1).unsqueeze(1), (w >> 32).unsqueeze(1))
    return limbs, emin


def _exact_from_limbs(sums, emin):
    """(hi, lo) doubles of sum_k sums[k] * 2^(32k + emin), sums int64 list."""
    import math
    t = sum(int(x) << (32 * k) for k, x in enumerate(sums))
    hi = float(t)
    lo = float(t - int(hi))
    return math.ldexp(hi, emin), math.ldexp(lo, emin)


def exact_sum(v):
    """Exact sum of a float CUDA tensor as (hi, lo): hi = the sum rounded to
    double, lo = the rest rounded.  Integer limb sums, no rounding."""
    limbs, emin = _limbs(v.double())
    return _exact_from_limbs(limbs.sum(0).tolist(), emin)


def exact_prefix_f64(v):
    """Exact inclusive prefix sums of a float CUDA tensor, each rounded to
    double (limb-wise int64 cumsum, then one conversion)."""
    import torch
    limbs, emin = _limbs(v.double())
    cum = torch.cumsum(limbs, 0)
    out = torch.zeros(v.numel(), dtype=torch.float64, device=v.device)
    for k in range(cum.shape[1] - 1, -1, -1):   # most significant limb first
        out += torch.ldexp(cum[:, k].double(), torch.tensor(32 * k + emin, device=v.device))
    return out


def bench_forall_dot(lib, reps=20, seed=6):
    """The forall daxpy body y += 2.5 x (24 B per element) and the dot
    product (16 B per element in FP64, 8 B in FP32) at 2^28 and 2^20
    elements, CUDA events over `reps` back-to-back calls (every input is
    larger than the L2 at 2^28; at 2^20 the data stays in L2)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    s = torch.cuda.current_stream().cuda_stream
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    res = {}
    peak = load_peaks().get("hbm_gbs")
    for log2n in (28, 20):
        n = 1 << log2n
        x = torch.rand(n, generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        y = torch.rand(n, generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        xf, yf = x.float(), y.float()
        calls = (("daxpy_f64", 24 * n, lambda: lib.b200_forall_axpy_f64(2.5, x.data_ptr(), y.data_ptr(), n, s)),
                 ("dot_f64", 16 * n, lambda: lib.b200_dot_f64(x.data_ptr(), y.data_ptr(), n, 0, out.data_ptr(), s)),
                 ("dot_f32", 8 * n, lambda: lib.b200_dot_f32(xf.data_ptr(), yf.data_ptr(), n, 0, out.data_ptr(), s)))
        for nm, nbytes, f in calls:
            for _ in range(3):
                f()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                rc = f()
                if rc != 0:
                    raise RuntimeError(f"{nm}: status {rc}")
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b) / reps
            gbs = nbytes / ms / 1e6
            res[f"{nm}_n2p{log2n}_ms"] = round(ms, 4)
            res[f"{nm}_n2p{log2n}_gbs"] = round(gbs, 1)
            if peak and log2n == 28:
                res[f"{nm}_n2p{log2n}_frac_of_measured_hbm"] = round(gbs / peak, 3)
        del x, y, xf, yf
    return res


def bench_accuracy(lib, seed=3):
    """Ill-conditioned FP32 sums / dots / scans at N=2^28 (sign +-1 times
    lognormal(0, 6) clipped to [1e-8, 1e8]; the last element cancels the
    sum of the others, which makes the sum's condition number ~1e10):
    naive FP32, compensated FP32 and naive FP64 against exact sums computed
    here with integer limbs."""
    import torch
    n = 1 << 28
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)

    def illcond():
        sign = torch.randint(0, 2, (n,), generator=g, device="cuda", dtype=torch.int8).float() * 2 - 1
        mag = torch.exp(torch.randn(n, generator=g, device="cuda") * 6.0).clamp_(1e-8, 1e8)
        return (sign * mag).float()

    x = illcond()
    y = illcond()
    head, _ = exact_sum(x[:-1])
    x[-1] = -head                     # rounded to FP32: the rest is the sum
    ex, exlo = exact_sum(x)
    if ex == 0.0:
        x[-1] = torch.nextafter(x[-1], torch.zeros_like(x[-1]))
        ex, exlo = exact_sum(x)
    abs_sum = float(x.double().abs().sum())
    s = torch.cuda.current_stream().cuda_stream
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    res = {"n": n, "cond_sum": abs_sum / abs(ex)}
    x64 = x.double()
    for nm, call in (("naive_f32", lambda: lib.b200_reduce_sum_f32(x.data_ptr(), n, 0, out.data_ptr(), s)),
                     ("comp_f32", lambda: lib.b200_reduce_sum_f32(x.data_ptr(), n, 1, out.data_ptr(), s)),
                     ("naive_f64", lambda: lib.b200_reduce_sum_f64(x64.data_ptr(), n, 0, out.data_ptr(), s))):
        assert call() == 0
        torch.cuda.synchronize()
        v = out[0].item()
        res[f"sum_rel_err_{nm}"] = abs((v - ex) - exlo) / abs(ex)
    # dot with an independent copy (products of two floats are exact in FP64)
    y64 = y.double()
    dx, dlo = exact_sum(x64 * y64)
    res["cond_dot"] = float((x64 * y64).abs().sum()) / abs(dx)
    for nm, call in (("naive_f32", lambda: lib.b200_dot_f32(x.data_ptr(), y.data_ptr(), n, 0, out.data_ptr(), s)),
                     ("comp_f32", lambda: lib.b200_dot_f32(x.data_ptr(), y.data_ptr(), n, 1, out.data_ptr(), s)),
                     ("naive_f64", lambda: lib.b200_dot_f64(x64.data_ptr(), y64.data_ptr(), n, 0, out.data_ptr(), s))):
        assert call() == 0
        torch.cuda.synchronize()
        v = out[0].item()
        res[f"dot_rel_err_{nm}"] = abs((v - dx) - dlo) / abs(dx)
    del x64, y64
    # inclusive scan of all 2^28 elements: max error over prefixes, relative
    # to sum|x| so far.  An FP32 output cannot be closer to the exact prefix
    # than its own rounding, so the floor for any FP32-output scan (the
    # exact prefixes rounded to FP32) is reported beside the modes.
    ref = exact_prefix_f64(x)
    absp = torch.cumsum(x.double().abs(), 0)
    o = torch.empty_like(x)
    for nm, mode in (("naive_f32", 0), ("comp_f32", 1)):
        assert lib.b200_scan_inclusive_f32(x.data_ptr(), o.data_ptr(), n, 0, mode, s) == 0
        torch.cuda.synchronize()
        res[f"scan_maxerr_over_abs_{nm}"] = float(((o.double() - ref).abs() / absp).max())
    del o
    res["scan_maxerr_over_abs_f32_rounding_floor"] = float(
        ((ref.float().double() - ref).abs() / absp).max())
    o64 = torch.empty(n, dtype=torch.float64, device="cuda")
    x64 = x.double()
    assert lib.b200_scan_inclusive_f64(x64.data_ptr(), o64.data_ptr(), n, 0, 0, s) == 0
    torch.cuda.synchronize()
    res["scan_maxerr_over_abs_naive_f64"] = float(((o64 - ref).abs() / absp).max())
    del o64, x64, ref, absp
    res["scan_n"] = n
    res["exact_reference"] = "int64 limb sums on the device (bench.py exact_sum / exact_prefix_f64)"
    # The FP32-compensated sum and dot return a double and can beat naive
    # FP64; the FP32 scan returns FP32 prefixes, so it is held to the FP32
    # rounding floor instead of to the FP64 scan.
    res["comp_f32_sum_and_dot_no_worse_than_naive_f64"] = bool(
        res["sum_rel_err_comp_f32"] <= res["sum_rel_err_naive_f64"] * 1.0000001 + 1e-300
        and res["dot_rel_err_comp_f32"] <= res["dot_rel_err_naive_f64"] * 1.0000001 + 1e-300)
    res["scan_comp_f32_err_over_f32_rounding_floor"] = round(
        res["scan_maxerr_over_abs_comp_f32"] / max(res["scan_maxerr_over_abs_f32_rounding_floor"], 1e-300), 3)
    return res


def bench_batched(lib, reps=5, seed=4):
    """4096 uneven loops (lognormal median 2000, sigma 1.5, clipped to
    [32, 2^20]): fp32 axpy + per-loop ReduceSum, one persistent autotuned
    launch (and a CUDA graph of it) against one launch per loop issued from
    C++ (the ordered WorkGroup runner's schedule)."""
    import numpy as np
    import torch

    import raja_gb300 as rg
    rng = np.random.default_rng(seed)
    lens = np.clip(np.round(np.exp(rng.normal(np.log(2000), 1.5, 4096))), 32, 1 << 20).astype(np.int64)
    total = int(lens.sum())
    x = torch.rand(total, device="cuda") * 2 - 1
    y = torch.rand(total, device="cuda") * 2 - 1
    offs = np.concatenate([[0], np.cumsum(lens)])
    px = torch.tensor([x.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    py = torch.tensor([y.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    sums = torch.zeros(len(lens), dtype=torch.float64, device="cuda")
    plan = rg.BatchPlan(lens)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    rg.batched_axpy_sum(plan, 1e-3, px, py, sums, autotune=True)
    info = plan.info()

    # one launch per loop in enqueue order, the schedule of RAJA's ordered
    # WorkGroup runner, issued from C++ (no per-loop Python cost)
    import ctypes as C
    h_lens = (C.c_int64 * len(lens))(*[int(v) for v in lens])
    h_x = (C.c_void_p * len(lens))(*[x.data_ptr() + 4 * int(o) for o in offs[:-1]])
    h_y = (C.c_void_p * len(lens))(*[y.data_ptr() + 4 * int(o) for o in offs[:-1]])

    def plain():
        rc = lib.b200_loops_axpy_sum_f32(len(lens), h_lens, C.c_float(1e-3), h_x, h_y,
                                         sums.data_ptr(), 1, s)
        if rc != 0:
            raise RuntimeError(f"b200_loops_axpy_sum_f32: status {rc}")

    def batched():
        lib.b200_batched_axpy_sum_f32(plan.handle, 1e-3, px.data_ptr(), py.data_ptr(),
                                      sums.data_ptr(), 1, s)

    out = {"loops": len(lens), "total_elems": total, "tile": info["tile"], "block": info["block"]}
    for nm, fn in (("plain_per_loop", plain), ("batched_persistent", batched)):
        fn()
        torch.cuda.synchronize()
        a, b = _events()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        out[nm + "_ms"] = round(a.elapsed_time(b) / reps, 4)
    # graph of `reps` batched sweeps
    cs = torch.cuda.Stream()
    with torch.cuda.stream(cs):
        gph = rg.Graph(cs)
        with gph:
            for _ in range(reps):
                lib.b200_batched_axpy_sum_f32(plan.handle, 1e-3, px.data_ptr(), py.data_ptr(),
                                              sums.data_ptr(), 1, cs.cuda_stream)
        gph.launch()
        cs.synchronize()
        a, b = _events()
        a.record(cs)
        gph.launch()
        b.record(cs)
        cs.synchronize()
        out["batched_graph_ms"] = round(a.elapsed_time(b) / reps, 4)
        gph.close()
    out["speedup_batched_vs_plain"] = round(out["plain_per_loop_ms"] / out["batched_persistent_ms"], 2)
    out["speedup_graph_vs_plain"] = round(out["plain_per_loop_ms"] / out["batched_graph_ms"], 2)
    out["batched_gbs"] = round(12 * total / out["batched_graph_ms"] / 1e6, 1)
    peak = load_peaks().get("hbm_gbs")
    if peak:
        out["batched_frac_of_measured_hbm"] = round(out["batched_gbs"] / peak, 3)
    # per-loop sum error (compensated FP32) vs naive FP64 over the same y
    import oracle
    yh = y.cpu().numpy()
    sh = sums.cpu().numpy()
    worst_c, worst_d = 0.0, 0.0
    for i in range(0, len(lens), 64):
        seg = yh[offs[i]:offs[i + 1]]
        ex, lo = oracle.exact_sum(seg)
        d = oracle.reduce_sum(seg.astype(np.float64))
        den = float(np.abs(seg.astype(np.float64)).sum()) or 1.0
        worst_c = max(worst_c, abs((sh[i] - ex) - lo) / den)
        worst_d = max(worst_d, abs((d - ex) - lo) / den)
    out["sum_err_over_abs_comp_f32"] = worst_c
    out["sum_err_over_abs_naive_f64_seq"] = worst_d
    # segmented scan (int32) and sort (u32) over 10,000 Pareto(1.5) segments
    seg = np.minimum(np.floor(32 * (1 - rng.random(10000)) ** (-1 / 1.5)), 1 << 20).astype(np.int64)
    splan = rg.BatchPlan(seg)
    st = splan.total
    v = torch.randint(0, 1 << 20, (st,), device="cuda", dtype=torch.int32)
    o = torch.empty_like(v)
    k = torch.randint(-2 ** 31, 2 ** 31, (st,), device="cuda", dtype=torch.int32)
    kk = k.clone()
    soffs = splan.offsets

    def segscan():
        lib.b200_segmented_scan_inclusive_i32(splan.handle, v.data_ptr(), o.data_ptr(), s)

    def segscan_plain():
        for i in range(len(seg)):
            a0, n0 = int(soffs[i]), int(seg[i])
            lib.b200_scan_inclusive_i32(v.data_ptr() + 4 * a0, o.data_ptr() + 4 * a0, n0, 0, s)

    def segsort():
        kk.copy_(k)
        lib.b200_segmented_sort_keys_u32(splan.handle, kk.data_ptr(), 0, s)

    def segsort_plain():
        kk.copy_(k)
        for i in range(len(seg)):
            a0, n0 = int(soffs[i]), int(seg[i])
            lib.b200_sort_keys_u32(kk.data_ptr() + 4 * a0, n0, 0, s)

    out["segments"] = len(seg)
    out["segment_elems"] = int(st)
    for nm, fn in (("segscan_one_launch", segscan), ("segscan_per_segment", segscan_plain),
                   ("segsort_batched", segsort), ("segsort_per_segment", segsort_plain)):
        fn()
        torch.cuda.synchronize()
        a, b = _events()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out[nm + "_ms"] = round(a.elapsed_time(b), 4)
    plan.close()
    splan.close()
    return out


def bench_jacobi(lib, sweeps=20, seed=5):
    """256 fp64 meshes with edges in {16..128}, 20 Jacobi 7-point sweeps
    with a per-mesh max residual: per-mesh launches vs one fused launch per
    sweep vs a CUDA graph of the 20 fused sweeps; plus one 512^3 mesh."""
    import numpy as np
    import torch

    import raja_gb300 as rg
    rng = np.random.default_rng(seed)
    shapes = [tuple(int(v) for v in r) for r in rng.integers(16, 129, (256, 3))]
    plan = rg.JacobiPlan(shapes)
    u = torch.rand(plan.total, dtype=torch.float64, device="cuda")
    un = u.clone()
    res = torch.zeros(sweeps * len(shapes), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    offs = plan.offsets

    def plain():
        for sw in range(sweeps):
            src, dst = (u, un) if sw % 2 == 0 else (un, u)
            for m, (a0, b0, c0) in enumerate(shapes):
                o = int(offs[m])
                lib.b200_jacobi_mesh_sweep_f64(a0, b0, c0, src.data_ptr() + 8 * o, dst.data_ptr() + 8 * o, None,
                                               res.data_ptr() + 8 * (sw * len(shapes) + m), s)

    def fused():
        for sw in range(sweeps):
            src, dst = (u, un) if sw % 2 == 0 else (un, u)
            lib.b200_jacobi_sweep_f64(plan.handle, src.data_ptr(), dst.data_ptr(), None,
                                      res.data_ptr() + 8 * sw * len(shapes), s)

    out = {"meshes": len(shapes), "sweeps": sweeps, "interior_points": plan.interior_points()}
    for nm, fn in (("plain_per_mesh", plain), ("fused", fused)):
        fn()
        torch.cuda.synchronize()
        a, b = _events()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out[nm + "_ms"] = round(a.elapsed_time(b), 4)
    cs = torch.cuda.Stream()
    with torch.cuda.stream(cs):
        gph = rg.Graph(cs)
        with gph:
            for sw in range(sweeps):
                src, dst = (u, un) if sw % 2 == 0 else (un, u)
                lib.b200_jacobi_sweep_f64(plan.handle, src.data_ptr(), dst.data_ptr(), None,
                                          res.data_ptr() + 8 * sw * len(shapes), cs.cuda_stream)
        gph.launch()
        cs.synchronize()
        a, b = _events()
        a.record(cs)
        gph.launch()
        b.record(cs)
        cs.synchronize()
        out["fused_graph_ms"] = round(a.elapsed_time(b), 4)
        gph.close()
    out["speedup_graph_vs_plain"] = round(out["plain_per_mesh_ms"] / out["fused_graph_ms"], 2)
    out["fused_gbs_16B_per_point"] = round(16 * out["interior_points"] * sweeps / out["fused_graph_ms"] / 1e6, 1)
    plan.close()
    del u, un
    # one 512^3 mesh, 20 sweeps
    big = rg.JacobiPlan([(512, 512, 512)])
    u = torch.rand(big.total, dtype=torch.float64, device="cuda")
    un = u.clone()
    r = torch.zeros(1, dtype=torch.float64, device="cuda")

    def big_sweeps():
        for sw in range(sweeps):
            src, dst = (u, un) if sw % 2 == 0 else (un, u)
            lib.b200_jacobi_sweep_f64(big.handle, src.data_ptr(), dst.data_ptr(), None, r.data_ptr(), s)

    big_sweeps()
    torch.cuda.synchronize()
    a, b = _events()
    a.record(stream)
    big_sweeps()
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    out["mesh512_ms_per_sweep"] = round(ms / sweeps, 4)
    out["mesh512_gbs_16B_per_point"] = round(16 * big.interior_points() * sweeps / ms / 1e6, 1)
    out["mesh512_gpoints_per_s"] = round(big.interior_points() * sweeps / ms / 1e6, 2)
    big.close()
    return out


def load_cub_arm():
    """baseline/libcubarm.so (built here if missing): CUB's DeviceScan and
    DeviceRadixSort, the calls RAJA's CUDA scan and sort make."""
    import ctypes as C
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "build_cub_arm", os.path.join(ROOT, "baseline", "build_cub_arm.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    lib = C.CDLL(mod.build())
    lib.cub_arm_error.restype = C.c_char_p
    lib.cub_arm_setup.argtypes = [C.c_size_t]
    for nm in ("cub_exclusive_scan_i64", "cub_sort_keys_u32", "cub_sort_keys_u64"):
        getattr(lib, nm).argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.cub_sort_pairs_f32_i32.argtypes = [C.c_void_p] * 4 + [C.c_size_t, C.c_void_p]
    return lib


def bench_cub(inputs, outs, n, stream, reps):
    """CUB on the same inputs as the library's scan and sorts, CUDA events
    over `reps` calls after one warm-up; each result is compared with the
    library's (already in `outs`).  Returns {primitive: {ms, equal}}."""
    import torch
    cub = load_cub_arm()
    if cub.cub_arm_setup(n) != 0:
        raise RuntimeError(cub.cub_arm_error().decode())
    s = stream.cuda_stream
    P = lambda x: x.data_ptr()  # noqa: E731
    o = {k: torch.empty_like(outs[k]) for k in ("scan_out", "u32_out", "u64_out", "pk_out", "pv_out")}
    calls = {
        "exclusive_scan_i64": (lambda: cub.cub_exclusive_scan_i64(P(inputs["scan_in"]), P(o["scan_out"]), n, s),
                               ["scan_out"]),
        "sort_u32": (lambda: cub.cub_sort_keys_u32(P(inputs["u32"]), P(o["u32_out"]), n, s), ["u32_out"]),
        "sort_u64": (lambda: cub.cub_sort_keys_u64(P(inputs["u64"]), P(o["u64_out"]), n, s), ["u64_out"]),
        "sort_pairs_f32_i32": (lambda: cub.cub_sort_pairs_f32_i32(P(inputs["pk"]), P(o["pk_out"]), P(inputs["pv"]),
                                                                  P(o["pv_out"]), n, s), ["pk_out", "pv_out"]),
    }
    res = {}
    for name, (fn, keys) in calls.items():
        if fn() != 0:
            raise RuntimeError(cub.cub_arm_error().decode())
        a, b = _events()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        eq = all(torch.equal(o[k].view(torch.uint8), outs[k].view(torch.uint8)) for k in keys)
        res[name] = {"ms": round(a.elapsed_time(b) / reps, 4), "equal": bool(eq)}
    cub.cub_arm_teardown()
    del o
    torch.cuda.empty_cache()
    return res


def bench_raja_api(lib):
    """The batched forms through the RAJA API on the b200 policies: forall
    over an IndexSet of 10,000 Pareto(1.5) segments (one launch for the
    whole set against one launch per segment; all-range sets and sets mixing
    range, strided and list segments), and a WorkGroup of 4096 lognormal
    loops with per-loop ReduceSum<b200_reduce, float> (one unordered run,
    fixed and tuned shape, synchronous and queued, against the ordered
    one-launch-per-loop run).
    The lambda bodies are C++ (tests/cpp/bench_raja_api.cu), built here
    with nvcc against the library."""
    import raja_gb300.build as b
    lib_path = b.build()
    out_dir = os.path.join(b.BUILD)
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "bench_raja_api")
    src = os.path.join(ROOT, "tests", "cpp", "bench_raja_api.cu")
    import glob
    deps = [src, lib_path] + glob.glob(os.path.join(ROOT, "include", "raja_b200", "*.hpp"))
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
        cmd = [b.nvcc(), "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr", "-O2", *b.ARCH,
               f"-I{ROOT}/include/raja_compat", f"-I{ROOT}/include", src, "-o", exe,
               f"-L{os.path.dirname(lib_path)}", "-lb200prims", "-Xlinker",
               f"-rpath={os.path.dirname(lib_path)}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("bench_raja_api build failed: " + r.stderr[-500:])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    if r.returncode != 0:
        raise RuntimeError("bench_raja_api failed: " + (r.stdout + r.stderr)[-500:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# bytes each launch of a named kernel moves, by the fixed convention
def kernel_bytes(name: str, n: int):
    per = {
        "b200_onesweep_k32": 2 * 4 * n,            # read + write every key once
        "b200_onesweep_k64": 2 * 8 * n,
        "b200_onesweep_k32_v32": 2 * 4 * n + 2 * 4 * n,
        "b200_sort_hist": None,                   # key read (bytes differ per key width)
        "b200_scan_exclusive_i64": 16 * n,
        "b200_reduce_sum_f32": 4 * n, "b200_reduce_sum_f64": 8 * n,
        "b200_reduce_minloc_f32": 4 * n, "b200_reduce_maxloc_f32": 4 * n,
        "b200_reduce_minloc_f64": 8 * n, "b200_reduce_maxloc_f64": 8 * n,
        "b200_histogram": 4 * n,
    }
    return per.get(name)


def roofline(kernels: dict, n: int, peak: float, src: str) -> dict:
    if not kernels:
        return None
    top = max(kernels.items(), key=lambda kv: kv[1]["ms_per_step"])
    total = sum(v["ms_per_step"] for v in kernels.values())
    name, v = top
    per_launch_bytes = kernel_bytes(name, n)
    avg_ms = v["ms_per_step"] / max(v["launches_per_step"], 1)
    achieved = per_launch_bytes / avg_ms / 1e6 if per_launch_bytes else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(tp) as f:
            tr = json.load(f)
        if name in tr:
            # captured on a smaller case; traffic scales with the units processed
            traffic = int(tr[name]["bytes_per_launch"] * n / tr[name]["n"])
    except (OSError, ValueError, KeyError):
        pass
    return {"kernel": name, "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None, "peak": peak,
            "peak_source": src, "unit": "GB/s",
            "frac": round(achieved / peak, 3) if achieved else None,
            "traffic": traffic, "algorithmic_bytes_per_launch": per_launch_bytes,
            "avg_launch_ms": round(avg_ms, 4),
            "share_of_step": round(v["ms_per_step"] / total, 3) if total else None}


# Inputs and outputs of each primitive of the step (keys of make_inputs /
# make_outputs), in step order.
E2E_PLAN = [
    ("reduce_sum_f32", ["f32"], ["sum"]), ("reduce_sum_f64", ["f64"], ["sum"]),
    ("minloc_f32", ["f32"], ["loc_f32", "idx"]), ("maxloc_f32", ["f32"], ["loc_f32", "idx"]),
    ("minloc_f64", ["f64"], ["loc_f64", "idx"]), ("maxloc_f64", ["f64"], ["loc_f64", "idx"]),
    ("exclusive_scan_i64", ["scan_in"], ["scan_out"]),
    ("sort_u32", ["u32"], ["u32_out"]), ("sort_u64", ["u64"], ["u64_out"]),
    ("sort_pairs_f32_i32", ["pk", "pv"], ["pk_out", "pv_out"]),
    ("histogram_256", ["z256"], ["h256"]), ("histogram_65536", ["z65536"], ["h65536"]),
]


def run_e2e(args, lib, inputs, outs, n, stream, table, dist):
    """Same step through the C ABI with host buffers: every step copies its
    inputs host->device from pinned memory and reads every result back.
    The copies run on two copy streams and overlap the primitives: each
    primitive waits for its own inputs only, its outputs are copied back as
    soon as it finishes, and events keep a buffer from being overwritten
    while an earlier step still reads it or copies it back.  Steps alternate
    between two sets of device buffers, so one step's inputs stream in while
    the step before it still computes and copies its results out (the host
    link carries both directions at once: 343 GB/s together, against 211
    GB/s in and 194 GB/s out alone)."""
    import torch
    keys_in = ["f32", "f64", "scan_in", "u32", "u64", "pk", "pv", "z256", "z65536"]
    host = {k: torch.empty(inputs[k].shape, dtype=inputs[k].dtype, pin_memory=True)
            for k in keys_in}
    for k in keys_in:
        host[k].copy_(inputs[k])
    out_keys = ["scan_out", "u32_out", "u64_out", "pk_out", "pv_out", "sum", "loc_f32",
                "loc_f64", "idx", "h256", "h65536"]
    host_out = {k: torch.empty(outs[k].shape, dtype=outs[k].dtype, pin_memory=True)
                for k in out_keys}
    h2d = sum(host[k].numel() * host[k].element_size() for k in keys_in)
    d2h = sum(host_out[k].numel() * host_out[k].element_size() for k in out_keys)
    inputs2 = {k: torch.empty_like(inputs[k]) for k in keys_in}
    outs2 = {k: torch.empty_like(outs[k]) for k in out_keys}
    sets = [(inputs, outs, dict(step_calls(lib, inputs, outs, n, stream.cuda_stream))),
            (inputs2, outs2, dict(step_calls(lib, inputs2, outs2, n, stream.cuda_stream)))]
    last_out = {}                       # output key -> index of its last writer
    for i, (_, _, os_) in enumerate(E2E_PLAN):
        for k in os_:
            last_out[k] = i
    h2d_s, d2h_s = torch.cuda.Stream(), torch.cuda.Stream()
    states = [{"in_free": {}, "out_free": {}}, {"in_free": {}, "out_free": {}}]

    def ev(s):
        e = torch.cuda.Event()
        e.record(s)
        return e

    def one(step, start=None):
        inputs, outs, calls = sets[step % 2]
        state = states[step % 2]
        in_free, out_free = state["in_free"], state["out_free"]
        ready = {}
        if start is not None:
            h2d_s.wait_event(start)
        for k in keys_in:
            if k in in_free:
                h2d_s.wait_event(in_free[k])
            with torch.cuda.stream(h2d_s):
                inputs[k].copy_(host[k], non_blocking=True)
            ready[k] = ev(h2d_s)
        nxt_in, nxt_out = {}, {}
        for i, (name, ins, os_) in enumerate(E2E_PLAN):
            for k in ins:
                stream.wait_event(ready[k])
            for k in os_:
                if k in out_free:
                    stream.wait_event(out_free.pop(k))
            if name.startswith("histogram"):
                outs[os_[0]].zero_()
            rc = calls[name]()
            if rc != 0:
                from raja_gb300 import _lib
                _lib.check(name, rc)
            done = ev(stream)
            for k in ins:
                nxt_in[k] = done
            for k in os_:
                if last_out[k] == i:
                    d2h_s.wait_event(done)
                    with torch.cuda.stream(d2h_s):
                        host_out[k].copy_(outs[k], non_blocking=True)
                    nxt_out[k] = ev(d2h_s)
        state["in_free"], state["out_free"] = nxt_in, nxt_out

    one(0)
    one(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for i in range(args.e2e_steps):
        one(i, start=a if i == 0 else None)
    stream.wait_stream(d2h_s)
    stream.wait_stream(h2d_s)
    b.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(a.elapsed_time(b), dist, "cuda")
    world = dist.get_world_size() if dist else 1
    value = aggregate_gbs(world, sum(table.values()), args.e2e_steps, ms)
    link = link_probe([(host[k], inputs[k]) for k in keys_in], [(host_out[k], outs[k]) for k in out_keys],
                      h2d_s, d2h_s)
    # the step's copies alone, both directions at once, bound the step
    bound_ms = link["all_copies_ms"]
    link["copy_bound_ms_per_step"] = round(bound_ms, 2)
    link["e2e_frac_of_copy_bound"] = round(bound_ms / (ms / args.e2e_steps), 3)
    return {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
            "ms_per_step": round(ms / args.e2e_steps, 3), "host_link": link,
            "path": "pinned host -> device copies (copy stream), C-ABI calls, device -> pinned "
                    "host copies (second copy stream), overlapped per primitive; steps alternate "
                    "between two sets of device buffers"}


def link_probe(ins, outs, h2d_s, d2h_s):
    """Host-link rates right after the end-to-end run, on the step's own
    pinned buffers: every input host-to-device alone, every result
    device-to-host alone, and both at once (the rates can differ between
    host buffers, so the probe covers all of them)."""
    import torch
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    torch.cuda.synchronize()
    nb_in = sum(h.numel() * h.element_size() for h, _ in ins)
    nb_out = sum(h.numel() * h.element_size() for h, _ in outs)

    def timed(do_in, do_out):
        a, b = ev(), ev()
        a.record(h2d_s)
        d2h_s.wait_event(a)
        if do_in:
            with torch.cuda.stream(h2d_s):
                for h, d in ins:
                    d.copy_(h, non_blocking=True)
        if do_out:
            with torch.cuda.stream(d2h_s):
                for h, d in outs:
                    h.copy_(d, non_blocking=True)
        h2d_s.wait_stream(d2h_s)
        b.record(h2d_s)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    t_in, t_out, t_both = timed(True, False), timed(False, True), timed(True, True)
    return {"h2d_gbs": round(nb_in / t_in / 1e9, 1), "d2h_gbs": round(nb_out / t_out / 1e9, 1),
            "bidir_gbs": round((nb_in + nb_out) / t_both / 1e9, 1),
            "all_copies_ms": round(1e3 * t_both, 2)}


def run_cpu_baseline(args):
    """One pass over every primitive at N=2^cpu_log2n (the same N as the
    device step by default) on all host cores, after one untimed pass."""
    import oracle
    oracle.build()
    n = 1 << args.cpu_log2n
    suite = CpuSuite(n, seed=1)
    t_gen = time.perf_counter()
    per, _ = cpu_suite_rotation(suite, len(suite.names), len(suite.names))
    ts = sum(per.values())
    value = sum(suite.table.values()) / ts / 1e9
    return {"value": round(value, 3), "unit": UNIT, "cores": oracle.max_threads(), "kind": "port",
            "sample": f"one timed pass of every primitive at N=2^{args.cpu_log2n} after one "
                      f"untimed pass (oracle OpenMP restatement of omp_parallel_for_exec), "
                      f"CPU {cpu_model()}",
            "seconds": round(ts, 2), "wall_s_with_setup": round(time.perf_counter() - t_gen, 1),
            "primitives_gbs": {nm: round(suite.table[nm] / per[nm] / 1e9, 3) for nm in suite.names}}


if __name__ == "__main__":
    main()
