"""Benchmark of the voxelization hot path (one JSON line on stdout).

Workload (one "step"): the displaced icosphere subdivided 8 times (1,310,720 fp32 triangles, seeded
synthetic mesh) voxelized at 512^3 four times -- surface and solid, linear and Morton order -- each
into a freshly zeroed bit table.  Metric: Mtris/s (triangles voxelized per second, 4 x 1.31M per
step).  Inputs (47 MB of triangles, 4 x 16 MiB of tables) are smaller than the 129 MB L2, so L2 is
flushed (a 512 MiB write) between timed steps, outside the timed region.  `value` times the step as
one cvx_plan (the four jobs captured once as a CUDA graph; the graph clears the tables).

Keys beyond the base contract:
  e2e          the same metric through the public host-buffer path: pinned host triangles copied in,
               four voxelizations, four tables copied out, all inside the timed region, as one
               cvx_plan_create_host graph launch per step (chunked upload, tables read back as soon
               as each is complete), K steps back to back on two such plans with their own buffers,
               launched on two streams in turn (one step's upload overlaps the previous step's
               read-back); single_step is one plan's round trip timed alone, plain_calls the same
               round trip through per-call API calls.
  step_per_call the four drop-in calls on four streams, enqueued from Python every step.
  step_sequential the four drop-in calls one after another on one stream.
  roofline     the step's dominant kernel against the measured HBM copy bandwidth
               (MEASURED_PEAKS.json), with DRAM traffic from the committed ncu summary when present.
  cpu_baseline the reference's own CPU voxelizer (src/cpu_voxelizer.cpp, OpenMP with a critical section
               per bit, built on this host by oracle/build_ref.sh; the oracle port where that build
               is missing) on the same workload, all 4 modes, at the host's fastest thread count
               (the whole mesh when it fits about 20 s; the solid modes without the triangles its
               solid loop could run outside its table, oracle/ref_safety.py).
  extras       the triangle-size stress soup (2M triangles at 1024^3; the reference CUDA kernel rebuilt
               for sm_103a is timed on it by --impl reference), the 256-mesh batched workload against
               plain per-mesh calls, and open-loop serving of that mix (Poisson arrivals, 40 GiB
               budget, p50/p99) against one-request-at-a-time launches.

--impl reference times the reference's CPU implementation of the path (its own build, as for
cpu_baseline) on the same workload, the whole mesh per step whenever the run fits about two minutes
(else the first 1/2^k of the triangles); it builds its voxinfo with the oracle's restatement of the
reference's setup and loads nothing of the engine.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

MODES = [(False, False), (True, False), (False, True), (True, True)]  # (morton, solid)
METRIC = "Mtris/s voxelized (icosphere 1.31M tris, 512^3, surface+solid x linear+Morton)"
SAMPLE_FRACTION = 32
E2E_SLOTS = 2  # host plans in flight in the e2e measurement
THREADS_NOTE = ("the fastest thread count on this host (seconds per thread count on a 1/128 calibration "
                "sample in threads_tried_s): the reference's OpenMP loop takes a critical section per bit")


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["engine", "reference"], default="engine")
    p.add_argument("--no-extras", action="store_true", help="skip the soup / batch / serve side measurements")
    p.add_argument("--profile-case", choices=sorted(PROFILE_CASES),
                   help="run one named workload 1 + --reps times for a profiler, then exit (no JSON line)")
    p.add_argument("--reps", type=int, default=1, help="runs after the warm-up run of --profile-case")
    p.add_argument("--serve-seconds", type=float, default=2.0,
                   help="length of the open-loop serving runs at 25%% and 50%% load and of the plain arms")
    p.add_argument("--serve-long-seconds", type=float, default=60.0,
                   help="length of the served arms' runs at 75%% and 90%% load (the served configuration: 60 s "
                        "per rate)")
    return p.parse_args(argv)


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        """Starts sampling and returns once the first sample has arrived, so that the timed region
        that follows is covered."""
        self.lines = []
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            first = self.proc.stdout.readline()
            if first:
                self.lines.append(first)
            self.reader = threading.Thread(target=self._drain, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None
        return self

    def _drain(self):
        for line in self.proc.stdout:
            self.lines.append(line)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.reader.join(timeout=5)
        self.out = "".join(self.lines)

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class NvmlClockSampler:
    """The same record as ClockSampler, sampled in-process through NVML (libnvidia-ml, read-only
    queries) every `period_s`, so that a timed region of a few milliseconds still gets dozens of
    samples.  Falls back to ClockSampler where NVML cannot be loaded."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index: int, period_s: float = 0.001):
        self.index = index
        self.period = period_s
        self.fallback = None

    def __enter__(self):
        import ctypes
        self.samples = []
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit failed")
            h = ctypes.c_void_p()
            if nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
                raise OSError("no NVML handle")
            reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint()
            nv.nvmlDeviceGetMaxClockInfo(h, self.SM, ctypes.byref(mx))
            self.max_mhz = float(mx.value)
        except (OSError, AttributeError):
            self.fallback = ClockSampler(self.index).__enter__()
            return self
        self.nv, self.h, self.reasons_fn = nv, h, reasons_fn
        self.stop = threading.Event()

        def loop():
            mhz = ctypes.c_uint()
            rs = ctypes.c_ulonglong()
            while not self.stop.is_set():
                if nv.nvmlDeviceGetClockInfo(h, self.SM, ctypes.byref(mhz)) == 0 and \
                        reasons_fn(h, ctypes.byref(rs)) == 0:
                    self.samples.append((float(mhz.value), int(rs.value)))
                time.sleep(self.period)

        self.thread = threading.Thread(target=loop, daemon=True)
        self.thread.start()
        while not self.samples and self.thread.is_alive():  # covered from the first sample on
            time.sleep(self.period)
        return self

    def __exit__(self, *a):
        if self.fallback:
            return self.fallback.__exit__(*a)
        self.stop.set()
        self.thread.join(timeout=5)
        self.nv.nvmlShutdown()

    def summary(self):
        if self.fallback:
            return self.fallback.summary()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        reasons = sorted({name for _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(m for m, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples), "source": "nvml, 1 ms period"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(kernel: str):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


def issue_roofline(kernel, per_launch_ms, clocks):
    """The dominant kernel against its instruction-issue bound: its warp instructions per launch
    (ncu, profiles/traffic.json) at 4 per SM per cycle on every SM at the measured clock."""
    import torch
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            inst = json.load(f)["warp_instructions"][kernel]
    except Exception:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    t_issue = inst / (sms * 4 * mhz * 1e6)
    return {"warp_instructions_per_launch": inst, "sms": sms, "sm_mhz": mhz, "t_issue_us": t_issue * 1e6,
            "t_measured_us": per_launch_ms * 1e3, "frac": t_issue / (per_launch_ms / 1e3)}


def step_roofline(cv, torch, T, table_bytes, hbm_gbs, ms_per_step):
    """Roofline of one step by bytes and atomics.  The 4 calls run concurrently and share HBM and
    the L2 atomic units, so t = max(sum B / BW, sum A / R_atom) with per call B = 36 T + table
    (+ table again for the solid flip table) and A the exact atomic count of the workload
    (profiles/atomic_terms.json, counted by the oracle); R_atom is the scattered 32-bit atomicOr
    rate measured here on a 128 MiB table."""
    from cuda_voxelizer_gb300 import _lib
    try:
        with open(os.path.join(ROOT, "profiles", "atomic_terms.json")) as f:
            terms = json.load(f)["icosphere_l8_512"]
    except Exception:
        return None
    words = 32 << 20
    buf = torch.zeros(words, dtype=torch.int32, device="cuda")
    r_atom = max(_lib.diag_lib().cvx_microbench_atomic_or(buf.data_ptr(), words, 0, 152 * 8, 64) for _ in range(3))
    del buf
    calls, sum_b, sum_a = {}, 0.0, 0.0
    for (morton, solid), name in zip(MODES, ("surface_linear", "surface_morton", "solid_linear", "solid_morton")):
        b = 36 * T + table_bytes * (2 if solid else 1)
        a = int(terms[name])
        tb, ta = b / (hbm_gbs * 1e9), a / r_atom
        calls[name] = {"bytes": b, "atomics": a, "t_bytes_us": tb * 1e6, "t_atomics_us": ta * 1e6}
        sum_b += tb
        sum_a += ta
    t_roof = max(sum_b, sum_a)
    return {"definition": "max(sum over the 4 calls of B/BW_hbm, sum of A/R_atom)", "r_atom_per_s": r_atom,
            "hbm_gbs": hbm_gbs, "calls": calls, "t_roof_us": t_roof * 1e6, "t_measured_us": ms_per_step * 1e3,
            "frac": t_roof / (ms_per_step / 1e3)}


def cpu_sample(tris, fraction=SAMPLE_FRACTION):
    """The first 1/fraction of the mesh's triangles (fraction 1: the whole mesh)."""
    n = tris.shape[0] // fraction
    return np.ascontiguousarray(tris[:n])


def cpu_work(info_bytes, tris):
    """The triangles the CPU legs give the reference's code in each of the 4 modes: all of them for
    surface; for solid, those oracle/ref_safety.py keeps (about 1% of the icosphere is dropped: the
    reference's solid loop can start its run at a negative or out-of-table x on the others and
    write outside its table -- its CPU loop stores a negative xmax in an unsigned int)."""
    import oracle
    from oracle.ref_safety import safe_triangles
    out = []
    for morton, solid in MODES:
        if solid:
            keep = safe_triangles(tris, oracle.with_count(info_bytes, tris.shape[0]), morton)
            out.append(np.ascontiguousarray(tris[keep]))
        else:
            out.append(tris)
    return out


def cpu_fraction(pass_s, passes, budget_s):
    """The largest power-of-two share 1/f of the workload (f = 1, 2, 4, ..., SAMPLE_FRACTION) whose
    `passes` runs fit `budget_s`, given the estimated seconds of one pass over the whole workload."""
    f = 1
    while f < SAMPLE_FRACTION and passes * pass_s / f > budget_s:
        f *= 2
    return f


def sample_desc(work, total, kind, fraction=SAMPLE_FRACTION):
    what = ("the whole workload" if fraction == 1 else
            f"the first 1/{fraction} of the triangles of the same mesh and grid")
    solid = work[2].shape[0]
    return (f"{what}, 4 modes: {work[0].shape[0]} triangles per surface mode, {solid} per solid mode (the "
            f"{work[0].shape[0] - solid} the reference's solid loop could run outside its table left out, "
            f"oracle/ref_safety.py); "
            + ("the reference's own src/cpu_voxelizer.cpp built on this host (OpenMP parallel-for, a critical "
               "section per bit)" if kind == "reference" else
               "the oracle port of src/cpu_voxelizer.cpp (OpenMP parallel-for, a critical section per bit)"))


def _omp_threads(n):
    """Thread count of the OpenMP parallel regions this thread starts next, in the OpenMP runtime
    the reference's CPU build links (libgomp): OMP_NUM_THREADS is read only once, at its first
    parallel region."""
    import ctypes
    os.environ["OMP_NUM_THREADS"] = str(n)
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(ctypes.c_int(int(n)))
    except (OSError, AttributeError):
        pass


def time_cpu_reference(info_bytes, work, threads):
    """The reference CPU algorithm over the 4 modes, mode i on the triangles work[i] (cpu_work; same
    grid); returns seconds.  Runs the reference's own build where it exists on this host, else the
    oracle port of it (same structure: OpenMP over triangles, a critical section per bit write)."""
    import oracle
    _omp_threads(threads)
    infos = [oracle.with_count(info_bytes, w.shape[0]) for w in work]
    t0 = time.perf_counter()
    for (morton, solid), w, info_s in zip(MODES, work, infos):
        if oracle.ref_cpu_available():
            oracle.ref_cpu_voxelize(info_s, w, morton=morton, solid=solid, quiet=True)
        else:
            oracle.voxelize_omp(info_s, w, morton=morton, solid=solid, threads=threads)
    return time.perf_counter() - t0


def cpu_threads(info_bytes, tris, max_threads):
    """The thread count the CPU legs run the reference's algorithm with: the fastest of 1, 2, 4, ...
    and all of this host's threads on a 1/128 sample (best of two runs each).  Its OpenMP loop takes
    a critical section for every bit it sets, so on this workload more threads can be slower than
    one; timing it with all threads regardless would understate the reference.  Returns (threads,
    {threads: seconds on the calibration sample}, estimated seconds of one pass over the whole
    workload at that thread count)."""
    small = cpu_work(info_bytes, np.ascontiguousarray(tris[:max(1024, tris.shape[0] // 128)]))
    cands = sorted({t for t in (1, 2, 4, 8, 16, 32, 64) if t < max_threads} | {max_threads})
    secs = {}
    for t in cands:
        time_cpu_reference(info_bytes, small, t)
        secs[t] = min(time_cpu_reference(info_bytes, small, t) for _ in range(2))
    best = min(secs, key=secs.get)
    return best, {str(t): round(v, 4) for t, v in secs.items()}, secs[best] * tris.shape[0] / small[0].shape[0]


def load_meshgen():
    """The seeded mesh generators, loaded from their file so that the reference arm does not import
    the engine's package (which loads libcvx.so)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_cvx_meshgen", os.path.join(ROOT, "cuda_voxelizer_gb300",
                                                                               "meshgen.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def reference_voxinfo(tris, g):
    """main()'s voxinfo setup (src/main.cpp:179-186) through the oracle's restatement of
    createMeshBBCube and the voxinfo constructor (src/util.h:56-110, pinned against the reference's
    own build by the golden fixtures): vertex bbox, padded to a cube, then a g^3 grid."""
    import oracle
    v = np.asarray(tris, dtype=np.float32).reshape(-1, 3)
    lo, hi = oracle.mesh_bbcube(v.min(axis=0), v.max(axis=0))
    return oracle.info_init(lo, hi, (g, g, g), v.shape[0] // 3)


def run_reference_arm(args, rank, world):
    """--impl reference: the reference's CPU implementation (its own src/cpu_voxelizer.cpp where it
    was built on this host, else the oracle port) over the 4 modes on the cpu_baseline sample, one
    sample per step.  Nothing of the engine (libcvx.so) is loaded."""
    if rank != 0:
        return
    import oracle
    meshgen = load_meshgen()
    tris = meshgen.icosphere(0, level=8)
    info = reference_voxinfo(tris, 512)
    threads, tried, pass_s = cpu_threads(info, tris, os.cpu_count() or 1)
    kind = "reference" if oracle.ref_cpu_available() else "port"
    # each step the whole workload when the run's warm-up and timed steps fit about two minutes,
    # else the largest power-of-two share of it that does
    frac = cpu_fraction(pass_s, args.steps + args.warmup, 120.0)
    work = cpu_work(info, cpu_sample(tris, frac))
    n = sum(w.shape[0] for w in work)
    for _ in range(args.warmup):
        time_cpu_reference(info, work, threads)
    ts = [time_cpu_reference(info, work, threads) for _ in range(args.steps)]
    sec = float(np.mean(ts))
    value = n / sec / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mtris/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced icosphere)",
            "config": {"workload": "icosphere level 8 (1,310,720 tris) at 512^3; surface+solid x linear+Morton "
                                   "per step", "gridsize": 512, "triangles": int(tris.shape[0]),
                       "triangles_per_step": n,
                       "sample": "the whole workload" if frac == 1 else f"first 1/{frac} of the triangles"},
            "cpu_baseline": {"value": value, "unit": "Mtris/s", "cores": threads, "kind": kind,
                             "sample": sample_desc(work, tris.shape[0], kind, frac), "threads_tried_s": tried,
                             "threads_note": THREADS_NOTE},
            "e2e": {"value": value, "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_extras:
        try:
            import torch
            if torch.cuda.is_available():
                line["extras"] = {"soup_1024_ref_cuda": ref_cuda_soup(meshgen)}
        except Exception as e:  # reference kernels not built on this host
            line["extras"] = {"soup_1024_ref_cuda": f"unavailable: {e}"}
    print(json.dumps(line), flush=True)


# ---- named workloads for kernel profiling (--profile-case) ---------------------------------------
# Each builds its seeded synthetic input and returns a function that runs the engine once; main()
# runs it 1 + --reps times, synchronising after each, so that a profiler can skip the warm-up
# launches (ncu -s) and capture the ones after.

def _pc_table(cv, torch, info):
    return torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")


def pc_ico8(cv, meshgen, torch):
    """displaced icosphere, 8 subdivisions (1,310,720 triangles) at 512^3, four calls: surface
    linear, surface Morton, solid linear, solid Morton"""
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tabs = [_pc_table(cv, torch, info) for _ in MODES]

    def run():
        for (morton, solid), tab in zip(MODES, tabs):
            tab.zero_()
            (cv.voxelize_solid if solid else cv.voxelize)(info, d, tab, morton)
    return run


def pc_ico8_plan(cv, meshgen, torch):
    """the benchmark step: the same four jobs as one cvx_plan that clears its tables (clear_ranges)"""
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tabs = [_pc_table(cv, torch, info) for _ in MODES]
    plan = cv.Plan([cv.Job(info, d, t, morton, solid) for (morton, solid), t in zip(MODES, tabs)], clear_tables=True)
    return plan.launch


def pc_soup(cv, meshgen, torch):
    """2,000,000-triangle soup (edges log-uniform in [0.25, 512] voxels) at 1024^3, surface"""
    tris = meshgen.soup(0, n=2_000_000)
    info = cv.make_voxinfo(tris, 1024)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tab = _pc_table(cv, torch, info)

    def run():
        tab.zero_()
        cv.voxelize(info, d, tab)
    return run


def pc_soup_bricks(cv, meshgen, torch):
    """the full soup with the brick rasterizer on (brick_pairs = 16)"""
    cv.set_tuning(torch.cuda.current_device(), brick_pairs=16)
    return pc_soup(cv, meshgen, torch)


def pc_soup200k(cv, meshgen, torch):
    """the first 200,000 triangles of that soup at 1024^3 (a small case of surf_rows and of the brick
    kernels), with the device's current tuning"""
    tris = meshgen.soup(0, n=2_000_000)[:200_000]
    info = cv.make_voxinfo(tris, 1024)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tab = _pc_table(cv, torch, info)

    def run():
        tab.zero_()
        cv.voxelize(info, d, tab)
    return run


def pc_soup200k_bricks(cv, meshgen, torch):
    """the same with the brick rasterizer on (brick_pairs = 16): the larger triangles binned to 32^3
    bricks, rasterized in shared memory, one global atomicOr per non-zero brick word"""
    cv.set_tuning(torch.cuda.current_device(), brick_pairs=16)
    return pc_soup200k(cv, meshgen, torch)


def _pc_mix_jobs(cv, meshgen, torch, select):
    jobs = []
    for spec in meshgen.batch_mix(0, 256):
        if not select(spec):
            continue
        t = spec.build()
        info = cv.make_voxinfo(t, spec.gridsize)
        jobs.append(cv.Job(info, torch.from_numpy(t.reshape(-1)).cuda(), _pc_table(cv, torch, info), spec.morton,
                           spec.solid))
    return jobs


def pc_batch(cv, meshgen, torch):
    """the 256-mesh uneven mix (triangle counts 1k-500k, grids 64-512, 3:1 surface:solid, 1:1
    linear:Morton) as one cvx_voxelize_batch"""
    jobs = _pc_mix_jobs(cv, meshgen, torch, lambda spec: True)

    def run():
        for j in jobs:
            j.table.zero_()
        cv.voxelize_batch(jobs)
    return run


def pc_batch_g512(cv, meshgen, torch):
    """the surface meshes of that mix gridded at 512^3, as one batch"""
    jobs = _pc_mix_jobs(cv, meshgen, torch, lambda spec: not spec.solid and spec.gridsize == 512)

    def run():
        for j in jobs:
            j.table.zero_()
        cv.voxelize_batch(jobs)
    return run


def pc_batch_g512_solid(cv, meshgen, torch):
    """the solid meshes of that mix gridded at 512^3, as one batch"""
    jobs = _pc_mix_jobs(cv, meshgen, torch, lambda spec: spec.solid and spec.gridsize == 512)

    def run():
        for j in jobs:
            j.table.zero_()
        cv.voxelize_batch(jobs)
    return run


def pc_io(cv, meshgen, torch):
    """a random 1024^3 table transcoded linear -> Morton -> linear, then the 512^3 solid icosphere's
    binvox payload and voxel list"""
    gen = torch.Generator(device="cuda").manual_seed(1)
    tab = torch.randint(-2 ** 31, 2 ** 31 - 1, (1024 ** 3 // 32,), dtype=torch.int32, device="cuda", generator=gen)
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    t512 = _pc_table(cv, torch, info)
    cv.voxelize_solid(info, torch.from_numpy(tris.reshape(-1)).cuda(), t512)

    def run():
        m = cv.transcode(tab, 1024, True)
        cv.transcode(m, 1024, False)
        cv.encode_binvox(info, t512)
        cv.encode_voxel_list(info, t512)
    return run


PROFILE_CASES = {"ico8": pc_ico8, "ico8_plan": pc_ico8_plan, "soup": pc_soup, "soup_bricks": pc_soup_bricks,
                 "soup200k": pc_soup200k,
                 "soup200k_bricks": pc_soup200k_bricks,
                 "batch": pc_batch, "batch_g512": pc_batch_g512, "batch_g512_solid": pc_batch_g512_solid,
                 "io": pc_io}


def run_profile_case(name, reps):
    import torch
    import cuda_voxelizer_gb300 as cv
    from cuda_voxelizer_gb300 import meshgen
    run = PROFILE_CASES[name](cv, meshgen, torch)
    for _ in range(1 + reps):
        run()
        torch.cuda.synchronize()
    cv.device_status()
    print(f"{name}: {1 + reps} runs done")


def main():
    args = parse()
    if args.profile_case:
        run_profile_case(args.profile_case, args.reps)
        return
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    import torch
    import cuda_voxelizer_gb300 as cv
    from cuda_voxelizer_gb300 import meshgen

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    # The autotuner's choice of the tuning knobs for this device (results never depend on them),
    # timed once here and cached; every number below runs with it.
    from cuda_voxelizer_gb300 import autotune
    default_tuning = cv.get_tuning(local)
    tuned = autotune.autotune(local, reps=3)
    tuning = {"choice": {k: tuned[k] for k in autotune.KNOBS}, "default": default_tuning,
              "tuning_set_ms": {"tuned": tuned["ms"], "default": tuned["default_ms"]}, "min_gain": tuned["min_gain"],
              "seconds": tuned["seconds"]}
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    T = tris.shape[0]
    W = cv.table_words(info)
    d_tris = torch.from_numpy(tris.reshape(-1)).cuda()
    tables = [torch.empty(W, dtype=torch.int32, device="cuda") for _ in MODES]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step_seq():
        for (morton, solid), tab in zip(MODES, tables):
            tab.zero_()
            (cv.voxelize_solid if solid else cv.voxelize)(info, d_tris, tab, morton)

    # The timed step: the 4 calls on 4 streams (each stream has its own queues and counters in the
    # engine), forked from and joined back into the timing stream.
    side = [torch.cuda.Stream() for _ in MODES]

    def step():
        fork = torch.cuda.Event()
        fork.record(stream)
        for (morton, solid), tab, s in zip(MODES, tables, side):
            s.wait_event(fork)
            with torch.cuda.stream(s):
                tab.zero_()
                (cv.voxelize_solid if solid else cv.voxelize)(info, d_tris, tab, morton, stream=s)
        for s in side:
            stream.wait_stream(s)

    # ---- device-resident throughput: the step as one cvx_plan (the engine's batch form: the 4
    # jobs captured once, tables cleared in-graph by one kernel, surface and solid lanes on parallel
    # captured streams), replayed once per step ----------------------------------------------------
    plan = cv.Plan([cv.Job(info, d_tris, tab, morton, solid) for (morton, solid), tab in zip(MODES, tables)],
                   clear_tables=True)

    def timed_steps(fn, n):
        out = []
        for _ in range(n):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b))
        return out

    for _ in range(max(3, args.warmup)):
        plan.launch()
    torch.cuda.synchronize()
    barrier(world)
    with NvmlClockSampler(local) as clk:
        times = timed_steps(plan.launch, args.steps)
    barrier(world)
    total_ms = max_over_ranks(float(sum(times)), world)
    ms = total_ms / args.steps
    value = world * 4 * T * args.steps / (total_ms / 1e3) / 1e6
    launches_per_step = plan.kernel_nodes()
    plan.close()

    # the same 4 calls through the per-call API: on 4 streams, and one after another on one stream
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    call_ms = float(np.mean(timed_steps(step, min(args.steps, 100))))
    seq_ms = float(np.mean(timed_steps(step_seq, min(args.steps, 100))))
    step_calls = {"ms_per_step": call_ms, "value": 4 * T / (call_ms / 1e3) / 1e6, "unit": "Mtris/s",
                  "note": "the 4 drop-in calls on 4 streams (tables zeroed by torch), enqueued per step"}
    step_seq_line = {"ms_per_step": seq_ms, "value": 4 * T / (seq_ms / 1e3) / 1e6, "unit": "Mtris/s",
                     "note": "the 4 drop-in calls one after another on one stream"}

    # ---- per-kernel times for the roofline ------------------------------------------------------
    cv.profile_enable(True)
    prof = {}
    reps = 5
    for _ in range(reps):
        flush.fill_(1)
        torch.cuda.synchronize()
        step_seq()
        torch.cuda.synchronize()
        for name, t in cv.profile_collect():
            prof.setdefault(name, []).append(t)
    cv.profile_enable(False)
    kernel_ms = {k: float(np.sum(v)) / reps for k, v in prof.items()}
    launches = {k: len(v) // reps for k, v in prof.items()}
    # the engine's kernels in one timed step: the plan graph's kernel nodes
    dom = max(kernel_ms, key=kernel_ms.get)
    # algorithmic bytes per launch: triangles read once (36 B each) + the table (g^3/8) for the
    # classify kernels; flip table read + table write (2 g^3/8) for the solid resolve.
    tbytes = 36 * T
    table_bytes = W * 4
    alg = {"surf_classify": tbytes + table_bytes, "solid_classify": tbytes, "surf_rows": 0, "solid_cols": 0,
           "solid_resolve": 2 * table_bytes, "solid_morton": 2 * table_bytes, "solid_zero": table_bytes}
    per_launch_ms = kernel_ms[dom] / max(1, launches[dom])
    achieved = alg.get(dom, 0) / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = traffic_from_profiles(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "kernel_ms_per_step": kernel_ms, "alg_bytes_per_launch": alg.get(dom, 0),
                "issue": issue_roofline(dom, per_launch_ms, clk.summary()),
                "step": step_roofline(cv, torch, T, table_bytes, peak, ms)}

    # ---- end to end through the public API with host buffers -------------------------------------
    h_tris = torch.from_numpy(tris.reshape(-1)).pin_memory()
    h_out = [torch.empty(W, dtype=torch.int32).pin_memory() for _ in MODES]

    # A host-buffer plan (cvx_plan_create_host) is one step's round trip: the triangles go up in 2
    # chunks, the surface jobs voxelize each chunk as it lands, the solid jobs follow, and each table
    # is copied down as soon as it is complete; its graph launch also takes the host's per-call
    # enqueue time out of the step.  Steps run back to back on E2E_SLOTS such plans
    # (cv.HostPipeline), each with its own device buffers and host tables, launched on their own
    # streams in turn: a step's upload and kernels run while the step before it is still copying its
    # tables down, so the host link (about 200 GB/s each way here, 333 GB/s both ways at once) is
    # busy in both directions.  A third slot measured no faster than two.
    slot_outs = []
    slot_jobs = []
    for _ in range(E2E_SLOTS):
        d_k = torch.empty_like(d_tris)
        tabs_k = [torch.empty_like(t) for t in tables]
        outs_k = [torch.empty(W, dtype=torch.int32).pin_memory() for _ in MODES]
        slot_outs.append(outs_k)
        slot_jobs.append([cv.HostJob(info, h_tris, d_k, out, tab, morton, solid)
                          for (morton, solid), tab, out in zip(MODES, tabs_k, outs_k)])
    pipe = cv.HostPipeline(slot_jobs, n_chunks=2)

    def e2e_steps(n):
        """n steps back to back, step k on slot k % E2E_SLOTS; returns the events around them."""
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pipe.begin(stream)
        for _ in range(n):
            pipe.submit()
        pipe.end(stream)
        b.record(stream)
        return a, b

    # a lone round trip: one host plan launched on the timing stream (over slot 0's buffers, never
    # while the pipeline runs)
    single = cv.HostPlan(slot_jobs[0], n_chunks=2)

    def e2e_step():
        single.launch(stream)

    def e2e_plain_step():
        d_tris.copy_(h_tris, non_blocking=True)
        for (morton, solid), tab, out in zip(MODES, tables, h_out):
            tab.zero_()
            (cv.voxelize_solid if solid else cv.voxelize)(info, d_tris, tab, morton)
            out.copy_(tab, non_blocking=True)

    for _ in range(3):
        e2e_plain_step()
    torch.cuda.synchronize()
    plain_times = []
    for _ in range(min(args.steps, 50)):
        flush.fill_(1)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e2e_plain_step()
        b.record(stream)
        torch.cuda.synchronize()
        plain_times.append(a.elapsed_time(b))
    plain_e2e_ms = float(np.mean(plain_times))

    # one host plan, one step at a time (L2 flushed and the device idle before each): the round trip's
    # latency
    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    single_times = []
    for _ in range(min(args.steps, 100)):
        flush.fill_(1)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e2e_step()
        b.record(stream)
        torch.cuda.synchronize()
        single_times.append(a.elapsed_time(b))
    single_ms = max_over_ranks(float(np.mean(single_times)), world)
    single.close()

    # the timed e2e: K steps back to back over the slots
    e2e_steps(max(3, args.warmup) * E2E_SLOTS)
    flush.fill_(1)
    torch.cuda.synchronize()
    barrier(world)
    a, b = e2e_steps(args.steps)
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(a.elapsed_time(b) / args.steps, world)

    # every host table must hold exactly what the device-resident step computes
    step()
    torch.cuda.synchronize()
    for k, tab in enumerate(tables):
        want = tab.cpu()
        for i, outs_k in enumerate(slot_outs):
            if not torch.equal(want, outs_k[k]):
                raise RuntimeError(f"e2e table {k} of slot {i} differs from the device-resident result")
        if not torch.equal(want, h_out[k]):
            raise RuntimeError(f"per-call e2e table {k} differs from the device-resident result")
    pipe.close()
    del pipe, slot_jobs, slot_outs
    # the link's bounds at the pinned copy rates measured here: one step alone moves every byte up,
    # then every byte down (no table can leave before the last triangle has arrived); back-to-back
    # steps can overlap one step's upload with another's read-back, at the rates each direction
    # keeps while the other runs, and finish the longer direction alone
    rates = copy_rates(torch, 256 << 20)
    copy_bound_ms = link_bound_s(tris.nbytes, 4 * W * 4, rates) * 1e3
    single_bound_ms = (tris.nbytes / (rates["h2d_gbs"] * 1e9) + 4 * W * 4 / (rates["d2h_gbs"] * 1e9)) * 1e3
    e2e = {"value": world * 4 * T / (e2e_ms / 1e3) / 1e6, "unit": "Mtris/s", "ms_per_step": e2e_ms,
           "h2d_bytes_per_step": int(tris.nbytes), "d2h_bytes_per_step": int(4 * W * 4),
           "path": f"cv.HostPipeline: {E2E_SLOTS} cvx_plan_create_host plans (own device buffers and host "
                   f"tables) launched on their own streams in turn, steps back to back; each plan: 2 upload "
                   f"chunks, surface jobs on each chunk as it lands, solid jobs after, each table read back as "
                   f"soon as it is complete",
           "l2": f"steps back to back over {E2E_SLOTS} buffer sets ({E2E_SLOTS} x 114 MB of device buffers, "
                 f"above the 129 MB L2); every step's triangles come up from pinned host memory inside the "
                 f"timed region",
           "copy_bound_ms": copy_bound_ms, "frac_of_copy_bound": copy_bound_ms / e2e_ms, "copy_rates": rates,
           "single_step": {"ms_per_step": single_ms, "value": world * 4 * T / (single_ms / 1e3) / 1e6,
                           "copy_bound_ms": single_bound_ms, "frac_of_copy_bound": single_bound_ms / single_ms,
                           "note": "one cv.HostPlan launch on the timing stream, one step at a time, L2 flushed "
                                   "before each: the round trip's latency"},
           "plain_calls": {"ms_per_step": plain_e2e_ms, "value": world * 4 * T / (plain_e2e_ms / 1e3) / 1e6,
                           "note": "upload, 4 calls and 4 read-backs in order on one stream, one step at a "
                                   "time"}}

    # ---- the JSON line; the reference CPU baseline and the side measurements on rank 0 -----------
    extras = {}
    line = {"metric": METRIC, "value": value, "unit": "Mtris/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced icosphere)",
            "config": {"workload": "icosphere level 8 (1,310,720 tris) at 512^3; surface+solid x linear+Morton "
                                   "per step", "gridsize": 512, "triangles": T, "l2": "flushed between steps "
                                   "(512 MiB write, untimed)",
                       "e2e_l2": f"steps back to back over {E2E_SLOTS} buffer sets ({E2E_SLOTS} x 114 MB of device "
                                 f"buffers, above the 129 MB L2), every step's triangles copied up from pinned host "
                                 f"memory inside the timed region; L2 flushed once before the timed steps",
                       "parallelism": f"replicas x{world}"},
            "clocks": clk.summary(), "gpu_launches": launches_per_step * args.steps, "e2e": e2e, "tuning": tuning,
            "roofline": roofline, "step_per_call": step_calls, "step_sequential": step_seq_line}

    if rank == 0:
        import oracle
        threads, tried, pass_s = cpu_threads(bytes(info), tris, os.cpu_count() or 1)
        kind = "reference" if oracle.ref_cpu_available() else "port"
        frac = cpu_fraction(pass_s, 3, 20.0)  # about 10-20 s of CPU work: the whole workload if it fits
        work = cpu_work(bytes(info), cpu_sample(tris, frac))
        time_cpu_reference(bytes(info), work, threads)  # warm-up
        sec = float(np.mean([time_cpu_reference(bytes(info), work, threads) for _ in range(2)]))
        line["cpu_baseline"] = {"value": sum(w.shape[0] for w in work) / sec / 1e6, "unit": "Mtris/s",
                                "cores": threads, "kind": kind, "sample": sample_desc(work, T, kind, frac),
                                "threads_tried_s": tried, "threads_note": THREADS_NOTE}
        if not args.no_extras:
            extras.update(bench_soup(cv, meshgen, torch, stream, flush))
            specs = meshgen.batch_mix(0, 256)
            mix = [(s, s.build()) for s in specs]
            extras.update(bench_io(cv, meshgen, torch, flush))
            extras.update(bench_batch(cv, torch, mix, default_tuning))
            extras.update(bench_serve(cv, meshgen, torch, mix, args.serve_seconds, args.serve_long_seconds,
                                      extras["batch_256"]["plan_meshes_s"]))
        line["extras"] = extras
        print(json.dumps(line), flush=True)


def bench_soup(cv, meshgen, torch, stream, flush):
    """2M-triangle size-stress soup at 1024^3: engine vs the reference CUDA kernel (sm_103a build)."""
    out = {}
    tris = meshgen.soup(0, n=2_000_000)
    info = cv.make_voxinfo(tris, 1024)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tab = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")

    def eng():
        tab.zero_()
        cv.voxelize(info, d, tab)

    eng()
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        flush.fill_(1)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    eng_ms = float(np.median(ts))
    out["soup_1024"] = {"triangles": 2_000_000, "engine_ms": eng_ms, "engine_mtris_s": 2.0 / (eng_ms / 1e3),
                        "ref_cuda": "timed by --impl reference (extras.soup_1024_ref_cuda)"}
    # roofline of the call: max(B / BW, A / R_atom), A from profiles/atomic_terms.json
    try:
        from cuda_voxelizer_gb300 import _lib
        with open(os.path.join(ROOT, "profiles", "atomic_terms.json")) as f:
            a = int(json.load(f)["soup_2m_1024"]["surface_linear"])
        words = 32 << 20
        buf = torch.zeros(words, dtype=torch.int32, device="cuda")
        r_atom = max(_lib.diag_lib().cvx_microbench_atomic_or(buf.data_ptr(), words, 0, 152 * 8, 64) for _ in range(3))
        del buf
        b = 36 * 2_000_000 + 4 * cv.table_words(info)
        hbm, _ = peaks()
        t_roof = max(b / (hbm * 1e9), a / r_atom)
        out["soup_1024"]["roofline"] = {"bytes": b, "atomics": a, "r_atom_per_s": r_atom,
                                        "t_bytes_ms": b / (hbm * 1e9) * 1e3, "t_atomics_ms": a / r_atom * 1e3,
                                        "frac": t_roof / (eng_ms / 1e3)}
    except Exception as e:
        out["soup_1024"]["roofline"] = f"unavailable: {e}"
    return out


def ref_cuda_soup(meshgen):
    """The reference CUDA surface kernel (its own source built for sm_103a) on the 2M-triangle soup
    at 1024^3, one timed launch after one warm-up on a small mesh."""
    import torch
    import oracle
    stream = torch.cuda.current_stream()
    ref = oracle.RefGPU()
    small = meshgen.torus(0)
    si = reference_voxinfo(small, 64)
    ds = torch.from_numpy(small.reshape(-1)).cuda()
    st = torch.zeros(oracle.table_words(si), dtype=torch.int32, device="cuda")
    ref.voxelize(si, ds.data_ptr(), st.data_ptr(), False, False, stream.cuda_stream)
    tris = meshgen.soup(0, n=2_000_000)
    info = reference_voxinfo(tris, 1024)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tab = torch.zeros(oracle.table_words(info), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ref.voxelize(info, d.data_ptr(), tab.data_ptr(), False, False, stream.cuda_stream)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    return {"triangles": 2_000_000, "ref_cuda_ms": ms, "ref_cuda_mtris_s": 2.0 / (ms / 1e3)}


def bench_io(cv, meshgen, torch, flush):
    """Ingest, layout and encoder kernels on large inputs, each against the HBM copy rate where it
    is a streaming kernel: device bbox of the 2M soup (72 MB read), indexed-mesh gather (2M faces
    of 1M vertices), Morton <-> linear transcode of a 1024^3 table (128 MiB read + 128 MiB
    written), binvox payload and voxel list of the 512^3 solid icosphere."""
    hbm, _ = peaks()
    stream = torch.cuda.current_stream()

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            flush.fill_(1)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    out = {}
    soup = torch.from_numpy(meshgen.soup(0, n=2_000_000).reshape(-1)).cuda()
    ms = timed(lambda: cv.mesh_bbox_device(soup))
    out["bbox_2m"] = {"ms": ms, "gbs": soup.numel() * 4 / (ms / 1e3) / 1e9, "note": "includes the 24-byte read-back"}
    gen = torch.Generator(device="cuda").manual_seed(1)
    verts = torch.rand(1_000_000 * 3, device="cuda", generator=gen)
    faces = torch.randint(0, 1_000_000, (2_000_000 * 3,), dtype=torch.int32, device="cuda", generator=gen)
    soup_out = torch.empty(2_000_000 * 9, dtype=torch.float32, device="cuda")
    from cuda_voxelizer_gb300 import _lib
    ms = timed(lambda: _lib.lib.cvx_gather_soup(verts.data_ptr(), 1_000_000, faces.data_ptr(), 2_000_000,
                                                   soup_out.data_ptr(), None, stream.cuda_stream))
    b = faces.numel() * 4 + soup_out.numel() * 4 + soup_out.numel() * 4
    out["gather_2m"] = {"ms": ms, "gbs": b / (ms / 1e3) / 1e9, "frac_of_hbm": b / (ms / 1e3) / 1e9 / hbm,
                        "bytes": b, "note": "faces + soup written + vertices read once per face corner"}
    g = 1024
    tab = torch.randint(-2 ** 31, 2 ** 31 - 1, (g ** 3 // 32,), dtype=torch.int32, device="cuda", generator=gen)
    dst = torch.empty_like(tab)
    for name, tm in (("linear_to_morton_1024", 1), ("morton_to_linear_1024", 0)):
        ms = timed(lambda: _lib.lib.cvx_transcode(tab.data_ptr(), dst.data_ptr(), g, tm, stream.cuda_stream))
        b = 2 * tab.numel() * 4
        out[name] = {"ms": ms, "gbs": b / (ms / 1e3) / 1e9, "frac_of_hbm": b / (ms / 1e3) / 1e9 / hbm}
    del tab, dst
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    t512 = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    cv.voxelize_solid(info, torch.from_numpy(tris.reshape(-1)).cuda(), t512)
    ms = timed(lambda: cv.encode_binvox(info, t512), reps=3)
    out["binvox_512_solid"] = {"ms": ms, "payload_bytes": len(cv.encode_binvox(info, t512)),
                               "note": "size pass + emit pass, synchronous, payload copied to the host"}
    ms = timed(lambda: cv.encode_voxel_list(info, t512), reps=3)
    out["voxel_list_512_solid"] = {"ms": ms, "voxels": int(cv.encode_voxel_list(info, t512).shape[0])}
    return {"io": out}


def bench_batch(cv, torch, mix, default_tuning=None):
    """256-mesh uneven mix: one graph launch (plan) vs plain per-mesh synchronous calls, with the
    autotuner's choice in effect; the plan is also timed with the default tuning."""
    jobs = []
    for s, t in mix:
        info = cv.make_voxinfo(t, s.gridsize)
        jobs.append(cv.Job(info, torch.from_numpy(t.reshape(-1)).cuda(),
                           torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda"), s.morton, s.solid))
    n_tris = sum(int(j.info.n_triangles) for j in jobs)
    reps = 10

    stream = torch.cuda.current_stream()

    def events_s(fn, blocks=5):
        """Seconds per call of fn: the median over `blocks` blocks of `reps` calls, each block timed
        between CUDA events on the launching stream."""
        out = []
        for _ in range(blocks):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b) / 1e3 / reps)
        return float(np.median(out))

    def time_plan():
        plan = cv.Plan(jobs, clear_tables=True)
        for _ in range(3):
            plan.launch()
        sec = events_s(plan.launch)
        plan.close()
        return sec

    plan_s = time_plan()
    default_plan_ms = None
    if default_tuning:
        tuned = cv.get_tuning(torch.cuda.current_device())
        if tuned == default_tuning:
            default_plan_ms = plan_s * 1e3  # the same thresholds: the same measurement
        else:
            cv.set_tuning(torch.cuda.current_device(), **default_tuning)
            default_plan_ms = time_plan() * 1e3
            cv.set_tuning(torch.cuda.current_device(), **tuned)
    # plain: what a caller of the reference drop-in does, one synchronous call per mesh
    def plain():
        for j in jobs:
            j.table.zero_()
            (cv.voxelize_solid if j.solid else cv.voxelize)(j.info, j.triangles, j.table, j.morton)
            torch.cuda.synchronize()
    plain()
    plain_s = events_s(plain, blocks=3)
    return {"batch_256": {"meshes": 256, "triangles": n_tris, "plan_ms": plan_s * 1e3, "plain_ms": plain_s * 1e3,
                          "plan_meshes_s": 256 / plan_s, "plain_meshes_s": 256 / plain_s,
                          "speedup_vs_plain": plain_s / plan_s, "plan_ms_default_tuning": default_plan_ms}}


def copy_rates(torch, nbytes=1 << 30):
    """Pinned host<->device copy rates (bytes/s): each direction alone and both at once."""
    h1 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d1 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):  # best of 3: a single duplex transfer varies by up to a third
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    def both():
        with torch.cuda.stream(s1):
            d1.copy_(h1, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    def split():
        """Both copies started together, each timed on its own stream (seconds)."""
        best = None
        for _ in range(4):
            a = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e2 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            s1.wait_event(a)
            s2.wait_event(a)
            with torch.cuda.stream(s1):
                d1.copy_(h1, non_blocking=True)
                e1.record(s1)
            with torch.cuda.stream(s2):
                h2.copy_(d2, non_blocking=True)
                e2.record(s2)
            torch.cuda.synchronize()
            t = (a.elapsed_time(e1) / 1e3, a.elapsed_time(e2) / 1e3)
            if best is None or max(t) < max(best):
                best = t
        return best

    h2d = nbytes / timed(lambda: d1.copy_(h1, non_blocking=True))
    d2h = nbytes / timed(lambda: h2.copy_(d2, non_blocking=True))
    duplex = 2 * nbytes / timed(both)
    # each direction's rate while the other runs: the copy that finishes first ran against the other
    # throughout; the other ran alone, at its own rate, for the rest of its time
    tu, td = split()
    if tu <= td:
        h2d_2 = nbytes / tu
        d2h_2 = min(max(nbytes - d2h * (td - tu), 0.05 * nbytes) / tu, d2h)
    else:
        d2h_2 = nbytes / td
        h2d_2 = min(max(nbytes - h2d * (tu - td), 0.05 * nbytes) / td, h2d)
    return {"h2d_gbs": h2d / 1e9, "d2h_gbs": d2h / 1e9, "both_directions_gbs": duplex / 1e9,
            "h2d_with_d2h_gbs": h2d_2 / 1e9, "d2h_with_h2d_gbs": d2h_2 / 1e9}


def link_bound_s(up, down, rates):
    """Least time to move `up` bytes to the device and `down` bytes back at the measured rates: both
    directions at once while both have bytes left (together faster than either alone), then the
    rest alone; or one after the other, if that were faster."""
    ru, rd = rates["h2d_gbs"] * 1e9, rates["d2h_gbs"] * 1e9
    ru2, rd2 = rates["h2d_with_d2h_gbs"] * 1e9, rates["d2h_with_h2d_gbs"] * 1e9
    tu, td = up / ru2, down / rd2
    overlapped = tu + (down - tu * rd2) / rd if tu <= td else td + (up - td * ru2) / ru
    return min(overlapped, up / ru + down / rd)


def link_jitter(torch, nbytes=4 << 20, n=1000):
    """Distribution of single pinned copies of nbytes each way (one at a time, CUDA events): the
    host-buffer serving arm moves a few MB per request, so a link that stalls now and then shows
    up here as a long tail even with nothing else running in this process."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    out = {"bytes": nbytes, "copies": n}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)), ("d2h", lambda: h.copy_(d, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for a, b in ev:
            a.record(s)
            fn()
            b.record(s)
        torch.cuda.synchronize()
        ms = np.array([a.elapsed_time(b) for a, b in ev])
        out[name] = {"p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
                     "max_ms": float(ms.max())}
    return out


def bench_serve(cv, meshgen, torch, mix, seconds, long_seconds, plan_meshes_s):
    """Open-loop serving of the 256-mesh distribution: Poisson arrivals, 40 GiB budget.  Two request
    kinds: host buffers (pinned triangles copied in, the table copied out) and device-resident
    buffers (triangles uploaded once, the table kept on the device; replay releases it at
    completion).  Capacity is measured with a burst (every request due at t=0); the Poisson sweep
    then runs at fractions of it.  The plain arm is the same server limited to one request at a
    time on one stream: one per-request launch sequence after another."""
    host_pool, dev_pool, keep = [], [], []
    in_bytes = out_bytes = 0
    for s, t in mix:
        info = cv.make_voxinfo(t, s.gridsize)
        h_t = torch.from_numpy(t.reshape(-1)).pin_memory()
        h_tab = torch.empty(cv.table_words(info), dtype=torch.int32).pin_memory()
        d_t = h_t.cuda()
        keep.append((h_t, h_tab, d_t))
        host_pool.append(cv.Server.request(info, h_t, h_tab, s.morton, s.solid))
        dev_pool.append(cv.Server.request(info, d_t, None, s.morton, s.solid))
        in_bytes += t.nbytes
        out_bytes += 4 * cv.table_words(info)
    torch.cuda.synchronize()
    rng = np.random.default_rng(7)

    def burst(srv, pool, n):
        lat = srv.replay(pool, rng.integers(0, len(pool), n), np.zeros(n))
        return n / (float(lat.max()) / 1e3)

    def poisson(srv, pool, rate, seed, secs):
        arr = meshgen.poisson_arrivals(rate, secs, seed=seed)
        lat = srv.replay(pool, rng.integers(0, len(pool), len(arr)), arr)
        span = float(np.max(arr + lat / 1e3))
        st = srv.stats()
        return {"rate_per_s": round(rate, 1), "seconds": secs, "requests": int(len(arr)), "meshes_s": len(arr) / span,
                "memory_peak_gib": st["memory_peak"] / 2 ** 30,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "queue_p99_ms": st["queue_p99_ms"], "batch_service_p50_ms": st["service_p50_ms"],
                "batch_service_p99_ms": st["service_p99_ms"], "batch_issue_p50_us": st["issue_p50_us"],
                "mean_batch": st["mean_batch"], "generator_late_p99_ms": st["replay_late_p99_ms"],
                "generator_late_max_ms": st["replay_late_max_ms"]}

    def arm(pool, max_batch, max_inflight, fracs, seed0, n_burst, long_fracs=()):
        mk = lambda: cv.Server(memory_budget_bytes=40 << 30, max_batch=max_batch, max_inflight=max_inflight)
        with mk() as srv:
            burst(srv, pool, max(64, n_burst // 8))
        with mk() as srv:
            cap = burst(srv, pool, n_burst)
            st = srv.stats()
        res = {"capacity_meshes_s": cap, "max_batch": max_batch, "max_inflight": max_inflight,
               "burst_requests": n_burst, "burst_mean_batch": st["mean_batch"], "burst_issue_p50_us": st["issue_p50_us"],
               "burst_memory_peak_gib": st["memory_peak"] / 2 ** 30}
        res["sweep"] = []
        for i, f in enumerate(fracs):  # a fresh server per rate: its stats cover that rate alone
            with mk() as srv:
                res["sweep"].append(poisson(srv, pool, f * cap, seed0 + i,
                                            long_seconds if f in long_fracs else seconds))
        return res

    rates = copy_rates(torch)
    jitter = link_jitter(torch)
    n = len(mix)
    per_req_in, per_req_out = in_bytes / n, out_bytes / n
    copy_cap = 1.0 / link_bound_s(per_req_in, per_req_out, rates)
    out = {"budget_gib": 40, "seconds_per_rate": {"served 75% and 90% load": long_seconds, "other rates": seconds},
           "pool": "256-mesh mix (same as batch_256)",
           "copy_rates": rates, "link_jitter_before": jitter,
           "bytes_per_request": {"in": per_req_in, "out": per_req_out}}
    fr = (0.25, 0.5, 0.75, 0.9)
    long_fr = (0.75, 0.9)
    # capacity bursts of about half a second: a shorter burst overstated the host-buffer arm's
    # sustained rate (a 4,096-request burst gave 31.4 k/s where 60 s of load sustained 27.3 k/s)
    host = {"served": arm(host_pool, 4, 32, fr, 0, 16384, long_fr), "plain": arm(host_pool, 1, 1, (0.5, 0.9), 10, 2048)}
    # the link's rates again after the host-buffer arms: the machine's host memory is shared, and a
    # drop here shows up as longer batch service times and queueing in the sweep above
    out["copy_rates_after_host_arms"] = copy_rates(torch)
    out["link_jitter_after_host_arms"] = link_jitter(torch)
    host["roofline_meshes_s"] = min(copy_cap, plan_meshes_s)
    host["served_frac_of_roofline"] = host["served"]["capacity_meshes_s"] / host["roofline_meshes_s"]
    host["served_vs_plain_capacity"] = host["served"]["capacity_meshes_s"] / host["plain"]["capacity_meshes_s"]
    dev = {"served": arm(dev_pool, 256, 4, fr, 20, 32768, long_fr), "plain": arm(dev_pool, 1, 1, (0.5, 0.9), 30, 4096)}
    dev["roofline_meshes_s"] = plan_meshes_s
    dev["served_frac_of_roofline"] = dev["served"]["capacity_meshes_s"] / plan_meshes_s
    dev["served_vs_plain_capacity"] = dev["served"]["capacity_meshes_s"] / dev["plain"]["capacity_meshes_s"]
    out["host_buffers"] = host
    out["device_resident"] = dev
    out["roofline_note"] = ("host buffers: min(copy-bound rate from the measured pinned copy rates, batched "
                            "compute rate of batch_256); device-resident: the batched compute rate")
    return {"serve": out}


if __name__ == "__main__":
    main()
