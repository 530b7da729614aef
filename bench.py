"""Benchmark: Coulomb (J) builds per second through the H2 representation of
the ERI tensor, C30H62 (all-trans zigzag, cc-pVDZ Cartesian, 760 basis
functions), QR tolerance 1e-8, one seeded density (n_occ = 121).

Default (GPU) arm: the representation is built on the host (set-up, not
timed) and uploaded once. One step is a batch of BUILDS_PER_STEP J builds
(uncontract -> H2 matvec -> contract), one per seeded density, each its own
single-density call, with the densities already in HBM; the timed region is
then long enough (about a second) for the clock sampler. The e2e figure
times the reference's own entry point H2ERI_build_Coulomb on page-locked host
buffers (density from host memory, J to host memory) for the same builds.
Precision: mixed (bases and leaf self blocks stored as FP32 pairs, other
blocks as FP32, anchored FP32 accumulation, FP64 output sums) when
available, else FP64; the FP64 figure is always reported beside it, together
with the relative error of each against the FP64 CPU oracle.

--impl reference: the reference's CPU implementation of this path, timed on
the host cores (the oracle restatement of H2ERI_build_Coulomb, OpenMP over
all host threads), same workload and metric.

Multi-GPU (torchrun): one independent replica per GPU (the path does not
shard: a J build has no exchange step); value = builds of all ranks / max
time over ranks.

--path exchange: K builds per second (H2ERI_build_exchange). --path setup:
seconds per host set-up (CPU only; with --impl reference the reference's own
set-up where its sources exist).
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "h2p-eri_gb300"))
sys.path.insert(0, REPO)

WORKLOADS = {
    # the headline configuration (fits one GPU)
    "c30": {"workload": "J build C30H62 cc-pVDZ (760 bf, cartesian), QR tol 1e-8, 1 density n_occ=121",
            "molecule": "C30H62", "n_carbon": 30, "qr_tol": 1e-8, "n_occ": 121, "seed": 2000,
            "inputs_vs_L2": "H2 representation ~1.8 GB read per step > 129 MB L2 (no flush needed)",
            "k_cpu_stride": 16},
    # the larger molecule of the mixed-precision configuration
    "c100": {"workload": "J build C100H202 cc-pVDZ (2510 bf, cartesian), QR tol 1e-8, 1 density n_occ=401",
             "molecule": "C100H202", "n_carbon": 100, "qr_tol": 1e-8, "n_occ": 401, "seed": 3000,
             "inputs_vs_L2": "H2 representation ~6.7 GB read per step > 129 MB L2 (no flush needed)",
             "k_cpu_stride": 64},
    # small case for profiler captures (the reference's CPU-runnable size)
    "c10": {"workload": "J build C10H22 cc-pVDZ (260 bf, cartesian), QR tol 1e-6, 1 density n_occ=41",
            "molecule": "C10H22", "n_carbon": 10, "qr_tol": 1e-6, "n_occ": 41, "seed": 1000,
            "inputs_vs_L2": "H2 representation ~0.28 GB read per step > 129 MB L2",
            "k_cpu_stride": 2, "k_check_full": True},
}
# the 3-D exchange case: a seeded cluster of 48 CH4 (a water cluster needs
# oxygen basis data, which is not available), K builds
WORKLOADS["ch4x48"] = {"workload": "K build, 3-D cluster of 48 CH4 (4x4x3 jittered cubic lattice 4 A apart, "
                                   "seeded orientations), cc-pVDZ cartesian (1680 bf), QR tol 1e-7, 1 density "
                                   "n_occ=240", "molecule": "(CH4)48", "cluster": [4, 4, 3], "qr_tol": 1e-7,
                       "n_occ": 240, "seed": 5000, "k_cpu_stride": 128,
                       "inputs_vs_L2": "H2 representation and K intermediates > 129 MB L2"}
# uneven batch: alkanes with lengths drawn from C8..C60 (seeded), two densities
# each; BATCH_SIZE molecules (the set-up of each runs on the host first)
WORKLOADS["batch"] = {"workload": "J builds for a batch of alkanes C8..C60 (seeded lengths), cc-pVDZ cartesian, "
                                  "QR tol 1e-8, 2 densities each", "qr_tol": 1e-8, "seed": 4242,
                      "inputs_vs_L2": "sum of the representations > 129 MB L2"}
WORKLOAD = dict(WORKLOADS["c30"])
METRIC = "J builds/s C30H62 (mixed vs FP64) at relerr<=1e-8"
# J builds per step (one single-density call each, distinct seeded densities)
BUILDS_PER_STEP = 128
# DRAM traffic of the tile kernels per J build, from an ncu capture of the
# same workload: key = value lines, read at run time and named in the output
TRAFFIC_FILE = os.path.join("profiles", "dram_traffic_J_C30H62.txt")
METRIC_K = "K builds/s (H2ERI_build_exchange path)"
CACHE_DIR = os.path.join(tempfile.gettempdir(), "h2eri_gb300_cache")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_name():
    if "cluster" in WORKLOAD:
        return "ch4c" + "x".join(str(n) for n in WORKLOAD["cluster"])
    return f"alk{WORKLOAD['n_carbon']}"


def geometry_kind():
    return "CH4 cluster" if "cluster" in WORKLOAD else "alkane"


def write_workload_mol(molecules, path):
    """The workload's molecule as a .mol file: an alkane or a CH4 cluster."""
    if "cluster" in WORKLOAD:
        molecules.write_methane_cluster(path, tuple(WORKLOAD["cluster"]), seed=WORKLOAD["seed"])
    else:
        molecules.write_alkane(path, WORKLOAD["n_carbon"])


def representation(hg, molecules, rank, ws, barrier):
    """Build (rank 0) or load the cached representation of the workload."""
    os.makedirs(CACHE_DIR, exist_ok=True)
    path = os.path.join(CACHE_DIR, f"{workload_name()}_{WORKLOAD['qr_tol']:g}.h2r")
    setup_s = None
    if rank == 0 and not os.path.exists(path):
        mol = os.path.join(CACHE_DIR, f"{workload_name()}.mol")
        write_workload_mol(molecules, mol)
        t0 = time.perf_counter()
        h = hg.H2ERI.from_mol(mol, qr_tol=WORKLOAD["qr_tol"])
        setup_s = time.perf_counter() - t0
        tmp = path + ".tmp"
        h.save(tmp)
        os.replace(tmp, path)
        log(f"set-up (not timed): {setup_s:.1f} s")
    else:
        h = None
    barrier()
    if h is None:
        h = hg.H2ERI.load(path)
    return h, setup_s


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
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
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, dist, device):
    """The largest value of x over the ranks (x itself with one process):
    every rank times its own replicas, and the job is as slow as its slowest
    rank."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, steps, ms_max):
    """J builds per second of the whole job: each of the ws ranks ran `steps`
    builds, and the slowest rank took ms_max milliseconds for its steps."""
    return ws * steps / (ms_max / 1e3)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def bf16_peak():
    """Dense bf16 tensor rate (TFLOP/s): measured burst, else the fallback figure."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def cpu_baseline(orc, h, D, budget_s=12.0, max_builds=100000):
    """Oracle restatement of H2ERI_build_Coulomb on the host cores."""
    J = np.zeros_like(D)
    orc.oracle_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)   # warm-up
    n, t0 = 0, time.perf_counter()
    while n < max_builds and time.perf_counter() - t0 < budget_s:
        orc.oracle_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, n, dt, J


def load_oracle():
    from oracle import build_oracle
    orc = ctypes.CDLL(build_oracle.build())
    for f in ("oracle_matvec", "oracle_build_Coulomb", "oracle_build_exchange"):
        getattr(orc, f).argtypes = [ctypes.c_void_p] * 3
        getattr(orc, f).restype = None
    orc.oracle_build_exchange_shells.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int]
    orc.oracle_build_exchange_shells.restype = None
    return orc


def exchange_cpu_sample(orc, h, D, stride, reps=1):
    """Oracle restatement of H2ERI_build_exchange on the host cores, over every
    stride-th outer shell N (the reference's outer loop); returns K builds/s
    scaled by the sampled share of shells and a description."""
    nsh = h.s.nshell
    shells = np.arange(0, nsh, max(1, stride), dtype=np.int32)
    K = np.zeros_like(D)
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.oracle_build_exchange_shells(h.handle, D.ctypes.data, K.ctypes.data, shells.ctypes.data, len(shells))
    dt = (time.perf_counter() - t0) / reps
    frac = len(shells) / nsh
    return frac / dt, f"{len(shells)} of {nsh} outer shells N (every {stride}-th) in {dt:.1f} s, scaled by {frac:.4f}"


def step_densities(molecules, nbf, n, seed0):
    """The n seeded densities of one step (seeds seed0 .. seed0 + n - 1)."""
    return np.stack([molecules.seeded_density(nbf, WORKLOAD["n_occ"], seed0 + i) for i in range(n)])


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.path == "exchange":
        return run_reference_exchange(args)
    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    hb.build()
    orc = load_oracle()
    h, _ = representation(hg, molecules, 0, 1, lambda: None)
    Ds = step_densities(molecules, h.num_bf, BUILDS_PER_STEP, WORKLOAD["seed"])
    J = np.zeros_like(Ds[0])

    def step():
        for i in range(BUILDS_PER_STEP):
            orc.oracle_build_Coulomb(h.handle, Ds[i].ctypes.data, J.ctypes.data)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    v = args.steps * BUILDS_PER_STEP / dt
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "J builds/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
           "builds_per_step": BUILDS_PER_STEP, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (generated alkane geometry, seeded densities)", "config": dict(WORKLOAD),
           "cpu_baseline": {"value": v, "unit": "J builds/s", "cores": cores, "kind": "port",
                            "sample": f"{args.steps} steps of {BUILDS_PER_STEP} J builds (oracle restatement of "
                                      f"H2ERI_build_Coulomb, OpenMP over {cores} threads)"},
           "e2e": {"value": v, "unit": "J builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    h.destroy()


def run_reference_exchange(args):
    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    hb.build()
    orc = load_oracle()
    h, _ = representation(hg, molecules, 0, 1, lambda: None)
    D = molecules.seeded_density(h.num_bf, WORKLOAD["n_occ"], WORKLOAD["seed"])
    stride = WORKLOAD.get("k_cpu_stride", 1)
    for _ in range(args.warmup):
        exchange_cpu_sample(orc, h, D, stride * 4)
    vals = []
    for _ in range(args.steps):
        v, sample = exchange_cpu_sample(orc, h, D, stride)
        vals.append(v)
    v = len(vals) / sum(1.0 / x for x in vals)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    out = {"impl": "reference", "metric": METRIC_K, "value": v, "unit": "K builds/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": f"synthetic (generated {geometry_kind()} geometry, seeded density)", "config": dict(WORKLOAD, path="exchange"),
           "cpu_baseline": {"value": v, "unit": "K builds/s", "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": "K builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    h.destroy()


def run_setup(args):
    """--path setup: seconds per set-up of the workload's molecule
    (H2ERI_init, CMS_read_mol_file, H2ERI_process_shells, H2ERI_partition,
    H2ERI_build_H2; OpenMP over the host cores). With --impl reference: the
    reference's own set-up, compiled from its sources (the integral engine of
    this package stands in for SIMINT), only where those sources exist."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    hb.build()
    mol = os.path.join(tempfile.mkdtemp(), f"{workload_name()}.mol")
    write_workload_mol(molecules, mol)
    qr = WORKLOAD["qr_tol"]
    if args.impl == "reference":
        from oracle import build_ref
        if not build_ref.available():
            print(json.dumps({"impl": "reference", "unavailable": "reference sources absent on this machine, "
                              "so its set-up cannot be compiled here"}), flush=True)
            return
        R = ctypes.CDLL(build_ref.build(verbose=False))
        R.oref_build.restype = ctypes.c_void_p
        R.oref_build.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]

        def one():
            R.oref_build(mol.encode(), 1e-10, 1e-10, qr, 0)   # the reference struct is not freed
    else:
        def one():
            hg.H2ERI.from_mol(mol, qr_tol=qr).destroy()
    steps = max(1, min(args.steps, 3))
    one()                                    # warm-up: library load, Boys table
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        one()
        times.append(time.perf_counter() - t0)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    out = {"metric": f"set-up seconds {WORKLOAD['molecule']} (H2ERI_build_H2 and the calls before it; integrals on "
                     f"the GPU when one is present, decompositions on the host)",
           "value": statistics.median(times), "unit": "s", "higher_is_better": False, "steps": steps,
           "warmup": 1, "samples_s": [round(t, 3) for t in times], "cores": cores, "dtype": "f64",
           "data": f"synthetic (generated {geometry_kind()} geometry)", "config": dict(WORKLOAD)}
    if args.impl == "reference":
        out["impl"] = "reference"
    print(json.dumps(out), flush=True)


def run_gpu_exchange(args):
    """K builds/s: the exchange path (H2ERI_build_exchange) on one GPU."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    if rank == 0:
        hb.build()
    h, setup_s = representation(hg, molecules, rank, ws, lambda: None)
    L = hg.lib()
    nbf = h.num_bf
    D = molecules.seeded_density(nbf, WORKLOAD["n_occ"], WORKLOAD["seed"])
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    dD = torch.tensor(D, device="cuda")
    dK = torch.empty_like(dD)
    torch.cuda.synchronize()
    t_plan = time.perf_counter()
    if L.H2ERI_build_exchange_device(h.handle, dD.data_ptr(), dK.data_ptr(), sp) != 0:
        raise RuntimeError(L.H2ERI_gpu_last_error().decode())
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t_plan
    modes = ["fp64"] if args.precision in ("auto", "fp64") else []
    if args.precision in ("auto", "mixed"):
        modes.append("mixed")

    def device_run(mode):
        L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if mode == "mixed" else hg.FP64)
        for _ in range(args.warmup):
            if L.H2ERI_build_exchange_device(h.handle, dD.data_ptr(), dK.data_ptr(), sp) != 0:
                raise RuntimeError(L.H2ERI_gpu_last_error().decode())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                L.H2ERI_build_exchange_device(h.handle, dD.data_ptr(), dK.data_ptr(), sp)
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1), dK.cpu().numpy(), clk.summary()

    res = {m: device_run(m) for m in modes}
    best = "mixed" if "mixed" in res else "fp64"
    L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if best == "mixed" else hg.FP64)
    ms, K, c = res[best]
    hD = torch.from_numpy(D).pin_memory()
    hK = torch.empty_like(hD).pin_memory()
    L.H2ERI_build_exchange_multi(h.handle, 1, hD.data_ptr(), hK.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.H2ERI_build_exchange_multi(h.handle, 1, hD.data_ptr(), hK.data_ptr())
    e2e_s = time.perf_counter() - t0
    xr = h.exchange_report()
    step_s = ms / 1e3 / args.steps
    orc = load_oracle()
    cpu = None
    if not args.skip_cpu:
        v, sample = exchange_cpu_sample(orc, h, D, WORKLOAD.get("k_cpu_stride", 1))
        cpu = {"value": v, "unit": "K builds/s", "cores": os.cpu_count(), "kind": "port", "sample": sample}
    K_ref = None
    if WORKLOAD.get("k_check_full", False):
        K_ref = np.zeros_like(D)
        orc.oracle_build_exchange(h.handle, D.ctypes.data, K_ref.ctypes.data)
    elif "fp64" in res:
        K_ref = res["fp64"][1]   # FP64 GPU K (equal to the oracle's to ~1e-15 where checked)

    def rel(X):
        return None if K_ref is None else float(np.linalg.norm(X - K_ref) / np.linalg.norm(K_ref))

    achieved = xr["flops"] / step_s / 1e12
    tc = best == "mixed" and xr.get("tensor_cores", 0) == 1
    if best == "fp64":
        peak, bound, peak_kind = 1.25, "fp64", "nominal FP64 (no measured FP64 peak)"
    elif tc:
        bfp, bkind = bf16_peak()
        peak, bound = bfp / 6.0, "tensor"
        peak_kind = (f"{bkind} dense bf16 rate {bfp:.0f} TFLOP/s / 6 (each FP32 product is six bf16 MMA products "
                     f"of its bf16x3 splits)")
    else:
        peak, bound, peak_kind = 74.0, "fp32-simt", "nominal FP32 FMA 152 SMs x 128 x 2 x 1.9 GHz"
    out = {
        "metric": METRIC_K, "value": args.steps / (ms / 1e3), "unit": "K builds/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if best == "fp64" else "f32+f64",
        "data": f"synthetic (generated {geometry_kind()} geometry, seeded density)",
        "config": dict(WORKLOAD, path="exchange", precision=best, parallelism="replicas x1"),
        "relerr_vs_fp64": rel(K),
        "relerr_reference": "FP64 CPU oracle" if WORKLOAD.get("k_check_full", False) else "FP64 GPU path",
        "fp64": ({"value": args.steps / (res["fp64"][0] / 1e3), "unit": "K builds/s",
                  "ms_per_step": res["fp64"][0] / args.steps, "relerr_vs_fp64_oracle":
                  rel(res["fp64"][1]) if WORKLOAD.get("k_check_full", False) else None}
                 if "fp64" in res and best != "fp64" else None),
        "e2e": {"value": args.steps / e2e_s, "unit": "K builds/s", "h2d_bytes_per_step": 8 * nbf * nbf,
                "d2h_bytes_per_step": 8 * nbf * nbf},
        "roofline": {"bound": bound, "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "kernel": ("k_gemm_tcp" if tc else "k_gemm") + " + k_near (all launches of one K build)",
                     "alg_flops_per_step": xr["flops"], "peak_kind": peak_kind},
        "cpu_baseline": cpu,
        "clocks": {"sm_mhz": c["sm_mhz"], "sm_max_mhz": c["sm_max_mhz"], "reasons": c["reasons"]},
        "gpu_launches": int(xr["launches"]) * args.steps,
        "plan": {"first_call_s": plan_s, "n_ranges": xr["n_ranges"], "work_bytes": xr["work_bytes"],
                 "near_items": xr["near_items"]},
        "setup_s": setup_s,
    }
    print(json.dumps(out), flush=True)
    h.destroy()


def run_gpu_batch(args):
    """Uneven batch: every molecule's J builds (two densities) in one
    H2ERI_build_Coulomb_batch call, against the same builds one molecule
    after another on one stream."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    hb.build()
    L = hg.lib()
    lengths = [int(n) for n in np.random.default_rng(WORKLOAD["seed"]).integers(8, 61, size=args.batch_size)]
    hs, t0 = [], time.perf_counter()
    os.makedirs(CACHE_DIR, exist_ok=True)
    for n in lengths:
        mol = os.path.join(CACHE_DIR, f"alk{n}.mol")
        molecules.write_alkane(mol, n)
        hs.append(hg.H2ERI.from_mol(mol, qr_tol=WORKLOAD["qr_tol"]))
    setup_s = time.perf_counter() - t0
    log(f"set-up of {len(hs)} molecules (host, not timed): {setup_s:.1f} s")
    best = "mixed" if args.precision in ("auto", "mixed") else "fp64"
    dDs, dJs, Ds = [], [], []
    choices = {}
    t_tune = time.perf_counter()
    # the whole batch resident in HBM: each structure's FP64 copy is freed, and
    # the tensor-core kernel (whose slice images would not fit for 64
    # molecules) is not used at 2 densities
    memory_note = None
    if best == "mixed" and args.batch_size > 8:
        os.environ["H2G_MMA_MIN_VEC"] = "3"
        memory_note = ("FP64 copies freed (H2ERI_gpu_drop_fp64) and the tensor-core kernel off at 2 densities "
                       "(H2G_MMA_MIN_VEC=3), so that every structure stays resident")
    for k, h in enumerate(hs):
        if L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if best == "mixed" else hg.FP64) != 0:
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())
        if memory_note and L.H2ERI_gpu_drop_fp64(h.handle) != 0:
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())
        if not args.no_autotune:
            c = h.autotune(2)["choice"]
            key = ",".join(f"{a}={b}" for a, b in sorted(c.items()))
            choices[key] = choices.get(key, 0) + 1
        n_occ = (8 * lengths[k] + 2) // 2   # electrons of C_nH_2n+2 / 2
        D = np.stack([molecules.seeded_density(h.num_bf, n_occ, 4000 + 10 * k + i) for i in range(2)])
        Ds.append(D)
        dDs.append(torch.tensor(D, device="cuda"))
        dJs.append(torch.empty_like(dDs[-1]))
    tune_s = time.perf_counter() - t_tune
    n = len(hs)
    harr = (ctypes.c_void_p * n)(*[h.handle.value for h in hs])
    narr = (ctypes.c_int * n)(*([2] * n))
    darr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dDs])
    jarr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dJs])
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def batched():
        if L.H2ERI_build_Coulomb_batch(n, harr, narr, darr, jarr, sp) != 0:
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())

    def one_by_one():
        for k in range(n):
            L.H2ERI_build_Coulomb_device(hs[k].handle, 2, dDs[k].data_ptr(), dJs[k].data_ptr(), sp)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, clk.summary()

    ms_seq, _ = timed(one_by_one)
    ms, c = timed(batched)
    # the same call with the tiles of all structures in shared launches
    os.environ["H2G_BATCH_MERGED"] = "1"
    ms_shared, _ = timed(batched)
    del os.environ["H2G_BATCH_MERGED"]
    orc = load_oracle()
    errs = []
    for k in (0, n - 1):
        Jo = np.zeros_like(Ds[k][0])
        orc.oracle_build_Coulomb(hs[k].handle, np.ascontiguousarray(Ds[k][0]).ctypes.data, Jo.ctypes.data)
        errs.append(float(np.linalg.norm(dJs[k][0].cpu().numpy() - Jo) / np.linalg.norm(Jo)))
    builds = 2 * n
    out = {"metric": "J builds/s, uneven batch of alkanes (one batched call)", "value": builds / (ms / 1e3),
           "unit": "J builds/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32x2+f64" if best == "mixed" else "f64",
           "data": "synthetic (generated alkane geometries, seeded densities)",
           "config": dict(WORKLOAD, molecules=[f"C{m}H{2 * m + 2}" for m in lengths], precision=best,
                          sample=f"{n} molecules (lengths from U{{8..60}}, seed 4242); 2 densities each"),
           "one_by_one_ms_per_step": ms_seq, "batch_speedup": ms_seq / ms, "device_memory": memory_note,
           "shared_launches_ms_per_step": ms_shared, "shared_launches_speedup": ms_seq / ms_shared,
           "autotune": {"choices_at_2_densities": choices, "tuning_and_upload_s": tune_s},
           "relerr_vs_fp64_oracle_sampled": max(errs),
           "clocks": {"sm_mhz": c["sm_mhz"], "sm_max_mhz": c["sm_max_mhz"], "reasons": c["reasons"]},
           "setup_s": setup_s}
    print(json.dumps(out), flush=True)
    for h in hs:
        h.destroy()


def fp64_peak_tflops(torch):
    """Measured FP64 rate of this GPU (cuBLAS DGEMM 4096^3 through torch,
    best of 5): the denominator of the FP64 path's roofline."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


def read_traffic():
    """DRAM traffic per J build from the committed capture summary (key = value
    lines), or None."""
    path = os.path.join(REPO, TRAFFIC_FILE)
    try:
        kv = {}
        with open(path) as f:
            for ln in f:
                if "=" in ln and not ln.lstrip().startswith("#"):
                    k, v = ln.split("=", 1)
                    kv[k.strip()] = v.strip()
        return float(kv["traffic_bytes_per_build"]), TRAFFIC_FILE
    except (OSError, KeyError, ValueError):
        return None, None


def run_gpu(args):
    if args.path == "exchange":
        return run_gpu_exchange(args)
    if args.workload == "batch":
        return run_gpu_batch(args)
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    import h2eri_gb300 as hg
    from h2eri_gb300 import build as hb, molecules
    if rank == 0:
        hb.build()
    barrier()
    h, setup_s = representation(hg, molecules, rank, ws, barrier)
    L = hg.lib()
    nbf = h.num_bf
    B = BUILDS_PER_STEP
    Ds = step_densities(molecules, nbf, B, WORKLOAD["seed"])
    # a dedicated stream: the library enqueues on it and the events below are
    # recorded on it (the legacy default stream would not order with the
    # library's non-blocking streams)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    dD = torch.tensor(Ds, device="cuda")
    dJ = torch.empty_like(dD)
    torch.cuda.synchronize()
    t_up = time.perf_counter()
    h.upload()
    upload_s = time.perf_counter() - t_up

    modes = [] if args.precision == "mixed" else ["fp64"]
    if args.precision in ("auto", "mixed"):
        if L.H2ERI_gpu_set_precision(h.handle, hg.MIXED) == 0:
            modes.append("mixed")
        elif args.precision == "mixed":
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())

    # the autotuner picks the launch choices of this structure (tile rows,
    # tiles per CTA, near-field lanes, tensor-core kernel for several
    # densities) by timing every candidate on the device; not timed here
    tuned = {}
    if not args.no_autotune:
        t_tune = time.perf_counter()
        for mode in modes:
            L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if mode == "mixed" else hg.FP64)
            tuned[f"{mode}_1"] = h.autotune(1)
            if mode == "mixed":
                tuned["mixed_16"] = h.autotune(16)
        tuned["tuning_s"] = time.perf_counter() - t_tune

    def one_step(nden):
        for i in range(0, B, nden):
            L.H2ERI_build_Coulomb_device(h.handle, nden, dD[i].data_ptr(), dJ[i].data_ptr(), sp)

    def device_run(mode, nden, min_s=0.0):
        """Timed steps of B builds, nden densities per call; ms per step.
        K steps (the headline); with min_s > 0 (the sub-figures), at least
        K steps and at least min_s seconds, the count set from the warm-up."""
        L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if mode == "mixed" else hg.FP64)
        if L.H2ERI_build_Coulomb_device(h.handle, nden, dD[0].data_ptr(), dJ[0].data_ptr(), sp) != 0:
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())
        torch.cuda.synchronize()
        t_w = time.perf_counter()
        for _ in range(args.warmup):
            one_step(nden)
        torch.cuda.synchronize()
        steps = args.steps
        if min_s > 0:
            per_step = (time.perf_counter() - t_w) / max(args.warmup, 1)
            steps = max(args.steps, int(math.ceil(min_s / max(per_step, 1e-6))))
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(steps):
                one_step(nden)
            e1.record(stream)
            torch.cuda.synchronize()
        barrier()
        if L.H2ERI_gpu_check(h.handle) != 0:
            raise RuntimeError(L.H2ERI_gpu_last_error().decode())
        ms_total = e0.elapsed_time(e1)
        summ = dict(clk.summary(), timed_steps=steps, timed_s=ms_total / 1e3)
        return ms_total / steps, dJ.cpu().numpy(), summ

    results = {}
    for mode in modes:
        ms, J, clk = device_run(mode, 1)
        results[mode] = {"ms": ms, "J": J, "clocks": clk}
    best = "mixed" if "mixed" in results else "fp64"
    n16 = 16
    ms16, J16, clk16 = device_run(best, n16, min_s=1.2)
    L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if best == "mixed" else hg.FP64)
    # kernels per single-density J build with the choices in use: the H2
    # matvec's launches plus the uncontract and contract kernels
    rep_best = h.report()
    launches_per_J = int(rep_best["launches_per_matvec"]) + 2

    # e2e: the reference's own entry point with page-locked host buffers
    # (density read from and J written to host memory by the kernels)
    hD = torch.from_numpy(Ds).pin_memory()
    hJ = torch.zeros(Ds.shape, dtype=torch.float64).pin_memory()

    def e2e_step():
        for i in range(B):
            L.H2ERI_build_Coulomb(h.handle, hD[i].data_ptr(), hJ[i].data_ptr())

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = time.perf_counter() - t0
    barrier()
    Je2e = hJ.numpy().copy()

    ms_best = max_over_ranks(results[best]["ms"], dist, "cuda")
    ms_fp64 = max_over_ranks(results["fp64"]["ms"], dist, "cuda") if "fp64" in results else float("nan")
    ms16 = max_over_ranks(ms16, dist, "cuda")
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    if rank != 0:
        barrier()
        return

    orc = load_oracle()
    J_ref = {}

    def oracle_J(i):
        if i not in J_ref:
            Jo = np.zeros_like(Ds[i])
            orc.oracle_build_Coulomb(h.handle, Ds[i].ctypes.data, Jo.ctypes.data)
            J_ref[i] = Jo
        return J_ref[i]

    def rel(J, i):
        return float(np.linalg.norm(J - oracle_J(i)) / np.linalg.norm(oracle_J(i)))

    sample = (0, B - 1)
    if args.skip_cpu:
        cpu_v, cpu_n, cpu_dt = None, 0, 0.0
    else:
        cpu_v, cpu_n, cpu_dt, _ = cpu_baseline(orc, h, Ds[0])

    value = replica_value(ws, args.steps * B, args.steps * ms_best)
    ms_build = ms_best / B
    rep_best = h.report()
    alg_bytes = rep_best["alg_matrix_bytes"] + rep_best["alg_vector_bytes"] + 2 * 8 * nbf * nbf
    peak, peak_kind = peaks()
    achieved = alg_bytes / (ms_build / 1e3) / 1e9
    traffic, traffic_src = read_traffic() if (best == "mixed" and WORKLOAD.get("n_carbon") == 30) else (None, None)
    clk = results[best]["clocks"]

    fp64 = None
    if "fp64" in results:
        L.H2ERI_gpu_set_precision(h.handle, hg.FP64)
        rep64 = h.report()
        L.H2ERI_gpu_set_precision(h.handle, hg.MIXED if best == "mixed" else hg.FP64)
        ms64_build = ms_fp64 / B
        bytes64 = rep64["alg_matrix_bytes"] + rep64["alg_vector_bytes"] + 2 * 8 * nbf * nbf
        fpk = fp64_peak_tflops(torch)
        tf = rep64["alg_flops"] / (ms64_build / 1e3) / 1e12
        fp64 = {"value": ws * args.steps * B / (ms_fp64 / 1e3 * args.steps), "unit": "J builds/s",
                "ms_per_step": ms_fp64, "ms_per_build": ms64_build,
                "relerr_vs_fp64_oracle": max(rel(results["fp64"]["J"][i], i) for i in sample),
                "roofline": {"bound": "fp64" if fpk * 1e12 / (rep64["alg_flops"] / bytes64) < peak * 1e9 else "hbm",
                             "achieved": tf, "peak": fpk, "unit": "TFLOP/s", "frac": tf / fpk,
                             "peak_kind": "measured (cuBLAS DGEMM 4096^3 in this run)",
                             "alg_flops_per_build": rep64["alg_flops"], "alg_bytes_per_build": bytes64,
                             "hbm_achieved_gbs": bytes64 / (ms64_build / 1e3) / 1e9,
                             "hbm_frac": bytes64 / (ms64_build / 1e3) / 1e9 / peak,
                             "note": "bound = min(HBM, FP64 rate x flops/byte); the FP64 FMA rate binds"},
                "clocks": {k: results["fp64"]["clocks"][k] for k in ("sm_mhz", "sm_max_mhz", "reasons")}}

    bytes16 = rep_best["alg_matrix_bytes"] + n16 * (rep_best["alg_vector_bytes"] + 2 * 8 * nbf * nbf)
    out = {
        "metric": METRIC, "value": value, "unit": "J builds/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_best, "builds_per_step": B, "ms_per_build": ms_build,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2+f64" if best == "mixed" else "f64", "precision": best, "parallelism": f"replicas x{ws}",
        "data": "synthetic (generated alkane geometry, seeded densities)",
        "config": dict(WORKLOAD),
        "fp64": fp64,
        "relerr_vs_fp64_oracle": max(rel(results[best]["J"][i], i) for i in sample),
        "relerr_sample": "builds 0 and %d of the step against the FP64 CPU oracle" % (B - 1),
        "e2e": {"value": ws * args.steps * B / e2e_s, "unit": "J builds/s",
                "h2d_bytes_per_step": 8 * nbf * nbf * B, "d2h_bytes_per_step": 8 * nbf * nbf * B,
                "api": "H2ERI_build_Coulomb (reference signature), page-locked host buffers",
                "relerr_vs_fp64_oracle": max(rel(Je2e[i], i) for i in sample)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": ("persistent tile kernel k_tile_px (one launch per J build, timed as the step / "
                                "builds)" if rep_best["persist"] and best == "mixed" else
                                "tile kernels %s (all launches of one J build, timed as the step / builds)"
                                % ("k_tile_mx" if best == "mixed" else "k_tile<FMT_F64>")),
                     "alg_bytes_per_build": alg_bytes, "peak_kind": peak_kind},
        "cpu_baseline": {"value": cpu_v, "unit": "J builds/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{cpu_n} J builds of the workload in {cpu_dt:.1f} s (oracle, OpenMP)"},
        "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"],
                   "samples": clk["samples"]},
        "gpu_launches": launches_per_J * B * args.steps,
        "phase_ms_last_host_call": {k: h.report()[k] for k in ("ms_fwd", "ms_mid", "ms_bwd", "ms_den", "ms_total")},
        "multi_density": {"n_den": n16, "value": ws * B / (ms16 / 1e3), "unit": "J builds/s",
                          "ms_per_launch": ms16 * n16 / B, "precision": best,
                          "relerr_vs_fp64_oracle_max": max(rel(J16[i], i) for i in range(n16)),
                          "sample": "all 16 densities of the first launch against the CPU oracle",
                          "roofline": {"bound": "hbm", "achieved": bytes16 / (ms16 * n16 / B / 1e3) / 1e9,
                                       "peak": peak, "unit": "GB/s",
                                       "frac": bytes16 / (ms16 * n16 / B / 1e3) / 1e9 / peak,
                                       "alg_bytes_per_launch": bytes16},
                          "timed_steps": clk16["timed_steps"], "timed_s": clk16["timed_s"],
                          "clocks": {k: clk16[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")}},
        "autotune": tuned,
        "setup_s": setup_s, "upload_s": upload_s,
    }
    print(json.dumps(out), flush=True)
    barrier()
    h.destroy()
    if dist is not None:
        dist.destroy_process_group()


def main():
    global BUILDS_PER_STEP
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--workload", default="c30", choices=sorted(WORKLOADS))
    ap.add_argument("--skip-cpu", action="store_true", help="skip the CPU baseline leg (profiler runs)")
    ap.add_argument("--no-autotune", action="store_true", help="default launch choices instead of tuned ones")
    ap.add_argument("--batch-size", type=int, default=8, help="molecules of the uneven batch workload")
    ap.add_argument("--builds-per-step", type=int, default=BUILDS_PER_STEP,
                    help="J builds per step (one density each); smaller for profiler captures")
    ap.add_argument("--path", default="coulomb", choices=["coulomb", "exchange", "setup"],
                    help="coulomb: J builds (the headline); exchange: K builds (H2ERI_build_exchange); "
                         "setup: seconds per host set-up (CPU only)")
    args = ap.parse_args()
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS[args.workload])
    BUILDS_PER_STEP = max(16, args.builds_per_step)
    if args.warmup < 3:
        args.warmup = 3
    if args.path == "setup":
        run_setup(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
