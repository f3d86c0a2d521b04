"""Benchmark: converged circuit solves/s of batched SPICE operating points on GB300.

Workload (the headline configuration): DC operating points of 16,384 seeded
single-stage BJT common-emitter amplifiers (IS log-U[1e-16, 1e-14] A, BF
U[50, 300], R1 R2 RC RE log-U[100 ohm, 1 Mohm], Vcc U[5, 15] V) at SPICE reltol
1e-6 / abstol 1e-12.  One step = one batched operating point of all circuits.

  plain  : generic kernel, FP64 LU, standard Newton start (InitJct): the
           reference's algorithm as it stands
  chosen : per-topology kernel, FP32 LU + FP64 Newton residual, the learned
           Newton start (BF16 MLP) refined by the FP32 Newton stage, then the
           FP64 Newton (FP64 device evaluation, the reference's convergence
           test and fallback chain) and the learned start's basin check

Every combination of kernel, LU precision, start and FP32 stage is timed as a
variant.  value is the chosen path with inputs resident in HBM; e2e is the same
through the C ABI with host buffers (values H2D, solutions D2H) inside the timed
region.  Between timed steps L2 is flushed (a 512 MB write); each step is timed
with CUDA events on the launching stream.  The chosen path's results are
checked against the CPU oracle (status per circuit, node voltages within
reltol/vntol) and the run exits 3 after printing its line when they are not.
With the headline workload the line also carries the op-amp workload
(65,536 two-stage CMOS op-amps, 24-D parameters, learned start) under
"cmos_opamp", measured the same way.  --impl reference times the CPU
restatement of the reference's Go path (the reference cannot be built here: no
Go toolchain) over all host cores on a bounded sample of the same workload.
"""
import argparse
import ctypes
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged circuit solves/s @ SPICE reltol, chosen vs plain GPU; Newton iters"
UNIT = "solves/s"
RELTOL = 1e-6
# workload -> (default circuits, compulsory bytes per solve: parameters in + node voltages out, 8 B each)
WORKLOADS = {"bjt_ce": (16384, (7 + 5) * 8), "cmos_opamp": (65536, (24 + 7) * 8), "rc_ladder": (4096, 0),
             "random_netlists": (8192, 0), "bjt_ce_ac": (16384, 0), "power_grid": (64, 0), "evo_lowpass": (16384, 0)}
# timed steps when --steps is not given (the headline times about 200 steps)
DEFAULT_STEPS = {"bjt_ce": 200, "cmos_opamp": 5, "rc_ladder": 20, "random_netlists": 1, "bjt_ce_ac": 20,
                 "power_grid": 1, "evo_lowpass": 5}
# most FP32 Newton iterations of the chosen path's start stage (its gmin / source-stepping chain included)
FP32_START = {"bjt_ce": 200, "cmos_opamp": 6000}
# torn power grid: 256 x 256 mesh in 4 x 4 pieces, 1,024 clamped loads, 500 backward-Euler steps of 0.1 ns
POWER_GRID = dict(N=256, P=4, loads=1024)
POWER_STEPS, POWER_H = 500, 0.1e-9
# AC workload: unit of work = the small-signal solve of one circuit at one frequency
AC_UNIT = "AC frequency points/s"
AC_SPEC = ("dec", 10, 10.0, 1e10)  # 10 points per decade, 10 Hz .. 10 GHz: 91 frequencies
RANDOM_SPEC = dict(step=5e-9, stop=2000 * 5e-9, fixed_step=True, method="trap")  # 2,000 TRAP steps of 5 ns
# transient workloads: unit of work = one accepted time point of one circuit
TRAN_UNIT = "accepted time points/s"
RC_LADDER_SPEC = dict(step=10e-9, stop=10e-6, fixed_step=True, method="trap")  # 1,000 TRAP steps of 10 ns


def generator(name):
    from kronspice_gb300 import workloads
    return {"bjt_ce": workloads.bjt_ce_batch, "cmos_opamp": workloads.cmos_opamp_batch,
            "rc_ladder": workloads.rc_ladder_batch, "bjt_ce_ac": workloads.bjt_ce_ac_batch}[name]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=0, help="timed steps (0: the workload's default)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--n-circ", type=int, default=0)
    p.add_argument("--workload", default="bjt_ce", choices=sorted(WORKLOADS))
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--tran-steps", type=int, default=0, help="time steps of the transient workloads (0: the workload's)")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                   help="LU precision of the chosen path")
    p.add_argument("--variants", type=int, default=1, help="also time every kernel/precision/start combination")
    p.add_argument("--start-cache", default=None,
                   help="learned-start network file (.npz): loaded when present, else trained and saved there")
    p.add_argument("--fp32-start", type=int, default=-1,
                   help="most FP32 Newton iterations of the chosen path's start stage (-1: the workload's, 0: off)")
    p.add_argument("--secondary", type=int, default=1,
                   help="with the headline workload, also run the op-amp learned-start workload")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(el, nn, vals, min_wall=1.0, max_passes=400):
    """Oracle (CPU restatement of the reference path) over all host threads."""
    from oracle import oracle as orc
    orc.build()
    nthreads = os.cpu_count() or 1
    pk = orc.Packed(el, nn, vals)
    opt = orc.options(reltol=RELTOL)
    orc.batch_op(pk, min(256, len(vals)), opt, nthreads=nthreads)  # warm-up
    done, t0 = 0, time.perf_counter()
    passes = 0
    while True:
        st, x, it = orc.batch_op(pk, len(vals), opt, nthreads=nthreads)
        done += int((st == 0).sum())
        passes += 1
        wall = time.perf_counter() - t0
        if wall >= min_wall or passes >= max_passes:
            break
    return {"value": done / wall, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d passes over the %d-circuit batch (%.2f s wall, %.1f core-s), oracle/ks_oracle.cpp "
                      "(C++ restatement of the Go path; no Go toolchain to build the reference)"
                      % (passes, len(vals), wall, wall * nthreads),
            "newton_iters_mean": float(it.mean())}


class Clocks:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, gpu_index):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [s.strip() for s in line.split(",")]
                if len(p) < 9 or p[0] != str(gpu_index):
                    continue
                try:
                    sm.append(float(p[1]))
                    smax = float(p[2])
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def traffic_from_profile():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_reference_tran(args):
    el, nn, vals = generator(args.workload)(args.n_circ, args.seed)
    from oracle import oracle as orc
    from kronspice_gb300 import analysis
    orc.build()
    nthreads = os.cpu_count() or 1
    sp = analysis.TranSpec(**RC_LADDER_SPEC)
    ospec = orc.TranSpec(sp.step, sp.stop, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    samp = min(len(vals), 512)  # a bounded sample of the batch per step
    pk = orc.Packed(el, nn, vals[:samp])
    opt = orc.options(reltol=RELTOL)
    for _ in range(args.warmup):
        orc.batch_tran(pk, samp, ospec, opt, nthreads=nthreads, record=False)
    t0 = time.perf_counter()
    pts = 0
    for _ in range(args.steps):
        st, _, steps, it = orc.batch_tran(pk, samp, ospec, opt, nthreads=nthreads, record=False)
        pts += int(steps[st == 0].sum())
    wall = time.perf_counter() - t0
    value = pts / wall
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox)",
            "config": {"workload": "rc_ladder_tran_%d" % args.n_circ, "n_circuits": args.n_circ,
                       "steps_per_circuit": 1000, "method": "trap", "reltol": RELTOL, "host_threads": nthreads},
            "cpu_baseline": {"value": value, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d of the %d circuits per step, 1,000 TRAP steps each, on %d host threads; "
                                       "oracle/ks_oracle.cpp (C++ restatement of the Go path)"
                                       % (samp, args.n_circ, nthreads)},
            "e2e": {"value": value, "unit": TRAN_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_multi(args):
    from kronspice_gb300 import workloads, analysis
    from oracle import oracle as orc
    import concurrent.futures as cf
    orc.build()
    nthreads = os.cpu_count() or 1
    circuits = workloads.random_netlists(args.n_circ, args.seed)
    sp = analysis.TranSpec(**RANDOM_SPEC)
    ospec = orc.TranSpec(sp.step, sp.stop, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    samp = circuits[:4 * nthreads]  # a bounded sample of the batch per step

    def one(c):
        el, vals, _ = c.pack()
        so, _, ss, _ = orc.batch_tran(orc.Packed(el, c.n_nodes, vals[None, :]), 1, ospec, orc.options(reltol=RELTOL),
                                      nthreads=1, record=False)
        return int(ss[0]) if so[0] == 0 else 0
    t0 = time.perf_counter()
    pts = 0
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        for _ in range(max(1, args.steps)):
            pts += sum(ex.map(one, samp))
    wall = time.perf_counter() - t0
    value = pts / wall
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / max(1, args.steps) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox): random connected netlists",
            "config": {"workload": "random_netlists_tran_%d" % args.n_circ, "n_circuits": args.n_circ,
                       "steps_per_circuit": 2000, "method": "trap", "reltol": RELTOL, "host_threads": nthreads},
            "cpu_baseline": {"value": value, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d of the %d circuits per step, one per host thread; oracle/ks_oracle.cpp"
                                       % (len(samp), args.n_circ)},
            "e2e": {"value": value, "unit": TRAN_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def oracle_ac_points(el, nn, vals, freqs, nthreads, reps_min_wall=1.0, max_reps=50):
    """AC sweeps of the oracle over a thread pool (each call releases the GIL):
    (converged frequency points per second, passes, wall seconds)."""
    from oracle import oracle as orc
    import concurrent.futures as cf
    opt = orc.options(reltol=RELTOL)

    def one(i):
        st, _, _ = orc.ac(orc.Packed(el, nn, vals[i]), freqs, opt)
        return len(freqs) if st == 0 else 0
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        list(ex.map(one, range(min(len(vals), nthreads))))  # warm-up
        t0 = time.perf_counter()
        pts, reps = 0, 0
        while True:
            pts += sum(ex.map(one, range(len(vals))))
            reps += 1
            wall = time.perf_counter() - t0
            if wall >= reps_min_wall or reps >= max_reps:
                break
    return pts / wall, reps, wall


def run_reference_ac(args):
    from kronspice_gb300 import analysis
    from oracle import oracle as orc
    orc.build()
    nthreads = os.cpu_count() or 1
    el, nn, vals = generator(args.workload)(args.n_circ, args.seed)
    freqs = analysis.ACSpec(*AC_SPEC).frequencies()
    samp = vals[:min(len(vals), 64 * nthreads)]  # a bounded sample of the batch per step
    oracle_ac_points(el, nn, samp[:nthreads], freqs, nthreads, 0.0, max(1, args.warmup))
    value, reps, wall = oracle_ac_points(el, nn, samp, freqs, nthreads, 0.0, max(1, args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": AC_UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / reps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 complex",
            "data": "synthetic (seeded Philox)",
            "config": {"workload": "bjt_ce_ac_%d" % args.n_circ, "n_circuits": args.n_circ,
                       "frequencies": len(freqs), "sweep": "dec 10 points, 10 Hz .. 10 GHz", "reltol": RELTOL,
                       "host_threads": nthreads},
            "cpu_baseline": {"value": value, "unit": AC_UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d of the %d circuits per step (operating point, polish and %d complex "
                                       "solves each) on %d host threads; oracle/ks_oracle.cpp (C++ restatement "
                                       "of the Go path)" % (len(samp), args.n_circ, len(freqs), nthreads)},
            "e2e": {"value": value, "unit": AC_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def oracle_grid_points(el, nn, vals, steps, min_wall=10.0):
    """Accepted points/s of the oracle's untorn sparse transient (the reference's
    backend for large systems) on the power grid: a bounded sample of steps of
    one variant per host thread, timed in parallel."""
    from oracle import oracle as orc
    import concurrent.futures as cf
    nthreads = os.cpu_count() or 1
    spec = orc.TranSpec(POWER_H, steps * POWER_H, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)

    def one(v):
        r = orc.tran(orc.Packed(el, nn, vals[v % len(vals)]), spec, orc.options(reltol=RELTOL), capacity=2,
                     currents=False)
        return r[4] if r[0] == 0 else 0
    t0 = time.perf_counter()
    pts, runs = 0, 0
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        while time.perf_counter() - t0 < min_wall or runs == 0:
            pts += sum(ex.map(one, range(runs, runs + nthreads)))
            runs += nthreads
    wall = time.perf_counter() - t0
    return pts / wall, runs, wall, nthreads


def run_reference_torn(args):
    from kronspice_gb300 import workloads
    from oracle import oracle as orc
    orc.build()
    el, nn, vals, torn, _ = workloads.power_grid_batch(min(args.n_circ, 16), args.seed, **POWER_GRID)
    steps = 2
    value, runs, wall, nthreads = oracle_grid_points(el, nn, vals, steps, min_wall=0.0)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": args.gpus,
            "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
            "config": {"workload": "power_grid_tran_%d" % args.n_circ, "variants": args.n_circ, "grid": "256x256",
                       "pieces": 16, "steps_per_variant": POWER_STEPS, "method": "be", "host_threads": nthreads},
            "cpu_baseline": {"value": value, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d runs of %d backward-Euler steps (one variant each, operating point "
                                       "included) with the oracle's untorn sparse LU, one run per host thread; the "
                                       "reference's torn path refactors a dense 4,096-unknown piece per change and is "
                                       "slower still" % (runs, steps)},
            "e2e": {"value": value, "unit": TRAN_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "rc_ladder":
        run_reference_tran(args)
        return
    if args.workload == "random_netlists":
        run_reference_multi(args)
        return
    if args.workload == "bjt_ce_ac":
        run_reference_ac(args)
        return
    if args.workload == "evo_lowpass":
        pop, objectives, spec = evo_population(min(args.n_circ, 4096), args.seed)
        vals = []
        for _ in range(args.warmup + args.steps):
            vals.append(evo_oracle_pool(pop, objectives, spec))
        v = [x[0] for x in vals[args.warmup:]]
        value = statistics.median(v)
        print(json.dumps({"impl": "reference", "metric": "candidates scored/s (batched evaluator: OP + AC objectives)",
                          "value": value, "unit": "candidates/s", "n_gpus": 1, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": len(pop) / value * 1e3, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded candidates)",
                          "config": {"workload": "evo_lowpass_%d" % args.n_circ},
                          "cpu_baseline": {"value": value, "unit": "candidates/s", "cores": vals[-1][2],
                                           "kind": "port", "sample": "%d candidates a step" % len(pop)},
                          "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    if args.workload == "power_grid":
        run_reference_torn(args)
        return
    el, nn, vals = generator(args.workload)(args.n_circ, args.seed)
    from oracle import oracle as orc
    orc.build()
    nthreads = os.cpu_count() or 1
    pk = orc.Packed(el, nn, vals)
    opt = orc.options(reltol=RELTOL)
    for _ in range(args.warmup):
        orc.batch_op(pk, len(vals), opt, nthreads=nthreads)
    t0 = time.perf_counter()
    done = 0
    its = []
    for _ in range(args.steps):
        st, x, it = orc.batch_op(pk, len(vals), opt, nthreads=nthreads)
        done += int((st == 0).sum())
        its.append(it)
    wall = time.perf_counter() - t0
    value = done / wall
    it = np.concatenate(its)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox)",
            "config": {"workload": "%s_op_%d" % (args.workload, args.n_circ), "n_circuits": args.n_circ, "reltol": RELTOL,
                       "abstol": 1e-12, "host_threads": nthreads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d steps of the full %d-circuit batch on %d host threads; oracle/ks_oracle.cpp, "
                                       "the C++ restatement of the reference's Go path (no Go toolchain here)"
                                       % (args.steps, args.n_circ, nthreads)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "newton_iters_mean": float(it.mean()), "newton_iters_max": int(it.max())}
    print(json.dumps(line))



def bench_tran(args):
    """The RC-ladder transient: 4,096 seeded 10-section ladders, 1,000 fixed TRAP
    steps of 10 ns each; unit of work = one accepted time point of one circuit."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kronspice_gb300 import analysis, build
    build.build()
    dev = torch.device("cuda", local)
    el, nn, vals = generator(args.workload)(args.n_circ, args.seed + rank)
    B = vals.shape[0]
    plan = analysis.Plan(el, nn, vals.shape[1])
    batch = analysis.Batch(plan, vals)
    n = plan.n
    sp = analysis.TranSpec(**RC_LADDER_SPEC)
    npts = int(round(sp.stop / sp.step)) + 1
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sh = ctypes.c_void_p(stream.cuda_stream)
    wave = torch.empty((npts, B, n), dtype=torch.float64, device=dev)
    ints = torch.empty((4, B), dtype=torch.int32, device=dev)  # npts, status, steps, iters
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    spec_info = None
    try:
        kname, csec = plan.specialize("tran")
        spec_info = {"kernel": kname, "nvrtc_s": csec}
    except RuntimeError as e:
        spec_info = {"kernel": None, "error": str(e)[:200]}
    spec_ok = spec_info["kernel"] is not None
    plain_opt = analysis.Options(reltol=RELTOL, precision="fp64", kernel="generic")
    chosen_opt = analysis.Options(reltol=RELTOL, precision=args.precision, kernel="specialized" if spec_ok else "generic")

    def step(opt):
        batch.tran_async(sp, opt, 0, None, wave.data_ptr(), ints[0].data_ptr(), ints[1].data_ptr(),
                         ints[2].data_ptr(), ints[3].data_ptr(), sh)

    def timed(opt):
        for _ in range(args.warmup):
            step(opt)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(opt)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        iv = ints.cpu().numpy()
        ok = iv[1] == 0
        pts = int(iv[2][ok].sum())
        return {"seconds": total, "ms_per_step": total / args.steps * 1e3, "points": pts, "ok": int(ok.sum()),
                "iters_per_point": float(iv[3][ok].sum() / max(pts, 1)), "status": iv[1].copy()}

    clk = Clocks(os.path.join(tempfile.gettempdir(),
                              "bench_clocks_%d.csv" % rank))
    variants = {}
    with clk:
        plain = timed(plain_opt)
        chosen = timed(chosen_opt)
        chosen_wave = wave[:, :64].cpu().numpy()  # parity sample
        if args.variants:
            for kern in (["generic", "specialized"] if spec_ok else ["generic"]):
                for prec in ("fp64", "mixed"):
                    r = timed(analysis.Options(reltol=RELTOL, precision=prec, kernel=kern))
                    variants["%s/%s" % (kern, prec)] = {"ms_per_step": r["ms_per_step"],
                                                         "points_per_s": r["points"] * args.steps / r["seconds"]}
    clocks = clk.summary(local)

    # end to end through the C ABI: pinned host values in, host waveforms out
    L = __import__("kronspice_gb300._lib", fromlist=["x"]).load()
    vals_pin = torch.from_numpy(vals.copy()).pin_memory()
    wave_host = torch.empty((npts, B, n), dtype=torch.float64).pin_memory()
    ints_host = torch.empty((4, B), dtype=torch.int32).pin_memory()
    o = chosen_opt.c()
    spc = sp.c()

    def e2e_step():  # ks_batch_set_values + ks_tran, both on host buffers
        rc = L.ks_batch_set_values(batch.handle, ctypes.c_void_p(vals_pin.data_ptr()), 0, sh)
        assert rc == 0
        ip = ints_host.data_ptr()
        rc = L.ks_tran(batch.handle, ctypes.byref(spc), ctypes.byref(o), 0, None, ctypes.c_void_p(wave_host.data_ptr()),
                       ctypes.c_void_p(ip), ctypes.c_void_p(ip + 4 * B), ctypes.c_void_p(ip + 8 * B),
                       ctypes.c_void_p(ip + 12 * B), sh)
        assert rc == 0
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize()
        e2e_t += time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_t], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_value = world * chosen["points"] * args.steps / e2e_t
    value = world * chosen["points"] * args.steps / chosen["seconds"]
    plain_value = world * plain["points"] * args.steps / plain["seconds"]
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    from oracle import oracle as orc
    ospec = orc.TranSpec(sp.step, sp.stop, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    so, xo, _, _ = orc.batch_tran(orc.Packed(el, nn, vals[:64]), 64, ospec, orc.options(reltol=RELTOL))
    okm = (so == 0) & (chosen["status"][:64] == 0)
    max_err = float(np.max(np.abs(chosen_wave[:, okm, :nn - 1] - xo[:, okm, :nn - 1]))) if okm.any() else None

    # CPU baseline: the oracle on a bounded sample of the same workload, all host threads
    nthreads = os.cpu_count() or 1
    samp = 256
    pk = orc.Packed(el, nn, vals[:samp])
    t0 = time.perf_counter()
    cpts, reps = 0, 0
    while True:
        st_c, _, steps_c, _ = orc.batch_tran(pk, samp, ospec, orc.options(reltol=RELTOL), nthreads=nthreads,
                                             record=False)
        cpts += int(steps_c[st_c == 0].sum())
        reps += 1
        if time.perf_counter() - t0 > 1.0 or reps >= 50:
            break
    cwall = time.perf_counter() - t0
    cpu = {"value": cpts / cwall, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
           "sample": "%d passes over %d of the circuits, 1,000 TRAP steps each (%.2f s wall); oracle/ks_oracle.cpp"
                     % (reps, samp, cwall)}

    per_launch_s = chosen["seconds"] / args.steps
    alg_bytes = B * (npts * n * 8 + vals.shape[1] * 8)  # recorded waveform + each circuit's values once
    achieved = alg_bytes / per_launch_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    kname = "ks_spec_tran" if chosen_opt.kernel == "specialized" else "k_tran"
    prof = traffic_from_profile().get("%s_rc_ladder" % kname, {})
    traffic = prof.get("dram_bytes_per_circuit")
    line = {
        "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": chosen["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 device eval + residual, f32 LU" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded Philox)",
        "config": {"workload": "rc_ladder_tran_%d" % B, "n_circuits_per_gpu": B, "n_unknowns": n,
                   "steps_per_circuit": npts - 1, "step_s": sp.step, "method": "trap", "reltol": RELTOL,
                   "l2": "flushed between timed steps (512 MB write); the 393 MB waveform output exceeds L2"},
        "plain": {"value": plain_value, "ms_per_step": plain["ms_per_step"], "precision": "fp64",
                  "kernel": "generic"},
        "chosen": {"value": value, "precision": args.precision, "kernel": chosen_opt.kernel,
                   "newton_iters_per_point": chosen["iters_per_point"]},
        "chosen_vs_plain": value / plain_value if plain_value else None,
        "per_topology_kernel": spec_info,
        "variants": variants or None,
        "max_node_voltage_err_vs_oracle": max_err,
        "e2e": {"value": e2e_value, "unit": TRAN_UNIT, "h2d_bytes_per_step": int(vals.nbytes),
                "d2h_bytes_per_step": int(wave_host.numel() * 8 + ints_host.numel() * 4)},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None if traffic is None else traffic * B, "kernel": kname,
                     "algorithmic_bytes_per_point": n * 8 + vals.shape[1] * 8 / (npts - 1),
                     "note": "the transient kernel is bound by FP64 issue per Newton step (one circuit per thread); "
                             "achieved counts the recorded waveform plus each circuit's value vector"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


def evo_population(n, seed):
    """n seeded candidates of a loaded RC low-pass (R 0.5-5 kOhm, C 1-100 nF, load
    2-20 kOhm), the value genome of a filter search, and its objectives: the gain
    at 1 kHz (-3 dB target, 51-point AC sweep 10 Hz-1 MHz), the output's operating
    point (1 V target), the supply power and the model-supplied power limit."""
    import numpy as np
    from kronspice_gb300 import analysis, evo
    from kronspice_gb300 import circuit as kc
    g = np.random.default_rng(seed)
    pop = []
    for r, c, rl in zip(g.uniform(500, 5e3, n), g.uniform(1e-9, 1e-7, n), g.uniform(2e3, 2e4, n)):
        b = kc.Builder("lowpass")
        b.voltage_source("V1", "in", "0", 2.0, ac=(1.0, 0.0))
        b.resistor("R1", "in", "out", r).capacitor("C1", "out", "0", c).resistor("RL", "out", "0", rl)
        pop.append(b.build())
    spec = analysis.ACSpec("dec", 10, 10.0, 1e6)
    objectives = [evo.gain_at_objective("out", "in", spec, 1e3, -3.0), evo.op_voltage("out", 1.0),
                  evo.supply_power("V1"), evo.model_supplied_limit(0.0)]
    return pop, objectives, spec


def bench_evo(args):
    """A generation of an evolutionary filter search scored by the batched
    evaluator (kronspice_gb300/evo.py): host circuits in, scored individuals out
    (validation, packing, the batched OP and AC on the GPU, the objectives).
    Unit = one scored candidate; a step = one generation of n_circ candidates.
    The CPU line is the reference's worker pool restated: the oracle's OP and AC
    per candidate on every host thread, the same objective code."""
    import numpy as np
    import torch
    from kronspice_gb300 import build, evo
    from oracle import oracle as orc
    build.build()
    orc.build()
    pop, objectives, spec = evo_population(args.n_circ, args.seed)
    for _ in range(max(1, args.warmup)):
        evo.evaluate(pop, objectives)
    torch.cuda.synchronize()
    clk = Clocks(os.path.join(tempfile.gettempdir(), "bench_clocks_evo.csv"))
    with clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out = evo.evaluate(pop, objectives)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    clocks = clk.summary(0)
    value = args.n_circ * args.steps / wall
    failures = sum(1 for ind in out if ind.failure)
    cpu_value, cpu_wall, nthreads, cpu_fit = evo_oracle_pool(pop[:min(len(pop), 4096)], objectives, spec)
    sample = pop[:len(cpu_fit)]
    gpu_fit = np.array([ind.fitness for ind in out[:len(sample)]])
    parity = float(np.max(np.abs(gpu_fit - np.array(cpu_fit)) / np.maximum(np.abs(cpu_fit), 1e-12)))
    el, v0, _ = pop[0].pack()
    n = int(orc.unknowns(orc.Packed.of(pop[0]))[0])
    nf = len(spec.frequencies())
    h2d = args.n_circ * len(v0) * 8 + len(el) * 48 + nf * 8
    d2h = args.n_circ * (8 * (n + len(el) * 7 + 8) + 8 * nf * n * 2 + 4 * 4)
    line = {
        "metric": "candidates scored/s (batched evaluator: OP + AC objectives)", "value": value,
        "unit": "candidates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded candidates)",
        "config": {"workload": "evo_lowpass_%d" % args.n_circ, "candidates": args.n_circ,
                   "objectives": [ob.name for ob in objectives], "ac_points": nf,
                   "l2": "a generation's arrays are far below L2; each step builds, uploads and solves anew"},
        "failures": failures, "max_fitness_rel_diff_vs_oracle": parity,
        "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": None,
        "roofline_note": "host-bound: per generation the candidates are packed and validated on the host and "
                         "the objectives read the batched results; the GPU analyses are a small part of a step",
        "gpu_launches": 9 * args.steps,
        "cpu_baseline": {"value": cpu_value, "unit": "candidates/s", "cores": nthreads, "kind": "port",
                         "sample": "%d candidates scored through the oracle's OP and AC, one per host thread "
                                   "at a time (%.1f s wall)" % (len(sample), cpu_wall)},
        "clocks": clocks,
    }
    print(json.dumps(line))


def evo_oracle_pool(sample, objectives, spec):
    """The reference's worker pool restated (evo/engine.go:518-543): each host
    thread scores one candidate at a time through the oracle's OP and AC and the
    same objective code.  (candidates/s, wall s, threads, fitnesses)."""
    import concurrent.futures as cf
    from kronspice_gb300 import analysis, evo
    from oracle import oracle as orc
    orc.build()
    freqs = spec.frequencies()

    class OracleEval:
        def __init__(self, ckt):
            self.circuit, self.model_supplied, self.pk = ckt, 0.0, orc.Packed.of(ckt)

        def op(self):
            st, x, elem, led, _, _ = orc.op_results(self.pk)
            err = analysis.status_error(st)
            if err:
                raise err
            return evo.OPResult(self.circuit, x, elem, led)

        def ac(self, sp):
            st, x, _ = orc.ac(self.pk, freqs)
            err = analysis.status_error(st)
            if err:
                raise err
            return evo.ACResult(self.circuit, freqs, x)

    def score(ckt):
        e = OracleEval(ckt)
        return sum(ob.weight * ob.eval(e) for ob in objectives)

    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(nthreads) as ex:
        fits = list(ex.map(score, sample))
    wall = time.perf_counter() - t0
    return len(sample) / wall, wall, nthreads, fits


def bench_multi(args):
    """8,192 seeded random netlists of 10-400 nodes (each its own topology), one
    transient of 2,000 fixed TRAP steps each; unit = one accepted time point of
    one circuit.  A step of the bench is the whole batch's transient."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kronspice_gb300 import analysis, build, workloads
    build.build()
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    circuits = workloads.random_netlists(args.n_circ, args.seed + rank)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    mb = analysis.MultiBatch(circuits)
    t_create = time.perf_counter() - t0
    sp = analysis.TranSpec(**RANDOM_SPEC)
    npts = int(round(sp.stop / sp.step)) + 1
    B, N = mb.n_circ, mb.total_unknowns
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sh = ctypes.c_void_p(stream.cuda_stream)
    wave = torch.empty(npts * N, dtype=torch.float64, device=dev)
    ints = torch.empty((4, B), dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    plain_opt = analysis.Options(reltol=RELTOL, precision="fp64")
    chosen_opt = analysis.Options(reltol=RELTOL, precision=args.precision)

    def step(opt):
        mb.tran_async(sp, opt, wave.data_ptr(), ints[0].data_ptr(), ints[1].data_ptr(), ints[2].data_ptr(),
                      ints[3].data_ptr(), sh)

    def timed(opt):
        for _ in range(args.warmup):
            step(opt)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(opt)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        iv = ints.cpu().numpy()
        ok = iv[1] == 0
        return {"seconds": total, "ms_per_step": total / args.steps * 1e3, "points": int(iv[2][ok].sum()),
                "ok": int(ok.sum()), "iters_per_point": float(iv[3][ok].sum() / max(1, iv[2][ok].sum())),
                "status": iv[1].copy()}

    clk = Clocks(os.path.join(tempfile.gettempdir(),
                              "bench_clocks_%d.csv" % rank))
    with clk:
        plain = timed(plain_opt)
        chosen = timed(chosen_opt)
        wave_h = wave.cpu().numpy()
    clocks = clk.summary(local)
    value = world * chosen["points"] * args.steps / chosen["seconds"]
    plain_value = world * plain["points"] * args.steps / plain["seconds"]
    # end to end through the C ABI with host buffers (ks_multi_tran)
    L = __import__("kronspice_gb300._lib", fromlist=["x"]).load()
    wave_host = torch.empty(npts * N, dtype=torch.float64).pin_memory()
    ints_host = torch.empty((4, B), dtype=torch.int32).pin_memory()
    o, spc = chosen_opt.c(), sp.c()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ip = ints_host.data_ptr()
    rc = L.ks_multi_tran(mb.handle, ctypes.byref(spc), ctypes.byref(o), ctypes.c_void_p(wave_host.data_ptr()),
                         ctypes.c_void_p(ip + 4 * B), ctypes.c_void_p(ip + 8 * B), ctypes.c_void_p(ip + 12 * B))
    assert rc == 0
    e2e_t = time.perf_counter() - t0
    e2e_value = world * chosen["points"] / e2e_t
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return
    # parity on a sample against the oracle, and the CPU baseline on a bounded sample
    from oracle import oracle as orc
    ospec = orc.TranSpec(sp.step, sp.stop, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    max_err, samp = 0.0, list(range(0, B, max(1, B // 16)))[:16]
    for k in samp:
        c = circuits[k]
        el, vals, _ = c.pack()
        so, xo, _, _ = orc.batch_tran(orc.Packed(el, c.n_nodes, vals[None, :]), 1, ospec, orc.options(reltol=RELTOL))
        if so[0] == 0 and chosen["status"][k] == 0:
            n = int(mb.n[k])
            w = wave_h[npts * mb.x_off[k]:npts * (mb.x_off[k] + n)].reshape(npts, n)
            nn = c.n_nodes - 1
            max_err = max(max_err, float(np.max(np.abs(w[:, :nn] - xo[:, 0, :nn]))))
    nthreads = os.cpu_count() or 1
    csamp = circuits[:64]
    t0 = time.perf_counter()
    cpts = 0
    import concurrent.futures as cf

    def one(c):
        el, vals, _ = c.pack()
        so, _, ss, _ = orc.batch_tran(orc.Packed(el, c.n_nodes, vals[None, :]), 1, ospec, orc.options(reltol=RELTOL),
                                      nthreads=1, record=False)
        return int(ss[0]) if so[0] == 0 else 0
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        cpts = sum(ex.map(one, csamp))
    cwall = time.perf_counter() - t0
    cpu = {"value": cpts / cwall, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
           "sample": "the first 64 of the circuits, 2,000 TRAP steps each, one circuit per host thread (%.1f s "
                     "wall); oracle/ks_oracle.cpp with the reference's dense/sparse solver rule" % cwall}
    line = {
        "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": chosen["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 device eval + residual, f32 LU" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded Philox): random connected netlists",
        "config": {"workload": "random_netlists_tran_%d" % B, "n_circuits_per_gpu": B, "nodes": "10-400",
                   "unknowns_total": N, "steps_per_circuit": npts - 1, "step_s": sp.step, "method": "trap",
                   "reltol": RELTOL, "lu_multiply_adds_per_factorization_of_all": mb.lu_flops,
                   "l2": "flushed between timed steps (512 MB write)",
                   "host_setup_s": {"generate": t_gen, "symbolic": t_create}},
        "plain": {"value": plain_value, "ms_per_step": plain["ms_per_step"], "precision": "fp64",
                  "ok": plain["ok"]},
        "chosen": {"value": value, "precision": args.precision, "ok": chosen["ok"],
                   "newton_iters_per_point": chosen["iters_per_point"]},
        "chosen_vs_plain": value / plain_value if plain_value else None,
        "max_node_voltage_err_vs_oracle": max_err,
        "e2e": {"value": e2e_value, "unit": TRAN_UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(npts * N * 8 + 12 * B),
                "note": "values are uploaded once at batch creation (ks_multi_create)"},
        "gpu_launches": args.steps * 2,
        "roofline": {"bound": "hbm", "achieved": None, "peak": None, "unit": "GB/s", "frac": None, "traffic": None,
                     "note": "latency bound: one warp per circuit walks its sparse factorization row by row"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


def bench_ac(args):
    """AC sweeps of 16,384 seeded common-emitter amplifiers (input coupling and
    emitter bypass capacitors, Gummel-Poon transistor with junction, transit-time
    and substrate charges), 91 frequencies from 10 Hz to 10 GHz; unit of work =
    one circuit's small-signal solve at one frequency.  One step = ks_ac_async:
    operating point + polish + model + sweep of every circuit."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kronspice_gb300 import analysis, build
    build.build()
    dev = torch.device("cuda", local)
    el, nn, vals = generator(args.workload)(args.n_circ, args.seed + rank)
    B = vals.shape[0]
    plan = analysis.Plan(el, nn, vals.shape[1])
    batch = analysis.Batch(plan, vals)
    n = plan.n
    freqs = analysis.ACSpec(*AC_SPEC).frequencies()
    nf = len(freqs)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sh = ctypes.c_void_p(stream.cuda_stream)
    f_dev = torch.from_numpy(freqs).to(dev)
    xac = torch.empty((B, nf, n, 2), dtype=torch.float64, device=dev)
    x_op = torch.empty((B, n), dtype=torch.float64, device=dev)
    ints = torch.empty((3, B), dtype=torch.int32, device=dev)  # status, iters, sweep status
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    try:
        kname, csec = plan.specialize("op")
        spec_info = {"kernel": kname, "nvrtc_s": csec}
    except RuntimeError as e:
        spec_info = {"kernel": None, "error": str(e)[:200]}
    spec_ok = spec_info["kernel"] is not None
    plain_opt = analysis.Options(reltol=RELTOL, precision="fp64", kernel="generic")
    chosen_opt = analysis.Options(reltol=RELTOL, precision="fp64", kernel="specialized" if spec_ok else "generic")

    def step(opt):
        batch.ac_async(opt, None, f_dev.data_ptr(), nf, xac.data_ptr(), ints[0].data_ptr(), ints[1].data_ptr(), sh)

    def sweep(opt):
        batch.ac_at_async(opt, x_op.data_ptr(), ints[0].data_ptr(), f_dev.data_ptr(), nf, xac.data_ptr(),
                          ints[2].data_ptr(), sh)

    def timed(fn, opt):
        for _ in range(args.warmup):
            fn(opt)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(opt)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        iv = ints.cpu().numpy()
        return {"seconds": total, "ms_per_step": total / args.steps * 1e3, "ok": int((iv[0] == 0).sum()),
                "iters_mean": float(iv[1].mean()), "status": iv[0].copy()}

    clk = Clocks(os.path.join(tempfile.gettempdir(),
                              "bench_clocks_%d.csv" % rank))
    with clk:
        plain = timed(step, plain_opt)
        chosen = timed(step, chosen_opt)
        x_chosen = xac[:64].cpu().numpy()
        st_chosen = chosen["status"]
        # the sweep alone (k_ac_model + k_ac_solve) about the operating points
        batch.op_async(chosen_opt, None, x_op.data_ptr(), ints[0].data_ptr(), ints[1].data_ptr(), sh)
        sw = timed(sweep, chosen_opt)
    clocks = clk.summary(local)

    # end to end through the C ABI: pinned host values in, host phasors out
    L = __import__("kronspice_gb300._lib", fromlist=["x"]).load()
    vals_pin = torch.from_numpy(vals.copy()).pin_memory()
    x_host = torch.empty((B, nf, n, 2), dtype=torch.float64).pin_memory()
    s_host = np.zeros(B, dtype=np.int32)
    i_host = np.zeros(B, dtype=np.int32)
    o = chosen_opt.c()

    def e2e_step():
        rc = L.ks_batch_set_values(batch.handle, ctypes.c_void_p(vals_pin.data_ptr()), 0, sh)
        assert rc == 0
        rc = L.ks_ac(batch.handle, ctypes.byref(o), None, freqs.ctypes.data, nf, ctypes.c_void_p(x_host.data_ptr()),
                     s_host.ctypes.data, i_host.ctypes.data, sh)
        assert rc == 0
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize()
        e2e_t += time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_t], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_value = world * int((s_host == 0).sum()) * nf * args.steps / e2e_t
    value = world * chosen["ok"] * nf * args.steps / chosen["seconds"]
    plain_value = world * plain["ok"] * nf * args.steps / plain["seconds"]
    sweep_value = world * sw["ok"] * nf * args.steps / sw["seconds"]
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    # accuracy against the oracle on a sample, relative to each unknown's largest magnitude over the sweep
    from oracle import oracle as orc
    orc.build()
    worst = 0.0
    for c in range(64):
        so, xo, _ = orc.ac(orc.Packed(el, nn, vals[c]), freqs, orc.options(reltol=RELTOL))
        if so or st_chosen[c]:
            continue
        xg = x_chosen[c, ..., 0] + 1j * x_chosen[c, ..., 1]
        scale = np.maximum(np.abs(xo).max(axis=0), 1e-5 * np.abs(xo).max())
        worst = max(worst, float((np.abs(xg - xo) / scale).max()))
    nthreads = os.cpu_count() or 1
    cval, reps, cwall = oracle_ac_points(el, nn, vals[:min(B, 16 * nthreads)], freqs, nthreads, 1.0, 20)
    cpu = {"value": cval, "unit": AC_UNIT, "cores": nthreads, "kind": "port",
           "sample": "%d passes over %d of the circuits (operating point, polish, %d complex solves each; %.2f s "
                     "wall); oracle/ks_oracle.cpp" % (reps, min(B, 16 * nthreads), nf, cwall)}

    # roofline of the sweep kernels: phasors out (16 B per unknown per point) plus each circuit's
    # values, operating point and G / C / b columns once; FP64-bound (complex LU per point)
    per_launch_s = sw["seconds"] / args.steps
    alg_bytes = B * (nf * n * 16 + vals.shape[1] * 8 + n * 8 + (2 * n * n + 2 * n) * 8 * 2)
    achieved = alg_bytes / per_launch_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    # FP64 operations of one point (complex multiply-add = 8): Y build 2n^2, LU sum_k (n-k-1)^2 * 8 +
    # (n-k-1) * 6, substitutions 8 n^2
    lu = sum((n - k - 1) ** 2 * 8 + (n - k - 1) * 6 for k in range(n))
    flops = 2 * n * n + lu + 8 * n * n
    prof = traffic_from_profile().get("k_ac_solve_bjt_ce_ac", {})
    traffic = prof.get("dram_bytes_per_circuit")
    line = {
        "metric": METRIC, "value": value, "unit": AC_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": chosen["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 complex", "data": "synthetic (seeded Philox)",
        "config": {"workload": "bjt_ce_ac_%d" % B, "n_circuits_per_gpu": B, "n_unknowns": n, "frequencies": nf,
                   "sweep": "dec 10 points, 10 Hz .. 10 GHz", "reltol": RELTOL,
                   "l2": "flushed between timed steps (512 MB write); the 238 MB phasor output is written once"},
        "plain": {"value": plain_value, "ms_per_step": plain["ms_per_step"], "op_kernel": "generic"},
        "chosen": {"value": value, "op_kernel": chosen_opt.kernel, "newton_iters_mean": chosen["iters_mean"]},
        "chosen_vs_plain": value / plain_value if plain_value else None,
        "sweep_only": {"value": sweep_value, "ms_per_step": sw["ms_per_step"]},
        "per_topology_kernel": spec_info,
        "max_phasor_err_vs_oracle_rel": worst,
        "e2e": {"value": e2e_value, "unit": AC_UNIT, "h2d_bytes_per_step": int(vals.nbytes + freqs.nbytes),
                "d2h_bytes_per_step": int(x_host.numel() * 8 + s_host.nbytes + i_host.nbytes)},
        "gpu_launches": 5 * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None if traffic is None else traffic * B, "kernel": "k_ac_model + k_ac_solve",
                     "algorithmic_bytes_per_circuit": alg_bytes / B, "kernel_ms": per_launch_s * 1e3,
                     "fp64_flops_per_point": flops,
                     "fp64_tflops": flops * B * nf / per_launch_s / 1e12,
                     "note": "the sweep is bound by FP64 issue (complex LU per point, one point per thread; "
                             "GB300 has 2 FP64 lanes/clk/SM, 1.25 TFLOP/s nominal), not by HBM"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


def bench_torn(args):
    """Torn transients of 64 seeded 256 x 256 power grids (65,568 unknowns each,
    16 pieces of about 4,100 unknowns, 1,024 diode-clamped PULSE loads), 500
    backward-Euler steps of 0.1 ns; unit of work = one accepted time point of one
    variant.  One step = one ks_torn_tran of every variant."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kronspice_gb300 import analysis, build, workloads
    build.build()
    dev = torch.device("cuda", local)
    nsteps = args.tran_steps or POWER_STEPS
    el, nn, vals, torn, circ = workloads.power_grid_batch(args.n_circ, args.seed + rank, **POWER_GRID)
    V = vals.shape[0]
    t0 = time.perf_counter()
    tb = analysis.TornBatch(el, nn, vals, torn)
    create_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(dev)
    tb.set_stream(ctypes.c_void_p(stream.cuda_stream))
    spec = analysis.TranSpec(step=POWER_H, stop=nsteps * POWER_H, fixed_step=True, method="be")
    names = [e.name for e in circ.elements]
    grid_nodes = [circ.node_index("g%d_%d" % (r, c)) - 1 for r in (0, 128, 255) for c in (0, 128, 255)]
    opt = analysis.Options(reltol=RELTOL, precision=args.precision)  # chosen: FP32 factors (mixed) by default
    opt64 = analysis.Options(reltol=RELTOL, precision="fp64")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(reuse, steps_timed, spec_, opt=opt):
        for _ in range(args.warmup):
            tb.tran(spec_, opt, reuse=reuse, probes=grid_nodes)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        tot, pts = 0.0, 0
        for _ in range(steps_timed):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            wave, x, st, steps, it, stats = tb.tran(spec_, opt, reuse=reuse, probes=grid_nodes)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1) / 1e3
            pts += int(steps[st == 0].sum())
        if world > 1:  # every rank's variants, the slowest rank's time
            t = torch.tensor([tot, float(pts)], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t[:1], op=torch.distributed.ReduceOp.MAX)
            torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
            tot, pts = float(t[0].item()), int(t[1].item())
        return {"seconds": tot, "points": pts, "stats": stats, "status": st, "iters": it, "wave": wave}

    clk = Clocks(os.path.join(tempfile.gettempdir(),
                              "bench_clocks_%d.csv" % rank))
    with clk:
        chosen = timed(True, args.steps, spec)
        plain_steps = max(2, nsteps // 50)
        plain_spec = analysis.TranSpec(step=POWER_H, stop=plain_steps * POWER_H, fixed_step=True, method="be")
        plain = timed(False, 1, plain_spec, opt64)
        reuse64 = timed(True, 1, spec, opt64) if args.variants else None  # FP64 factors kept (no FP32 copies)
    clocks = clk.summary(local)
    value = chosen["points"] / chosen["seconds"]
    plain_value = plain["points"] / plain["seconds"]

    # end to end: the torn batch made from the host values (symbolic plan, upload, per-variant setup) and the
    # transient's probe waveforms back on the host, both inside the timed region
    e2e_t, e2e_pts = 0.0, 0
    for _ in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tb2 = analysis.TornBatch(el, nn, vals, torn)
        wave, x, st, steps, it, stats = tb2.tran(spec, opt, reuse=True, probes=grid_nodes)
        del tb2
        torch.cuda.synchronize()
        e2e_t += time.perf_counter() - t0
        e2e_pts += int(steps[st == 0].sum())
    if world > 1:
        t = torch.tensor([e2e_t, float(e2e_pts)], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t[:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
        e2e_t, e2e_pts = float(t[0].item()), int(t[1].item())
    e2e_value = e2e_pts / e2e_t
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    # accuracy: the first few steps of variant 0 against the oracle's untorn transient
    from oracle import oracle as orc
    orc.build()
    chk = 3
    ospec = orc.TranSpec(POWER_H, chk * POWER_H, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    r = orc.tran(orc.Packed(el, nn, vals[0]), ospec, orc.options(reltol=RELTOL), capacity=chk + 1, currents=False)
    max_err = float(np.abs(chosen["wave"][:chk + 1, 0, :] - r[2][:, grid_nodes]).max()) if r[0] == 0 else None
    cval, cruns, cwall, nthreads = oracle_grid_points(el, nn, vals, 2, min_wall=5.0)
    cpu = {"value": cval, "unit": TRAN_UNIT, "cores": nthreads, "kind": "port",
           "sample": "%d runs of 2 backward-Euler steps of one variant (operating point included, which the rate "
                     "counts against: an upper bound on the oracle's speed per step is not claimed) with the oracle's "
                     "untorn sparse LU, one run per host thread (%.1f s wall)" % (cruns, cwall)}

    st = chosen["stats"]
    n, P, R = tb.n, tb.pieces, tb.coupling_rows
    # algorithmic bytes of one transient: every application of the torn factors streams the band factors of all
    # pieces twice (z = B^-1 b, then x = B^-1 (b - P w)) and the interconnection factors once
    applies = st["solves"] + st["refines"]
    fw = 4 if args.precision == "mixed" else 8  # bytes per factor entry streamed
    per_apply = V * (2 * st["band_doubles"] * fw + R * R * fw)
    per_run_s = chosen["seconds"] / args.steps
    achieved = applies * per_apply / per_run_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": METRIC, "value": value, "unit": TRAN_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": chosen["seconds"] / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 loads and residuals, f32 factors" if args.precision == "mixed" else "f64", "data": "synthetic (seeded Philox)",
        "config": {"workload": "power_grid_tran_%d" % V, "variants": V, "grid": "256x256", "unknowns": n,
                   "pieces": P, "coupling_rows": R, "largest_piece": tb.max_piece, "band": tb.max_band,
                   "steps_per_variant": nsteps, "method": "be", "step_s": POWER_H, "reltol": RELTOL,
                   "l2": "flushed before each timed transient (512 MB write); factors exceed L2"},
        "chosen": {"value": value, "reuse": True, "factors": "fp32 copies streamed, fp64 refinement" if
                   args.precision == "mixed" else "fp64", "stats": st},
        "plain": {"value": plain_value, "reuse": False, "factors": "fp64", "steps_timed": plain_steps,
                  "stats": plain["stats"]},
        "variants": None if reuse64 is None else {
            "reuse/fp64": {"points_per_s": reuse64["points"] / reuse64["seconds"], "stats": reuse64["stats"]}},
        "chosen_vs_plain": value / plain_value if plain_value else None,
        "create_s": create_s,
        "max_node_voltage_err_vs_oracle": max_err,
        "e2e": {"value": e2e_value, "unit": TRAN_UNIT, "h2d_bytes_per_step": int(vals.nbytes),
                "d2h_bytes_per_step": int((nsteps + 1) * V * len(grid_nodes) * 8 + V * n * 8)},
        "gpu_launches": int(st["launches"]) * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "k_tl_band_solve + k_tl_ic_solve (factor streaming)",
                     "algorithmic_bytes_per_apply": per_apply, "applies_per_run": applies,
                     "note": "achieved = factor bytes streamed by every application of the torn factors over the "
                             "whole transient's event time (refactors, loads and convergence tests included)"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


def op_workload(args, name, B, steps, warmup, with_variants, cache, dev, stream, world, rank):
    """One operating-point workload: plain (generic kernel, FP64, InitJct) against
    chosen (per-topology kernel where the system fits in registers, FP32 LU + FP64
    residual, learned start refined by the FP32 Newton stage, the learned start's
    basin check), each step one batched operating point of all B circuits, L2
    flushed between steps, CUDA events on the launching stream.  Returns the
    numbers of both paths, the variants, the end-to-end rate through the C ABI
    with host buffers, the one-time costs and the parity against the oracle."""
    import torch
    from kronspice_gb300 import analysis, learned_start
    el, nn, vals = generator(name)(B, args.seed + rank)
    plan = analysis.Plan(el, nn, vals.shape[1])
    batch = analysis.Batch(plan, vals)
    n = plan.n
    sh = ctypes.c_void_p(stream.cuda_stream)
    x_dev = torch.empty((B, n), dtype=torch.float64, device=dev)
    st_dev = torch.empty(B, dtype=torch.int32, device=dev)
    it_dev = torch.empty(B, dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    learned = learned_start.for_workload(name, el, nn, vals, batch, dev, cache=cache)

    def step(opt, x0_dev=None):
        batch.op_async(opt, None if x0_dev is None else x0_dev.data_ptr(), x_dev.data_ptr(), st_dev.data_ptr(),
                       it_dev.data_ptr(), sh)

    def timed(opt, with_start, k=steps):
        launches = 1 + (learned.launches_per_step if with_start else 0)
        for _ in range(warmup):
            step(opt, learned.predict(stream) if with_start else None)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        times = []
        for _ in range(k):
            flush.fill_(1.0)
            e0, em, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            x0 = learned.predict(stream) if with_start else None
            em.record(stream)
            step(opt, x0)
            e1.record(stream)
            times.append((e0, em, e1))
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(c) for a, b, c in times) / 1e3
        op_s = sum(b.elapsed_time(c) for a, b, c in times) / 1e3 / k
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        st = st_dev.cpu().numpy()
        it = it_dev.cpu().numpy()
        return {"seconds": total, "ms_per_step": total / k * 1e3, "ok": int((st == 0).sum()), "op_kernel_s": op_s,
                "iters_mean": float(it.mean()), "iters_max": int(it.max()), "launches": launches * k,
                "x": x_dev.cpu().numpy(), "status": st, "steps": k}

    def rate(r):
        return world * r["ok"] * r["steps"] / r["seconds"] if r["seconds"] > 0 else 0.0

    spec_info = {"kernel": None}
    if n <= 6:  # systems that fit in registers get the per-topology kernel
        try:
            kname, csec = plan.specialize("op")
            spec_info = {"kernel": kname, "nvrtc_s": csec}
        except RuntimeError as e:
            spec_info = {"kernel": None, "error": str(e)[:200]}
    spec_ok = spec_info["kernel"] is not None
    kern = "specialized" if spec_ok else "generic"
    s32 = FP32_START.get(name, 200) if args.fp32_start < 0 else args.fp32_start
    plain_opt = analysis.Options(reltol=RELTOL, precision="fp64", kernel="generic")
    chosen_opt = analysis.Options(reltol=RELTOL, precision=args.precision, kernel=kern, fp32_start_iters=s32,
                                  start_check=learned.start_check)
    clk = Clocks(os.path.join(tempfile.gettempdir(), "bench_clocks_%s_%d.csv" % (name, rank)))
    variants = {}
    with clk:
        plain = timed(plain_opt, False)
        chosen = timed(chosen_opt, True)
        if with_variants:  # each ingredient of the chosen path alone and combined
            kerns = ["generic", "specialized"] if spec_ok else ["generic"]
            precs = ("fp64", "mixed") if name == "bjt_ce" else ("mixed",)
            for kn in kerns:
                for prec in precs:
                    for ws in (False, True):
                        for st32 in (0, s32):
                            o = analysis.Options(reltol=RELTOL, precision=prec, kernel=kn, fp32_start_iters=st32,
                                                 start_check=learned.start_check if ws else 0.0)
                            r = timed(o, ws)
                            variants["%s/%s/%s%s" % (kn, prec, "learned" if ws else "InitJct",
                                                     "+fp32stage" if st32 else "")] = {
                                "ms_per_step": r["ms_per_step"], "solves_per_s": rate(r),
                                "newton_iters_mean": r["iters_mean"], "newton_iters_max": r["iters_max"]}
    clocks = clk.summary(dev.index)

    # end to end through the C ABI: pinned host values in, host solutions out
    vals_pin = torch.from_numpy(vals.copy()).pin_memory()
    x_host = torch.empty((B, n), dtype=torch.float64).pin_memory()
    s_host = torch.empty(B, dtype=torch.int32).pin_memory()
    i_host = torch.empty(B, dtype=torch.int32).pin_memory()
    L = __import__("kronspice_gb300._lib", fromlist=["x"]).load()
    o = chosen_opt.c()

    def e2e_step():
        rc = L.ks_batch_set_values(batch.handle, ctypes.c_void_p(vals_pin.data_ptr()), 0, sh)
        assert rc == 0
        x0 = learned.predict(stream)
        rc = L.ks_op_async(batch.handle, ctypes.byref(o), ctypes.c_void_p(x0.data_ptr()), x_dev.data_ptr(),
                           st_dev.data_ptr(), it_dev.data_ptr(), sh)
        assert rc == 0
        x_host.copy_(x_dev, non_blocking=True)
        s_host.copy_(st_dev, non_blocking=True)
        i_host.copy_(it_dev, non_blocking=True)
        stream.synchronize()
    for _ in range(warmup):
        e2e_step()
    torch.cuda.synchronize()
    e2e_t = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_t], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e = {"value": world * B * steps / e2e_t, "unit": UNIT, "h2d_bytes_per_step": int(vals.nbytes),
           "d2h_bytes_per_step": int(B * n * 8 + 2 * B * 4)}

    # parity of the chosen path against the CPU oracle: status and node voltages
    from oracle import oracle as orc
    samp = min(B if name == "bjt_ce" else 8192, B)
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals[:samp]), samp, orc.options(reltol=RELTOL))
    okm = (so == 0) & (chosen["status"][:samp] == 0)
    xc = chosen["x"][:samp]
    dv = np.abs(xc[okm, :nn - 1] - xo[okm, :nn - 1])
    tolv = 1e-6 + RELTOL * np.abs(xo[okm, :nn - 1])
    parity = {"circuits": int(samp), "status_equal": bool(np.array_equal(chosen["status"][:samp], so)),
              "max_node_voltage_err_v": float(dv.max()) if dv.size else None,
              "within_tolerance": bool(np.all(dv <= tolv)), "tolerance": "1e-6 V + 1e-6 |v| per node (reltol/vntol)"}
    parity["ok"] = parity["status_equal"] and parity["within_tolerance"]

    value, plain_value = rate(chosen), rate(plain)
    info = dict(learned.info)
    one_time = {"nvrtc_s": spec_info.get("nvrtc_s"), "train_solve_s": info.get("train_solve_s"),
                "train_s": info.get("train_s")}
    if info.get("loaded_from"):
        one_time["note"] = "network loaded from %s (trained in an earlier run)" % info["loaded_from"]
    total_once = sum(v for v in (one_time["train_solve_s"], one_time["train_s"], one_time["nvrtc_s"]) if v)
    saved = (plain["ms_per_step"] - chosen["ms_per_step"]) / 1e3
    one_time["total_s"] = total_once
    one_time["saved_per_batch_s"] = saved
    one_time["break_even_batches"] = total_once / saved if saved > 0 else None
    return {"name": name, "B": B, "n": n, "nn": nn, "el": el, "vals": vals, "plain": plain, "chosen": chosen,
            "value": value, "plain_value": plain_value, "variants": variants, "e2e": e2e, "parity": parity,
            "spec_info": spec_info, "learned": info, "one_time": one_time, "clocks": clocks,
            "chosen_opt": chosen_opt, "s32": s32, "steps": steps}


def main():
    args = parse()
    if args.n_circ <= 0:
        args.n_circ = WORKLOADS[args.workload][0]
    if args.steps <= 0:
        args.steps = DEFAULT_STEPS[args.workload]
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "rc_ladder":
        bench_tran(args)
        return
    if args.workload == "random_netlists":
        bench_multi(args)
        return
    if args.workload == "bjt_ce_ac":
        bench_ac(args)
        return
    if args.workload == "power_grid":
        bench_torn(args)
        return
    if args.workload == "evo_lowpass":
        bench_evo(args)
        return
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kronspice_gb300 import build, _lib
    build.build()
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)  # a real stream: kernels and events on the same one
    torch.cuda.set_stream(stream)
    r = op_workload(args, args.workload, args.n_circ, args.steps, args.warmup, bool(args.variants), args.start_cache,
                    dev, stream, world, rank)
    second = None
    if args.workload == "bjt_ce" and args.secondary:
        cache2 = None
        if args.start_cache:
            base, ext = os.path.splitext(args.start_cache)
            cache2 = base + "_cmos_opamp" + (ext or ".npz")
        second = op_workload(args, "cmos_opamp", WORKLOADS["cmos_opamp"][0], DEFAULT_STEPS["cmos_opamp"],
                             min(args.warmup, 3), True, cache2, dev, stream, world, rank)
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    B, n, chosen = r["B"], r["n"], r["chosen"]
    cpu = cpu_baseline(r["el"], r["nn"], r["vals"])
    per_launch_s = chosen["op_kernel_s"]  # the operating-point kernel alone (events around its launch)
    kname = "ks_spec_op" if r["chosen_opt"].kernel == "specialized" else "k_op"
    # algorithmic bytes of one solve: its value vector in, its solution, status and iteration count out
    nv = r["vals"].shape[1]
    alg_bytes = (nv + n) * 8 + 8
    achieved = alg_bytes * B / per_launch_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    prof = traffic_from_profile().get("%s_%s" % (kname, args.workload), {})
    traffic = prof.get("dram_bytes_per_circuit")
    # FP64 roofline: the kernel's FP64 operations per circuit (ncu instruction
    # counts of the same launch) over its event time, against this device's FP64
    # FMA rate measured now
    fp64_peak, fma_clk = ctypes.c_double(), ctypes.c_double()
    L = _lib.load()
    fp64 = None
    if L.ks_fp64_peak(ctypes.byref(fp64_peak), ctypes.byref(fma_clk)) == 0:
        flops_c = prof.get("fp64_flops_per_circuit")
        fp64 = {"bound": "fp64", "peak": fp64_peak.value / 1e12, "unit": "TFLOP/s",
                "peak_fma_lanes_per_clk_per_sm": fma_clk.value,
                "peak_source": "ks_fp64_peak: FMA chains on every SM of this device, measured in this run",
                "achieved": None if flops_c is None else flops_c * B / per_launch_s / 1e12,
                "flops_per_circuit": flops_c, "kernel": kname,
                "lanes_per_fp64_instruction": prof.get("fp64_lanes_per_instruction"),
                "source": prof.get("source")}
        if fp64["achieved"] is not None:
            fp64["frac"] = fp64["achieved"] / fp64["peak"]
    plain = r["plain"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": chosen["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 device eval + residual, f32 LU" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded Philox)",
        "config": {"workload": "%s_op_%d" % (args.workload, B), "n_circuits_per_gpu": B, "n_unknowns": n,
                   "reltol": RELTOL, "abstol": 1e-12, "l2": "flushed between timed steps (512 MB write)",
                   "learned_start": True, "fp32_start_iters": r["s32"]},
        "plain": {"value": r["plain_value"], "ms_per_step": plain["ms_per_step"],
                  "newton_iters_mean": plain["iters_mean"], "newton_iters_max": plain["iters_max"],
                  "precision": "fp64", "kernel": "generic", "start": "InitJct"},
        "chosen": {"value": r["value"], "ms_per_step": chosen["ms_per_step"],
                   "newton_iters_mean": chosen["iters_mean"], "newton_iters_max": chosen["iters_max"],
                   "newton_iters_note": "FP64 Newton solves per circuit (the FP32 stage's iterations not counted)",
                   "precision": "fp32 LU + fp64 residual" if args.precision == "mixed" else "fp64",
                   "kernel": r["chosen_opt"].kernel,
                   "start": "learned (MLP) refined by the FP32 Newton stage; basin check at %.3g V"
                            % r["chosen_opt"].start_check},
        "per_topology_kernel": r["spec_info"],
        "variants": r["variants"] or None,
        "chosen_vs_plain": r["value"] / r["plain_value"] if r["plain_value"] else None,
        "learned_start": r["learned"],
        "one_time_costs": r["one_time"],
        "parity_vs_oracle": r["parity"],
        "max_node_voltage_err_vs_oracle": r["parity"]["max_node_voltage_err_v"],
        "e2e": r["e2e"],
        "gpu_launches": chosen["launches"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None if traffic is None else traffic * B, "kernel": kname,
                     "algorithmic_bytes_per_solve": alg_bytes, "kernel_ms": per_launch_s * 1e3,
                     "note": "the operating-point kernel is bound by FP64 issue, not by HBM: achieved counts the "
                             "value vector in and the solution out per solve over the launch's event time, peak "
                             "is the measured copy bandwidth; roofline_fp64 gives the FP64 fraction"},
        "roofline_fp64": fp64,
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
    }
    if second is not None:
        s2 = second
        line["cmos_opamp"] = {
            "config": {"workload": "cmos_opamp_op_%d" % s2["B"], "n_unknowns": s2["n"], "steps": s2["steps"],
                       "fp32_start_iters": s2["s32"]},
            "plain": {"value": s2["plain_value"], "ms_per_step": s2["plain"]["ms_per_step"],
                      "newton_iters_mean": s2["plain"]["iters_mean"], "newton_iters_max": s2["plain"]["iters_max"]},
            "chosen": {"value": s2["value"], "ms_per_step": s2["chosen"]["ms_per_step"],
                       "newton_iters_mean": s2["chosen"]["iters_mean"], "newton_iters_max": s2["chosen"]["iters_max"],
                       "kernel": s2["chosen_opt"].kernel},
            "chosen_vs_plain": s2["value"] / s2["plain_value"] if s2["plain_value"] else None,
            "variants": s2["variants"], "learned_start": s2["learned"], "one_time_costs": s2["one_time"],
            "parity_vs_oracle": s2["parity"], "e2e": s2["e2e"], "clocks": s2["clocks"]}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()
    # a chosen path whose results leave the oracle's tolerance is not a result
    if not r["parity"]["ok"] or (second is not None and not second["parity"]["ok"]):
        sys.stderr.write("bench: chosen path fails parity against the oracle\n")
        sys.exit(3)


if __name__ == "__main__":
    main()
