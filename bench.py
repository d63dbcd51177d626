"""Benchmark: segment x group x polar integrations per second of MOC source
iteration on the 17 x 17 pin lattice, 70 groups, 64 azimuthal angles,
0.05 cm spacing, 3 polar angles per half space (TY-6), reflective.

A step is one full source iteration (FSR sources, transport sweep, add
source, keff + normalisation, residual) over the whole problem, inputs
resident in HBM; integrations per step = 2 * F * S (F = G * polar/2), the
count OpenMOC uses in its timer report (src/Solver.cpp:1901).  L2 is flushed
(a 2 x L2 buffer is overwritten) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times OpenMOC's CPU path on the host cores with every host
thread, on the same problem: OpenMOC's own CPUSolver (oracle/openmoc_run.cpp
linked against OpenMOC's library, timed by its own Timer splits) where that
build exists on the host, else the C restatement in oracle/moc_oracle.c.  It
never loads the GPU library: its tracks come from a host-only build of the
track generator (oracle/_build/libmoc_tracks.so).
"""
from __future__ import annotations

import argparse
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

WORKLOAD = "17x17 pin lattice, 70 groups, 64 azimuthal, 0.05 cm, TY-6 (3 polar), reflective"
METRIC = "segment*group*polar integrations/s"
FLOPS_PER_INTEGRATION = 30     # FP32 flops of one 2D integration (FMA = 2)
FLOPS_PER_INTEGRATION_3D = 28  # 3D: no 1/sin(theta) scaling
# linear source (2D): the rational G(x) (11 FMA, a reciprocal, a multiply),
# F1/F2/H from it, the flat and linear source terms, the update and the
# scalar-flux and x/y moment tallies, per (segment, group, polar)
FLOPS_PER_LS_INTEGRATION = 48
# linear source on explicit 3D tracks, per (segment, group): the same
# attenuation (44) with no polar angles to share the per-segment terms
# (optical length, flat and linear source with z, 12) and x / y / z moment
# tallies (11) -- counted from the 3D sweep instances
FLOPS_PER_LS_INTEGRATION_3D = 68
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one sweep launch
# of this workload, from one ncu capture per sweep shape (lanes per track
# direction, group pairs per lane, exponential kind); the summaries are under
# profiles/ (sweep_kernel_17x17_70g.txt).
SWEEP_DRAM_BYTES = {(8, 5, 1): 50_877_440 + 1_314_560}


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(x, dist, device):
    """The largest value of x over the ranks (x itself without a process
    group)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, steps, world, slowest_ms):
    """Units of all `world` replicas per second of the slowest one."""
    return world * units_per_step * steps / (slowest_ms * 1e-3)


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def algorithmic_bytes(p, ls=False, otf=False):
    """Compulsory HBM bytes of one sweep: packed segments read once (8 B;
    16 B with the linear source's start position, 20 B with its z on 3D
    tracks), per-track offsets/links/flags (16 B), angular flux in and out
    for both directions (16 B per track and flux value), sources read and
    tallies written (8 B per FSR and group; 24 B with the x / y source and
    flux moments, 32 B with z)."""
    F = p.fluxes_per_track
    ls3d = ls and bool(p.solve_3d)
    if otf:
        # a 32-byte description per 3D track and the radial segments (12 B)
        # instead of the stored 3D segments
        seg = 32 * p.num_tracks + 12 * p.otf["rad_len"].size
    else:
        seg = (20 if ls3d else 16 if ls else 8) * p.num_segments
    return (seg + 16 * p.num_tracks + 16 * p.num_tracks * F
            + (32 if ls3d else 24 if ls else 8) * p.num_fsrs * p.num_groups)


class Clocks:
    """nvidia-smi clock / throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="moc_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            if os.path.exists(self.path):
                os.remove(self.path)
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


# The headline workload and the other single-solve configurations
# (--workload): description, builder.
WORKLOADS = {
    "assembly70": WORKLOAD,
    "core51": "51x51 pins (3x3 assemblies), 7 groups, 3 fuel sets in a checkerboard, "
              "128 azimuthal, 0.03 cm, TY-6, vacuum on +x/+y, reflective on -x/-y",
    "assembly3d": "17x17 assembly extruded to 20 cm (fuel below 16 cm, moderator above), "
                  "7 groups, explicit 3D tracks: 16 azimuthal, 6 polar, 0.1 cm radial, "
                  "0.5 cm axial; reflective radially, vacuum top and bottom",
    "assembly70_ls": WORKLOAD + ", linear source (CPULSSolver)",
    "assembly3d_ls": "17x17 assembly extruded to 20 cm (fuel below 16 cm, moderator above), "
                     "7 groups, explicit 3D tracks: 16 azimuthal, 6 polar, 0.1 cm radial, "
                     "0.5 cm axial; linear source (CPULSSolver, x / y / z moments)",
    "assembly3d_otf": "17x17 assembly extruded to 20 cm (fuel below 16 cm, moderator above), "
                      "7 groups, 16 azimuthal, 6 polar, 0.1 cm radial, 0.5 cm axial; 3D "
                      "tracks cut from the radial segments during the sweep (on-the-fly)",
}


def is_ls(workload):
    return workload.endswith("_ls")


def build_problem(workload="assembly70"):
    from openmoc_gb300 import lattice
    if workload == "core51":
        return lattice.core_51x51()
    if workload in ("assembly3d", "assembly3d_otf"):
        return lattice.assembly_17x17_3d()
    if workload == "assembly70_ls":
        return lattice.assembly_17x17(linear_source=True)
    if workload == "assembly3d_ls":
        return lattice.assembly_17x17_3d(linear_source=True)
    return lattice.assembly_17x17()


# Workloads OpenMOC's own driver (oracle/openmoc_run.cpp) can build
OPENMOC_CONFIGS = {"assembly70": "assembly70", "core51": "core51"}
OPENMOC_RUNNER = os.path.join(ROOT, "oracle", "_ref", "openmoc_run_f32")
ORACLE_TRACKS = os.path.join(ROOT, "oracle", "_build", "libmoc_tracks.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def bench_config(p, workload, world):
    """The workload description both arms report (the same keys and values,
    so the two lines compare like for like)."""
    return {"workload": WORKLOADS[workload], "fsrs": p.num_fsrs, "tracks": p.num_tracks,
            "segments": p.num_segments, "groups": p.num_groups,
            "integrations_per_step": p.integrations_per_sweep,
            "l2": "GPU: a 2 x L2 buffer is overwritten before every timed step",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def openmoc_rate(workload, warmup, iters, threads):
    """OpenMOC's own CPUSolver on the workload (FP32 build, OpenMP over
    `threads`), timed by its Timer splits: integrations per second of whole
    source iterations ("Total time" less "Solver initialization") and of the
    "Transport Sweep" split alone.  None where the OpenMOC build is absent
    or does not run on this host."""
    if workload not in OPENMOC_CONFIGS or not os.access(OPENMOC_RUNNER, os.X_OK):
        return None
    try:
        r = subprocess.run([OPENMOC_RUNNER, OPENMOC_CONFIGS[workload], "time",
                            str(warmup), str(iters), str(threads)],
                           capture_output=True, text=True, timeout=1800)
    except OSError:
        return None
    if r.returncode != 0:
        return None
    d = json.loads(r.stdout.strip().splitlines()[-1])
    iter_s = d["total_s"] - d["init_s"]
    d["value"] = d["integrations_per_iteration"] * d["iterations"] / iter_s
    d["sweep_value"] = d["integrations_per_iteration"] * d["iterations"] / d["transport_sweep_s"]
    d["seconds_per_iteration"] = iter_s / d["iterations"]
    return d


def cpu_reference_rate(p, iters, threads):
    """Integrations/s of the oracle's source iteration on the host cores
    (CPULSSolver's when the problem carries a linear source)."""
    from oracle.oracle import LSOracle, Oracle
    if p.linear_source is not None:
        o = LSOracle(p, p.linear_source, "f32", num_threads=threads)
        o.constants()
    else:
        o = Oracle(p, "f32", num_threads=threads)
    o.keff = 1.0
    o.phi[:] = 1.0
    o.normalize()
    o.store()
    t0 = time.perf_counter()
    for i in range(iters):
        o.compute_sources(i)
        o.sweep()
        o.add_source()
        o.compute_keff()
        o.normalize()
        o.residual_of(1)
        o.store()
    dt = time.perf_counter() - t0
    return p.integrations_per_sweep * iters / dt, dt


def cpu_baseline(p, workload, iters):
    """The CPU baseline beside the GPU number: OpenMOC's CPUSolver where it
    was built on this host, else the oracle port; every host thread."""
    threads = os.cpu_count() or 1
    d = openmoc_rate(workload, 1, iters, threads)
    if d is not None:
        return {"value": d["value"], "unit": "integrations/s", "cores": threads,
                "kind": "reference",
                "sample": f"{iters} source iterations of OpenMOC's CPUSolver (FP32) on "
                          f"the workload after 1 warm-up iteration, Timer splits; "
                          f"transport sweep alone {d['sweep_value']:.4g}/s"}
    r, dt = cpu_reference_rate(p, iters, threads)
    return {"value": r, "unit": "integrations/s", "cores": threads, "kind": "port",
            "sample": f"{iters} full source iterations of the workload "
                      f"({dt:.1f} s, oracle/moc_oracle.c, OpenMP, FP32; OpenMOC's "
                      "own build is absent on this host)"}


def accuracy(p, workload, keff, flux, iters):
    """Errors of a GPU result after `iters` source iterations from the flat
    guess: against OpenMOC's FP64 CPUSolver at the same iteration count
    (tests/golden/openmoc_<config>_f64.json: its 4096-flux sample and group
    sums) and against the FP64 oracle's full flux."""
    from oracle.oracle import FISSION_SOURCE, Oracle
    out = {"iterations": iters}
    flux = np.asarray(flux, np.float64).ravel()
    path = os.path.join(GOLDEN, f"openmoc_{OPENMOC_CONFIGS.get(workload, '-')}_f64.json")
    if os.path.exists(path):
        with open(path) as f:
            g = json.load(f)
        if int(g["iterations"]) == iters:
            idx = np.asarray(g["flux_sample_index"], np.int64)
            ref = np.asarray(g["flux_sample"], np.float64)
            sums = flux.reshape(-1, p.num_groups).sum(axis=0)
            rs = np.asarray(g["group_flux_sums"], np.float64)
            out["vs_openmoc_fp64"] = {
                "keff_abs_err": abs(keff - g["keff"]),
                "flux_max_rel_err": float(np.max(np.abs(flux[idx] - ref) / np.abs(ref))),
                "group_sum_max_rel_err": float(np.max(np.abs(sums - rs) / np.abs(rs))),
                "fluxes_compared": int(idx.size) + p.num_groups}
    o = Oracle(p, "f64", num_threads=os.cpu_count() or 1)
    t0 = time.perf_counter()
    o.compute_eigenvalue(iters, FISSION_SOURCE, 1e-30)
    out["vs_fp64_oracle"] = {
        "keff_abs_err": abs(keff - o.keff),
        "flux_max_rel_err": float(np.max(np.abs(flux - o.phi) / np.abs(o.phi))),
        "fluxes_compared": int(flux.size), "oracle_s": time.perf_counter() - t0}
    out["bar"] = {"keff_abs": 1e-5, "flux_rel": 1e-4}
    return out


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    from openmoc_gb300 import lattice
    if not os.path.exists(ORACLE_TRACKS):
        subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build.sh")])
    lattice.use_host_library(ORACLE_TRACKS)
    p = build_problem(args.workload)
    threads = os.cpu_count() or 1
    t_all = time.perf_counter()
    d = openmoc_rate(args.workload, args.warmup, args.steps, threads)
    if d is not None:
        assert (d["fsrs"], d["tracks"], d["segments"]) == (
            p.num_fsrs, p.num_tracks, p.num_segments), "OpenMOC built a different problem"
        value = d["value"]
        ms_per_step = 1e3 * d["seconds_per_iteration"]
        base = {"kind": "reference",
                "sample": f"{args.steps} source iterations of OpenMOC's CPUSolver (FP32 "
                          f"build) after {args.warmup} warm-up iterations, timed by its "
                          f"Timer splits; transport sweep alone {d['sweep_value']:.4g}/s"}
    else:
        rates = []
        for _ in range(args.warmup):
            cpu_reference_rate(p, 1, threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r, _ = cpu_reference_rate(p, 1, threads)
            rates.append(r)
        value = float(np.mean(rates))
        ms_per_step = 1e3 * (time.perf_counter() - t0) / args.steps
        base = {"kind": "port",
                "sample": f"{args.steps} full source iterations of the workload "
                          "(oracle/moc_oracle.c, OpenMP, FP32): OpenMOC's own build "
                          "does not exist on this host (no OpenMOC source tree here, "
                          "and builds made elsewhere do not run on this CPU)"}
    out = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "integrations/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded cross sections, generated tracks)",
        "config": bench_config(p, args.workload, world),
        "cpu_baseline": dict(value=value, unit="integrations/s", cores=threads, **base),
        "e2e": {"value": value, "unit": "integrations/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t_all,
    }
    print(json.dumps(out), flush=True)


def run_gpu(args):
    import torch
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from openmoc_gb300 import GB300LSSolver, GB300Solver
    from openmoc_gb300.solver import FISSION_SOURCE

    p = build_problem(args.workload)
    ls = is_ls(args.workload)
    otf = args.workload.endswith("_otf")
    peaks, peak_kind = load_peaks()
    s = (GB300LSSolver if ls else GB300Solver)(device=local)
    if args.workload.endswith("_otf"):
        s.setSegmentFormation("otf")
    s.setTrackGenerator(p)
    if args.shape:
        # a fixed kernel shape (e.g. to profile one instance)
        lps, slots, exp_kind = (int(v) for v in args.shape.split(","))
        s.setSweepShape(lps, slots)
        if not ls:
            (s.useExponentialIntrinsic if exp_kind else s.useExponentialInterpolation)()
        tuning = []
    else:
        lps, slots, exp_kind = s.autotune()
        tuning = s.getTuningLog()
    # warm-up (also JIT-free: the library is ahead-of-time sm_103a code)
    s.benchIterations(max(args.warmup, 3), FISSION_SOURCE, True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches_before = s.getLaunchCount()
    with Clocks(local) as clk:
        t_wall = time.perf_counter()
        step_ms, sweep_ms = s.benchIterations(args.steps, FISSION_SOURCE, True)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    gpu_launches = s.getLaunchCount() - launches_before
    # the source contraction both ways: 3xTF32 tensor cores (the default at
    # 70 groups) against the FP32 CUDA-core kernel, same iterations
    sources = {"kernel": ("linear source: flat + x/y moments, FP32 CUDA cores" if ls
                          else s.getSourceContraction())}
    kinds = ("fp32", "tf32x3") if 64 <= p.num_groups <= 96 and not ls else ()
    for kind in kinds:
        s.setSourceContraction(kind)
        st, sw = s.benchIterations(max(args.steps // 2, 5), FISSION_SOURCE, True)
        sources[f"{kind}_ms_per_step"] = float(np.mean(st))
        sources[f"{kind}_non_sweep_ms"] = float(np.mean(np.asarray(st) - np.asarray(sw)))
    s.setSourceContraction("auto")
    clocks = clk.summary()
    # replicas: the slowest rank's time, every rank's integrations
    total_ms = max_over_ranks(float(np.sum(step_ms)), dist, "cuda")
    if dist:
        dist.barrier()
    ms_per_step = total_ms / args.steps
    ints = p.integrations_per_sweep
    value = whole_job_rate(ints, args.steps, world, total_ms)

    # roofline of the dominant kernel (the sweep)
    sweep_avg = float(np.mean(sweep_ms))
    nbytes = algorithmic_bytes(p, ls, otf)
    achieved = nbytes / (sweep_avg * 1e-3) / 1e9
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = (SWEEP_DRAM_BYTES.get((lps, slots, exp_kind))
               if args.workload == "assembly70" else None)
    sm_mhz = clocks.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    flops_per_int = ((FLOPS_PER_LS_INTEGRATION_3D if p.solve_3d else
                      FLOPS_PER_LS_INTEGRATION) if ls else
                     FLOPS_PER_INTEGRATION_3D if p.solve_3d else FLOPS_PER_INTEGRATION)
    fp32_achieved = ints * flops_per_int / (sweep_avg * 1e-3) / 1e12

    # end to end through the public API: host buffers (pinned), upload,
    # 20 iterations, fluxes back
    e2e = None
    if args.e2e_iters > 0:
        e2e = end_to_end(p, args, local, torch, otf=args.workload.endswith("_otf"))

    cpu = None
    acc = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(p, args.workload, args.cpu_iters)
        # the error of the end-to-end result against the FP64 references
        if e2e is not None and not ls and not args.no_accuracy:
            acc = accuracy(p, args.workload, e2e.pop("keff"), e2e.pop("flux"),
                           args.e2e_iters)
    if e2e is not None:
        e2e.pop("keff", None)
        e2e.pop("flux", None)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "integrations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded cross sections, generated tracks)",
            "config": bench_config(p, args.workload, world),
            "sweep_shape": {"lanes_per_track_direction": lps,
                            "group_pairs_per_lane": slots,
                            "exponential": ("rational G(x), F1/F2/H from it"
                                            if ls else "hardware ex2" if otf
                                            else ["shared-memory table",
                                                  "hardware ex2"][exp_kind])},
            "autotune_ms": {f"{a}x{b}/{'table' if e == 0 else 'ex2'}": round(t, 4)
                            for a, b, e, t in tuning},
            "sweep_ms_per_step": sweep_avg,
            "sources": sources,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": nbytes,
                         "binding": {"bound": "fp32", "achieved": fp32_achieved,
                                     "peak": fp32_peak, "unit": "TFLOP/s",
                                     "frac": fp32_achieved / fp32_peak,
                                     "flops_per_integration": flops_per_int}},
            "clocks": clocks,
            "gpu_launches": gpu_launches,
            "wall_s": t_wall,
        }
        if e2e:
            out["e2e"] = e2e
        if cpu:
            out["cpu_baseline"] = cpu
        if acc:
            out["accuracy"] = acc
        if args.batch > 0:
            out["batched_instances"] = run_instances(p, args)
        core = None
        if world == 1 and args.workload == "assembly70" and not args.no_raytrace:
            out["ray_tracing"], core = ray_tracing(local)
        if world == 1 and args.workload == "assembly70" and not args.no_configs:
            # the other single-solve configurations, measured in the same run
            from openmoc_gb300 import lattice as lat
            if core is None:
                core = lat.core_51x51(device=local)
            out["configs"] = {
                "core51": single_config(core, WORKLOADS["core51"], local),
                "assembly3d": single_config(lat.assembly_17x17_3d(),
                                            WORKLOADS["assembly3d"], local),
                "assembly70_ls": single_config(
                    lat.assembly_17x17(linear_source=True),
                    WORKLOADS["assembly70_ls"], local),
                "assembly3d_ls": single_config(
                    lat.assembly_17x17_3d(linear_source=True),
                    WORKLOADS["assembly3d_ls"], local)}
        if world == 1 and args.workload == "assembly70" and not args.no_cmfd:
            # the regime CMFD is for: a core whose sweeps are expensive and
            # whose plain source iteration needs a thousand iterations
            from openmoc_gb300 import lattice as lat
            if core is None:
                core = lat.core_51x51(device=local)
            out["cmfd"] = cmfd_acceleration(core, local, label="51x51 core, 7 groups",
                                            groups=[[1, 2, 3], [4, 5, 6, 7]])
            # and the assembly whose sweeps are cheap (8 coarse groups)
            out["cmfd_assembly"] = cmfd_acceleration(p, local, coarse_groups=8,
                                                     label="17x17 assembly, 70 groups")
        if world == 1 and not args.no_serving and args.workload == "assembly70":
            # the second half of the headline: the request stream through the
            # batched server against the plain per-solve loop
            sv = run_serving(args)
            out["serving"] = {k: sv[k] for k in ("metric", "value", "unit", "config",
                                                 "batched", "plain", "speedup",
                                                 "ceiling", "by_class", "agreement")}
            if args.serving_ls_requests > 0:
                sv = run_serving(args, ls=True)
                out["serving_ls"] = {k: sv[k] for k in (
                    "metric", "value", "unit", "config", "batched", "plain", "speedup",
                    "ceiling", "by_class", "agreement")}
        print(json.dumps(out), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


def cmfd_acceleration(p, device, tol=1e-5, coarse_groups=8, label=None, groups=None):
    """Time to solution, computeEigenvalue to a 1e-5 fission-source
    residual, without and with CMFD (pin-cell mesh, the groups condensed to
    `coarse_groups` contiguous bands): iterations, wall seconds, and the
    coarse solve's power iterations and SOR sweeps; the CMFD solve with the
    coarse power iteration cell-parallel (the default) and on one block."""
    from openmoc_gb300 import Cmfd, GB300Solver
    G = p.num_groups
    bands = ([np.array(g) for g in groups] if groups is not None
             else np.array_split(np.arange(1, G + 1), coarse_groups))
    res = {"workload": (label or f"{p.meta.get('nx', 17)}x{p.meta.get('ny', 17)} pins, "
                                 f"{G} groups")
                       + f"; CMFD on the pin mesh with {len(bands)} coarse groups",
           "tolerance": tol}
    for name, use, kind in (("plain", False, None), ("cmfd", True, "auto"),
                            ("cmfd_one_block", True, "block")):
        s = GB300Solver(p, device=device)
        s.setConvergenceThreshold(tol)
        if use:
            c = Cmfd()
            c.setLatticeStructure(int(p.meta.get("nx", 17)), int(p.meta.get("ny", 17)))
            c.setGroupStructure([b.tolist() for b in bands])
            c.setDeviceSolver(kind)
            s.setCmfd(c)
        s.computeEigenvalue(5, 1)                 # tuning and module load
        t0 = time.perf_counter()
        s.computeEigenvalue(5000, 1)
        dt = time.perf_counter() - t0
        res[name] = {"iterations": s.getNumIterations(), "seconds": dt,
                     "ms_per_iteration": 1e3 * dt / max(1, s.getNumIterations()),
                     "keff": s.getKeff()}
        if use:
            info = s.getCmfdInfo()
            res[name]["coarse_power_iterations_last"] = info["power_iterations"]
            res[name]["coarse_sor_sweeps_last"] = info["linear_iterations"]
        s.close()
    res["speedup"] = res["plain"]["seconds"] / res["cmfd"]["seconds"]
    res["speedup_one_block"] = res["plain"]["seconds"] / res["cmfd_one_block"]["seconds"]
    res["keff_difference"] = res["cmfd"]["keff"] - res["plain"]["keff"]
    return res


def cmfd_solve_only(workload="core", kind="auto", device=0):
    """One CMFD-accelerated solve alone (for profiling), to 1e-5: the 51x51
    core traced on the device (pin mesh, two coarse groups) or the 17x17
    70-group assembly (pin mesh, 8 coarse groups), with the coarse power
    iteration cell-parallel ("cells"), on one block ("block") or chosen
    ("auto"); after a 5-iteration warm-up solve."""
    from openmoc_gb300 import Cmfd, GB300Solver
    from openmoc_gb300 import lattice as lat
    if workload == "core":
        p, n = lat.core_51x51(device=device), 51
        bands = [[1, 2, 3], [4, 5, 6, 7]]
        label = "51x51 core, 7 groups; CMFD on the pin mesh with 2 coarse groups"
    else:
        p, n = lat.assembly_17x17(), 17
        bands = [b.tolist() for b in np.array_split(np.arange(1, 71), 8)]
        label = "17x17 assembly, 70 groups; CMFD on the pin mesh with 8 coarse groups"
    s = GB300Solver(p, device=device)
    s.setConvergenceThreshold(1e-5)
    c = Cmfd()
    c.setLatticeStructure(n, n)
    c.setGroupStructure(bands)
    c.setDeviceSolver(kind)
    s.setCmfd(c)
    s.computeEigenvalue(5, 1)
    t0 = time.perf_counter()
    s.computeEigenvalue(1000, 1)
    dt = time.perf_counter() - t0
    out = {"workload": label, "device_solver": kind,
           "iterations": s.getNumIterations(), "seconds": dt, "keff": s.getKeff(),
           "cmfd": s.getCmfdInfo()}
    s.close()
    return out


def single_config(p, label, device, steps=10):
    """One more benchmark configuration solved alone: the autotuned sweep
    shape and the device-timed source iteration (L2 flushed between
    iterations, as for the headline), integrations per second; with the
    linear source (CPULSSolver) when the problem carries its geometry."""
    from openmoc_gb300 import GB300LSSolver, GB300Solver
    from openmoc_gb300.solver import FISSION_SOURCE
    s = (GB300LSSolver if p.linear_source is not None else GB300Solver)(
        p, device=device)
    lps, slots, exp_kind = s.autotune()
    s.benchIterations(3, FISSION_SOURCE, True)
    st, sw = s.benchIterations(steps, FISSION_SOURCE, True)
    s.close()
    step = float(np.mean(st))
    return {"workload": label, "fsrs": int(p.num_fsrs), "tracks": int(p.num_tracks),
            "segments": int(p.num_segments), "groups": int(p.num_groups),
            "integrations_per_sweep": int(p.integrations_per_sweep),
            "sweep_shape": [int(lps), int(slots),
                            "rational G(x)" if p.linear_source is not None else
                            "ex2" if exp_kind else "table"],
            "ms_per_step": step, "sweep_ms_per_step": float(np.mean(sw)),
            "value": p.integrations_per_sweep / (step * 1e-3),
            "unit": "integrations/s", "steps": steps}


def ray_tracing(device):
    """Track generation of the 51x51 core on the host cores against the
    device ray tracer (laydown on the host, segmentation, FSR numbering and
    volumes on the GPU); both produce the same segments.  Returns the
    timings and the device-traced problem."""
    from openmoc_gb300 import lattice as lat
    lat.pin_cell(7, device=device)            # CUDA context and module load
    t0 = time.perf_counter()
    h = lat.core_51x51()
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    d = lat.core_51x51(device=device)
    t_dev = time.perf_counter() - t0
    same = all(np.array_equal(getattr(h, k), getattr(d, k)) for k in (
        "seg_len", "seg_fsr", "seg_off", "track_ang", "next", "flags", "fsr_mat"))
    return ({"workload": "51x51 pins, 128 azimuthal, 0.03 cm, TY-6: "
                         f"{d.num_tracks} tracks, {d.num_segments} segments",
             "host_s": t_host, "host_threads": os.cpu_count(), "device_s": t_dev,
             "segments_per_s_device": d.num_segments / t_dev,
             "speedup": t_host / t_dev, "identical_segments": bool(same)}, d)


def end_to_end(p, args, device, torch, otf=False):
    """The metric through GB300Solver: per step, upload the problem from
    pinned host memory, run a fixed number of iterations, copy the fluxes
    back."""
    from openmoc_gb300 import GB300LSSolver, GB300Solver, Problem
    pinned = {}
    h2d = 0
    for k in ("seg_len", "seg_fsr", "seg_off", "track_ang", "next", "flags", "weights",
              "inv_sin", "sigma_t", "sigma_s", "nu_sigma_f", "chi", "fsr_mat", "fsr_vol"):
        a = getattr(p, k)
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = a.view(np.uint8)
        pinned[k] = (t, t.numpy().view(a.dtype))
        h2d += a.nbytes
    q = Problem(**{f: getattr(p, f) for f in p.__dataclass_fields__})
    for k, (_, arr) in pinned.items():
        setattr(q, k, arr)
    if otf:
        q.otf = {}
        for k, a in p.otf.items():
            t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
            t.numpy()[:] = a.view(np.uint8)
            pinned["otf_" + k] = (t, t.numpy().view(a.dtype))
            q.otf[k] = pinned["otf_" + k][1]
            h2d += a.nbytes
    if p.linear_source is not None:
        q.linear_source = {}
        for k, a in p.linear_source.items():
            if k == "centroid":
                continue
            t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
            t.numpy()[:] = a.view(np.uint8)
            pinned["ls_" + k] = (t, t.numpy().view(a.dtype))
            q.linear_source[k] = pinned["ls_" + k][1]
            h2d += a.nbytes
    d2h = p.num_fsrs * p.num_groups * 4
    times = []
    setups = []
    for i in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = (GB300LSSolver if p.linear_source is not None else GB300Solver)(
            device=device)
        if otf:
            s.setSegmentFormation("otf")
        s.setTrackGenerator(q)
        setup = time.perf_counter() - t0
        s.setConvergenceThreshold(1e-30)
        s.computeEigenvalue(args.e2e_iters)
        flux = s.getFluxes()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        keff = s.getKeff()
        s.close()
        if i > 0:
            times.append(dt)
            setups.append(setup)
        assert np.isfinite(flux).all()
    t = float(np.mean(times))
    return {"value": p.integrations_per_sweep * args.e2e_iters / t, "unit": "integrations/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "iterations_per_step": args.e2e_iters, "seconds_per_step": t,
            "setup_seconds_per_step": float(np.mean(setups)),
            "keff": keff, "flux": flux}


def run_instances(p, args, iters=10):
    """args.batch cross-section-perturbed instances of `p` (the same tracks,
    lognormal(0, 0.05) factors per material and group), `iters` eigenvalue
    iterations each, two ways: as one solve of the instances side by side
    (moc_set_instances: every sweep carries all instances' groups along each
    track, read once; device time of the timed iterations, CUDA events) and
    in one server pool (each instance its own copy of the tracks; the pool's
    device time).  Both against one instance alone (its sweep time x the
    instance count)."""
    from openmoc_gb300 import GB300Solver, instances, lattice
    from openmoc_gb300.serving import Server, pool_capacity
    from openmoc_gb300.solver import FISSION_SOURCE
    n = args.batch
    sets = []
    insts = []
    for i in range(n):
        mats = lattice._fuel_mod(0, p.num_groups, 1, perturb=(7000 + i, 0.05))
        sets.append(lattice.pack_materials(mats))
        insts.append(p.with_xs(*sets[-1]))
    ints_one = p.integrations_per_sweep
    out = {"instances": n, "iterations_each": iters}
    # one instance alone
    s = GB300Solver(insts[0])
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(3, FISSION_SOURCE)
    st, sw = s.benchIterations(iters, FISSION_SOURCE, True)
    s.close()
    out["alone"] = {"ms_per_iteration": float(np.mean(st)),
                    "integrations_per_s": ints_one / (float(np.mean(st)) * 1e-3)}
    # side by side: one solve of n instances
    wide = instances(p, sets)
    s = GB300Solver(wide)
    s.setInstances(n)
    s.setConvergenceThreshold(1e-30)
    lps, slots, kind = s.autotune()
    s.computeEigenvalue(3, FISSION_SOURCE)
    st, sw = s.benchIterations(iters, FISSION_SOURCE, True)
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters, FISSION_SOURCE)
    keffs = s.getInstanceKeffs().tolist()
    s.close()
    t_wide = float(np.mean(st))
    out["side_by_side"] = {
        "ms_per_iteration": t_wide, "sweep_ms_per_iteration": float(np.mean(sw)),
        "integrations_per_s": n * ints_one / (t_wide * 1e-3),
        "speedup_vs_alone_one_by_one": n * out["alone"]["ms_per_iteration"] / t_wide,
        "sweep_shape": [lps, slots], "keff": keffs}
    # one server pool
    srv = Server(iterations_per_poll=iters)
    srv.add_pool(p.num_groups, p.num_polar_half, **pool_capacity(insts, n))
    t0 = time.perf_counter()
    tickets = [srv.submit(q, "eigenvalue", iters, 1, threshold=1e-30) for q in insts]
    srv.run_until_idle()
    res = [srv.wait(t, timeout=0) for t in tickets]
    wall = time.perf_counter() - t0
    st = srv.stats()
    pool = srv.pool_stats(0)
    srv.close()
    total = sum(r["iterations"] for r in res) * ints_one
    out["pool"] = {"integrations_per_s_device": total / st["gpu_busy_s"],
                   "integrations_per_s_wall": total / wall,
                   "device_s": st["gpu_busy_s"], "wall_s": wall,
                   "sweep_shape": [pool["lanes"], pool["pairs"]],
                   "keff": [r["keff"] for r in res]}
    return out


# ---------------------------------------------------------------- serving
SERVING_WORKLOAD = ("request stream: Poisson arrivals, 70% eigenvalue / 30% fixed-source; "
                    "pin cell, 3x3, 7x7 or 17x17 (guide tubes) lattice; 2, 7, 16 or 70 groups; "
                    "lognormal(0, 0.05) cross-section factors; 16-64 azimuthal; 0.05-0.1 cm")
SERVING_GEOMS = ("pin", "3x3", "7x7", "17x17")
SERVING_GROUPS = (2, 7, 16, 70)
SERVING_AZIM = (16, 32, 48, 64)
SERVING_SPACING = (0.05, 0.075, 0.1)
SOURCE_KEFF = 3.0   # fixed eigenvalue of the source solves, above every request's own k
# the linear-source stream: the same request classes without the 17x17
# assemblies and the 70-group sets
SERVING_LS_WORKLOAD = ("linear-source request stream (CPULSSolver): Poisson arrivals, "
                       "70% eigenvalue / 30% fixed-source; pin cell, 3x3 or 7x7 lattice; "
                       "2, 7 or 16 groups; lognormal(0, 0.05) cross-section factors; "
                       "16-64 azimuthal; 0.05-0.1 cm")
SERVING_LS_GEOMS = ("pin", "3x3", "7x7")
SERVING_LS_GROUPS = (2, 7, 16)


def serving_stream(n, seed, mean_gap_ms, geoms=SERVING_GEOMS, groups=SERVING_GROUPS):
    """n requests: arrival time, geometry, groups, quadrature, kind, seed."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(mean_gap_ms * 1e-3)
        out.append(dict(
            i=i, arrival=t, geom=geoms[rng.integers(len(geoms))],
            G=int(groups[rng.integers(len(groups))]),
            azim=int(SERVING_AZIM[rng.integers(4)]),
            spacing=float(SERVING_SPACING[rng.integers(3)]),
            kind="source" if rng.random() < 0.3 else "eigenvalue"))
    return out


def serving_problems(stream, ls=False):
    """Problems of a request stream; track laydowns are generated once per
    (geometry, quadrature) and each request gets its own perturbed cross
    sections (factor on sigma_t and the same row of scattering).  ls: with
    the linear-source geometry."""
    from openmoc_gb300 import lattice
    tracks = {}
    probs = []
    for r in stream:
        key = (r["geom"], r["azim"], r["spacing"])
        if key not in tracks:
            if r["geom"] == "pin":
                tracks[key] = lattice.pin_cell(2, r["azim"], r["spacing"],
                                               linear_source=ls)
            elif r["geom"] == "17x17":
                tracks[key] = lattice.assembly_17x17(2, r["azim"], r["spacing"], config=0,
                                                     linear_source=ls)
            else:
                n = int(r["geom"][0])
                tracks[key] = lattice.square_lattice(n, 2, r["azim"], r["spacing"], config=0,
                                                     linear_source=ls)
        mats = lattice._fuel_mod(0, r["G"], 1, perturb=(1000 + r["i"], 0.05))
        p = tracks[key].with_xs(*lattice.pack_materials(mats))
        fs = None
        if r["kind"] == "source":
            fs = np.zeros((p.num_fsrs, p.num_groups), np.float32)
            fs[p.fsr_mat == 0, :] = 1.0
        probs.append((p, fs))
    return probs


def serve_plain(stream, probs, max_iters, ls=False):
    """The plain loop: one GB300Solver (GB300LSSolver with ls) per request,
    one at a time, in arrival order (upload, solve, fluxes back)."""
    from openmoc_gb300 import GB300LSSolver, GB300Solver
    out = []
    t0 = time.perf_counter()
    clock = 0.0
    for r, (p, fs) in zip(stream, probs):
        now = time.perf_counter() - t0
        if now < r["arrival"]:
            time.sleep(r["arrival"] - now)
        t_start = time.perf_counter()
        s = GB300LSSolver(p) if ls else GB300Solver(p)
        s.setAutotune(False)
        if not ls:
            s.useExponentialIntrinsic()
        s.setConvergenceThreshold(1e-5)
        if fs is not None:
            s.setFixedSources(fs)
            s.computeSource(max_iters, SOURCE_KEFF, 2)
        else:
            s.computeEigenvalue(max_iters, 1)
        flux = s.getFluxes()
        out.append(dict(keff=s.getKeff(), iterations=s.getNumIterations(), flux=flux,
                        sweep_s=s.getSweepTime()[0] * 1e-3))
        s.close()
        clock = time.perf_counter() - t0
        out[-1]["solve_s"] = time.perf_counter() - t_start
        out[-1]["latency"] = clock - r["arrival"]
    return out, clock


def serve_batched(stream, probs, max_iters, max_solves, k, priorities=True,
                  hot_bytes=0, ls=False):
    """The server: requests submitted at their arrival times from this
    thread while the request loop runs on its own (ls: linear-source
    pools and requests)."""
    from openmoc_gb300.serving import Server, pool_capacity
    srv = Server(iterations_per_poll=k, priorities=priorities, hot_bytes=hot_bytes)
    by_g = {}
    for p, _ in probs:
        by_g.setdefault(p.num_groups, []).append(p)
    pools = []
    for G, ps in sorted(by_g.items()):
        pools.append(srv.add_pool(G, ps[0].num_polar_half, linear_source=ls,
                                  **pool_capacity(ps, max_solves)))
    srv.start()
    t0 = time.perf_counter()
    tickets = []
    for r, (p, fs) in zip(stream, probs):
        now = time.perf_counter() - t0
        if now < r["arrival"]:
            time.sleep(r["arrival"] - now)
        if fs is not None:
            t = srv.submit(p, "source", max_iters, 2, k_eff=SOURCE_KEFF, fixed_source=fs,
                           linear_source=ls)
        else:
            t = srv.submit(p, "eigenvalue", max_iters, 1, linear_source=ls)
        tickets.append(t)
    res = [srv.wait(t) for t in tickets]
    clock = time.perf_counter() - t0
    stats = srv.stats()
    stats["pools"] = [srv.pool_stats(i) for i in pools]
    srv.stop()
    srv.close()
    # submission happens at the arrival time
    for x in res:
        x["latency"] = x["t_done"] - x["t_submit"]
    return res, clock, stats


def run_serving(args, ls=False):
    """The request-stream benchmark; ls: the linear-source stream through
    linear-source pools against a plain loop of GB300LSSolver."""
    import torch  # noqa: F401  (CUDA context and device checks)
    if ls:
        stream = serving_stream(args.serving_ls_requests, 0xC0FFEE + 3,
                                args.serving_ls_gap_ms, SERVING_LS_GEOMS,
                                SERVING_LS_GROUPS)
    else:
        stream = serving_stream(args.serving_requests, 0xC0FFEE + 2, args.serving_gap_ms)
    t_prep = time.perf_counter()
    probs = serving_problems(stream, ls)
    t_prep = time.perf_counter() - t_prep
    # warm both paths (kernel loading, autotune caches) on a few requests
    serve_plain(stream[:4], probs[:4], args.serving_iters, ls)
    batched, t_b, stats = serve_batched(stream, probs, args.serving_iters,
                                        args.serving_slots, args.serving_k,
                                        not args.serving_no_priorities,
                                        args.serving_hot_mb << 20, ls)
    plain, t_p = serve_plain(stream, probs, args.serving_iters, ls)
    diffs = []
    for r, a, b in zip(stream, batched, plain):
        fa, fb = a["flux"].astype(np.float64), b["flux"].astype(np.float64)
        diffs.append(dict(
            request=r["i"], cls=f'{r["geom"]}/{r["G"]}g/{r["kind"]}',
            dk=abs(a["keff"] - b["keff"]),
            dflux=float(np.max(np.abs(fa - fb) / np.abs(fb))),
            iterations=(a["iterations"], b["iterations"])))
    dk = max(d["dk"] for d in diffs)
    df = max(d["dflux"] for d in diffs)
    df_same = max([d["dflux"] for d in diffs if d["iterations"][0] == d["iterations"][1]]
                  or [0.0])
    worst = sorted(diffs, key=lambda d: -d["dflux"])[:5]
    classes = {}
    for r, (p, _), a in zip(stream, probs, plain):
        c = classes.setdefault(f'{r["geom"]}/{r["G"]}g', dict(
            requests=0, plain_solve_s=0.0, plain_sweep_s=0.0, iterations=0,
            integrations=0.0))
        c["requests"] += 1
        c["plain_solve_s"] += a["solve_s"]
        c["plain_sweep_s"] += a["sweep_s"]
        c["iterations"] += a["iterations"]
        c["integrations"] += float(p.integrations_per_sweep) * a["iterations"]
    # per class: the batched solves' latencies beside the plain loop's
    for r, b in zip(stream, batched):
        c = classes[f'{r["geom"]}/{r["G"]}g']
        c.setdefault("batched_latency_s", []).append(b["latency"])
    for c in classes.values():
        lat = np.array(c.pop("batched_latency_s"))
        c["batched_p50_latency_s"] = float(np.percentile(lat, 50))
        c["batched_p99_latency_s"] = float(np.percentile(lat, 99))
        c["plain_integrations_per_s"] = c["integrations"] / max(c["plain_sweep_s"], 1e-12)
    lat_b = np.array([x["latency"] for x in batched])
    lat_p = np.array([x["latency"] for x in plain])
    n = len(stream)
    # The ceiling of the mix: every request's integrations at the rate the
    # fastest class sweeps at alone (the large 70-group solves, FP32-bound),
    # i.e. a batched makespan no shorter than the stream's total work at the
    # best single-problem sweep rate; and the same at the FP32 peak.
    total_int = sum(c["integrations"] for c in classes.values())
    best_rate = max(c["plain_integrations_per_s"] for c in classes.values())
    import torch
    props = torch.cuda.get_device_properties(0)
    fp32_rate = props.multi_processor_count * 128 * 2 * 2.07e9 / FLOPS_PER_INTEGRATION
    ceiling = {"stream_integrations": total_int,
               "best_single_problem_rate": best_rate,
               "min_makespan_s_at_best_rate": total_int / best_rate,
               "speedup_ceiling_at_best_rate": t_p / (total_int / best_rate)}
    if not ls:   # the flat sweep's flops per integration
        ceiling.update({"min_makespan_s_at_fp32_peak": total_int / fp32_rate,
                        "speedup_ceiling_at_fp32_peak": t_p / (total_int / fp32_rate)})
    out = {
        "metric": "solves/s (batched server vs plain per-solve loop)",
        "value": n / t_b, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
        "data": "synthetic (seeded cross sections, generated tracks)",
        "config": {"workload": SERVING_LS_WORKLOAD if ls else SERVING_WORKLOAD,
                   "requests": n,
                   "mean_interarrival_ms": (args.serving_ls_gap_ms if ls
                                            else args.serving_gap_ms),
                   "source_keff": SOURCE_KEFF, "max_iters": args.serving_iters,
                   "solves_per_pool": args.serving_slots,
                   "iterations_per_poll": args.serving_k,
                   "stream_priorities": not args.serving_no_priorities,
                   "hot_bytes_budget_mb": args.serving_hot_mb,
                   "problem_prep_s": t_prep},
        "batched": {"solves_per_s": n / t_b, "makespan_s": t_b,
                    "p50_latency_s": float(np.percentile(lat_b, 50)),
                    "p99_latency_s": float(np.percentile(lat_b, 99)), "stats": stats},
        "plain": {"solves_per_s": n / t_p, "makespan_s": t_p,
                  "p50_latency_s": float(np.percentile(lat_p, 50)),
                  "p99_latency_s": float(np.percentile(lat_p, 99))},
        "speedup": t_p / t_b,
        "ceiling": ceiling,
        "by_class": classes,
        # a request whose two solves stopped one iteration apart can differ
        # in fluxes that are still decaying from the flat guess (1e-9 of the
        # peak); df_same covers the requests that ran the same iterations
        "agreement": {"max_abs_keff_diff": dk, "max_rel_flux_diff": df,
                      "max_rel_flux_diff_same_iterations": df_same,
                      "same_iterations": int(sum(d["iterations"][0] == d["iterations"][1]
                                                 for d in diffs)),
                      "unconverged": int(sum(not x["converged"] for x in batched)),
                      "worst": worst},
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-iters", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="leave out the FP64 comparison of the end-to-end result")
    ap.add_argument("--shape", default="",
                    help="lanes,group_pairs_per_lane,exp (0 table, 1 ex2) instead of autotuning")
    ap.add_argument("--workload", default="assembly70", choices=sorted(WORKLOADS),
                    help="single-solve configuration (default: the headline one)")
    ap.add_argument("--batch", type=int, default=0,
                    help="with --workload: also run this many cross-section-perturbed "
                         "instances in one server pool (one launch per kernel)")
    ap.add_argument("--serving", action="store_true",
                    help="the request-stream benchmark (batched server vs plain loop)")
    ap.add_argument("--serving-requests", type=int, default=512)
    ap.add_argument("--serving-ls", action="store_true",
                    help="the linear-source request stream alone (with --serving)")
    ap.add_argument("--serving-ls-requests", type=int, default=256,
                    help="requests of the linear-source stream (0: leave it out "
                         "of the default line)")
    ap.add_argument("--serving-ls-gap-ms", type=float, default=0.25,
                    help="mean interarrival time of the linear-source stream (its "
                         "solves are short: a 2 ms gap leaves the server idle)")
    ap.add_argument("--serving-gap-ms", type=float, default=2.0)
    ap.add_argument("--serving-iters", type=int, default=1000)
    ap.add_argument("--serving-slots", type=int, default=64)
    ap.add_argument("--serving-k", type=int, default=8)
    ap.add_argument("--serving-no-priorities", action="store_true")
    ap.add_argument("--serving-hot-mb", type=int, default=32,
                    help="L2 budget of the live solves' sources and tallies")
    ap.add_argument("--no-configs", action="store_true",
                    help="leave the 51x51 core and 3D assembly single-solve figures out")
    ap.add_argument("--no-raytrace", action="store_true",
                    help="skip the track-generation timing (host vs device ray tracing)")
    ap.add_argument("--no-cmfd", action="store_true",
                    help="leave the CMFD time-to-solution comparison out")
    ap.add_argument("--cmfd-only", nargs="?", const="core", choices=("core", "assembly"),
                    help="only one CMFD-accelerated solve (for profiling): the 51x51 "
                         "core (default) or the 17x17 70-group assembly; prints its "
                         "iterations, seconds and coarse-solve statistics")
    ap.add_argument("--cmfd-solver", default="auto", choices=("auto", "cells", "block"),
                    help="with --cmfd-only: the device coarse solve")
    ap.add_argument("--no-serving", action="store_true",
                    help="leave the request-stream benchmark out of the default line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.cmfd_only:
        print(json.dumps(cmfd_solve_only(args.cmfd_only, args.cmfd_solver)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.serving:
        print(json.dumps(run_serving(args, ls=args.serving_ls)), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
