"""Benchmark of the simulation step: Gcell-updates/s (hydro + ionization) on one GB300,
the HBM-roofline fraction of the dominant kernel, and the CPU baseline beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step" = one main-phase simulation step, sim.py:1099-1114, plus the FUV field
on the viewer's cadence): the turbulent sheet at 256^3 FP32 (Gaussian slab n = 50, k^-4
velocity field of rms Mach 5, log-normal density sigma 0.5), six stars with log-uniform
photon rates, winds on, ionization every 3 steps with 512 x 1024 rays (dr = dx), FUV every
16 steps on a 160 x 160 x 320 grid -- the reference Sim's fast-mode budgets for this grid
(sim.py:753-759).  HLL + minmod, RK2, CFL 0.3, cs_n = 1, cs_i = 12.  Synthetic seeded data.

The step runs on the package's default library build (libnebula_fast.so: FMA contraction,
approximate division / square root, within the path's tolerance of the exact build); the same
line reports the exact build (libnebula.so, bit-identical to the reference's kernel source in float32) on the same
workload under "arith_exact".  --arith picks the build of the headline.

--impl reference times the reference scheme's CPU implementation (the CPU restatement of its
kernels in oracle/, all host threads) on the same workload and metric.
Under torchrun (N > 1) every rank advances its own independent instance (replicas; the path
does not shard) and the job throughput is N x cells x steps / max-over-ranks time.

Other workloads (--workload): batch32 (32 uneven instances, persistent kernels + CUDA graphs,
beside the same instances stepped one at a time), served (Poisson branch requests from device
snapshots under an HBM budget, p50/p99), cliff1024 (the 1024^3 cloud wall with the -x plane
source, FP64 totals), stirred256 (the stirring phase at 256^3: hydro without sources + drive),
render256 (the renderer's voxel pack + prefilter of the 256^3 sheet).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s (hydro+ion)"
UNIT = "Gcell-updates/s"
RES = 256


def workload(res):
    rays = "512x1024" if res <= 256 else "1024x2048"
    fuv = "128x128x256" if res <= 192 else ("160x160x320" if res <= 256 else "256x256x512")
    return (f"turbulent sheet {res}^3 fp32, 6 stars, wind on, ionization every 3 steps ({rays} rays, dr=dx), "
            f"FUV every {8 if res <= 160 else 16} steps ({fuv} grid), HLL+minmod RK2 CFL 0.3")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """per-launch DRAM bytes of kernels at this workload, from the committed ncu summary"""
    p = os.path.join(ROOT, "profiles", "traffic_sheet256.txt")   # per-launch DRAM bytes at 256^3
    out = {}
    if os.path.exists(p):
        for line in open(p):
            parts = line.split()
            if len(parts) >= 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 20 ms; the summary keeps the samples that
    arrived while the timed region ran.  `start()` may launch the sampler ahead of the region (before
    the warm-up), so that it is already sampling when a short region begins.  The region is also
    marked as the NVTX range "timed" (ncu --nvtx --nvtx-include timed/ captures only it)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.arrived = []                        # (monotonic arrival time, csv line)
        self.window = None

    def start(self):
        if self.p is not None:
            return self
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "20"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except OSError:
            self.p = None
            return self
        import atexit
        import threading
        atexit.register(self._stop)              # never outlive the process, whatever happens

        def read(out):
            for ln in out:
                if ln.strip():
                    self.arrived.append((time.monotonic(), ln))
        self.reader = threading.Thread(target=read, args=(self.p.stdout,), daemon=True)
        self.reader.start()
        return self

    def _stop(self):
        if self.p is not None and self.p.poll() is None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.p.wait()
        if getattr(self, "reader", None) is not None:
            self.reader.join(timeout=5)

    def __enter__(self):
        self.start()
        import torch
        torch.cuda.nvtx.range_push("timed")
        self.t_enter = time.monotonic()
        return self

    def __exit__(self, *a):
        import torch
        t_exit = time.monotonic()
        torch.cuda.nvtx.range_pop()
        time.sleep(0.03)                         # the sample taken at the end of the region arrives
        self._stop()
        self.window = (self.t_enter, t_exit + 0.03)
        self.lines = [ln for t, ln in list(self.arrived) if self.window[0] <= t <= self.window[1]]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def replica_throughput(local_ms, cells, steps, dist=None, device="cpu"):
    """whole-job Gcell-updates/s of N independent replicas: every rank advanced `cells` cells for
    `steps` steps; the job time is the slowest rank's (max over ranks)"""
    import torch
    ws = 1
    t_max = float(local_ms)
    if dist is not None and dist.is_initialized():
        ws = dist.get_world_size()
        t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    return ws * cells * steps / (t_max * 1e-3) / 1e9, t_max


def algorithmic_bytes(kind, ncell, nstars):
    """compulsory HBM bytes of one launch of each kernel kind (per cell: float32 state)"""
    per = {"stage1": 36, "stage2": 52, "cast_rays": 4 * nstars, "apply_front": 6, "smooth": 24,
           "cast_fuv": 8 * nstars, "apply_fuv": 2, "max_speed": 20, "ctrl": 0}
    return per.get(kind, 0) * ncell


def ray_march_samples(star, L, dr, nsteps, nu, nphi, rfront=None, rcap=None, rstop=None):
    """Samples the reference's ray loops evaluate for one star's (nu, nphi) rays.

    Each ray runs n over [int(t_in / dr), min(nsteps, int(t_out / dr) + 2)) with (t_in, t_out)
    the slab test against [0, L] (box_range, nebula3d.py:229-244).  cast_rays (nebula3d.py:247-270)
    leaves the loop at the front crossing: a front rf < rcap lies in [n dr, (n + 1) dr) of the
    crossing sample n, which is the last one evaluated.  cast_fuv (nebula3d.py:320-352) leaves it
    once r = (n + 1/2) dr reaches rstop = nr * binr (its last radial bin).  Geometry in float64:
    a ray whose bound falls on a sample boundary in float32 may count one sample more or less."""
    import numpy as np
    u = -1.0 + (np.arange(nu) + 0.5) * 2.0 / nu
    s = np.sqrt(np.maximum(1.0 - u * u, 0.0))
    phi = (np.arange(nphi) + 0.5) * 2.0 * np.pi / nphi
    d = np.stack([s[:, None] * np.cos(phi)[None, :], s[:, None] * np.sin(phi)[None, :],
                  np.broadcast_to(u[:, None], (nu, nphi))])
    t0 = np.zeros((nu, nphi))
    t1 = np.full((nu, nphi), 1e9)
    for a in range(3):
        o, da = float(star[a]), d[a]
        flat = np.abs(da) < 1e-9
        with np.errstate(divide="ignore", invalid="ignore"):
            ta = np.where(flat, 0.0, (0.0 - o) / da)
            tb = np.where(flat, 0.0, (float(L[a]) - o) / da)
        t0 = np.where(flat, t0, np.maximum(t0, np.minimum(ta, tb)))
        t1 = np.where(flat, np.where((o < 0.0) | (o > L[a]), -1.0, t1), np.minimum(t1, np.maximum(ta, tb)))
    n0 = np.trunc(t0 / dr)
    n1 = np.minimum(nsteps, np.trunc(t1 / dr) + 2)
    if rfront is not None:
        rf = np.asarray(rfront, np.float64).reshape(nu, nphi)
        n1 = np.where(rf < rcap, np.minimum(n1, np.floor(rf / dr) + 1), n1)
    if rstop is not None:
        n1 = np.minimum(n1, math.ceil(rstop / dr - 0.5) + 1)
    return int(np.maximum(n1 - n0, 0).sum())


def ray_rates(sim, lib, kinds):
    """Ray samples per second of the ionizing and FUV ray kernels: the samples the reference's
    loops evaluate for the active stars (ray_march_samples; the ionizing fronts re-cast from the
    final state) over the mean launch time of each kernel.  Our kernels may evaluate a few more
    (G lanes step G samples at a time) or fewer (the FUV rays stop once exp(-tau) is 0.0f)."""
    import ctypes as C
    import torch
    from nebulaviewer_gb300 import _lib
    act = sim.active_stars()
    nu, nphi = sim.rfront.shape
    rf = torch.empty((nu, nphi), dtype=torch.float32, device=sim._rho.device)
    ion = fuv = 0
    for x, y, z, qf, _ in act:
        xyz = (C.c_double * 3)(x, y, z)
        _lib.check(lib.nb_cast_rays(sim._h, xyz, qf * sim.P["q_main"], C.c_void_p(rf.data_ptr())), sim._h,
                   "nb_cast_rays")
        ion += ray_march_samples((x, y, z), sim.L, sim.dr, sim.nsteps, nu, nphi, rfront=rf.cpu().numpy(),
                                 rcap=sim.diag)
        fuv += ray_march_samples((x, y, z), sim.L, sim.dr, sim.nsteps, sim.att.shape[1], sim.att.shape[2],
                                 rstop=sim.diag)       # nr * binr, binr = diag / nr (sim.py:957-958)
    out = {"stars": len(act)}
    for kind, n in (("cast_rays", ion), ("cast_fuv", fuv)):
        if kind in kinds:
            ms, launches = kinds[kind]
            out[kind] = {"samples_per_launch": n, "gsamples_per_s": n / (ms / launches * 1e-3) / 1e9}
    return out


def cpu_sample(ic_host, steps=3):
    """the oracle (reference scheme, CPU restatement) on a bounded sample of the workload"""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from nebulaviewer_gb300.params import make_params, sound_speeds
    P = make_params(base=ic_host["P"])
    cn2, ci2, vmax = sound_speeds(P)
    o = O.OracleSim(ic_host["shape"], ic_host["dx"], ic_host["rho"], ic_host["stars"], ic_host["kinds"],
                    ic_host["jets"], ic_host["jkinds"], P, mom=ic_host["mom"], cn2=cn2, ci2=ci2, vmax=vmax)
    t0 = time.perf_counter()
    o.step(steps)
    t1 = time.perf_counter()
    o.fuv_field()
    t2 = time.perf_counter()
    # per step: the steps (1 ionization in 3) plus the FUV field amortized on its cadence
    per_step = (t1 - t0) / steps + (t2 - t1) / o.fuv_every
    ncell = math.prod(ic_host["shape"])
    return ncell / per_step / 1e9, O.threads(), per_step, o


def host_ic(sim):
    """the instance's initial state on the host (the CPU arm starts from the same fields)"""
    import numpy as np
    return dict(shape=sim.shape, dx=sim.dx, rho=sim.rho.numpy().astype(np.float32),
                mom=[sim.mx.numpy(), sim.my.numpy(), sim.mz.numpy()], stars=list(sim.stars),
                kinds=list(sim.kinds), jets=list(sim.jets), jkinds=list(sim.jkinds), P=dict(sim.P))


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import torch
    from nebulaviewer_gb300 import ics
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    ic = ics.sheet(res=args.res, device=dev)
    ic_host = dict(ic, rho=ic["rho"].cpu().numpy(), mom=[m.cpu().numpy() for m in ic["mom"]])
    del ic
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from nebulaviewer_gb300.params import make_params, sound_speeds
    P = make_params(base=ic_host["P"])
    cn2, ci2, vmax = sound_speeds(P)
    o = O.OracleSim(ic_host["shape"], ic_host["dx"], ic_host["rho"], ic_host["stars"], ic_host["kinds"],
                    ic_host["jets"], ic_host["jkinds"], P, mom=ic_host["mom"], cn2=cn2, ci2=ci2, vmax=vmax)
    for _ in range(min(args.warmup, 1)):
        o.step(1)
    budget = 150.0
    t0 = time.perf_counter()
    done = 0
    for n in range(args.steps):
        o.step(1)
        if o.version % o.fuv_every == 0:
            o.fuv_field()
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    ncell = math.prod(ic_host["shape"])
    val = ncell * done / el / 1e9
    cores = O.threads()
    sample = f"{done} of {args.steps} requested steps of the {workload(args.res)} (bounded to {budget:.0f} s)"
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": done,
            "warmup": min(args.warmup, 1), "ms_per_step": el / done * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload(args.res), "grid": [args.res] * 3, "parallelism": "cpu threads"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import ctypes as C
    import torch
    ws, rank, local = dist_env()
    from nebulaviewer_gb300 import build as nb_build
    if rank == 0:
        nb_build.build(verbose=False)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist.barrier()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from nebulaviewer_gb300 import _lib
    from nebulaviewer_gb300.sim import Sim
    arith = _lib.arith_of(args.arith)
    lib = _lib.load(arith)
    sim = Sim("sheet", res=args.res, device=dev, verbose=False, arith=arith)
    ncell = sim._n
    nstars = len(sim.stars)
    ic_host = host_ic(sim) if (rank == 0 and ws == 1 and not args.no_cpu_baseline) else None
    pinned0 = [t.detach().to("cpu").pin_memory() for t in (sim._rho, sim._mx, sim._my, sim._mz)]
    stream = torch.cuda.current_stream(dev)

    def device_steps(k):
        for _ in range(k):
            sim.step(1, sync=False)
            if sim.version % sim.fuv_every == 0:          # the render-field cadence (sim.py:997-1002)
                sim.fuv_field()

    from nebulaviewer_gb300.autotune import autotune
    tuning = {k: v[0] for k, v in autotune(sim).items()}       # untimed: launch shapes for this problem
    clk = ClockSampler(local).start()          # sampling before the timed region begins
    device_steps(args.warmup)
    torch.cuda.synchronize(dev)
    # ---------------- device-resident throughput (the metric's value)
    lib.nb_profile(sim._h, 1)
    prof_ms = (C.c_double * 16)()
    prof_n = (C.c_longlong * 16)()
    lib.nb_profile_read(sim._h, prof_ms, prof_n)          # discard the warm-up records
    l0 = C.c_longlong()
    lib.nb_counters(sim._h, C.byref(l0))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with clk:
        ev0.record(stream)
        device_steps(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    el_ms = ev0.elapsed_time(ev1)
    lib.nb_profile_read(sim._h, prof_ms, prof_n)
    lib.nb_profile(sim._h, 0)
    l1 = C.c_longlong()
    lib.nb_counters(sim._h, C.byref(l1))
    launches = int(l1.value - l0.value)
    value, t_max = replica_throughput(el_ms, ncell, args.steps, dist, dev)
    # ---------------- end to end through the public API with host buffers
    # every step: sim.step(1) (returns after the step finished), the live-parameter block
    # pushed H2D as a caller that edits P each step does (bake.py), and the clock read D2H
    # (sim.t, as bake.py reads it every step); around the steps: the initial state uploaded
    # from pinned host memory and the result fields (rho, xi) read back to pinned memory.
    out_host = [torch.empty(sim.shape, dtype=torch.float32).pin_memory() for _ in range(2)]
    e2e_steps = args.steps
    h2d_live = C.sizeof(_lib.NbLive)

    def e2e_pass():
        """one end-to-end pass: the same initial state uploaded, K blocking steps, results read back"""
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for dst, src in zip((sim._rho, sim._mx, sim._my, sim._mz), pinned0):
            dst.copy_(src, non_blocking=True)
        sim.invalidate()
        for _ in range(e2e_steps):
            sim._live_key = None                           # force the H2D push of the live block
            sim.step(1)
            sim.update_render_fields()
            _ = sim.t
        out_host[0].copy_(sim._rho, non_blocking=True)
        out_host[1].copy_(sim._xi, non_blocking=True)
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t0

    # one untimed pass, then five identical timed passes (each restarts from the same uploaded
    # state); the median is reported: a host-timed pass swings with the host's scheduling (about one
    # pass in three lost ~10 ms over 96 steps)
    e2e_pass()
    e2e_runs = [e2e_pass() for _ in range(5)]
    e2e_s = sorted(e2e_runs)[2]
    if dist:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_val = ws * ncell * e2e_steps / e2e_s / 1e9
    h2d = (16 * ncell) / e2e_steps + h2d_live
    d2h = (8 * ncell) / e2e_steps + C.sizeof(_lib.NbClock)
    # ---------------- roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    kinds = {}
    for i, name in enumerate(_lib.PROF_KINDS):
        if prof_n[i]:
            kinds[name] = (prof_ms[i], int(prof_n[i]))
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms, dom_n = kinds[dom]
    dom_bytes = algorithmic_bytes(dom, ncell, nstars)
    achieved = dom_bytes / (dom_ms / dom_n * 1e-3) / 1e9
    traffic = ncu_traffic().get(dom) if args.res == RES else None
    ion_every, fuv_every = sim.ion_every, sim.fuv_every
    b_step = 108 + (4 * nstars + 14) / ion_every + (8 * nstars + 2) / fuv_every
    step_gbs = b_step * ncell * args.steps / (el_ms * 1e-3) / 1e9
    clocks = clk.summary()
    res = None
    if rank == 0:
        try:
            rays = ray_rates(sim, lib, kinds)
        except Exception as e:        # an auxiliary figure: its failure must not cost the bench line
            rays = {"error": f"{type(e).__name__}: {e}"}
        res = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload(args.res), "grid": list(sim.shape), "stars": nstars, "ion_every": ion_every,
                       "fuv_every": fuv_every, "rays": list(sim.rfront.shape), "fuv_grid": list(sim.att.shape),
                       "parallelism": f"replicas x{ws}", "l2": f"state {40 * ncell / 1e9:.2f} GB vs 129 MB L2 (no flush)",
                       "tuning": tuning},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes_per_launch": dom_bytes,
                         "avg_launch_ms": dom_ms / dom_n},
            "step_roofline": {"bytes_per_cell_step": b_step, "achieved": step_gbs, "peak": peak, "unit": "GB/s",
                              "frac": step_gbs / peak},
            "kernels_ms": {k: {"ms_total": v[0], "launches": v[1], "share": v[0] / sum(x[0] for x in kinds.values())}
                           for k, v in kinds.items()},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "how": "Sim.step(1) + update_render_fields + clock read per step; state upload from pinned "
                           "host memory and rho/xi read-back inside the timed region; median of 5 passes after an untimed one",
                    "passes": [ws * ncell * e2e_steps / t / 1e9 for t in e2e_runs]},
            "gpu_launches": launches,
            "clocks": clocks,
            "ray_samples": rays,
        }
    sim.close()
    if rank == 0:
        # the other library build on the same workload, device-resident, for comparison
        other = "exact" if arith == "fast" else "fast"
        s2 = Sim("sheet", res=args.res, device=dev, verbose=False, arith=other)
        autotune(s2)
        for _ in range(args.warmup):
            s2.step(1, sync=False)
            if s2.version % s2.fuv_every == 0:
                s2.fuv_field()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            s2.step(1, sync=False)
            if s2.version % s2.fuv_every == 0:
                s2.fuv_field()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms2 = e0.elapsed_time(e1)
        res["arith"] = arith
        res[f"arith_{other}"] = {"value": ncell * args.steps / (ms2 * 1e-3) / 1e9, "unit": UNIT,
                                 "ms_per_step": ms2 / args.steps}
        s2.close()
    if rank == 0 and ws == 1 and not args.no_added_forms and args.res == RES:
        res.update(added_forms(args))
    if rank == 0 and ic_host is not None:
        n_cpu = 9                      # ~8 s of oracle work on 16 host cores at 256^3, 3 ionizations
        cv, cores, per_step, _ = cpu_sample(ic_host, steps=n_cpu)
        res["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{n_cpu} steps ({n_cpu // 3} ionizations) + 1 FUV field amortized over "
                                         f"{fuv_every} steps of the same "
                                         f"{args.res}^3 workload, oracle/ref_cpu.cpp with OpenMP ({per_step:.2f} s/step)"}
    if rank == 0:
        print(json.dumps(res), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def batch_result(args, steps, warmup):
    """The batched workload: 32 instances (cubes 64^3-192^3 + slabs such as 96x160x288; torus or
    sheet; 1-8 stars; own seeds) advanced together (persistent kernels, CUDA graphs), beside the
    same instances stepped one after another through the plain drop-in Sim.step(1), which blocks
    every step as the reference's does."""
    import torch
    from nebulaviewer_gb300 import build as nb_build
    nb_build.build(verbose=False)
    from nebulaviewer_gb300.batch import BatchSim, batch_workload
    dev = torch.device("cuda", 0)
    sims = batch_workload(n=args.instances, device=dev, verbose=False, arith=args.arith)
    cells = sum(s._n for s in sims)
    # plain: each instance alone, blocking steps (the reference's calling pattern)
    plain_steps = max(3, steps // 5)
    t0 = time.perf_counter()
    for s in sims:
        for _ in range(plain_steps):
            s.step(1)
    plain_s = time.perf_counter() - t0
    plain = cells * plain_steps / plain_s / 1e9
    B = BatchSim(sims, graphs=True)
    clk = ClockSampler(0).start()              # sampling before the timed region begins
    B.step(warmup)
    torch.cuda.synchronize(dev)
    l0 = B.launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clk:
        ev0.record()
        B.step(steps, sync=False)
        ev1.record()
        torch.cuda.synchronize(dev)
    B.check_status()
    el = ev0.elapsed_time(ev1)
    val = cells * steps / (el * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    res = {"metric": METRIC + " batched", "value": val, "unit": UNIT, "n_gpus": 1, "steps": steps,
           "warmup": warmup, "ms_per_step": el / steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{len(sims)} instances, {cells / 1e6:.1f} M cells, cubes 64^3-192^3 + slabs, "
                                  "torus/sheet, 1-8 stars each, persistent stage kernels + CUDA graphs",
                      "shapes": [list(s.shape) for s in sims]},
           "plain_sequential": {"value": plain, "unit": UNIT, "steps_per_instance": plain_steps,
                                "how": "each instance alone through Sim.step(1), blocking per step"},
           "batched_over_plain": val / plain,
           "step_roofline": {"bytes_per_cell_step": 108.0, "achieved": 108.0 * val, "peak": peak, "unit": "GB/s",
                             "frac": 108.0 * val / peak, "peak_source": peak_kind,
                             "note": "hydro bytes only (the ionization share varies per instance)"},
           "gpu_launches": B.launches() - l0, "clocks": clk.summary(), "arith": sims[0].arith}
    B.close()
    for sm in sims:
        sm.close()
    return res


def run_batch(args):
    print(json.dumps(batch_result(args, args.steps, args.warmup)), flush=True)
    return 0


def served_result(args, requests):
    """Served: Poisson arrivals; each request branches from a device snapshot of a 96^3-320^3
    instance, changes one star's photon rate or the wind by +-50% and runs 10-100 steps;
    admission under a 150 GB HBM budget charging each instance its device footprint; continuous
    batching of the instances below --solo-cells cells, the larger ones stepped alone in the same
    ticks (--solo-cells 0: every instance batched)."""
    import torch
    from nebulaviewer_gb300 import build as nb_build
    nb_build.build(verbose=False)
    from nebulaviewer_gb300 import ics, serve
    from nebulaviewer_gb300.sim import Sim
    dev = torch.device("cuda", 0)
    snaps = []
    for m, e in enumerate((96, 160, 256, 320)):
        ic = (ics.sheet(res=e, seed=40 + m, nstars=4, device=dev) if m % 2 == 0 else
              ics.torus(seed=50 + m, device=dev, shape=(e, e, e), nstars=3))
        s = Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                           ic["P"], mom=ic["mom"], device=dev, arith=args.arith)
        s.step(8)
        snaps.append(serve.Snapshot(s))
        s.close()
        del ic
    torch.cuda.synchronize(dev)
    reqs = serve.poisson_requests(snaps, requests, rate=args.rate, seed=1)
    # the warm pool a server keeps for this traffic: one idle instance per request of each snapshot
    # (all of them arrive within a fraction of a second), built before the clock starts
    warm = {}
    for r in reqs:
        warm[r.snap] = warm.get(r.snap, 0) + 1
    solo = serve.SOLO_CELLS if args.solo_cells is None else (args.solo_cells if args.solo_cells > 0 else None)
    srv = serve.Server(snaps, budget_bytes=150e9, max_slots=64, solo_cells=solo)
    clk = ClockSampler(0).start()
    with clk:
        stats, done = srv.run(reqs, realtime=True, warm=warm)
    # the same requests one after another through the plain drop-in (a warm instance per snapshot,
    # branched into by device copies; Sim.step blocks per step as the reference's does)
    plain_reqs = serve.poisson_requests(snaps, requests, rate=args.rate, seed=1)
    plain_sims = {}
    for r in plain_reqs:
        if r.snap not in plain_sims:
            plain_sims[r.snap] = snaps[r.snap].branch()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plain_cells = 0
    for r in plain_reqs:
        s = plain_sims[r.snap]
        snaps[r.snap].branch_into(s, r.mod)
        s.step(r.nsteps)
        serve.result_of(s, keep_state=False)
        plain_cells += s._n * r.nsteps
    plain_s = time.perf_counter() - t0
    for s in plain_sims.values():
        s.close()
    plain = plain_cells / plain_s / 1e9
    res = {"metric": "served p50/p99 latency and Gcell-updates/s", "value": stats["gcells_per_s"], "unit": UNIT,
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
           "plain_sequential": {"value": plain, "unit": UNIT, "wall_s": plain_s,
                                "how": "the same requests one after another through Sim.step on a warm instance "
                                       "per snapshot (branched into by device copies)"},
           "served_over_plain": stats["gcells_per_s"] / plain,
           "config": {"workload": f"{requests} requests, Poisson {args.rate:g}/s, snapshots 96^3/160^3/256^3/320^3, "
                                  "+-50% on a star's Q or the wind, 10-100 steps, 150 GB budget charging each pooled "
                                  "instance its device footprint (fields + library scratch); warm pool of one idle "
                                  "instance per request of each snapshot, built before the clock starts; "
                                  + (f"instances of {solo} cells or more stepped alone, the rest batched" if solo else
                                     "every instance batched"),
                      "footprint_bytes_per_cell": {f"{s.shape[0]}^3": s.footprint / s.cells for s in snaps}},
           "stats": stats, "clocks": clk.summary(), "arith": snaps[0].arith}
    return res


def run_served(args):
    print(json.dumps(served_result(args, args.requests)), flush=True)
    return 0


def run_stirred(args):
    """The stirring phase at 256^3 (torus_stirred: log-normal background, solenoidal forcing on the
    1/24-unit grid cross-faded every pre_corr): hydro without sources + the drive kernel with the
    fused CFL max speed, forcing fields pushed ahead into the device ring (host syncs once per
    ring-sized chunk).  pre_t is raised so the timed steps all stay in the stirring phase."""
    import ctypes as C
    import torch
    from nebulaviewer_gb300 import _lib, build as nb_build
    nb_build.build(verbose=False)
    from nebulaviewer_gb300.sim import Sim
    dev = torch.device("cuda", 0)
    res = (args.res if args.res != RES else 256) // 2
    sim = Sim("torus_stirred", res=res, device=dev, verbose=False, arith=args.arith, params=dict(pre_t=1e9))
    lib = sim._lib
    clk = ClockSampler(0).start()              # sampling before the timed region begins
    sim.step(args.warmup)
    torch.cuda.synchronize(dev)
    lib.nb_profile(sim._h, 1)
    prof_ms, prof_n = (C.c_double * 16)(), (C.c_longlong * 16)()
    lib.nb_profile_read(sim._h, prof_ms, prof_n)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clk:
        ev0.record()
        sim.step(args.steps, sync=False)
        ev1.record()
        torch.cuda.synchronize(dev)
    el = ev0.elapsed_time(ev1)
    lib.nb_profile_read(sim._h, prof_ms, prof_n)
    lib.nb_profile(sim._h, 0)
    cells = sim._n
    val = cells * args.steps / (el * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    kinds = {name: (prof_ms[i], int(prof_n[i])) for i, name in enumerate(_lib.PROF_KINDS) if prof_n[i]}
    d_ms, d_n = kinds.get("drive", (0.0, 0))
    drive_gbs = 32.0 * cells / (d_ms / max(d_n, 1) * 1e-3) / 1e9 if d_n else None
    b_step = 36.0 + 52.0 + 32.0                     # stage 1, stage 2, drive (+ max speed)
    res_d = {"metric": METRIC + " stirring phase", "value": val, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
             "warmup": args.warmup, "ms_per_step": el / args.steps, "higher_is_better": True, "dtype": "f32",
             "data": "synthetic",
             "config": {"workload": f"torus_stirred {list(sim.shape)} stirring phase: forcing grid "
                                    f"{list(sim.sshape)} (dxs {sim.dxs:.4g}), pre_corr {sim.P['pre_corr']}, "
                                    f"pre_amp {sim.P['pre_amp']}", "grid": list(sim.shape)},
             "roofline": {"bound": "hbm", "kernel": "drive", "achieved": drive_gbs, "peak": peak, "unit": "GB/s",
                          "frac": drive_gbs / peak if drive_gbs else None, "peak_source": peak_kind,
                          "traffic": ncu_traffic().get("drive") if tuple(sim.shape) == (256, 256, 256) else None,
                          "algorithmic_bytes_per_launch": 32 * cells,
                          "avg_launch_ms": d_ms / max(d_n, 1)},
             "step_roofline": {"bytes_per_cell_step": b_step, "achieved": b_step * val, "peak": peak, "unit": "GB/s",
                               "frac": b_step * val / peak, "peak_source": peak_kind},
             "kernels_ms": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kinds.items()},
             "clocks": clk.summary(), "arith": sim.arith}
    sim.close()
    print(json.dumps(res_d), flush=True)
    return 0


def run_render(args):
    """The renderer's voxel pack (render.py:176-205 pack_volume_lm with the shock proxy inline +
    the three [1 4 1] prefilter passes of render.py:281-298) on the 256^3 sheet after a few steps:
    the per-frame cost of handing the fields to the display side."""
    import ctypes as C
    import torch
    from nebulaviewer_gb300 import _lib, build as nb_build
    nb_build.build(verbose=False)
    from nebulaviewer_gb300.sim import Sim
    dev = torch.device("cuda", 0)
    sim = Sim("sheet", res=args.res, device=dev, verbose=False, arith=args.arith)
    sim.step(3)
    sim.update_render_fields(force=True)
    L = sim.L
    pp = {"c_ha": (0.33, 0.675, 1.5), "c_o3": (0.45, 1.125, 1.5), "c_s2": (1.2, 0.66, 0.3), "c_dg": (0.07, 0.035, 0.01),
          "c_sh": (0.02, 0.007, 0.009), "gs": 12.0, "ambient": 0.1, "edge": 0.08, "inv_L": [1.0 / v for v in L],
          "dx": sim.dx}
    clk = ClockSampler(0).start()              # sampling before the timed region begins
    for _ in range(args.warmup):
        sim.render_pack(pp)
    torch.cuda.synchronize(dev)
    lib = sim._lib
    lib.nb_profile(sim._h, 1)
    prof_ms, prof_n = (C.c_double * 16)(), (C.c_longlong * 16)()
    lib.nb_profile_read(sim._h, prof_ms, prof_n)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clk:
        ev0.record()
        for _ in range(args.steps):
            sim.render_pack(pp)
        ev1.record()
        torch.cuda.synchronize(dev)
    el = ev0.elapsed_time(ev1) / args.steps
    lib.nb_profile_read(sim._h, prof_ms, prof_n)
    lib.nb_profile(sim._h, 0)
    cells = sim._n
    peak, peak_kind = measured_peaks()
    b_cell = 32.0 + 3 * 16.0            # pack: rho, xi, dfront, g0, m (shock) in, 8 B out; 3 passes of 8 B in + out
    res_d = {"metric": "render pack Gcell/s", "value": cells / (el * 1e-3) / 1e9, "unit": "Gcell/s", "n_gpus": 1,
             "steps": args.steps, "warmup": args.warmup, "ms_per_pack": el, "higher_is_better": True,
             "dtype": "f32->f16", "data": "synthetic",
             "config": {"workload": f"voxel pack + [1 4 1] prefilter of the sheet {list(sim.shape)} (shock proxy on)",
                        "grid": list(sim.shape)},
             "roofline": {"bound": "hbm", "kernel": "render pack + 3 prefilter passes", "achieved": b_cell * cells / (el * 1e-3) / 1e9,
                          "peak": peak, "unit": "GB/s", "frac": b_cell * cells / (el * 1e-3) / 1e9 / peak,
                          "peak_source": peak_kind, "algorithmic_bytes_per_cell": b_cell},
             "gpu_launches": 4 * args.steps, "clocks": clk.summary(), "arith": sim.arith}
    sim.close()
    print(json.dumps(res_d), flush=True)
    return 0


def cliff_result(args, steps, warmup, res=1024):
    """The large single instance: the 1024^3 ionized cloud wall (density step n = 1 -> 200, 40
    clumps, the -x plane-parallel source + 3 stars, FUV on), FP64 conservation totals."""
    import torch
    from nebulaviewer_gb300 import build as nb_build
    nb_build.build(verbose=False)
    from nebulaviewer_gb300.sim import Sim
    dev = torch.device("cuda", 0)
    sim = Sim("cliffwall", res=res, device=dev, verbose=False, arith=args.arith)
    m0 = sim.conservation()
    clk = ClockSampler(0).start()              # sampling before the timed region begins
    sim.step(warmup)
    torch.cuda.synchronize(dev)
    m1 = sim.conservation()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with clk:
        ev0.record()
        for _ in range(steps):
            sim.step(1, sync=False)
            if sim.version % sim.fuv_every == 0:
                sim.fuv_field()
        ev1.record()
        torch.cuda.synchronize(dev)
    el = ev0.elapsed_time(ev1)
    m2 = sim.conservation()
    sim._clock()                               # raises if a hydro stage's bounded wait gave up
    cells = sim._n
    val = cells * steps / (el * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    n = len(sim.stars)
    b_step = 108 + (4 * n + 14 + 4) / sim.ion_every + (8 * n + 2 + 8) / sim.fuv_every
    res_d = {"metric": METRIC + " 1024^3 cliff wall", "value": val, "unit": UNIT, "n_gpus": 1, "steps": steps,
             "warmup": warmup, "ms_per_step": el / steps, "higher_is_better": True, "dtype": "f32",
             "data": "synthetic",
             "config": {"workload": f"ionized cloud wall {res}^3 fp32 (step n=1->200, 40 clumps), -x plane-parallel "
                                    f"source + 3 stars, FUV every {sim.fuv_every}", "grid": list(sim.shape),
                        "state_gb": 40 * cells / 1e9},
             "fp64_totals": {"mass_t0": m0[0], "mass_after_warmup": m1[0], "mass_end": m2[0],
                             "rel_change_over_timed_steps": (m2[0] - m1[0]) / m1[0], "momentum_end": list(m2[1:]),
                             "t_end": sim.t},
             "step_roofline": {"bytes_per_cell_step": b_step, "achieved": b_step * val, "peak": peak, "unit": "GB/s",
                               "frac": b_step * val / peak, "peak_source": peak_kind},
             "clocks": clk.summary(), "arith": sim.arith}
    sim.close()
    return res_d


def run_cliff(args):
    print(json.dumps(cliff_result(args, args.steps, args.warmup, args.res if args.res != RES else 1024)), flush=True)
    return 0


def added_forms(args):
    """The three added forms on short runs, for the default bench line: the batch of 32 uneven
    instances (10 timed batch steps), the served Poisson mix (40 requests) and the 1024^3 cloud
    wall (10 timed steps).  Each keeps its own clocks; a failure is reported in place of its
    numbers without costing the headline line."""
    out = {}
    for key, fn in (("batched", lambda: batch_result(args, 10, 3)), ("served", lambda: served_result(args, 40)),
                    ("cliff1024", lambda: cliff_result(args, 10, 3))):
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as e:
            out[key] = {"error": f"{type(e).__name__}: {e}"}
            continue
        keep = ("value", "unit", "ms_per_step", "steps", "warmup", "p50_ms", "p99_ms", "plain_sequential",
                "batched_over_plain", "served_over_plain", "gpu_launches", "clocks", "fp64_totals", "step_roofline",
                "arith")
        d = {k: r[k] for k in keep if k in r}
        d["workload"] = r["config"]["workload"]
        if key == "served":
            for k in ("requests", "wall_s", "instances_built", "instances_prewarmed", "branches_in_place", "evicted",
                      "batch_rebuilds", "peak_pool_bytes", "solo_ticks", "ticks"):
                d[k] = r["stats"][k]
            d["footprint_bytes_per_cell"] = r["config"]["footprint_bytes_per_cell"]
        d["run_s"] = time.perf_counter() - t0
        out[key] = d
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=96)
    ap.add_argument("--warmup", type=int, default=6)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-added-forms", action="store_true",
                    help="leave the batched / served / 1024^3 results out of the default line")
    ap.add_argument("--res", type=int, default=RES, help="grid size (the workload is defined at 256)")
    ap.add_argument("--workload", default="sheet256",
                    choices=["sheet256", "batch32", "served", "cliff1024", "stirred256", "render256"])
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--solo-cells", type=int, default=None,
                    help="served: instances of this many cells or more step alone (default: the server's; 0: none)")
    ap.add_argument("--instances", type=int, default=32)
    ap.add_argument("--arith", default=None, choices=["exact", "fast"],
                    help="library build: exact (bit-identical to the reference's kernel source in float32) or fast (FMA, approximate "
                         "division / square root); default: the package default")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch32":
        return run_batch(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "render256":
        return run_render(args)
    if args.workload == "stirred256":
        return run_stirred(args)
    if args.workload == "cliff1024":
        return run_cliff(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
