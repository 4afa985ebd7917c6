"""Benchmark: batched multi-shot 2D elastic RTM (the reference's RTM path,
W/rtm-mod-adj.f90:132-496, run for a survey of shots) on GB300.

Workload (the 64-shot survey): full grid nx=2000 x nz=800, dx=5 m,
dt=0.5 ms, nt=6000, 40-cell sponge, 15 Hz Ricker; seeded smooth random Vp
1800-4000 m/s (Gaussian filter, 200 m correlation), Vs=Vp/1.73, Gardner
density; 64 shots 75 m apart, each on its own subgrid 600-2000 cells wide;
receivers at every subgrid column at z=50 m recording Vx and Vz.  Seeded
synthetic traces stand in for field data (content does not change the cost).

One step = one group of shots (group_max shots) migrated end to end:
forward propagation with FP16 source snapshots, adjoint propagation with the
fused imaging condition, stacking.  The default --steps 16 covers the 64-shot
survey once.  Metric: Gcell-updates/s counting the forward and the adjoint
propagation (2 x nz x width x nt per shot); shots/s is reported beside it.

The same JSON line carries, from the same run:
- error_vs_fp64: the headline path's error (FP16 snapshots, FP32 fields)
  against the float64 oracle, per image, on the survey's widest group over a
  truncated window, with Born-modelled traces;
- secondary: bounded samples of the other workloads, each with its own
  clocks and roofline -- the 3D acoustic propagator (1024 x 1024 x 512), the
  learned preconditioner (training rate and learned-vs-LSRTM-10 time to
  residual, reduced pair count) and one group of the 256-shot survey
  (checkpoint-restart);
- cpu_baseline: the reference's own RTM path on the host cores.

--impl reference times the reference's CPU path on the host cores: its
Fortran modules executed through oracle/f90c.py with its C recursion
(oracle/_ref, built where the reference's sources are present), else the
oracle's C restatement; one shot per core on the survey grid over a
truncated time window.  It also times the reference's own CUDA adjoint
kernel (rtmlib-modC-gpu.cu built for sm_103a) beside this library's on the
single-shot grid.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(nz=800, nx=2000, dx=5.0, dt=5e-4, nt=6000, abc=40, fp=15.0, nsource=250, nshots=64, spacing=15,
           wmin=600, wmax=2000, zsrc=10, zrec=10, comp_mask=3, seed=2,
           desc="batched multi-shot 2D elastic RTM, 64-shot survey: 2000x800 grid, dx=5 m, dt=0.5 ms, nt=6000, "
                "64 shots on 600-2000-cell subgrids")
# The 256-shot end-to-end imaging survey: 6000 x 2000 cells,
# dx=5 m, dt=0.4 ms, nt=10000, 256 shots on 1000-6000-cell subgrids; the
# FP16 snapshots of every level would need ~1 TB per 4-shot group, so the
# engine runs in checkpoint-restart mode.  A bounded sample of groups is
# timed (the whole survey is ~64 groups).
CFG5 = dict(nz=2000, nx=6000, dx=5.0, dt=4e-4, nt=10000, abc=40, fp=15.0, nsource=250, nshots=256, spacing=23,
            wmin=1000, wmax=6000, zsrc=10, zrec=10, comp_mask=3, seed=5,
            desc="batched multi-shot 2D elastic RTM, 256-shot survey: 6000x2000 grid, dx=5 m, dt=0.4 ms, "
                 "nt=10000, 256 shots on 1000-6000-cell subgrids (smooth random background), checkpoint-restart "
                 "of the source wavefield")
BYTES_FWD = 80     # algorithmic bytes per forward cell-update
BYTES_ADJ = 112    # per adjoint cell-update with the imaging condition


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks(key="hbm_gbs"):
    """Roofline denominator: the measured copy bandwidth (GB/s) or
    BF16 GEMM rate (TFLOP/s), else the recorded fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if key in d:
            return float(d[key]), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}[key], "fallback"


def profile_traffic():
    """DRAM bytes per cell-update of the adjoint kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "step2d_adjoint_imaging_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_cell")
    return None


def build_survey():
    from elastic_gb300 import synth
    c = CFG
    vp = synth.smooth_random_model(c["nz"], c["nx"], c["dx"], 200.0, 1800.0, 4000.0, seed=c["seed"])
    rho, lam, mu = synth.lame_from_vp(vp)
    x0, nxs, xsrc = synth.uneven_survey(c["nx"], c["nshots"], c["spacing"], c["wmin"], c["wmax"], seed=c["seed"])
    n = len(nxs)
    zs = np.full(n, c["zsrc"], np.int32)
    zr = np.full(n, c["zrec"], np.int32)
    return rho, lam, mu, x0, nxs, xsrc, zs, zr


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples (the JSON line carries their summary); directory from
        # ELASTIC_CLOCKS_DIR, else the system's temporary directory
        self.path = os.path.join(os.environ.get("ELASTIC_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"elastic_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    os.environ["ELASTIC_RTM_DEVICE"] = str(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from elastic_gb300.batch import BatchRTM
    from elastic_gb300 import synth
    from elastic_gb300._lib import load
    c = CFG
    rho, lam, mu, x0, nxs, xsrc, zs, zr = build_survey()
    eng = BatchRTM(c["nz"], c["nx"], c["nt"], c["dx"], c["dt"], c["fp"], c["abc"], rho, lam, mu, x0, nxs, xsrc, zs,
                   zr, comp_mask=c["comp_mask"], group_max=args.group, nsource=c["nsource"])
    groups = eng.groups()
    eng.set_tma(args.staging == "tma")
    # autotuner: tile width per pass, timed on the widest group (untimed)
    widest = max(groups, key=lambda g: int(eng.nxs[g[0]:g[0] + g[1]].sum()))
    tune = eng.autotune(widest[0], widest[1], steps=args.tune_steps)
    # shard groups over ranks (shots are independent)
    from elastic_gb300.shard import aggregate, shard_groups
    mine = shard_groups(groups, rank, world)
    tmax = max(eng.trace_count(s, n) for s, n in groups)
    traces_host = synth.synthetic_traces(tmax, seed=c["seed"])
    # device-resident copy for the `value` measurement; pinned host copy for e2e
    traces_dev = torch.from_numpy(traces_host).to(f"cuda:{local}")
    lib = load()
    import ctypes
    pin = lib.rtm_host_alloc(tmax * 4)
    pinned = np.ctypeslib.as_array(ctypes.cast(pin, ctypes.POINTER(ctypes.c_float)), shape=(tmax,))
    pinned[:] = traces_host
    pf = 3 * c["nz"] * c["nx"]
    img_dev = torch.zeros(pf, dtype=torch.float32, device=f"cuda:{local}")
    ipin = lib.rtm_host_alloc(pf * 4)
    img_host = np.ctypeslib.as_array(ctypes.cast(ipin, ctypes.POINTER(ctypes.c_float)), shape=(pf,))
    img_host[:] = 0

    def step(k, e2e):
        s0, n = mine[k % len(mine)]
        if e2e:
            eng.migrate(s0, n, pinned, img_host, traces_on_device=False, image_on_device=False)
        else:
            eng.migrate(s0, n, traces_dev, img_dev, traces_on_device=True, image_on_device=True)
        st = eng.stats()
        return n, st

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for k in range(args.warmup):
        step(k, False)
    barrier()
    cells_done = 0
    shots_done = 0
    dev_ms = 0.0
    fwd_ms = adj_ms = 0.0
    fwd_launch = adj_launch = 0
    adj_cells = 0
    kernels = 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            n, st = step(k, False)
            cells_done += 2 * st["cells"] * c["nt"]
            shots_done += n
            dev_ms += st["total_ms"]
            fwd_ms += st["fwd_ms"]
            adj_ms += st["adj_ms"]
            fwd_launch += c["nt"] - 1
            adj_launch += c["nt"]
            adj_cells += st["cells"] * c["nt"]
            kernels += st["kernels"] + 4 * n
        barrier()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    # end-to-end: host traces in pinned memory, host image out, every step
    barrier()
    e2e_ms = 0.0
    e2e_cells = 0
    te0 = time.perf_counter()
    for k in range(args.steps):
        n, st = step(k, True)
        e2e_cells += 2 * st["cells"] * c["nt"]
    barrier()
    e2e_wall = time.perf_counter() - te0
    h2d = 4 * sum(eng.trace_count(*mine[k % len(mine)]) for k in range(args.steps)) / args.steps + 4 * pf
    d2h = 4 * pf
    # max over ranks of the times, sum of the work
    (t_dev, t_e2e), (cells_all, shots_all, e2e_cells_all) = aggregate(
        [dev_ms / 1e3, e2e_wall], [cells_done, shots_done, e2e_cells], device=f"cuda:{local}")
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    adj_launch_ms = adj_ms / adj_launch
    cells_per_launch = adj_cells / adj_launch
    achieved = cells_per_launch * BYTES_ADJ / (adj_launch_ms * 1e-3) / 1e9
    tpc = profile_traffic()
    value = cells_all / t_dev / 1e9
    line = {
        "metric": "Gcell-updates/s",
        "value": round(value, 3),
        "unit": "Gcell/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * t_dev / args.steps, 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": c["desc"] + f"; one step = one group of {args.group} shots (forward + adjoint with "
                               "imaging); FP16 source snapshots",
                   "group_shots": args.group, "checkpoint_interval": st["checkpoint"],
                   "tile_staging": "tensor-memory-access bulk loads" if st["tma"] else "per-thread cp.async",
                   "inputs_vs_l2": "inputs larger than L2 (snapshots or checkpoints ~100+ GB)",
                   "forward_kernel": "marching strips (8-column chunks, 128 rows)" if st["march"] else "tiles",
                   "autotune_ms_per_launch_fwd_marching": round(tune["tune_ms_march"], 4),
                   "adjoint_kernel": "marching strips (8-column chunks, 128 rows)" if st["march_adj"] else "tiles",
                   "autotune_ms_per_launch_adj_marching": round(tune["tune_ms_march_adj"], 4),
                   "tile": {"forward_tx": tune["tile_x"], "adjoint_tx": tune["tile_x_adj"], "tz": 128,
                            "forward_stages": tune["stages"], "adjoint_stages": tune["stages_adj"],
                            "forward_threads": tune["threads"], "adjoint_threads": tune["threads_adj"],
                            "autotune_ms_per_launch_fwd_tx8_16_32_x_s1t256_s2t256_s1t512_s2t512":
                                [[round(x, 4) for x in r] for r in tune["tune_ms_fwd_variants"]],
                            "autotune_ms_per_launch_adj_tx8_16_32_x_s1t256_s2t256_s1t512_s2t512":
                                [[round(x, 4) for x in r] for r in tune["tune_ms_adj_variants"]]},
                   "shots_per_s": round(shots_all / t_dev, 3),
                   "wall_s": round(wall, 3),
                   "fwd_ms_per_step": round(fwd_ms / args.steps, 2),
                   "adj_ms_per_step": round(adj_ms / args.steps, 2)},
        "e2e": {"value": round(e2e_cells_all / t_e2e / 1e9, 3), "unit": "Gcell/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(kernels),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "kernel": ("k_adj_march" if st["march_adj"] else "k_step2d_v2") +
                               " adjoint + fused imaging (112 algorithmic B/cell)" +
                               (" (checkpoint-restart: the adjoint pass time includes the segment recompute)"
                                if st["checkpoint"] else ""),
                     "traffic": (round(tpc * cells_per_launch) if tpc else None)},
        "clocks": clocks,
    }
    line["_survey"] = (rho, lam, mu, x0, nxs, xsrc, zs, zr, widest, st["march"], st["march_adj"])
    eng.close()
    del traces_dev, img_dev
    torch.cuda.empty_cache()
    return line


# --------------------------------------------------------------- error block
def _fp64_shot(spec):
    """float64 RTM of one shot (oracle, ora_rtm_lowmem) for error_block."""
    nthreads, rho, lam, mu, D, kw = spec
    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O.rtm_lowmem(rho, lam, mu, D, **kw)


def error_block(survey, nt_err=600):
    """The headline path's error against the float64 oracle.

    The widest group of the survey is migrated by the batch engine on the
    kernels the autotuner chose (FP32 fields, FP16 source snapshots, Kahan
    imaging) over a truncated window of nt_err levels, from the Vx, Vz traces
    that the drop-in Born operator (rtm_op_c_, linear) models from the true
    model: the background times a dipping-reflector perturbation between
    rows 46 and 90 (synth.dipping_reflectivity: just below the 45-row sponge,
    so that its reflections reach the receivers within the window).  Every
    shot is migrated by the float64
    oracle (ora_rtm_lowmem: the reference's RTM algorithm in double
    precision) and stacked; the relative L2 error of each image is
    reported.  The full window (nt = 6000) would need 100 GB of float64
    history per shot in the oracle.  The oracle's shots run in parallel
    processes (spawned), their threads sharing the host cores."""
    import multiprocessing as mp
    from elastic_gb300 import rtm as R
    from elastic_gb300 import synth
    from elastic_gb300.batch import BatchRTM
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    c = CFG
    rho, lam, mu, x0, nxs, xsrc, zs, zr, widest, march_f, march_a = survey
    s0, k = widest
    sel = list(range(s0, s0 + k))
    nz, nx, dx, dt = c["nz"], c["nx"], c["dx"], c["dt"]
    refl = synth.dipping_reflectivity(nz, nx, seed=c["seed"], top=46, bottom=90)
    traces = []
    R.set_exact(False)
    try:
        for s in sel:
            a, w = int(x0[s] - 1), int(nxs[s])
            sl = lambda m: np.ascontiguousarray(m[a:a + w])
            op = R.RtmOperator(nz, dx, w, dx, dt, int(xsrc[s] - a), int(zs[s]), int(zr[s]), c["fp"], nt_err, c["abc"],
                               sl(rho), sl(lam), sl(mu), nsource=c["nsource"], linear=True)
            dm = [np.ascontiguousarray((refl[a:a + w] * m[a:a + w]).astype(np.float32)) for m in (rho, lam, mu)]
            D = [np.zeros((w, nt_err), np.float32) for _ in range(5)]
            op.rtm_op(False, *dm, *D)
            traces.append(D[:2])
    finally:
        R.set_exact(True)
    eng = BatchRTM(nz, nx, nt_err, dx, dt, c["fp"], c["abc"], rho, lam, mu, x0[sel], nxs[sel], xsrc[sel], zs[sel],
                   zr[sel], comp_mask=3, group_max=k, nsource=c["nsource"])
    eng.set_march((1 if march_f else 0) | (2 if march_a else 0))
    img = np.zeros(3 * nz * nx, np.float32)
    eng.migrate(0, k, np.concatenate([np.concatenate([t[0].ravel(), t[1].ravel()]) for t in traces]), img)
    eng.close()
    img = img.reshape(3, nx, nz)
    t0 = time.perf_counter()
    nthreads = max(1, (os.cpu_count() or 1) // len(sel))
    specs = []
    for j, s in enumerate(sel):
        a, w = int(x0[s] - 1), int(nxs[s])
        sl = lambda m: np.ascontiguousarray(m[a:a + w], np.float64)
        D = [traces[j][0].astype(np.float64), traces[j][1].astype(np.float64)] + [np.zeros((w, nt_err))] * 3
        kw = dict(dx=dx, dt=dt, nt=nt_err, zsrc=int(zs[s]), xsrc=int(xsrc[s] - a), zrec=int(zr[s]), fp=c["fp"],
                  abc=c["abc"], nsource=c["nsource"])
        specs.append((nthreads, sl(rho), sl(lam), sl(mu), D, kw))
    with mp.get_context("spawn").Pool(len(sel)) as pool:
        dms = pool.map(_fp64_shot, specs)
    ref = [np.zeros((nx, nz)) for _ in range(3)]
    for j, s in enumerate(sel):
        a, w = int(x0[s] - 1), int(nxs[s])
        for i in range(3):
            ref[i][a:a + w] += dms[j][i]
    oracle_s = time.perf_counter() - t0
    rel = [float(np.linalg.norm(img[i].astype(np.float64) - ref[i]) / np.linalg.norm(ref[i])) for i in range(3)]
    return {"drho": float("%.3g" % rel[0]), "dlambda": float("%.3g" % rel[1]), "dmu": float("%.3g" % rel[2]),
            "measure": "relative L2 of each stacked image against the float64 oracle",
            "window_nt": nt_err, "of_nt": c["nt"], "shots": [int(v) for v in nxs[sel]],
            "path": "batch engine as benchmarked: FP32 fields, FP16 per-level-scaled source snapshots, "
                    "Kahan-compensated imaging; %s forward, %s adjoint" % ("marching" if march_f else "tile",
                                                                           "marching" if march_a else "tile"),
            "traces": "Vx, Vz Born-modelled (linear, rtm_op_c_) from the background times a dipping-reflector "
                      "perturbation (seeded) between rows 46 and 90",
            "oracle": "ora_rtm_lowmem float64 (the reference's RTM algorithm), %d host threads, %.0f s"
                      % (os.cpu_count() or 1, oracle_s)}


# --------------------------------------------------------------- CPU arm
def _cpu_worker(spec):
    """One shot of the RTM (forward source wavefield, image_init, adjoint
    recursion, imaging) on its subgrid, truncated to nt levels.  kind
    "reference": the reference's own Fortran modules (executed through
    oracle/f90c.py) and its C recursion, exactly as its main program calls
    them; kind "port": the oracle's C restatement of the same code."""
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    nz, w, nt, seed, kind = spec
    c = CFG
    from elastic_gb300 import synth
    vp = synth.smooth_random_model(nz, w, c["dx"], 200.0, 1800.0, 4000.0, seed=seed)
    rho, lam, mu = synth.lame_from_vp(vp)
    rng = np.random.default_rng(seed)
    D = [(1e-3 * rng.standard_normal((w, nt))).astype(np.float32) for _ in range(5)]
    dm = [np.zeros((w, nz), np.float32) for _ in range(3)]
    t0 = time.perf_counter()
    if kind == "reference":
        O.ref90_rtm(True, rho, lam, mu, dm, D, c["dx"], c["dt"], nt, c["zsrc"], w // 2, c["zrec"], c["fp"], c["abc"])
    else:
        O.rtm_op2(True, rho, lam, mu, dm, D, np.float32(c["dx"]), np.float32(c["dt"]), nt, c["zsrc"], w // 2,
                  c["zrec"], np.float32(c["fp"]), c["abc"], c["nsource"])
    return time.perf_counter() - t0, 2 * nz * w * nt


def cpu_baseline(seconds_target=15.0):
    """The reference's RTM path on the host cores, one shot per core (as many
    as the memory of its full histories allows), over a truncated window of
    nt = 59 levels (the reference's C divides by nt/59 in its progress
    output, so 59 is its shortest window)."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=True)
    kind = "reference" if os.path.exists(O.REF90_PATH) else "port"
    nproc = os.cpu_count() or 1
    nz, w, nt = CFG["nz"], 1300, 59  # 1300: the mean subgrid width of the survey
    # full histories: 11 volumes of nz*w*nt (plus 5 padded copies in the reference's C)
    mem_gb = (16 if kind == "reference" else 11) * nz * w * nt * 4 / 1e9
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE") / 1e9
    except Exception:
        avail = 64.0
    procs = int(max(1, min(nproc, 0.5 * avail // max(mem_gb, 1e-3))))
    ctx = mp.get_context("spawn")
    res, rounds = [], 0
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        # rounds of one shot per process until the sample lasts seconds_target
        while rounds < 8 and (rounds == 0 or time.perf_counter() - t0 < seconds_target):
            res += pool.map(_cpu_worker, [(nz, w, nt, rounds * procs + s, kind) for s in range(procs)])
            rounds += 1
    wall = time.perf_counter() - t0
    total = sum(r[1] for r in res)
    what = ("the reference's own Fortran modules (executed through oracle/f90c.py) with its C recursion "
            "rtmlib-modC.c" if kind == "reference" else "the oracle's C restatement of the reference's Fortran and C")
    return {"value": round(total / wall / 1e9, 5), "unit": "Gcell/s", "cores": procs, "nproc": nproc, "kind": kind,
            "sample": f"{len(res)} shots ({rounds} rounds of one per process, {procs} processes, single-threaded as "
                      f"the reference) of the RTM "
                      f"(forward + adjoint + imaging, full histories) by {what}, on {nz}x{w} subgrids of the "
                      f"survey, nt window {nt} of {CFG['nt']} (per-level rate); {wall:.0f} s"}


def _ref_gpu_worker(which):
    """The adjoint recursion rtm_op3_c_ on the single-shot grid (200 x 400,
    nt = 2000) through `which`'s library: "reference" = the reference's
    rtmlib-modC.c with its own gpu.h (levels nt-3..nt-9 on the CPU, the rest
    by its CUDA kernel rtmlib-modC-gpu.cu, whole histories copied to the
    device and back); "ours" = libelastic_rtm.so's drop-in rtm_op3_c_ (exact
    arithmetic) and, on the reference's padded layout, its rtm_gpu_func.
    Returns wall seconds of the whole call and device seconds per level."""
    import ctypes
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from elastic_gb300 import synth
    nz, nx, nt = 200, 400, 2000
    (rho, lam, mu), _ = synth.single_shot_models(nz=nz, nx=nx)
    coefs = O.coefficients(rho, lam, mu, np.float32(10.0), np.float32(1e-3))
    rng = np.random.default_rng(1)
    H = [(1e-3 * rng.standard_normal((nt, nx, nz))).astype(np.float32) for _ in range(5)]
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    out = {}
    if which == "reference":
        lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "librefgpu.so"))
        err = tempfile.TemporaryFile(mode="w+b")
        saved = os.dup(2)
        os.dup2(err.fileno(), 2)
        try:
            t0 = time.perf_counter()
            lib.rtm_op3_c_(nt, nz, nx, 1, *[P(h) for h in H], *[P(c) for c in coefs])
            out["wall_s"] = time.perf_counter() - t0
        finally:
            os.dup2(saved, 2)
        err.seek(0)
        text = err.read().decode(errors="replace")
        for ln in text.splitlines():
            if ln.startswith("GPU time per step"):
                out["device_s_per_level"] = float(ln.split()[-1])
        out["levels_on_gpu"] = nt - 9
    else:
        from elastic_gb300 import rtm as R
        from elastic_gb300._lib import load
        R.set_exact(True)
        t0 = time.perf_counter()
        R.rtm_op3(nt, nz, nx, 1, *H, *coefs)
        out["wall_s"] = time.perf_counter() - t0
        # rtm_gpu_func on the reference's padded layout, levels nt-10..0
        pad = lambda a: np.pad(a, [(5, 5)] * a.ndim)
        Hp = [pad(h) for h in H]
        Cp = [pad(c) for c in coefs]
        lib = load()
        ps = np.zeros(1, np.float64)
        lib.rtm_gpu_init(nt, nz, nx)
        lib.rtm_gpu_func(nt - 10, nt, nz, nx, *[P(h) for h in Hp], *[P(c) for c in Cp], None, P(ps))
        lib.rtm_gpu_final()
        out["device_s_per_level"] = float(ps[0])
        out["levels_on_gpu"] = nt - 9
    return out


def ref_gpu_comparison():
    """The reference's CUDA adjoint and this library's, same machine, same
    grid; each in a process of its own."""
    import multiprocessing as mp
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "librefgpu.so")):
        return {"unavailable": "the reference's CUDA file was not built (its sources are absent)"}
    ctx = mp.get_context("spawn")
    res = {}
    for which in ("reference", "ours"):
        with ctx.Pool(1) as pool:
            res[which] = pool.apply(_ref_gpu_worker, (which,))
    cells = 200 * 400
    r, o = res["reference"], res["ours"]
    return {"workload": "adjoint recursion rtm_op3_c_ on the single-shot grid 200 x 400, nt = 2000, host "
                        "histories in and out",
            "reference_kernel": "rtmlib-modC-gpu.cu built unchanged for sm_103a (cudaThreadSynchronize mapped to "
                                "cudaDeviceSynchronize); 20x20 tiles, one launch and synchronisation per level",
            "reference_device_ms_per_level": round(1e3 * r.get("device_s_per_level", float("nan")), 4),
            "ours_device_ms_per_level": round(1e3 * o["device_s_per_level"], 4),
            "reference_gcells_per_level_device": round(cells / r.get("device_s_per_level", float("nan")) / 1e9, 3),
            "ours_gcells_per_level_device": round(cells / o["device_s_per_level"] / 1e9, 3),
            "reference_whole_call_s": round(r["wall_s"], 3), "ours_whole_call_s": round(o["wall_s"], 3),
            "note": "device time per level: the reference's own CUDA-event timing of its kernel loop and this "
                    "library's rtm_gpu_func on the same padded layout; whole call: rtm_op3_c_ wall time including "
                    "padding, host-device copies of all histories and the reference's CPU levels"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cb = cpu_baseline(args.cpu_seconds)
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": cb["value"], "unit": "Gcell/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched multi-shot 2D elastic RTM, 64-shot survey on a 2000x800 grid (CPU sample: "
                                   + cb["sample"] + ")"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_ref_gpu:
        try:
            line["reference_gpu"] = ref_gpu_comparison()
        except Exception as e:  # the comparator is informative; the CPU arm stands without it
            line["reference_gpu"] = {"unavailable": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- config 4
CFG4 = dict(n1=512, n2=1024, n3=1024, d=10.0, dt=1e-3, nt=3000, vmin=1500.0, vmax=4500.0, fp=20.0, damp_a=30,
            damp_b=0.005, zr=11, seed=4)
CFL_LIMIT_3D = 0.4419  # 2 / sqrt(3 * 6.8267): leapfrog limit of the 10th-order 3D Laplacian


K3D_NAMES = {"slab": "k_acoustic3d_s", "slab-paired": "k_acoustic3d_s", "ring": "k_acoustic3d_t",
             "pipelined": "k_acoustic3d_p"}


def acoustic3d_block(args, steps, warmup, nt=None, n3=None):
    """3D acoustic 10th-order forward modelling,
    1024 x 1024 x 512 cells, dx=10 m, dt=1 ms, 20 Hz Ricker point source,
    1024 x 1024 surface receivers (interior), 30-cell sponge.  One step = a
    window of nt/10 time steps from rest (10 steps = the full nt)."""
    import torch
    from elastic_gb300 import acoustic3d as A
    from elastic_gb300._lib import load
    c = dict(CFG4)
    if n3:
        c["n3"] = n3
    if nt:
        c["nt"] = nt
    n1, n2, n3 = c["n1"], c["n2"], c["n3"]
    dev = "cuda:0"
    g = torch.Generator(device=dev).manual_seed(c["seed"])
    w = torch.randn((n3 // 4, n2 // 4, n1 // 4), device=dev, generator=g)
    # smooth random field: low-pass in Fourier space, upsampled
    f = torch.fft.rfftn(w)
    k = [torch.fft.fftfreq(n, device=dev) for n in w.shape[:2]] + [torch.fft.rfftfreq(w.shape[2], device=dev)]
    kk = k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + k[2][None, None, :] ** 2
    sm = torch.fft.irfftn(f * torch.exp(-kk * 400.0), s=w.shape)
    sm = torch.nn.functional.interpolate(sm[None, None], size=(n3, n2, n1), mode="trilinear")[0, 0]
    sm = (sm - sm.min()) / (sm.max() - sm.min())
    # the configured range 1500-4500 m/s gives v dt/dx = 0.45 > the stability
    # limit 0.442 of this scheme at dt = 1 ms; the realised maximum is kept
    # at 4400 m/s (0.44) and reported
    vmax = min(c["vmax"], 0.995 * CFL_LIMIT_3D * c["d"] / c["dt"])
    vp = c["vmin"] + (vmax - c["vmin"]) * sm
    vel2 = ((vp * c["dt"] / c["d"]) ** 2).contiguous().float()
    del w, f, kk, sm, vp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from elastic_gb300 import rtm as R
    window = max(2, c["nt"] // 10)
    wav = R.source_op2(window, c["dt"], c["fp"], 50)
    src = (11, n2 // 2, n3 // 2)
    A.set_shape(args.tile3d, 0)
    A.set_kernel(args.kernel3d)
    for _ in range(warmup):
        A.forward(vel2, (c["d"],) * 3, c["damp_a"], c["damp_b"], src, wav[:8], c["zr"], on_device=True)
    torch.cuda.synchronize()
    cells = (n1 - 10) * (n2 - 10) * (n3 - 10)
    total_ms = 0.0
    with ClockSampler(0) as clk:
        for _ in range(steps):
            _, _, _, ms = A.forward(vel2, (c["d"],) * 3, c["damp_a"], c["damp_b"], src, wav, c["zr"], on_device=True)
            total_ms += ms
        torch.cuda.synchronize()
    clocks = clk.summary()
    # e2e: host velocity model in, host traces out, every step
    vel_h = vel2.cpu().numpy()
    te = time.perf_counter()
    A.forward(vel_h, (c["d"],) * 3, c["damp_a"], c["damp_b"], src, wav, c["zr"])
    e2e_s = time.perf_counter() - te
    del vel2
    torch.cuda.empty_cache()
    peak, kind = measured_peaks()
    rate = cells * window * steps / (total_ms * 1e-3) / 1e9
    line = {"metric": "Gcell-updates/s", "value": round(rate, 2), "unit": "Gcell/s", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": round(total_ms / steps, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"3D acoustic 10th-order forward modelling, {n1}x{n2}x{n3}, "
                                   f"one step = {window} time steps, receivers on plane z={c['zr']}",
                       "vmax_realised": round(float(vmax), 1), "cfl": round(float(vmax) * c["dt"] / c["d"], 4),
                       "cfl_limit": CFL_LIMIT_3D, "kernel": args.kernel3d,
                       "tile_x": args.tile3d if args.kernel3d == "pipelined" else 16,
                       "inputs_vs_l2": "inputs larger than L2"},
            "e2e": {"value": round(cells * window / e2e_s / 1e9, 2), "unit": "Gcell/s",
                    "h2d_bytes_per_step": 4 * n1 * n2 * n3, "d2h_bytes_per_step": 4 * window * n2 * n3 + 8 * n1 * n2 * n3},
            "gpu_launches": window * steps,
            "roofline": {"bound": "hbm", "achieved": round(rate * 16, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(rate * 16 / peak, 4), "peak_kind": kind,
                         "kernel": K3D_NAMES[args.kernel3d] + " (16 B/cell)",
                         "traffic": None},
            "clocks": clocks}
    return line


def run_acoustic3d(args):
    print(json.dumps(acoustic3d_block(args, args.steps, args.warmup, args.nt, args.n3)), flush=True)


# --------------------------------------------------------------- config 3
# The single-shot configuration's 40-cell sponge with source and receivers at
# 50 m puts the acquisition inside the sponge, where recorded reflections are
# damped by about 1e-3; the preconditioner study uses a 20-cell sponge with
# source and receivers just below it.
CFG3 = dict(nx=256, nz=256, nz_model=200, dx=10.0, dt=1e-3, nt=2000, fp=15.0, abc=20, nsource=250, zsrc=26, zrec=26,
            pairs=4096, ntest=4, batch=32, lr=1e-3, train_steps=3000, seed=3)


def unet_train_flops(table, batch):
    """Algorithmic FLOPs of one training step: forward, backward-data (all
    layers but the first) and backward-weights GEMMs of every convolution,
    2 * pixels * (ks^2 * cin) * cout each."""
    f = 0.0
    for i, (ks, ci, co, coutp, kp, woff, boff, H, W) in enumerate(table):
        one = 2.0 * batch * H * W * ks * ks * ci * co
        f += one * (3 if i else 2)
    return f


def precond_block(args, steps, warmup, pairs=None, train_steps=None, ntest=None, nt=None):
    """The learned preconditioner workload.  (Reflectivity,
    migrated image) pairs from the project's Born modelling and migration on
    256 x 256 windows of the smoothed single-shot background, U-Net training
    (Adam, batch 32) on the GPU; one step = one training step.  Then the
    learned migration (migration + network + least-squares scale) is timed
    against 10-iteration plain LSRTM at their Born data residuals."""
    import torch
    from elastic_gb300 import precond as PC
    from elastic_gb300 import unet as UN
    UN.set_gemm({"tma": "tcgen05_tma", "tc": "tcgen05", "mma": "mma_sync"}[args.gemm])
    c = dict(CFG3)
    if pairs:
        c["pairs"] = pairs
    if train_steps:
        c["train_steps"] = train_steps
    if ntest:
        c["ntest"] = ntest
    if nt:
        c["nt"] = nt
    rho, lam, mu = PC.background_window(c["nx"], c["nz"], nz_model=c["nz_model"])
    pb = PC.Problem(rho, lam, mu, c["dx"], c["dt"], c["nt"], c["nx"] // 2 + 1, c["zsrc"], c["zrec"], c["fp"], c["abc"],
                    c["nsource"])
    rng = np.random.default_rng(c["seed"])
    ntr, nte = c["pairs"], c["ntest"]
    t0 = time.perf_counter()
    r = PC.random_reflectivity(rng, ntr + nte, c["nx"], c["nz"], c["abc"] + 2)
    img = np.concatenate([pb.normal(r[i:min(ntr, i + 64)] * pb.bg[None]) for i in range(0, ntr, 64)])
    d_test, _ = pb.born_migrate(r[ntr:] * pb.bg[None])
    gen_s = time.perf_counter() - t0
    pc = PC.Preconditioner(c["nx"], c["nz"], batch=c["batch"], seed=0, margin=c["abc"] + 2)
    pc.fit_scales(img)
    x = torch.from_numpy(pc.inputs(img)).cuda()
    y = torch.from_numpy(PC.to_nhwc(r[:ntr] * pc.out_scale)).cuda()
    del img
    g = torch.Generator().manual_seed(c["seed"])

    def step():
        idx = torch.randint(0, ntr, (c["batch"],), generator=g).cuda()
        return pc.net.train_step(x.index_select(0, idx).contiguous(), y.index_select(0, idx).contiguous(), lr=c["lr"])

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        losses = [step() for _ in range(steps)]
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
    clocks = clk.summary()
    # rest of the training budget (untimed)
    t1 = time.perf_counter()
    for _ in range(max(0, c["train_steps"] - steps - warmup)):
        losses.append(step())
    rest_s = time.perf_counter() - t1
    # learned migration vs LSRTM-10 on held-out pairs
    res_nn, res_ls, res_rtm, t_nn, t_ls, refl_err = [], [], [], [], [], []
    for k in range(nte):
        t0 = time.perf_counter()
        im = pb.migrate(d_test[k:k + 1])
        m = pc.apply(im, pb.bg)
        res_nn.append(float(PC.scaled_residual(pb, m, d_test[k:k + 1])[0]))
        t_nn.append(time.perf_counter() - t0)
        rt = r[ntr + k]
        refl_err.append(float(np.linalg.norm(m[0] / pb.bg - rt) / np.linalg.norm(rt)))
        res_rtm.append(float(PC.scaled_residual(pb, im, d_test[k:k + 1])[0]))
        _, resid, tl = pb.lsrtm(d_test[k], 10)
        res_ls.append(float(resid[-1] / resid[0]))
        t_ls.append(tl)
    table = pc.net.layer_table()
    flops = unet_train_flops(table, c["batch"])
    tflops = flops * steps / train_s / 1e12
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, kind = (json.load(open(pk))["bf16_tflops"], "measured") if os.path.exists(pk) else (1900.0, "fallback")
    rate = c["batch"] * steps / train_s
    train_gb = x.numel() * 8 / 1e9
    del x, y
    torch.cuda.empty_cache()
    line = {"metric": "training images/s (learned preconditioner)", "value": round(rate, 2), "unit": "images/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": round(1e3 * train_s / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"learned preconditioner: 3->3 channel 4-level U-Net, "
                                   f"{pc.net.nparam} parameters, {c['nx']}x{c['nz']} patches, batch {c['batch']}, "
                                   f"Adam lr {c['lr']}; {ntr} training pairs (Born-modelled then migrated, one shot, "
                                   f"Vx/Vz receivers, nt={c['nt']})",
                       "pair_generation_s": round(gen_s, 1), "train_steps": len(losses) + warmup,
                       "training_s": round(train_s + rest_s, 1),
                       "input_normalisation": "per channel and depth row RMS over the imaging region, clipped to +-20",
                       "loss_first_last": [round(losses[0], 5), round(float(np.mean(losses[-50:])), 5)],
                       "inputs_vs_l2": "training set (%.1f GB) larger than L2" % train_gb},
            "time_to_residual": {"learned_residual": round(float(np.mean(res_nn)), 4),
                                 "lsrtm10_residual": round(float(np.mean(res_ls)), 4),
                                 "rtm_residual": round(float(np.mean(res_rtm)), 4),
                                 "learned_s": round(float(np.mean(t_nn)), 4), "lsrtm10_s": round(float(np.mean(t_ls)), 4),
                                 "lsrtm10_over_learned_time": round(float(np.mean(t_ls) / np.mean(t_nn)), 2),
                                 "held_out_pairs": nte,
                                 "learned_reflectivity_rel_err": round(float(np.mean(refl_err)), 4),
                                 "note": "residual = ||L m - d|| / ||d|| on Vx/Vz; learned = migration + network + "
                                         "least-squares scale (one Born); RTM with its best scale"},
            "e2e": {"value": round(rate, 2), "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8,
                    "note": "training batches are gathered on the device from the resident training set; the loss "
                            "is read back every step"},
            "gpu_launches": None,
            "roofline": {"bound": "tensor", "achieved": round(tflops, 2), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(tflops / peak, 4), "peak_kind": kind + " bf16 (cuBLAS burst)",
                         "kernel": {"tma": "k_conv_tc (tcgen05, bulk-copied convolution taps) + k_gemm_tc + k_gemm "
                                           "(mma.sync, backward-weights)",
                                    "tc": "k_gemm_tc (tcgen05, forward and backward-data) + k_gemm (mma.sync, "
                                          "backward-weights)",
                                    "mma": "k_gemm (mma.sync m16n8k16 BF16)"}[args.gemm]
                                   + " over the whole training step", "traffic": None},
            "clocks": clocks}
    return line


def run_precond(args):
    print(json.dumps(precond_block(args, args.steps, args.warmup, pairs=args.pairs, train_steps=args.train_steps,
                                   nt=args.nt)), flush=True)


def run_unet(args):
    """U-Net training step alone (the network of the precond workload: 256 x
    256 patches, batch 32, Adam) on seeded synthetic input/target patches
    resident in HBM: the kernel-level rate and roofline of the learned
    preconditioner's training, without pair generation."""
    import torch
    from elastic_gb300 import unet as UN
    UN.set_gemm({"tma": "tcgen05_tma", "tc": "tcgen05", "mma": "mma_sync"}[args.gemm])
    c = dict(CFG3)
    net = UN.UNet(c["nx"], c["nz"], c["batch"], seed=0)
    g = torch.Generator(device="cuda").manual_seed(c["seed"])
    nb = 8  # distinct batches cycled through (64 MB of inputs, larger than L2 with the activations)
    x = torch.randn((nb, c["batch"], c["nx"], c["nz"], 3), device="cuda", generator=g)
    y = 0.1 * torch.randn((nb, c["batch"], c["nx"], c["nz"], 3), device="cuda", generator=g)
    for i in range(args.warmup):
        net.train_step(x[i % nb], y[i % nb], lr=c["lr"])
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record()
        for i in range(args.steps):
            net.train_step(x[i % nb], y[i % nb], lr=c["lr"])
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    flops = unet_train_flops(net.layer_table(), c["batch"])
    peak, kind = measured_peaks("bf16_tflops")
    tf = flops / (ms * 1e-3) / 1e12
    print(json.dumps({"metric": "training images/s (learned preconditioner U-Net)", "value": round(c["batch"] / ms * 1e3, 2),
                      "unit": "images/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "bf16", "data": "synthetic",
                      "config": {"workload": f"U-Net training step, {c['nx']}x{c['nz']} patches, batch {c['batch']}, "
                                             f"Adam; seeded random inputs and targets", "gemm": args.gemm},
                      "roofline": {"bound": "tensor", "achieved": round(tf, 2), "peak": peak, "unit": "TFLOP/s",
                                   "frac": round(tf / peak, 4), "peak_kind": kind, "traffic": None},
                      "clocks": clk.summary()}), flush=True)


def elastic3d_block(args, steps, warmup, n=None):
    """One step of the reference's 3D elastic kernel test
    (kernel_3d_test/rtmlib-modC.c:277-590: nine fields, six coefficient
    planes, 10th-order staggered differences along z, x and y) on an n^3
    interior (padded by 5 on every side), seeded random planes resident in
    HBM; exact arithmetic (bit-identical to the reference's CPU step)."""
    import torch
    from elastic_gb300 import elastic3d as E
    E.set_kernel(args.k3_kernel)
    n = n or 384
    g = torch.Generator(device="cuda").manual_seed(11)
    shape = (n + 10, n + 10, n + 10)
    mk = lambda: (torch.rand(shape, device="cuda", generator=g) * 2 - 1).contiguous()
    inp, in1, out, m = [mk() for _ in range(9)], [mk() for _ in range(9)], [mk() for _ in range(9)], [mk() for _ in range(6)]
    for _ in range(warmup):
        E.step_dev(inp, in1, out, m, exact=True)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record()
        for _ in range(steps):
            E.step_dev(inp, in1, out, m, exact=True)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    cells = n ** 3
    rate = cells / (ms * 1e-3) / 1e9
    peak, kind = measured_peaks()
    # e2e: the reference-shaped drop-in (host planes in, step, nine out)
    h = [a.cpu().numpy() for a in inp + in1 + out + m]
    te = time.perf_counter()
    E.step(h[:9], h[9:18], h[18:27], h[27:], exact=True)
    e2e_s = time.perf_counter() - te
    del inp, in1, out, m
    torch.cuda.empty_cache()
    return {"metric": "Gcell-updates/s (3D elastic step)", "value": round(rate, 3), "unit": "Gcell/s", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"3D elastic kernel test step, {n}^3 interior (nine fields, six coefficients), "
                                   "exact arithmetic", "inputs_vs_l2": "inputs larger than L2",
                       "kernel": args.k3_kernel},
            "e2e": {"value": round(cells / e2e_s / 1e9, 3), "unit": "Gcell/s",
                    "h2d_bytes_per_step": 33 * 4 * (n + 10) ** 3, "d2h_bytes_per_step": 9 * 4 * (n + 10) ** 3},
            "gpu_launches": steps,
            "roofline": {"bound": "hbm", "achieved": round(rate * 168, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(rate * 168 / peak, 4), "peak_kind": kind,
                         "kernel": "k_k3_step (168 algorithmic B/cell: 33 planes read, 9 written)", "traffic": None},
            "clocks": clk.summary()}


def run_elastic3d(args):
    print(json.dumps(elastic3d_block(args, args.steps, args.warmup, args.n3)), flush=True)


# --------------------------------------------------------------- PML Born modelling
PML_BYTES = 332  # algorithmic bytes per cell and level: background 35 planes, scattered 48


def pml_block(args, steps=3, warmup=3, Tt=0.5, cpu_levels=60):
    """The reference's split-field PML Born modelling program
    (working_Src/born.f90: background and scattered wavefields, 20 split
    planes each, PML 60 cells wide, Ricker source, receiver lines, two
    snapshots) on the 2000 x 800 survey grid, dx = 10 m, Ttime = 0.5 s
    (nt = 707 levels); model resident in HBM, exact arithmetic (bit-identical
    to the reference's CPU execution).  A step is one whole modelling run."""
    import torch
    from elastic_gb300 import pml
    pml.set_kernel(args.pml_kernel)
    nz, nx, abc = 800, 2000, 60
    rng = np.random.default_rng(5)
    z = np.arange(nz)[None, :]
    vp = (np.where(z < nz // 3, 2000.0, np.where(z < 2 * nz // 3, 2600.0, 3200.0)) * np.ones((nx, 1))
          * (1 + 0.02 * rng.standard_normal((nx, nz)))).astype(np.float32)
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    dvp, dvs = (0.1 * vp).astype(np.float32), (0.1 * vs).astype(np.float32)
    drho = (rho * rng.uniform(0.01, 0.05, (nx, nz))).astype(np.float32)
    model = [vp, vs, rho, dvp, dvs, drho]
    P = pml.params(10.0, Tt, fp=25.0)
    nt, nseis, nsnap = P["nt"], P["nseis"], 2
    kw = dict(dx=10.0, dt=P["dt"], nt=nt, xsource=nx // 2, zsource=70, nsource=P["nsource"], fp=25.0, abc=abc,
              zrec=70)
    dev = [torch.from_numpy(a).cuda() for a in model]
    seis = [torch.empty((nx - 2 * abc, nseis), device="cuda") for _ in range(6)]
    snap = [torch.empty((nsnap, nx, nz), device="cuda") for _ in range(6)]
    for _ in range(warmup):
        pml.born_dev(dev, seis, snap, **kw)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record()
        for _ in range(steps):
            pml.born_dev(dev, seis, snap, **kw)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    launches = pml.launches()
    cells = nz * nx * nt
    rate = cells / (ms * 1e-3) / 1e9
    peak, kind = measured_peaks()
    # e2e: the host-array entry (copies in, run, copies out), one untimed
    # call first (its staging buffers are allocated on first use)
    pml.born(*model, nsnap=nsnap, nseis=nseis, **kw)
    te = time.perf_counter()
    pml.born(*model, nsnap=nsnap, nseis=nseis, **kw)
    e2e_s = time.perf_counter() - te
    del dev, seis, snap
    torch.cuda.empty_cache()
    out = {"metric": "Gcell-updates/s (PML Born modelling, background + scattered)", "value": round(rate, 3),
           "unit": "Gcell/s", "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": round(ms, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "split-field PML Born modelling, 2000 x 800 cells, 60-cell PML, nt = %d, "
                                  "2 snapshots, exact arithmetic" % nt, "inputs_vs_l2": "inputs larger than L2",
                      "kernel": args.pml_kernel},
           "e2e": {"value": round(cells / e2e_s / 1e9, 3), "unit": "Gcell/s",
                   "h2d_bytes_per_step": 6 * 4 * nz * nx,
                   "d2h_bytes_per_step": 4 * 6 * ((nx - 2 * abc) * nseis + nsnap * nz * nx)},
           "gpu_launches": steps * launches,
           "roofline": {"bound": "hbm", "achieved": round(rate * PML_BYTES, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(rate * PML_BYTES / peak, 4), "peak_kind": kind,
                        "kernel": "k_pml_step (332 algorithmic B per cell and level: background reads 25 planes "
                                  "and 5 coefficients, writes 10; scattered reads 28 planes and 10 coefficients, "
                                  "writes 10)", "traffic": None},
           "clocks": clk.summary()}
    if not args.no_cpu:
        out["cpu_baseline"] = pml_cpu_baseline(model, dict(kw, nt=cpu_levels, nsnap=1, nseis=nseis))
    return out


def _pml_cpu_worker(job):
    """One single-threaded run of the reference's PML Born program (its
    Fortran modules translated by oracle/f90c.py), or of the oracle's
    restatement when the reference's sources are absent; wall seconds."""
    model, kw, kind = job
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    (O.refpml_born if kind == "reference" else O.pml_born)(*model, **kw)
    return time.perf_counter() - t0


def pml_cpu_baseline(model, kw):
    """The reference's own PML Born program on the host cores: one
    single-threaded run of the first kw["nt"] levels on the same grid per
    process (the translation runs its OpenMP loops serially), as many
    processes as cores and memory allow."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=True)
    kind = "reference" if os.path.exists(O.REFPML_PATH) else "port"
    nx, nz = model[0].shape
    nproc = os.cpu_count() or 1
    mem_gb = 75 * nz * nx * 4 / 1e9  # 60 split planes, 10 coefficients, model and outputs
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE") / 1e9
    except Exception:
        avail = 64.0
    procs = int(max(1, min(nproc, 0.5 * avail // max(mem_gb, 1e-3))))
    env_threads = os.environ.get("OMP_NUM_THREADS")
    os.environ["OMP_NUM_THREADS"] = "1"  # the restatement's loops, if it stands in, run serially too
    try:
        ctx = mp.get_context("spawn")
        t0 = time.perf_counter()
        with ctx.Pool(procs) as pool:
            pool.map(_pml_cpu_worker, [(model, kw, kind)] * procs)
        wall = time.perf_counter() - t0
    finally:
        if env_threads is None:
            os.environ.pop("OMP_NUM_THREADS", None)
        else:
            os.environ["OMP_NUM_THREADS"] = env_threads
    what = ("the reference's own Fortran modules (working_Src/born-mod.f90 and the modules it uses, executed "
            "through oracle/f90c.py)" if kind == "reference" else "the oracle's restatement")
    return {"value": round(procs * nz * nx * kw["nt"] / wall / 1e9, 4), "unit": "Gcell/s", "cores": procs,
            "nproc": nproc, "kind": kind,
            "sample": "%d single-threaded runs in parallel of %s on the %d x %d grid, first %d levels (per-level "
                      "rate, process start-up included); %.0f s" % (procs, what, nz, nx, kw["nt"], wall)}


def run_pml(args):
    print(json.dumps(pml_block(args, steps=args.steps, warmup=args.warmup)), flush=True)


# --------------------------------------------------------------- config 5 sample
def c5_block(args, warmup=1, steps=1):
    """One 4-shot group of the 256-shot survey (6000 x 2000 cells, dx=5 m,
    dt=0.4 ms, nt=10000, subgrids 1000-6000 wide) migrated end to end in
    checkpoint-restart mode (all levels' FP16 snapshots would need ~1 TB), on
    the marching kernels; timed like the headline (device time of the group,
    forward and adjoint counted)."""
    import torch
    from elastic_gb300 import synth
    from elastic_gb300.batch import BatchRTM
    c = dict(CFG5)
    vp = synth.smooth_random_model(c["nz"], c["nx"], c["dx"], 200.0, 1800.0, 4000.0, seed=c["seed"])
    rho, lam, mu = synth.lame_from_vp(vp)
    x0, nxs, xsrc = synth.uneven_survey(c["nx"], c["nshots"], c["spacing"], c["wmin"], c["wmax"], seed=c["seed"])
    n = len(nxs)
    zs, zr = np.full(n, c["zsrc"], np.int32), np.full(n, c["zrec"], np.int32)
    eng = BatchRTM(c["nz"], c["nx"], c["nt"], c["dx"], c["dt"], c["fp"], c["abc"], rho, lam, mu, x0, nxs, xsrc, zs, zr,
                   comp_mask=c["comp_mask"], group_max=4, nsource=c["nsource"])
    eng.set_march(3)
    groups = eng.groups()
    # a group of mean width: the sample stands for the survey's average group
    mean_w = float(nxs.sum()) / len(groups)
    g = min(groups, key=lambda q: abs(int(nxs[q[0]:q[0] + q[1]].sum()) - mean_w))
    tmax = eng.trace_count(*g)
    traces = torch.from_numpy(synth.synthetic_traces(tmax, seed=c["seed"])).cuda()
    img = torch.zeros(3 * c["nz"] * c["nx"], dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        eng.migrate(g[0], g[1], traces, img, traces_on_device=True, image_on_device=True)
    torch.cuda.synchronize()
    dev_ms = fwd_ms = adj_ms = 0.0
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(steps):
            eng.migrate(g[0], g[1], traces, img, traces_on_device=True, image_on_device=True)
            st = eng.stats()
            dev_ms += st["total_ms"]
            fwd_ms += st["fwd_ms"]
            adj_ms += st["adj_ms"]
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    eng.close()
    del traces, img
    torch.cuda.empty_cache()
    cells = 2 * st["cells"] * c["nt"] * steps
    return {"metric": "Gcell-updates/s", "value": round(cells / (dev_ms * 1e-3) / 1e9, 3), "unit": "Gcell/s",
            "steps": steps, "warmup": warmup, "ms_per_step": round(dev_ms / steps, 1),
            "shots_per_s": round(g[1] * steps / (dev_ms * 1e-3), 4),
            "config": {"workload": c["desc"] + "; one step = one group of %d shots (widths %s)"
                                   % (g[1], [int(v) for v in nxs[g[0]:g[0] + g[1]]]),
                       "checkpoint_interval": st["checkpoint"],
                       "fwd_ms_per_step": round(fwd_ms / steps, 1), "adj_ms_per_step": round(adj_ms / steps, 1),
                       "note": "the adjoint pass includes the recomputation of each checkpoint segment (one more "
                               "forward propagation), not counted in the cell-updates",
                       "survey_estimate_s": round(dev_ms / steps * 1e-3 * len(groups), 1), "wall_s": round(wall, 2)},
            "clocks": clocks}


def run_default(args):
    """The headline (the 64-shot survey) and, at N=1, the blocks measured
    beside it in the same run."""
    line = run_gpu(args)
    if line is None:
        return
    survey = line.pop("_survey")
    if line["n_gpus"] == 1:
        if not args.no_error:
            line["error_vs_fp64"] = error_block(survey)
        if not args.no_secondary:
            sec = {}
            sec["acoustic3d"] = acoustic3d_block(args, steps=3, warmup=3)
            sec["elastic3d"] = elastic3d_block(args, steps=10, warmup=3, n=384)
            sec["pml_born"] = pml_block(args)
            sec["rtm2d_256shot_group"] = c5_block(args)
            sec["precond"] = precond_block(args, steps=100, warmup=5, pairs=args.sec_pairs,
                                           train_steps=args.sec_train_steps, ntest=2)
            sec["precond"]["config"]["reduced"] = (
                "bounded sample: %d training pairs (of 4096) and %d Adam steps (of 3000), %d held-out pairs"
                % (args.sec_pairs, args.sec_train_steps, 2))
            line["secondary"] = sec
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--group", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--tune-steps", type=int, default=20)
    ap.add_argument("--workload", default="rtm2d", choices=["rtm2d", "rtm2d_c5", "acoustic3d", "precond", "unet", "elastic3d", "pml"])
    ap.add_argument("--pairs", type=int, default=None, help="training pairs of the precond workload")
    ap.add_argument("--train-steps", type=int, default=None, help="Adam steps of the precond workload")
    ap.add_argument("--staging", default="tma", choices=["cpasync", "tma"], help="step-kernel tile staging")
    ap.add_argument("--n3", type=int, default=None, help="override n3 of the 3D workload (profiling only)")
    ap.add_argument("--tile3d", type=int, default=16)
    ap.add_argument("--kernel3d", default="slab", choices=list(K3D_NAMES), help="3D step kernel")
    ap.add_argument("--gemm", default="tma", choices=["tma", "tc", "mma"],
                    help="U-Net GEMMs of the forward and backward-data passes: tcgen05 with bulk-copied "
                         "convolution taps, tcgen05 with thread-gathered operands, or mma.sync")
    ap.add_argument("--k3-kernel", default="paired-bound",
                    choices=["cell", "paired", "paired-prefetch", "paired-bound", "paired-prefetch-bound"],
                    help="3D elastic step kernel form")
    ap.add_argument("--pml-kernel", default="cell-prefetch-b6",
                    choices=["rows4", "cell", "rows4-prefetch", "cell-prefetch", "tile", "tile-prefetch",
                             "cell-prefetch-b5", "cell-prefetch-b6", "cell-prefetch-b8", "fused"],
                    help="PML Born step kernel form")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-error", action="store_true", help="skip the float64 error block")
    ap.add_argument("--no-secondary", action="store_true", help="skip the secondary workload blocks")
    ap.add_argument("--no-ref-gpu", action="store_true", help="reference arm: skip the reference CUDA comparator")
    ap.add_argument("--sec-pairs", type=int, default=1024, help="training pairs of the secondary precond block")
    ap.add_argument("--sec-train-steps", type=int, default=2000, help="Adam steps of the secondary precond block")
    ap.add_argument("--nt", type=int, default=None, help="override nt (profiling captures only)")
    ap.add_argument("--shots", type=int, default=None, help="override the shot count (profiling captures only)")
    args = ap.parse_args()
    if args.workload == "rtm2d_c5":
        CFG.update(CFG5)
    if args.nt:
        CFG["nt"] = args.nt
    if args.shots:
        CFG["nshots"] = args.shots
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "acoustic3d":
        run_acoustic3d(args)
    elif args.workload == "unet":
        run_unet(args)
    elif args.workload == "elastic3d":
        run_elastic3d(args)
    elif args.workload == "pml":
        run_pml(args)
    elif args.workload == "precond":
        run_precond(args)
    elif args.workload == "rtm2d":
        run_default(args)
    else:
        line = run_gpu(args)
        if line is not None:
            line.pop("_survey")
            print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
