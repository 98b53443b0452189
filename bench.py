#!/usr/bin/env python
"""Benchmark: time-steps/s of the droplet projection hot path at 256^3.

Workload: the splash-on-wall case, 256^3 interior cells (258^3 nodes), 3 m/s
impact, pressure solved to 1e-8 relative residual, laminar: the reference's
explicit k-epsilon update (main.f:1888-2026) overflows on this drop by its third
step, so the k-epsilon variant of the case has no finite state to time.  A
"step" is one body of the main.f time loop (VOF advection, CFL check, CSF force,
momentum + pressure projection) with every field resident in HBM.  The
headline solve is FP64 defect correction around FP32 V-cycles (FP32 full
multigrid start, V(3,3) on the finest level and V(8,8) below, omega 1.5,
trilinear prolongation); the plain FP64 multigrid (the reference's FMG with
V(4,4), then FP64 V-cycles to the same tolerance) is timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  With N>1 (torchrun) every rank advances its own
independent droplet replica (weak scaling, no collective on the data path).
``--impl reference`` times the CPU reference restatement (the oracle: plain
FP64 multigrid to the same tolerance, single thread, as the reference is
serial) on the same workload and step window: W untimed warm-up steps from the
initial condition, then steps W+1 ... W+k.
"""
import argparse
import importlib
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "3d_droplet_simulation_2007_gb300"

METRIC = "time-steps/s at 256^3, plain FP64 MG vs FP32-refined+learned warm-start, 1e-8 resid"
UNIT = "time-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256, help="interior cells per side")
    ap.add_argument("--mode", default="best", help="best|tol_fp64|tol_mixed|learned|ref_exact")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--inner", type=int, default=0,
                    help="FP32 V-cycles per FP64 defect (mixed modes; 0: adaptive)")
    ap.add_argument("--no-graphs", action="store_true", help="launch the mixed solve without CUDA graphs")
    ap.add_argument("--start", type=int, default=None,
                    help="initial guess of the mixed solve: 0 FMG, 1 previous pressure, 2 zero (default: config)")
    ap.add_argument("--sweeps32", type=str, default=None,
                    help="pre,post sweeps of the FP32 V-cycles (default: the configuration's)")
    ap.add_argument("--omega32", type=float, default=None,
                    help="relaxation factor of the FP32 V-cycles (default: the library configuration's)")
    ap.add_argument("--prolong32", type=int, default=None,
                    help="FP32 prolongation: 0 trilinear, 1 injection (default: the library configuration's)")
    ap.add_argument("--fmg32", type=int, default=None,
                    help="V-cycles per level of the FP32 FMG start (default: the library configuration's)")
    ap.add_argument("--fine-sweeps32", type=str, default=None,
                    help="pre,post sweeps of the FP32 V-cycles on the finest level (default: as on the others)")
    ap.add_argument("--small-sweeps32", type=str, default=None,
                    help="pre,post sweeps of the FP32 V-cycles on the levels of at most 18^3 nodes")
    ap.add_argument("--mid-sweeps32", type=str, default=None,
                    help="pre,post sweeps of the FP32 V-cycles on the level below the finest")
    ap.add_argument("--krylov", type=int, default=None,
                    help="mixed modes: 1 GCR over the FP32 V-cycle, 0 V-cycles alone (default: the configuration's)")
    ap.add_argument("--fmg32-fine", type=int, default=None,
                    help="V-cycles of the FP32 FMG start on the finest level (default: as on the others)")
    ap.add_argument("--tail-nodes", type=int, default=0,
                    help="largest FP32 level (nodes) of the single-block coarse tail (0: default, -1: off)")
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 reference point")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned warm-start point")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the 16-member ensemble point recorded beside the headline")
    ap.add_argument("--ensemble", type=int, default=0,
                    help="time the droplet-study ensemble of this many members instead (48-160^3 grids)")
    ap.add_argument("--workers", type=int, default=0, help="ensemble host threads (0: autotune)")
    ap.add_argument("--no-batched", action="store_true",
                    help="ensemble: skip the batched-solve point (a launch per multigrid pass over a group of "
                         "members, CUDA graphs, autotuned tiles)")
    ap.add_argument("--groups", type=int, default=0,
                    help="batched ensemble: cost-balanced groups solved side by side (0: the fastest of 1, 2, 4, 8)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(dsg, n, mode, tol, inner=0, graphs=True, tail_nodes=0, omega32=None, start=None, sweeps32=None,
             prolong32=None, fmg32=None, fine_sweeps32=None, mid_sweeps32=None, small_sweeps32=None, krylov=None,
             fmg32_fine=None):
    cfg = dsg.config
    inp = cfg.droplet(n, steps=1000, impact_speed=3.0, noise_si=1e-4, mode=mode, tol=tol,
                      npre=4, npost=4, ntop=4).replace(inner_vcycles=inner, use_graphs=1 if graphs else 0,
                                                       tail_nodes=tail_nodes)
    inp = inp if omega32 is None else inp.replace(mg32_omega=omega32)
    inp = inp if start is None else inp.replace(warm_start=start)
    inp = inp if prolong32 is None else inp.replace(mg32_prolong=prolong32)
    inp = inp if fmg32 is None else inp.replace(mg32_fmg_cycles=fmg32)
    inp = inp if krylov is None else inp.replace(mg32_krylov=krylov)
    inp = inp if fmg32_fine is None else inp.replace(mg32_fmg_fine_cycles=fmg32_fine)
    if small_sweeps32:
        a, b = (int(x) for x in small_sweeps32.split(","))
        inp = inp.replace(mg32_small_npre=a, mg32_small_npost=b)
    if mid_sweeps32:
        a, b = (int(x) for x in mid_sweeps32.split(","))
        inp = inp.replace(mg32_mid_npre=a, mg32_mid_npost=b)
    if fine_sweeps32:
        a, b = (int(x) for x in fine_sweeps32.split(","))
        inp = inp.replace(mg32_fine_npre=a, mg32_fine_npost=b)
    if sweeps32:
        a, b = (int(x) for x in sweeps32.split(","))
        inp = inp.replace(mg32_npre=a, mg32_npost=b)
    return inp


def schedule(inp, mode, dsg):
    """The pressure solve the line measured, in words."""
    m = dsg.config.MODE_NAMES
    if mode in (m["tol_mixed"], m["learned"]):
        fine = (inp.mg32_fine_npre or inp.mg32_npre, inp.mg32_fine_npost or inp.mg32_npost)
        fmg = "FP32 full multigrid (%d V-cycle(s) per level below the finest, %d on the finest)" % (
            inp.mg32_fmg_cycles or inp.cycles, inp.mg32_fmg_fine_cycles or inp.mg32_fmg_cycles or inp.cycles)
        start = fmg + " with the guarded learned correction" if mode == m["learned"] else \
            {0: fmg, 1: "previous-step pressure", 2: "zero"}[inp.warm_start]
        return ("FP64 defect correction (FP64 residual, correction and projection) around FP32 V-cycles%s: "
                "%s start, V(%d,%d) on the finest level and V(%d,%d) below, omega %.2f, %s prolongation, "
                "red-black Gauss-Seidel, to %.0e relative residual"
                % (" preconditioning GCR steps" if inp.mg32_krylov else "", start, fine[0], fine[1],
                   inp.mg32_npre, inp.mg32_npost, inp.mg32_omega,
                   "trilinear" if inp.mg32_prolong == 0 else "piecewise-constant", inp.tol))
    if mode == m["ref_exact"]:
        return "the reference's FP64 FMG (fixed cycles, V(%d,%d), omega %.2f), no residual test" % (
            inp.npre, inp.npost, inp.omega)
    return ("plain FP64: the reference's FMG, V(%d,%d), omega %.2f, then FP64 V-cycles to %.0e relative residual"
            % (inp.npre, inp.npost, inp.omega, inp.tol))


def dtype_of(mode, dsg):
    m = dsg.config.MODE_NAMES
    return "f32+f64" if mode in (m["tol_mixed"], m["learned"]) else "f64"


LAMINAR = ("laminar: with k-epsilon on, the reference's explicit k-epsilon update (main.f:1888-2026) "
           "overflows on the drop by its third step, so that variant has no finite state to time")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def committed_traffic(kernel, n):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    e = d.get("%s@%d" % (kernel, n))
    return None if e is None else e.get("dram_bytes_per_launch")


class Clocks:
    """nvidia-smi sampler over the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler is producing samples
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for ln in f:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) >= 8:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = sorted(float(r[0]) for r in rows if r[0].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": float(rows[0][1]) if rows[0][1].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def host_cpu():
    """CPU model and logical core count of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read()
        m = re.search(r"^model name\s*:\s*(.+)$", info, re.M)
        if m:
            model = m.group(1).strip()
        else:
            imp = re.search(r"^CPU implementer\s*:\s*(\S+)$", info, re.M)
            part = re.search(r"^CPU part\s*:\s*(\S+)$", info, re.M)
            if imp and part:
                model = "arm implementer %s part %s" % (imp.group(1), part.group(1))
    except OSError:
        pass
    return {"model": model or platform.machine(), "nproc": os.cpu_count()}


STATE = ["cc", "p", "res", "rhs", "a", "b", "c", "ei", "u", "v", "w",
         "s11", "s22", "s33", "s12", "s13", "s23", "rhon", "mun"]
STATE_SCALARS = ("tau", "tauh", "time", "tauh2", "tswap", "npre", "npost", "ntop")


def oracle_from_solver(dsg, solver, tol):
    """A plain FP64 oracle (tol mode) holding the solver's current state."""
    from oracle import Oracle
    ora = Oracle(solver.inp.replace(mode=dsg.config.MODE_TOL_FP64, tol=tol).as_dict())
    for f in STATE:
        solver.download_into(f, ora.field(f).reshape(-1, order="F"))
    so, sg = ora.scalars(), solver.scalars()
    for k in STATE_SCALARS:
        setattr(so, k, getattr(sg, k))
    ora.set_scalars(so)
    return ora


def field_errors(get, ora):
    """max|x - oracle| / max|oracle| per field, and the liquid volume's
    relative difference."""
    import numpy as np
    out = {}
    for f in ("p", "u", "v", "w", "cc"):
        o = ora.field(f)
        g = get(f)
        scale = float(np.max(np.abs(o)))
        out[f] = float(np.max(np.abs(g - o))) / (scale if scale > 0 else 1.0)
    return out


def run_reference(args):
    """The reference arm: the oracle (plain FP64 multigrid to tol, one
    thread) on the same workload and step window as the GPU arm."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    dsg = importlib.import_module(PKG)
    from oracle import Oracle
    inp = workload(dsg, args.n, dsg.config.MODE_TOL_FP64, args.tol)
    ora = Oracle(inp.as_dict())
    w0 = time.perf_counter()
    for t in range(1, args.warmup + 1):
        ora.step(t)
    warm_s = time.perf_counter() - w0
    # at most 3 timed steps (about 15 s each on one core at 256^3)
    k = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for t in range(args.warmup + 1, args.warmup + k + 1):
        ora.step(t)
    dt = time.perf_counter() - t0
    value = k / dt
    cb = {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "host": host_cpu(),
          "sample": "time steps %d-%d of the %d^3 workload (after %d untimed warm-up steps, %.0f s), C oracle "
                    "(plain FP64 FMG + V-cycles to %.0e), 1 thread (the reference is serial), %.1f s"
                    % (args.warmup + 1, args.warmup + k, args.n, args.warmup, warm_s, args.tol, dt)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
            "steps_requested": args.steps, "warmup": args.warmup, "window": [args.warmup + 1, args.warmup + k],
            "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "splash-on-wall droplet %d^3 cells (%d^3 nodes), 3 m/s, %s"
                                   % (args.n, args.n + 2, LAMINAR),
                       "solver": schedule(inp, dsg.config.MODE_TOL_FP64, dsg)},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def relax_roofline(prof, step_ms, n):
    """Roofline entry of the finest-level relax from the live CUDA-event
    profile: algorithmic bytes per call / mean call time against the measured
    HBM copy bandwidth."""
    peak, peak_kind = measured_peaks()
    achieved = None
    if prof["relax_calls"]:
        per_call_ms = prof["relax_ms"] / prof["relax_calls"]
        per_call_bytes = prof["relax_bytes"] / prof["relax_calls"]
        achieved = per_call_bytes / (per_call_ms / 1e3) / 1e9
    split = prof.get("relax_bits") == 32
    kname = "k_relax32_split" if split else "k_relax_colour"
    return {"bound": "hbm",
            "kernel": ("%s: finest-level relax, colour-split FP32 red-black sweep, 2 launches per relax "
                       "(other colour, own colour r+w, own rhs, cc: 24 B/cell)" % kname if split
                       else "%s: finest-level relax, 2 red-black FP64 colour passes (u r+w, a, b, c, rhs: "
                            "48 B/cell)" % kname),
            "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": committed_traffic(kname, n),
            "peak_kind": peak_kind,
            "bytes_per_launch": (prof["relax_bytes"] / prof["relax_calls"]) if prof["relax_calls"] else None,
            "relax_calls": prof["relax_calls"],
            "share_of_step": (prof["relax_ms"] / step_ms) if step_ms else None}


def mode_of(dsg, name):
    names = dsg.config.MODE_NAMES
    if name == "best":
        return names["tol_mixed"]
    return names[name]


def time_steps(torch, solver, k, t0):
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    stats = []
    for t in range(t0, t0 + k):
        stats.append(solver.step(t))
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1), stats


def max_over_ranks(x, dist, device=None):
    """The largest value of x over all ranks (x itself without a process group)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gb300(args):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    # one dedicated stream for the library and the timing events
    torch.cuda.set_stream(torch.cuda.Stream())
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dsg = importlib.import_module(PKG)
    dsg.load()
    mode = mode_of(dsg, args.mode)
    inp = workload(dsg, args.n, mode, args.tol, args.inner, not args.no_graphs, args.tail_nodes, args.omega32,
                   args.start, args.sweeps32, args.prolong32, args.fmg32, args.fine_sweeps32,
                   args.mid_sweeps32, args.small_sweeps32, args.krylov, args.fmg32_fine)
    solver = dsg.Solver(inp)
    solver.set_stream(torch.cuda.current_stream().cuda_stream)
    for t in range(1, args.warmup + 1):
        solver.step(t)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    solver.profile_enable(True)
    ms, stats = time_steps(torch, solver, args.steps, args.warmup + 1)
    prof = solver.profile_read()
    solver.profile_enable(False)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms_max = max_over_ranks(ms, dist, "cuda")
    value = ws * args.steps / (ms_max / 1e3)
    vcycles = [s["vcycles"] for s in stats]

    # plain FP64 reference point of the metric (same replica, continued)
    plain = None
    if mode != dsg.config.MODE_TOL_FP64 and not args.no_plain:
        p_inp = workload(dsg, args.n, dsg.config.MODE_TOL_FP64, args.tol)
        ps = dsg.Solver(p_inp)
        ps.set_stream(torch.cuda.current_stream().cuda_stream)
        for t in range(1, args.warmup + 1):
            ps.step(t)
        ps.profile_enable(True)
        pms, pst = time_steps(torch, ps, args.steps, args.warmup + 1)
        pprof = ps.profile_read()
        ps.profile_enable(False)
        plain = {"value": args.steps / (pms / 1e3), "ms_per_step": pms / args.steps,
                 "vcycles": [s["vcycles"] for s in pst], "solver": schedule(p_inp, p_inp.mode, dsg),
                 "roofline": relax_roofline(pprof, pms, args.n)}
        ps.close()

    # the learned warm start (committed weights), same workload, as a measured
    # secondary point: the headline uses the faster FMG start
    learned = None
    if not args.no_learned and mode == dsg.config.MODE_TOL_MIXED:
        lmod = importlib.import_module(PKG + ".learned")
        if os.path.exists(lmod.WEIGHTS):
            net = lmod.Net(args.n).load()
            ls = dsg.Solver(inp.replace(mode=dsg.config.MODE_LEARNED))
            ls.set_stream(torch.cuda.current_stream().cuda_stream)
            net.attach(ls)
            for t in range(1, args.warmup + 1):
                ls.step(t)
            lms, lst = time_steps(torch, ls, args.steps, args.warmup + 1)
            ran = [s for s in lst if s["relres_net"] >= 0.0]
            learned = {"value": args.steps / (lms / 1e3), "vcycles": [s["vcycles"] for s in lst],
                       "network_runs": len(ran), "kept": sum(1 - s["fallback"] for s in ran),
                       "defect_ratio_median": (float(np.median([s["relres_net"] / s["relres_base"] for s in ran]))
                                               if ran else None),
                       "relres_fmg_median": float(np.median([s["relres_base"] for s in lst])),
                       "guard": "network correction of the FP32 FMG start, scaled to the least FP64 defect, kept "
                                "only if it cuts the expected V-cycles; after a rejection the network rests "
                                "1, 2, 4 .. 32 steps"}
            lmod.detach(ls)
            ls.close()
            net.close()

    # error against the FP64 oracle from one shared state: the state after
    # the timed steps goes into the oracle (plain FP64 to the same tolerance)
    # and into a plain FP64 GPU solver; one more step of each, and of the
    # headline solver, is compared field by field.  The oracle step is also
    # the CPU baseline: one step of the same workload in the same window.
    t_next = args.warmup + args.steps + 1
    cb, err = None, None
    if ws == 1 and rank == 0 and not args.no_cpu_baseline:
        ora = oracle_from_solver(dsg, solver, args.tol)
        p2 = None
        if mode != dsg.config.MODE_TOL_FP64:
            p2 = dsg.Solver(inp.replace(mode=dsg.config.MODE_TOL_FP64), init=False)
            p2.set_stream(torch.cuda.current_stream().cuda_stream)
            for f in STATE:
                p2.upload(f, ora.field(f))
            p2.set_scalars(solver.scalars())
        c0 = time.perf_counter()
        ora.step(t_next)
        cdt = time.perf_counter() - c0
        cb = {"value": 1.0 / cdt, "unit": UNIT, "cores": 1, "kind": "port", "host": host_cpu(),
              "sample": "time step %d of the %d^3 workload from the GPU state after the timed steps, C oracle "
                        "(plain FP64 FMG + V-cycles to %.0e), 1 thread (the reference is serial), %.1f s"
                        % (t_next, args.n, args.tol, cdt)}
        st_h = solver.step(t_next)
        vo = ora.liquid_volume()
        err = {"step": t_next, "state": "GPU state after the timed steps, loaded into both",
               "norm": "max|x - oracle| / max|oracle| over the whole field",
               "oracle": "C oracle, plain FP64 multigrid to %.0e" % args.tol,
               "oracle_relres": ora.scalars().last_relres,
               "headline": field_errors(solver.field, ora)}
        err["headline"]["volume"] = abs(solver.liquid_volume() - vo) / abs(vo)
        err["headline"]["relres"] = st_h["relres"]
        if p2 is not None:
            st_p = p2.step(t_next)
            err["plain_fp64"] = field_errors(p2.field, ora)
            err["plain_fp64"]["volume"] = abs(p2.liquid_volume() - vo) / abs(vo)
            err["plain_fp64"]["relres"] = st_p["relres"]
            p2.close()
        ora.close()
        t_next += 1

    # end to end through the public API: pinned host state in, results out,
    # every step through dsg_step_host (the copies overlap the step's phases)
    e2e = None
    if not args.no_e2e:
        n_cells = inp.nx * inp.ny * inp.nz
        ins = ["cc", "u", "v", "w", "s12", "s13", "s23"]
        outs = ["p", "cc", "u", "v", "w"]
        host = {}
        for nm in set(ins + outs):
            host[nm] = torch.empty(n_cells, dtype=torch.float64, pin_memory=True).numpy()
        for nm in ins:
            solver.download_into(nm, host[nm])
        k2 = max(1, args.e2e_steps)
        torch.cuda.synchronize()
        t_start = time.perf_counter()
        t = t_next - 1
        for _ in range(k2):
            t += 1
            solver.step_host({nm: host[nm] for nm in ins}, {nm: host[nm] for nm in outs}, t)
        torch.cuda.synchronize()
        el = time.perf_counter() - t_start
        e2e = {"value": ws * k2 / el, "unit": UNIT, "h2d_bytes_per_step": len(ins) * n_cells * 8,
               "d2h_bytes_per_step": len(outs) * n_cells * 8}
    solver.close()

    # a bounded droplet-study ensemble on the same GPU, recorded beside the
    # headline (the full study is `bench.py --ensemble 64`)
    ens = None
    if not args.no_ensemble and ws == 1:
        n_ens, k_ens = 16, 4
        cfgs = dsg.ensemble.study_configs(n_ens, tol=args.tol)
        m = measure_ensemble(dsg, dsg.load(), cfgs, k_ens, 2, 0, [4])
        ens = {"value": n_ens * k_ens / m["el"], "unit": "member-steps/s", "members": n_ens, "steps": k_ens,
               "workload": "%d droplets on wall, interior sides 48-160, Weber 50-800, mixed pressure to %.0e"
                           % (n_ens, args.tol),
               "cells_per_step": sum((c.nx - 2) * (c.ny - 2) * (c.nz - 2) for c in cfgs),
               "workers": m["workers"], "ms_per_step": 1e3 * m["el"] / k_ens,
               "timing": "host clock between synchronisations of all member streams",
               "clocks": m["clocks"], "batched": batched_entry(n_ens, k_ens, m["batched"])}

    if rank == 0:
        roof = relax_roofline(prof, ms, args.n)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "window": [args.warmup + 1, args.warmup + args.steps],
                "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": dtype_of(mode, dsg), "data": "synthetic",
                "config": {"workload": "splash-on-wall droplet %d^3 cells (%d^3 nodes), 3 m/s, %s"
                                       % (args.n, args.n + 2, LAMINAR),
                           "solver": schedule(inp, mode, dsg),
                           "mode": [k for k, v in dsg.config.MODE_NAMES.items() if v == mode][0],
                           "l2": "inputs larger than L2: per-step working set %.1f GB >> 129 MB L2, no flush"
                                 % (solver_bytes_estimate(inp) / 1e9),
                           "parallelism": "replicas" if ws > 1 else "single"},
                "vcycles_per_step": vcycles, "gpu_launches": prof["launches"], "roofline": roof,
                "phase_ms_per_step": {k: v / args.steps for k, v in prof["phase_ms"].items()},
                "cpu_baseline": cb, "e2e": e2e, "clocks": clk, "error_vs_fp64": err}
        if plain:
            line["plain_fp64"] = plain
        if learned:
            line["learned_warm_start"] = learned
        if ens:
            line["ensemble"] = ens
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def measure_ensemble(dsg, lib, cfgs, steps, warmup, workers, group_cands, dist=None):
    """Time the members `cfgs` (this rank's share) as an ensemble: the worker
    pool (worker count autotuned when `workers` <= 0), then, if
    `group_cands` is not empty, the batched pressure solve with the fastest
    group count among them (tail depth and tile shapes autotuned).  The
    timed region is bracketed by a synchronisation of every member's stream
    and measured with the host clock (the work spans many streams)."""
    with dsg.Ensemble(cfgs, workers=max(workers, 1)) as e:
        tuned = e.autotune(steps_per_trial=2) if workers <= 0 else None
        for _ in range(warmup):
            e.step()

        def timed(k):
            for i in range(e.n):
                e.member(i).synchronize()
            if dist:
                dist.barrier()
            l0 = lib.dsg_launch_count()
            t0 = time.perf_counter()
            stats = [e.step() for _ in range(k)]
            for i in range(e.n):
                e.member(i).synchronize()
            el = time.perf_counter() - t0
            if dist:
                dist.barrier()
            return el, lib.dsg_launch_count() - l0, stats

        clocks = Clocks(torch_device_index())
        clocks.start()
        el, launches, stats = timed(steps)
        clk = clocks.stop()
        out = {"el": el, "launches": launches, "stats": stats, "workers": e.workers, "tuned": tuned is not None,
               "clocks": clk, "n": e.n}
        # the batched pressure solve, same members and workers, after the
        # timed steps: the fastest group count, coarse-tail depth and tile
        # shapes autotuned, then timed the same way
        if group_cands:
            group_ms = {}
            for g in group_cands:
                e.set_batched(g)
                e.autotune_tiles(reps=3)
                e.step()
                t0 = time.perf_counter()
                e.step()
                e.step()
                group_ms[g] = 1e3 * (time.perf_counter() - t0) / 2
            groups = min(group_ms, key=group_ms.get)
            e.set_batched(groups)
            tiles = e.autotune_tiles(reps=3)
            e.step()
            bel, blaunch, _ = timed(steps)
            out["batched"] = {"el": bel, "groups": groups, "tiles": tiles, "tail_nodes": e.batch_tail_nodes,
                              "launches": blaunch, "group_ms": {k: round(v, 1) for k, v in group_ms.items()}}
            e.set_batched(0)
        e.set_workers(1)
        out["el1"], _, _ = timed(1)
    return out


def torch_device_index():
    import torch
    return torch.cuda.current_device()


def batched_entry(n_members, steps, b):
    return {"value": n_members * steps / b["el"], "unit": "member-steps/s",
            "ms_per_step": 1e3 * b["el"] / steps,
            "solve": ("batched pressure solves: one launch per multigrid pass over each of %d cost-balanced "
                      "groups (each worker steps whole groups), CUDA graphs, %d pass tile shapes autotuned, "
                      "levels of at most %d nodes in each member's single-block tail"
                      % (b["groups"], b["tiles"], b["tail_nodes"])),
            "step_ms_per_group_count": b["group_ms"], "gpu_launches": b["launches"]}


def run_ensemble(args):
    """Member time steps per second of the droplet-study ensemble: members
    of 48-160^3 cells, Weber 50-800, mixed-precision pressure to tol.  The
    members run on their own streams from a pool of host threads.  With N
    ranks the members are sharded across the GPUs by cost (no data-path
    collective); the time is the slowest rank's."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dsg = importlib.import_module(PKG)
    lib = dsg.load()
    cfgs = dsg.ensemble.study_configs(args.ensemble, tol=args.tol)
    mine = dsg.ensemble.shard(cfgs, rank, ws)
    cells = sum((c.nx - 2) * (c.ny - 2) * (c.nz - 2) for c in cfgs)
    cands = [] if args.no_batched else (
        [args.groups] if args.groups > 0 else [g for g in (1, 2, 4, 8, 16) if g <= len(mine)])
    m = measure_ensemble(dsg, lib, [cfgs[i] for i in mine], args.steps, args.warmup, args.workers, cands, dist)
    if "batched" in m:
        m["batched"]["el"] = max_over_ranks(m["batched"]["el"], dist, "cuda")
    el = max_over_ranks(m["el"], dist, "cuda")
    el1 = max_over_ranks(m["el1"], dist, "cuda")
    value = args.ensemble * args.steps / el
    if rank == 0:
        stats = m["stats"]
        line = {"metric": "member time-steps/s, droplet-study ensemble", "value": value,
                "unit": "member-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "%d droplets on wall, interior sides 48/64/96/128/160, Weber 50-800 "
                                       "log-uniform, D = 2 mm, mixed-precision pressure to %.0e"
                                       % (args.ensemble, args.tol),
                           "cells_per_step": cells, "workers": m["workers"], "autotuned": m["tuned"],
                           "pressure_solve": "one mixed-precision solve per member (CUDA graphs per member)",
                           "members_rank0": len(mine),
                           "parallelism": "members sharded by cost over %d GPU(s)" % ws,
                           "timing": "host clock between synchronisations of all member streams"},
                "one_worker_value": args.ensemble / el1,
                "vcycles_mean": float(sum(s["vcycles"] for st in stats for s in st) / max(1, len(stats) * m["n"])),
                "gpu_launches": m["launches"], "clocks": m["clocks"]}
        if "batched" in m:
            line["batched"] = batched_entry(args.ensemble, args.steps, m["batched"])
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def solver_bytes_estimate(inp):
    return 20.0 * inp.nx * inp.ny * inp.nz * 8


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.ensemble:
        return run_ensemble(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
