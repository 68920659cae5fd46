#!/usr/bin/env python
"""Benchmark: AMRD FAS multigrid solves per second on GB300.

Workload (one step = one elliptic solve): the 3-D conformal-factor equation
lap(psi) + 2 pi rho psi^5 = 0 on [-10,10]^3, 129^3 base grid plus two nested
2:1 levels of 65^3 boxes (7 MG levels down to 9^3), V(2,2) FAS cycles until
the finest residual is 1e-10 of its initial value -- the hierarchy the
reference's solve_elliptics (amrd/mg.c:20) runs on. Seeded synthetic rho
(pamr_amrd_gb300.workloads.conformal3d); rank r uses seed r.

Each step resets psi to its initial guess (device copy) and solves; L2 is
flushed between steps (512 MiB write, outside the timed events). `value` is
solves/s with inputs resident in HBM; `e2e` is the same through the C ABI
with host buffers (host->device copy of psi and rho, solve, device->host
copy of psi). `cpu_baseline` times the oracle port (a C restatement of the
reference's path) on this machine's host cores.

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
N>1 runs N independent replicas (one per GPU, launched by torch.distributed.run).

python bench.py --workload poisson3d_learned [--pairs P --epochs E] trains the
learned initial guess on P multigrid-generated pairs and prints one line
comparing plain solves with guessed ones (V-cycles and solves/s).
python bench.py --workload lapse_bo [--bo-steps S] times the lapse solves of
an S-step Berger-Oliger sequence (default 400) in both forms.
"""
from __future__ import annotations

import argparse
import copy
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s to 1e-10 rel. residual: plain FP64 vs chosen form; smoother HBM GB/s"
UNIT = "solves/s"
WORKLOAD = ("conformal3d_129_65: lap(psi)+2*pi*rho*psi^5=0 on [-10,10]^3, 129^3 base + 2 nested "
            "65^3 levels (7 MG levels, coarsest 9^3), V(2,2) FAS to 1e-10 relative residual")
FALLBACK_HBM_GBS = 6800.0


def _case(seed: int):
    """the workload of rank `seed` (each replica solves its own source)"""
    from pamr_amrd_gb300 import workloads as W
    return W.conformal3d(129, 65, seed=seed)


def max_over_ranks(x: float, dist, torch, device: str) -> float:
    """the job's time is its slowest replica's: MAX over ranks (identity
    without a process group); device "cuda" under NCCL, "cpu" under gloo"""
    if not dist:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ CPU side --
def _pin(seed: int):
    """one solve per core: the process that solves seed s runs on core s mod n"""
    try:
        cores = sorted(os.sched_getaffinity(0))
        os.sched_setaffinity(0, {cores[seed % len(cores)]})
    except (AttributeError, OSError):
        pass


def _port_solve(seed: int, keep_u: bool = False):
    from oracle import portrun
    _pin(seed)
    t = time.perf_counter()
    r = portrun.solve(_case(seed), fast=True)
    return time.perf_counter() - t, (r["u"] if keep_u else None)


def _port_solve_keep(seed: int):
    return _port_solve(seed, keep_u=seed == 0)


def _port_solve_poisson3d(seed: int):
    from oracle import portrun
    from pamr_amrd_gb300 import workloads as W
    _pin(seed)
    t = time.perf_counter()
    portrun.solve(W.poisson3d(129, seed=seed), fast=True)
    return time.perf_counter() - t, None


def cpu_round(nproc: int, seed0: int = 0, solve=_port_solve) -> dict:
    """one bounded sample: nproc oracle-port solves of the workload, one per
    host core (pinned), in parallel (spawned processes); the port is built
    -O3 -march=native for this (portrun.LIB_FAST)"""
    from oracle import portrun
    portrun.build(fast=True)
    ctx = mp.get_context("spawn")
    t = time.perf_counter()
    with ctx.Pool(nproc) as pool:
        out = pool.map(solve, [seed0 + i for i in range(nproc)])
    wall = time.perf_counter() - t
    per = [o[0] for o in out]
    u0 = next((o[1] for o in out if o[1] is not None), None)
    return {"solves": nproc, "wall_s": wall, "per_solve_s": statistics.median(per), "u_seed0": u0}


def cpu_model() -> str:
    """the host CPU's model name (lscpu, else /proc/cpuinfo, else platform)"""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def solve_model_bytes(sv, nu1: int, nu2: int, b_sweep: float) -> dict:
    """Algorithmic HBM bytes of one V(nu1,nu2) cycle of the FAS multigrid
    (amrd/mg.c:84-201): per level with N interior points, nu1+nu2 sweeps of
    b_sweep bytes per point, the residual (32), L_op (24), compute_MG_rhs (40)
    and the coarse-grid correction (24); per restriction into a level, the
    fine and coarse points of the three restricted fields (res, u, src: 8 B
    each). The coarsest level's loop is counted per sweep with
    coarsest_point_sweep_bytes. cmask traffic counts 0 (derivable from the box
    table)."""
    nlev = sv.num_levels()
    n = []
    for L in range(1, nlev + 1):
        tot = 0
        for b in range(sv.level_nbox(L)):
            sh = sv.box_info(L, b)["shape"]
            pts = 1
            for d in sh:
                pts *= max(d - 2, 1) if d > 1 else 1
            tot += pts
        n.append(tot)
    per_cycle = sum(N * ((nu1 + nu2) * b_sweep + 32 + 24 + 40 + 24) for N in n[1:])
    per_cycle += sum(3 * 8 * (n[L] + n[L - 1]) for L in range(1, nlev))
    return {"bytes_per_cycle": float(per_cycle), "coarsest_point_sweep_bytes": float(n[0] * b_sweep),
            "interior_points": n}


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# -------------------------------------------------------------- clocks --
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
            return
        # the timed region starts once the sampler has written its first line
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.p.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.02)

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = float(json.load(f)["hbm_gbs"])
        return v, "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# the FP32 sweep kernel of each value the mixed form's autotuner reports
# (pgb_level_tuning's sweeps_per_launch), and the committed ncu summaries
# that hold its DRAM bytes per launch on the workload's 129^3 level and on
# the 385^3 grid
SWEEP_KERNELS = {0: "k_relax32, one launch per colour pass", 1: "k_sweep32<1>, one sweep per launch",
                 2: "k_sweep32<2>, two sweeps per launch", 3: "k_sweep32z, one-pass plane marching",
                 4: "k_sweep32t<60>, TMA-staged one pass", 5: "k_sweep32t<28>, TMA-staged one pass",
                 6: "k_sweep32t2<24>, TMA-staged, two sweeps per pass",
                 7: "k_sweep32t2<56>, TMA-staged, two sweeps per pass"}
SWEEP_PROFILE_129 = {5: "k_sweep32t_129cube_level.md", 6: "k_sweep32t2_129cube_level.md"}
SWEEP_PROFILE_385 = {4: "k_sweep32t_385cube.md"}


def ncu_traffic(summary: str):
    """DRAM bytes (read + write) per launch of a kernel, from a committed ncu
    summary under profiles/ (its line 'dram_bytes_per_launch: <n>'), or
    None where there is none"""
    p = os.path.join(ROOT, "profiles", summary)
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def sweep_beyond_l2(S, torch, np, peak, n: int = 385):
    """the same FP32 sweep on one n^3 grid whose three FP32 arrays (3 x 228
    MB at n = 385) exceed the 129 MB L2, so that each sweep streams them
    from HBM: the HBM efficiency of the smoother itself, apart from the
    launch and L2 latency that bound it on the workload's 129^3 level"""
    from pamr_amrd_gb300 import workloads as W
    bbox = (-10.0, 10.0, -10.0, 10.0, -10.0, 10.0)
    g = W.Grid(1, bbox, (n, n, n))
    prm = W.MGParams()
    prm.precision = 1
    case = W.Case(f"poisson3d_{n}", W.POISSON, 3, (n, n, n), bbox, [g], [], [], prm)
    sv = S.Solver(case)
    z = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()   # the solver copies on its own stream
    sv.set_inputs_device([z.data_ptr()], [z.data_ptr()])
    sv.prepare()
    L = sv.num_levels()
    torch.cuda.nvtx.range_push("time_relax_beyond_l2")
    ms, by = sv.time_relax(L, reps=10)
    torch.cuda.nvtx.range_pop()
    tz, fuse = sv.level_tuning(L)
    sv.close()
    gbs = by / (ms / 1e3) / 1e9
    return {"grid": f"{n}^3", "ms_per_sweep": ms, "bytes_per_sweep": by, "achieved": gbs,
            "frac": gbs / peak, "tuned": {"tile_planes": tz, "sweeps_per_launch": fuse}}


# --------------------------------------------- Berger-Oliger lapse run --
LAPSE_WORKLOAD = ("lapse2d_bo_257_L4: maximal-slicing lapse lap(alpha) = alpha*S at every coarse step of a "
                  "400-step Berger-Oliger sequence (Courant 0.5), 257^2 base on [-10,10]^2 + 3 nested 2:1 "
                  "levels (3.7 M points), S = breathing Gaussian shell, each solve warm-started from the "
                  "previous lapse, V(2,2) to 1e-10 of the step-0 residual")


def _lapse_port_solve(seed: int) -> float:
    from oracle import portrun
    from pamr_amrd_gb300 import workloads as W
    _pin(seed)
    t = time.perf_counter()
    portrun.solve(W.lapse2d_bo(257, seed=seed, levels=4), fast=True)
    return time.perf_counter() - t


def lapse_main(args):
    """the whole lapse sequence in both forms and with two initial guesses
    per step: the previous step's lapse, and its time extrapolation from the
    two previous steps by the device Berger-Oliger bookkeeping (evolve.c's
    2nd-order extrapolation from extrap_tm1/tm2, rotated after each solve).
    Per coarse step the shell's source is evaluated on the device and the
    solve runs to the fixed tolerance."""
    import numpy as np
    import torch
    from pamr_amrd_gb300 import bo
    from pamr_amrd_gb300 import solver as S
    from pamr_amrd_gb300 import workloads as W
    torch.cuda.set_device(0)
    steps = args.bo_steps
    case = W.lapse2d_bo(257, seed=0, levels=4, steps=steps)
    r0, amp, w = W.lapse_shell(0)
    dt = 0.5 * 20.0 / (257 - 1)   # Courant 0.5 on the base grid
    levels = [g.level for g in case.grids]
    sizes = [g.size for g in case.grids]
    radius = []
    for g in case.grids:
        x = torch.tensor(g.coords(0), device="cuda").view(1, -1)
        y = torch.tensor(g.coords(1), device="cuda").view(-1, 1)
        radius.append(torch.sqrt(x * x + y * y).reshape(-1).contiguous())
    src = [torch.empty_like(r) for r in radius]
    ones = [torch.ones_like(r) for r in radius]
    u = [torch.empty_like(r) for r in radius]
    guess = [torch.empty_like(r) for r in radius]
    etm1 = [torch.empty_like(r) for r in radius]
    etm2 = [torch.empty_like(r) for r in radius]
    ptr = lambda ts: [t.data_ptr() for t in ts]   # noqa: E731
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()   # the solver copies on its own stream
    out, finals = {}, {}
    for prec, form in ((0, "fp64"), (1, "mixed")):
        c = copy.deepcopy(case)
        c.params.precision = prec
        sv = S.Solver(c)
        st = torch.cuda.ExternalStream(sv.stream())

        def run(k, start):
            R = W.shell_radius(r0, k, steps)
            with torch.cuda.stream(st):
                for s_, r_ in zip(src, radius):
                    torch.mul(torch.exp(-((r_ - R) / w) ** 2), amp, out=s_)
            sv.set_inputs_device(ptr(start), ptr(src))
            res = sv.solve()
            for i, a in enumerate(u):
                S._check(S.lib().pgb_get_grid_device(sv.h, i, a.data_ptr()))
            return res

        for _ in range(args.warmup):   # cold solves of step 0, untimed
            run(0, ones)
        for guess_kind in ("previous", "extrapolated"):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            clk = Clocks(torch.cuda.current_device()) if prec == 1 and guess_kind == "extrapolated" else None
            l0 = S.launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            iters, ok = [], True
            for k in range(steps):
                if k == 0:
                    start = ones
                elif guess_kind == "previous" or k == 1:
                    start = u
                else:
                    t = k * dt
                    for i in range(len(u)):
                        bo.mg_extrap(bo.ETM1, t, t, dt, dt, guess[i].data_ptr(), 0, etm1[i].data_ptr(),
                                     etm2[i].data_ptr(), sizes[i], sv.stream())
                    start = guess
                r = run(k, start)
                if guess_kind == "extrapolated":
                    bo.update_mg_extrap_vars(1, max(levels), [2] * 8, levels, ptr(etm1), ptr(etm2), ptr(u),
                                             ptr(u), sizes, 0.0, sv.stream())
                iters.append(r["iters"])
                ok = ok and r["res_final"] <= c.params.tol
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            out[f"{form}_{guess_kind}"] = {
                "solves_per_s": 1e3 * steps / ms, "ms_per_solve": ms / steps,
                "vcycles_per_solve": statistics.mean(iters), "vcycles_step0": iters[0],
                "all_converged": ok, "gpu_launches": S.launch_count() - l0,
                "clocks": clk.stop() if clk else None}
            finals[f"{form}_{guess_kind}"] = [a.cpu().numpy() for a in u]
        sv.close()
    ref = finals["fp64_previous"]
    umax = max(float(np.abs(a).max()) for a in ref)
    emax = max(float(np.abs(a - b).max()) for a, b in zip(finals["mixed_extrapolated"], ref))
    cpu = None
    if not args.no_cpu_baseline:
        nproc = min(host_cores(), 16)
        from oracle import portrun
        portrun.build(fast=True)
        ctx = mp.get_context("spawn")
        t0 = time.perf_counter()
        with ctx.Pool(nproc) as pool:
            per = pool.map(_lapse_port_solve, list(range(nproc)))
        wall = time.perf_counter() - t0
        cpu = {"value": nproc / wall, "unit": "solves/s", "cores": nproc, "kind": "port",
               "sample": f"{nproc} concurrent oracle-port cold solves of step 0 (seeds 0..{nproc - 1}; "
                         f"median {statistics.median(per):.1f} s per solve)"}
    mx = out["mixed_extrapolated"]
    line = {"metric": "lapse solves/s over a Berger-Oliger sequence, mixed form, extrapolated guess "
                      "(FP64 form and previous-step guess beside it)",
            "value": mx["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": mx["ms_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded shell: radius, amplitude, width from seed 0)",
            "config": {"workload": LAPSE_WORKLOAD, "points": case.total_points(),
                       "l2": "not flushed between steps: the sequence runs back to back (3.7 M points, "
                             "arrays larger than L2)"},
            "runs": out, "fp64_solves_per_s": out["fp64_extrapolated"]["solves_per_s"],
            "speedup_vs_fp64": mx["solves_per_s"] / out["fp64_extrapolated"]["solves_per_s"],
            "error_vs_fp64_final_step": {"max_abs": emax, "max_rel": emax / umax},
            "gpu_launches": mx["gpu_launches"], "cpu_baseline": cpu, "clocks": mx["clocks"]}
    print(json.dumps(line))


# ------------------------------------------------ learned initial guess --
LEARNED_WORKLOAD = ("poisson3d_129: lap u = rho on [-10,10]^3, one 129^3 grid (6 MG levels), "
                    "rho = 4 seeded Gaussians, V(2,2) to 1e-10 relative residual; guess = 6-level "
                    "BF16 tensor-core encoder-decoder trained on multigrid-generated pairs")


def stream_solves(sv, st, model, rhos, zero, torch, pipelined: bool) -> dict:
    """solves/s of the sources in `rhos` solved back to back on solver sv
    (stream st): from u = 0, or (pipelined) each from the net's guess, the
    guess of source k+1 predicted on a second stream while solve k runs
    (two guess buffers; the prediction into a buffer waits until the solver
    has copied its previous content in)"""
    import statistics as stats
    n = len(rhos)
    ps = torch.cuda.Stream()
    gbuf = [torch.zeros_like(zero), torch.zeros_like(zero)]
    ready = [torch.cuda.Event() for _ in range(2)]
    taken = [torch.cuda.Event() for _ in range(2)]

    def predict(k):
        b = k % 2
        with torch.cuda.stream(ps):
            if k >= 2:
                ps.wait_event(taken[b])
            model.predict(rhos[k], gbuf[b], ps.cuda_stream)
            ready[b].record(ps)

    torch.cuda.synchronize()
    if pipelined:
        predict(0)
    t0 = time.perf_counter()
    iters = []
    for k in range(n):
        if pipelined:
            if k + 1 < n:
                predict(k + 1)
            st.wait_event(ready[k % 2])
            sv.set_inputs_device([gbuf[k % 2].data_ptr()], [rhos[k].data_ptr()])
            taken[k % 2].record(st)
        else:
            sv.set_inputs_device([zero.data_ptr()], [rhos[k].data_ptr()])
        iters.append(sv.solve()["iters"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    key = "guess_pipelined" if pipelined else "plain"
    return {f"{key}_solves_per_s": n / wall, f"{key}_vcycles": stats.mean(iters)}


def learned_main(args):
    """plain solves against solves started from the net's guess (prediction
    plus energy-norm rescale, timed with the solve), both precision forms,
    on held-out sources; the guess policy's solves/s is `value`"""
    import numpy as np
    import torch
    from pamr_amrd_gb300 import learned as Lm
    from pamr_amrd_gb300 import solver as S
    from pamr_amrd_gb300 import workloads as W
    torch.cuda.set_device(0)
    n = 129
    h = 20.0 / (n - 1)
    t0 = time.perf_counter()
    if args.pairs_from == "sequence":   # pairs along time-stepped runs, 20 coarse steps each
        blobs, U = Lm.make_sequence_dataset(n, range((args.pairs + 19) // 20), 20, torch)
    else:
        blobs, U = Lm.make_dataset(n, range(args.pairs), torch)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    gain = Lm.fit_gain(n, blobs, U, torch)
    model = Lm.Scaled(Lm.Net(n, seed=1), gain, h)
    t0 = time.perf_counter()
    losses = Lm.train(model, blobs, U, torch, epochs=args.epochs, lr=args.lr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del U

    seeds = [100000 + k for k in range(args.warmup + args.steps)]
    rhos = [Lm.rho_on_device(n, W.poisson3d_blobs(sd), torch) for sd in seeds]
    zero = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    guess = torch.zeros_like(zero)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {}
    for prec, form in ((0, "fp64"), (1, "mixed")):
        case = W.poisson3d(n, seed=seeds[0])
        case.params.precision = prec
        sv = S.Solver(case)
        st = torch.cuda.ExternalStream(sv.stream())
        u_plain = torch.empty_like(zero)
        res = {"plain": [], "guess": []}
        errs = []
        for k, rho in enumerate(rhos):
            for mode in ("plain", "guess"):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                if mode == "guess":
                    model.predict(rho, guess, sv.stream())
                    sv.set_inputs_device([guess.data_ptr()], [rho.data_ptr()])
                else:
                    sv.set_inputs_device([zero.data_ptr()], [rho.data_ptr()])
                r = sv.solve()
                e1.record(st)
                e1.synchronize()
                if k < args.warmup:
                    continue
                res[mode].append((e0.elapsed_time(e1), r["iters"], r["res_final"] <= case.params.tol))
                if mode == "plain":
                    S._check(S.lib().pgb_get_grid_device(sv.h, 0, u_plain.data_ptr()))
            if k >= args.warmup and prec == 1:
                model.predict(rho, guess, sv.stream())
                torch.cuda.synchronize()
                d = guess - u_plain
                errs.append((float(d.abs().max() / u_plain.abs().max()),
                             float(d.norm() / u_plain.norm())))
        # The same held-out sources as one stream of solves, back to back (no
        # L2 flush, host wall clock over the whole stream): plain from u = 0,
        # and with each guess predicted on a second stream while the solve
        # before it runs (a stream of elliptic solves, as a Berger-Oliger run
        # or an ensemble issues them; the small levels of a V-cycle leave
        # most SMs idle, which the prediction fills)
        stream_rates = stream_solves(sv, st, model, rhos[args.warmup:], zero, torch, pipelined=False)
        if prec == 1:
            stream_rates.update(stream_solves(sv, st, model, rhos[args.warmup:], zero, torch, pipelined=True))
        # the guess policy over the same sources: one plain solve first, then
        # guesses while they cut cycles
        pol = Lm.GuessPolicy()
        pol_ms, used = 0.0, 0
        for k in range(args.steps):
            use = pol.use_guess()
            ms, it, _ = res["guess" if use else "plain"][k]
            pol.record(it, use, ms)
            pol_ms += ms
            used += use
        out[form] = {
            "plain_solves_per_s": 1e3 * args.steps / sum(m for m, _, _ in res["plain"]),
            "guess_solves_per_s": 1e3 * args.steps / sum(m for m, _, _ in res["guess"]),
            "policy_solves_per_s": 1e3 * args.steps / pol_ms,
            "plain_vcycles": statistics.mean(i for _, i, _ in res["plain"]),
            "guess_vcycles": statistics.mean(i for _, i, _ in res["guess"]),
            "policy_guessed_solves": used, "policy_enabled_at_end": pol.enabled, "stream": stream_rates,
            "all_converged": all(c for _, _, c in res["plain"] + res["guess"])}
        sv.close()
    # prediction alone (forward + rescale)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for _ in range(3):
        model.predict(rhos[0], guess)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("predict_only")   # lets a profiler select these launches
    ev[0].record()
    for _ in range(10):
        model.predict(rhos[0], guess)
    ev[1].record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    mx = out["mixed"]
    cpu = None
    if not args.no_cpu_baseline:
        nproc = min(host_cores(), 32)
        cr = cpu_round(nproc, seed0=100000, solve=_port_solve_poisson3d)
        cpu = {"value": cr["solves"] / cr["wall_s"], "unit": "solves/s", "cores": nproc, "kind": "port",
               "sample": f"{nproc} concurrent oracle-port FP64 solves of poisson3d_129 from u = 0 "
                         f"(the reference has no learned guess), median {cr['per_solve_s']:.2f} s each"}
    line = {"metric": "poisson3d_129 solves/s with the learned initial guess (guess policy), mixed form",
            "value": mx["policy_solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 / mx["policy_solves_per_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 guess + f32/f64 solve",
            "data": "synthetic (seeded rho; training seeds 0..pairs-1, timed on held-out seeds 100000+)",
            "config": {"workload": LEARNED_WORKLOAD, "l2": "flushed between steps (512 MiB write)",
                       "pairs": args.pairs, "pairs_from": args.pairs_from, "epochs": args.epochs, "lr": args.lr},
            "forms": out, "cpu_baseline": cpu, "predict_ms": ev[0].elapsed_time(ev[1]) / 10,
            # the spec ratio on a stream of solves (both back to back,
            # no L2 flush): learned-guess mixed solver against plain FP64
            "stream_ratio_vs_fp64_plain": {
                "mixed_learned_guess_pipelined": out["mixed"]["stream"]["guess_pipelined_solves_per_s"] /
                out["fp64"]["stream"]["plain_solves_per_s"],
                "mixed_plain": out["mixed"]["stream"]["plain_solves_per_s"] / out["fp64"]["stream"]["plain_solves_per_s"]},
            "guess_error_vs_solution": {"max_rel": statistics.mean(e[0] for e in errs),
                                        "l2_rel": statistics.mean(e[1] for e in errs)},
            "training": {"dataset_s": t_data, "train_s": t_train, "epoch_loss": losses,
                         "params": model.net.num_params()}}
    print(json.dumps(line))


def other_workload(S, make, torch, np, flush, steps: int, warmup: int) -> dict:
    """solves/s of both forms on one more workload (device-resident inputs,
    L2 flushed between steps, CUDA events on the solver's stream) and the
    mixed form's error against the FP64 form. A workload with several
    elliptic variables or sources has every one of them reset from the host
    before the timed region of each step (the solve alone is timed)"""
    out = {}
    sols = {}
    for prec, form in ((0, "fp64"), (1, "mixed")):
        case = make()
        case.params.precision = prec
        multi = case.nvar > 1 or bool(case.src_extra)
        sv = S.Solver(case)
        d_u0 = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in case.u0]
        d_src = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in case.src]
        st = torch.cuda.ExternalStream(sv.stream())
        times, iters = [], []
        for k in range(warmup + steps):
            flush.fill_(1.0)
            if multi:
                sv.set_inputs()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            if not multi:
                sv.set_inputs_device([t.data_ptr() for t in d_u0], [t.data_ptr() for t in d_src])
            r = sv.solve()
            e1.record(st)
            e1.synchronize()
            if k >= warmup:
                times.append(e0.elapsed_time(e1))
                iters.append(r["iters"])
        sols[form] = [a for var in sv.get_vars() for a in var] if case.nvar > 1 else sv.get_u()
        out[form] = {"solves_per_s": 1e3 * steps / sum(times), "vcycles_per_solve": statistics.mean(iters),
                     "converged": r["res_final"] <= case.params.tol}
        sv.close()
    umax = max(float(np.max(np.abs(a))) for a in sols["fp64"])
    out["speedup_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["error_vs_fp64_gpu_form_max_rel"] = max(float(np.max(np.abs(a - b))) for a, b in
                                                zip(sols["mixed"], sols["fp64"])) / umax
    out["points"] = make().total_points()
    return out


# ---------------------------------------------------------------- main --
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="conformal3d", choices=["conformal3d", "poisson3d_learned", "lapse_bo"],
                    help="poisson3d_learned: solves with and without the learned initial guess; "
                         "lapse_bo: the lapse solves of a Berger-Oliger sequence")
    ap.add_argument("--bo-steps", type=int, default=400, help="coarse steps of the sequence (lapse_bo)")
    ap.add_argument("--pairs", type=int, default=2000, help="training pairs (poisson3d_learned)")
    ap.add_argument("--pairs-from", default="sequence", choices=["sequence", "seeds"],
                    help="training pairs from time-stepped runs with drifting sources (20 steps per run, each "
                         "solve started from the last) or from independent seeded sources (poisson3d_learned)")
    ap.add_argument("--epochs", type=int, default=4, help="training epochs (poisson3d_learned; 6 with this schedule diverged in its third epoch)")
    ap.add_argument("--lr", type=float, default=1e-3, help="peak learning rate (poisson3d_learned)")
    args = ap.parse_args()
    if args.workload == "lapse_bo":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "timed by this line's cpu_baseline "
                                                                   "(the oracle port of the reference's path)"}))
        elif int(os.environ.get("RANK", "0")) == 0:
            lapse_main(args)
        return
    if args.workload == "poisson3d_learned":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned initial guess"}))
        elif int(os.environ.get("RANK", "0")) == 0:
            learned_main(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        nproc = min(host_cores(), 32)
        for _ in range(min(args.warmup, 1)):
            cpu_round(nproc, seed0=100)
        # one step = one solve per host core (about 12 s); at most 5 steps,
        # so that the run stays within a few minutes whatever --steps asks
        nrounds = min(args.steps, 5)
        rounds = [cpu_round(nproc, seed0=i * nproc) for i in range(nrounds)]
        solves = sum(r["solves"] for r in rounds)
        wall = sum(r["wall_s"] for r in rounds)
        v = solves / wall
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": nrounds, "steps_requested": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * wall / nrounds,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded rho)", "config": {"workload": WORKLOAD,
                                                             "sample": f"{nproc} solves per step"},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": nproc, "kind": "port",
                                 "sample": f"{nproc} concurrent oracle-port solves per step, "
                                           f"{nrounds} steps"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import numpy as np
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    from pamr_amrd_gb300 import solver as S
    case = _case(rank)
    case64 = copy.deepcopy(case)
    case64.params.precision = 0
    casemx = copy.deepcopy(case)
    casemx.params.precision = 1
    s64 = S.Solver(case64)
    smx = S.Solver(casemx)
    # device-resident inputs
    d_u0 = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in case.u0]
    d_src = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in case.src]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(s):
        s.set_inputs_device([t.data_ptr() for t in d_u0], [t.data_ptr() for t in d_src])
        return s.solve()

    def timed(s, label, clocks=None):
        stream = torch.cuda.ExternalStream(s.stream())
        for _ in range(args.warmup):
            flush.fill_(1.0)
            step(s)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clk = Clocks(torch.cuda.current_device()) if clocks else None
        l0 = S.launch_count()
        times, iters, finals = [], [], []
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(f"timed_{label}")   # lets a profiler select these steps
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = step(s)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            iters.append(r["iters"])
            finals.append(r["res_final"])
        torch.cuda.synchronize()
        wall = 1e3 * (time.perf_counter() - t_wall)
        torch.cuda.nvtx.range_pop()
        launches = S.launch_count() - l0
        ck = clk.stop() if clk else None
        if dist:
            dist.barrier()
        total = max_over_ranks(sum(times), dist, torch, "cuda")
        return {"total_ms": total, "iters": iters, "finals": finals, "wall_ms": wall,
                "launches": launches, "clocks": ck}

    # clocks sampled over both timed loops (the FP64 loop alone lasts seconds)
    clk = Clocks(torch.cuda.current_device()) if rank == 0 else None
    tm64 = timed(s64, "fp64")
    tmx = timed(smx, "mixed")
    clocks = clk.stop() if clk else None
    value = world * args.steps / (tmx["total_ms"] / 1e3)
    fp64_value = world * args.steps / (tm64["total_ms"] / 1e3)
    ms_per_step = tmx["total_ms"] / args.steps
    converged = all(f <= case.params.tol for f in tmx["finals"] + tm64["finals"])
    u64, umx = s64.get_u(), smx.get_u()
    umax = max(float(np.max(np.abs(a))) for a in u64)
    emax = max(float(np.max(np.abs(a - b))) for a, b in zip(umx, u64))
    el2 = float(np.sqrt(sum(float(np.sum((a - b) ** 2)) for a, b in zip(umx, u64)) /
                        sum(a.size for a in u64)))

    # e2e through the C ABI with host buffers (chosen form)
    pin_u = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in case.u0]
    pin_s = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in case.src]
    out_u = [torch.empty(g.size, dtype=torch.float64).pin_memory() for g in case.grids]
    h2d = sum(2 * 8 * g.size for g in case.grids)
    d2h = sum(8 * g.size for g in case.grids)
    dp = S.C.POINTER(S.C.c_double)
    e2e_ms = []
    for k in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(len(case.grids)):
            S._check(S.lib().pgb_set_grid(smx.h, i, S.C.cast(pin_u[i].data_ptr(), dp),
                                          S.C.cast(pin_s[i].data_ptr(), dp)))
        smx.solve()
        for i in range(len(case.grids)):
            S._check(S.lib().pgb_get_grid(smx.h, i, S.C.cast(out_u[i].data_ptr(), dp)))
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = max_over_ranks(sum(e2e_ms), dist, torch, "cuda")
    e2e_value = world * args.steps / (e2e_total / 1e3)

    # configs 1 and 3 of the same metric beside the headline workload: the
    # 129^2 Poisson grid and the uneven 5-level hierarchy, both forms; and a
    # coupled pair of elliptic variables on the headline's grids
    extra = {}
    if rank == 0:
        from pamr_amrd_gb300 import workloads as W
        for name, make in (("config1_poisson2d_129", lambda: W.poisson2d(129, seed=0)),
                           ("config3_poisson2d_uneven", lambda: W.poisson2d_uneven(seed=0)),
                           ("coupled_pair_conformal3d_129_65",
                            lambda: W.coupled_from(W.conformal3d(129, 65, seed=0), seed=1))):
            try:
                n = max(3, min(args.steps, 5 if name.startswith("coupled") else 20))
                extra[name] = other_workload(S, make, torch, np, flush, steps=n, warmup=args.warmup)
            except Exception as exc:   # a report, never a reason to lose the bench line
                extra[name] = {"error": str(exc)}

    # roofline of the dominant smoother: FP32 sweep of the mixed form on the
    # 129^3 level (and the FP64 sweep of the plain form beside it)
    big = max(range(1, smx.num_levels() + 1),
              key=lambda L: max(smx.box_info(L, b)["shape"][0] for b in range(smx.level_nbox(L))))
    flush.fill_(1.0)
    torch.cuda.nvtx.range_push("time_relax_mixed")
    ms_sweep, bytes_sweep = smx.time_relax(big, reps=20)
    torch.cuda.nvtx.range_pop()
    ms64_sweep, bytes64_sweep = s64.time_relax(big, reps=10)
    tz, fuse = smx.level_tuning(big)
    # algorithmic bytes count 16 B per relaxed point per sweep; a launch of
    # the two-sweep kernels runs two sweeps (and streams E, D and C once)
    per_launch = 2 if fuse in (2, 6, 7) and smx.case.params.pre_swp >= 2 else 1
    ms_launch = per_launch * ms_sweep
    achieved = per_launch * bytes_sweep / (ms_launch / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    prof = SWEEP_PROFILE_129.get(fuse)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": ncu_traffic(prof) if prof else None, "peak_source": peak_kind,
            "kernel": "FP32 red+black sweep on the correction as the V-cycle runs it (129^3 level; "
                      + SWEEP_KERNELS.get(fuse, str(fuse)) + ")",
            "tuned": {"tile_planes": tz, "sweeps_per_launch": fuse},
            "sweeps_per_launch": per_launch, "ms_per_launch": ms_launch, "bytes_per_launch": per_launch * bytes_sweep,
            "ms_per_sweep": ms_sweep, "bytes_per_sweep": bytes_sweep,
            "fp64_sweep": {"kernel": "k_relax (FP64 Newton-GS sweep, 129^3 level)",
                           "ms_per_sweep": ms64_sweep,
                           "achieved_gbs": bytes64_sweep / (ms64_sweep / 1e3) / 1e9}}

    roof["beyond_l2"] = sweep_beyond_l2(S, torch, np, peak)
    prof = SWEEP_PROFILE_385.get(roof["beyond_l2"]["tuned"]["sweeps_per_launch"])
    roof["beyond_l2"]["traffic"] = ncu_traffic(prof) if prof else None

    # whole-solve roofline: algorithmic bytes of the cycles each form ran
    # (FP32 sweeps count 16 B per point, FP64 ones 32) over the timed solve
    solve_roof = None
    try:
        solve_roof = {}
        for form, sv, tm, bsw in (("mixed", smx, tmx, 16.0), ("fp64", s64, tm64, 32.0)):
            mb = solve_model_bytes(sv, case.params.pre_swp, case.params.pst_swp, bsw)
            cyc = statistics.mean(tm["iters"])
            citers = sv.stats()["coarsest_iters"]
            byt = cyc * mb["bytes_per_cycle"] + citers * mb["coarsest_point_sweep_bytes"]
            t = tm["total_ms"] / args.steps / 1e3
            solve_roof[form] = {"bytes_per_solve": byt, "achieved_gbs": byt / t / 1e9,
                                "frac": byt / t / 1e9 / peak, "coarsest_sweeps": citers}
    except Exception as exc:   # a report, never a reason to lose the bench line
        solve_roof = {"error": str(exc)}

    cpu = None
    err_oracle = None
    if rank == 0 and not args.no_cpu_baseline:
        nproc = min(host_cores(), 32)
        cr = cpu_round(nproc, solve=_port_solve_keep)
        cpu = {"value": cr["solves"] / cr["wall_s"], "unit": UNIT, "cores": nproc, "kind": "port",
               "sample": f"{nproc} concurrent oracle-port solves of the workload "
                         f"(median {cr['per_solve_s']:.1f} s per solve)",
               "per_core_value": 1.0 / cr["per_solve_s"], "cpu_model": cpu_model(),
               "build": "oracle port, gcc -O3 -march=native -ffp-contract=off, one process per core, pinned"}
        if cr["u_seed0"] is not None:   # the same seed as the GPU solves (rank 0)
            omax = max(float(np.max(np.abs(a))) for a in cr["u_seed0"])
            err_oracle = {
                "fp64": {"max_abs": max(float(np.max(np.abs(a - b))) for a, b in zip(u64, cr["u_seed0"])),
                         "bit_identical": all(np.array_equal(a, b) for a, b in zip(u64, cr["u_seed0"]))},
                "mixed": {"max_abs": max(float(np.max(np.abs(a - b))) for a, b in zip(umx, cr["u_seed0"]))}}
            err_oracle["mixed"]["max_rel"] = err_oracle["mixed"]["max_abs"] / omax

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded rho, rank r uses seed r)",
                "config": {"workload": WORKLOAD, "l2": "flushed between steps (512 MiB write)",
                           "points": case.total_points(), "mg_levels": smx.num_levels(),
                           "parallelism": f"replicas x{world}"},
                "chosen_form": "mixed: FP32 smoothing and prolongation in FP64 defect correction",
                "fp64_solves_per_s": fp64_value, "speedup_vs_fp64": value / fp64_value,
                "vcycles_per_solve": statistics.mean(tmx["iters"]),
                "fp64_vcycles_per_solve": statistics.mean(tm64["iters"]),
                "converged": converged,
                "error_vs_fp64_gpu_form": {"max_abs": emax, "max_rel": emax / umax, "l2": el2},
                "error_vs_fp64_oracle": err_oracle,
                "learned_guess_in_timed_solves": False,
                "other_configs": extra,
                "wall_ms_timed": tmx["wall_ms"],
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": tmx["launches"],
                "roofline": roof, "solve_roofline": solve_roof, "cpu_baseline": cpu,
                "clocks": clocks,
                "ms_x_median_sm_mhz": (ms_per_step * clocks["sm_mhz"]) if clocks and clocks.get("sm_mhz") else None}
        print(json.dumps(line))
    s64.close()
    smx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
