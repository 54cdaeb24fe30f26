"""Benchmark: two-site HxV throughput of the GB300 engine.

Workload (one GPU, N=1): Hubbard chain t=1, U/t=4, L=64, open boundaries,
U(1)xU(1) at half filling (N=64, Sz=0), two-site pivot in the middle of a
seeded random MPS at bond dimension D=4096 (N(0,1) blocks, QR/LQ normalised
towards the pivot), environments built by the engine's contract_L/contract_R.
A step is one HxV of that pivot (Lanczos' inner operation).

  value : HxV/s, split precision (BF16x3, FP32 accumulate), vectors resident in
          HBM, timed with CUDA events on the engine's stream, CUDA graph replay
  e2e   : HxV/s through the C ABI call vmps_hxv with pinned host buffers: the
          host->device copy of Vin, the HxV and the device->host copy of Vout
          are inside the timed region of every step

Also reported: the plain FP64 HxV/s, the ground-state energy of the pivot
problem from FP64 Lanczos vs split-precision Lanczos + FP64 refinement, the
roofline of the dominant kernel and the CPU oracle (reference restatement)
timed on the host cores.

--gpus N runs N independent replicas (the path does not shard; one process
per GPU under torchrun); value is the sum over ranks with max-over-ranks time.
--impl reference times the CPU restatement of the reference path instead.
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

import faulthandler  # noqa: E402

import numpy as np  # noqa: E402

faulthandler.enable()

METRIC = "HxV/s (two-site effective Hamiltonian, split-precision BF16x3 GPU vs FP64 GPU vs CPU)"
L2_BYTES = 129 * 1024 * 1024


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 0, 1, None
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, local, ws, dist


def reduce_max(dist, x, local):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_oracle_hxv_rate(L, R, V, W1, W2, threads, n_hxv, warm=1):
    import oracle
    oracle.set_threads(threads)
    op = oracle.OraclePivot(2, 2, L, R, V, W1, W2)
    v = np.random.default_rng(5).standard_normal(V.data.size)
    for _ in range(warm):
        op.hxv(v)
    t0 = time.perf_counter()
    for _ in range(n_hxv):
        op.hxv(v)
    dt = time.perf_counter() - t0
    return n_hxv / dt, dt, oracle.blas_kind()


def oracle_check(L, R, V, W1, W2, v0, h64, hsp, e_ref, e64, es, x64, xs):
    """The engine's results at the bench pivot against the FP64 oracle (CPU
    restatement of OxV, all host threads): both HxVs of v0, the ground-state energy
    from the oracle's own Lanczos (numpy three-term recurrence on the oracle's
    HxV), and the Rayleigh quotient and residual of the engine's returned vectors
    under the oracle's operator."""
    import oracle
    oracle.set_threads(os.cpu_count() or 1)
    op = oracle.OraclePivot(2, 2, L, R, V, W1, W2)
    t0 = time.perf_counter()
    ref = op.hxv(v0)
    out = {"hxv_fp64_rel_err": float(np.linalg.norm(h64 - ref) / np.linalg.norm(ref)),
           "hxv_split_rel_err": float(np.linalg.norm(hsp - ref) / np.linalg.norm(ref))}
    e_or, steps = oracle.lanczos_ground(op.hxv, v0, tol=1e-14)
    out.update({"E_oracle": e_or, "oracle_lanczos_steps": steps, "oracle_s": round(time.perf_counter() - t0, 1),
                "E_ref_fp64_rel_err": abs(e_ref - e_or) / abs(e_or),
                "E_fp64_rel_err": abs(e64 - e_or) / abs(e_or), "E_split_rel_err": abs(es - e_or) / abs(e_or)})
    for tag, x in (("fp64", x64), ("split", xs)):
        x = x / np.linalg.norm(x)
        hx = op.hxv(x)
        rq = float(x @ hx)
        out[f"{tag}_vector"] = {"rayleigh_rel_err": abs(rq - e_or) / abs(e_or),
                                "residual": float(np.linalg.norm(hx - rq * x))}
    return out


def autotune_small(ctx):
    """The autotuner on the small and middle pivots of the configurations: the
    two-site middle pivots of the Heisenberg chain L=32 D=64 (C1's model and size),
    the Hubbard chain at D=256 and D=1024 (C2's first stage), and the C5 pivot
    (Hubbard D=512, N=63): tuned against default ms per split HxV (CUDA events)."""
    from vmps_gb300.pivot import PivotMatrix2
    from vmps_gb300.workloads import hubbard_two_site, heisenberg_two_site
    out = {}
    cases = [("heisenberg_L32_D64", lambda: heisenberg_two_site(ctx, L=32, D=64, seed=1)),
             ("hubbard_L64_D256", lambda: hubbard_two_site(ctx, L=64, D=256, seed=2)),
             ("hubbard_L64_D512_N63", lambda: hubbard_two_site(ctx, L=64, D=512, seed=5, Qtot=(63, -1))),
             ("hubbard_L64_D1024", lambda: hubbard_two_site(ctx, L=64, D=1024, seed=2))]
    for name, make in cases:
        model, mps, Lenv, Renv, W1, W2, V, info = make()
        H = PivotMatrix2(ctx, model.sym, Lenv, Renv, W1, W2, V)
        t = H.autotune(trials=10)
        t["speedup"] = t["ms_default"] / t["ms_best"] if t["ms_best"] > 0 else None
        t["dim_V"] = H.dim
        out[name] = t
        H.close()
    return out


def step_trace(a, b):
    """per-step comparison of two sweeps run from the same MPS: relative energy
    difference of every local solve, the first step where it exceeds 1e-10 (-1: none)
    and the split-precision HxVs of run a"""
    ea = np.array([s[2] for s in a["steps"]])
    eb = np.array([s[2] for s in b["steps"]])
    d = np.abs(ea - eb) / np.abs(eb)
    first = int(np.argmax(d > 1e-10)) if np.any(d > 1e-10) else -1
    return {"steps": int(d.size), "max_rel_diff": float(d.max()), "first_step_above_1e-10": first,
            "site_of_first": int(a["steps"][first][1]) if first >= 0 else None,
            "max_rel_diff_before_first": float(d[:first].max()) if first > 0 else (float(d.max()) if first < 0 else None),
            "rel_diff_first_12": [float(x) for x in d[:12]], "split_hxv": int(sum(s[3] for s in a["steps"])),
            "fp64_hxv": int(sum(s[4] for s in a["steps"]))}


def sweep_bench(ctx, args, with_cpu=True):
    """Single-site DMRG sweep times.

    * Heisenberg L=32, D=64: GPU FP64 and the CPU oracle, 2 sweeps each.
    * Hubbard L=64, D=1024 (U(1)xU(1), half filling), single-site:
      - from the same random MPS, 2 sweeps in FP64 and 2 in split precision
        (BF16x3 + FP64 refinement).  Far from convergence the sweep is a chaotic
        map, so the two trajectories reach different intermediate energies;
      - after 4 more split sweeps (near convergence), one more sweep in each
        precision from the same MPS: there the energies agree to the
        tolerance, which is the |dE/E| the metric asks for.
    * the same chain with two-site DMRG at Dmax=1024 (SVD truncation on the host
      cores), one sweep in each precision from the same random MPS.
    HxV, Lanczos and contract_L/R run on the GPU; the QR / SVD gauge steps on the
    host.  Per-sweep timers split lanczos / precalc / gauge / lr."""
    import copy

    from vmps_gb300 import models
    from vmps_gb300.dmrg import dmrg1
    from vmps_gb300.mps import RandomMPS
    out = {}
    model = models.heisenberg_u1(32)
    mps = RandomMPS(model, (0,), 64, seed=1, profile="gaussian", sigma=[4.0]).canonicalize(0, 0)
    mps_cpu = copy.deepcopy(mps)
    g = dmrg1(ctx, model, mps, n_sweeps=2, precision="fp64", tol_eigval=1e-12, tol_state=1e-8)
    out["heisenberg_L32_D64"] = {"gpu_fp64_s_per_sweep": g["sweep_times"], "E_gpu": g["energies"],
                                 "hxv": g["hxv"]}
    if with_cpu:
        from oracle.dmrg_cpu import dmrg1_cpu
        c = dmrg1_cpu(model, mps_cpu, n_sweeps=2)
        out["heisenberg_L32_D64"].update({"cpu_s_per_sweep": c["sweep_times"], "E_cpu": c["energies"],
                                          "E_rel_diff": abs(c["energies"][-1] - g["energies"][-1]) /
                                          abs(c["energies"][-1])})
    if args.D >= 1024:
        model = models.hubbard_u1xu1(64, t=1.0, U=4.0)
        mps0 = RandomMPS(model, (64, 0), 1024, seed=2, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(0, 0)
        tol = dict(tol_eigval=1e-10, tol_state=1e-6)        # sweep tolerances
        tight = dict(tol_eigval=1e-13, tol_state=1e-10)     # converged comparisons
        split_kw = dict(precision=args.precision, refine_iters=10, **tol)

        def summary(r):
            return {"s_per_sweep": r["sweep_times"], "E": r["energies"], "hxv": r["hxv"],
                    "timers_s": [{k: round(v, 4) for k, v in t.items()} for t in r["timers"]],
                    "lanczos": r["solves"]}

        hub = {"tolerances": dict(refine_iters=10, **tol), "tight": tight}
        mps = copy.deepcopy(mps0)
        rs = dmrg1(ctx, model, mps, n_sweeps=2, **split_kw)
        r6 = dmrg1(ctx, model, copy.deepcopy(mps0), n_sweeps=2, precision="fp64", **tol)
        hub["from_random_split"] = summary(rs)
        hub["from_random_fp64"] = summary(r6)
        hub["from_random_trace"] = step_trace(rs, r6)
        w = dmrg1(ctx, model, mps, n_sweeps=4, **split_kw)
        hub["warm_split_sweeps"] = summary(w)
        # near convergence, one sweep in each precision with tight tolerances; the split
        # run skips the FP64 probe, so that its local solves do run split-precision HxVs
        r64 = dmrg1(ctx, model, copy.deepcopy(mps), n_sweeps=1, precision="fp64", **tight)
        rsp = dmrg1(ctx, model, copy.deepcopy(mps), n_sweeps=1, precision=args.precision, refine_iters=10,
                    probe=False, **tight)
        hub["converged_fp64"] = summary(r64)
        hub["converged_split_no_probe"] = summary(rsp)
        hub["converged_trace"] = step_trace(rsp, r64)
        hub["converged_rel_diff"] = abs(rsp["energies"][-1] - r64["energies"][-1]) / abs(r64["energies"][-1])
        out["hubbard_L64_D1024"] = hub
        # two-site DMRG (the sweep of the metric's configuration) at Dmax=1024 from the same
        # random MPS: one sweep in each precision (timings and the per-step trace), an FP64
        # control from the MPS perturbed by 1e-12 (where FP64 parts from FP64), then three
        # more split sweeps to convergence and one more sweep in each precision with tight
        # tolerances (split HxVs forced: no FP64 probe)
        from vmps_gb300.dmrg import dmrg2
        two = {"tolerances": dict(refine_iters=3, **tol), "Dmax": 1024}
        mps_s = copy.deepcopy(mps0)
        rs = dmrg2(ctx, model, mps_s, n_sweeps=1, Dmax=1024, precision=args.precision, refine_iters=3, **tol)
        r6 = dmrg2(ctx, model, copy.deepcopy(mps0), n_sweeps=1, Dmax=1024, precision="fp64", **tol)
        mps_p = copy.deepcopy(mps0)
        noise = np.random.default_rng(99)
        for A in mps_p.A:
            A.data *= 1.0 + 1e-12 * noise.standard_normal(A.data.size)
        rc = dmrg2(ctx, model, mps_p, n_sweeps=1, Dmax=1024, precision="fp64", **tol)
        for tag, r in (("split", rs), ("fp64", r6)):
            two[tag] = dict(summary(r), truncation=r["truncation"], max_bond_dim=r["max_bond_dim"])
        two["sweep_speedup"] = two["fp64"]["s_per_sweep"][0] / two["split"]["s_per_sweep"][0]
        two["trace_split_vs_fp64"] = step_trace(rs, r6)
        two["trace_fp64_vs_perturbed_fp64"] = step_trace(rc, r6)
        conv = dmrg2(ctx, model, mps_s, n_sweeps=3, Dmax=1024, precision=args.precision, refine_iters=10,
                     tol_eigval=1e-12, tol_state=1e-8)
        c64 = dmrg2(ctx, model, copy.deepcopy(mps_s), n_sweeps=1, Dmax=1024, precision="fp64", **tight)
        csp = dmrg2(ctx, model, copy.deepcopy(mps_s), n_sweeps=1, Dmax=1024, precision=args.precision,
                    refine_iters=10, probe=False, **tight)
        two["converging_split_E"] = conv["energies"]
        two["converged"] = {"fp64": dict(summary(c64), truncation=c64["truncation"]),
                            "split_no_probe": dict(summary(csp), truncation=csp["truncation"]),
                            "trace": step_trace(csp, c64),
                            "E_rel_diff": abs(csp["energies"][-1] - c64["energies"][-1]) / abs(c64["energies"][-1])}
        out["hubbard_L64_D1024_two_site"] = two
    if args.D >= 4096 and not args.no_window:
        # two-site DMRG at D=4096: a window of bonds around the middle of the chain
        # (4 bonds to the right and back, 8 two-site steps), in each precision from
        # the same seeded MPS; a full sweep at this D is 126 such steps
        from vmps_gb300.dmrg import dmrg2
        model = models.hubbard_u1xu1(64, t=1.0, U=4.0)
        lo, width = 31, 4
        mps0 = RandomMPS(model, (64, 0), 4096, seed=args.seed, profile="gaussian",
                         sigma=[2.5, 2.5]).canonicalize(lo, lo + 1)
        win = {"window": [lo, lo + width], "steps": 2 * width, "Dmax": 4096,
               "tolerances": dict(refine_iters=3, tol_eigval=1e-10, tol_state=1e-6)}
        runs = {}
        for tag, prec, kw in (("split", args.precision, dict(refine_iters=3)), ("fp64", "fp64", {})):
            r = dmrg2(ctx, model, copy.deepcopy(mps0), n_sweeps=1, Dmax=4096, precision=prec,
                      tol_eigval=1e-10, tol_state=1e-6, window=(lo, lo + width), **kw)
            runs[tag] = r
            win[tag] = dict(summary(r), s_per_step=r["sweep_times"][0] / (2 * width), truncation=r["truncation"])
        win["E_rel_diff"] = abs(win["split"]["E"][-1] - win["fp64"]["E"][-1]) / abs(win["fp64"]["E"][-1])
        win["trace"] = step_trace(runs["split"], runs["fp64"])
        win["step_speedup"] = win["fp64"]["s_per_step"] / win["split"]["s_per_step"]
        out["hubbard_L64_D4096_two_site_window"] = win
    return out


def su2_cylinder_bench(ctx, args):
    """Config C3: Hubbard SU(2)xU(1), width-4 cylinder as a 64-site snake, U/t=8, 1/8 hole
    doping (N=56, S=0), MPO w=10, D=2000 multiplets (~5,800 states); the two-site pivot of
    the middle.  Device-resident HxV (CUDA graph, events) in FP64 and split precision, the
    split error, the Lanczos ground state of the pivot in both precisions, one single-site
    DMRG sweep of the cylinder in each precision and two-site DMRG (SU(2) two-site
    contraction and split) over a window of the middle in each precision."""
    from vmps_gb300.pivot import DeviceVector, PivotMatrix2, time_hxv
    from vmps_gb300.workloads import hubbard_su2xu1_cylinder_two_site
    model, mps, Lenv, Renv, W1, W2, V, info = hubbard_su2xu1_cylinder_two_site(ctx)
    H = PivotMatrix2(ctx, model.sym, Lenv, Renv, W1, W2, V)
    st64, sts = H.stats("fp64"), H.stats(args.precision)
    a, b = DeviceVector(H, V.data), DeviceVector(H)
    for p in ("fp64", args.precision):
        time_hxv(H, a, b, p, n_iter=3)
    ms64, _ = time_hxv(H, a, b, "fp64", n_iter=10)
    mss, _ = time_hxv(H, a, b, args.precision, n_iter=50)
    a.close()
    b.close()
    h64, hs = H.apply(V.data, "fp64"), H.apply(V.data, args.precision)
    err = float(np.linalg.norm(hs - h64) / np.linalg.norm(h64))
    v0 = np.random.default_rng(7).standard_normal(H.dim)
    tol = dict(tol_eigval=1e-10, tol_state=1e-6)
    e64, _, l64 = H.lanczos(v0, "fp64", max_iter=300, **tol)
    es, _, ls = H.lanczos(v0, args.precision, max_iter=300, refine_iters=4, **tol)
    H.close()
    orc = None
    if not args.no_cpu:
        # the same pivot on the oracle's SU(2) restatement: both HxVs of V, and the
        # ground-state energy from the oracle's Lanczos on the dot-weighted operator
        import oracle
        oracle.set_threads(os.cpu_count() or 1)
        op = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, W1, W2, sym=model.sym)
        t0 = time.perf_counter()
        ref = op.hxv(V.data)
        w = oracle.dot_weights(V, model.sym)
        e_or, steps = oracle.lanczos_ground(lambda x: w * op.hxv(x / w), w * v0, tol=1e-14)
        orc = {"hxv_fp64_rel_err": float(np.linalg.norm(h64 - ref) / np.linalg.norm(ref)),
               "hxv_split_rel_err": float(np.linalg.norm(hs - ref) / np.linalg.norm(ref)),
               "E_oracle": e_or, "oracle_lanczos_steps": steps, "oracle_s": round(time.perf_counter() - t0, 1),
               "E_fp64_rel_err": abs(e64 - e_or) / abs(e_or), "E_split_rel_err": abs(es - e_or) / abs(e_or)}
    # single-site DMRG sweep of the cylinder: one sweep in each precision from the same
    # seeded MPS (D=2000 multiplets, centre on site 0)
    import copy

    from vmps_gb300.dmrg import dmrg1
    from vmps_gb300.mps import RandomMPS
    mps0 = RandomMPS(model, (1, info["N"]), 2000, seed=3, profile="gaussian", sigma=[3.0, 3.0]).canonicalize(0, 0)
    sweep, runs = {}, {}
    for tag, prec, kw in (("split", args.precision, dict(refine_iters=10)), ("fp64", "fp64", {})):
        r = dmrg1(ctx, model, copy.deepcopy(mps0), n_sweeps=1, precision=prec, **tol, **kw)
        runs[tag] = r
        sweep[tag] = {"s_per_sweep": r["sweep_times"], "E": r["energies"], "lanczos": r["solves"],
                      "timers_s": [{k: round(v, 4) for k, v in t.items()} for t in r["timers"]]}
    sweep["trace"] = step_trace(runs["split"], runs["fp64"])
    sweep["sweep_speedup"] = sweep["fp64"]["s_per_sweep"][0] / sweep["split"]["s_per_sweep"][0]
    # two-site DMRG (SU(2) contract_AA2 / split_AA2) over a window of four bonds in the middle
    # (eight steps), from the same seeded MPS in each precision, Dmax = 2000 multiplets
    from vmps_gb300.dmrg import dmrg2
    lo, hi = 30, 34
    mps1 = RandomMPS(model, (1, info["N"]), 2000, seed=3, profile="gaussian", sigma=[3.0, 3.0]).canonicalize(lo, lo + 1)
    two, runs2 = {}, {}
    for tag, prec, kw in (("split", args.precision, dict(refine_iters=10)), ("fp64", "fp64", {})):
        r = dmrg2(ctx, model, copy.deepcopy(mps1), n_sweeps=1, Dmax=2000, precision=prec, window=(lo, hi), **tol, **kw)
        runs2[tag] = r
        two[tag] = {"s": r["sweep_times"][0], "E": r["energies"][-1], "lanczos": r["solves"],
                    "timers_s": {k: round(v, 4) for k, v in r["timers"][0].items()}}
    two["window"] = [lo, hi]
    two["steps"] = 2 * (hi - lo)
    two["trace"] = step_trace(runs2["split"], runs2["fp64"])
    two["step_speedup"] = two["fp64"]["s"] / two["split"]["s"]
    return dict(info, n_tasks=st64["n_tasks"], flops_per_hxv=st64["flops_merged"], single_site_sweep=sweep,
                two_site_window=two,
                hxv_fp64={"ms": ms64, "per_s": 1e3 / ms64, "tflops": st64["flops_merged"] / ms64 * 1e-9},
                hxv_split={"ms": mss, "per_s": 1e3 / mss, "tflops_useful": sts["flops_merged"] / mss * 1e-9,
                           "tensor_tflops_issued": (sts["tensor_flops_phase1"] + sts["tensor_flops_phase2"]) /
                           mss * 1e-9},
                split_over_fp64=ms64 / mss, hxv_split_rel_err=err,
                oracle=orc,
                lanczos={"E_fp64": e64, "E_split": es, "rel_diff": abs(es - e64) / abs(e64),
                         "ms_fp64": l64["ms_total"], "ms_split": ls["ms_total"],
                         "hxv_fp64": l64["hxv_fp64"], "split_hxv": [ls["hxv_split"], ls["hxv_fp64"]]})


def vumps_bench(ctx, args):
    """Config C4: the spin-1/2 Heisenberg chain with SU(2) as a uniform MPS: a seeded random
    N(0,1) state with 512 multiplets per bond, gauge fixed (AL C = C AR).  A one-site cell
    cannot carry it (the bond spin alternates between integer and half-integer), so the
    cell has two sites.  Times and reports, in FP64 and in split precision: the MPO
    environments (the triangular slot build, GMRES on the transfer operator for the
    identity slots), the energy density and the VUMPS gradient norm |H_AC(AC) - AL H_C(C)|,
    each against the same steps on the oracle; the transfer-operator application and the
    H_AC / H_C HxVs alone."""
    from vmps_gb300 import models
    from vmps_gb300.pivot import DeviceVector, PivotMatrix0, PivotMatrix1, time_hxv
    from vmps_gb300.uniform import UniformEnvironment, UniformMPS, bond_bases_su2
    from vmps_gb300.vumps import MpoTransferMatrix
    m = models.heisenberg_su2(8)
    order, W = m.basis_order_map(4), [m.W[4], m.W[5]]
    dims = bond_bases_su2(512, 20)
    t0 = time.perf_counter()
    u = UniformMPS(m, dims, seed=4)
    g = u.gauge()
    out = {"multiplets_per_bond": [sum(d.values()) for d in dims],
           "states_per_bond": [sum(q[0] * n for q, n in d.items()) for d in dims], "cell": 2,
           "gauge": dict(g, s=round(time.perf_counter() - t0, 2))}
    res = {}
    for prec in ("fp64", args.precision):
        E = UniformEnvironment(ctx, m, u, W, order, precision=prec, tol=1e-12)
        t0 = time.perf_counter()
        E.left()
        E.right()
        t1 = time.perf_counter()
        gn, parts = E.gradient()
        t2 = time.perf_counter()
        # the same environments with the host GMRES loop over device operator applications
        Eh = UniformEnvironment(ctx, m, u, W, order, precision=prec, tol=1e-12, solver="host")
        t3 = time.perf_counter()
        Eh.left()
        Eh.right()
        t4 = time.perf_counter()
        res[prec] = {"e": E.energy_density(), "gradient_norm": gn, "environments_s": round(t1 - t0, 3),
                     "gradient_s": round(t2 - t1, 3), "gmres": E.info, "solver": "device",
                     "environments_s_host_gmres": round(t4 - t3, 3),
                     "host_gmres_e_rel_diff": abs(Eh.energy_density() - E.energy_density()) / abs(E.energy_density())}
        if prec == "fp64":
            E64 = E
    out["environments"] = res
    if not args.no_cpu:
        import oracle
        from oracle.vumps_cpu import transfer_hxv
        oracle.set_threads(os.cpu_count() or 1)
        sym = m.sym

        def env(side, mode, fixed_ab, order_, Eo, Abra, Wl, Aket):
            return oracle.OracleEnv(side, sym.nq, Eo, Abra, Wl, Aket, mode=mode, fixed_ab=fixed_ab, order=order_,
                                    sym=sym).run(Eo, Abra, Aket)

        class OracleTransfer(MpoTransferMatrix):
            def __init__(self, side, A, Wl, LR, ab, order_, V):
                self.sym, self.V, self.ab = sym, V, ab
                self.ab_key = {v: k for k, v in order_.items()}[ab]
                self.args = (side, A, Wl, LR, ab, order_)

            def hxv(self, vin, precision="fp64"):
                side, A, Wl, LR, ab, order_ = self.args
                return transfer_hxv(side, sym.nq, A, A, Wl, LR, ab, order_, self.V, vin, sym.dot_weight, sym=sym)

            def close(self):
                pass

        def transfer(side, A, Wl, LR, ab, order_, V, b):
            return OracleTransfer(side, A, Wl, LR, ab, order_, V).solve_linear(b, tol=1e-12, dimK=100)

        def apply(kind, L, R, Wl, V, x):
            if kind == 1:
                return oracle.OraclePivot(1, sym.nq, L, R, V, Wl, sym=sym).hxv(x)
            return oracle.OraclePivot(0, sym.nq, L, R, V, sym=sym).hxv(x)
        t0 = time.perf_counter()
        ref = UniformEnvironment(None, m, u, W, order, env=env, transfer=transfer, apply=apply)
        ref.left()
        ref.right()
        g_ref, _ = ref.gradient()
        e_ref = ref.energy_density()
        out["oracle"] = {"e": e_ref, "gradient_norm": g_ref, "s": round(time.perf_counter() - t0, 1)}
        for prec, r in res.items():
            r["e_rel_err_vs_oracle"] = abs(r["e"] - e_ref) / abs(e_ref)
            r["gradient_rel_err_vs_oracle"] = abs(r["gradient_norm"] - g_ref) / g_ref
    # the pieces alone: transfer operator (left, identity slot) and H_AC / H_C HxVs
    R = {q: M @ M.T for q, M in u.C[0].items()}
    V = E64._identity(E64.last).like()
    T = MpoTransferMatrix(ctx, m.sym, "L", u.AL, u.AL, W, E64._blocks_of(R), E64.last, order, V)
    v = np.random.default_rng(5).standard_normal(V.data.size)
    for p in ("fp64", args.precision):
        T.hxv(v, p)
        t0 = time.perf_counter()
        for _ in range(5):
            T.hxv(v, p)
        out[f"transfer_hxv_ms_{p}"] = (time.perf_counter() - t0) / 5 * 1e3
    T.close()
    L1 = E64.env("L", "FULL", 0, order, E64.L, u.AL[0], W[0], u.AL[0])
    HAC = PivotMatrix1(ctx, m.sym, E64.L, E64.env("R", "FULL", 0, order, E64.R, u.AR[1], W[1], u.AR[1]), W[0], u.AC[0])
    HC = PivotMatrix0(ctx, m.sym, L1, E64.env("R", "FULL", 0, order, E64.R, u.AR[1], W[1], u.AR[1]), u.C_blocks(1))
    for name, H, vec in (("hac", HAC, u.AC[0].data), ("hc", HC, u.C_blocks(1).data)):
        a, bb = DeviceVector(H, vec), DeviceVector(H)
        for p in ("fp64", args.precision):
            time_hxv(H, a, bb, p, n_iter=3)
            out[f"{name}_hxv_ms_{p}"] = time_hxv(H, a, bb, p, n_iter=20)[0]
        out[f"{name}_dim"] = H.dim
        a.close()
        bb.close()
        H.close()
    return out


def chebyshev_bench(ctx, args):
    """Config C5: Hubbard L=64, U=4, U(1)xU(1); ground state |0> at D=512 (two-site DMRG
    from a seeded random MPS); the two-site pivot of the middle.  Start vectors: the
    momentum-resolved P c_{k,s}|0> (standing waves k = pi n/65 of the open chain, 16
    momenta, both spins: 32 vectors in two quantum-number layouts, (N-1, 2Sz=-1) and
    (N-1, +1); vmps_gb300.spectral), advanced together on the union pivot of the two
    sectors (one grouped HxV per step for all 32) for N=1000 Chebyshev moments of the
    rescaled H in [-1, 1] (2 % margin).  Moments accumulate in FP64; every moment's error
    of the split-precision run is taken against the FP64 run, relative to mu_0; the budget
    is stated on what the moments are for, the KPM spectral density of each start vector
    (Jackson kernel): within 1 % of the FP64 density (max over frequencies, relative to its
    maximum).  The split HxV's error enters every step and the recursion carries it on, so
    the per-moment error grows about linearly in n."""
    from vmps_gb300 import models
    from vmps_gb300.dmrg import dmrg2
    from vmps_gb300.mps import RandomMPS
    from vmps_gb300.pivot import PivotMatrix2
    from vmps_gb300.spectral import SpectralPivot
    L, D, l, nk, nmom = 64, 512, 31, 16, 1000
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    t0 = time.perf_counter()
    mps = RandomMPS(model, (L, 0), D, seed=5, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(0, 0)
    gs = dmrg2(ctx, model, mps, n_sweeps=3, Dmax=D, precision=args.precision, tol_eigval=1e-11, tol_state=1e-7,
               refine_iters=10)
    t_gs = time.perf_counter() - t0
    mps.canonicalize(l, l + 1)
    t0 = time.perf_counter()
    sp = SpectralPivot(ctx, model, mps, l)
    ns = [int(round((m + 0.5) * L / nk)) for m in range(nk)]
    X = {s: sp.start_vectors(ns, s) for s in ("up", "dn")}
    U = sp.union()
    t_start = time.perf_counter() - t0
    Xu = U.join([X["up"], X["dn"]])
    nk_up = [float(v @ v) for v in X["up"]]   # <0| c+_k c_k |0> on the pivot: momentum distribution
    # bounds of the whole spectrum (a random start reaches every eigenvector; start vectors
    # of c_k|0> hold little weight at the top, and T_n grows outside [-1, 1])
    lo, hi = U.H.spectral_bounds(np.random.default_rng(7).standard_normal(U.H.dim), iters=160)
    a, b = (hi - lo) / (2 * 0.98), (hi + lo) / 2
    mu64, s64 = U.chebyshev_moments(Xu, nmom, a, b, "fp64")
    mus, ss = U.chebyshev_moments(Xu, nmom, a, b, args.precision)
    rel = np.abs(mus - mu64) / np.maximum(np.abs(mu64[..., :1]), 1e-300)   # per vector, part, moment
    err = rel.reshape(-1, nmom).max(axis=0)
    # the same work without the union: each sector's pivot with its 16 vectors, two launches per step
    sep = 0.0
    for p, spin in enumerate(("up", "dn")):
        Lp, Rp, Vp = sp.sector(spin)
        Hp = PivotMatrix2(ctx, model.sym, Lp, Rp, model.W[l], model.W[l + 1], Vp)
        _, sp_ = Hp.chebyshev_moments(X[spin], nmom, a, b, args.precision)
        sep += sp_["ms_device"]
        Hp.close()
    mut, st32 = U.chebyshev_moments(Xu, nmom, a, b, "tf32x3")
    # what the moments are for: the KPM spectral density of each start vector (Jackson kernel
    # of order m), rho(w) = (g_0 mu_0 + 2 sum_{n<m} g_n mu_n T_n(w)) / (pi sqrt(1 - w^2)), on
    # 2000 Chebyshev nodes; its error against the FP64 density, max over frequencies relative
    # to the density's maximum, worst of the 32 vectors
    w = np.cos(np.pi * (np.arange(2000) + 0.5) / 2000)
    Tn = np.cos(np.outer(np.arccos(w), np.arange(nmom)))   # T_n(w), 2000 x nmom

    def density(mu, m):
        nn = np.arange(m)
        g = ((m - nn + 1) * np.cos(np.pi * nn / (m + 1)) + np.sin(np.pi * nn / (m + 1)) / np.tan(np.pi / (m + 1))) / (m + 1)
        cw = g * np.where(nn == 0, 1.0, 2.0)
        return (mu.reshape(-1, nmom)[:, :m] * cw) @ Tn[:, :m].T / (np.pi * np.sqrt(1 - w * w))

    def dens_err(mu, m):
        r64, r = density(mu64, m), density(mu, m)
        return float((np.abs(r - r64).max(axis=1) / np.abs(r64).max(axis=1)).max())
    orders = [50, 100, 200, 500, 1000]
    dens = {"bf16x3": {m: dens_err(mus, m) for m in orders}, "tf32x3": {m: dens_err(mut, m) for m in orders}}
    errt = (np.abs(mut - mu64) / np.maximum(np.abs(mu64[..., :1]), 1e-300)).reshape(-1, nmom).max(axis=0)
    budget = 1e-2
    dens_err_full = dens[args.precision][nmom] if args.precision in dens else dens["bf16x3"][nmom]
    out = {"workload": "hubbard_u1xu1_L64_D512_ground_state_two_site_middle_c_k",
           "ground_state": {"E": float(gs["energies"][-1]), "sweeps": 3, "Dmax": D, "s": round(t_gs, 2)},
           "start_vectors": {"momenta_n": ns, "spins": ["up", "dn"], "layouts": ["(63,-1)", "(63,+1)"],
                             "dims": U.dims, "n_k_up_on_pivot": nk_up, "s": round(t_start, 2)},
           "nrhs": int(Xu.shape[0]), "vectors": int(Xu.shape[0]) * 2, "nmom": nmom,
           "spectrum": [lo, hi], "a": a, "b": b, "steps": ss["steps"],
           "split": {"ms_total_device": ss["ms_device"], "ms_per_step": ss["ms_per_step"],
                     "hxv_per_s": 2 * ss["hxv"] / (ss["ms_device"] * 1e-3)},
           "fp64": {"ms_total_device": s64["ms_device"], "ms_per_step": s64["ms_per_step"],
                    "hxv_per_s": 2 * s64["hxv"] / (s64["ms_device"] * 1e-3)},
           "split_speedup": s64["ms_device"] / ss["ms_device"],
           "separate_sectors_split_ms_total": sep, "union_gain": sep / ss["ms_device"],
           "kpm_density_rel_err_vs_fp64": {"budget": budget, "within_budget": bool(dens_err_full <= budget),
                                           "max": dens_err_full, "kernel": "Jackson", "points": 2000,
                                           "by_order": {k: {str(m): v for m, v in d.items()} for k, d in dens.items()},
                                           "orders_within_budget": {k: [m for m, v in d.items() if v <= budget]
                                                                    for k, d in dens.items()}},
           "tf32x3": {"ms_per_step": st32["ms_per_step"], "ms_total_device": st32["ms_device"],
                      "moment_rel_err_max": float(errt.max()), "n=999": float(errt[999])},
           "moment_rel_err_vs_fp64": {"max": float(err.max()), "n=1": float(err[1]), "n=10": float(err[10]),
                                      "n=100": float(err[100]), "n=500": float(err[500]), "n=999": float(err[999])}}
    U.close()
    return out


def mps_chebyshev_bench(ctx, args):
    """The Chebyshev recursion of whole MPS (MpsCompressor::polyCompress, solvers/
    MpsCompressor.h:1372-1564, in polyIter, DmrgLinearAlgebra.h:550-566): Hubbard L=32,
    U=4, U(1)xU(1); ground state |0> at D=384 (two-site DMRG, FP64); start vector
    c_{k,up}|0> (k = pi 8/33) fitted as an MPS of charge (31, -1) from a seeded random MPS
    (two sweeps); then t_{n+1} = 2 H' t_n - t_{n-1}, H' = (H - b)/a, each vector fitted by
    one two-site sweep of at most 384 states per bond (vmps_gb300.compress: per step one
    tagged two-site application per distinct source MPS, H t_n and t_n as one summed MPO,
    contract_L / contract_R between the fitted and the source MPS, the truncated split
    through the Gram matrix on the device, singular values below 1e-7 of the largest
    dropped), 16 moments in FP64 and in split precision.  The bounds: E_0 of the ground
    state and -E_0(-H) in the (31, -1) sector (DMRG at D=64), 5 % margin.  The oracle
    (its contract_L / contract_R and two-site HxV on the host's cores) runs the first
    moment's fit from the same FP64 start vector."""
    from vmps_gb300 import models
    from vmps_gb300.compress import Compressor, copy_mps
    from vmps_gb300.dmrg import dmrg2
    from vmps_gb300.mps import RandomMPS
    from vmps_gb300.spectral import annihilator, annihilator_mpo, standing_wave
    L, D, n, nmom, eps = 32, 384, 8, 16, 1e-7
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    t0 = time.perf_counter()
    gs = RandomMPS(model, (L, 0), D, seed=5).canonicalize(0, 0)
    E0 = float(dmrg2(ctx, model, gs, n_sweeps=3, Dmax=D, precision="fp64")["energies"][-1])
    dq = annihilator(model, "up")[1]
    Q = tuple(a + b for a, b in zip((L, 0), dq))
    neg = models.hubbard_u1xu1(L, t=-1.0, U=-4.0)
    top = RandomMPS(neg, Q, 64, seed=6).canonicalize(0, 0)
    Emax = -float(dmrg2(ctx, neg, top, n_sweeps=3, Dmax=64, precision="fp64")["energies"][-1])
    t_setup = time.perf_counter() - t0
    a, b = (Emax - E0) / (2 * 0.95), (Emax + E0) / 2
    W = annihilator_mpo(model, standing_wave(L, n), "up")

    def start(comp):
        psi0 = RandomMPS(model, Q, D, seed=17)
        return psi0, comp.fit(psi0, [(W, gs, 1.0)], Dmax=D, sweeps=2, eps_svd=eps)

    def moments(comp, psi0, nm):
        comp.applications = 0
        t0 = time.perf_counter()
        mu, info = comp.chebyshev_moments(psi0, nm, a, b, Dmax=D, sweeps=1, eps_svd=eps)
        dt = time.perf_counter() - t0
        return mu, {"s_total": round(dt, 3), "s_per_moment": dt / (nm - 1),
                    "two_site_applications": comp.applications, "discarded_max": max(info["discarded"]),
                    "max_bond": info["max_bond"]}
    res = {}
    for prec in ("fp64", args.precision):
        comp = Compressor(ctx, model, precision=prec, factor="eigh")
        t0 = time.perf_counter()
        psi0, d0 = start(comp)
        ts = time.perf_counter() - t0
        mu, r = moments(comp, psi0, nmom)
        res[prec] = dict(r, start_s=round(ts, 3), start_discarded=d0, mu_first=[float(x) for x in mu[:4]])
        if prec == "fp64":
            mu64, psi64 = mu, psi0
        else:
            res[prec]["moment_rel_err_vs_fp64"] = float(np.max(np.abs(mu - mu64)) / abs(mu64[0]))
    out = {"workload": "hubbard_u1xu1_L32_D384_c_k_up_mps_chebyshev", "E0": E0, "Emax_sector": Emax,
           "bounds_margin": 0.05, "setup_s": round(t_setup, 2), "nmom": nmom, "n_k": float(mu64[0]),
           "Dmax": D, "eps_svd": eps, "sweeps_per_moment": 1, "runs": res}
    if not args.no_cpu:
        import oracle
        oracle.set_threads(os.cpu_count() or 1)

        def env(side, E, Abra, Wl, Aket):
            return (oracle.contract_L if side == "L" else oracle.contract_R)(Wl.nq, E, Abra, Wl, Aket)

        def apply2(sym, Le, Re, W1, W2, V, x):
            return oracle.OraclePivot(2, sym.nq, Le, Re, V, W1, W2).hxv(x)
        comp = Compressor(None, model, env=env, apply2=apply2, factor="eigh")
        mu, r = moments(comp, copy_mps(psi64), 2)
        # the same sample on the engine (the fit of t_1 has one source MPS, later ones two)
        _, re = moments(Compressor(ctx, model, precision="fp64", factor="eigh"), copy_mps(psi64), 2)
        out["oracle"] = {"moments": 1, "s_per_moment": r["s_per_moment"], "threads": os.cpu_count() or 1,
                         "sample": "the fit of t_1 (one sweep) from the FP64 start vector",
                         "engine_fp64_s_same_sample": re["s_per_moment"],
                         "moment_rel_err_vs_engine_fp64": float(np.max(np.abs(mu - mu64[:2])) / abs(mu64[0])),
                         "speedup_engine_fp64": r["s_per_moment"] / re["s_per_moment"]}
    return out


def optional_row(name, fn):
    """one of the configuration rows beside the headline HxV: a failure is reported in the
    row (and on stderr) instead of ending the run before the headline line is printed"""
    try:
        return fn()
    except Exception as e:   # noqa: BLE001 -- reported, not swallowed
        import traceback
        traceback.print_exc()
        print(f"bench row {name} failed: {e!r}", file=sys.stderr, flush=True)
        return {"error": repr(e)}


def cpu_model():
    """CPU model string of the host (lscpu's "Model name", else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def loaded_native_libs():
    """shared libraries of this repository mapped into the process (from /proc/self/maps)"""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for ln in f:
                path = ln.split()[-1] if ln.strip() else ""
                if path.endswith(".so") and path.startswith(ROOT):
                    libs.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(libs)


def workload_config(args, info, world):
    """The `config` object of the bench line; both arms print the same one.  `l2` says
    how the timed region avoids L2 reuse: the two-site vectors (in + out) and the
    environments alone are larger than the 129 MB L2."""
    n = info["dim_V"]
    io_bytes = 2 * 8 * n + 8 * (info["env_elems"])
    return {"workload": f"hubbard_u1xu1_L{args.L}_D{args.D}_two_site_middle", "L": args.L, "D": args.D,
            "U": 4.0, "seed": args.seed, "D_left": info["D_left"], "sectors": info["sectors_left"], "dim_V": n,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2" if io_bytes > L2_BYTES else "inputs fit L2"}


def oracle_two_site_workload(L, D, seed, U=4.0, sigma=2.5):
    """The frozen two-site pivot of the bench built on the host only: the same seeded
    MPS (numpy QR/LQ normalisation), environments from the oracle's contract_L /
    contract_R, the two-site tensor from numpy block products.  No GPU and no
    engine library is touched."""
    import oracle
    from vmps_gb300 import models
    from vmps_gb300.mps import RandomMPS, contract_two_sites
    from vmps_gb300.blocks import Blocks
    model = models.hubbard_u1xu1(L, t=1.0, U=U)
    site = L // 2 - 1
    mps = RandomMPS(model, (L, 0), D, seed=seed, profile="gaussian", sigma=[sigma, sigma])
    mps.canonicalize(site, site + 1)
    sym, nq = model.sym, model.sym.nq
    v = sym.vacuum()
    Lenv = Blocks.from_entries(nq, [(0, v, v, v, np.ones((1, 1)))], tripod=True)
    for l in range(site):
        Lenv = oracle.contract_L(nq, Lenv, mps.A[l], model.W[l], mps.A[l])
    Renv = Blocks.from_entries(nq, [(0, (L, 0), (L, 0), v, np.ones((1, 1)))], tripod=True)
    for l in range(L - 1, site + 1, -1):
        Renv = oracle.contract_R(nq, Renv, mps.A[l], model.W[l], mps.A[l])
    V = contract_two_sites(sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, nq)
    info = dict(D_left=mps.bond_dim(site), sectors_left=len(mps.dims[site]), dim_V=int(V.data.size),
                env_elems=int(Lenv.data.size + Renv.data.size))
    return model, Lenv, Renv, model.W[site], model.W[site + 1], V, info


def run_reference(args):
    """CPU restatement of the reference path (the oracle), all host threads.  The
    inputs are made on the host with numpy and the oracle: this arm loads no GPU
    code and no engine library."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    model, L, R, W1, W2, V, info = oracle_two_site_workload(args.L, args.D, args.seed)
    setup_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    op = oracle.OraclePivot(2, 2, L, R, V, W1, W2)
    v = np.random.default_rng(5).standard_normal(V.data.size)
    for _ in range(args.warmup):
        op.hxv(v)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        op.hxv(v)
    dt = time.perf_counter() - t0
    rate = args.steps / dt
    line = {"metric": METRIC, "value": rate, "unit": "HxV/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(args, info, world),
            "cpu_baseline": {"value": rate, "unit": "HxV/s", "cores": threads, "kind": "port",
                             "cpu": cpu_model(), "sample": f"{args.steps} full HxV of the workload",
                             "gemm": oracle.blas_kind()},
            "e2e": {"value": rate, "unit": "HxV/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": round(setup_s, 2), "native_libs_loaded": loaded_native_libs()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--D", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--precision", default="bf16x3")
    ap.add_argument("--cpu-hxv", type=int, default=250,
                    help="HxV applications in the CPU-baseline sample (about 13 s on 16 cores)")
    ap.add_argument("--cpu-hxv-1t", type=int, default=12,
                    help="HxV applications in the single-thread CPU sample (about 10 s)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-energy", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-chebyshev", action="store_true")
    ap.add_argument("--no-su2", action="store_true")
    ap.add_argument("--no-vumps", action="store_true")
    ap.add_argument("--no-mps-chebyshev", action="store_true")
    ap.add_argument("--no-window", action="store_true", help="skip the D=4096 two-site window")
    ap.add_argument("--no-tune-small", action="store_true", help="skip the autotuner on the smaller pivots")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    if args.impl == "reference":
        run_reference(args)
        return

    rank, local, world, dist = dist_init()
    import __graft_entry__
    __graft_entry__.build()
    import ctypes as C
    import torch
    from vmps_gb300.pivot import Context, DeviceVector, PivotMatrix2, time_hxv
    from vmps_gb300.workloads import hubbard_two_site
    from vmps_gb300 import _native as N

    ctx = Context(local)
    model, mps, Lenv, Renv, W1, W2, V, info = hubbard_two_site(ctx, L=args.L, D=args.D, seed=args.seed)
    H = PivotMatrix2(ctx, model.sym, Lenv, Renv, W1, W2, V)
    # tile shape and split-K of the split plan: timed candidates on this pivot (autotuner)
    tune = H.autotune(trials=5) if args.precision == "bf16x3" else None
    st_split = H.stats(args.precision)
    st64 = H.stats("fp64")
    n = H.dim
    rng = np.random.default_rng(7)
    v0 = rng.standard_normal(n)
    vin = DeviceVector(H, v0)
    vout = DeviceVector(H, None)
    working_set = 2 * 8 * n + st_split["bytes_intermediate"] + 4 * (Lenv.data.size + Renv.data.size)
    l2_note = "inputs larger than L2" if working_set > L2_BYTES else "working set fits L2"

    # ---- device-resident HxV (value)
    time_hxv(H, vin, vout, args.precision, n_iter=args.warmup, use_graph=True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    torch.cuda.synchronize(local)
    ms, ms2 = time_hxv(H, vin, vout, args.precision, n_iter=args.steps, use_graph=True)
    torch.cuda.synchronize(local)
    barrier(dist)
    clk = clocks.stop()
    ms = reduce_max(dist, ms, local)
    value = world * 1000.0 / ms

    # ---- FP64 plain form
    n64 = max(3, args.steps // 5)
    time_hxv(H, vin, vout, "fp64", n_iter=2, use_graph=True)
    ms64, ms64_2 = time_hxv(H, vin, vout, "fp64", n_iter=n64, use_graph=True)
    ms64 = reduce_max(dist, ms64, local)

    # ---- e2e through the C ABI with pinned host buffers
    hin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    hout = torch.empty(n, dtype=torch.float64, pin_memory=True)
    hin.copy_(torch.from_numpy(v0))
    lib = N.lib()
    pin = C.cast(C.c_void_p(hin.data_ptr()), N.f64p)
    pout = C.cast(C.c_void_p(hout.data_ptr()), N.f64p)
    prec = 1 if args.precision == "bf16x3" else 0
    for _ in range(args.warmup):
        N.check(lib.vmps_hxv(H._h, pin, pout, prec))
    barrier(dist)
    torch.cuda.synchronize(local)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        N.check(lib.vmps_hxv(H._h, pin, pout, prec))
    torch.cuda.synchronize(local)
    e2e_s = reduce_max(dist, time.perf_counter() - t0, local)
    barrier(dist)
    e2e = world * args.steps / e2e_s

    # ---- the pivot's task list matched on the GPU (default) and on the host: pivot creation
    # (matching, plan-independent set-up, L/R upload) with each, median of 3
    builder = {}
    chains = {}
    for name, env in (("device", None), ("host", "1")):
        if env:
            os.environ["VMPS_HOST_BUILDER"] = env
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            Hb = PivotMatrix2(ctx, model.sym, Lenv, Renv, W1, W2, V)
            ts.append(time.perf_counter() - t0)
            chains[name] = Hb.chains()
            Hb.close()
        os.environ.pop("VMPS_HOST_BUILDER", None)
        builder[name + "_pivot_create_ms"] = 1e3 * float(np.median(ts))
    builder["chains"] = int(len(chains["device"][0]))
    builder["identical_chains"] = bool(np.array_equal(chains["device"][0], chains["host"][0]) and
                                       np.array_equal(chains["device"][1], chains["host"][1]) and
                                       chains["device"][2] == chains["host"][2])

    # ---- split vs FP64 numerics on this input
    h64 = H.apply(v0, "fp64")
    hsp = H.apply(v0, args.precision)
    hxv_rel_err = float(np.linalg.norm(hsp - h64) / np.linalg.norm(h64))

    # ---- the alternative split form (3xTF32): device-resident HxV and its error
    tf32 = None
    if args.precision == "bf16x3" and rank == 0:
        time_hxv(H, vin, vout, "tf32x3", n_iter=3, use_graph=True)
        mst, mst2 = time_hxv(H, vin, vout, "tf32x3", n_iter=args.steps, use_graph=True)
        htf = H.apply(v0, "tf32x3")
        st_tf = H.stats("tf32x3")
        tf32 = {"ms_per_hxv": mst, "hxv_per_s": 1000.0 / mst, "phase2_ms": mst2,
                "rel_err_vs_fp64": float(np.linalg.norm(htf - h64) / np.linalg.norm(h64)),
                "bf16x3_rel_err_vs_fp64": hxv_rel_err, "over_bf16x3_time": mst / ms,
                "tensor_flops_phase2": st_tf["tensor_flops_phase2"]}

    energy = None
    if not args.no_energy and rank == 0:
        # Lanczos ground state of this pivot from the same start vector: a tight
        # FP64 reference, then FP64 and split precision (+ refinement rounds:
        # FP64 residual, split Lanczos from it) at the sweep tolerances
        keys = ("iterations", "refine_iterations", "hxv_split", "hxv_fp64", "residual", "ms_total", "ms_wait")
        e_ref, _, s_ref = H.lanczos(v0, "fp64", max_iter=300, tol_eigval=1e-14, tol_state=1e-9)
        e64, x64, s64 = H.lanczos(v0, "fp64", max_iter=300, tol_eigval=1e-10, tol_state=1e-6)
        es, xs, ss = H.lanczos(v0, args.precision, max_iter=300, tol_eigval=1e-10, tol_state=1e-6, refine_iters=10)
        et, _, stt = H.lanczos(v0, "tf32x3", max_iter=300, tol_eigval=1e-10, tol_state=1e-6, refine_iters=10)
        energy = {"E_ref_fp64": e_ref, "tolerances": {"tol_eigval": 1e-10, "tol_state": 1e-6, "refine_iters": 10},
                  "fp64": dict({k: s64[k] for k in keys}, rel_err=abs(e64 - e_ref) / abs(e_ref)),
                  "split": dict({k: ss[k] for k in keys}, rel_err=abs(es - e_ref) / abs(e_ref),
                                energy_first_rel_err=abs(ss["energy_first"] - e_ref) / abs(e_ref)),
                  "split_speedup": s64["ms_total"] / ss["ms_total"],
                  "tf32x3": dict({k: stt[k] for k in keys}, rel_err=abs(et - e_ref) / abs(e_ref))}
        if not args.no_cpu and world == 1:
            energy["oracle"] = oracle_check(Lenv, Renv, V, W1, W2, v0, h64, hsp, e_ref, e64, es, x64, xs)

    # ---- roofline of the dominant kernel (the larger of the two grouped-GEMM phases)
    hbm, bf16, peak_kind = load_peaks()
    ms1 = max(ms - ms2, 1e-9)
    phase = "phase2" if ms2 >= ms1 else "phase1"
    flops_phase = st_split["flops_phase2"] if phase == "phase2" else st_split["flops_phase1"]
    t_phase = ms2 if phase == "phase2" else ms1
    tensor_flops = 3.0 * flops_phase / (t_phase * 1e-3) / 1e12     # bf16 tensor-core flops issued
    prof = None
    engine = "gg_umma_kernel"
    pf = os.path.join(ROOT, "profiles", f"{engine}_hubbard_D4096.json")
    if os.path.exists(pf):
        with open(pf) as f:
            prof = json.load(f)
    roofline = {"bound": "tensor", "achieved": tensor_flops, "peak": bf16, "unit": "TFLOP/s",
                "frac": tensor_flops / bf16, "traffic": (prof or {}).get(f"traffic_{phase}"),
                "traffic_commit": (prof or {}).get("commit"),
                "kernel": f"{engine} ({phase})", "peak_source": f"bf16_tflops of {peak_kind}",
                "useful_tflops": flops_phase / (t_phase * 1e-3) / 1e12,
                "issued_tflops": st_split[f"tensor_flops_{phase}"] / (t_phase * 1e-3) / 1e12,
                "note": "achieved: 3 bf16 products per useful FMA (hi*hi + hi*lo + lo*hi); issued: the MMAs "
                        "the engine runs, tile padding included"}

    sweep = None
    if not args.no_sweep and rank == 0:
        sweep = optional_row("dmrg_sweep", lambda: sweep_bench(ctx, args, with_cpu=not args.no_cpu and world == 1))
    cheb = None
    if not args.no_chebyshev and rank == 0:
        cheb = optional_row("chebyshev", lambda: chebyshev_bench(ctx, args))
    su2 = None
    if not args.no_su2 and rank == 0:
        su2 = optional_row("su2xu1_cylinder", lambda: su2_cylinder_bench(ctx, args))
    vum = None
    if not args.no_vumps and rank == 0:
        vum = optional_row("vumps_cell", lambda: vumps_bench(ctx, args))
    mcheb = None
    if not args.no_mps_chebyshev and rank == 0:
        mcheb = optional_row("mps_chebyshev", lambda: mps_chebyshev_bench(ctx, args))

    tune_small = None
    if rank == 0 and args.precision == "bf16x3" and not args.no_tune_small:
        tune_small = optional_row("autotune_small", lambda: autotune_small(ctx))

    cpu = None
    if not args.no_cpu and world == 1 and rank == 0:
        threads = os.cpu_count() or 1
        rate, dt, gemm = cpu_oracle_hxv_rate(Lenv, Renv, V, W1, W2, threads, args.cpu_hxv)
        rate1, dt1, _ = cpu_oracle_hxv_rate(Lenv, Renv, V, W1, W2, 1, args.cpu_hxv_1t)
        cpu = {"value": rate, "unit": "HxV/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
               "sample": f"{args.cpu_hxv} full HxV of the workload ({dt:.1f} s)", "gemm": gemm,
               "flops_per_hxv": st_split["flops_reference"],
               "single_thread": {"value": rate1, "unit": "HxV/s", "cores": 1,
                                 "sample": f"{args.cpu_hxv_1t} full HxV ({dt1:.1f} s)"}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "HxV/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3->f32 (f64 vectors)", "data": "synthetic",
            "config": workload_config(args, info, world),
            "timing": {"working_set_MB": round(working_set / 2 ** 20, 1), "l2_note": l2_note,
                       "graph": "CUDA graph per HxV (vector split + 2 grouped-GEMM launches)"},
            "e2e": {"value": e2e, "unit": "HxV/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n},
            "gpu_launches": ((3 + (1 if tune and tune["splitk"] > 1 else 0)) if args.precision == "bf16x3" else 2)
                            * args.steps,
            "autotune": {"headline_pivot": tune, "small_pivots": tune_small},
            "task_builder": builder,
            "fp64": {"value": world * 1000.0 / ms64, "unit": "HxV/s", "ms_per_step": ms64,
                     "phase2_ms": ms64_2, "flops_executed": st64["flops_executed"]},
            "split_over_fp64": ms64 / ms,
            "hxv_split_rel_err_vs_fp64": hxv_rel_err,
            "tf32x3": tf32,
            "energy": energy,
            "plan": {k: st_split[k] for k in ("n_tasks", "n_chains", "n_intermediates", "n_out_blocks",
                                              "n_tiles_phase1", "n_tiles_phase2", "flops_reference",
                                              "flops_merged", "flops_executed", "flops_phase1", "flops_phase2",
                                              "bytes_intermediate")},
            "phase_ms": {"phase1": ms1, "phase2": ms2},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "dmrg_sweep": sweep,
            "chebyshev": cheb,
            "su2xu1_cylinder": su2,
            "vumps_cell": vum,
            "mps_chebyshev": mcheb,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    vin.close()
    vout.close()
    H.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
