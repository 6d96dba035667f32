"""Benchmark: Chebyshev probe-steps/s (N*M*S per solve / time) of the GB300 KPM engine.

Workload (one "step" = one solve): Kondo-lattice-style cubic lattice L=64
(262,144 sites, 2x2 complex spin blocks, N = 524,288 scalar rows,
nnzb = 1,835,008), M = 1000 Chebyshev moments, S = 256 probe columns; the solve
is moments(M) followed by autodiff_matrix(c, D) on H's pattern, with c the
zero-temperature Fermi-energy expansion. Synthetic seeded data: random unit
spins, seeded unit-phase colour probes. Every vector (N x S x 16 B = 2 GiB) is
far larger than the 129 MB L2, so no L2 flush is needed between steps.

  value  device-resident throughput: H and R already on the GPU, solves enqueued
         back to back, timed with CUDA events on the engine's stream.
  e2e    the same metric through the public API with host buffers: every step
         uploads H and the colour probes' nonzeros (set_R_sparse) from pinned host
         memory and reads back mu and D; e2e_dense_R does the same with the dense
         n x S probe block (set_R, what the reference's transfer_R moves).
  roofline        HBM roofline of the dominant kernel (the fused adjoint step):
                  algorithmic bytes per launch / live CUDA-event launch time.
  roofline_issue  (float-float) the same launch against the GPU's warp-instruction
                  issue rate, from the ncu instruction count of the L=32 capture.
  --impl reference: the reference's CPU engine restated (oracle port), all host
         threads, each step a bounded sample (same workload, smaller M).
Multi-GPU (torchrun): replicas only -- every rank solves its own copy; value is
the sum over ranks divided by the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Chebyshev probe-steps/s (N*M*S per solve: moments + autodiff_matrix), err vs FP64 stated"
UNIT = "probe-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="ds", choices=["ds", "fp64", "fp32"])
    p.add_argument("--L", type=int, default=64)
    p.add_argument("--M", type=int, default=1000)
    p.add_argument("--S", type=int, default=256)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-M", type=int, default=8)
    p.add_argument("--workload", default="solve", choices=["solve", "precision", "batch", "serve", "cfg1", "square"])
    p.add_argument("--serve-requests", type=int, default=24)
    p.add_argument("--serve-max-sites", type=float, default=1e6)
    return p.parse_args()


# ---------------------------------------------------------------------------- dist
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        return rank, ws, dist
    return 0, 1, None


def replica_value(per_solve, steps, ws, ms_max):
    """Whole-job rate of N replicas: every rank's solves over the slowest rank's time."""
    return per_solve * steps * ws / (ms_max / 1e3)


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------- workload
def workload(args):
    from fastkpm_gb300 import workloads as W
    cfg = W.config2(L=args.L, S=args.S)
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], cfg["realisations"], cfg["probe_seed"])
    R = R[:, :args.S] if R.shape[1] > args.S else R
    c = W.fermi_coefficients(args.M, es, "fermi_energy")
    return H, es, np.asfortranarray(R), c


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def adjoint_bytes_per_launch(N, S, nnzb, b, sv, fused):
    """Algorithmic bytes of one adjoint launch (the kernel walks all S columns itself): read alpha_m,
    alpha_{m+1}, beta_{m+1}, beta_{m+2}, write alpha_{m-1}, beta_m (6 vectors), H once (entries +
    4-byte column index), row_ptr, and, when the D epilogue is fused, the D accumulator read + write
    (8 bytes per real: double or float-float)."""
    vec = 6 * N * S * sv
    h = nnzb * (b * b * sv + 4) + 4 * (N // b + 1)
    d = 2 * nnzb * b * b * 16 if fused else 0
    return vec + h + d


# DRAM bytes per row of one fused DS adjoint launch (k_adjoint_pipe) from the ncu capture on the
# cubic L=32 case (profiles/k_adjoint_step_ds_cubic32.md: 1.600 GB read + 0.530 GB written for
# 65,536 rows); traffic grows in proportion to the rows, so the L=64 launch's traffic is this times N.
ADJ_DS_TRAFFIC_PER_ROW = (1.600211e9 + 0.529769e9) / 65536
# Warp instructions per row of the same launch (smsp__inst_executed.sum = 1,108,457,856 for 65,536
# rows): the fused float-float adjoint is bound by instruction issue, not by DRAM. Issue peak of
# the GPU: 152 SMs x 4 schedulers x 1 warp instruction per cycle at the maximum SM clock.
ADJ_DS_WARP_INST_PER_ROW = 1108457856 / 65536
ISSUE_PEAK_WARP_INST_PER_CYCLE = 152 * 4


def probe_entries(R):
    """Nonzeros of a probe block, k per row (k = the most any row has; shorter rows padded with
    column 0 and value 0, which adds nothing): (s, cols (n, k), vals (n, k))."""
    nz = R != 0
    k = max(1, int(nz.sum(axis=1).max()))
    n = R.shape[0]
    cols = np.zeros((n, k), np.int32)
    vals = np.zeros((n, k), R.dtype)
    rows, cs = np.nonzero(nz)
    slot = np.arange(len(rows)) - np.searchsorted(rows, rows)
    cols[rows, slot] = cs
    vals[rows, slot] = R[rows, cs]
    return R.shape[1], cols, vals


def run_e2e(args, fk, Lb, H, es, R, c, D, M, per_solve, ws, dist, dev, sparse):
    """moments + autodiff_matrix through the public API, every step uploading H and the probes
    from pinned host memory and reading mu and D back; wall and device clocks, max over ranks."""
    lib = Lb.load()
    hv = np.ascontiguousarray(H.val)
    if sparse:
        s, cols, vals = probe_entries(R)
        cols = np.ascontiguousarray(cols)
        vals = np.ascontiguousarray(vals)
        probe_bufs = [cols, vals]
    else:
        Rf = np.asfortranarray(R)
        probe_bufs = [Rf]
    pinned = all(lib.fk_host_register(b.ctypes.data, b.nbytes) == 0 for b in probe_bufs + [hv])
    e2 = fk.Engine(True, args.precision, device=dev)

    def set_probes():
        if sparse:
            e2.set_R_sparse(R.shape[0], s, cols, vals)
        else:
            e2.set_R(Rf)

    e2.set_H(H, es)
    set_probes()
    e2.moments(M)
    e2.autodiff_matrix(c, D)
    barrier(dist)
    e2.synchronize()
    phases = np.zeros(4)   # wall ms per step: set_H, set_R, moments (+ mu read), autodiff (+ D read)
    t0 = time.perf_counter()
    e2.timer_start()
    for _ in range(args.steps):
        tp = [time.perf_counter()]
        e2.set_H(H, es)
        tp.append(time.perf_counter())
        set_probes()
        tp.append(time.perf_counter())
        e2.moments(M)
        tp.append(time.perf_counter())
        e2.autodiff_matrix(c, D)
        tp.append(time.perf_counter())
        phases += np.diff(tp) * 1e3
    e2_ms_dev = e2.timer_stop()
    e2_ms_wall = (time.perf_counter() - t0) * 1e3
    barrier(dist)
    e2_ms = max_over_ranks(dist, max(e2_ms_dev, e2_ms_wall))
    h2d = int(H.row_ptr.nbytes + H.col_idx.nbytes + hv.nbytes + sum(b.nbytes for b in probe_bufs))
    d2h = int(M * 8 + D.val.nbytes)
    for b in probe_bufs + [hv]:
        lib.fk_host_unregister(b.ctypes.data)
    e2.close()
    return {"value": per_solve * args.steps * ws / (e2_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": e2_ms / args.steps, "host_buffers_pinned": pinned,
            "probes": "nonzeros (set_R_sparse)" if sparse else "dense n x S (set_R)",
            "phases_ms_per_step": {k: float(v) / args.steps for k, v in
                                   zip(["set_H", "set_R", "moments", "autodiff_matrix"], phases)}}


# ---------------------------------------------------------------------------- arms
def run_gb300(args, rank, ws, dist):
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import _lib as Lb
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    H, es, R, c = workload(args)
    N, S, M = R.shape[0], R.shape[1], args.M
    D = H.pattern_like(True)
    eng = fk.Engine(True, args.precision, device=dev)
    eng.set_H(H, es)
    eng.set_R(R)
    per_solve = float(N) * M * S

    # ---- device-resident throughput ----
    for _ in range(args.warmup):
        eng.moments_async(M)
        eng.autodiff_matrix_async(c, D)
    eng.synchronize()
    eng.set_profiling(1)
    eng.profile_reset()
    barrier(dist)
    eng.synchronize()
    with ClockSampler(dev) as clk:
        eng.timer_start()
        for _ in range(args.steps):
            eng.moments_async(M)
            eng.autodiff_matrix_async(c, D)
        ms = eng.timer_stop()
    eng.synchronize()
    barrier(dist)
    prof = {k: eng.profile(k) for k in range(4)}
    eng.set_profiling(0)
    ms_max = max_over_ranks(dist, ms)
    value = replica_value(per_solve, args.steps, ws, ms_max)
    mu = eng.fetch_moments(M)
    eng.fetch_D(D)

    # roofline of the dominant kernel (the adjoint step)
    n_adj, t_adj = prof[1]
    n_step, t_step = prof[0]
    sv = 8 if args.precision == "fp32" else 16
    fuse_opt = eng.get_option(Lb.FK_OPT_FUSE_D)
    fused = fuse_opt != 0
    bytes_adj = adjoint_bytes_per_launch(N, S, H.n_blocks(), 2, sv, fused)
    avg_adj_ms = t_adj / max(n_adj, 1)
    achieved = bytes_adj / (avg_adj_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = ADJ_DS_TRAFFIC_PER_ROW * N if (args.precision == "ds" and S == 256 and fused) else None
    issue = None
    if traffic is not None:
        clk_mhz = max(clk.summary().get("sm_mhz") or 2070.0, 1.0)
        inst_rate = ADJ_DS_WARP_INST_PER_ROW * N / (avg_adj_ms * 1e-3)          # warp instructions / s
        peak_rate = ISSUE_PEAK_WARP_INST_PER_CYCLE * clk_mhz * 1e6
        issue = {"bound": "instruction issue (FP32 pipe: float-float arithmetic)", "achieved": inst_rate / 1e12,
                 "peak": peak_rate / 1e12, "unit": "T warp-instructions/s", "frac": inst_rate / peak_rate,
                 "instructions": "ncu smsp__inst_executed.sum of the L=32 launch scaled by rows (profiles/)",
                 "peak_clock_mhz": clk_mhz}
    launches = sum(v[0] for v in prof.values())

    # ---- end to end through the public API with pinned host buffers ----
    # The probe block goes up as its nonzeros (set_R_sparse: colour probes have one entry per row
    # and realisation, 21 MB here) for "e2e", and as the dense column-major n x S block (set_R,
    # what the reference's transfer_R moves, 2.1 GB) for "e2e_dense_R"; H, mu and D as in both.
    e2e = e2e_dense = None
    if not args.no_e2e:
        e2e = run_e2e(args, fk, Lb, H, es, R, c, D, M, per_solve, ws, dist, dev, sparse=True)
        e2e_dense = run_e2e(args, fk, Lb, H, es, R, c, D, M, per_solve, ws, dist, dev, sparse=False)

    # ---- error vs the FP64 engine on the same workload (bounded: M = 40) ----
    err = None
    if args.precision != "fp64":
        Mv = min(40, M)
        cv = c[:Mv].copy()
        ref = fk.Engine(True, "fp64", device=dev)
        ref.set_H(H, es)
        ref.set_R(R)
        mu_r = ref.moments(Mv)
        Dr = H.pattern_like(True)
        ref.autodiff_matrix(cv, Dr)
        ref.close()
        eng.set_R(R)
        mu_t = eng.moments(Mv)
        Dt = H.pattern_like(True)
        eng.autodiff_matrix(cv, Dt)
        err = {"moments_max_rel_mu0": float(np.max(np.abs(mu_t - mu_r)) / abs(mu_r[0])),
               "D_rel_fro": float(np.linalg.norm(Dt.val - Dr.val) / np.linalg.norm(Dr.val)),
               "vs": "native FP64 GPU engine, same H and R, M=%d" % Mv}
    eng.close()
    return dict(value=value, ms=ms_max, clocks=clk.summary(), prof=prof, achieved=achieved, peak=peak,
                peak_kind=peak_kind, traffic=traffic, launches=launches, e2e=e2e, e2e_dense=e2e_dense, issue=issue, err=err, N=N, S=S, M=M,
                nnzb=H.n_blocks(), mu0=float(mu[0]), bytes_adj=bytes_adj, fused=fused, avg_adj_ms=avg_adj_ms,
                avg_step_ms=t_step / max(n_step, 1), n_adj=n_adj, n_step=n_step)


def cpu_port_rate(args, M_sample, H=None, es=None, R=None):
    """Oracle port of the reference's CPU engine on all host threads: one moments + autodiff solve
    at order M_sample on the full workload; returns (probe-steps/s, seconds, threads)."""
    from fastkpm_gb300 import workloads as W
    from oracle import oracle as O
    if H is None:
        H, es, R, _ = workload(args)
    c = W.fermi_coefficients(M_sample, es, "fermi_energy")
    orc = O.OracleEngine(True, nthreads=0)
    orc.set_H(H, es)
    orc.set_R(R)
    t0 = time.perf_counter()
    orc.moments(M_sample)
    orc.autodiff_matrix(c, H.pattern_like(True))
    dt = time.perf_counter() - t0
    N, S = R.shape
    return float(N) * M_sample * S / dt, dt, orc.threads


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    H, es, R, _ = workload(args)
    Ms = args.cpu_M
    for _ in range(args.warmup):
        cpu_port_rate(args, Ms, H, es, R)
    rates, secs = [], []
    threads = 1
    for _ in range(args.steps):
        r, dt, threads = cpu_port_rate(args, Ms, H, es, R)
        rates.append(r)
        secs.append(dt)
    value = float(np.sum([float(R.shape[0]) * Ms * R.shape[1]] * len(secs)) / np.sum(secs))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(secs) * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "cubic L=%d spin-block KPM solve (moments + autodiff_matrix), sample M=%d"
                       % (args.L, Ms), "N": int(R.shape[0]), "S": int(R.shape[1]), "M": Ms, "b": 2,
                       "nnzb": int(H.n_blocks())},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "one moments(%d) + autodiff_matrix solve of the full cubic L=%d, S=%d "
                                       "workload per step (reference CPU engine restated, %d threads)"
                                       % (Ms, args.L, R.shape[1], threads)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- other configurations
def _mu_err(mu, ref):
    return float(np.max(np.abs(np.asarray(mu) - ref)) / abs(ref[0]))


def _d_err(d, ref):
    return float(np.linalg.norm(d - ref) / np.linalg.norm(ref))


def _solve_timed(eng, M, c, D, steps, warmup):
    for _ in range(warmup):
        eng.moments_async(M)
        eng.autodiff_matrix_async(c, D)
    eng.synchronize()
    eng.timer_start()
    for _ in range(steps):
        eng.moments_async(M)
        eng.autodiff_matrix_async(c, D)
    return eng.timer_stop() / steps


def run_precision(args):
    """Triangular L=512 spin lattice, M=2000, S=128: FP32 recursion vs native FP64 (and DS)."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import workloads as W
    cfg = W.config3(L=args.L if args.L != 64 else 512)
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], 1, cfg["probe_seed"])
    M = args.M if args.M != 1000 else cfg["M"]
    c = W.fermi_coefficients(M, es, "fermi_energy")
    N, S = R.shape
    out = {}
    for prec in ["fp64", "ds", "fp32"]:
        eng = fk.Engine(True, prec)
        eng.set_H(H, es)
        eng.set_R(R)
        D = H.pattern_like(True)
        ms = _solve_timed(eng, M, c, D, 1, 1)
        mu = eng.fetch_moments(M)
        eng.fetch_D(D)
        out[prec] = dict(ms=ms, mu=mu, D=D.val.copy())
        eng.close()
    ref = out["fp64"]
    res = {}
    for prec in ["ds", "fp32"]:
        res[prec] = {"moments_max_rel_mu0": _mu_err(out[prec]["mu"], ref["mu"]),
                     "D_rel_fro": _d_err(out[prec]["D"], ref["D"]),
                     "ms_per_solve": out[prec]["ms"], "speedup_vs_fp64": ref["ms"] / out[prec]["ms"]}
    per = float(N) * M * S
    line = {"metric": METRIC, "value": per / (out["fp32"]["ms"] / 1e3), "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": out["fp32"]["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 recursion, f64 accumulation", "data": "synthetic",
            "config": {"workload": "triangular L=%d spin-block lattice, J=2, M=%d, S=%d colour probes: "
                                   "moments + autodiff_matrix" % (cfg["H"].n_rows ** 0.5, M, S),
                       "N": N, "M": M, "S": S, "nnzb": H.n_blocks()},
            "fp64_ms_per_solve": ref["ms"], "precision": res}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """64 square lattices (L ~ U{32..256}, W ~ U[0,4]), M=500, S=32: one FP32 launch per step for all
    systems, recursion replayed from a CUDA graph, autotuned mapping; vs 64 sequential FP64 solves."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import _lib as Lb
    from fastkpm_gb300 import workloads as W
    systems = W.config4()
    M = 500
    Rs = [fk.probe_uncorrelated(s["H"].n_rows, s["S"], fk.RNG(s["probe_seed"])) for s in systems]
    total_rows = sum(s["H"].n_rows for s in systems)
    S = systems[0]["S"]
    bt = fk.Batch(False, "fp32")
    for s, R in zip(systems, Rs):
        bt.add(s["H"], s["es"], R)
    bt.commit()
    tune = bt.autotune(8)
    bt.set_option(Lb.FK_OPT_GRAPHS, 1)
    for _ in range(max(args.warmup, 1)):
        mu_b = bt.moments(M)
    with ClockSampler(0) as clk:
        bt.timer_start()
        for _ in range(args.steps):
            mu_b = bt.moments(M)
        ms_b = bt.timer_stop() / args.steps
    # sequential plain FP64 solves (moments only, the batched output)
    eng = fk.Engine(False, "fp64")
    t_seq = 0.0
    err = 0.0
    for k, (s, R) in enumerate(zip(systems, Rs)):
        eng.set_H(s["H"], s["es"])
        eng.set_R(R)
        eng.moments(M)
        eng.timer_start()
        mu = eng.moments(M)
        t_seq += eng.timer_stop()
        err = max(err, _mu_err(mu_b[k], mu))
    # full solve (moments + autodiff_matrix with each system's own Fermi-energy coefficients):
    # batched FP32 vs sequential plain FP64, wall clock around the synchronous calls
    cs = np.stack([W.fermi_coefficients(M, s["es"], "fermi_energy") for s in systems])
    d_out = np.zeros(sum(s["H"].n_blocks() for s in systems))   # b = 1 real: one value per block
    lib = Lb.load()
    pinned = lib.fk_host_register(d_out.ctypes.data, d_out.nbytes) == 0
    bt.moments(M)
    bt.autodiff_matrix(M, cs, out=d_out)
    n_solve = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(n_solve):
        bt.moments(M)
        Ds_b = bt.autodiff_matrix(M, cs, out=d_out)
    ms_solve = (time.perf_counter() - t0) * 1e3 / n_solve
    t_seq_solve = 0.0
    d_err = 0.0
    for k, (s, R) in enumerate(zip(systems, Rs)):
        eng.set_H(s["H"], s["es"])
        eng.set_R(R)
        D = s["H"].pattern_like(False)
        eng.moments(M)
        eng.autodiff_matrix(cs[k], D)
        t0 = time.perf_counter()
        eng.moments(M)
        eng.autodiff_matrix(cs[k], D)
        t_seq_solve += (time.perf_counter() - t0) * 1e3
        d_err = max(d_err, float(np.linalg.norm(Ds_b[k].val - D.val) / np.linalg.norm(D.val)))
    eng.close()
    if pinned:
        lib.fk_host_unregister(d_out.ctypes.data)
    solve = {"what": "moments(M) + autodiff_matrix(c_sys) for all 64 systems (host wall clock, D copied out)",
             "ms": ms_solve, "value": float(total_rows) * M * S / (ms_solve / 1e3), "unit": UNIT,
             "sequential_fp64_ms": t_seq_solve, "speedup_vs_sequential_fp64": t_seq_solve / ms_solve,
             "D_rel_fro_vs_fp64": d_err, "D_buffer_pinned": pinned}
    per = float(total_rows) * M * S
    bytes_step = 3 * total_rows * S * 4 + sum(s["H"].n_blocks() * 8 + 4 * (s["H"].n_rows + 1) for s in systems)
    achieved = bytes_step / (ms_b / (M // 2) * 1e-3) / 1e9
    peak, kind = peaks()
    line = {"metric": METRIC, "value": per / (ms_b / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 recursion, f64 accumulation", "data": "synthetic",
            "config": {"workload": "64 square lattices L~U{32..256}, W~U[0,4], b=1 real, M=500, S=32: "
                                   "batched moments, CUDA graph, autotuned", "total_rows": total_rows, "M": M, "S": S,
                       "systems": len(systems)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "kernel": "k_cheb_step (batched)", "peak_source": kind},
            "sequential_fp64_ms": t_seq, "speedup_vs_sequential_fp64": t_seq / ms_b,
            "moments_max_rel_mu0_vs_fp64": err, "solve": solve, "autotune": tune, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def serve_requests(n_req, seed, max_sites):
    """Mixed-size KPM solve requests: cubic or square lattice (50/50), sites log-uniform over
    10^3 .. max_sites, b=1 real or b=2 complex spin-exchange (50/50), M in {200,500,1000,2000},
    S in {32,64,128} by colour probing; Poisson arrival offsets (rate 4/s)."""
    from fastkpm_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    reqs = []
    t = 0.0
    for k in range(n_req):
        t += rng.exponential(0.25)
        cubic = rng.random() < 0.5
        spin = rng.random() < 0.5
        sites = 10 ** rng.uniform(3, np.log10(max_sites))
        M = int(rng.choice([200, 500, 1000, 2000]))
        S = int(rng.choice([32, 64, 128]))
        if cubic:
            L = max(8, int(round(sites ** (1 / 3) / 8)) * 8)
            if spin:
                H, es, _ = W.cubic_spin_lattice(L, -1.0, 1.0, seed + k)
                p = {32: (2, 2, 4), 64: (4, 4, 2), 128: (4, 4, 4)}[S]
                idx = np.arange(L ** 3)
                col = idx % L % p[0] + p[0] * ((idx // L % L) % p[1] + p[1] * ((idx // (L * L)) % p[2]))
                groups = np.stack([2 * col, 2 * col + 1], 1).reshape(-1)
            else:
                H, es = _cubic_real(L, seed + k)
                p = {32: (4, 4, 2), 64: (4, 4, 4), 128: (8, 4, 4)}[S]
                idx = np.arange(L ** 3)
                groups = idx % L % p[0] + p[0] * ((idx // L % L) % p[1] + p[1] * ((idx // (L * L)) % p[2]))
        else:
            L = max(8, int(round(sites ** 0.5 / 8)) * 8)
            if spin:
                H, es, _ = W.triangular_spin_lattice(L, -1.0, 1.0, seed + k)
                px, py = {32: (4, 4), 64: (8, 4), 128: (8, 8)}[S]
                groups = W.square_colour_groups(L, px, py, spin=True)
            else:
                H, es = W.square_lattice(L, -1.0, 1.0, seed + k)
                px, py = {32: (8, 4), 64: (8, 8), 128: (16, 8)}[S]
                groups = W.square_colour_groups(L, px, py)
        # colour probes travel as their nonzeros (one per row): Engine.set_R_sparse
        entries = W.phase_probe_entries(groups, 1, seed + k, complex_values=spin)
        c = W.fermi_coefficients(M, es, "fermi_energy")
        reqs.append(dict(H=H, es=es, entries=entries, n=len(groups), M=M, c=c, t=t, spin=spin))
    return reqs


def _cubic_real(L, seed):
    from fastkpm_gb300 import workloads as W
    from fastkpm_gb300.engine import EnergyScale
    rng = np.random.default_rng(seed)
    n = L ** 3
    idx = np.arange(n)
    x, y, z = idx % L, (idx // L) % L, idx // (L * L)
    site = lambda a, b_, c_: (a % L) + L * ((b_ % L) + L * (c_ % L))
    nbrs = [site(x + 1, y, z), site(x - 1, y, z), site(x, y + 1, z), site(x, y - 1, z), site(x, y, z + 1),
            site(x, y, z - 1)]
    rows = np.concatenate([idx] * 7)
    cols = np.concatenate(nbrs + [idx])
    vals = np.concatenate([np.full(n, -1.0)] * 6 + [rng.uniform(-0.5, 0.5, n)])
    H = W._bsr_from_coo(n, 1, rows, cols, vals[:, None], False)
    return H, EnergyScale(-6.3, 6.3)


def run_serve(args):
    """Continuous-batching server (FP32 recursion) on a Poisson stream of mixed-size requests;
    p50/p99 latency and aggregate probe-steps/s vs the same requests solved one by one with the
    plain FP64 engine; each request's result checked against its FP64 solve."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300.serve import Request, Server
    reqs = serve_requests(args.serve_requests, 5, args.serve_max_sites)
    srv = Server(max_slots=8, memory_budget=int(120e9))
    t0 = time.perf_counter()
    tickets = []
    for r in reqs:
        now = time.perf_counter() - t0
        if r["t"] > now:
            time.sleep(r["t"] - now)
        tickets.append(srv.submit(Request(r["H"], r["es"], None, r["M"], r["c"], "autodiff", "fp32",
                                          R_entries=r["entries"])))
    srv.drain()
    st = srv.stats()
    srv.stop()
    # serial plain FP64 engine on the same requests (in arrival order, for at most ~90 s of solves;
    # its rate is taken over the requests it finished)
    t_ser = 0.0
    worst = 0.0
    work_ser = 0.0
    n_ser = 0
    for r, tk in zip(reqs, tickets):
        if t_ser > 90.0:
            break
        eng = fk.Engine(r["spin"], "fp64")
        eng.set_H(r["H"], r["es"])
        eng.set_R_sparse(r["n"], *r["entries"])
        t = time.perf_counter()
        mu = eng.moments(r["M"])
        D = r["H"].pattern_like(r["spin"])
        eng.autodiff_matrix(r["c"], D)
        t_ser += time.perf_counter() - t
        eng.close()
        work_ser += float(r["n"]) * r["M"] * r["entries"][0]
        n_ser += 1
        if tk.error is None:
            worst = max(worst, _mu_err(tk.mu, mu))
    work = work_ser
    line = {"metric": METRIC, "value": st["probe_steps_per_s"], "unit": UNIT, "n_gpus": 1, "steps": len(reqs),
            "warmup": 0, "ms_per_step": st["wall_s"] * 1e3 / max(len(reqs), 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 recursion, f64 accumulation", "data": "synthetic",
            "config": {"workload": "Poisson stream of %d mixed KPM solves (moments + autodiff D), sites 1e3..%g"
                                   % (len(reqs), args.serve_max_sites), "slots": 8},
            "latency_p50_s": st["p50_s"], "latency_p99_s": st["p99_s"], "completed": st["completed"],
            "rejected": st["rejected"], "max_concurrent": st["max_concurrent"],
            "serial_fp64_probe_steps_per_s": work / t_ser, "speedup_vs_serial_fp64": (work / t_ser and
                                                                                  st["probe_steps_per_s"] / (work / t_ser)),
            "moments_max_rel_mu0_vs_fp64": worst, "serial_fp64_requests": n_ser}
    peak, kind = peaks()
    gbs = st["algorithmic_bytes"] / max(st["busy_s"], 1e-9) / 1e9
    line["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "over": "time with at least one solve in service (%.2f s of %.2f s wall)"
                                % (st["busy_s"], st["wall_s"]),
                        "bytes": "sum of each solve's algorithmic bytes (forward steps + fused reverse steps)",
                        "peak_source": kind}
    print(json.dumps(line), flush=True)


def run_square(args):
    """One large square lattice (L = --L, default 1448: 2.1 M sites), b=1 real, S = --S (default 32)
    +-1 probes, moments(M) in --precision (default fp32): the narrow-row step kernel of the batched
    workload at a size above L2, with its roofline; error vs the FP64 engine on the first 40 moments."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import _lib as Lb
    from fastkpm_gb300 import workloads as W
    L = args.L if args.L != 64 else 1448
    S = args.S if args.S != 256 else 32
    prec = args.precision if args.precision != "ds" else "fp32"
    M = args.M
    H, es = W.square_lattice(L, -1.0, 1.0, 7)
    R = fk.probe_uncorrelated(H.n_rows, S, fk.RNG(7))
    eng = fk.Engine(False, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    eng.set_option(Lb.FK_OPT_GRAPHS, 1)
    for _ in range(max(args.warmup, 1)):
        mu = eng.moments(M)
    eng.set_profiling(1)
    eng.profile_reset()
    eng.moments(M)
    n_step, t_step = eng.profile(0)
    eng.set_profiling(0)
    with ClockSampler(0) as clk:
        eng.timer_start()
        for _ in range(args.steps):
            eng.moments_async(M)
        ms = eng.timer_stop() / args.steps
    mu = eng.fetch_moments(M)
    Mv = min(40, M)
    ref = fk.Engine(False, "fp64")
    ref.set_H(H, es)
    ref.set_R(R)
    err = _mu_err(mu[:Mv], ref.moments(Mv))
    ref.close()
    sv = {"fp32": 4, "ds": 8, "fp64": 8}[prec]
    bytes_step = 3 * H.n_rows * S * sv + H.n_blocks() * (sv + 4) + 4 * (H.n_rows + 1)
    achieved = bytes_step / (t_step / n_step * 1e-3) / 1e9
    peak, kind = peaks()
    per = float(H.n_rows) * M * S
    line = {"metric": METRIC, "value": per / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": prec, "data": "synthetic",
            "config": {"workload": "square lattice L=%d (N=%d), b=1 real, S=%d, M=%d: moments, CUDA graph" % (L, H.n_rows, S, M),
                       "l2": "inputs larger than L2" if 3 * H.n_rows * S * sv > 129e6 else "L2-resident"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "kernel": "k_cheb_step", "peak_source": kind, "bytes_per_launch": bytes_step,
                         "avg_launch_ms": t_step / n_step},
            "moments_max_rel_mu0_vs_fp64": err, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    eng.close()


def run_cfg1(args):
    """32x32 square lattice, M=200, S=64, FP64: moments + stoch_matrix; oracle timed beside it."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import workloads as W
    from oracle import oracle as O
    cfg = W.config1()
    H, es, M, S = cfg["H"], cfg["es"], cfg["M"], cfg["S"]
    R = fk.probe_uncorrelated(H.n_rows, S, fk.RNG(cfg["probe_seed"]))
    c = W.fermi_coefficients(M, es)
    D = H.pattern_like()
    eng = fk.Engine(False, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    for _ in range(3):
        eng.moments(M)
        eng.stoch_matrix(c, D)
    eng.timer_start()
    for _ in range(args.steps):
        eng.moments_async(M)
        eng.stoch_matrix_async(c, D)
    ms_direct = eng.timer_stop() / args.steps
    # the same solves replayed from CUDA graphs (captured once for this shape): the ~400 launches
    # of a few microseconds each dominate this L2-resident problem
    from fastkpm_gb300 import _lib as Lb
    eng.set_option(Lb.FK_OPT_GRAPHS, 1)
    for _ in range(3):
        eng.moments(M)
        eng.stoch_matrix(c, D)
    eng.timer_start()
    for _ in range(args.steps):
        eng.moments_async(M)
        eng.stoch_matrix_async(c, D)
    ms = eng.timer_stop() / args.steps
    mu = eng.fetch_moments(M)
    eng.fetch_D(D)
    orc = O.OracleEngine(False)
    orc.set_H(H, es)
    orc.set_R(R)
    t = time.perf_counter()
    mu_r = orc.moments(M)
    D_r = orc.stoch_matrix(c, D)
    t_cpu = time.perf_counter() - t
    per = float(H.n_rows) * M * S
    line = {"metric": METRIC, "value": per / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": 3, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "square L=32, M=200, S=64: moments + stoch_matrix (L2-resident), CUDA-graph replay"},
            "ms_per_step_direct_launches": ms_direct,
            "moments_max_rel_mu0_vs_oracle": _mu_err(mu, mu_r), "D_rel_fro_vs_oracle": _d_err(D.val, D_r),
            "cpu_baseline": {"value": per / t_cpu, "unit": UNIT, "cores": orc.threads, "kind": "port",
                             "sample": "the same solve on the oracle port"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, ws, dist = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
        return
    if args.workload != "solve":
        if rank == 0:
            {"precision": run_precision, "batch": run_batch, "serve": run_serve, "cfg1": run_cfg1,
             "square": run_square}[args.workload](args)
        return
    r = run_gb300(args, rank, ws, dist)
    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, dt, threads = cpu_port_rate(args, args.cpu_M)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one moments(%d) + autodiff_matrix solve of the full workload (%.1f s on %d threads), "
                         "the reference CPU engine restated" % (args.cpu_M, dt, threads)}
    if rank != 0:
        return
    dtype = {"ds": "f64 (double-single float-float storage and arithmetic)", "fp64": "f64",
             "fp32": "f32 recursion, f64 accumulation"}[args.precision]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": "cubic L=%d Kondo-lattice spin-block KPM solve: moments(M) + autodiff_matrix(c, D) "
                               "on H's pattern" % args.L,
                   "N": r["N"], "sites": r["N"] // 2, "b": 2, "nnzb": r["nnzb"], "M": r["M"], "S": r["S"],
                   "precision": args.precision, "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 (2 GiB per vector), no flush"},
        "roofline": {"bound": "hbm", "achieved": r["achieved"], "peak": r["peak"], "unit": "GB/s",
                     "frac": r["achieved"] / r["peak"], "traffic": r["traffic"],
                     "kernel": "k_adjoint_step (reverse-mode step, both recursions%s)" % (
                         " + fused D epilogue" if r["fused"] else "; D outer product in k_outer"),
                     "traffic_source": "ncu capture of the L=32 case scaled by rows (profiles/)" if r["traffic"] else None,
                     "peak_source": r["peak_kind"], "bytes_per_launch": r["bytes_adj"],
                     "avg_launch_ms": r["avg_adj_ms"], "launches": r["n_adj"]},
        "cpu_baseline": cpu,
        "roofline_issue": r["issue"],
        "e2e": r["e2e"],
        "e2e_dense_R": r["e2e_dense"],
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "err_vs_fp64": r["err"],
        "kernels": {"step_avg_ms": r["avg_step_ms"], "step_launches": r["n_step"],
                    "adjoint_avg_ms": r["avg_adj_ms"], "adjoint_launches": r["n_adj"],
                    "d_epilogue_fused": r["fused"]},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
