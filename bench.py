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
         uploads H and R from pinned host memory and reads back mu and D.
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


def adjoint_bytes_per_launch(eng_info, N, nnzb, b, sv):
    """Algorithmic bytes of one fused adjoint launch over one column slice: read alpha_m, alpha_{m+1},
    beta_{m+1}, beta_{m+2}, write alpha_{m-1}, beta_m (6 vectors of the slice), H once (entries +
    4-byte column index), row_ptr, and the FP64 complex D accumulator read + write."""
    cols, entry_bytes = eng_info
    vec = 6 * N * cols * sv
    h = nnzb * (b * b * entry_bytes + 4) + 4 * (N // b + 1)
    d = 2 * nnzb * b * b * 16
    return vec + h + d


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
    value = per_solve * args.steps * ws / (ms_max / 1e3)
    mu = eng.fetch_moments(M)
    eng.fetch_D(D)

    # roofline of the dominant kernel (fused adjoint step)
    n_adj, t_adj = prof[1]
    n_step, t_step = prof[0]
    P = S   # complex FP64-class: one element per 16-byte packet; DS/FP64 entries 16 B, FP32 8 B
    sv = 8 if args.precision == "fp32" else 16
    np_opt = eng.get_option(Lb.FK_OPT_NP)
    epp = 16 // sv
    packets = (S + epp - 1) // epp
    slice_packets = min(packets, 32 * np_opt) if packets > 32 else packets
    slices = (packets + slice_packets - 1) // slice_packets
    cols = S / slices
    bytes_adj = adjoint_bytes_per_launch((cols, sv), N, H.n_blocks() + 0, 2, sv)
    avg_adj_ms = t_adj / max(n_adj, 1)
    achieved = bytes_adj / (avg_adj_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", "adjoint_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get(args.precision)
        except Exception:
            traffic = None
    launches = sum(v[0] for v in prof.values())

    # ---- end to end through the public API with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        lib = Lb.load()
        Rf = np.asfortranarray(R)
        hv = np.ascontiguousarray(H.val)
        lib.fk_host_register(Rf.ctypes.data, Rf.nbytes)
        lib.fk_host_register(hv.ctypes.data, hv.nbytes)
        e2 = fk.Engine(True, args.precision, device=dev)
        mu_h = np.zeros(M)
        for _ in range(1):
            e2.set_H(H, es)
            e2.set_R(Rf)
            e2.moments(M)
            e2.autodiff_matrix(c, D)
        barrier(dist)
        e2.synchronize()
        t0 = time.perf_counter()
        e2.timer_start()
        for _ in range(args.steps):
            e2.set_H(H, es)
            e2.set_R(Rf)
            mu_h = e2.moments(M)
            e2.autodiff_matrix(c, D)
        e2_ms_dev = e2.timer_stop()
        e2_ms_wall = (time.perf_counter() - t0) * 1e3
        barrier(dist)
        e2_ms = max_over_ranks(dist, max(e2_ms_dev, e2_ms_wall))
        h2d = int(H.row_ptr.nbytes + H.col_idx.nbytes + hv.nbytes + Rf.nbytes)
        d2h = int(M * 8 + D.val.nbytes)
        e2e = {"value": per_solve * args.steps * ws / (e2_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2_ms / args.steps}
        lib.fk_host_unregister(Rf.ctypes.data)
        lib.fk_host_unregister(hv.ctypes.data)
        e2.close()

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
                peak_kind=peak_kind, traffic=traffic, launches=launches, e2e=e2e, err=err, N=N, S=S, M=M,
                nnzb=H.n_blocks(), mu0=float(mu[0]), bytes_adj=bytes_adj, slices=slices, avg_adj_ms=avg_adj_ms,
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


def main():
    args = parse()
    rank, ws, dist = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
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
                     "kernel": "k_adjoint_step (fused reverse-mode step + D epilogue)",
                     "peak_source": r["peak_kind"], "bytes_per_launch": r["bytes_adj"],
                     "avg_launch_ms": r["avg_adj_ms"], "launches": r["n_adj"]},
        "cpu_baseline": cpu,
        "e2e": r["e2e"],
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "err_vs_fp64": r["err"],
        "kernels": {"step_avg_ms": r["avg_step_ms"], "step_launches": r["n_step"],
                    "adjoint_avg_ms": r["avg_adj_ms"], "adjoint_launches": r["n_adj"],
                    "column_slices": r["slices"]},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
