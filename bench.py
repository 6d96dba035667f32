"""Benchmark: Chebyshev probe-steps/s (N*M*S per solve / time) of the GB300 KPM engine.

Workload (one "step" = one solve): Kondo-lattice-style cubic lattice L=64
(262,144 sites, 2x2 complex spin blocks, N = 524,288 scalar rows,
nnzb = 1,835,008), M = 1000 Chebyshev moments, S = 256 probe columns; the solve
is moments(M) followed by autodiff_matrix(c, D) on H's pattern, with c the
zero-temperature Fermi-energy expansion. Synthetic seeded data: random unit
spins, seeded unit-phase colour probes. Every vector (N x S x 16 B = 2 GiB) is
far larger than the 129 MB L2, so no L2 flush is needed between steps.

The headline line is the native-FP64 engine (--precision fp64, the reference's
arithmetic). The same line carries "legs": the float-float (ds) and FP32-recursion
engines on the same workload, each with its own rate, rooflines, end-to-end rate
and its error against the FP64 engine at the full M (same H, R and c).

  value  device-resident throughput: H and R already on the GPU, solves enqueued
         back to back, timed with CUDA events on the engine's stream.
  e2e    the same metric through the public API with host buffers: every step
         uploads H and the colour probes' nonzeros (set_R_sparse) from pinned host
         memory and reads back mu and D (--e2e-dense: also with the dense n x S R).
  roofline           HBM roofline of the dominant kernel (the fused adjoint step):
                     algorithmic bytes per launch / live CUDA-event launch time.
  roofline_fp64_pipe (FP64) the same launch's algorithmic FP64 flops against the
                     device's FP64 FMA rate measured in this run.
  roofline_issue     (float-float) the launch against the GPU's warp-instruction issue
                     rate, from the ncu instruction count of the L=32 capture.
  cpu_baseline  the oracle port of the reference CPU engine on all host threads: one
         moments + autodiff_matrix solve at M=8 and one at M=16 of the full workload,
         the solve time extrapolated linearly in M to M=1000 (t = F + M c).
  --impl reference: that CPU engine restated (oracle port), all host threads, each step
         a M=8 solve of the full workload, the rate extrapolated to M=1000 as above; the
         one-thread rate is measured on the L=32 lattice. Loads only the oracle library.
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
    p.add_argument("--precision", default=None, choices=["ds", "fp64", "fp32"],
                   help="engine of the headline value (default fp64, the reference's arithmetic; "
                        "--workload square: fp32)")
    p.add_argument("--legs", default="ds,fp32", help="other precisions timed on the same workload ('' for none)")
    p.add_argument("--leg-steps", type=int, default=0, help="timed solves per leg (0: ds min(steps,3), fp32 min(steps,5))")
    p.add_argument("--e2e-steps", type=int, default=1, help="timed end-to-end solves per engine (0: no e2e)")
    p.add_argument("--e2e-dense", action="store_true", help="also time e2e with the dense n x S probe block")
    p.add_argument("--L", type=int, default=64)
    p.add_argument("--M", type=int, default=1000)
    p.add_argument("--S", type=int, default=256)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-M", default="8,16", help="orders of the two CPU sample solves (extrapolated in M)")
    p.add_argument("--cpu-L1", type=int, default=32, help="lattice of the one-thread CPU sample (reference arm)")
    p.add_argument("--workload", default="solve", choices=["solve", "precision", "batch", "serve", "cfg1", "square"])
    p.add_argument("--batch-systems", type=int, default=64, help="systems of the batch workload")
    p.add_argument("--batch-M", type=int, default=500, help="Chebyshev order of the batch workload")
    p.add_argument("--batch-only", action="store_true", help="batch workload: batched moments only (no FP64 "
                   "comparison, no full solve); a short run to profile the batched step kernel")
    p.add_argument("--serve-requests", type=int, default=24)
    p.add_argument("--serve-max-sites", type=float, default=1e6)
    p.add_argument("--serve-rate", type=float, default=4.0, help="Poisson arrival rate of the request stream (1/s)")
    p.add_argument("--serve-cta-waves", type=int, default=8, help="FK_OPT_CTA_WAVES of the serving engines")
    p.add_argument("--serve-pack-bytes", type=float, default=256 << 20,
                   help="footprint bound of requests that share batched launches (0: no packing)")
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
def workload(args, coefficients=None, L=None):
    """(H, es, R, c) of the cubic spin-lattice solve; numpy only, except the coefficients:
    `coefficients(M, es)` when given (the reference arm passes the oracle's), else the
    library's FP64 expansion_coefficients."""
    from fastkpm_gb300 import workloads as W
    cfg = W.config2(L=L or args.L, S=args.S)
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], cfg["realisations"], cfg["probe_seed"])
    R = R[:, :args.S] if R.shape[1] > args.S else R
    c = coefficients(args.M, es) if coefficients else W.fermi_coefficients(args.M, es, "fermi_energy")
    return H, es, np.asfortranarray(R), c


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def h_bytes(nnzb, b, sv, n_b):
    return nnzb * (b * b * sv + 4) + 4 * (n_b + 1)


def adjoint_bytes_per_launch(N, S, nnzb, b, sv, fused, cplx=True):
    """Algorithmic bytes of one adjoint launch (the kernel walks all S columns itself): read alpha_m,
    alpha_{m+1}, beta_{m+1}, beta_{m+2}, write alpha_{m-1}, beta_m (6 vectors), H once (entries +
    4-byte column index), row_ptr, and, when the D epilogue is fused, the D accumulator read + write
    (8 bytes per real: double or float-float; two reals per complex entry)."""
    d = 2 * nnzb * b * b * (16 if cplx else 8) if fused else 0
    return 6 * N * S * sv + h_bytes(nnzb, b, sv, N // b) + d


def step_bytes_per_launch(N, S, nnzb, b, sv):
    """Algorithmic bytes of one moments step: read x (gathered) and z, write y, H once."""
    return 3 * N * S * sv + h_bytes(nnzb, b, sv, N // b)


def block_classes(H):
    """(hopping blocks: real multiples of the identity, general blocks) of a b=2 complex H."""
    v = H.val.reshape(-1, 4)
    ident = (v[:, 1] == 0) & (v[:, 2] == 0) & (v[:, 0] == v[:, 3]) & (v.imag == 0).all(axis=1)
    return int(ident.sum()), int((~ident).sum())


def adjoint_flops_per_launch(H, S):
    """Algorithmic FP64 flops of one fused adjoint launch (complex b=2, H's pattern): per block and
    column, both recursions (a hopping block t I2: 2 complex x real MACs of 4 flops each; a general
    block: 4 complex MACs of 8 flops) and the epilogue's 4 complex MACs; per scalar row and column,
    2 alpha_m+1 - alpha_m-1 style finishes (4 flops each) and beta's 3 coefficient terms (12 flops)."""
    hop, gen = block_classes(H)
    per_col = hop * (2 * 8 + 32) + gen * (2 * 32 + 32) + H.n_rows * 2 * 20
    return float(per_col) * S


def step_flops_per_launch(H, S):
    """Algorithmic FP64 flops of one moments step: the block products, the finish and the two dots."""
    hop, gen = block_classes(H)
    return float(hop * 8 + gen * 32 + H.n_rows * 2 * 12) * S


# DRAM bytes (read + write) of one fused reverse step, all its launches, at the cubic L=64, S=256
# workload (524,288 rows), from ncu captures summarised under profiles/. Float-float runs the step
# as four column-sweep launches (FK_OPT_ADJ_SWEEP): their sum. Keys: (precision, FP64
# accumulators). Other workloads, and engine forms without a capture of their kernels, report null.
# (Traffic does not grow in proportion to the rows: at L=32 the rows gathered a lattice plane
# later still hit L2, at L=64 they do not.)
ADJ_TRAFFIC_L64 = {("fp64", 1): 18615305216 + 6046837248,
                   ("fp32", 1): 8037847296 + 2240859904,
                   ("ds", 0): 14741449984 + 4654563072}
ADJ_TRAFFIC_ROWS = 524288
# warp instructions per row of the float-float reverse step (cubic L=32 capture, one launch over
# whole rows; the four sweeps add the per-row setup three more times)
ADJ_WARP_INST_PER_ROW = {("ds", 0): 914440192 / 65536}
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


def run_e2e(prec, steps, wl, M, per_solve, ws, dist, dev, sparse):
    """moments + autodiff_matrix through the public API, every step uploading H and the probes
    from pinned host memory and reading mu and D back; wall and device clocks, max over ranks.
    One untimed solve first (allocation of the engine's buffers)."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import _lib as Lb
    H, es, R, c = wl
    D = H.pattern_like(True)
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
    e2 = fk.Engine(True, prec, device=dev)

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
    for _ in range(steps):
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
    return {"value": per_solve * steps * ws / (e2_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": e2_ms / steps, "steps": steps, "host_buffers_pinned": pinned,
            "probes": "nonzeros (set_R_sparse)" if sparse else "dense n x S (set_R)",
            "phases_ms_per_step": {k: float(v) / steps for k, v in
                                   zip(["set_H", "set_R", "moments", "autodiff_matrix"], phases)}}


# ---------------------------------------------------------------------------- one engine, timed
def run_leg(args, prec, steps, warmup, wl, ws, dist, dev, e2e_steps, options=None):
    """W untimed and K timed solves of one engine precision, device-resident; kernel times from
    CUDA events around every launch on the engine's stream; rooflines of the adjoint and step
    kernels; the last solve's mu and D; optional end-to-end timing. options: engine options."""
    import fastkpm_gb300 as fk
    from fastkpm_gb300 import _lib as Lb
    H, es, R, c = wl
    N, S, M = R.shape[0], R.shape[1], args.M
    D = H.pattern_like(True)
    eng = fk.Engine(True, prec, device=dev)
    for k, v in (options or {}).items():
        eng.set_option(k, v)
    eng.set_H(H, es)
    eng.set_R(R)
    per_solve = float(N) * M * S
    for _ in range(warmup):
        eng.moments_async(M)
        eng.autodiff_matrix_async(c, D)
    eng.synchronize()
    eng.set_profiling(1)
    eng.profile_reset()
    barrier(dist)
    eng.synchronize()
    with ClockSampler(dev) as clk:
        eng.timer_start()
        for _ in range(steps):
            eng.moments_async(M)
            eng.autodiff_matrix_async(c, D)
        ms = eng.timer_stop()
    eng.synchronize()
    barrier(dist)
    prof = {k: eng.profile(k) for k in range(4)}
    eng.set_profiling(0)
    ms_max = max_over_ranks(dist, ms)
    mu = eng.fetch_moments(M)
    eng.fetch_D(D)
    fused = eng.get_option(Lb.FK_OPT_FUSE_D) != 0
    acc64 = eng.get_option(Lb.FK_OPT_ACC64)
    # kernel launches per reverse step: one, or one per column chunk when the engine sweeps
    sweeps = 1
    if eng.get_option(Lb.FK_OPT_ADJ_SWEEP):
        packets = S * (8 if prec == "fp32" else 16) // 16
        sweeps = max(1, packets // (32 * eng.get_option(Lb.FK_OPT_NP_ADJOINT)))
    eng.close()

    n_adj, t_adj = prof[1]   # reverse steps (each `sweeps` kernel launches)
    n_step, t_step = prof[0]
    sv = 8 if prec == "fp32" else 16
    nnzb = H.n_blocks()
    peak, peak_kind = peaks()
    avg_adj_ms = t_adj / max(n_adj, 1)
    avg_step_ms = t_step / max(n_step, 1)
    bytes_adj = adjoint_bytes_per_launch(N, S, nnzb, 2, sv, fused)
    bytes_step = step_bytes_per_launch(N, S, nnzb, 2, sv)
    ach_adj = bytes_adj / (avg_adj_ms * 1e-3) / 1e9
    ach_step = bytes_step / (avg_step_ms * 1e-3) / 1e9
    key = (prec, acc64)
    traffic = (ADJ_TRAFFIC_L64[key] if (key in ADJ_TRAFFIC_L64 and N == ADJ_TRAFFIC_ROWS and S == 256 and fused)
               else None)
    clocks = clk.summary()
    out = dict(prec=prec, value=replica_value(per_solve, steps, ws, ms_max), ms=ms_max, steps=steps, warmup=warmup,
               clocks=clocks, launches=sum(v[0] for v in prof.values()) + (sweeps - 1) * n_adj, mu=mu, D=D.val.copy(), fused=fused,
               N=N, S=S, M=M, nnzb=nnzb, n_adj=n_adj, n_step=n_step, avg_adj_ms=avg_adj_ms, avg_step_ms=avg_step_ms,
               acc64=acc64)
    out["roofline"] = {"bound": "hbm", "achieved": ach_adj, "peak": peak, "unit": "GB/s", "frac": ach_adj / peak,
                       "traffic": traffic,
                       "kernel": "fused adjoint step (both recursions%s)" % (
                           " + D epilogue" if fused else "; D outer product apart"),
                       "traffic_source": ("ncu DRAM bytes of one reverse step of this workload (profiles/)"
                                          if traffic else None),
                       "peak_source": peak_kind, "bytes_per_launch": bytes_adj, "avg_launch_ms": avg_adj_ms,
                       "launches": n_adj, "kernel_launches_per_reverse_step": sweeps}
    out["roofline_step"] = {"bound": "hbm", "achieved": ach_step, "peak": peak, "unit": "GB/s",
                            "frac": ach_step / peak, "kernel": "Chebyshev step (moments)",
                            "bytes_per_launch": bytes_step, "avg_launch_ms": avg_step_ms, "launches": n_step}
    if prec == "fp64":
        from fastkpm_gb300 import _lib as Lb2
        import ctypes as C
        rate = C.c_double(0.0)
        st = Lb2.load().fk_device_fma_rate(dev, 1, C.byref(rate))
        fl_adj = adjoint_flops_per_launch(H, S)
        fl_step = step_flops_per_launch(H, S)
        a_adj = fl_adj / (avg_adj_ms * 1e-3) / 1e12
        a_step = fl_step / (avg_step_ms * 1e-3) / 1e12
        pk = rate.value if st == 0 else None
        out["roofline_fp64_pipe"] = {
            "bound": "FP64 pipe (DFMA)", "unit": "TFLOP/s", "peak": pk,
            "peak_source": "fk_device_fma_rate: independent DFMA chains timed on this GPU in this run",
            "adjoint": {"achieved": a_adj, "frac": a_adj / pk if pk else None, "flops_per_launch": fl_adj},
            "step": {"achieved": a_step, "frac": a_step / pk if pk else None, "flops_per_launch": fl_step}}
    if key in ADJ_WARP_INST_PER_ROW and S == 256 and fused:
        clk_mhz = max(clocks.get("sm_mhz") or 2070.0, 1.0)
        inst_rate = ADJ_WARP_INST_PER_ROW[key] * N / (avg_adj_ms * 1e-3)
        peak_rate = ISSUE_PEAK_WARP_INST_PER_CYCLE * clk_mhz * 1e6
        out["roofline_issue"] = {"bound": "instruction issue (FP32 pipe: float-float arithmetic)",
                                 "achieved": inst_rate / 1e12, "peak": peak_rate / 1e12,
                                 "unit": "T warp-instructions/s", "frac": inst_rate / peak_rate,
                                 "instructions": "ncu smsp__inst_executed.sum of the L=32 launch scaled by rows",
                                 "peak_clock_mhz": clk_mhz}
    if e2e_steps > 0:
        out["e2e"] = run_e2e(prec, e2e_steps, wl, M, per_solve, ws, dist, dev, sparse=True)
        if args.e2e_dense:
            out["e2e_dense_R"] = run_e2e(prec, e2e_steps, wl, M, per_solve, ws, dist, dev, sparse=False)
    return out


# ---------------------------------------------------------------------------- CPU samples
def oracle_coefficients(M, es):
    from oracle import oracle as O
    return O.expansion_coefficients(M, 2 * M, "fermi_energy", 0.0, 0.0, es.lo, es.hi)


def cpu_solve_times(H, es, R, Ms, nthreads=0, orc=None):
    """Seconds of one moments(M) + autodiff_matrix(c_M, D) solve of the oracle port per M in Ms."""
    from oracle import oracle as O
    if orc is None:
        orc = O.OracleEngine(True, nthreads=nthreads)
        orc.set_H(H, es)
        orc.set_R(R)
    times = {}
    for M in Ms:
        c = oracle_coefficients(M, es)
        t0 = time.perf_counter()
        orc.moments(M)
        orc.autodiff_matrix(c, H.pattern_like(True))
        times[M] = time.perf_counter() - t0
    return times, orc


def extrapolate(t_lo, M_lo, t_hi, M_hi, M):
    """Solve time at order M from two timed orders: t = F + M c (fixed per-solve work F, c per order)."""
    c = (t_hi - t_lo) / (M_hi - M_lo)
    F = t_lo - M_lo * c
    return F + M * c, F, c


def cpu_baseline(args, wl):
    """The oracle port on all host threads: one solve at each of the two sample orders on the full
    workload, extrapolated to the benchmark's M."""
    H, es, R, _ = wl
    Ms = [int(x) for x in args.cpu_M.split(",")]
    times, orc = cpu_solve_times(H, es, R, Ms)
    t_full, F, cM = extrapolate(times[Ms[0]], Ms[0], times[Ms[1]], Ms[1], args.M)
    N, S = R.shape
    return {"value": float(N) * args.M * S / t_full, "unit": UNIT, "cores": orc.threads, "kind": "port",
            "sample": "one moments(M) + autodiff_matrix solve of the full workload at M = %d (%.1f s) and M = %d "
                      "(%.1f s) on %d threads; solve time extrapolated linearly in M to M = %d (fixed %.2f s + "
                      "%.3f s per order): the reference CPU engine restated" % (
                          Ms[0], times[Ms[0]], Ms[1], times[Ms[1]], orc.threads, args.M, F, cM)}


def run_reference(args, rank, ws, dist):
    """The reference's CPU engine (oracle port) on all host threads. Each step is one solve of the
    full workload at the lower sample order; one solve at the higher order (before the timed
    steps) fixes the extrapolation to M. Loads the oracle library only."""
    if rank != 0:
        return
    import fastkpm_gb300
    Ms = [int(x) for x in args.cpu_M.split(",")]
    wl = workload(args, coefficients=oracle_coefficients)
    H, es, R, _ = wl
    N, S = R.shape
    orc = None
    for _ in range(args.warmup):
        _, orc = cpu_solve_times(H, es, R, [Ms[0]], orc=orc)
    t_hi, orc = cpu_solve_times(H, es, R, [Ms[1]], orc=orc)
    secs = []
    for _ in range(args.steps):
        t, orc = cpu_solve_times(H, es, R, [Ms[0]], orc=orc)
        secs.append(t[Ms[0]])
    t_lo = float(np.mean(secs))
    t_full, F, cM = extrapolate(t_lo, Ms[0], t_hi[Ms[1]], Ms[1], args.M)
    value = float(N) * args.M * S / t_full
    threads = orc.threads
    del orc
    # one thread, on the L = cpu-L1 lattice of the same family (the reference engine is single-threaded)
    wl1 = workload(args, coefficients=oracle_coefficients, L=args.cpu_L1)
    H1, es1, R1, _ = wl1
    t1, _ = cpu_solve_times(H1, es1, R1, Ms, nthreads=1)
    t1_full, _, _ = extrapolate(t1[Ms[0]], Ms[0], t1[Ms[1]], Ms[1], args.M)
    rate1 = float(R1.shape[0]) * args.M * R1.shape[1] / t1_full
    sample = ("each step one moments(%d) + autodiff_matrix solve of the full cubic L=%d, S=%d workload on %d "
              "threads (mean %.2f s); one M=%d solve (%.2f s) before the timed steps; value = N*M*S of the M=%d "
              "solve over its time extrapolated linearly in M (fixed %.2f s + %.3f s per order)"
              % (Ms[0], args.L, S, threads, t_lo, Ms[1], t_hi[Ms[1]], args.M, F, cM))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_lo * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "cubic L=%d spin-block KPM solve (moments + autodiff_matrix), M=%d extrapolated "
                                   "from timed M=%d and M=%d solves" % (args.L, args.M, Ms[0], Ms[1]),
                       "N": int(N), "S": int(S), "M": args.M, "sample_M": Ms, "b": 2, "nnzb": int(H.n_blocks())},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "rate_1_thread": {"value": rate1, "unit": UNIT, "cores": 1,
                              "sample": "cubic L=%d (N=%d), S=%d: M=%d (%.1f s) and M=%d (%.1f s) solves, extrapolated "
                                        "to M=%d" % (args.cpu_L1, R1.shape[0], R1.shape[1], Ms[0], t1[Ms[0]], Ms[1],
                                                     t1[Ms[1]], args.M)},
            "product_library_loaded": fastkpm_gb300._lib._lib is not None,
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
    systems = W.config4(n_systems=args.batch_systems)
    M = args.batch_M
    Rs = [fk.probe_uncorrelated(s["H"].n_rows, s["S"], fk.RNG(s["probe_seed"])) for s in systems]
    total_rows = sum(s["H"].n_rows for s in systems)
    S = systems[0]["S"]
    bt = fk.Batch(False, "fp32")
    for s, R in zip(systems, Rs):
        bt.add(s["H"], s["es"], R)
    bt.commit()
    if args.batch_only:
        # the batched step in both accumulator forms (FK_OPT_ACC64 0 then 1), fixed mapping, direct launches
        for acc in (0, 1):
            bt.set_option(Lb.FK_OPT_ACC64, acc)
            for _ in range(max(args.warmup, 1)):
                bt.moments(M)
            bt.timer_start()
            for _ in range(args.steps):
                bt.moments(M)
            print(json.dumps({"workload": "batch moments only", "acc64": acc, "ms": bt.timer_stop() / args.steps}),
                  flush=True)
        return
    tune = bt.autotune(8)
    bt.set_option(Lb.FK_OPT_GRAPHS, 1)
    for _ in range(max(args.warmup, 1)):
        mu_b = bt.moments(M)
    with ClockSampler(0) as clk:
        bt.timer_start()
        for _ in range(args.steps):
            mu_b = bt.moments(M)
        ms_b = bt.timer_stop() / args.steps
    # time between kernels inside the replayed graph: the same moments(M) with direct launches,
    # every step launch bracketed by events, against the graph replay's time per batch
    kern_ms, n_launch = bt.profile_moments(M)
    gaps = {"graph_ms": ms_b, "kernel_ms_sum": kern_ms, "launches": n_launch,
            "gap_fraction": max(0.0, 1.0 - kern_ms / ms_b),
            "how": "sum of per-launch CUDA-event times of moments(M) with direct launches vs the CUDA-graph "
                   "replay time of the same moments(M)"}
    # the same batch with FP64 per-thread moment sums (FK_OPT_ACC64 = 1; the batch default is 0)
    bt.set_option(Lb.FK_OPT_ACC64, 1)
    for _ in range(max(args.warmup, 1)):
        mu_a = bt.moments(M)
    bt.timer_start()
    for _ in range(args.steps):
        mu_a = bt.moments(M)
    acc64_line = {"ms": bt.timer_stop() / args.steps, "what": "batched moments with FP64 per-thread sums (FK_OPT_ACC64 1)"}
    bt.set_option(Lb.FK_OPT_ACC64, 0)
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
        acc64_line["moments_max_rel_mu0_vs_fp64"] = max(acc64_line.get("moments_max_rel_mu0_vs_fp64", 0.0),
                                                        _mu_err(mu_a[k], mu))
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
    per = float(total_rows) * M * S
    bytes_step = 3 * total_rows * S * 4 + sum(s["H"].n_blocks() * 8 + 4 * (s["H"].n_rows + 1) for s in systems)
    achieved = bytes_step / (ms_b / (M // 2) * 1e-3) / 1e9
    peak, kind = peaks()
    # the whole solve's algorithmic bytes: M/2 forward steps and M/2 - 1 fused reverse steps (b=1 real
    # FP32, D accumulator 8 bytes per entry), over the host wall clock of moments + autodiff_matrix
    nnzb_all = sum(s["H"].n_blocks() for s in systems)
    bytes_adj = sum(adjoint_bytes_per_launch(s["H"].n_rows, S, s["H"].n_blocks(), 1, 4, True, cplx=False)
                    for s in systems)
    solve_bytes = (M // 2) * bytes_step + (M // 2 - 1) * bytes_adj
    ach_solve = solve_bytes / (ms_solve * 1e-3) / 1e9
    solve = {"what": "moments(M) + autodiff_matrix(c_sys) for all 64 systems (host wall clock, D copied out)",
             "ms": ms_solve, "value": float(total_rows) * M * S / (ms_solve / 1e3), "unit": UNIT,
             "sequential_fp64_ms": t_seq_solve, "speedup_vs_sequential_fp64": t_seq_solve / ms_solve,
             "D_rel_fro_vs_fp64": d_err, "D_buffer_pinned": pinned,
             "roofline_over_wall": {"bound": "hbm", "achieved": ach_solve, "peak": peak, "unit": "GB/s",
                                    "frac": ach_solve / peak, "bytes_per_solve": solve_bytes,
                                    "blocks": nnzb_all, "peak_source": kind,
                                    "over": "host wall clock of the whole solve (moments graph, batched reverse "
                                            "steps, D copied out to pinned memory)"}}
    line = {"metric": METRIC, "value": per / (ms_b / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 recursion; float-float per-thread sums, f64 across CTAs (FK_OPT_ACC64 0)",
            "data": "synthetic",
            "config": {"workload": "%d square lattices L~U{32..256}, W~U[0,4], b=1 real, M=%d, S=%d: batched moments, "
                                   "CUDA graph, autotuned" % (len(systems), M, S), "total_rows": total_rows, "M": M, "S": S,
                       "systems": len(systems)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "kernel": "k_cheb_step (batched)", "peak_source": kind},
            "sequential_fp64_ms": t_seq, "speedup_vs_sequential_fp64": t_seq / ms_b,
            "moments_max_rel_mu0_vs_fp64": err, "solve": solve, "autotune": tune, "graph_gaps": gaps, "acc64": acc64_line,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def serve_requests(n_req, seed, max_sites, rate=4.0):
    """Mixed-size KPM solve requests: cubic or square lattice (50/50), sites log-uniform over
    10^3 .. max_sites, b=1 real or b=2 complex spin-exchange (50/50), M in {200,500,1000,2000},
    S in {32,64,128} by colour probing; Poisson arrival offsets (`rate` per second)."""
    from fastkpm_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    reqs = []
    t = 0.0
    for k in range(n_req):
        t += rng.exponential(1.0 / rate)
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
    reqs = serve_requests(args.serve_requests, 5, args.serve_max_sites, args.serve_rate)
    srv = Server(max_slots=8, memory_budget=int(120e9), pack_bytes=int(args.serve_pack_bytes),
                 pack_max=16 if args.serve_pack_bytes > 0 else 1, cta_waves=args.serve_cta_waves)
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
            "config": {"workload": "Poisson stream of %d mixed KPM solves (moments + autodiff D), sites 1e3..%g, "
                                   "%g arrivals/s" % (len(reqs), args.serve_max_sites, args.serve_rate), "slots": 8,
                       "cta_waves": args.serve_cta_waves},
            "latency_p50_s": st["p50_s"], "latency_p99_s": st["p99_s"], "queue_wait_p50_s": st["queue_p50_s"],
            "service_p50_s": st["service_p50_s"], "completed": st["completed"],
            "rejected": st["rejected"], "max_concurrent": st["max_concurrent"],
            "packs": {"batches": st["packs"], "requests": st["packed_requests"], "pack_bytes": int(args.serve_pack_bytes),
                      "what": "requests solved together by one batch (one launch per Chebyshev step)"},
            "serial_fp64_probe_steps_per_s": work / t_ser, "speedup_vs_serial_fp64": (work / t_ser and
                                                                                  st["probe_steps_per_s"] / (work / t_ser)),
            "moments_max_rel_mu0_vs_fp64": worst, "serial_fp64_requests": n_ser,
            "requests": {"columns": ["rows", "M", "S", "queue_s", "service_s"],
                         "rows": [[t.n_rows, t.M, t.s, round(t.admitted - t.arrival, 4), round(t.finished - t.admitted, 4)]
                                  for t in tickets if t.error is None and t.admitted is not None]}}
    peak, kind = peaks()
    gbs = st["algorithmic_bytes"] / max(st["busy_s"], 1e-9) / 1e9
    line["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "over": "time with at least one solve in service (%.2f s of %.2f s wall)"
                                % (st["busy_s"], st["wall_s"]),
                        "bytes": "sum of each solve's algorithmic bytes (forward steps + fused reverse steps)",
                        "peak_source": kind}
    gbs_wall = st["algorithmic_bytes"] / max(st["wall_s"], 1e-9) / 1e9
    line["roofline_wall"] = {"bound": "hbm", "achieved": gbs_wall, "peak": peak, "unit": "GB/s", "frac": gbs_wall / peak,
                             "over": "wall time from the first arrival to the last completion (%.2f s)" % st["wall_s"]}
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
    prec = args.precision or "fp32"
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


def _leg_summary(r, ref):
    """JSON of one engine run; errors against the reference engine's last solve (same H, R, c, M)."""
    d = {"value": r["value"], "unit": UNIT, "ms_per_step": r["ms"] / r["steps"], "steps": r["steps"],
         "warmup": r["warmup"], "dtype": {"ds": "float-float (2 x FP32, ~48-bit significand, 8-bit exponent)",
                                          "fp32": "f32 recursion and SpMM, %s moment sums and D accumulator" % (
                                              "f64" if r["acc64"] else "float-float"),
                                          "fp64": "f64"}[r["prec"]],
         "roofline": r["roofline"], "roofline_step": r["roofline_step"], "clocks": r["clocks"],
         "kernels": {"step_avg_ms": r["avg_step_ms"], "step_launches": r["n_step"],
                     "adjoint_avg_ms": r["avg_adj_ms"], "adjoint_launches": r["n_adj"],
                     "d_epilogue_fused": r["fused"]}}
    for k in ("roofline_issue", "roofline_fp64_pipe", "e2e", "e2e_dense_R"):
        if k in r:
            d[k] = r[k]
    if ref is not None and ref is not r:
        d["err_vs_fp64"] = {"moments_max_rel_mu0": float(np.max(np.abs(r["mu"] - ref["mu"])) / abs(ref["mu"][0])),
                            "D_rel_fro": float(np.linalg.norm(r["D"] - ref["D"]) / np.linalg.norm(ref["D"])),
                            "vs": "native FP64 GPU engine, same H, R and c, M=%d" % r["M"]}
        d["speedup_vs_fp64"] = (ref["ms"] / ref["steps"]) / (r["ms"] / r["steps"])
    return d


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
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    args.precision = args.precision or "fp64"
    wl = workload(args)
    e2e_steps = 0 if args.no_e2e else args.e2e_steps
    head = run_leg(args, args.precision, args.steps, args.warmup, wl, ws, dist, dev, e2e_steps)
    legs = {}
    for prec in [p for p in args.legs.split(",") if p and p != args.precision]:
        k = args.leg_steps or {"ds": min(args.steps, 3), "fp32": min(args.steps, 5), "fp64": min(args.steps, 2)}[prec]
        legs[prec] = run_leg(args, prec, k, min(args.warmup, 2), wl, ws, dist, dev, e2e_steps)
    if args.precision == "fp32" or "fp32" in legs:
        # the FP32 engine with float-float accumulators (FK_OPT_ACC64 = 0): the cost of its FP64 sums
        from fastkpm_gb300 import _lib as Lb
        legs["fp32_float_float_sums"] = run_leg(args, "fp32", min(args.steps, 3), 1, wl, ws, dist, dev, 0,
                                                {Lb.FK_OPT_ACC64: 0})
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args, wl)
    if rank != 0:
        return
    ref = head if args.precision == "fp64" else legs.get("fp64")
    hs = _leg_summary(head, ref)
    H = wl[0]
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "ds": "float-float", "fp32": "f32"}[args.precision],
        "data": "synthetic",
        "config": {"workload": "cubic L=%d Kondo-lattice spin-block KPM solve: moments(M) + autodiff_matrix(c, D) "
                               "on H's pattern" % args.L,
                   "N": head["N"], "sites": head["N"] // 2, "b": 2, "nnzb": head["nnzb"], "M": head["M"], "S": head["S"],
                   "precision": args.precision, "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 (2 GiB per vector), no flush"},
        "roofline": hs["roofline"],
        "roofline_step": hs["roofline_step"],
        "cpu_baseline": cpu,
        "e2e": hs.get("e2e"),
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
        "kernels": hs["kernels"],
    }
    for k in ("roofline_fp64_pipe", "roofline_issue", "e2e_dense_R", "err_vs_fp64"):
        if k in hs:
            line[k] = hs[k]
    line["legs"] = {p: _leg_summary(r, ref) for p, r in legs.items()}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
