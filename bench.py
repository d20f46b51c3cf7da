#!/usr/bin/env python3
"""Benchmark of the local ensemble square-root analysis (OAK locAnalysis) on GB300.

Workload (default): the local FP64 configuration -- 360 x 180 x 20 grid, one variable,
N = 64 members, m = 50,000 observations (70 % on tracks), 64,800 column zones, Gaspari-Cohn
localisation radius 12 cells. Synthetic seeded inputs of those shapes (oak_gb300.workloads).

One step = one oakg_locanalysis call over all zones (observation binning, selection + Gram,
eigensolve + transform, ensemble update). The metric is local analyses (zones) per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference algorithm on the host cores: the C/OpenMP restatement
of rrsqrt.F90 / assimilation.F90 (oracle/oakref.c with LAPACK dsyev), a port because the
Fortran reference cannot be compiled here (no Fortran compiler).
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

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")  # BLAS inside each OpenMP thread (CPU leg)

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = ("local analyses/s: mixed-prec vs FP64 on GB300 at ≤1e-4 rel err; adjoint cost")
UNIT = "local analyses/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--scale", type=float, default=1.0, help="horizontal scale of the workload")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="target CPU time of the cpu_baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-mixed", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-global", action="store_true")
    p.add_argument("--no-graph", action="store_true")
    p.add_argument("--no-layout", action="store_true")
    p.add_argument("--no-rows", action="store_true",
                   help="skip the ensemble / SMWCovar / rrsqrt-wrapper section")
    p.add_argument("--batched-scale", type=float, default=1.0,
                   help="horizontal scale of the 5-variable N = 100 batched workload, FP32 "
                        "storage, generated on the GPU (0 skips it)")
    p.add_argument("--large-scale", type=float, default=1.0,
                   help="horizontal scale of the 2-variable N = 128 large workload, FP32 "
                        "storage, generated on the GPU (0 skips it)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(c, scale):
    return {"workload": c.name, "zones": int(c.Z), "n": int(c.n), "N": int(c.N), "m": int(c.m),
            "localisation": "Gaspari-Cohn locfun(d/6), maxLength 12 cells",
            "precision": "fp64 (plain form: FP64 selection, weights, eigensolve and update; "
                         "the Gram and the square-root transform's U (I+L)^-1/2 U^T as exact "
                         "integer products of 8-bit slices on the BF16 tensor cores)",
            "horizontal_scale": scale,
            "l2": "inputs larger than L2 (Sf and Sa 664 MB each at full scale)"}


# --------------------------------------------------------------------------- CPU baseline

def cpu_sample(c, target_zones):
    """A bounded sample of the workload: every k-th zone, all observations (the reference's
    brute-force selection over all m observations stays in the sample's cost)."""
    k = max(1, c.Z // max(1, target_zones))
    zsel = np.arange(0, c.Z, k)
    starts = np.concatenate([[0], np.cumsum(c.zone_size)[:-1]])
    rows = np.concatenate([np.arange(starts[z], starts[z] + c.zone_size[z]) for z in zsel])
    return zsel, rows


def run_cpu_oracle(c, zsel, rows, threads, keep=None):
    """Times one oracle pass over the zones `zsel` (state rows `rows`); with a list `keep`,
    keeps the pass's outputs (zsel, rows, xa, Sa, nobs) in it for the parity record."""
    from oracle import cref
    t0 = time.perf_counter()
    xa, Sa, _, nobs = cref.locanalysis(
        c.zone_size[zsel], c.xf[rows], c.Hxf, c.yo, c.Sf[rows], c.HSf, c.r_diag,
        c.zone_pos[zsel], c.obs_pos, c.corr_len[zsel], c.max_len[zsel], kind=c.weight,
        metric=c.metric, loctype=c.loctype, nthreads=threads)
    dt = time.perf_counter() - t0
    if keep is not None:
        keep[:] = [(zsel, rows, xa, Sa, nobs)]
    return dt


def cpu_baseline(c, seconds, threads, keep=None):
    """Times the C/OpenMP oracle for ~`seconds` of CPU work: whole passes over the workload
    while one pass fits the budget, else a zone sample sized from a calibration run. The last
    pass's outputs go to `keep` (see run_cpu_oracle)."""
    zsel, rows = cpu_sample(c, 2048)
    dt = run_cpu_oracle(c, zsel, rows, threads, keep)    # calibration
    per_zone = dt / len(zsel)
    if per_zone * c.Z <= seconds:
        zsel, rows = np.arange(c.Z), np.arange(c.n)
        total, passes = 0.0, 0
        while total < seconds and passes < 8:
            total += run_cpu_oracle(c, zsel, rows, threads, keep)
            passes += 1
        return {"value": passes * c.Z / total, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"{passes} full passes over all {c.Z} zones and {c.m} observations "
                          f"({total:.1f} s), brute-force selection as "
                          f"assimilation.F90:3745-3757, LAPACK dsyev via SciPy, OpenMP dynamic "
                          f"schedule"}
    target = int(min(c.Z, max(256, seconds / max(per_zone, 1e-9))))
    zsel, rows = cpu_sample(c, target)
    dt = run_cpu_oracle(c, zsel, rows, threads, keep)
    return {"value": len(zsel) / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(zsel)} of {c.Z} zones (every {c.Z // len(zsel)}-th), all {c.m} "
                      f"observations, brute-force selection as assimilation.F90:3745-3757, "
                      f"LAPACK dsyev via SciPy, OpenMP dynamic schedule, {dt:.2f} s"}


def parity_record(xa_d, Sa_d, nobs_d, c, ref, tol):
    """Errors of one form's outputs (device tensors xa (n), Sa (n, N), nobs (Z)) against the
    oracle pass in `ref` (zsel, rows, xa, Sa, nobs): the increment-relative error of the mean
    ||xa - xa_o|| / ||xa_o - xf||, the relative Frobenius error of the anomalies, and the
    selection counts (compared exactly). Rows of zones whose count differs are left out of
    the norms (none, for the Cartesian metric)."""
    zsel, rows, xa_o, Sa_o, nobs_o = ref
    full = len(rows) == c.n
    xa = xa_d.cpu().numpy() if full else xa_d[torch_index(xa_d, rows)].cpu().numpy()
    Sa = Sa_d.cpu().numpy() if full else Sa_d[torch_index(Sa_d, rows)].cpu().numpy()
    nobs = nobs_d.cpu().numpy()[zsel]
    same = nobs == nobs_o
    keep = np.repeat(same, c.zone_size[zsel])
    xf = c.xf[rows][keep]
    inc = max(float(np.linalg.norm(xa_o[keep] - xf)), 1e-300)
    e_mean = float(np.linalg.norm(xa[keep] - xa_o[keep])) / inc
    e_anom = float(np.linalg.norm(Sa[keep] - Sa_o[keep]) / max(np.linalg.norm(Sa_o[keep]), 1e-300))
    e_abs = float(np.linalg.norm(xa[keep] - xa_o[keep]) / max(np.linalg.norm(xa_o[keep]), 1e-300))
    return {"zones": int(len(zsel)), "zones_same_selection": int(same.sum()),
            "rel_err_mean_increment": e_mean, "rel_err_mean": e_abs,
            "rel_err_anomalies": e_anom, "tolerance": tol,
            "pass": bool(same.all() and e_mean <= tol and e_anom <= tol)}


def update_bytes(n, N, nobs, zone_size, s):
    """Algorithmic bytes of one update stage: Sf read and Sa written (n x N), xf read and xa
    written (n), all of s bytes; T (N x N FP32) read for every zone with observations."""
    return 2 * n * N * s + 2 * n * s + int((np.asarray(nobs) > 0).sum()) * N * N * 4


def torch_index(t, rows):
    import torch
    return torch.as_tensor(rows, device=t.device)


# --------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- GPU arm

def algorithmic_work(c, nobs, stage):
    """Algorithmic FP64 flops of one launch of a stage (per-zone counts x zones):
    gram: p N (N+1) + 2 p N   (lower-triangular HS^T diag(c) HS plus HS^T diag(c) d)
    eig:  9 N^3 (Householder tridiagonalisation + QR with vectors) + 2 N^3 + 4 N^2 (T, ampl),
          less T_sym's N^2 (N+1) where it runs on the tensor cores (N <= 64): the count is
          the FP64-pipe work, set against the FP64 peak
    update: 2 nz N^2 + 2 nz N (Sf T and Sf ampl), zones with observations."""
    N = c.N
    act = nobs > 0
    p = nobs[act].astype(np.float64)
    nz = c.zone_size[act].astype(np.float64)
    if stage == "gram":
        return float(np.sum(p * N * (N + 1) + 2 * p * N))
    if stage == "eig":
        tsym_tc = float(N * N * (N + 1)) if N <= 64 else 0.0
        return float(act.sum() * (11.0 * N ** 3 + 4.0 * N ** 2 - tsym_tc))
    return float(np.sum(2 * nz * N * N + 2 * nz * N))


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    import torch
    import oak_gb300
    from oak_gb300 import build as _build
    from oak_gb300.workloads import local_case

    # workload first (numpy), CPU baseline before any CUDA work
    c = local_case(scale=args.scale)
    cpu = None
    oracle_out = []   # the oracle's outputs of its last timed pass, for the parity record
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(c, args.cpu_seconds, os.cpu_count() or 1, oracle_out)

    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _build.build()
    L = oak_gb300.lib()

    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
    d_args = (T(c.zone_size), T(c.xf), T(c.Hxf), T(c.yo), F(c.Sf), F(c.HSf), T(c.r_diag),
              T(c.zone_pos), tuple(T(x) for x in c.obs_pos), T(c.corr_len), T(c.max_len))
    stream = torch.cuda.current_stream(dev)
    L.oakg_set_stream(ctypes_ptr(stream.cuda_stream))

    def step():
        return oak_gb300.loc_analysis(*d_args, weight=c.weight, metric=c.metric,
                                      loctype=c.loctype, want_ampl=False)

    out = None
    for _ in range(args.warmup):
        out = step()
    nobs = out[3].cpu().numpy()
    peak_fp64 = ctypes_double()
    L.oakg_fp64_peak(ctypes_ref(peak_fp64))

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    stage_ms = {"obs_prep": 0.0, "gram": 0.0, "eig": 0.0, "update": 0.0, "total": 0.0}
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize(dev)
    launches0 = L.oakg_launch_count()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
        for k, v in oak_gb300.last_timings().items():
            stage_ms[k] += v
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    launches = L.oakg_launch_count() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * c.Z / (ms / 1e3)
    parity = None
    if oracle_out:
        parity = {"oracle": "oracle/oakref.c (C/OpenMP restatement, LAPACK dsyev), the passes "
                            "of cpu_baseline",
                  "fp64": parity_record(out[0], out[1], out[3], c,
                                        oracle_out[0], 1e-10)}

    # mixed-precision form on the same device inputs; errors against the FP64 form's outputs
    mixed = None
    if not args.no_mixed:
        ref_xa, ref_Sa = out[0].clone(), out[1].clone()

        def timed_form(prec):
            def mstep():
                return oak_gb300.loc_analysis(*d_args, weight=c.weight, metric=c.metric,
                                              loctype=c.loctype, want_ampl=False,
                                              precision=prec)
            for _ in range(args.warmup):
                mout = mstep()
            mstage = {"obs_prep": 0.0, "gram": 0.0, "eig": 0.0, "update": 0.0, "total": 0.0}
            barrier()
            torch.cuda.synchronize(dev)
            m0 = torch.cuda.Event(enable_timing=True)
            m1 = torch.cuda.Event(enable_timing=True)
            m0.record(stream)
            for _ in range(args.steps):
                mout = mstep()
                for k, v in oak_gb300.last_timings().items():
                    mstage[k] += v
            m1.record(stream)
            torch.cuda.synchronize(dev)
            barrier()
            mms = m0.elapsed_time(m1) / args.steps
            xf_d = d_args[1]
            e_mean = float(torch.linalg.norm(mout[0] - ref_xa) / torch.linalg.norm(ref_xa - xf_d))
            e_anom = float(torch.linalg.norm(mout[1] - ref_Sa) / torch.linalg.norm(ref_Sa))
            st = {k: v / args.steps for k, v in mstage.items()}
            res = {"value": ws * c.Z / (mms / 1e3), "unit": UNIT, "ms_per_step": mms,
                   "speedup_vs_fp64": ms / mms, "rel_err_mean_increment": e_mean,
                   "rel_err_anomalies": e_anom, "stage_ms_per_step": st,
                   "update_GBs": update_bytes(c.n, c.N, nobs, c.zone_size, 8) / (st["update"] / 1e3)
                   / 1e9}
            return res, mout

        mixed, mout = timed_form(oak_gb300.PREC_MIXED)
        mixed["precision"] = ("FP64 selection and (1+lambda)^-1/2 scaling; FP32 Gram (tensor "
                              "cores) and eigensolve; FP32 update (CUDA cores: 20-element zones); "
                              "compensated FP32 innovation sums")
        if parity is not None:
            parity["mixed"] = parity_record(mout[0], mout[1], mout[3], c, oracle_out[0], 1e-4)
        del mout
        mixed64, mout = timed_form(oak_gb300.PREC_MIXED_FP64EIG)
        mixed64["precision"] = ("the mixed form with the FP32 eigenpairs refined to FP64 "
                                "accuracy (Ogita-Aishima, exact FP32 products): FP64 accuracy "
                                "for the eigensolve and the (1+lambda)^-1/2 scalings only")
        if parity is not None:
            parity["mixed_fp64eig"] = parity_record(mout[0], mout[1], mout[3], c, oracle_out[0],
                                                    1e-4)
        mixed["fp64_eigensolve"] = mixed64
        del ref_xa, ref_Sa, mout

    # adjoint cost: J = mean over a 60 x 40 column sub-region (all levels) of (xa - x_true)^2,
    # gradients w.r.t. yo, r, the localisation length factor and the prior inflation (1.05)
    adjoint = None
    if not args.no_adjoint:
        nx = int(round(360 * args.scale))
        zc = np.arange(c.Z)
        subz = ((zc % nx) >= nx // 3) & ((zc % nx) < nx // 3 + max(1, round(60 * args.scale))) & \
               ((zc // nx) >= 60 * args.scale) & ((zc // nx) < 60 * args.scale + max(1, round(40 * args.scale)))
        sub = np.repeat(subz, c.zone_size)
        xt_d = T(c.x_true)
        sub_d = T(sub.astype(np.float64))
        xa_fwd = step()[0]
        seed = 2.0 * (xa_fwd - xt_d) * sub_d / float(sub.sum())
        a_args = (d_args[0], d_args[2], d_args[3], d_args[4], d_args[5], d_args[6], d_args[7],
                  d_args[8], d_args[9], d_args[10])

        def astep():
            return oak_gb300.loc_analysis_adjoint(*a_args, seed, inflation=1.05, weight=c.weight,
                                                  metric=c.metric, loctype=c.loctype)
        for _ in range(args.warmup):
            astep()
        torch.cuda.synchronize(dev)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            ga = astep()
        a1.record(stream)
        torch.cuda.synchronize(dev)
        ams = a0.elapsed_time(a1) / args.steps
        # worst case: a cost over the whole domain seeds every zone
        seed_all = 2.0 * (xa_fwd - xt_d) / float(c.n)

        def astep_all():
            return oak_gb300.loc_analysis_adjoint(*a_args, seed_all, inflation=1.05,
                                                  weight=c.weight, metric=c.metric,
                                                  loctype=c.loctype)
        astep_all()
        torch.cuda.synchronize(dev)
        a0.record(stream)
        for _ in range(args.steps):
            astep_all()
        a1.record(stream)
        torch.cuda.synchronize(dev)
        ams_all = a0.elapsed_time(a1) / args.steps
        adjoint = {"ms_per_call": ams, "cost_vs_forward_fp64": ams / ms,
                   "ms_per_call_all_zones": ams_all,
                   "cost_vs_forward_fp64_all_zones": ams_all / ms,
                   "dJ_dinfl_posterior_mult": 0.0,
                   "cost_vs_forward_mixed": (ams / mixed["ms_per_step"]) if mixed else None,
                   "cost": "J = mean over a 60x40 column sub-region (all levels) of "
                           "(xa - x_true)^2; gradients w.r.t. all yo, r, the localisation "
                           "length factor and the prior inflation 1.05 (the scaling of Sf and "
                           "HSf, ErrorSpace.scale); the posterior inflation.mult scales Sa "
                           "only, so its derivative of a mean-based J is 0",
                   "zones_seeded": int(subz.sum()), "dJ_dlen": ga[2], "dJ_dinfl": ga[3]}

    # prepared analyses replayed as CUDA graphs (oakg_plan_*): FP64 with the default cell edge,
    # mixed with the tuned one; each execution waits for its status
    graph = None
    if not args.no_graph:
        def time_plan(pl, k):
            for _ in range(2):
                pl.execute(stream)
            torch.cuda.synchronize(dev)
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            for _ in range(k):
                pl.execute(stream)
            p1.record(stream)
            torch.cuda.synchronize(dev)
            return p0.elapsed_time(p1) / k
        kw = dict(weight=c.weight, metric=c.metric, loctype=c.loctype)
        pl = oak_gb300.Plan(*d_args, **kw)
        g64 = time_plan(pl, args.steps)
        nodes64 = pl.info["graph_nodes"]
        pl.close()
        pl = oak_gb300.Plan(*d_args, precision=oak_gb300.PREC_MIXED, tune=True, **kw)
        gmx = time_plan(pl, max(args.steps, 5))
        info = pl.info
        pl.close()
        graph = {"fp64_ms_per_step": g64, "fp64_graph_nodes": nodes64,
                 "mixed_tuned_ms_per_step": gmx,
                 "mixed_tuned_value": ws * c.Z / (gmx / 1e3),
                 "mixed_tuned_speedup_vs_fp64": ms / gmx,
                 "mixed_cell_size": info["cell_size"], "mixed_graph_nodes": info["graph_nodes"],
                 "tuning_cell_ms": info["tuning"], "mixed_zone_order": info["zone_order"],
                 "zone_order_gram_ms": info["zone_order_ms"]}

    # global analysis (rrsqrt.F90:196-208) of the 100 x 80, N = 30, m = 500 configuration:
    # device-resident time per analysis, and the CPU port on the host cores beside it
    glob = None
    if not args.no_global and rank == 0:
        from oak_gb300.workloads import global_case
        g = global_case()
        gd = (T(g.xf), T(g.Hxf), T(g.yo), F(g.Sf), F(g.HSf), T(g.r_diag))
        for _ in range(max(3, args.warmup)):
            oak_gb300.analysis(*gd)
        torch.cuda.synchronize(dev)
        kg = 50
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(kg):
            oak_gb300.analysis(*gd)
        g1.record(stream)
        torch.cuda.synchronize(dev)
        gms = g0.elapsed_time(g1) / kg
        glob = {"workload": g.name, "ms_per_analysis": gms,
                "note": "device-resident inputs; each call synchronises (status read-back)"}
        if not args.no_cpu_baseline:
            from oracle import cref
            cref.analysis(g.xf, g.Hxf, g.yo, g.Sf, g.HSf, g.r_diag)
            t0 = time.perf_counter()
            for _ in range(10):
                cref.analysis(g.xf, g.Hxf, g.yo, g.Sf, g.HSf, g.r_diag)
            glob["cpu_ms_per_analysis"] = (time.perf_counter() - t0) / 10 * 1e3
            glob["cpu_kind"] = "port (oracle/oakref.c, LAPACK dsyev)"

    # column workloads of the mixed-precision configurations at full size, FP32 storage,
    # generated on the GPU (column_section): both forms, oracle parity on a zone sample
    #   batched: 5 variables on 720 x 360 columns of 121 elements, N = 100, 200,000 bilinear
    #            observations on track segments;
    #   large:   2 variables on 1440 x 720 columns of 100 elements, N = 128, 1M clustered
    #            observations, with the adjoint of J = mean over a 200 x 200 column sub-region
    batched = None
    if args.batched_scale > 0:
        from oak_gb300.workloads import batched_case_device
        dc = batched_case_device(scale=args.batched_scale, device=dev)
        batched = column_section(torch, dev, stream, args, barrier, ws, dc, args.batched_scale)
        del dc
        torch.cuda.empty_cache()
    large = None
    if args.large_scale > 0:
        from oak_gb300.workloads import large_case_device
        dc = large_case_device(scale=args.large_scale, device=dev)
        large = column_section(torch, dev, stream, args, barrier, ws, dc, args.large_scale,
                               adjoint_sub=200)
        del dc
        torch.cuda.empty_cache()

    # layout builders on one 3-D variable of 720 x 360 x 50 points (x fastest), zones = the
    # 259,200 columns (partition = column number), a land mask, 10^6 observations: zone
    # layout (initPartition), sea packing, rectilinear observation operator (cinterp), the
    # zone-order permutation of a 16-member ensemble; CPU: the oracle on bounded samples
    layout = None
    if not args.no_layout:
        layout = layout_section(torch, dev, stream, args, barrier)

    # the analysis path's neighbours on the same workload: the whole-ensemble entry (H Ef,
    # prologue, local analysis, epilogue), the SMWCovar observation covariance (k = 8), and the
    # rrsqrt.F90 wrappers (ens2sqrt / sqrt2ens, ensAnalysis, biasedLocAnalysis)
    rows = None
    if not args.no_rows and rank == 0:
        rows = rows_section(torch, dev, stream, args, c, d_args, ms, T, F)

    # e2e through the public API with host (pinned) buffers: H2D + D2H inside the timed region
    e2e = None
    if not args.no_e2e:
        def pinned(a, fortran=False):
            a = np.asarray(a)
            if fortran:
                t = torch.empty((a.shape[1], a.shape[0]), dtype=torch.float64, pin_memory=True)
                t.numpy()[...] = a.T
                return t.numpy().T
            t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0].copy()).dtype, pin_memory=True)
            t.numpy()[...] = a
            return t.numpy()
        h = (pinned(c.zone_size), pinned(c.xf), pinned(c.Hxf), pinned(c.yo),
             pinned(c.Sf, True), pinned(c.HSf, True), pinned(c.r_diag), pinned(c.zone_pos),
             tuple(pinned(x) for x in c.obs_pos[:2]), pinned(c.corr_len), pinned(c.max_len))
        h2d = sum(x.nbytes for x in h[:8]) + sum(x.nbytes for x in h[8]) + h[9].nbytes + h[10].nbytes
        d2h = c.xf.nbytes + c.Sf.nbytes + c.Z * 4
        outs = (pinned(np.zeros(c.n)), pinned(np.zeros((c.n, c.N)), True))

        def hstep():
            return oak_gb300.loc_analysis(*h, weight=c.weight, metric=c.metric,
                                          loctype=c.loctype, want_ampl=False, out=outs)
        hstep()
        ksteps = max(1, min(args.steps, 3))
        barrier()
        torch.cuda.synchronize(dev)
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(ksteps):
            hstep()
        g1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        ems = g0.elapsed_time(g1) / ksteps
        e2e = {"value": ws * c.Z / (ems / 1e3), "unit": UNIT, "ms_per_step": ems,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "host_buffers": "pinned"}
    L.oakg_set_stream(None)

    if rank != 0:
        return
    per_step = {k: v / args.steps for k, v in stage_ms.items()}
    dom = max(("gram", "eig", "update"), key=lambda k: per_step[k])
    kernel = {"gram": "k_zone_gram_oz", "eig": "k_zone_eig_fp64",
              "update": "k_zone_update_fp64"}[dom]
    work = algorithmic_work(c, nobs, dom)
    achieved = work / (per_step[dom] / 1e3) / 1e12
    peak = peak_fp64.value
    traffic = read_traffic(kernel)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, BASELINE shapes)",
        "config": workload_config(c, args.scale) | {"parallelism": f"zones sharded, {ws} GPU(s)",
                                                     "zones_with_obs": int((nobs > 0).sum())},
        "e2e": e2e,
        "parity": parity,
        "mixed": mixed,
        "batched": batched,
        "large": large,
        "adjoint": adjoint,
        "global_analysis": glob,
        "layout": layout,
        "rows": rows,
        "graph": graph,
        "gpu_launches": int(launches),
        "stage_ms_per_step": per_step,
        "roofline": {"kernel": kernel, "bound": "fp64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak if peak > 0 else None,
                     "peak_source": "measured FP64 FMA loop (oakg_fp64_peak) on this GPU",
                     "kernels": ("E1-E4: k_eig_tridiag, k_eig_tridiag_values, "
                                 "k_eig_vectors_fp64, k_eig_transform, k_zone_tsym_oz"
                                 if kernel == "k_zone_eig_fp64" else kernel),
                     "traffic": traffic,
                     "algorithmic_flops_per_launch": work},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


def column_oracle_sample(dc, nobs, k=96, seed=7):
    """The oracle on a zone sample of a device workload: the k zones with the most observations
    and k random zones with observations; inputs are the FP32 arrays widened to FP64, every
    observation tested (brute-force selection). Returns (zsel, rows, xa, Sa, nobs)."""
    from oracle import cref
    rng = np.random.default_rng(seed)
    act = np.flatnonzero(nobs > 0)
    top = np.argsort(-nobs, kind="stable")[:k]
    rnd = rng.choice(act, size=min(k, act.size), replace=False) if act.size else act
    zsel = np.unique(np.concatenate([top, rnd]))
    starts = np.concatenate([[0], np.cumsum(dc.zone_size)[:-1]])
    rows = np.concatenate([np.arange(starts[z], starts[z] + dc.zone_size[z]) for z in zsel])
    import torch
    rows_d = torch.as_tensor(rows, device=dc.Sf.device)
    Sf = dc.Sf[rows_d].double().cpu().numpy()
    xf = dc.xf[rows_d].double().cpu().numpy()
    HSf = dc.HSf.double().cpu().numpy()
    xa, Sa, _, nob = cref.locanalysis(
        dc.zone_size[zsel], xf, dc.Hxf.double().cpu().numpy(), dc.yo.double().cpu().numpy(),
        Sf, HSf, dc.r_diag.double().cpu().numpy(), dc.zone_pos[zsel], dc.obs_pos,
        dc.corr_len[zsel], dc.max_len[zsel], kind=dc.weight, metric=dc.metric,
        loctype=dc.loctype, nthreads=os.cpu_count() or 1)
    return zsel, rows, xa, Sa, nob, xf


def column_parity(xa_d, Sa_d, nobs_d, ref, zone_size, tol):
    """Errors of one form's outputs against the oracle sample (see parity_record)."""
    import torch
    zsel, rows, xa_o, Sa_o, nobs_o, xf = ref
    rows_d = torch.as_tensor(rows, device=xa_d.device)
    xa = xa_d[rows_d].double().cpu().numpy()
    Sa = Sa_d[rows_d].double().cpu().numpy()
    nobs = nobs_d.cpu().numpy()[zsel]
    same = nobs == nobs_o
    keep = np.repeat(same, zone_size[zsel])
    inc = max(float(np.linalg.norm(xa_o[keep] - xf[keep])), 1e-300)
    e_mean = float(np.linalg.norm(xa[keep] - xa_o[keep])) / inc
    e_anom = float(np.linalg.norm(Sa[keep] - Sa_o[keep]) / max(np.linalg.norm(Sa_o[keep]), 1e-300))
    return {"zones": int(len(zsel)), "zones_same_selection": int(same.sum()),
            "obs_per_zone_max_in_sample": int(nobs_o.max()) if len(nobs_o) else 0,
            "rel_err_mean_increment": e_mean, "rel_err_anomalies": e_anom, "tolerance": tol,
            "pass": bool(same.all() and e_mean <= tol and e_anom <= tol)}


def column_section(torch, dev, stream, args, barrier, ws, dc, scale, adjoint_sub=None):
    """Both forms on a column workload held on the GPU in FP32 (oakg_locanalysis_f32): the
    mixed form, then the FP64 form (FP32 inputs widened, FP64 products, outputs rounded to FP32),
    each checked against the oracle on a zone sample; the mixed form's errors against the FP64
    form's outputs over every zone; with adjoint_sub, the FP64 adjoint of J = mean over an
    adjoint_sub^2 column sub-region (scaled with the grid) of (xa - x_true)^2."""
    import oak_gb300
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    bd = (T(dc.zone_size), dc.xf, dc.Hxf, dc.yo, dc.Sf, dc.HSf, dc.r_diag, T(dc.zone_pos),
          tuple(T(x) for x in dc.obs_pos), T(dc.corr_len), T(dc.max_len))
    n, N = dc.n, dc.N
    xa = torch.empty(n, dtype=torch.float32, device=dev)
    Sa = torch.empty((N, n), dtype=torch.float32, device=dev).t()

    def bstep(prec):
        return oak_gb300.loc_analysis(*bd, weight=dc.weight, metric=dc.metric,
                                      loctype=dc.loctype, want_ampl=False, precision=prec,
                                      out=(xa, Sa))

    def timed(fn, warm, steps):
        for _ in range(warm):
            o = fn()
        st = {"obs_prep": 0.0, "gram": 0.0, "eig": 0.0, "update": 0.0, "total": 0.0}
        barrier()
        torch.cuda.synchronize(dev)
        b0 = torch.cuda.Event(enable_timing=True)
        b1 = torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        for _ in range(steps):
            o = fn()
            for k, v in oak_gb300.last_timings().items():
                st[k] += v
        b1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        return o, b0.elapsed_time(b1) / steps, {k: v / steps for k, v in st.items()}

    # the FP64 form costs ~N^3 FP64 flops a zone: bounded warm-up and steps at full size
    big = dc.Z * N ** 3 > 4e11
    wm, sm = (2, 3) if big else (args.warmup, args.steps)
    w64, s64 = (1, 1) if big else (args.warmup, args.steps)
    om, msm, stm = timed(lambda: bstep(oak_gb300.PREC_MIXED), wm, sm)
    nobs = om[3].cpu().numpy()
    ref = column_oracle_sample(dc, nobs)
    par_m = column_parity(xa, Sa, om[3], ref, dc.zone_size, 1e-4)
    oe, mse, ste = timed(lambda: bstep(oak_gb300.PREC_MIXED_FP64EIG), wm, sm)
    par_e = column_parity(xa, Sa, oe[3], ref, dc.zone_size, 1e-4)
    del oe
    om, _, _ = timed(lambda: bstep(oak_gb300.PREC_MIXED), 0, 1)  # the mixed outputs again
    xam, Sam = xa.clone(), Sa.clone()
    o64, ms64, st64 = timed(lambda: bstep(oak_gb300.PREC_FP64), w64, s64)
    # FP64 products, outputs rounded to FP32: the rounding bounds the error against the oracle
    par_64 = column_parity(xa, Sa, o64[3], ref, dc.zone_size, 1e-5)
    inc = torch.linalg.norm(xa.double() - dc.xf.double())
    e_mean = float(torch.linalg.norm(xam.double() - xa.double()) / inc)
    d2 = s2 = 0.0
    for k in range(N):  # member by member: FP64 temporaries of one column only
        a64, m64 = Sa[:, k].double(), Sam[:, k].double()
        d2 += float(torch.sum((m64 - a64) ** 2))
        s2 += float(torch.sum(a64 ** 2))
    e_anom = (d2 / max(s2, 1e-300)) ** 0.5
    del xam, Sam
    res = {"workload": dc.name, "scale": scale, "zones": dc.Z, "N": N, "m": dc.m,
           "storage": "fp32 (oakg_locanalysis_f32)",
           "obs_per_zone_max": int(nobs.max()), "obs_per_zone_mean": float(nobs.mean()),
           "mixed": {"value": ws * dc.Z / (msm / 1e3), "unit": UNIT, "ms_per_step": msm,
                     "warmup": wm, "steps": sm, "stage_ms_per_step": stm,
                     "update_GBs": update_bytes(n, N, nobs, dc.zone_size, 4)
                     / (stm["update"] / 1e3) / 1e9,
                     "parity_oracle_sample": par_m},
           "mixed_fp64_eigensolve": {
               "value": ws * dc.Z / (mse / 1e3), "unit": UNIT, "ms_per_step": mse,
               "warmup": wm, "steps": sm, "stage_ms_per_step": ste,
               "parity_oracle_sample": par_e,
               "precision": "the FP32 eigenpairs refined to FP64 accuracy (Ogita-Aishima, "
                            "exact FP32 products)"},
           "fp64": {"value": ws * dc.Z / (ms64 / 1e3), "unit": UNIT, "ms_per_step": ms64,
                    "warmup": w64, "steps": s64, "stage_ms_per_step": st64,
                    "parity_oracle_sample": par_64},
           "speedup_vs_fp64": ms64 / msm,
           "speedup_vs_fp64_fp64_eigensolve": ms64 / mse,
           "mixed_vs_fp64_rel_err_mean_increment": e_mean,
           "mixed_vs_fp64_rel_err_anomalies": e_anom,
           "generation": "seeded Gaussian random fields generated on the GPU (torch FFTs, FP32)",
           "update_bytes_per_step_fp32": int(2 * n * N * 4 + 2 * n * 4)}
    if adjoint_sub is not None:
        res["adjoint"] = column_adjoint(torch, dev, stream, dc, xa, scale, adjoint_sub, ms64,
                                        msm, timed)
    del xa, Sa, bd
    return res


def column_adjoint(torch, dev, stream, dc, xa, scale, sub, ms64, msm, timed):
    """The FP64 adjoint of J = mean over a sub x sub column sub-region of (xa - x_true)^2. Only
    the zones of the sub-region have a non-zero seed; zones are independent, so the adjoint
    runs on the sub-problem of those zones (their rows of Sf, all observations), widened to
    FP64, which gives the same gradients as the whole state."""
    import oak_gb300
    nx = dc.nx
    w = max(1, int(round(sub * scale)))
    zc = np.arange(dc.Z)
    subz = ((zc % nx) >= nx // 3) & ((zc % nx) < nx // 3 + w) & \
           ((zc // nx) >= w // 2) & ((zc // nx) < w // 2 + w)
    zsel = np.flatnonzero(subz)
    starts = np.concatenate([[0], np.cumsum(dc.zone_size)[:-1]])
    rows = np.concatenate([np.arange(starts[z], starts[z] + dc.zone_size[z]) for z in zsel])
    rows_d = torch.as_tensor(rows, device=dev)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    Sf_sub = dc.Sf[rows_d].double().t().contiguous().t()
    HSf = dc.HSf.double().t().contiguous().t()
    seed = 2.0 * (xa[rows_d].double() - dc.x_true[rows_d].double()) / float(rows.size)
    a_args = (T(dc.zone_size[zsel]), dc.Hxf.double(), dc.yo.double(), Sf_sub, HSf,
              dc.r_diag.double(), T(dc.zone_pos[zsel]), tuple(T(x) for x in dc.obs_pos),
              T(dc.corr_len[zsel]), T(dc.max_len[zsel]))
    ga, ams, _ = timed(lambda: oak_gb300.loc_analysis_adjoint(
        *a_args, seed, inflation=1.05, weight=dc.weight, metric=dc.metric,
        loctype=dc.loctype), 2, 3)
    return {"ms_per_call": ams, "cost_vs_forward_fp64": ams / ms64,
            "cost_vs_forward_mixed": ams / msm, "zones_seeded": int(zsel.size),
            "cost": f"J = mean over a {w}x{w} column sub-region (all levels) of "
                    "(xa - x_true)^2 at the FP64 analysis; gradients w.r.t. all yo, r, the "
                    "localisation length factor and the prior inflation 1.05; run on the "
                    "sub-region's zones (FP64 copies of their rows), which the seed confines "
                    "the adjoint to",
            "dJ_dlen": ga[2], "dJ_dinfl": ga[3]}


def layout_section(torch, dev, stream, args, barrier):
    import oak_gb300
    nx, ny, nz = 720, 360, 50
    n = nx * ny * nz
    Z = nx * ny
    rng = np.random.default_rng(12)
    e = torch.arange(n, device=dev, dtype=torch.int64)
    part = (e % Z + 1).to(torch.int32)
    del e
    x = np.linspace(-180.0, 179.5, nx)
    y = np.linspace(-89.75, 89.75, ny)
    z = np.cumsum(rng.uniform(1.0, 50.0, nz))
    mask = np.zeros((nx, ny, nz), dtype=bool)
    mask[100:200, 50:120, :] = True
    mask[:, :, 30:] |= (np.arange(nx)[:, None, None] % 5 == 0)
    mask_d = torch.as_tensor(mask.reshape(-1, order="F"), device=dev)
    m = 1_000_000
    pos = [torch.as_tensor(rng.uniform(-180.0, 179.5, m), device=dev),
           torch.as_tensor(rng.uniform(-89.75, 89.75, m), device=dev),
           torch.as_tensor(rng.uniform(z[0], z[-1], m), device=dev)]
    axes = [torch.as_tensor(a, device=dev) for a in (x, y, z)]
    ens = torch.empty((16, n), dtype=torch.float64, device=dev).normal_().t()

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            out = fn()
        barrier()
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            out = fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return out, a.elapsed_time(b) / args.steps

    L = oak_gb300.lib()
    l0 = L.oakg_launch_count()
    (zs, zi, inv), ms_layout = timed(lambda: oak_gb300.zone_layout(part, Z))
    (sea, nsea), ms_sea = timed(lambda: oak_gb300.sea_index(mask_d))
    (idx, w), ms_oper = timed(lambda: oak_gb300.obsoper_rectilinear(axes, pos, sea=sea))
    _, ms_perm = timed(lambda: oak_gb300.permute_rows(zi, ens))
    launches = L.oakg_launch_count() - l0
    ok_layout = bool((zs == nz).all().item()) and int(zi[nz - 1].item()) == (nz - 1) * Z
    inside = float((idx[:, 0] >= 0).float().mean().item())
    perm_bytes = n * 16 * 16 + n * 4
    res = {"grid": f"{nx} x {ny} x {nz} points, x fastest; {Z} column zones; {m} observations",
           "zone_layout": {"ms": ms_layout, "elements_per_s": n / (ms_layout / 1e3),
                           "check": ok_layout},
           "sea_index": {"ms": ms_sea, "points_per_s": n / (ms_sea / 1e3), "nsea": nsea},
           "obsoper_rectilinear": {"ms": ms_oper, "obs_per_s": m / (ms_oper / 1e3),
                                   "inside_fraction": inside},
           "permute_rows": {"ms": ms_perm, "columns": 16,
                            "achieved_GBs": perm_bytes / (ms_perm / 1e3) / 1e9,
                            "algorithmic_bytes": perm_bytes},
           "gpu_launches": int(launches),
           "note": "timed through the Python API (device arrays), includes the host "
                   "allocation of the outputs; steps as --steps"}
    del idx, w, zs, zi, inv, sea, ens
    if not args.no_cpu_baseline:
        from oracle import oakref as R
        ps = part[:1_000_000].cpu().numpy()
        t0 = time.perf_counter()
        R.init_partition(ps)
        t_part = time.perf_counter() - t0
        ns = 300
        ph = [p[:ns].cpu().numpy() for p in pos]
        sea_h, _ = R.sea_index(mask.reshape(-1, order="F"))
        t0 = time.perf_counter()
        R.obsoper_rectilinear([x, y, z], ph, sea=sea_h)
        t_oper = time.perf_counter() - t0
        res["cpu_baseline"] = {
            "kind": "port", "cores": 1,
            "zone_layout_elements_per_s": ps.size / t_part,
            "obsoper_obs_per_s": ns / t_oper,
            "sample": f"oracle init_partition on {ps.size} elements, "
                      f"obsoper_rectilinear on {ns} observations (NumPy, one thread)"}
    return res


def rows_cpu_baseline(c, N, zones=128):
    """The oracle (NumPy, one core, a port) beside the rows section: the prologue's mean and
    anomalies of a 10^6 x N ensemble, and the SMWCovar (k = 8) and diagonal-R local analyses on
    a sample of every k-th zone with all observations."""
    import time
    from oracle import oakref as R
    rng = np.random.default_rng(3)
    Eh = np.asfortranarray(rng.normal(size=(1_000_000, N)))
    t0 = time.perf_counter()
    mu = Eh.mean(axis=1)
    _ = (Eh - mu[:, None]) / np.sqrt(N - 1.0)
    t_pro = time.perf_counter() - t0
    del Eh, _
    zsel, rows = cpu_sample(c, zones)
    sel = R.geometric_selector(c.zone_pos[zsel], c.obs_pos, c.corr_len[zsel], c.max_len[zsel],
                               c.metric, c.loctype, c.weight)
    B = np.random.default_rng(4).normal(0.0, 0.05, size=(c.m, 8))
    out = {"kind": "port", "cores": 1, "prologue_rows_per_s": 1_000_000 / t_pro}
    for name, smw in (("loc_analysis", None), ("smw_loc_analysis", B)):
        t0 = time.perf_counter()
        R.loc_analysis(c.zone_size[zsel], sel, c.xf[rows], c.Hxf, c.yo, c.Sf[rows], c.HSf,
                       c.r_diag, smw_B=smw)
        out[name + "_zones_per_s"] = len(zsel) / (time.perf_counter() - t0)
    out["sample"] = (f"NumPy mean and scaled anomalies of a 10^6 x {N} ensemble; the oracle's "
                     f"local analyses (diagonal R and SMWCovar k = 8) on {len(zsel)} of "
                     f"{c.Z} zones with all {c.m} observations, one core")
    return out


def rows_section(torch, dev, stream, args, c, d_args, fp64_ms, T, F):
    import oak_gb300

    def timed(fn, k=None):
        k = k or args.steps
        for _ in range(max(args.warmup, 3)):
            out = fn()
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(k):
            out = fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return out, a.elapsed_time(b) / k

    res = {}
    try:
        zs, xf, Hxf, yo, Sf, HSf, r, zp, op, corr, maxl = d_args
        n, N = int(Sf.shape[0]), int(Sf.shape[1])
        m = int(yo.shape[0])
        kw = dict(weight=c.weight, metric=c.metric, loctype=c.loctype)
        # row 1: the ensemble (xf + sqrt(N-1) Sf) through H Ef, mean and anomalies, the local
        # analysis, inflation and Ea
        Ef = (xf[:, None] + Sf * float(np.sqrt(N - 1.0))).t().contiguous().t()
        Hi = torch.as_tensor(np.asarray(c.obs_index, dtype=np.int64)[:, None], device=dev)
        Hw = torch.ones((m, 1), dtype=torch.float64, device=dev)
        _, ms1 = timed(lambda: oak_gb300.ens_loc_analysis(zs, Ef, Hi, Hw, yo, r, zp, op, corr,
                                                           maxl, inflation=1.02, **kw))
        res["ens_loc_analysis"] = {
            "ms_per_call": ms1, "value": c.Z / (ms1 / 1e3), "unit": "local analyses/s",
            "overhead_vs_loc_analysis_ms": ms1 - fp64_ms,
            "what": "H Ef (K = 1), mean and anomalies, FP64 local analysis, inflation 1.02, "
                    "Ea = xa + sqrt(N-1) Sa, all on the device"}
        _, msp = timed(lambda: oak_gb300.ensemble_prologue(Ef, Hi, Hw))
        pro_bytes = 2 * n * N * 8 + 2 * m * N * 8 + n * 8
        res["ensemble_prologue"] = {"ms": msp, "achieved_GBs": pro_bytes / (msp / 1e3) / 1e9,
                                    "algorithmic_bytes": pro_bytes}
        # row 4: ens2sqrt / sqrt2ens
        (mean, S), ms_e2s = timed(lambda: oak_gb300.ens2sqrt(Ef))
        _, ms_s2e = timed(lambda: oak_gb300.sqrt2ens(mean, S))
        th_rng = np.random.default_rng(77)
        theta = np.linalg.qr(th_rng.standard_normal((N - 1, N - 1)))[0]
        theta_d = torch.as_tensor(np.ascontiguousarray(theta.T), device=dev).t()
        _, ms_s2e_th = timed(lambda: oak_gb300.sqrt2ens(mean, S, theta_d))
        e_bytes = 2 * n * N * 8
        res["ens2sqrt"] = {"ms": ms_e2s, "achieved_GBs": e_bytes / (ms_e2s / 1e3) / 1e9}
        res["sqrt2ens"] = {"ms": ms_s2e, "achieved_GBs": e_bytes / (ms_s2e / 1e3) / 1e9,
                           "theta": "identity (closed form, one read of S and one write of E)"}
        res["sqrt2ens_random_theta"] = {
            "ms": ms_s2e_th, "achieved_GBs": e_bytes / (ms_s2e_th / 1e3) / 1e9,
            "gemm_tflops": 2.0 * n * N * (N - 1) / (ms_s2e_th / 1e3) / 1e12,
            "theta": "random orthogonal (N-1) x (N-1): E = mean + S Om^T by cuBLAS DGEMM over E "
                     "pre-filled with the mean"}
        del Ef, mean, S
        # row 2: R = diag(r) + B B^T with k = 8 columns
        kB = 8
        B = torch.empty((kB, m), dtype=torch.float64, device=dev).normal_(0.0, 0.05).t()
        _, ms2 = timed(lambda: oak_gb300.loc_analysis(*d_args, want_ampl=False, smw_B=B, **kw))
        res["smw_loc_analysis"] = {"ms_per_call": ms2, "value": c.Z / (ms2 / 1e3),
                                   "unit": "local analyses/s", "k": kB,
                                   "cost_vs_diagonal_R": ms2 / fp64_ms}
        del B
        # row 4: biasedLocAnalysis (two local analyses) on the same device inputs, gamma 0.3
        bf = torch.zeros_like(xf)
        _, ms3 = timed(lambda: oak_gb300.biased_loc_analysis(
            0.3, zs, xf, bf, Hxf, yo, Sf, HSf, r, zp, op, corr, maxl, Hi, Hw, want_sa=False,
            **kw), k=2)
        res["biased_loc_analysis"] = {"ms_per_call": ms3, "cost_vs_loc_analysis": ms3 / fp64_ms}
        # row 4: ensAnalysis on the global configuration (100 x 80, N = 30, m = 500)
        from oak_gb300.workloads import global_case
        g = global_case(keep_ensemble=True)
        gE, gH = F(g.Ef), F(g.HEf)
        gy, gr = T(g.yo), T(g.r_diag)
        _, ms4 = timed(lambda: oak_gb300.ens_analysis(gE, gH, gy, gr), k=20)
        res["ens_analysis_global"] = {"ms_per_call": ms4}
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = rows_cpu_baseline(c, N)
        res["gpu_rows_per_s_prologue"] = n / (msp / 1e3)
    except Exception as ex:  # the section is auxiliary: report, keep the bench line
        res["error"] = f"{type(ex).__name__}: {ex}"
    return res


def read_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        parts = ln.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def run_reference(args, ws, rank):
    """The reference algorithm on the host cores (C/OpenMP port of rrsqrt.F90), rank 0 only."""
    if rank != 0:
        return
    from oak_gb300.workloads import local_case
    c = local_case(scale=args.scale)
    threads = os.cpu_count() or 1
    # size each step's sample for a few seconds of CPU work
    zsel, rows = cpu_sample(c, 256)
    per_zone = run_cpu_oracle(c, zsel, rows, threads) / len(zsel)
    budget = 150.0 / max(1, args.steps + args.warmup)
    target = int(min(c.Z, max(256, budget / max(per_zone, 1e-9))))
    zsel, rows = cpu_sample(c, target)
    for _ in range(args.warmup):
        run_cpu_oracle(c, zsel, rows, threads)
    t = 0.0
    for _ in range(args.steps):
        t += run_cpu_oracle(c, zsel, rows, threads)
    v = args.steps * len(zsel) / t
    sample = (f"{len(zsel)} of {c.Z} zones per step (every {c.Z // len(zsel)}-th), all {c.m} "
              f"observations, brute-force selection, LAPACK dsyev via SciPy, OpenMP dynamic")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded, BASELINE shapes)",
        "config": workload_config(c, args.scale),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ctypes helpers (kept local so the module imports without the library)
def ctypes_ptr(x):
    import ctypes
    return ctypes.c_void_p(x)


def ctypes_double():
    import ctypes
    return ctypes.c_double(0.0)


def ctypes_ref(x):
    import ctypes
    return ctypes.byref(x)


if __name__ == "__main__":
    main()
