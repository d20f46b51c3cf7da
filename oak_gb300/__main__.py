"""Command-line runner for the synthetic local-analysis workloads.

  python -m oak_gb300 local [--scale S] [--precision P] [--calls K] [--N N] [--m M]
  python -m oak_gb300 batched [--scale S] [--precision P] [--calls K] [--N N] [--fp32]
  python -m oak_gb300 large [--scale S] [--precision P] [--calls K]
  python -m oak_gb300 layout [--obs M] [--calls K]

P is fp64 (the plain form), mixed or mixed_fp64eig (the mixed form with the FP64-accurate
eigensolve).

``local`` builds the seeded single-variable case (360 x 180 x 20 columns scaled horizontally by
S, N = 64, Gaspari-Cohn radius 12 cells); ``batched`` the 5-variable case (720 x 360 columns of
121 elements scaled by S, N = 100, bilinear observations clustered on tracks); ``large`` the
2-variable case (1440 x 720 columns of 100 elements scaled by S, N = 128, 1M clustered
observations). ``batched --fp32`` and ``large`` generate the case on the GPU with FP32 storage
(oakg_locanalysis_f32), the others on the host in FP64, moved to cuda:0. Then
:func:`oak_gb300.loc_analysis` is called K times, printing the device time of
each stage of the last call. Used to run one precision's kernels in isolation (profiling,
quick timing); the full benchmark is bench.py. ``layout`` runs the layout builders on one
3-D variable of 720 x 360 x 50 points with a land mask and 259,200 column zones: the zone
layout, the sea packing and the rectilinear observation operator for M observations (K
calls each), printing the last call's wall time per builder.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def main(argv=None):
    p = argparse.ArgumentParser(prog="python -m oak_gb300")
    sub = p.add_subparsers(dest="cmd", required=True)
    lp = sub.add_parser("local", help="run the local analysis workload on cuda:0")
    lp.add_argument("--scale", type=float, default=0.5)
    lp.add_argument("--precision", choices=["fp64", "mixed", "mixed_fp64eig"], default="fp64")
    lp.add_argument("--calls", type=int, default=2)
    lp.add_argument("--N", type=int, default=64)
    lp.add_argument("--m", type=int, default=50000,
                    help="observations at scale 1 (the case scales them by S^2)")
    bp = sub.add_parser("batched", help="run the 5-variable batched workload on cuda:0")
    bp.add_argument("--scale", type=float, default=0.25)
    bp.add_argument("--precision", choices=["fp64", "mixed", "mixed_fp64eig"], default="fp64")
    bp.add_argument("--calls", type=int, default=2)
    bp.add_argument("--N", type=int, default=100)
    bp.add_argument("--fp32", action="store_true",
                    help="generate on the GPU with FP32 storage at the boundary")
    gp = sub.add_parser("large", help="run the 2-variable N = 128 workload on cuda:0 (FP32)")
    gp.add_argument("--scale", type=float, default=0.125)
    gp.add_argument("--precision", choices=["fp64", "mixed", "mixed_fp64eig"], default="mixed")
    gp.add_argument("--calls", type=int, default=2)
    yp = sub.add_parser("layout", help="run the layout builders on cuda:0")
    yp.add_argument("--obs", type=int, default=1_000_000)
    yp.add_argument("--calls", type=int, default=2)
    a = p.parse_args(argv)

    import torch
    import oak_gb300
    from oak_gb300.workloads import batched_case, local_case

    if a.cmd == "layout":
        layout(a, torch, oak_gb300)
        return

    dev = torch.device("cuda", 0)
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x), device=dev)
    F = lambda x: torch.as_tensor(np.ascontiguousarray(np.asarray(x).T), device=dev).t()
    if a.cmd == "large" or (a.cmd == "batched" and a.fp32):
        from oak_gb300.workloads import batched_case_device, large_case_device
        c = (large_case_device(scale=a.scale, device=dev) if a.cmd == "large"
             else batched_case_device(scale=a.scale, device=dev, N=a.N))
        args = (T(c.zone_size), c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag, T(c.zone_pos),
                tuple(T(x) for x in c.obs_pos), T(c.corr_len), T(c.max_len))
    else:
        if a.cmd == "local":
            c = local_case(scale=a.scale, N=a.N, m=a.m)
        else:
            c = batched_case(scale=a.scale, N=a.N)
        args = (T(c.zone_size), T(c.xf), T(c.Hxf), T(c.yo), F(c.Sf), F(c.HSf), T(c.r_diag),
                T(c.zone_pos), tuple(T(x) for x in c.obs_pos), T(c.corr_len), T(c.max_len))
    prec = {"fp64": oak_gb300.PREC_FP64, "mixed": oak_gb300.PREC_MIXED,
            "mixed_fp64eig": oak_gb300.PREC_MIXED_FP64EIG}[a.precision]
    for _ in range(a.calls):
        oak_gb300.loc_analysis(*args, weight=c.weight, metric=c.metric, loctype=c.loctype,
                               want_ampl=False, precision=prec)
    torch.cuda.synchronize(dev)
    print(json.dumps({"workload": c.name, "zones": int(c.Z), "N": int(c.N), "m": int(c.m),
                      "precision": a.precision, "calls": a.calls,
                      "stage_ms_last_call": oak_gb300.last_timings()}))


def layout(a, torch, oak_gb300):
    import time
    dev = torch.device("cuda", 0)
    nx, ny, nz = 720, 360, 50
    rng = np.random.default_rng(12)
    part = (torch.arange(nx * ny * nz, device=dev) % (nx * ny) + 1).to(torch.int32)
    mask = np.zeros((nx, ny, nz), dtype=bool)
    mask[100:200, 50:120, :] = True
    mask_d = torch.as_tensor(mask.reshape(-1, order="F"), device=dev)
    z = np.cumsum(rng.uniform(1.0, 50.0, nz))
    axes = [torch.as_tensor(v, device=dev) for v in
            (np.linspace(-180.0, 179.5, nx), np.linspace(-89.75, 89.75, ny), z)]
    pos = [torch.as_tensor(rng.uniform(lo, hi, a.obs), device=dev)
           for lo, hi in ((-180.0, 179.5), (-89.75, 89.75), (z[0], z[-1]))]
    ms = {}
    for name, fn in (("zone_layout", lambda: oak_gb300.zone_layout(part, nx * ny)),
                     ("sea_index", lambda: oak_gb300.sea_index(mask_d)),
                     ("obsoper_rectilinear",
                      lambda: oak_gb300.obsoper_rectilinear(axes, pos,
                                                            sea=oak_gb300.sea_index(mask_d)[0]))):
        for _ in range(a.calls):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize(dev)
            ms[name] = (time.perf_counter() - t0) * 1e3
    print(json.dumps({"grid": [nx, ny, nz], "zones": nx * ny, "obs": a.obs, "calls": a.calls,
                      "wall_ms_last_call": ms}))


if __name__ == "__main__":
    main()
