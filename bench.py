"""Benchmark of the GB300 mLW step: zone-updates/s on the 2-D Orszag-Tang
vortex, 512 x 512 cells, 2.5-D MHD (mlw_m3, 9 FP64 arrays), periodic box.

One benchmark step = `--mlw-steps` (default 100) iterations of the reference
time loop (cfl -> t += dt -> mlw_m3 -> bnd) kept on the device and replayed
as a CUDA graph.  L2 is flushed (256 MiB write) between benchmark steps; the
state itself (2 x 19 MB) fits in L2 and stays there across the iterations of
one step, as it does in a production run of this size.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU restatement of the reference Fortran (the
oracle, with every host thread) on the same workload.  Under torchrun every
rank runs an independent replica ("replicas only": the mLW path has no
exchange on one GPU per run); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "mLW MHD zone-updates/s"
UNIT = "zone-updates/s"
N_CELLS = 512
B_PER_ZONE = 144  # mlw_m3: 9 arrays read once and written once, 8 B each
# floating-point operations of one reference mlw_m3 step and cfl_m3 per
# interior zone of the 512^2 vortex (adds, multiplies, divides, square
# roots: 791.8 + 19.2), from the oracle's counting build (oracle/opcount.cpp,
# held exact in tests/test_oracle.py); the counts do not depend on the data
REF_FLOPS_PER_ZONE = 811.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--mlw-steps", type=int, default=100)
    p.add_argument("--n", type=int, default=N_CELLS)
    p.add_argument("--exact", action="store_true", help="exact arithmetic policy")
    p.add_argument("--df64", action="store_true",
                   help="double-float policy of the 2-D mlw_m3 step (FP32 pipes, FP64 "
                        "accumulation)")
    p.add_argument("--tile", type=int, default=-1,
                   help="2-D tile configuration (default: autotuned); also the tile of the "
                        "mlw2d profile case")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the secondary 3-D and 1-D workloads")
    p.add_argument("--adjoint-export", default=None, metavar="PATH",
                   help="run the adjoint configuration once and write its initial state, "
                        "dt sequence, J and gradient to PATH (.npz) for the long-double "
                        "finite-difference check (oracle/adjoint_fd_longdouble.py), and exit")
    p.add_argument("--parity-full", action="store_true",
                   help="only the 3-D parity legs at 256^3 x 200 steps for mLW, Roe-MUSCL "
                        "and HLLD, both policies, against the oracle; prints one JSON line")
    p.add_argument("--profile-case", default=None,
                   choices=["mlw3d", "roe3d", "hlld3d", "adjoint2d", "batch", "roe2d",
                            "gravity2d", "resistive2d", "gravity3d", "resistive3d",
                            "spicule", "spicule_group", "single", "mlw2d", "mlw2d_df",
                            "mlw3d_df"],
                   help="run one small fixed case of a secondary path (for ncu) and exit")
    return p.parse_args()


def profile_case(case, n, tile=-1, df64=False):
    """A small fixed case of one secondary path: a few device iterations of
    the 3-D steps on an n^3 box, 20 reverse steps of the 2-D adjoint on n^2,
    or 5 batched iterations of 8 shear layers; prints one JSON line."""
    import torch
    from utrip_gb300 import capi, drivers, setups
    if case in ("roe2d", "gravity2d", "resistive2d"):
        s = {"roe2d": lambda: setups.orszag_tang(n, solver="roe_m3"),
             "gravity2d": lambda: setups.mhd_gravity_wave(n, solver="mlw_m3"),
             "resistive2d": lambda: setups.magnetic_reconnection(n)}[case]()
        run = drivers.make_run(s)
        run.push(s["state"])
        run.start(nstop=3, safety=s["safety"], dtmin=1e-10)
        run.advance(3)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "steps": int(st.nexec), "merr": int(st.merr)}
    elif case == "spicule":
        s = setups.spicule_1d(n)
        run = drivers.make_run(s, df64=df64)
        run.push(s["state"])
        run.start(nstop=200, tend=s["tend"], safety=s["safety"], dtmin=s["dtmin"])
        run.advance(200)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "steps": int(st.nexec), "merr": int(st.merr)}
    elif case == "spicule_group":
        # the spicule beta sweep's group launch: n runs of 1024 cells (beta
        # log-uniform in [0.1, 10]), 100 loop iterations each
        rng = np.random.default_rng(11)
        runs = []
        for k, b in enumerate(10.0 ** rng.uniform(-1.0, 1.0, size=n)):
            s = setups.spicule_1d(1024, beta=float(b), seed=k)
            run = drivers.make_run(s, df64=df64)
            run.push(s["state"])
            run.start(tend=s["tend"], nstop=s["nstop"], safety=s["safety"], dtmin=s["dtmin"])
            runs.append(run)
        capi.Run.advance_group(runs, 100)
        done = [int(r.query().nexec) for r in runs]
        for r in runs:
            r.close()
        out = {"case": case, "runs": n, "steps": min(done), "df64": df64}
    elif case in ("gravity3d", "resistive3d"):
        s = (setups.emerging_flux_3d(n, max(2, n // 4), n) if case == "gravity3d"
             else setups.magnetic_reconnection_3d(n, max(4, n // 4)))
        run = drivers.make_run(s)
        run.push(s["state"])
        run.start(nstop=3, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(3)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "steps": int(st.nexec), "merr": int(st.merr)}
    elif case == "single":
        # the one-at-a-time baseline of the beta sweep: 5 plain-launch
        # iterations of a 128^2 and then of a 384^2 shear layer
        out = {"case": case}
        for m in (128, 384):
            s = setups.shear_layer(m, beta=1.0, seed=4)
            run = drivers.make_run(s)
            run.set_graph(False)
            run.push(s["state"])
            run.start(nstop=5, safety=0.4, dtmin=1e-10)
            run.advance(5)
            out[str(m)] = int(run.query().nexec)
            run.close()
    elif case == "mlw2d":
        # the FP64 fast-policy step of the vortex on n^2: 4 iterations with the
        # given tile, or with the autotuner's pick
        s = setups.orszag_tang(n)
        run = drivers.make_run(s, tile=tile)
        run.push(s["state"])
        if tile < 0:
            tile = run.autotune(2)
            run.push(s["state"])
        run.start(nstop=4, safety=s["safety"], dtmin=1e-10)
        run.advance(4)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "tile": tile, "steps": int(st.nexec), "merr": int(st.merr)}
    elif case in ("mlw2d_df", "mlw3d_df"):
        # the double-float steps: 4 iterations of the vortex (n^2, y-marching
        # tile) or of the turbulence box (n^3)
        s = setups.orszag_tang(n) if case == "mlw2d_df" else setups.turbulence_3d(n)
        run = drivers.make_run(s, df64=True, tile=4 if case == "mlw2d_df" else 0)
        run.push(s["state"])
        run.start(nstop=4, safety=s["safety"], dtmin=1e-10)
        run.advance(4)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "steps": int(st.nexec), "merr": int(st.merr)}
    elif case in ("mlw3d", "roe3d", "hlld3d"):
        solver = {"mlw3d": "mlw_m_3d", "roe3d": "roe_m_3d", "hlld3d": "hlld_3d"}[case]
        s = setups.turbulence_3d(n, solver=solver)
        run = drivers.make_run(s, df64=df64)
        run.push(s["state"])
        run.start(nstop=3, safety=0.2, dtmin=1e-10)
        run.advance(3)
        st = run.query()
        run.close()
        out = {"case": case, "n": n, "steps": int(st.nexec), "merr": int(st.merr),
               "df64": df64}
    elif case == "adjoint2d":
        s = setups.shear_layer(n, beta=1.0, seed=4)
        run = drivers.make_run(s)
        run.push(s["state"])
        dts, J = run.record_dts(20)
        J2, _, nf = run.adjoint(dts, nsnap=4)
        run.close()
        out = {"case": case, "n": n, "steps": 20, "J": J, "J_equal": J == J2, "nfwd": nf}
    else:
        runs = [setups.shear_layer(m, beta=b, seed=k) for k, (m, b) in
                enumerate(zip([n, n // 2, n, n // 2] * 2, [0.2, 0.5, 1.0, 2.0] * 2))]
        b = capi.Batch(runs)
        for g, r in enumerate(runs):
            b.push(g, r["state"])
        b.start(nstop=5, safety=0.4, dtmin=1e-10)
        b.advance(5)
        out = {"case": case, "n": n, "runs": len(runs), "done": bool(b.query(0).done)}
        b.close()
    torch.cuda.synchronize()
    print(json.dumps(out))


def extra_workloads(stream, exact=False):
    """Secondary measurements reported beside the headline: the 3-D beta=1
    turbulence box (256^3 interior, 8 arrays, 128 B/zone) and the 1-D MHD
    shock tube run to t = 0.1 as one cluster launch."""
    import torch
    from utrip_gb300 import capi, drivers, setups
    out = {}
    hbm_peak, _ = measured_peaks()
    # ---- 3-D: 20 loop iterations timed with events, step kernel profiled
    s3 = setups.turbulence_3d(256)
    run = drivers.make_run(s3, exact=exact, stream=stream.cuda_stream)
    run.push(s3["state"])
    tile = run.autotune(2)
    run.start(tend=1e30, nstop=10 ** 12, safety=s3["safety"], dtmin=s3["dtmin"])
    run.advance(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = 20
    e0.record(stream)
    run.advance(iters)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    step_ms, iter_ms = run.profile(10)
    st = run.query()
    zones = 256 ** 3
    kstep = step_ms / 10
    out["turbulence_256^3_mlw_m"] = {
        "zone_updates_per_s": zones * iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
        "step_kernel_ms": kstep, "tile": tile, "hbm_gbs": 128 * zones / (kstep * 1e-3) / 1e9,
        "hbm_frac": 128 * zones / (kstep * 1e-3) / 1e9 / hbm_peak, "bytes_per_zone": 128,
        "steps_done": int(st.nexec), "merr": int(st.merr)}
    run.close()
    # the same box in the double-float policy
    run = drivers.make_run(s3, stream=stream.cuda_stream, df64=True)
    run.push(s3["state"])
    tile = run.autotune(2)
    run.push(s3["state"])
    run.start(tend=1e30, nstop=10 ** 12, safety=s3["safety"], dtmin=s3["dtmin"])
    run.advance(3)
    torch.cuda.synchronize()
    e0.record(stream)
    run.advance(iters)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    step_ms, _ = run.profile(10)
    st = run.query()
    kstep = step_ms / 10
    out["turbulence_256^3_mlw_m_df64"] = {
        "zone_updates_per_s": zones * iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
        "step_kernel_ms": kstep, "tile": tile, "hbm_gbs": 128 * zones / (kstep * 1e-3) / 1e9,
        "hbm_frac": 128 * zones / (kstep * 1e-3) / 1e9 / hbm_peak, "bytes_per_zone": 128,
        "steps_done": int(st.nexec), "merr": int(st.merr), "policy": "df64",
        "parity": "parity_vs_oracle.turbulence_256^3_mlw_m_3d_200_steps.df64_rel_linf"}
    run.close()
    del s3
    # ---- 1-D: the whole shock-tube run to t = 0.1 in one cluster launch
    s1 = setups.shock_tube_1d(1024)
    run = drivers.make_run(s1, exact=exact, stream=stream.cuda_stream)
    best = None
    for _ in range(3):
        run.push(s1["state"])
        torch.cuda.synchronize()
        e0.record(stream)
        run.start(tend=s1["tend"], nstop=10 ** 6, safety=s1["safety"], dtmin=s1["dtmin"])
        run.advance(10 ** 6)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    st = run.query()
    got = run.pull()
    import oracle
    ref = setups.copy_state(s1)
    t_ref, ns_ref, _, _ = oracle.run_1d(s1, ref, 10 ** 6)
    out["shock_tube_1024_to_t0.1_mlw_m_1d"] = {
        "ms_to_tend": best, "steps": int(st.ns), "t": st.t, "merr": int(st.merr),
        "us_per_step": best * 1e3 / max(1, st.ns),
        "zone_updates_per_s": 1024 * st.ns / (best * 1e-3), "launches_per_run": 2,
        "oracle_steps": int(ns_ref),
        "rel_linf_vs_oracle": {k: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
                               for k, a, b in zip(s1["names"], got, ref)}}
    run.close()
    # ---- 3-D Roe-MUSCL and HLLD steps on the same turbulence box (margin 3)
    for solver, safety in (("roe_m_3d", None), ("hlld_3d", 0.2)):
        out[f"turbulence_256^3_{solver}"] = riemann_3d(stream, solver, safety, exact)
        if not exact:  # the face flux in double-float
            out[f"turbulence_256^3_{solver}_df64"] = riemann_3d(stream, solver, safety, False,
                                                                df64=True)
    out["orszag_tang_512^2_roe_m3"] = roe_2d(stream, exact)
    if not exact:
        out["orszag_tang_512^2_roe_m3_df64"] = roe_2d(stream, False, df64=True)
    out["mhd_gravity_wave_512^2_mlw_m3_g"] = loop_2d(
        stream, exact, lambda m: setups.mhd_gravity_wave(m, solver="mlw_m3"), 512, 100, 256, 500,
        "gravity-wave model")
    out["emerging_flux_256x64x256_mlw_m_g"] = loop_3d(
        stream, exact, setups.emerging_flux_3d, (256, 64, 256), 20, (96, 32, 96), 100,
        "emerging-flux model")
    out["reconnection_512^2_mlw_m_e"] = loop_2d(
        stream, exact, setups.magnetic_reconnection, 512, 100, 256, 500, "reconnection model")
    out["reconnection_256x256x64_mlw_m_e"] = loop_3d(
        stream, exact, lambda nx, ny, nz: setups.magnetic_reconnection_3d(nx, nz),
        (256, 256, 64), 20, (96, 96, 16), 50, "3-D reconnection model")
    out["hlld_brio_wu_1024_to_t0.1"] = hlld_brio_wu(stream, exact)
    out["spicule_1024_100000_steps_mlw_m_bg"] = spicule_workload(stream)
    out["spicule_beta_sweep_64x1024_2000_steps"] = spicule_beta_sweep(stream)
    # a group too small to cover the SMs takes clusters of 8 SMs a run
    out["spicule_beta_sweep_8x1024_2000_steps"] = spicule_beta_sweep(stream, nruns=8,
                                                                      cpu_steps=0)
    out["literal_drop_in_orszag_tang_512^2"] = literal_drop_in(stream)
    out["beta_sweep_64x2d_1000_steps"] = beta_sweep(stream, exact)
    out["adjoint_shear_256^2_2000_steps"] = adjoint_workload(stream)
    return out


def riemann_3d(stream, solver, safety, exact, iters=10, df64=False):
    """Two-stage Riemann-solver step on the 3-D beta = 1 box, 256^3 interior
    cells + 3 ghost layers: loop iterations timed with events (graph), the
    four step kernels profiled.  HLLD runs in Heaviside units; its reference
    driver pairs that state with the CANS-unit cfl_m, which at safety 0.4 is
    beyond the three-axis stability limit, so it runs at safety 0.2.  df64
    evaluates the face flux in double-float (the oracle sample is then left
    to the FP64 leg)."""
    import torch
    from utrip_gb300 import drivers, setups
    s = setups.turbulence_3d(256, solver=solver)
    if safety is not None:
        s["safety"] = safety
    run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream, df64=df64)
    run.push(s["state"])
    run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
    run.advance(2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run.advance(iters)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    step_ms, _ = run.profile(4)
    st = run.query()
    run.close()
    zones = 256 ** 3
    out = {"zone_updates_per_s": zones * iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
           "step_kernels_ms": step_ms / 4, "safety": s["safety"],
           "bound": "fp32 pipes (double-float flux)" if df64 else "fp64",
           "steps_done": int(st.nexec), "merr": int(st.merr),
           "policy": "df64" if df64 else ("exact" if exact else "fast")}
    if not df64:
        out["cpu_oracle"] = cpu_sample_3d(solver, safety)
    return out


def roe_2d(stream, exact, n=512, iters=50, cpu_n=256, cpu_steps=300, df64=False):
    """The 2-D Roe-MUSCL step (roe_m3, margin 2) on the Orszag-Tang vortex of
    the headline, loop iterations timed with events (graph), the four step
    kernels profiled; the oracle on a bounded sample (cpu_n^2, all host
    threads) beside it."""
    from utrip_gb300 import setups
    return loop_2d(stream, exact, lambda m: setups.orszag_tang(m, solver="roe_m3"), n, iters,
                   cpu_n, cpu_steps, "vortex", df64=df64)


def loop_2d(stream, exact, make, n, iters, cpu_n, cpu_steps, what, df64=False):
    """A 2-D model loop on the device (graph-replayed iterations timed with
    events, step kernels profiled) and the oracle on a bounded sample of the
    same model (cpu_n^2, all host threads; left to the FP64 leg when df64
    selects the double-float policy)."""
    import torch
    import oracle
    from utrip_gb300 import drivers, setups
    s = make(n)
    run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream, df64=df64)
    run.push(s["state"])
    run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
    run.advance(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run.advance(iters)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    step_ms, _ = run.profile(10)
    st = run.query()
    run.close()
    if df64:
        return {"zone_updates_per_s": n * n * iters / (ms * 1e-3),
                "ms_per_iteration": ms / iters, "step_kernels_ms": step_ms / 10,
                "bound": "fp32 pipes (double-float flux)", "steps_done": int(st.nexec),
                "merr": int(st.merr), "policy": "df64"}
    c = make(cpu_n)
    cs = setups.copy_state(c)
    t0 = time.perf_counter()
    oracle.run_2d(c, cs, cpu_steps)
    el = time.perf_counter() - t0
    return {"zone_updates_per_s": n * n * iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
            "step_kernels_ms": step_ms / 10, "bound": "fp64", "steps_done": int(st.nexec),
            "merr": int(st.merr), "policy": "exact" if exact else "fast",
            "cpu_oracle": {"zone_updates_per_s": cpu_n * cpu_n * cpu_steps / el,
                           "cores": oracle.get_threads(), "kind": "port",
                           "sample": f"{cpu_steps} loop iterations of the {cpu_n}^2 {what} "
                                     f"in {el:.2f} s"}}


def loop_3d(stream, exact, make, shape, iters, cpu_shape, cpu_steps, what):
    """A 3-D model loop on the device (graph-replayed iterations timed with
    events, step kernels profiled) and the oracle on a bounded sample of the
    same model (all host threads)."""
    import torch
    import oracle
    from utrip_gb300 import drivers, setups
    s = make(*shape)
    run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream)
    run.push(s["state"])
    tile = run.autotune(2)
    run.push(s["state"])
    run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
    run.advance(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run.advance(iters)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    step_ms, _ = run.profile(5)
    st = run.query()
    run.close()
    zones = int(np.prod(shape))
    c = make(*cpu_shape)
    cs = setups.copy_state(c)
    t0 = time.perf_counter()
    oracle.run_3d(c, cs, cpu_steps)
    el = time.perf_counter() - t0
    return {"zone_updates_per_s": zones * iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
            "step_kernels_ms": step_ms / 5, "tile": tile, "bound": "fp64",
            "steps_done": int(st.nexec), "merr": int(st.merr),
            "policy": "exact" if exact else "fast",
            "cpu_oracle": {"zone_updates_per_s": int(np.prod(cpu_shape)) * cpu_steps / el,
                           "cores": oracle.get_threads(), "kind": "port",
                           "sample": f"{cpu_steps} loop iterations of the "
                                     f"{'x'.join(map(str, cpu_shape))} {what} in {el:.2f} s"}}


def cpu_sample_3d(solver, safety, n=96, steps=2):
    """The CPU restatement of the reference step (the oracle, OpenMP over
    every host thread) on a bounded sample of the same workload: the 96^3
    turbulence box, one untimed step, then `steps` timed loop iterations."""
    import oracle
    from utrip_gb300 import setups
    s = setups.turbulence_3d(n, solver=solver)
    st = setups.copy_state(s)
    sf = safety if safety is not None else s["safety"]
    dt, _ = oracle.cfl_3d(s, st, sf)
    oracle.step_3d(s, st, dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        dt, _ = oracle.cfl_3d(s, st, sf)
        oracle.step_3d(s, st, dt)
        oracle.apply_bc_program_3d(st, s["bc"], s["margin"], s)
    el = time.perf_counter() - t0
    return {"zone_updates_per_s": n ** 3 * steps / el, "cores": oracle.get_threads(),
            "kind": "port", "sample": f"{steps} loop iterations of the {n}^3 box in {el:.2f} s"}


def hlld_brio_wu(stream, exact):
    """The HLLD shock tube of md_mhdshktb/hdhlld-x (1024 cells, x only) run to
    t = 0.1 on the device, graph-replayed."""
    import torch
    from utrip_gb300 import drivers, setups
    s = setups.shock_tube_hlld_1d(1024)
    run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for _ in range(3):
        run.push(s["state"])
        torch.cuda.synchronize()
        e0.record(stream)
        run.start(tend=s["tend"], nstop=10 ** 6, safety=s["safety"], dtmin=s["dtmin"])
        while not run.query().done:
            run.advance(256)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    st = run.query()
    run.close()
    return {"ms_to_tend": best, "steps": int(st.ns), "t": st.t, "merr": int(st.merr),
            "us_per_step": best * 1e3 / max(1, st.ns)}


def spicule_workload(stream, nstop=100000, cpu_steps=4000):
    """The reference's spicule run (cans1d/md_spicule/hdmlw: 1024 cells,
    100000 iterations of cfl_m, mlw_m_bg, the random torque, bnd and chkdav)
    as one cluster launch, in the fast, exact and double-float policies,
    against the output the reference ships for this run
    (tests/golden/spicule_reference.npz: the time reached and the ro, pr, vx
    profiles; vy and by follow the random torque, whose stream differs) and
    against the oracle's loop timed on a bounded sample of the same run on
    one host core."""
    import torch
    from utrip_gb300 import drivers, setups
    import oracle
    s = setups.spicule_1d()
    gold = dict(np.load(ROOT / "tests" / "golden" / "spicule_reference.npz"))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {}
    for policy, exact, df64 in (("fast", False, False), ("exact", True, False),
                                ("df64", False, True)):
        run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream, df64=df64)
        run.push(s["state"])
        torch.cuda.synchronize()
        e0.record(stream)
        run.start(tend=s["tend"], nstop=nstop, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(nstop)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st = run.query()
        got = run.pull()
        run.close()
        t_ref = float(gold["t_records"][1])
        l2 = {name: float(np.linalg.norm(got[k] - gold[f"{name}_records"][1]) /
                          np.linalg.norm(gold[f"{name}_records"][1]))
              for k, name in enumerate(s["names"]) if name in ("ro", "pr", "vx")}
        res[policy] = {"ms": ms, "us_per_step": ms * 1e3 / max(1, st.ns), "steps": int(st.ns),
                       "t": st.t, "merr": int(st.merr), "chkdav_events": int(st.n_floor),
                       "zone_updates_per_s": 1024 * st.ns / (ms * 1e-3),
                       "t_rel_diff_vs_reference_output": abs(st.t - t_ref) / t_ref,
                       "rel_l2_vs_reference_output": l2}
    ref = setups.copy_state(s)
    t0 = time.perf_counter()
    oracle.run_spicule_c(s, ref, cpu_steps)
    cpu_s = time.perf_counter() - t0
    res["cpu_oracle"] = {"us_per_step": cpu_s * 1e6 / cpu_steps, "cores": 1,
                         "sample": f"first {cpu_steps} iterations of the same run"}
    res["speedup_vs_cpu_oracle"] = res["cpu_oracle"]["us_per_step"] / res["fast"]["us_per_step"]
    return res


def spicule_beta_sweep(stream, nruns=64, steps=2000, cpu_steps=1000, seed=11):
    """The reference's parameter studies on their own model: nruns spicule
    runs (cans1d/md_spicule/hdmlw, 1024 cells, torque and floor on) with the
    plasma beta at the base (model.f's onebeta) log-uniform in [0.1, 10] and
    their own torque seeds, `steps` loop iterations each, advanced in one
    launch (cans_run_advance_group: one cluster per run) against the same
    runs one at a time (each run's loop as its own cluster launch, as
    cans_run_advance gives it), the same group in the double-float policy,
    and the oracle's loop timed on one host core (the reference runs each
    model as one serial process; cpu_steps = 0 leaves that leg out)."""
    import torch
    from utrip_gb300 import capi, drivers, setups
    import oracle
    rng = np.random.default_rng(seed)
    betas = 10.0 ** rng.uniform(-1.0, 1.0, size=nruns)
    sets = [setups.spicule_1d(1024, beta=float(b), seed=k) for k, b in enumerate(betas)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def started(s, df64=False):
        run = drivers.make_run(s, stream=stream.cuda_stream, df64=df64)
        run.push(s["state"])
        run.start(tend=s["tend"], nstop=s["nstop"], safety=s["safety"], dtmin=s["dtmin"])
        return run

    def group(df64):
        runs = [started(s, df64) for s in sets]
        torch.cuda.synchronize()
        e0.record(stream)
        capi.Run.advance_group(runs, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        states = [r.query() for r in runs]
        final = [runs[k].pull() for k in (0, nruns - 1)]
        for r in runs:
            r.close()
        return ms, states, final

    group_ms, states, group_final = group(False)
    # the same runs in the double-float policy (the step on the FP32 pipes)
    df_ms, df_states, df_final = group(True)
    alone_ms, alone_final = 0.0, []
    for k, s in enumerate(sets):
        run = started(s)
        torch.cuda.synchronize()
        e0.record(stream)
        run.advance(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        alone_ms += e0.elapsed_time(e1)
        if k in (0, nruns - 1):
            alone_final.append(run.pull())
        run.close()
    def rel(f1, f2):  # per variable, the larger over the first and last run
        return {name: max(float(np.max(np.abs(a[v] - b[v]))) /
                          max(float(np.max(np.abs(b[v]))), 1e-300)
                          for a, b in zip(f1, f2))
                for v, name in enumerate(sets[0]["names"])}

    # the fast policy: the group kernel may fuse multiply-adds differently
    # (vx of this model amplifies one rounding of the energy up to ~1e-5)
    diff = rel(group_final, alone_final)
    run_steps = nruns * steps
    res = {
        "runs": nruns, "cells": 1024, "steps_per_run": steps,
        "beta_range": [float(betas.min()), float(betas.max())],
        "all_runs_completed": all(st.nexec == steps and st.merr == 0 for st in states),
        "group_ms": group_ms, "one_at_a_time_ms": alone_ms,
        "speedup_group_vs_one_at_a_time": alone_ms / group_ms,
        "group_run_steps_per_s": run_steps / (group_ms * 1e-3),
        "group_us_per_run_step_each_run": group_ms * 1e3 / steps,
        "group_zone_updates_per_s": 1024 * run_steps / (group_ms * 1e-3),
        "first_and_last_run_rel_linf_vs_alone": diff,
        "df64_policy": {
            "group_ms": df_ms,
            "all_runs_completed": all(st.nexec == steps and st.merr == 0 for st in df_states),
            "speedup_vs_fp64_group": group_ms / df_ms,
            "speedup_vs_fp64_one_at_a_time": alone_ms / df_ms,
            "group_zone_updates_per_s": 1024 * run_steps / (df_ms * 1e-3),
            "first_and_last_run_rel_linf_vs_fp64_group": rel(df_final, group_final),
        },
    }
    if cpu_steps > 0:
        ref = setups.copy_state(sets[0])
        t0 = time.perf_counter()
        oracle.run_spicule_c(sets[0], ref, cpu_steps)
        cpu_us = (time.perf_counter() - t0) * 1e6 / cpu_steps
        res["cpu_oracle"] = {"us_per_step": cpu_us, "cores": 1,
                             "sample": f"first {cpu_steps} iterations of the first run"}
        res["speedup_group_vs_one_cpu_core"] = cpu_us * run_steps / (group_ms * 1e3)
    return res


def adjoint_workload(stream, nsteps=2000, nsnap=32, ndir=16, n_oracle_dirs=2, h=1e-6,
                     h_smooth=2e-5):
    """The differentiation pattern on the 2-D shear layer at beta = 1 (256^2,
    mlw_m3, 2000 steps, J = final magnetic energy): the reverse sweep with
    binomial checkpointing in 32 stored states timed against the forward run
    of the same frozen dt sequence, and its directional derivatives on 16
    seeded directions of the initial vy field, and dJ/dbeta, checked against
    FP64 central differences.

    Two properties of J set the terms of the check.  (1) Its rounding noise:
    J of the fast and of the exact policy differ by about 1e-14 of J (the
    unstable shear layer amplifies rounding over 2000 steps), so a central
    difference at h = 1e-6 carries an error near 1e-14 J / h, a few 1e-6 of
    the smaller directional derivatives.  The h = 1e-6 difference is
    reported; the 1e-6 criterion is taken on the fourth-order difference
    from h_smooth and 2 h_smooth, where J (qav = 0) is smooth and the noise
    is 20 times smaller.  (2) The artificial viscosity q = qav dxm
    max(0, |dv| - 1e-4) is piecewise affine in dv and the shear layer has
    velocity jumps at 1e-4 everywhere: at qav = 3 every direction crosses
    about a million face switches within +-h (counted).  The adjoint is the
    derivative of the branches the base run took; the check holding every
    face at its recorded branch (cans_run_objective_frozen_av) is smooth but
    leaves negative viscosity on faces pushed past their switch, which makes
    it strongly non-linear (it diverges beyond about 1e-5).  So qav = 3 is
    reported, not held to 1e-6; qav = 0 carries the 1e-6 check, with two
    directions also against the CPU oracle's forward."""
    import torch
    import oracle
    from utrip_gb300 import drivers, setups

    def base(beta, qav):
        s = setups.shear_layer(256, beta=beta, seed=4)
        s["qav"] = qav
        oracle.apply_bc_program(s["state"], s["bc"], s["margin"], s)
        return s

    def shifted(s, z, step):
        return [np.asfortranarray(a + step * b) for a, b in zip(s["state"], z)]

    def smooth_direction(rng, n, kmax=8):
        """A seeded random field of unit RMS made of the Fourier modes
        |k| <= kmax of the periodic box (the perturbation's own scale)."""
        k = np.fft.fftfreq(n, d=1.0 / n)
        kr = np.fft.rfftfreq(n, d=1.0 / n)
        KX, KY = np.meshgrid(k, kr, indexing="ij")
        mask = (KX ** 2 + KY ** 2) <= kmax ** 2
        mask[0, 0] = False
        spec = np.zeros(mask.shape, dtype=np.complex128)
        spec[mask] = rng.standard_normal(int(mask.sum())) + 1j * rng.standard_normal(int(mask.sum()))
        f = np.fft.irfft2(spec, s=(n, n))
        return f / np.sqrt(np.mean(f ** 2))

    def extend(s, d):
        z = [np.zeros_like(a) for a in s["state"]]
        z[3][1:-1, 1:-1] = d
        oracle.apply_bc_program(z, s["bc"], s["margin"], s)
        return z

    def fd24(J, hh):
        """second-order differences at hh and 2 hh, and the fourth-order one."""
        d1 = (J[1] - J[-1]) / (2 * hh)
        d2 = (J[2] - J[-2]) / (4 * hh)
        return d1, d2, (4.0 * d1 - d2) / 3.0

    def oracle_J(s, st, dts):
        st = [np.asfortranarray(a) for a in st]
        for dt in dts:
            oracle.step_2d(s, st, dt)
            oracle.apply_bc_program(st, s["bc"], s["margin"], s)
        w = np.outer(s["dx"], s["dy"])[1:-1, 1:-1]
        e = (st[5] ** 2 + st[6] ** 2 + st[7] ** 2)[1:-1, 1:-1]
        return float(np.sum(e * w)) / np.pi / 8.0

    out = {"nsteps": nsteps, "nsnap": nsnap, "h": h, "h_smooth": h_smooth,
           "directions": "seeded unit-RMS fields of the |k| <= 8 Fourier modes of vy",
           "criterion": "|adjoint - fd4(h_smooth)| <= 1e-6 |fd4| at qav = 0"}
    for qav in (3.0, 0.0):
        s = base(1.0, qav)
        run = drivers.make_run(s, stream=stream.cuda_stream)
        run.push(s["state"])
        dts, J = run.record_dts(nsteps)
        run.objective(dts)  # warm-up
        if qav == 3.0:
            run.adjoint(dts, nsnap=nsnap)  # warm-up (builds the checkpoint schedule)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J_fwd = run.objective(dts)
        fwd_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        J_adj, grad, nfwd = run.adjoint(dts, nsnap=nsnap)
        adj_s = time.perf_counter() - t0
        if qav == 3.0:  # the same reverse sweep with every state stored
            run.adjoint(dts, nsnap=nsteps + 1)
            t0 = time.perf_counter()
            _, g_all, nfwd_all = run.adjoint(dts, nsnap=nsteps + 1)
            out["store_all_states"] = {
                "adjoint_s": time.perf_counter() - t0, "forward_steps_in_adjoint": int(nfwd_all),
                "grad_equal_to_checkpointed": all(np.array_equal(a, b)
                                                  for a, b in zip(g_all, grad))}
            # the same sweep with its reverse arithmetic in FP64
            run.set_adjoint_df64(False)
            run.adjoint(dts, nsnap=nsnap)
            t0 = time.perf_counter()
            _, g64, _ = run.adjoint(dts, nsnap=nsnap)
            out["reverse_in_fp64"] = {
                "adjoint_s": time.perf_counter() - t0,
                "grad_max_rel_diff_vs_double_float": max(
                    float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)
                    for a, b in zip(grad, g64))}
            run.set_adjoint_df64(True)
        rx = drivers.make_run(s, exact=True, stream=stream.cuda_stream)
        rx.push(s["state"])
        J_exact = rx.objective(dts)
        rx.close()
        if qav == 3.0:
            run.av_record(dts)
            J_held0, flips0 = run.objective_frozen_av(dts)
        rng = np.random.default_rng(5)
        dirs, n_pass, n_pass_1e6 = [], 0, 0
        for k in range(ndir):
            d = smooth_direction(rng, 256)
            z = extend(s, d)
            ad = sum(float(np.sum(g * e)) for g, e in zip(grad, z))
            Jh = {}
            for m in (1, -1):
                run.push(shifted(s, z, m * h))
                Jh[m] = run.objective(dts)
            fd_h = (Jh[1] - Jh[-1]) / (2 * h)
            row = {"adjoint": ad, "fd2_h_rel_err": abs(ad - fd_h) / abs(fd_h),
                   "fd2_h_noise_floor_rel": abs(J - J_exact) / h / abs(ad)}
            n_pass_1e6 += abs(ad - fd_h) <= 1e-6 * abs(fd_h)
            if qav == 3.0:
                Jf, fl = {}, {}
                for m in (1, -1, 2, -2):
                    run.push(shifted(s, z, m * h))
                    Jf[m], fl[m] = run.objective_frozen_av(dts)
                f1, _, f4 = fd24(Jf, h)
                row.update({"held_fd2_h_rel_err": abs(ad - f1) / abs(f4),
                            "held_fd4_h_rel_err": abs(ad - f4) / abs(f4),
                            "switches_crossed_plus_h": int(fl[1]),
                            "switches_crossed_minus_h": int(fl[-1])})
            else:
                Js = {}
                for m in (1, -1, 2, -2):
                    run.push(shifted(s, z, m * h_smooth))
                    Js[m] = run.objective(dts)
                _, _, f4 = fd24(Js, h_smooth)
                row["fd4_smooth_rel_err"] = abs(ad - f4) / abs(f4)
                n_pass += abs(ad - f4) <= 1e-6 * abs(f4)
                if k < n_oracle_dirs:
                    Jo = {m: oracle_J(s, shifted(s, z, m * h_smooth), dts) for m in (1, -1, 2, -2)}
                    _, _, o4 = fd24(Jo, h_smooth)
                    row["oracle_fd4_smooth_rel_err"] = abs(ad - o4) / abs(o4)
            dirs.append(row)
        # dJ/dbeta: p = 0.625 beta in every cell
        dbeta = 0.625 * float(np.sum(grad[1]))
        hb = h_smooth if qav == 0.0 else h
        Jb = {}
        for m in (1, -1, 2, -2):
            run.push(base(1.0 + m * hb, qav)["state"])
            Jb[m] = run.objective_frozen_av(dts)[0] if qav == 3.0 else run.objective(dts)
        b1, _, b4 = fd24(Jb, hb)
        run.push(base(1.0 + h, qav)["state"])
        jbp = run.objective(dts)
        run.push(base(1.0 - h, qav)["state"])
        jbm = run.objective(dts)
        run.close()
        leg = {"J": J, "J_replay_equal": J_fwd == J and J_adj == J,
               "J_rel_diff_fast_vs_exact_policy": abs(J - J_exact) / abs(J),
               "forward_s": fwd_s, "adjoint_s": adj_s, "adjoint_over_forward": adj_s / fwd_s,
               "forward_steps_in_adjoint": int(nfwd),
               "fd2_h_within_1e-6": f"{n_pass_1e6}/{ndir}",
               "fd2_h_rel_err_median": float(np.median([r["fd2_h_rel_err"] for r in dirs])),
               "dJ_dbeta": dbeta,
               "dJ_dbeta_fd2_h_rel_err": abs(dbeta - (jbp - jbm) / (2 * h)) /
               abs((jbp - jbm) / (2 * h)),
               "directions": dirs}
        if qav == 0.0:
            e4 = [r["fd4_smooth_rel_err"] for r in dirs]
            leg.update({"fd4_smooth_within_1e-6": f"{n_pass}/{ndir}",
                        "fd4_smooth_rel_err_max": max(e4),
                        "fd4_smooth_rel_err_median": float(np.median(e4)),
                        "dJ_dbeta_fd4_smooth_rel_err": abs(dbeta - b4) / abs(b4)})
        else:
            e4 = [r["held_fd4_h_rel_err"] for r in dirs]
            leg.update({"J_held_equal": J_held0 == J and flips0 == 0,
                        "held_fd4_h_rel_err_median": float(np.median(e4)),
                        "held_fd4_h_rel_err_max": max(e4),
                        "switches_crossed_per_direction": [
                            r["switches_crossed_plus_h"] + r["switches_crossed_minus_h"]
                            for r in dirs],
                        "dJ_dbeta_held_fd4_h_rel_err": abs(dbeta - b4) / abs(b4)})
        out[f"qav{qav:g}"] = leg
    if "store_all_states" in out:
        out["store_all_states"]["adjoint_over_forward"] = (out["store_all_states"]["adjoint_s"]
                                                           / out["qav3"]["forward_s"])
        out["reverse_in_fp64"]["adjoint_over_forward"] = (out["reverse_in_fp64"]["adjoint_s"]
                                                          / out["qav3"]["forward_s"])
    out["reverse_arithmetic"] = ("double-float on the FP32 pipes (cans_run_set_adjoint_df64); "
                                 "forward recomputation in FP64")
    return out


def adjoint_export(path, n=256, nsteps=2000, nsnap=32, qav=3.0, beta=1.0, seed=4,
                   exact=False):
    """The adjoint configuration (shear layer, beta = 1, qav = 3, 2000
    steps, 32 stored states) run once on the GPU; writes what the
    long-double finite-difference check needs: the initial state (its
    transcendental set-up values as this host computed them), the frozen dt
    sequence, J and the gradient dJ/dP_0 of every variable."""
    import oracle
    from utrip_gb300 import drivers, setups
    s = setups.shear_layer(n, beta=beta, seed=seed)
    s["qav"] = qav
    oracle.apply_bc_program(s["state"], s["bc"], s["margin"], s)
    run = drivers.make_run(s, exact=exact)
    try:
        run.push(s["state"])
        dts, J = run.record_dts(nsteps)
        J_adj, grad, nfwd = run.adjoint(dts, nsnap=nsnap)
        run.set_adjoint_df64(False)  # the same sweep with its reverse arithmetic in FP64
        _, grad64, _ = run.adjoint(dts, nsnap=nsnap)
        run.set_adjoint_df64(True)
        # the same sweep about the exact policy's forward run of the same dts
        rx = drivers.make_run(s, exact=True)
        try:
            rx.push(s["state"])
            J_ex, grad_ex, _ = rx.adjoint(dts, nsnap=nsnap)
        finally:
            rx.close()
        # the viscosity branches of the run the adjoint linearises, as bit
        # planes (bit 0: active, bit 1: dv < 0) of every step
        run.av_record(dts)
        br = [run.av_branches(k) for k in range(nsteps)]
        active = np.packbits(np.stack([b & 1 for b in br]).astype(bool), axis=1)
        negative = np.packbits(np.stack([(b >> 1) & 1 for b in br]).astype(bool), axis=1)
        J_held, flips = run.objective_frozen_av(dts)
    finally:
        run.close()
    np.savez_compressed(path, n=n, beta=beta, seed=seed, qav=qav, nsnap=nsnap, exact=exact,
                        state=np.stack([np.asarray(a) for a in s["state"]]),
                        dts=np.asarray(dts), J=J, J_adjoint_replay=J_adj, J_held=J_held,
                        forward_steps=int(nfwd), grad=np.stack([np.asarray(g) for g in grad]),
                        grad_fp64_reverse=np.stack([np.asarray(g) for g in grad64]),
                        J_exact_policy=J_ex,
                        grad_exact_policy=np.stack([np.asarray(g) for g in grad_ex]),
                        av_active=active, av_negative=negative)
    print(json.dumps({"adjoint_export": str(path), "J": J, "steps": nsteps,
                      "forward_steps_in_adjoint": int(nfwd)}))


def literal_drop_in(stream, n=512, steps=(10, 100)):
    """The reference driver's own call pattern (cans2d/md_mhdkh/hdmlw/main.f:
    169,179,182): per step cfl_m3 -> t += dt -> mlw_m3 -> bnd (one bd* call
    per variable and axis), each a drop-in C-ABI call on the caller's host
    arrays.  Unregistered, every call copies its arrays to the device and
    back; registered (cans_gpu_register), the same calls run on device
    mirrors and only dt crosses to the host.  Orszag-Tang n^2, wall time of
    the host loop (it synchronises every call)."""
    import torch
    from utrip_gb300 import drivers, setups
    s = setups.orszag_tang(n)
    arr = (n + 2) * (n + 2) * 8
    nvar = len(s["names"])
    nbd = sum(1 for v, f, k, q in s["bc"] if f % 2 == 0)  # bdper* fills both faces
    out = {"workload": f"orszag_tang_{n}x{n}_mlw_m3", "host_arrays": "pageable (numpy)"}
    for mode, nsteps in (("unregistered", steps[0]), ("registered", steps[1])):
        st = setups.copy_state(s)
        drivers.run_literal(s, st, 2, resident=mode == "registered")  # warm-up
        st = setups.copy_state(s)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        drivers.run_literal(s, st, nsteps, resident=mode == "registered")
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if mode == "unregistered":
            h2d = (8 + nvar + nbd) * arr  # cfl_m3 (8 arrays), mlw_m3, each bd call
            d2h = (nvar + nbd) * arr + 8
        else:  # registration pushes and the final pull happen once per loop
            h2d = nvar * arr / nsteps
            d2h = nvar * arr / nsteps + 8
        out[mode] = {"steps": nsteps, "ms_per_step": el * 1e3 / nsteps,
                     "zone_updates_per_s": n * n * nsteps / el,
                     "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                     "calls_per_step": 2 + nbd}
    return out


def sweep_setups(nruns=64, seed=4):
    """64 magnetised shear layers, sizes drawn from {128,192,256,384}^2 and
    plasma beta log-uniform in [0.1, 10] (seeded)."""
    from utrip_gb300 import setups
    rng = np.random.default_rng(seed)
    sizes = rng.choice([128, 192, 256, 384], size=nruns)
    betas = 10.0 ** rng.uniform(-1.0, 1.0, size=nruns)
    return [setups.shear_layer(int(n), beta=float(b), seed=seed + k)
            for k, (n, b) in enumerate(zip(sizes, betas))], sizes, betas


def beta_sweep(stream, exact=False, nsteps=1000):
    """The batched sweep (one persistent step launch per iteration for all 64
    runs, graph-replayed, autotuned) against the same 64 runs done one at a
    time with plain launches (one launch per stage) and with graphs."""
    import torch
    from utrip_gb300 import capi, drivers
    runs, sizes, betas = sweep_setups()
    zones = float(sum(int(n) * int(n) for n in sizes)) * nsteps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b = capi.Batch(runs, exact=exact, stream=stream.cuda_stream)
    for g, s in enumerate(runs):
        b.push(g, s["state"])
    b.start(nstop=nsteps, safety=0.4, dtmin=1e-10)
    cfg = b.autotune(2)
    torch.cuda.synchronize()
    e0.record(stream)
    b.advance(nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1)
    done = all(b.query(g).nexec == nsteps for g in range(len(runs)))
    batch_final = [b.pull(g) for g in (0, len(runs) - 1)]
    b.close()
    single, by_size = {}, {}
    for mode in ("plain", "graph"):
        total = 0.0
        finals = []
        for g, s in enumerate(runs):
            run = drivers.make_run(s, exact=exact, stream=stream.cuda_stream)
            run.set_graph(mode == "graph")
            run.push(s["state"])
            run.start(nstop=nsteps, safety=0.4, dtmin=1e-10)
            torch.cuda.synchronize()
            e0.record(stream)
            run.advance(nsteps)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            total += ms
            if mode == "plain":
                d = by_size.setdefault(str(int(sizes[g])), {"runs": 0, "ms": 0.0})
                d["runs"] += 1
                d["ms"] += ms
            if g in (0, len(runs) - 1):
                finals.append(run.pull())
            run.close()
        single[mode] = total
        diff = max(float(np.max(np.abs(x - y))) / max(float(np.max(np.abs(y))), 1e-300)
                   for f1, f2 in zip(finals, batch_final) for x, y in zip(f1, f2))
    for k, d in by_size.items():
        d["zone_updates_per_s"] = int(k) ** 2 * nsteps * d["runs"] / (d["ms"] * 1e-3)
    # A batch can at best run every zone-update at the rate of a step kernel
    # that fills the GPU (it is FP64-bound there): the best of the batched
    # rate and the largest grids' one-at-a-time rate.
    best_rate = max([zones / (batched_ms * 1e-3)] +
                    [d["zone_updates_per_s"] for d in by_size.values()])
    ideal_ms = zones / best_rate * 1e3
    return {"runs": len(runs), "steps_per_run": nsteps, "config": cfg,
            "one_at_a_time_plain_by_size": by_size,
            "fp64_bound_ideal_ms": ideal_ms,
            "max_speedup_vs_plain_if_fp64_bound": single["plain"] / ideal_ms,
            "sizes": {str(k): int(np.sum(sizes == k)) for k in (128, 192, 256, 384)},
            "beta_range": [float(betas.min()), float(betas.max())],
            "batched_ms": batched_ms, "one_at_a_time_plain_ms": single["plain"],
            "one_at_a_time_graph_ms": single["graph"],
            "speedup_vs_plain": single["plain"] / batched_ms,
            "speedup_vs_graph": single["graph"] / batched_ms,
            "batched_zone_updates_per_s": zones / (batched_ms * 1e-3),
            "all_runs_completed": bool(done),
            "max_rel_diff_batched_vs_single": diff}


def _rel_linf(names, got, ref):
    """Relative L-infinity per variable (to the field's largest value; absolute
    for a field that is zero everywhere)."""
    return {k: float(np.max(np.abs(a - b)) / (np.max(np.abs(b)) or 1.0))
            for k, a, b in zip(names, got, ref)}


def _totals(s, st):
    """Interior totals of mass, momentum, total energy and B of a 2-D or 3-D
    state (magnetic energy B^2/8pi in CANS units; B^2/2mu for the HLLD state,
    which is in Heaviside units)."""
    ro, pr, vx, vy, vz, bx, by, bz = st[:8]
    three = ro.ndim == 3
    if three:
        w = (s["dx"][:, None, None] * s["dy"][None, :, None] * s["dz"][None, None, :])
        m = s["margin"]
        inner = (slice(m, -m),) * 3
    else:
        w = np.outer(s["dx"], s["dy"])
        m = s["margin"]
        inner = (slice(m, -m),) * 2
    w = w[inner]
    bfac = 1.0 / (2.0 * s["mu"]) if s["solver"] == "hlld_3d" else 1.0 / (8 * np.pi)
    ee = pr / (s["gm"] - 1) + 0.5 * ro * (vx ** 2 + vy ** 2 + vz ** 2) + \
        (bx ** 2 + by ** 2 + bz ** 2) * bfac
    q = {"mass": ro, "energy": ee, "momentum_x": ro * vx, "momentum_y": ro * vy,
         "momentum_z": ro * vz, "bx": bx, "by": by, "bz": bz}
    return {k: float(np.sum(a[inner] * w)) for k, a in q.items()}


def _drift(t0, t1):
    return {k: (t1[k] - t0[k]) / abs(t0[k]) if abs(t0[k]) > 1e-12 else t1[k] - t0[k]
            for k in t0}


def parity_check(n, stream, nsteps=100, c3_n=256, c3_steps=200, c3_riemann_steps=20):
    """The benchmark configurations checked against the CPU oracle from the
    same initial states.

    2-D Orszag-Tang n^2 (the headline): 100 loop iterations, and the whole
    run to t = pi/2; relative L-infinity per variable of the fast policy, the
    number of cells that differ in the exact policy, and the drift of the
    conserved totals (mass, momentum, total energy, B) in the periodic box.
    3-D beta = 1 turbulence c3_n^3: the mLW loop for c3_steps iterations
    (both policies), the Roe-MUSCL and HLLD loops for c3_riemann_steps
    (fast policy), each with the drift of its totals.  The shock tube of
    md_shktb with B = 0 in 1-D, 2-D and 3-D against the exact solution of
    its shktb_analytic.pro: L1 distances and their order under refinement."""
    import oracle
    from oracle import shktb_analytic as an
    from utrip_gb300 import drivers, setups
    out = {}
    s = setups.orszag_tang(n)
    for label, nstop in (("orszag_tang_100_steps", nsteps),
                         ("orszag_tang_to_t_pi_over_2", 10 ** 6)):
        ref = setups.copy_state(s)
        t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, nstop)
        leg = {"steps": int(ns_ref), "t": t_ref}
        for policy in ("fast", "exact", "df64"):
            got = setups.copy_state(s)
            run = drivers.make_run(s, exact=policy == "exact", stream=stream.cuda_stream,
                                   df64=policy == "df64")
            t, ns, merr, _ = drivers.run_resident(s, got, nstop, run=run)
            run.close()
            if policy == "exact":
                leg["exact_cells_differing"] = int(sum(int(np.sum(a != b))
                                                       for a, b in zip(got, ref)))
                leg["exact_same_t_and_steps"] = bool(t == t_ref and ns == ns_ref)
            else:
                leg[f"{policy}_rel_linf"] = _rel_linf(s["names"], got, ref)
                leg[f"{policy}_steps"] = int(ns)
                leg[f"conservation_drift_{policy}"] = _drift(_totals(s, s["state"]),
                                                             _totals(s, got))
        leg["conservation_drift_oracle"] = _drift(_totals(s, s["state"]), _totals(s, ref))
        out[label] = leg
    out["conservation_note"] = ("relative change of the interior totals over the run; "
                                "absolute change where the total is zero")
    del s
    for solver, steps in (("mlw_m_3d", c3_steps), ("roe_m_3d", c3_riemann_steps),
                          ("hlld_3d", c3_riemann_steps)):
        leg = parity_3d(stream, solver, c3_n, steps, True)
        if solver != "mlw_m_3d":
            leg["oracle_one_ulp_input_noise_rel_linf"] = one_ulp_conditioning(solver, 64, steps)
            leg["note"] = ("the mean field lies along x, so the x faces sit at the c_f = c_a "
                           "degeneracy, where the reference algorithm amplifies rounding: "
                           "one ulp of input noise in the oracle alone grows to the "
                           "oracle_one_ulp_input_noise figure (64^3, same steps); the exact "
                           "policy reproduces the reference's rounding bit for bit")
        out[f"turbulence_{c3_n}^3_{solver}_{steps}_steps"] = leg
    out["sod_shock_tube_exact_solution"] = parity_sod(stream, an)
    return out


def parity_3d(stream, solver, n, steps, exact_too):
    """One 3-D loop of the beta = 1 turbulence box against the oracle: fast
    and double-float policy relative L-infinity and conservation drift
    (device and oracle), and with exact_too the cells that differ in the
    exact policy.  HLLD runs at safety 0.2 (see riemann_3d)."""
    import oracle
    from utrip_gb300 import drivers, setups
    s = setups.turbulence_3d(n, solver=solver)
    if solver == "hlld_3d":
        s["safety"] = 0.2
    ref = setups.copy_state(s)
    t0 = time.perf_counter()
    t_ref, ns_ref, _, _ = oracle.run_3d(s, ref, steps)
    leg = {"steps": int(ns_ref), "oracle_s": time.perf_counter() - t0,
           "oracle_cores": oracle.get_threads()}
    tot0 = _totals(s, s["state"])
    policies = ["fast"] + (["exact"] if exact_too else []) + ["df64"]
    for policy in policies:
        got = setups.copy_state(s)
        t, ns, merr, _ = drivers.run_resident(s, got, steps, exact=policy == "exact",
                                              df64=policy == "df64")
        if policy == "exact":
            leg["exact_cells_differing"] = int(sum(int(np.sum(a != b)) for a, b in zip(got, ref)))
        else:
            leg[f"{policy}_rel_linf"] = _rel_linf(s["names"], got, ref)
            leg[f"conservation_drift_{policy}"] = _drift(tot0, _totals(s, got))
        del got
    leg["conservation_drift_oracle"] = _drift(tot0, _totals(s, ref))
    return leg


def one_ulp_conditioning(solver, n, steps):
    """Relative L-infinity per variable between two oracle runs of the n^3
    beta = 1 box whose initial velocities differ by at most one ulp."""
    import oracle
    from utrip_gb300 import setups
    s = setups.turbulence_3d(n, solver=solver)
    if solver == "hlld_3d":
        s["safety"] = 0.2
    a, b = setups.copy_state(s), setups.copy_state(s)
    rng = np.random.default_rng(1)
    for k in (2, 3, 4):
        b[k] = np.asfortranarray(b[k] * (1.0 + np.finfo(np.float64).eps *
                                         rng.choice([-1.0, 0.0, 1.0], size=b[k].shape)))
    oracle.apply_bc_program_3d(b, s["bc"], s["margin"], s)
    oracle.run_3d(s, a, steps)
    oracle.run_3d(s, b, steps)
    return _rel_linf(s["names"], b, a)


def parity_sod(stream, an, ns=(256, 512, 1024, 2048)):
    """The md_shktb shock tube with B = 0 on the device (fast policy) to
    tend = 0.14154: L1 distance of rho, p, vx from the exact solution and the
    observed order, for the mLW step in 1-D (mlw_m), 2-D (mlw_m3) and 3-D
    (mlw_m), and for the Riemann-solver steps (1-D roe_m through its
    drop-in calls, 2-D roe_m3, 3-D roe_m, the HLLD engine along x)."""
    from utrip_gb300 import drivers, setups
    out = {}
    cases = [(f"{d}d", lambda n, d=d: setups.sod_shock_tube(n, d)) for d in (1, 2, 3)]
    cases += [(sv, lambda n, sv=sv: setups.sod_shock_tube_riemann(n, sv))
              for sv in ("roe_m_1d", "roe_m3", "roe_m_3d", "hlld_3d")]
    for name, make in cases:
        errs = []
        for n in ns:
            s = make(n)
            got = setups.copy_state(s)
            if s["solver"] == "roe_m_1d":
                t, nsteps, merr, _ = drivers.run_literal(s, got, 10 ** 6, resident=True)
            else:
                t, nsteps, merr, _ = drivers.run_resident(s, got, 10 ** 6)
            x, dx, ro, pr, vx = setups.sod_interior_profile(s, got)
            sd = s["sod"]
            errs.append(an.l1_errors(x, dx, ro, pr, vx, t, sd["x0"], sd["gm"], sd["ro1"],
                                     sd["pr1"]))
        out[name] = {"cells": list(ns), "l1": {k: [e[k] for e in errs] for k in errs[0]},
                     "order": {k: an.observed_order(ns, [e[k] for e in errs])
                               for k in errs[0]}}
    return out


def parity_full(n=256, steps=200):
    """The 3-D configuration at its stated size and length: 256^3 interior
    cells, 200 loop iterations of mLW, Roe-MUSCL and HLLD, each in both
    policies against the oracle (all host threads); about a quarter of an
    hour of CPU time for the oracle."""
    import torch
    import oracle
    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    out = {"parity_full": f"turbulence_{n}^3_{steps}_steps"}
    for solver in ("mlw_m_3d", "roe_m_3d", "hlld_3d"):
        out[solver] = parity_3d(stream, solver, n, steps, True)
        print(json.dumps({solver: out[solver]}), flush=True)
    print(json.dumps(out), flush=True)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("CANS_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        try:
            lines = Path(self.f.name).read_text().strip().splitlines()
        except OSError:
            lines = []
        rows = [[c.strip() for c in ln.split(",")] for ln in lines if ln.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        loaded = [v for v in sm if smax and v >= 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def probe_peaks():
    """FP64 and FP32 FMA throughput of the device in TFLOP/s, measured now by
    the benchmark's probe library (utrip_gb300/_lib/libcansprobe.so)."""
    import ctypes
    lib = ctypes.CDLL(str(ROOT / "utrip_gb300" / "_lib" / "libcansprobe.so"))
    out = []
    for name in ("cans_probe_fp64_tflops", "cans_probe_fp32_tflops"):
        x = ctypes.c_double(0.0)
        if getattr(lib, name)(ctypes.byref(x)) != 0:
            raise RuntimeError(f"{name} failed")
        out.append(x.value)
    return out[0], out[1]


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_summary():
    """Per-launch DRAM bytes and FP64 operation counts of the step kernel from
    the committed ncu summary (profiles/), if present."""
    out = {}
    p = ROOT / "profiles" / "ncu_mlw2d_step_ot512.txt"
    if p.exists():
        for ln in p.read_text().splitlines():
            if ":" in ln and ln.split(":", 1)[0].strip() in (
                    "dram_bytes_per_launch", "fp64_flops_per_zone"):
                k, v = ln.split(":", 1)
                try:
                    out[k.strip()] = float(v.split()[0])
                except (ValueError, IndexError):
                    pass
    return out


def cpu_baseline(n, seconds_target=15.0):
    """The oracle (C restatement of the reference) on the host cores."""
    import oracle
    from utrip_gb300 import setups
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    s = setups.orszag_tang(n)
    st = setups.copy_state(s)
    oracle.run_2d(s, st, 1)  # warm the arena
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds_target or steps < 2:
        oracle.run_2d(s, st, 1)
        steps += 1
    el = time.perf_counter() - t0
    zones = n * n * steps
    # the reference itself is serial per process: the same loop on one core
    oracle.set_threads(1)
    try:
        steps1, t1 = 0, time.perf_counter()
        while time.perf_counter() - t1 < seconds_target / 3 or steps1 < 2:
            oracle.run_2d(s, st, 1)
            steps1 += 1
        el1 = time.perf_counter() - t1
    finally:
        oracle.set_threads(threads)
    return {"value": zones / el, "unit": UNIT, "cores": oracle.get_threads(), "kind": "port",
            "sample": f"{steps} loop iterations (cfl_m3+mlw_m3+bnd) of Orszag-Tang {n}x{n} "
                      f"in {el:.1f} s",
            "one_core": {"value": n * n * steps1 / el1, "unit": UNIT, "cores": 1,
                         "sample": f"{steps1} loop iterations in {el1:.1f} s"}}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    import oracle
    from utrip_gb300 import setups
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = args.n
    s = setups.orszag_tang(n)
    st = setups.copy_state(s)
    t0 = time.perf_counter()
    oracle.run_2d(s, st, 1)
    per_iter = time.perf_counter() - t0
    iters = max(1, int(3.0 / max(per_iter, 1e-6)))  # about 3 s per benchmark step
    for _ in range(args.warmup):
        oracle.run_2d(s, st, iters)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.run_2d(s, st, iters)
    el = time.perf_counter() - t0
    value = n * n * iters * args.steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"orszag_tang_{n}x{n}_mlw_m3", "solver": "mlw_m3",
                       "mlw_steps_per_bench_step": iters, "parallelism": "openmp"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.get_threads(),
                             "kind": "port",
                             "sample": f"{args.steps} x {iters} loop iterations of "
                                       f"Orszag-Tang {n}x{n}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def policy_line(n, steps, warmup, m, stream, df64, hbm_peak, fp32_peak):
    """The headline workload in one arithmetic policy, measured as the main
    line is: autotuned tile, graph-replayed iterations timed with events on
    the run's stream with the L2 flushed between benchmark steps, the step
    kernel timed alone, and the same through the public API with host
    buffers copied in and out every benchmark step."""
    import torch
    from utrip_gb300 import capi, drivers, setups
    s = setups.orszag_tang(n)
    run = drivers.make_run(s, stream=stream.cuda_stream, df64=df64)
    run.push(setups.copy_state(s))
    tile = run.autotune(5)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
    for _ in range(warmup):
        flush.fill_(1.0)
        run.advance(m)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    c0 = capi.launch_count()
    for k in range(steps):
        flush.fill_(1.0)
        ev[k][0].record(stream)
        run.advance(m)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    launches = capi.launch_count() - c0
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    st = run.query()
    step_ms, iter_ms = run.profile(200)
    step_avg = step_ms / 200
    host = [torch.empty((n + 2, n + 2), dtype=torch.float64, pin_memory=True).numpy().T
            for _ in range(run.nvar)]
    for h, a in zip(host, s["state"]):
        h[...] = a
    e2e_steps = max(3, steps // 2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        run.push(host)
        run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(m)
        run.pull(host)
    e1.record(stream)
    torch.cuda.synchronize()
    nbytes = run.nvar * (n + 2) * (n + 2) * 8
    run.close()
    achieved = B_PER_ZONE * n * n / (step_avg * 1e-3) / 1e9
    return {"value": n * n * m * steps / (dev_ms * 1e-3), "unit": UNIT,
            "ms_per_step": dev_ms / steps, "tile": tile, "gpu_launches": int(launches),
            "steps_done": int(st.nexec), "merr": int(st.merr),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "bytes_per_zone": B_PER_ZONE,
                         "step_kernel_ms": step_avg, "iteration_ms": iter_ms / 200},
            "e2e": {"value": n * n * m * e2e_steps / (e0.elapsed_time(e1) * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "fp32_peak_tflops_measured": fp32_peak}


def run_ours(args, ws, rank, local):
    import torch
    from utrip_gb300 import capi, drivers, setups
    torch.cuda.set_device(local)
    capi.load()
    if not capi.device_ok():
        raise SystemExit("no usable sm_103 device")
    n = args.n
    s = setups.orszag_tang(n)
    # a dedicated (non-null) stream: the run launches on it and the events,
    # the L2 flush and the copies are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    run = drivers.make_run(s, exact=args.exact, stream=stream.cuda_stream, tile=args.tile,
                           df64=args.df64)
    run.push(setups.copy_state(s))
    tile = run.autotune(5) if args.tile < 0 else args.tile
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    m = args.mlw_steps
    total_iters = (args.warmup + args.steps) * m
    run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
    for _ in range(args.warmup):
        flush.fill_(1.0)
        run.advance(m)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    c0 = capi.launch_count()
    with Clocks(local) as clk:
        w0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(1.0)
            ev[k][0].record(stream)
            run.advance(m)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    barrier(ws)
    launches = capi.launch_count() - c0
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    st = run.query()
    assert st.nexec == total_iters and st.merr == 0, (st.nexec, total_iters, st.merr)
    dev_ms = max_over_ranks(dev_ms, ws)
    zones = n * n * m * args.steps
    value = zones * ws / (dev_ms * 1e-3)

    # dominant kernel: the fused step, timed alone inside un-graphed iterations
    prof_iters = 200
    step_ms, iter_ms = run.profile(prof_iters)
    step_avg = step_ms / prof_iters
    hbm_peak, peak_kind = measured_peaks()
    achieved = B_PER_ZONE * n * n / (step_avg * 1e-3) / 1e9
    ncu = ncu_summary()
    traffic = ncu.get("dram_bytes_per_launch")
    fp64_peak, fp32_peak = probe_peaks()
    flops_zone = ncu.get("fp64_flops_per_zone")
    fp64 = None
    if flops_zone:
        ach = flops_zone * n * n / (step_avg * 1e-3) / 1e12
        fp64 = {"achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                "flops_per_zone": flops_zone, "peak_kind": "measured live (FP64 FMA chains)"}
        # the reference algorithm's own arithmetic per zone-update (mlw_m3 and
        # cfl_m3 at 512^2), counted by oracle/opcount.cpp: the rate at which
        # the loop delivers it, step and bookkeeping included
        ref_ach = REF_FLOPS_PER_ZONE * value / 1e12
        fp64.update({"reference_algorithm_flops_per_zone": REF_FLOPS_PER_ZONE,
                     "reference_algorithm_tflops_delivered": ref_ach,
                     "reference_algorithm_frac_of_peak": ref_ach / fp64_peak})

    # end to end through the public API with pinned host buffers
    host = [torch.empty((n + 2, n + 2), dtype=torch.float64, pin_memory=True).numpy().T
            for _ in range(run.nvar)]
    for h, a in zip(host, s["state"]):
        h[...] = a
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        run.push(host)
        run.start(tend=1e30, nstop=10 ** 12, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(m)
        run.pull(host)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), ws)
    e2e_val = n * n * m * e2e_steps * ws / (e2e_ms * 1e-3)
    nbytes = run.nvar * (n + 2) * (n + 2) * 8
    run.close()
    df64_line = None
    if not args.exact and not args.df64:
        hbm_peak0, _ = measured_peaks()
        df64_line = policy_line(n, args.steps, args.warmup, m, stream, True, hbm_peak0,
                                fp32_peak)
        df64_line["policy"] = ("double-float: the step's arithmetic as pairs of floats on the "
                               "FP32 pipes, density and field accumulated in FP64 "
                               "(cans_run_set_df64); its parity against the oracle is "
                               "parity_vs_oracle.orszag_tang_*.df64_rel_linf")
    parity = parity_check(n, stream) if rank == 0 and not args.no_extras else None
    extras = None if args.no_extras else extra_workloads(stream, exact=args.exact)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"orszag_tang_{n}x{n}_mlw_m3", "solver": "mlw_m3",
                   "grid": [n + 2, n + 2], "mlw_steps_per_bench_step": m,
                   "policy": "exact" if args.exact else ("df64" if args.df64 else "fast"),
                   "tile": tile,
                   "l2": "flushed between benchmark steps (256 MiB write)",
                   "parallelism": "replicas" if ws > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "peak_kind": peak_kind, "bytes_per_zone": B_PER_ZONE,
                     "step_kernel_ms": step_avg, "iteration_ms": iter_ms / prof_iters},
        "roofline_fp64": fp64,
        "fp64_peak_tflops_measured": fp64_peak,
        "fp32_peak_tflops_measured": fp32_peak,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": int(launches),
        "wall_s": wall,
        "clocks": clk.summary(),
    }
    if df64_line is not None:
        line["df64_policy"] = df64_line
    if parity is not None:
        line["parity_vs_oracle"] = parity
    if extras is not None:
        line["workloads"] = extras
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(n)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case, args.n, args.tile, args.df64)
        return
    if args.parity_full:
        parity_full()
        return
    if args.adjoint_export:
        adjoint_export(args.adjoint_export, exact=args.exact)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
