"""Finite-difference check of the adjoint in long double -- TEST
INFRASTRUCTURE ONLY (x86-64: long double is the 64-bit-significand x87
format there; on other hosts it may be a slow software type).

The adjoint configuration (256^2 shear layer at beta = 1, qav = 3, 2000
mlw_m3 steps of a frozen dt sequence, J the final magnetic energy) is
checked against central differences of the forward run.  Two properties of
that run defeat an FP64 difference at h = 1e-6: the artificial viscosity
q = qav dxm max(0, |dv| - 1e-4) switches on about a million faces within
+-h of the base point, and the run amplifies rounding so that J carries a
noise of about 1e-14 of itself.  Here the forward run is the oracle's
restatement in long double (mlw2d_ld.c), with every viscosity face held at
the branch it took on the base trajectory (the derivative the adjoint
computes is that of the branches taken), so the difference measures the
derivative to far below 1e-6.

Input: the .npz written on the GPU by `bench.py --adjoint-export PATH`
(initial state, dt sequence, J and the adjoint gradient of the GPU run).
The 16 directions are the benchmark's: seeded unit-RMS fields of the
|k| <= 8 Fourier modes of vy (rng seed 5).  Output: one JSON document with,
per direction, the adjoint's directional derivative, the second- and
fourth-order differences and their relative distance, and the same for
dJ/dbeta.

    python oracle/adjoint_fd_longdouble.py export.npz [--h 1e-7] [--dirs 16]
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from utrip_gb300 import setups  # noqa: E402

LD = np.longdouble


def smooth_direction(rng, n, kmax=8):
    """A seeded random field of unit RMS made of the Fourier modes
    |k| <= kmax of the periodic box (the benchmark's directions)."""
    k = np.fft.fftfreq(n, d=1.0 / n)
    kr = np.fft.rfftfreq(n, d=1.0 / n)
    KX, KY = np.meshgrid(k, kr, indexing="ij")
    mask = (KX ** 2 + KY ** 2) <= kmax ** 2
    mask[0, 0] = False
    spec = np.zeros(mask.shape, dtype=np.complex128)
    spec[mask] = rng.standard_normal(int(mask.sum())) + 1j * rng.standard_normal(int(mask.sum()))
    f = np.fft.irfft2(spec, s=(n, n))
    return f / np.sqrt(np.mean(f ** 2))


def apply_bc_ld(state, program, margin):
    """The shear layer's boundary program (periodic x, bdsppy in y; margin
    1) on long-double arrays: the copies of bdperx.f and bdsppy.f."""
    assert margin == 1
    for axis in (0, 1):
        for var, face, kind, _ in program:
            if face // 2 != axis:
                continue
            q = state[var]
            if kind == oracle.BD_PER and axis == 0:
                if face % 2 == 0:
                    q[0, :] = q[-2, :]
                else:
                    q[-1, :] = q[1, :]
            elif kind == oracle.BD_SPP and axis == 1:
                if face % 2 == 0:
                    q[:, 0] = q[:, 1]
                else:
                    q[:, -1] = q[:, -2]
            else:
                raise ValueError(f"boundary kind {kind} on axis {axis} is not the shear layer's")


def objective_ld(s, state0, dts, rec, mode, grid):
    """J of the long-double run from state0 with the frozen dt sequence:
    mode 1 records every step's viscosity branches into rec[step], mode 2
    holds them."""
    st = [np.asfortranarray(a, dtype=LD) for a in state0]
    try:
        for k, dt in enumerate(dts):
            oracle.set_av_branch(mode, rec[k], long_double=True)
            oracle.mlw_m3_ld(*st, dt, s["qav"], s["gm"], grid["dx"], grid["dxm"], grid["dy"],
                             grid["dym"])
            apply_bc_ld(st, s["bc"], s["margin"])
    finally:
        oracle.set_av_branch(0, long_double=True)
    w = np.outer(grid["dx"], grid["dy"])[1:-1, 1:-1]
    e = (st[5] ** 2 + st[6] ** 2 + st[7] ** 2)[1:-1, 1:-1]
    return np.sum(e * w) / np.arccos(LD(-1.0)) / LD(8.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("export")
    ap.add_argument("--h", type=float, default=1e-7)
    ap.add_argument("--dirs", type=int, default=16)
    args = ap.parse_args()
    z = np.load(args.export)
    n = int(z["n"])
    s = setups.shear_layer(n, beta=float(z["beta"]), seed=int(z["seed"]))
    s["qav"] = float(z["qav"])
    state0 = [np.asfortranarray(a) for a in z["state"]]
    grad = [np.asfortranarray(a) for a in z["grad"]]
    # the same reverse sweep about the exact policy's FP64 forward run of the
    # same dts: how far FP64 rounding of the forward moves the derivative
    grad_ex = [np.asfortranarray(a) for a in z["grad_exact_policy"]]
    dts = [float(x) for x in z["dts"]]
    grid = {k: np.asarray(s[k], dtype=LD) for k in ("dx", "dxm", "dy", "dym")}
    nf = 2 * state0[0].size
    # the branches of the long-double base run
    own = np.zeros((len(dts), nf), dtype=np.uint8)
    t0 = time.perf_counter()
    J0 = objective_ld(s, state0, dts, own, 1, grid)
    t_run = time.perf_counter() - t0
    # the branches of the GPU run the adjoint linearises: the runs below hold
    # these (near the switch the two base runs can take different branches)
    act = np.unpackbits(z["av_active"], axis=1, count=nf)
    neg = np.unpackbits(z["av_negative"], axis=1, count=nf)
    rec = (act | (neg << 1)).astype(np.uint8)
    diff = own != rec
    J_held0 = objective_ld(s, state0, dts, rec, 2, grid)
    out = {"n": n, "steps": len(dts), "qav": s["qav"], "h": args.h,
           "J_gpu": float(z["J"]), "J_long_double": float(J0),
           "J_rel_diff": abs(float(J0) - float(z["J"])) / abs(float(z["J"])),
           "J_long_double_held_at_gpu_branches": float(J_held0),
           "active_face_steps": int(np.count_nonzero(rec & 1)),
           "face_steps_on_other_branch_than_gpu": int(np.count_nonzero(diff)),
           "steps_with_such_faces": int(np.count_nonzero(diff.any(axis=1))),
           "seconds_per_run": t_run, "directions": []}
    print(json.dumps({k: v for k, v in out.items() if k != "directions"}), file=sys.stderr,
          flush=True)
    h = LD(args.h)

    def fd(J):
        d1 = (J[1] - J[-1]) / (2 * h)
        d2 = (J[2] - J[-2]) / (4 * h)
        return d1, (4 * d1 - d2) / 3

    rng = np.random.default_rng(5)
    for k in range(args.dirs):
        d = smooth_direction(rng, n)
        zz = [np.zeros_like(a) for a in state0]
        zz[3][1:-1, 1:-1] = d
        oracle.apply_bc_program(zz, s["bc"], s["margin"], s)
        ad = sum(float(np.sum(g * e)) for g, e in zip(grad, zz))
        ad_ex = sum(float(np.sum(g * e)) for g, e in zip(grad_ex, zz))
        cancel = sum(float(np.sum(np.abs(g * e))) for g, e in zip(grad, zz)) / abs(ad)
        J = {m: objective_ld(s, [np.asarray(a, dtype=LD) + m * h * np.asarray(e, dtype=LD)
                                 for a, e in zip(state0, zz)], dts, rec, 2, grid)
             for m in (1, -1, 2, -2)}
        d1, d4 = fd(J)
        row = {"adjoint": ad, "adjoint_exact_policy_forward": ad_ex, "fd2": float(d1),
               "fd4": float(d4),
               "fd2_rel_err": abs(ad - float(d1)) / abs(float(d4)),
               "fd4_rel_err": abs(ad - float(d4)) / abs(float(d4)),
               "fd4_rel_err_exact_policy_adjoint": abs(ad_ex - float(d4)) / abs(float(d4)),
               "fast_vs_exact_forward_adjoints_rel": abs(ad - ad_ex) / abs(float(d4)),
               "cancellation_sum_abs_over_abs": cancel}
        out["directions"].append(row)
        print(json.dumps({"direction": k, **row}), file=sys.stderr, flush=True)
    # dJ/dbeta: p = 0.625 beta in every cell
    dbeta = 0.625 * float(np.sum(grad[1]))
    dbeta_ex = 0.625 * float(np.sum(grad_ex[1]))
    J = {}
    for m in (1, -1, 2, -2):
        st = [np.asarray(a, dtype=LD) for a in state0]
        st[1] = st[1] + m * h * LD(0.625)
        J[m] = objective_ld(s, st, dts, rec, 2, grid)
    d1, d4 = fd(J)
    out["dJ_dbeta"] = {"adjoint": dbeta, "adjoint_exact_policy_forward": dbeta_ex,
                       "fd2": float(d1), "fd4": float(d4),
                       "fd4_rel_err": abs(dbeta - float(d4)) / abs(float(d4)),
                       "fast_vs_exact_forward_adjoints_rel": abs(dbeta - dbeta_ex) /
                       abs(float(d4))}
    e4 = [r["fd4_rel_err"] for r in out["directions"]]
    out["fd4_within_1e-6"] = f"{sum(e <= 1e-6 for e in e4)}/{len(e4)}"
    out["fd4_rel_err_max"] = max(e4) if e4 else None
    out["fd4_rel_err_median"] = float(np.median(e4)) if e4 else None
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
