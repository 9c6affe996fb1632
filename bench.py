#!/usr/bin/env python
"""Throughput of the RI occupied-virtual transform + RI-K on GB300.

Workload (one step): nbas=600, naux=2400, nocc=60, nvir=540.  ri3ao B
[600, 600, 2400] float64 (6.9 GB, larger than L2) from the seeded synthetic
generator, C = Q of the QR factorisation of a seeded N(0,1) 600x600 matrix.
A step produces ov[i,a,P] (622 MB) and K[mu,nu] from the shared
half-transform X^P = B^P C_occ.  Algorithmic work per step (float64
equivalent, no symmetry credit): naux*(4*nb^2*nocc + 2*nb*nocc*nvir) =
3.007e11 FLOP.

`value` is the split-precision form (BF16 digit planes on tcgen05) with
inputs resident in HBM; the float64 form, the split form's error against it,
the end-to-end number through the host-pointer C ABI, the dominant kernel's
roofline and the CPU baseline are reported beside it on the same JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RI transform+RI-K TFLOP/s: split-prec vs FP64 on one GB300 at err≤1e-10"
NB, NAUX, NOCC = 600, 2400, 60
NVIR = NB - NOCC
FLOPS_PER_SLAB = 4 * NB * NB * NOCC + 2 * NB * NOCC * NVIR
FLOPS = NAUX * FLOPS_PER_SLAB  # 3.007e11


FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
# float64 FMA rate of a GB300, from a DFMA throughput probe of this repository
# (register-resident chains, all SMs); used as RI-J's roofline.
DFMA_TFLOPS = 1.20
DFMA_SOURCE = "DFMA throughput probe on GB300 (1.20 TFLOP/s); MEASURED_PEAKS.json holds no float64 rate"


def workload():
    return f"ri_ov_transform_plus_rik nbas={NB} naux={NAUX} nocc={NOCC} nvir={NVIR}"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--nslices", type=int, default=7)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--sweep", default="", help="comma list of slice counts to also report (time, errors)")
    p.add_argument("--naux", type=int, default=NAUX, help="auxiliary slabs (smaller values only for profiling runs)")
    p.add_argument("--batch-mols", type=int, default=64, help="molecules of the batched uneven-size leg (0: skip)")
    p.add_argument("--batch-steps", type=int, default=20)
    p.add_argument("--large", type=int, default=1, help="run the nbas=1200 / naux=4800 system with Davidson (0: skip)")
    p.add_argument("--outputs", type=int, default=1,
                   help="also time the full ri3mo transform and the (ia|jb) block of this workload (0: skip)")
    p.add_argument("--large-steps", type=int, default=3)
    p.add_argument("--large-full", type=int, default=1,
                   help="also run Davidson on the full 129600-state space of the large system (0: skip)")
    p.add_argument("--large-full-cycles", type=int, default=1200)
    p.add_argument("--large-full-residual", type=int, default=4000,
                   help="also run the full space to residual 1e-8 (tol 1e-16, lindep 1e-24; cycles given here, 0: skip)")
    p.add_argument("--scf", type=int, default=1,
                   help="also time lapack_power and lapack_dspgvx on the device eigensolver (0: skip)")
    p.add_argument("--dropin", type=int, default=1,
                   help="also time the drop-in ri_ao2mo_f_ end to end on host buffers, both forms (0: skip)")
    p.add_argument("--dropin-child", action="store_true", help=argparse.SUPPRESS)
    p.add_argument("--ri3fn", type=int, default=1,
                   help="also time the ri3fn metric step (special_dgemm_f_01) on this workload's tensor (0: skip)")
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return d, "measured"
    except Exception:
        return dict(FALLBACK_PEAKS), "fallback"


# ----------------------------------------------------------------- clocks --
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(gpu_index)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i in range(4) if r[i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------ batched leg --
def batch_shapes(seed: int, n: int):
    """n molecules: nbas uniform in [40, 400], naux = 4 nbas, nocc = round(nbas / 10)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for nb in rng.integers(40, 401, size=n):
        nb = int(nb)
        out.append((nb, 4 * nb, int(round(nb / 10))))
    return out


def batched_leg(args, rt, torch, stream):
    """Many molecules of uneven size, one grouped launch per product, replayed from a CUDA graph."""
    from rest_tensors_gb300 import autotune

    shapes = batch_shapes(args.seed, args.batch_mols)
    probs, flops = [], 0.0
    for k, (nb, naux, nocc) in enumerate(shapes):
        nvir = nb - nocc
        probs.append(dict(C=rt.synth_coef(k, nb), B=rt.synth_ri3ao(k, nb, naux), nb=nb, naux=naux, nocc=nocc,
                          nvir=nvir,
                          ov=torch.empty(nocc * nvir * naux, dtype=torch.float64, device="cuda"),
                          K=torch.empty(nb * nb, dtype=torch.float64, device="cuda")))
        flops += naux * (4.0 * nb * nb * nocc + 2.0 * nb * nocc * nvir)
    S = args.nslices
    out = {"workload": f"{len(shapes)} molecules, nbas uniform in [40, 400] (seed {args.seed}), naux = 4 nbas, "
                       f"nocc = round(nbas/10); ov transform + RI-K per molecule",
           "molecules": len(shapes), "flop_per_step": flops,
           "ri3ao_gb": sum(nb * nb * naux for nb, naux, _ in shapes) * 8 / 1e9,
           "graph": "one CUDA graph per form, captured once and replayed each step"}
    res = {}
    for form in ("fp64", "split"):
        tuning = autotune.lookup(probs, form, S, stream=stream) if form == "split" else None
        rt.ri_ov_k_batched(probs, form=form, nslices=S, tuning=tuning, stream=stream)
        rt.sync_status()
        if form == "fp64":
            ref = [(q["ov"].clone(), q["K"].clone()) for q in probs]
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            rt.ri_ov_k_batched(probs, form=form, nslices=S, tuning=tuning)
        steps = max(1, args.batch_steps if form == "split" else max(1, args.batch_steps // 10))
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        n0 = rt.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cs = torch.cuda.current_stream()
        e0.record(cs)
        for _ in range(steps):
            g.replay()
        e1.record(cs)
        torch.cuda.synchronize()
        rt.sync_status()
        ms = e0.elapsed_time(e1) / steps
        res[form] = {"tflops": flops / ms / 1e9, "ms_per_step": ms, "steps": steps}
        if tuning is not None:
            res[form]["tuning"] = {"fuse": tuning.fuse, "chunks_per_item": tuning.chunks_per_item,
                                   "table": autotune.table_path()}
        del g
    ov_err = max(float((q["ov"] - r[0]).abs().max()) for q, r in zip(probs, ref))
    k_err = max(float((q["K"] - r[1]).abs().max() / r[1].abs().max()) for q, r in zip(probs, ref))
    out.update(res)
    out["speedup_vs_fp64"] = res["fp64"]["ms_per_step"] / res["split"]["ms_per_step"]
    out["errors_vs_fp64"] = {"ov_max_abs": ov_err, "K_max_rel": k_err}
    if not args.no_cpu:
        # The oracle on every molecule's own inputs (copied back from the device), as checker of both forms.
        import numpy as np

        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        ev = {f: {"ov_max_abs": 0.0, "K_max_rel": 0.0} for f in ("fp64", "split")}
        t0 = time.perf_counter()
        for q, r in zip(probs, ref):
            nb, naux, nocc, nvir = q["nb"], q["naux"], q["nocc"], q["nvir"]
            ov_o, K_o = oracle.ri_ov_k(fortran_view(q["C"], (nb, nb)), fortran_view(q["B"], (nb, nb, naux)), nocc)
            for f, (ovd, Kd) in (("fp64", r), ("split", (q["ov"], q["K"]))):
                ev[f]["ov_max_abs"] = max(ev[f]["ov_max_abs"],
                                          float(np.abs(fortran_view(ovd, (nocc, nvir, naux)) - ov_o).max()))
                ev[f]["K_max_rel"] = max(ev[f]["K_max_rel"], float(np.abs(fortran_view(Kd, (nb, nb)) - K_o).max()
                                                                   / np.abs(K_o).max()))
        ev["inputs"] = f"all {len(probs)} molecules, the device's inputs copied to the host"
        ev["oracle_seconds"] = time.perf_counter() - t0
        out["errors_vs_oracle"] = ev
    del probs, ref
    torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------- large leg --
def large_leg(args, rt, torch, stream):
    """nbas=1200, naux=4800 (55 GB of ri3ao in HBM), nocc=120: split RI-K against float64, then
    Davidson for the 8 lowest roots of the 14400 x 14400 response matrix diag(delta) + B_ov B_ov^T
    over the 120 occupied x 120 lowest virtual orbitals (tol 1e-8 in the reference's sense:
    eigenvalue change below tol, residual norm below sqrt(tol))."""
    nb, naux, nocc = 1200, 4800, 120
    nvir = nb - nocc
    flops = naux * (4.0 * nb * nb * nocc + 2.0 * nb * nocc * nvir)
    B = rt.synth_ri3ao(args.seed, nb, naux)
    C = rt.synth_coef(args.seed, nb)
    Cm = C.view(nb, nb).t()
    D = (Cm[:, :nocc] @ Cm[:, :nocc].t()).t().contiguous().view(-1)
    ov = torch.empty(nocc * nvir * naux, dtype=torch.float64, device="cuda")
    K = torch.empty(nb * nb, dtype=torch.float64, device="cuda")
    S = args.nslices
    out = {"workload": f"ri_ov_transform_plus_rik nbas={nb} naux={naux} nocc={nocc} nvir={nvir}",
           "ri3ao_gb": nb * nb * naux * 8 / 1e9, "flop_per_step": flops}

    def timed(form, steps):
        rt.ri_ov_k(C, B, nb, naux, nocc, nvir, ov=ov, K=K, form=form, nslices=S, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            rt.ri_ov_k(C, B, nb, naux, nocc, nvir, ov=ov, K=K, form=form, nslices=S, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        rt.sync_status()
        return e0.elapsed_time(e1) / steps

    ms64 = timed("fp64", 1)
    ov64, K64 = ov.clone(), K.clone()
    ex64 = rt.exchange_energy(D, K64, nb).item()
    ms = timed("split", max(1, args.large_steps))
    ex = rt.exchange_energy(D, K, nb).item()
    out["split"] = {"tflops": flops / ms / 1e9, "ms_per_step": ms, "nslices": S}
    out["fp64"] = {"tflops": flops / ms64 / 1e9, "ms_per_step": ms64}
    out["speedup_vs_fp64"] = ms64 / ms
    out["errors_vs_fp64"] = {"ov_max_abs": float((ov - ov64).abs().max()),
                             "K_max_rel": float((K - K64).abs().max() / K64.abs().max()),
                             "ex_abs": abs(ex - ex64), "ex_fp64": ex64}
    if not args.no_cpu:
        # The oracle on a slab subset (the whole tensor is 55 GB): the measured run's ov slabs
        # against it in both forms, and K and E_x over the same slabs from the GPU entry point.
        import numpy as np

        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        nsub = 96
        Bs = B[: nsub * nb * nb]
        t0 = time.perf_counter()
        Ch = fortran_view(C, (nb, nb))
        ov_o, K_o = oracle.ri_ov_k(Ch, fortran_view(Bs, (nb, nb, nsub)), nocc)
        Co = Ch[:, :nocc]
        ex_o = oracle.exchange_energy(np.asfortranarray(Co @ Co.T), K_o)
        ev = {"inputs": f"slabs 0..{nsub - 1} of {naux}, the device's inputs copied to the host",
              "oracle_seconds": time.perf_counter() - t0, "ex_oracle_subset": ex_o}
        nsl = nocc * nvir * nsub
        for f, ovd in (("fp64", ov64), ("split", ov)):
            _, Ks = rt.ri_ov_k(C, Bs, nb, nsub, nocc, nvir, form=f, nslices=S, want_ov=False, stream=stream)
            ex_s = rt.exchange_energy(D, Ks, nb).item()
            ev[f] = {"ov_max_abs": float(np.abs(fortran_view(ovd[:nsl], (nocc, nvir, nsub)) - ov_o).max()),
                     "K_max_rel": float(np.abs(fortran_view(Ks, (nb, nb)) - K_o).max() / np.abs(K_o).max()),
                     "ex_abs": abs(ex_s - ex_o)}
            del Ks
        out["errors_vs_oracle"] = ev
        del Bs
    J = rt.ri_j(B, D, nb, naux)[1]
    out["J_norm"] = float(J.norm())
    del ov64, K64, J

    # Response problems: B_ov^P from the split transform, couplings scaled so the
    # mean of diag(B_ov B_ov^T) is 0.09 Eh against delta in [0.5, 3] Eh.
    #   * the 14400 x 14400 window (120 occupied x 120 lowest virtuals) at tol 1e-8 (the reference's
    #     semantics: |de| < tol and |r| < sqrt(tol) = 1e-4), as before;
    #   * the same window to |r| < 1e-8: tol 1e-16 (sqrt(tol) = 1e-8) with DavidsonParams.lindep lowered
    #     from 1e-14 to 1e-24, so that preconditioned residuals of norm ~1e-8 are not dropped as linearly
    #     dependent; split and float64 matvecs;
    #   * optionally the full 129600-state space.
    runs = [("window_120x120", nocc, dict(tol=1e-8, maxcyc=400, maxspace=40, nroots=8), "split"),
            ("window_120x120_residual_1e-8", nocc,
             dict(tol=1e-16, maxcyc=600, maxspace=40, nroots=8, lindep=1e-24), "split"),
            ("window_120x120_residual_1e-8_fp64_matvec", nocc,
             dict(tol=1e-16, maxcyc=600, maxspace=40, nroots=8, lindep=1e-24), "fp64")]
    if args.large_full:
        runs.append(("full_120x1080", nvir, dict(tol=1e-8, maxcyc=args.large_full_cycles, maxspace=100, nroots=8,
                                                 lindep=1e-24), "split"))
    if args.large_full_residual > 0:
        runs.append(("full_120x1080_residual_1e-8", nvir, dict(tol=1e-16, maxcyc=args.large_full_residual, maxspace=100,
                                                               nroots=8, lindep=1e-24), "split"))
    dav = {}
    windows = {}
    for label, nv, prm, mform in runs:
        nov = nocc * nv
        if nv not in windows:
            if nv == nvir:
                Bov = ov
            else:
                Bov, _ = rt.ri_ov_k(C[: nb * (nocc + nv)], B, nb, naux, nocc, nv, form="split", nslices=S,
                                    want_k=False, stream=stream)
            Bv = Bov.view(naux, nov)
            rowsq = (Bv * Bv).sum(0)
            gamma = 0.3 / float(rowsq.mean().sqrt())
            Bov.mul_(gamma)
            rowsq.mul_(gamma * gamma)
            windows[nv] = (Bov, Bv, rowsq, gamma)
        Bov, Bv, rowsq, gamma = windows[nv]
        delta = rt.synth_delta(args.seed, nov)
        hd = delta + rowsq
        x0 = torch.zeros(nov, dtype=torch.float64, device="cuda")
        x0[int(torch.argmin(hd))] = 1.0
        p = rt.DavidsonParams(**prm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        conv, e, x, its = rt.davidson_ri_response(Bov, delta, nov, naux, x0, p, form=mform, nslices=S,
                                                  stream=stream)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # residual norms of the returned pairs, recomputed in float64
        Xc = x.contiguous()
        AXc = delta[None, :] * Xc + (Xc @ Bv.t()) @ Bv
        ev = torch.tensor(e, dtype=torch.float64, device="cuda")
        res = (AXc - ev[:, None] * Xc).norm(dim=1)
        d = {"nov": nov, "coupling_scale": gamma, "params": prm, "matvec": mform, "converged": conv,
             "iterations": its, "seconds": dt, "eigenvalues": e, "max_residual_norm": float(res.max())}
        if nov <= 20000:
            try:
                A = torch.diag(delta) + Bv.t() @ Bv
                ex_e = torch.linalg.eigvalsh(A)[:8].cpu().tolist()
                d["max_abs_vs_dense_eigvalsh"] = max(abs(a - b) for a, b in zip(e, ex_e))
                del A
            except Exception as exc:  # the dense check is verification only
                d["dense_check"] = f"unavailable: {type(exc).__name__}"
        dav[label] = d
        del Xc, AXc
    for nv, (Bov, _, _, _) in windows.items():
        if nv != nvir:
            del Bov
    del windows
    out["davidson"] = dav
    del B, ov, K
    torch.cuda.empty_cache()
    return out


# -------------------------------------------------- other outputs of config 2 --
def outputs_leg(args, rt, torch, stream, B, C, ov):
    """The full ri3mo transform [naux, nbas, nbas] and the (ia|jb) block (nocc nvir)^2,
    split form against the float64 form (one timed call each after a warm-up)."""
    S = args.nslices

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        rt.sync_status()
        return out, e0.elapsed_time(e1)

    res = {}
    # ri3mo: naux (2 nb^2 ns + 2 nb ns^2) with ns = nb
    fl = NAUX * 4.0 * NB ** 3
    r64 = torch.empty(NAUX * NB * NB, dtype=torch.float64, device="cuda")
    rsp = torch.empty_like(r64)
    _, ms64 = timed(lambda: rt.ri_ao2mo(C, B, NB, NB, NAUX, out=r64, form="fp64", stream=stream))
    _, mssp = timed(lambda: rt.ri_ao2mo(C, B, NB, NB, NAUX, out=rsp, form="split", nslices=S, stream=stream))
    res["ri3mo"] = {"shape": [NAUX, NB, NB], "flop": fl, "split": {"ms": mssp, "tflops": fl / mssp / 1e9},
                    "fp64": {"ms": ms64, "tflops": fl / ms64 / 1e9}, "speedup_vs_fp64": ms64 / mssp,
                    "max_abs_err": float((rsp - r64).abs().max())}
    del r64, rsp
    # (ia|jb) = sum_P B_ia^P B_jb^P, B_ov = ov as [nocc nvir, naux]
    nov = NOCC * NVIR
    fl = 2.0 * nov * nov * NAUX
    m64 = torch.empty(nov * nov, dtype=torch.float64, device="cuda")
    msp = torch.empty_like(m64)
    _, ms64 = timed(lambda: rt.ri_iajb(ov, nov, NAUX, M=m64, form="fp64", stream=stream))
    _, mssp = timed(lambda: rt.ri_iajb(ov, nov, NAUX, M=msp, form="split", nslices=S, stream=stream))
    res["iajb"] = {"shape": [nov, nov], "flop": fl, "split": {"ms": mssp, "tflops": fl / mssp / 1e9},
                   "fp64": {"ms": ms64, "tflops": fl / ms64 / 1e9}, "speedup_vs_fp64": ms64 / mssp,
                   "max_rel_err": float((msp - m64).abs().max() / m64.abs().max())}
    del m64, msp
    torch.cuda.empty_cache()
    return res


# ------------------------------------------ the drop-in ri_ao2mo_f_ end to end --
def dropin_ao2mo_once(rt, Ch, Bh, R):
    """One warm-up call and one timed call of the ri_ao2mo_f_ symbol on pageable host buffers."""
    rt.ri_ao2mo_f(Ch, Bh, R, NB, NB, NAUX)
    t0 = time.perf_counter()
    rt.ri_ao2mo_f(Ch, Bh, R, NB, NB, NAUX)
    return time.perf_counter() - t0


def dropin_child(args):
    """Child process of the drop-in leg (run with RT_FORM set): the same inputs, the symbol timed once
    after a warm-up, the result compared with the device float64 transform."""
    import numpy as np
    import torch

    import rest_tensors_gb300 as rt

    B = rt.synth_ri3ao(args.seed, NB, NAUX)
    C = rt.synth_coef(args.seed, NB)
    Bh, Ch = B.cpu().numpy(), C.cpu().numpy()
    R = np.empty(NAUX * NB * NB)
    dt = dropin_ao2mo_once(rt, Ch, Bh, R)
    R64 = rt.ri_ao2mo(C, B, NB, NB, NAUX, form="fp64").cpu().numpy()
    torch.cuda.synchronize()
    print(json.dumps({"seconds": dt, "max_abs_vs_device_fp64": float(np.abs(R - R64).max())}), flush=True)


def dropin_ao2mo_leg(args, rt, B, C):
    """ri_ao2mo_f_ (the reference's own seam, src/external_libs/ffi_restmatr.rs:5-11) end to end on pageable
    host buffers, as a Rust Vec would be: the full transform [naux, nbas, nbas] (2.07e12 FLOP), with 6.9 GB in
    and 6.9 GB out inside the timing.  Float64 (the default) in this process; the split form in a child
    process with RT_FORM=split, because the seam reads its form once per process."""
    import numpy as np

    fl = NAUX * 4.0 * NB ** 3
    Bh, Ch = B.cpu().numpy(), C.cpu().numpy()
    R = np.empty(NAUX * NB * NB)
    res = {"flop": fl, "h2d_bytes": 8 * (NB * NB * NAUX + NB * NB), "d2h_bytes": 8 * NAUX * NB * NB,
           "host_memory": "pageable (numpy), as a Rust Vec", "path": "ri_ao2mo_f_ -> rt_ri_ao2mo_host"}
    if os.environ.get("RT_FORM", "fp64").lower() in ("", "fp64"):
        dt = dropin_ao2mo_once(rt, Ch, Bh, R)
        res["fp64"] = {"ms": dt * 1e3, "tflops": fl / dt / 1e12}
    del R
    env = {**os.environ, "RT_FORM": "split", "RT_NSLICES": str(args.nslices)}
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--dropin-child", "--seed", str(args.seed)],
                       env=env, capture_output=True, text=True, timeout=900)
    if r.returncode == 0 and r.stdout.strip():
        d = json.loads(r.stdout.strip().splitlines()[-1])
        res["split"] = {"ms": d["seconds"] * 1e3, "tflops": fl / d["seconds"] / 1e12, "nslices": args.nslices,
                        "max_abs_vs_device_fp64": d["max_abs_vs_device_fp64"], "env": "RT_FORM=split"}
    else:
        res["split"] = {"error": (r.stderr or r.stdout)[-400:]}
    if not args.no_cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        nsl = 240
        Bf = Bh.reshape(NAUX, NB, NB).transpose(2, 1, 0)
        Cf = Ch.reshape(NB, NB).T
        oracle.ri_ao2mo(Cf, Bf[:, :, :24])  # warm-up
        t0 = time.perf_counter()
        oracle.ri_ao2mo(Cf, Bf[:, :, :nsl])
        dt = time.perf_counter() - t0
        res["cpu"] = {"tflops": nsl * 4.0 * NB ** 3 / dt / 1e12, "cores": oracle.get_threads(), "seconds": dt,
                      "sample": f"{nsl} of {NAUX} aux slabs, C restatement of restmatr.f90:158-194 over OpenBLAS"}
    return res


# ------------------------------------------------ ri3fn metric step (special_dgemm_f_01) --
def ri3fn_leg(args, rt, torch, stream, B):
    """The O_V V^{-1/2} step of the ri3fn preparation on this workload's tensor
    [nbas, nbas, naux]: every (mu, nu) row times an [naux, naux] matrix, in place.
    The matrix is an orthogonal stand-in for V^{-1/2} (Q of a seeded QR).
    Split and float64 forms are timed once each after a warm-up; both are checked
    on three nu-slices against the oracle's float64 product on the host, and an
    OpenBLAS sample on the host cores gives the CPU rate."""
    import numpy as np

    S = args.nslices
    M = rt.synth_coef(args.seed + 7, NAUX)
    size_a, size_b = (NB, NB, NAUX), (NAUX, NAUX)
    fl = 2.0 * NB * NB * NAUX * NAUX

    def call(T, form):
        rt.special_dgemm_01(T, size_a, range(NB), range(NAUX), M, size_b, range(NAUX), range(NAUX), 1.0, 0.0,
                            form=form, nslices=S, stream=stream)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        rt.sync_status()
        return e0.elapsed_time(e1)

    T = B.clone()
    call(T, "split")  # warm-up (scratch pool, kernels)
    T.copy_(B)
    ms_sp = timed(lambda: call(T, "split"))
    T64 = B.clone()
    ms_64 = timed(lambda: call(T64, "fp64"))
    Mh = M.cpu().numpy().reshape(NAUX, NAUX, order="F")
    Bv = B.view(NAUX, NB, NB)  # [P][nu][mu]
    errs = {"split": 0.0, "fp64": 0.0}
    for nu in (0, NB // 2 + 1, NB - 1):
        slab = Bv[:, nu, :].cpu().numpy().T  # [mu, P]
        want = slab @ Mh
        scale = float(np.abs(want).max())
        for name, t in (("split", T), ("fp64", T64)):
            got = t.view(NAUX, NB, NB)[:, nu, :].cpu().numpy().T
            errs[name] = max(errs[name], float(np.abs(got - want).max()) / scale)
    split_vs_fp64 = float((T - T64).abs().max() / T64.abs().max())
    del T, T64
    torch.cuda.empty_cache()
    # The drop-in symbol on pageable host memory (what a Rust Vec is): transfers inside the timing.
    ny = NB // 10
    th = np.ascontiguousarray(Bv[:, :ny, :].cpu().numpy())  # [P][nu < ny][mu] = ten3_a [NB, ny, NAUX]
    th = th.reshape(-1)
    t0 = time.perf_counter()
    rt.special_dgemm_f_01(th, (NB, ny, NAUX), range(NB), 0, range(NAUX), Mh.reshape(-1, order="F"), size_b,
                          range(NAUX), range(NAUX), 1.0, 0.0)
    dt_h = time.perf_counter() - t0
    fl_h = 2.0 * NB * ny * NAUX * NAUX
    e2e_dropin = {"tflops": fl_h / dt_h / 1e12, "ms": dt_h * 1e3, "h2d_bytes": 8 * NB * ny * NAUX + 8 * NAUX * NAUX,
                  "d2h_bytes": 8 * NB * ny * NAUX,
                  "sample": f"special_dgemm_f_01_ (float64 form) on a pageable [{NB}, {ny}, {NAUX}] host tensor, "
                            f"copies in and out inside the timing"}
    del th
    res = {"shape": {"ten3_a": list(size_a), "matr_b": list(size_b)}, "flop": fl, "e2e_dropin": e2e_dropin,
           "split": {"ms": ms_sp, "tflops": fl / ms_sp / 1e9},
           "fp64": {"ms": ms_64, "tflops": fl / ms_64 / 1e9}, "speedup_vs_fp64": ms_64 / ms_sp,
           "max_rel_err_vs_oracle": errs, "split_vs_fp64_max_rel": split_vs_fp64,
           "matr_b": "orthogonal stand-in for V^-1/2 (Q of a seeded N(0,1) QR)"}
    if not args.no_cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        ny = 32
        rng = np.random.default_rng(args.seed)
        t = rng.standard_normal(NB * ny * NAUX)
        oracle.special_dgemm_f_01(t, (NB, ny, NAUX), (0, NB), (0, NAUX), Mh.reshape(-1, order="F"), size_b,
                                  (0, NAUX), (0, NAUX), 1.0, 0.0)  # warm-up
        t0 = time.perf_counter()
        oracle.special_dgemm_f_01(t, (NB, ny, NAUX), (0, NB), (0, NAUX), Mh.reshape(-1, order="F"), size_b,
                                  (0, NAUX), (0, NAUX), 1.0, 0.0)
        dt = time.perf_counter() - t0
        res["cpu"] = {"tflops": 2.0 * NB * ny * NAUX * NAUX / dt / 1e12, "cores": oracle.get_threads(),
                      "sample": f"{ny} of {NB} nu-slices, C restatement of restmatr.f90:111-154 over OpenBLAS",
                      "seconds": dt}
    return res


# --------------------------------------------------- Newton-Schulz inverse square root --
def newton_schulz_leg(args, rt, torch, stream):
    """_newton_schulz_inverse_square_root_v02 on a [naux, naux] symmetric positive stand-in for the
    Coulomb metric V: Q diag(d) Q^T with d uniform in [0.5, 3] (seeded) and Q the seeded orthogonal
    matrix of the ri3fn leg.  The reference's own parameters: threshold 1e-8 scaled to 1e-10, mixing
    1.0, 100 iterations, level shift [0.0].  Both forms once after a warm-up, and the oracle on the
    host cores."""
    import numpy as np

    n = NAUX
    Q = rt.synth_coef(args.seed + 7, n).view(n, n)  # column-major: Q[col][row]
    d = torch.from_numpy(np.random.default_rng(args.seed + 11).uniform(0.5, 3.0, n)).cuda()
    S = (Q.t() * d) @ Q  # [row][col] view of a symmetric matrix; its flat data is the column-major matrix
    S = (0.5 * (S + S.t())).contiguous().view(-1)
    args_ns = (1e-10, 1.0, 100, [0.0])

    def run(form):
        return rt.newton_schulz_inverse_square_root_v02(S, n, *args_ns, form=form, nslices=args.nslices,
                                                         stream=stream)

    res = {"n": n, "threshold": 1e-10, "mix_parameter": 1.0, "num_iter": 100, "level_shift": [0.0],
           "matrix": "Q diag(d) Q^T, d ~ U[0.5, 3], stand-in for the Coulomb metric"}
    outs = {}
    for form in ("split", "fp64"):
        run(form)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, _, conv, evals = run(form)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        fl = evals * 3 * 2.0 * n ** 3
        res[form] = {"ms": dt * 1e3, "converged": conv, "evaluations": evals, "tflops": fl / dt / 1e12}
        outs[form] = X
    Xf = outs["fp64"].view(n, n)
    Sm = S.view(n, n)
    res["fp64"]["max_abs_residual_XSX_minus_I"] = float((Xf @ Sm @ Xf - torch.eye(n, dtype=torch.float64,
                                                                                 device="cuda")).abs().max())
    res["split_vs_fp64_max_rel"] = float((outs["split"] - outs["fp64"]).abs().max() / outs["fp64"].abs().max())
    res["speedup_vs_fp64"] = res["fp64"]["ms"] / res["split"]["ms"]
    res["timing"] = "host clock around the call (it synchronises once per evaluation)"
    if not args.no_cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        Sh = S.cpu().numpy().reshape(n, n, order="F")
        t0 = time.perf_counter()
        Xo, _, conv_o, evals_o = oracle.newton_schulz_inverse_square_root_v02(Sh, *args_ns)
        dt = time.perf_counter() - t0
        res["cpu"] = {"ms": dt * 1e3, "converged": conv_o, "evaluations": evals_o,
                      "tflops": evals_o * 6.0 * n ** 3 / dt / 1e12, "cores": oracle.get_threads(),
                      "sample": "the whole call: numpy restatement of matrix_blas_lapack.rs:1710-1932 over OpenBLAS"}
        res["fp64"]["max_rel_err_vs_oracle"] = float(np.abs(outs["fp64"].cpu().numpy().reshape(n, n, order="F") - Xo).max()
                                                     / np.abs(Xo).max())
    del outs, S, Q
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------ SCF-side dense LAPACK --
def scf_lapack_leg(args, rt, torch):
    """lapack_power (S^-1/2 of an overlap-sized matrix and of a metric-sized one) and lapack_dspgvx (all
    eigenpairs of F x = e S x) on the device eigensolver, each timed once after a warm-up with the host clock
    (the calls synchronise), beside the oracle over OpenBLAS on the host cores.  Matrices: S = Q diag(d) Q^T,
    d ~ U[0.5, 3]; F = Q' diag(f) Q'^T, f ~ U[-20, 5] (seeded stand-ins for an overlap and a Fock matrix)."""
    import numpy as np

    import oracle

    def spd(n, seed, lo, hi):
        Q = rt.synth_coef(seed, n).view(n, n)
        d = torch.from_numpy(np.random.default_rng(seed).uniform(lo, hi, n)).cuda()
        M = (Q.t() * d) @ Q
        return (0.5 * (M + M.t())).contiguous().view(-1)

    def packed(M, n):  # MatrixUpper storage: column j holds rows 0..j
        return oracle.full_to_upper_packed(M.cpu().numpy().reshape(n, n, order="F"))

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    oracle.set_threads(os.cpu_count() or 1)
    res = {"matrices": "S = Q diag(d) Q^T, d ~ U[0.5, 3]; F = Q' diag(f) Q'^T, f ~ U[-20, 5] (seeded)"}
    for n in (600, 2400):
        S = spd(n, 31 + n, 0.5, 3.0)
        (out, kept), dt = timed(lambda: rt.lapack_power(S, n, -0.5, 1e-10, form="fp64"))
        d = {"gpu_ms": dt * 1e3, "kept": kept}
        if not args.no_cpu:
            Sh = S.cpu().numpy().reshape(n, n, order="F")
            t0 = time.perf_counter()
            ref, _ = oracle.lapack_power(Sh, -0.5, 1e-10)
            d["cpu_ms"] = (time.perf_counter() - t0) * 1e3
            d["cpu_cores"] = oracle.get_threads()
            d["speedup_vs_cpu"] = d["cpu_ms"] / d["gpu_ms"]
            d["max_rel_err_vs_oracle"] = float(np.abs(out.cpu().numpy().reshape(n, n, order="F") - ref).max()
                                               / np.abs(ref).max())
        res[f"lapack_power_n{n}"] = d
        del S, out
    for n in (600, 1200):
        S = spd(n, 41 + n, 0.5, 3.0)
        F = spd(n, 51 + n, -20.0, 5.0)
        ap, bp = packed(F, n), packed(S, n)
        dap, dbp = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
        (z, w), dt = timed(lambda: rt.dspgvx(dap, dbp, n, n, form="fp64"))
        d = {"gpu_ms": dt * 1e3, "num_orb": n}
        if not args.no_cpu:
            t0 = time.perf_counter()
            z_ref, w_ref, _ = oracle.dspgvx(ap, bp, n, n)
            d["cpu_ms"] = (time.perf_counter() - t0) * 1e3
            d["cpu_cores"] = oracle.get_threads()
            d["speedup_vs_cpu"] = d["cpu_ms"] / d["gpu_ms"]
            d["eigenvalue_max_rel_err_vs_oracle"] = float(np.abs(w.cpu().numpy() - w_ref).max() / np.abs(w_ref).max())
        res[f"dspgvx_n{n}"] = d
        del S, F, dap, dbp, z, w
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------- layout utilities --
def layout_leg(args, rt, torch, stream, B):
    """RIFull transposes and the symmetric pair packing on this workload's ri3ao
    tensor [nbas, nbas, naux] (6.9 GB): bytes moved per call (read + write) over
    CUDA-event time, as GB/s and as a fraction of the measured copy rate."""
    hbm = peaks()[0]["hbm_gbs"]
    nel = NB * NB * NAUX
    out = torch.empty(nel, dtype=torch.float64, device="cuda")
    res = {}

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        rt.sync_status()
        return e0.elapsed_time(e1) / reps

    for order in ("jik", "jki", "kji", "ikj"):
        ms = timed(lambda: rt.ri_transpose(B, (NB, NB, NAUX), order, out=out, stream=stream))
        gbs = 16.0 * nel / ms / 1e6
        res["transpose_" + order] = {"ms": ms, "gbs": gbs, "frac_of_copy": gbs / hbm}
    half = NAUX // 2
    ms = timed(lambda: rt.copy_rr((NB, NB, half), B, (NB, NB, NAUX), (0, 0, half), out, (NB, NB, NAUX), (0, 0, 0),
                                  stream=stream))
    gbs = 16.0 * NB * NB * half / ms / 1e6
    res["copy_rr_half"] = {"ms": ms, "gbs": gbs, "frac_of_copy": gbs / hbm}
    npair = NB * (NB + 1) // 2
    ms = timed(lambda: rt.ri_pack_symm(B, NB, NAUX, out=out, stream=stream))
    gbs = 16.0 * npair * NAUX / ms / 1e6
    res["pack_symm"] = {"ms": ms, "gbs": gbs, "frac_of_copy": gbs / hbm}
    res["note"] = ("inputs 6.9 GB (larger than L2); transposes count one read of the input and one write of the "
                   "output; pack_symm counts the upper triangles it reads and writes (3.46 GB each); copy rate "
                   "from the measured peaks")
    del out
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------ CPU baseline --
def fortran_view(t, shape):
    """Host numpy view of a flat column-major device tensor, Fortran-ordered (no copy after the transfer)."""
    return t.cpu().numpy().reshape(tuple(reversed(shape))).transpose(*reversed(range(len(shape))))


def cpu_baseline(B, C, outs, budget_s: float = 12.0):
    """The oracle (C restatement of restmatr.f90 + OpenBLAS, all host threads) on the same inputs the
    GPU ran, copied back from the device: timed over a bounded slab range (the whole workload when it
    fits the budget) as the CPU baseline, and run over every slab as the checker of the GPU outputs.

    outs: {form: (ov, K, E_x)} device results of the measured workload."""
    import numpy as np

    import oracle

    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    Bh = fortran_view(B, (NB, NB, NAUX))
    Ch = fortran_view(C, (NB, NB))
    probe = 24
    oracle.ri_ov_k(Ch, Bh[:, :, :probe], NOCC)  # warm-up (threads, pages)
    t0 = time.perf_counter()
    oracle.ri_ov_k(Ch, Bh[:, :, :probe], NOCC)
    per_slab = (time.perf_counter() - t0) / probe
    nslab = int(max(probe, min(NAUX, budget_s / max(per_slab, 1e-9))))
    t0 = time.perf_counter()
    ov_ref, K_ref = oracle.ri_ov_k(Ch, Bh[:, :, :nslab], NOCC)
    dt = time.perf_counter() - t0
    if nslab < NAUX:
        ov_ref, K_ref = oracle.ri_ov_k(Ch, Bh, NOCC)
    Co = Ch[:, :NOCC]
    ex_ref = oracle.exchange_energy(np.asfortranarray(Co @ Co.T), K_ref)
    errs = {}
    for form, (ov, K, ex) in outs.items():
        ov_h = fortran_view(ov, (NOCC, NVIR, NAUX))
        K_h = fortran_view(K, (NB, NB))
        errs[form] = {"ov_max_abs": float(np.abs(ov_h - ov_ref).max()),
                      "ov_max_rel": float(np.abs(ov_h - ov_ref).max() / np.abs(ov_ref).max()),
                      "K_max_rel": float(np.abs(K_h - K_ref).max() / np.abs(K_ref).max()),
                      "ex_abs": abs(ex - ex_ref), "ex_rel": abs(ex - ex_ref) / abs(ex_ref)}
    errs["ex_oracle"] = ex_ref
    errs["inputs"] = "the device's ri3ao and C, copied to the host; oracle over all slabs"
    del Bh, ov_ref, K_ref
    cpu = {"value": nslab * FLOPS_PER_SLAB / dt / 1e12, "unit": "TFLOP/s", "cores": oracle.get_threads(),
           "kind": "port",
           "sample": f"{nslab} of {NAUX} aux slabs of the same workload ({dt:.2f} s), C restatement of "
                     f"restmatr.f90 per-slab dgemms over OpenBLAS (scipy bundle)",
           "seconds": dt}
    return cpu, errs


def run_reference(args, rank: int):
    global NAUX, FLOPS
    NAUX = args.naux
    FLOPS = NAUX * FLOPS_PER_SLAB
    if rank != 0:
        return
    per_step_budget = max(1.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
    import oracle

    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    C = oracle.synth_coef(args.seed, NB)
    probe = max(1, min(24, NAUX))
    B = oracle.synth_ri3ao(args.seed, NB, NAUX, 0, probe)
    oracle.ri_ov_k(C, B, NOCC)
    t0 = time.perf_counter()
    oracle.ri_ov_k(C, B, NOCC)
    per_slab = (time.perf_counter() - t0) / probe
    nslab = int(max(probe, min(NAUX, per_step_budget / max(per_slab, 1e-9))))  # at most NAUX slabs
    B = oracle.synth_ri3ao(args.seed, NB, NAUX, 0, nslab)
    for _ in range(args.warmup):
        oracle.ri_ov_k(C, B, NOCC)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.ri_ov_k(C, B, NOCC)
    dt = (time.perf_counter() - t0) / max(1, args.steps)
    v = nslab * FLOPS_PER_SLAB / dt / 1e12
    sample = (f"each step: {nslab} of {NAUX} aux slabs of the same workload, C restatement of restmatr.f90 "
              f"per-slab dgemms over OpenBLAS (the reference's own path cannot be built: Rust+Fortran "
              f"toolchains absent)")
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload(), "nbas": NB, "naux": NAUX, "nocc": NOCC, "nvir": NVIR,
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": oracle.get_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------------- ours --
def main():
    global NAUX, FLOPS
    args = parse()
    NAUX = args.naux
    FLOPS = NAUX * FLOPS_PER_SLAB
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.dropin_child:
        dropin_child(args)
        return
    assert args.warmup >= 3, "at least 3 warm-up steps"
    import torch

    import rest_tensors_gb300 as rt
    from rest_tensors_gb300 import replicas

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    S = args.nslices

    B = rt.synth_ri3ao(args.seed, NB, NAUX)
    C = rt.synth_coef(args.seed, NB)
    Cm = C.view(NB, NB).t()  # Cm[mu, p] (column-major storage)
    D = (Cm[:, :NOCC] @ Cm[:, :NOCC].t()).t().contiguous().view(-1)
    ov = torch.empty(NOCC * NVIR * NAUX, dtype=torch.float64, device=dev)
    K = torch.empty(NB * NB, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()

    def step(form, nsl):
        rt.ri_ov_k(C, B, NB, NAUX, NOCC, NVIR, ov=ov, K=K, form=form, nslices=nsl, stream=stream)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(form, nsl, steps, prof=False):
        barrier()
        n0 = rt.launch_count()
        if prof:
            rt.profile_enable(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(form, nsl)
        e1.record(stream)
        barrier()
        ms = replicas.max_over_ranks(e0.elapsed_time(e1) / steps, dev)
        launches = rt.launch_count() - n0
        return ms, launches

    # ---- float64 reference result and its timing
    step("fp64", 0)
    rt.sync_status()
    ov64, K64 = ov.clone(), K.clone()
    ex64 = rt.exchange_energy(D, K64, NB).item()
    fp64_ms, _ = timed("fp64", 0, args.fp64_steps)
    # The allocation-free float64 entry (fixed 32 MiB scratch, slabs streamed through it), one call.
    rt.ri_ov_k_fp64_noalloc(C, B, NB, NAUX, NOCC, NVIR, ov=ov, K=K, stream=stream)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rt.ri_ov_k_fp64_noalloc(C, B, NB, NAUX, NOCC, NVIR, ov=ov, K=K, stream=stream)
    e1.record(stream)
    barrier()
    noalloc_ms = e0.elapsed_time(e1)
    # Accurate E_x reference: the occupied-occupied block B_ij^P = (C_occ^T B^P C_occ)_ij
    # in float64 (600-term dot products per element), then -sum of squares with a tree sum.
    Coo = torch.cat([C[: NB * NOCC], C[: NB * NOCC]])
    oo, _ = rt.ri_ov_k(Coo, B, NB, NAUX, NOCC, NOCC, form="fp64", want_k=False, stream=stream)
    ex_ref = -float((oo * oo).sum())
    del oo

    def errors():
        ex = rt.exchange_energy(D, K, NB).item()
        return {"ov_max_abs": float((ov - ov64).abs().max()),
                "K_max_rel": float((K - K64).abs().max() / K64.abs().max()),
                "ex_abs": abs(ex - ex64), "ex_rel": abs(ex - ex64) / abs(ex64), "ex_fp64": ex64,
                "ex_abs_vs_oo_ref": abs(ex - ex_ref), "ex_fp64_abs_vs_oo_ref": abs(ex64 - ex_ref),
                "ex_oo_ref": ex_ref}

    sweep = {}
    for s in [int(x) for x in args.sweep.split(",") if x.strip()]:
        for _ in range(2):
            step("split", s)
        ms_s, _ = timed("split", s, max(3, args.steps // 5))
        sweep[str(s)] = {"ms_per_step": ms_s, "tflops": FLOPS / ms_s / 1e9, **errors()}

    # ---- split form: warm-up, then the timed region (clocks sampled meanwhile)
    for _ in range(args.warmup):
        step("split", S)
    rt.sync_status()
    err = errors()
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    gpu_index = int(vis.split(",")[local]) if vis and vis.split(",")[local].strip().isdigit() else local
    sampler = ClockSampler(gpu_index) if rank == 0 else None
    ms, launches = timed("split", S, args.steps, prof=True)
    clocks = sampler.stop() if sampler else None
    g_ms, g_n, g_flops = rt.profile_get(rt.PROF_OZ_GEMM)
    s_ms, s_n, s_bytes = rt.profile_get(rt.PROF_OZ_SLICE)
    rt.profile_enable(False)
    rt.sync_status()

    value = replicas.job_throughput([FLOPS] * world, ms * 1e-3) / 1e12  # TFLOP/s over all ranks
    pk, pk_kind = peaks()
    achieved = g_flops / g_ms / 1e9 if g_ms > 0 else None
    peak = pk.get("bf16_tflops_sustained", FALLBACK_PEAKS["bf16_tflops_sustained"])
    roofline = {"kernel": "oz_gemm_kernel (tcgen05 BF16 digit-pair GEMM)", "bound": "tensor",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved else None,
                # DRAM bytes per step of the three launches, from an ncu capture of the same
                # kernels at naux=256 (1.703 GB), scaled by the slab count.
                "traffic": 1.703e9 * NAUX / 256 if S == 7 else None, "traffic_unit": "bytes per step",
                "peak_source": f"{pk_kind} bf16_tflops_sustained (kernel timed inside a continuous step loop)",
                "launches_per_step": g_n / args.steps, "share_of_step": g_ms / (ms * args.steps),
                "slicing": {"kernel": "emax/slice kernels (HBM)", "achieved_gbs": s_bytes / s_ms / 1e6 if s_ms else None,
                            "peak_gbs": pk.get("hbm_gbs"), "share_of_step": s_ms / (ms * args.steps)}}

    # ---- ri3ao prepared once (REST's SCF loop: ri3fn fixed, orbitals change): per-step time
    # without slicing ri3ao, beside the headline, which slices it every step.
    prepared = None
    if world == 1:
        ov_h, K_h = ov.clone(), K.clone()
        barrier()
        t0 = time.perf_counter()
        prep = rt.Ri3aoPrepared(B, NB, NAUX, nslices=S, stream=stream)
        prep_ms = (time.perf_counter() - t0) * 1e3
        for _ in range(3):
            prep.ri_ov_k(C, NOCC, NVIR, ov=ov, K=K, stream=stream)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            prep.ri_ov_k(C, NOCC, NVIR, ov=ov, K=K, stream=stream)
        e1.record(stream)
        barrier()
        pms = e0.elapsed_time(e1) / args.steps
        prepared = {"ms_per_step": pms, "tflops": FLOPS / pms / 1e9, "prepare_ms_once": prep_ms,
                    "device_bytes_held": prep.nbytes(),
                    "bitwise_equal_to_headline": bool(torch.equal(ov, ov_h) and torch.equal(K, K_h)),
                    "path": "rt_ri3ao_prepare once, then rt_ri_ov_k_prepared per step (no ri3ao slicing per step)"}
        prep.release()
        del ov_h, K_h

    # ---- CPU baseline, and the oracle as checker of both forms' outputs at this workload
    cpu = errors_vs_oracle = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ex_sp = rt.exchange_energy(D, K, NB).item()
        cpu, errors_vs_oracle = cpu_baseline(B, C, {"fp64": (ov64, K64, ex64), "split": (ov, K, ex_sp)})
    del ov64, K64

    # ---- RI-J: two streaming passes over ri3ao (HBM-bound), timed on its own
    w_j = torch.empty(NAUX, dtype=torch.float64, device=dev)
    J_j = torch.empty(NB * NB, dtype=torch.float64, device=dev)
    for _ in range(3):
        rt.ri_j(B, D, NB, NAUX, w=w_j, J=J_j, stream=stream)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(10):
        rt.ri_j(B, D, NB, NAUX, w=w_j, J=J_j, stream=stream)
    e1.record(stream)
    barrier()
    rij_ms = e0.elapsed_time(e1) / 10
    # Bytes moved: two reads of ri3ao (w, then J), D and J; the algorithmic minimum is one read.
    rij_bytes = 2.0 * 8 * NB * NB * NAUX + 8.0 * 3 * NB * NB
    one_read = 8.0 * NB * NB * NAUX + 8.0 * 2 * NB * NB
    hbm = peaks()[0].get("hbm_gbs", FALLBACK_PEAKS["hbm_gbs"])
    # Both passes do one float64 FMA per element of ri3ao: the DFMA rate bounds them.
    rij_flop = 2.0 * 2 * NB * NB * NAUX
    rij = {"ms": rij_ms, "achieved_gbs": rij_bytes / rij_ms / 1e6, "peak_gbs": hbm,
           "frac": rij_bytes / rij_ms / 1e6 / hbm, "bytes": rij_bytes,
           "frac_vs_one_read": one_read / rij_ms / 1e6 / hbm, "one_read_bytes": one_read,
           "dfma": {"bound": "dfma", "flop": rij_flop, "achieved_tflops": rij_flop / rij_ms / 1e9,
                    "peak_tflops": DFMA_TFLOPS, "frac": rij_flop / rij_ms / 1e9 / DFMA_TFLOPS,
                    "peak_source": DFMA_SOURCE},
           "kernels": "rij_w_kernel + rij_j_kernel (float64, two streaming reads of ri3ao)"}
    # The same on symmetric slabs (rt_ri_j_symmetric): upper triangles only, each product once.
    w_s = torch.empty(NAUX, dtype=torch.float64, device=dev)
    J_s = torch.empty(NB * NB, dtype=torch.float64, device=dev)
    for _ in range(3):
        rt.ri_j(B, D, NB, NAUX, w=w_s, J=J_s, stream=stream, symmetric=True)
    barrier()
    e0.record(stream)
    for _ in range(10):
        rt.ri_j(B, D, NB, NAUX, w=w_s, J=J_s, stream=stream, symmetric=True)
    e1.record(stream)
    barrier()
    sym_ms = e0.elapsed_time(e1) / 10
    tri = NB * (NB + 1) / 2.0
    sym_flop, sym_bytes = 2.0 * 2 * tri * NAUX, 2.0 * 8 * tri * NAUX
    rij["symmetric"] = {
        "ms": sym_ms, "speedup_vs_full": rij_ms / sym_ms,
        "achieved_tflops": sym_flop / sym_ms / 1e9, "dfma_frac": sym_flop / sym_ms / 1e9 / DFMA_TFLOPS,
        "achieved_gbs": sym_bytes / sym_ms / 1e6, "hbm_frac": sym_bytes / sym_ms / 1e6 / hbm,
        "w_max_rel_vs_full": float((w_s - w_j).abs().max() / w_j.abs().max()),
        "J_max_rel_vs_full": float((J_s - J_j).abs().max() / J_j.abs().max()),
        "kernels": "rij_w_sym_kernel + rij_j_sym_kernel + rij_j_sym_finish (upper triangles of ri3ao and D)"}
    del w_j, J_j, w_s, J_s

    # ---- end to end through the host-pointer C ABI (pinned host buffers)
    e2e = e2e_full = None
    if args.e2e_steps > 0:
        hB = torch.empty(NB * NB * NAUX, dtype=torch.float64, pin_memory=True)
        hB.copy_(B)
        hC = torch.empty(NB * NB, dtype=torch.float64, pin_memory=True)
        hC.copy_(C)
        hO = torch.empty(NOCC * NVIR * NAUX, dtype=torch.float64, pin_memory=True)
        hK = torch.empty(NB * NB, dtype=torch.float64, pin_memory=True)
        d2h = 8 * (NOCC * NVIR * NAUX + NB * NB)

        def run_host(symmetric):
            # three untimed calls: the first maps the pinned pages for the device and takes 2-3x longer
            for _ in range(3):
                rt.ri_ov_k_host(hC.data_ptr(), hB.data_ptr(), NB, NAUX, NOCC, NVIR, hO.data_ptr(), hK.data_ptr(),
                                form="split", nslices=S, stream=stream, symmetric=symmetric)
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                rt.ri_ov_k_host(hC.data_ptr(), hB.data_ptr(), NB, NAUX, NOCC, NVIR, hO.data_ptr(), hK.data_ptr(),
                                form="split", nslices=S, stream=stream, symmetric=symmetric)
            return replicas.max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, dev)

        # The workload's ri3ao is symmetric in mu, nu: from pinned memory the symmetric
        # entry reads each slab's upper triangle (mu <= nu) over the host link and
        # mirrors it on the device.
        sym_bytes = 8 * NAUX * (NB * (NB + 1) // 2)
        e2e_s = run_host(True)
        e2e = {"value": replicas.job_throughput([FLOPS] * world, e2e_s) / 1e12, "unit": "TFLOP/s",
               "ms_per_step": e2e_s * 1e3, "h2d_bytes_per_step": sym_bytes + 8 * NB * NB, "d2h_bytes_per_step": d2h,
               "path": "rt_ri_ov_k_host_symmetric (C ABI, pinned host buffers, transfers inside the timed region; "
                       "ri3ao slabs symmetric: upper triangles read over the host link, mirrored on the device)"}
        full_s = run_host(False)
        e2e_full = {"value": replicas.job_throughput([FLOPS] * world, full_s) / 1e12, "unit": "TFLOP/s",
                    "ms_per_step": full_s * 1e3, "h2d_bytes_per_step": 8 * (NB * NB * NAUX + NB * NB),
                    "d2h_bytes_per_step": d2h,
                    "path": "rt_ri_ov_k_host (C ABI, pinned host buffers, whole ri3ao read by the SMs over the host link)"}
        del hB

    outputs = None
    if args.outputs:
        outputs = outputs_leg(args, rt, torch, stream, B, C, ov)

    dropin = None
    if args.dropin and world == 1:
        dropin = dropin_ao2mo_leg(args, rt, B, C)

    ri3fn = None
    if args.ri3fn:
        ri3fn = ri3fn_leg(args, rt, torch, stream, B)
        ri3fn["layout"] = layout_leg(args, rt, torch, stream, B)
        ri3fn["newton_schulz"] = newton_schulz_leg(args, rt, torch, stream)

    scf = None
    if args.scf and world == 1:
        scf = scf_lapack_leg(args, rt, torch)

    batched = None
    if args.batch_mols > 0:
        del ov, K
        torch.cuda.empty_cache()
        batched = batched_leg(args, rt, torch, stream)

    large = None
    if args.large:
        del B
        torch.cuda.empty_cache()
        large = large_leg(args, rt, torch, stream)

    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload(), "nbas": NB, "naux": NAUX, "nocc": NOCC, "nvir": NVIR,
                       "form": f"split: {S} BF16 digits per float64, exact FP32 accumulate, int64 recombination",
                       "nslices": S, "l2": f"inputs larger than L2 ({8e-9 * NB * NB * NAUX:.2f} GB ri3ao read per step)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "fp64": {"value": world * FLOPS / fp64_ms / 1e9, "unit": "TFLOP/s", "ms_per_step": fp64_ms,
                     "form": "float64 DFMA tiled GEMM",
                     "noalloc": {"ms": noalloc_ms, "tflops": FLOPS / noalloc_ms / 1e9,
                                 "entry": "rt_ri_ov_k_fp64_noalloc (no device allocation; 32 MiB fixed scratch)"}},
            "speedup_vs_fp64": fp64_ms / ms,
            "errors_vs_fp64": err, "errors_vs_oracle": errors_vs_oracle, "gpu_launches": launches, "clocks": clocks, "roofline": roofline,
            "e2e": e2e, "e2e_full_input": e2e_full, "rij": rij, "cpu_baseline": cpu}
    if sweep:
        line["sweep"] = sweep
    if outputs:
        line["outputs"] = outputs
    if prepared:
        line["prepared_ri3ao"] = prepared
    if dropin:
        line["e2e_dropin_ao2mo"] = dropin
    if scf:
        line["scf_lapack"] = scf
    if ri3fn:
        line["ri3fn"] = ri3fn
    if batched:
        line["batched"] = batched
    if large:
        line["large_system"] = large
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
