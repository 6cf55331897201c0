"""Benchmark of the IZEM RHS hot path on GB300: Mcell-steps/s.

Workload (one "step" = one full time step of the reference driver,
izem.f90:242-389: timestep, then the three SSP-RK3 stages, plus the two
Strang chemistry half-steps when chemistry is on): the temporal H2/air mixing
layer on 256 x 256 x 128 cells, 9 species, WENO5 characteristic fluxes,
EGLIB viscous and diffusive fluxes (--transport fitted: the mixture-averaged
fits), Newton temperature, Strang BDF chemistry, seeded synthetic initial
field (numpy PCG64 seed 20261203).

Printed JSON (one line, rank 0):
  value       device throughput, inputs resident in HBM
  e2e         the same metric through the C ABI with host arrays: every step
              uploads the state from pinned host memory and downloads it back
  roofline    dominant kernel: algorithmic bytes / measured launch time vs the
              measured HBM copy bandwidth; fp64 gives its FP64 rate vs the
              measured FP64 FMA peak of this GPU
  cpu_baseline the C++ restatement of the reference (the oracle) on the host
              cores on a bounded sub-block of the same workload

--impl reference times that CPU restatement alone (the reference is Fortran
and cannot be built here or on the GPU host).
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

HBM_FALLBACK_GBS = 6800.0
FP64_PEAK_FALLBACK_GFLOPS = 1194.4   # FP64 FMA rate of an earlier GB300 measurement, if the live one fails


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", HBM_FALLBACK_GBS)), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def fp64_peak():
    """The FP64 peak of the rooflines: the device's FMA throughput measured
    now (izem_gpu_fp64_rate), or the earlier measurement if that fails."""
    from phd_gb300.izem import fp64_rate
    try:
        r = fp64_rate()
        if r > 0:
            return r, "measured in this run (FP64 FMA-throughput kernel, best of 3)"
    except Exception:
        pass
    return FP64_PEAK_FALLBACK_GFLOPS, "fallback (an earlier FP64 FMA-throughput measurement)"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, idx=0):
        self.idx = idx
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            if len(s) > 8:
                for nm, val in zip(names, s[5:9]):
                    if val.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def build_workload(args):
    from phd_gb300 import ics
    from phd_gb300.izem import metrics_dscalar
    if args.workload == "tgv":
        return ics.tgv(args.n, lib_dscalar=metrics_dscalar)
    return ics.mixing_layer(args.nx, args.ny, args.nz, lib_dscalar=metrics_dscalar)


def euler_face_bytes(cfg):
    """Algorithmic bytes of one x-face-flux launch: each of the nfaces faces
    reads its cell's conserved variables and 8 primitives once (the stencil
    re-reads are cache hits) and writes nv face fluxes."""
    nv = 5 + cfg.nrv
    nf = (cfg.nx + 1) * cfg.ny * cfg.nz
    return nf * (nv * 8 + 8 * 8 + 1 + nv * 8)


def chem_window(cfg):
    """Reactors of one chemistry half step: the reaction_dvode window skips
    ng + 1 cells at every face, and its z bound uses ey
    (module_reaction.f90:155-159)."""
    ng = cfg.ng
    wx = min(cfg.nx, cfg.nx - ng - 1) - ng
    wy = min(cfg.ny, cfg.ny - ng - 1) - ng
    wz = min(cfg.ny, cfg.nz - ng - 1) - ng
    return max(wx, 0) * max(wy, 0) * max(wz, 0)


# one window reactor: reads rho, rho*Y (9) and T, writes rho*Y (9) and T
CHEM_BYTES_PER_REACTOR = 11 * 8 + 10 * 8
# FP64 flops per BDF step of the persistent chemistry kernel with the
# generated right-hand side (2 DFMA + DADD + DMUL per thread, summed by ncu
# over one launch on the 64x64x32 mixing-layer window, 81,225 reactors and
# 243,675 BDF steps, / those steps)
CHEM_FLOP_PER_BDF_STEP = 6712
# DRAM bytes (read + write) per reactor of that launch, scaled by reactors to
# other windows: the per-thread BDF state in local memory that the L2 does
# not hold
CHEM_TRAFFIC_PER_REACTOR = 11071

# FP64 flops per face of k_euler_face (2 DFMA + DADD + DMUL per thread, summed
# by ncu over one launch of the 9-species mixing layer, / faces)
EULER_FLOP_PER_FACE = {9: 1869}


def make_stepper(g, chem, mode=0):
    """The reference main loop's step (phd_gb300.izem.TimeLoop) with per-half-step
    chemistry statistics for the JSON line."""
    from phd_gb300.izem import TimeLoop

    class Stepper(TimeLoop):
        def __init__(self):
            super().__init__(g, chem, chem_mode=mode)
            self.g = g
            self.log = []   # surrogate half steps: (dt, window cells, fallback cells, ms, network ms)
            self.bdf_steps = []   # BDF steps summed over the window, per BDF half step

        def chem(self, dt):
            d = super().chem(dt)
            if self.mode == 0:
                self.bdf_steps.append(self.g.chem_stats()["total_steps"])
            else:
                s = self.g.surrogate_stats()
                self.log.append((dt, s["cells"], s["fallback"], s["ms"], s["ms_network"]))
            return d

    return Stepper()


def run_gpu(args, rank, world):
    from phd_gb300.izem import IzemGPU
    from phd_gb300.mech import h2_mechanism
    cfg, thd, adi, dxi, st, info = build_workload(args)
    chem = args.workload == "mix" and not args.no_chem
    cfg.reaction = 1 if chem else 0
    eg = args.workload == "mix" and args.transport == "eglib"
    cfg.eglib = 1 if eg else 0
    if args.vis_dt:
        cfg.vis_dt = 1
    g = IzemGPU(cfg, thd, adi)
    if eg:
        from phd_gb300.thd import eglib_link, load_species
        g.set_eglib(eglib_link(load_species("h2air9")))
    g.set_grid(*dxi)
    g.upload(**st)
    g.finalize_ic()
    if chem:
        g.set_mechanism(h2_mechanism())
    options = {}
    if args.les is not None:
        g.set_les(mu_sgs_factor=args.les)
        options["les"] = "Smagorinsky under EGLIB, MU_SGS_FACTOR %g" % args.les
    if args.dvodesimp and chem:
        from phd_gb300.thd import load_species
        names = load_species("h2air9")["names"]
        ih2, in2 = names.index("H2"), names.index("N2")
        yf = np.zeros(9); yf[ih2] = 0.5; yf[in2] = 0.5                               # the fuel stream
        yo = np.zeros(9); yo[names.index("O2")] = 0.233; yo[in2] = 0.767             # the air stream
        g.set_chem_skip(yf, yo, ih2, in2)
        options["dvodesimp"] = "chemistry skipped in the pure streams and where rates are negligible"
    if args.vis_dt:
        options["vis_dt"] = "Fourier time-step criteria"
    stp = make_stepper(g, chem)
    ncell = cfg.nx * cfg.ny * cfg.nz
    # warm-up, then the thread blocks of the dominant kernels chosen by timing
    # them on this state (the CUDA graph of RK3 is captured afterwards)
    for _ in range(args.warmup):
        stp.step()
    _, dt_tune = g.timestep(DTmax=stp.DTmax, dtmin=stp.dtmin)
    tuning = g.autotune(chem_dt=0.5 * dt_tune if chem and args.chem_variant is None else 0.0)
    if chem and args.chem_variant is not None:
        g.set_chem_variant(args.chem_variant)
        tuning["chem_psr"] = {"chosen": "variant %d (pinned)" % args.chem_variant}
    stp.step()
    g.synchronize()
    g.newton_stats(reset=True)
    barrier(world)
    # timed steps without per-kernel events: `value`
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        g.timer_start()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            stp.step()
        ms = g.timer_stop()
        wall = time.perf_counter() - t0
    # the same number of steps again with an event pair around every launch:
    # the per-kernel split, launch count and the rooflines
    g.set_kernel_timing(True)
    stp.bdf_steps.clear()
    g.timer_start()
    for _ in range(args.steps):
        stp.step()
    ms_instr = g.timer_stop()
    timed_bdf = list(stp.bdf_steps)
    newton_it, newton_unconv = g.newton_stats()
    kt = g.kernel_times()
    g.set_kernel_timing(False)
    ms = max_over_ranks(ms, world)
    value = world * ncell * args.steps / (ms * 1e-3) / 1e6
    # ---- end-to-end through the C ABI with host (pinned) arrays
    host = g.download()
    e2e_steps = max(1, min(args.steps, 3))
    pinned = {k: pin(a) for k, a in host.items()}
    pinned_out = {k: pin(a) for k, a in host.items()}   # results read back into pinned memory
    h2d = sum(a.nbytes for a in pinned.values())
    g.synchronize()
    t_copy = 0.0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        g.upload(**pinned)
        tb = time.perf_counter()
        stp.step()
        tc = time.perf_counter()
        out = g.download(out=pinned_out)
        t_copy += (tb - ta) + (time.perf_counter() - tc)
    e2e_s = time.perf_counter() - t0
    d2h = sum(a.nbytes for a in out.values())
    e2e_value = world * ncell * e2e_steps / e2e_s / 1e6
    # ---- roofline of the dominant kernel
    hbm, hbm_src = measured_peaks()
    f64, f64_src = fp64_peak()
    dom = max(kt.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_n, dom_ms) = dom
    fx = kt.get("euler_face_x", (0, 0.0))
    rl = rl_chem = None
    nre = chem_window(cfg) if chem else 0
    if chem and kt.get("chem_psr", (0, 0.0))[0]:
        n_l, ms_l = kt["chem_psr"]
        avg_s = ms_l / n_l * 1e-3
        byts = nre * CHEM_BYTES_PER_REACTOR
        rl_chem = {"bound": "hbm", "kernel": "k_psr_field (persistent BDF chemistry, dominant)",
                   "achieved": byts / avg_s / 1e9, "peak": hbm, "unit": "GB/s", "frac": byts / avg_s / 1e9 / hbm,
                   "traffic": CHEM_TRAFFIC_PER_REACTOR * nre if CHEM_TRAFFIC_PER_REACTOR else None,
                   "peak_source": hbm_src + " (MEASURED_PEAKS.json hbm_gbs)",
                   "reactors_per_launch": nre, "bdf_steps_per_launch": timed_bdf}
        if CHEM_FLOP_PER_BDF_STEP and timed_bdf:
            gf = CHEM_FLOP_PER_BDF_STEP * sum(timed_bdf) / (ms_l * 1e-3) / 1e9
            rl_chem["fp64"] = {"achieved": gf, "peak": f64, "unit": "GFLOP/s", "frac": gf / f64,
                               "peak_source": f64_src}
    if fx[0]:
        avg_s = fx[1] / fx[0] * 1e-3
        byts = euler_face_bytes(cfg)
        nf = (cfg.nx + 1) * cfg.ny * cfg.nz
        rl = {"bound": "hbm", "kernel": "k_euler_face (x sweep)", "achieved": byts / avg_s / 1e9, "peak": hbm,
              "unit": "GB/s", "frac": byts / avg_s / 1e9 / hbm, "traffic": TRAFFIC_PER_LAUNCH.get(args.workload),
              "peak_source": hbm_src + " (MEASURED_PEAKS.json hbm_gbs)"}
        if cfg.nrv in EULER_FLOP_PER_FACE:
            flops = nf * EULER_FLOP_PER_FACE[cfg.nrv]
            rl["fp64"] = {"achieved": flops / avg_s / 1e9, "peak": f64, "unit": "GFLOP/s",
                          "frac": flops / avg_s / 1e9 / f64, "peak_source": f64_src}
    launches = sum(n for n, _ in kt.values())
    mlp = run_mlp_chem(args, g, stp, ncell, world) if chem and not args.no_mlp else None
    res = {
        "metric": "reacting RHS Mcell-steps/s, FP64 plain vs MLP-chem (<=1% dT err) on 1 GB300",
        "value": value, "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64 %d)" % info.get("seed", 0),
        "config": {"workload": info["name"] + workload_note(chem, eg), "cells": ncell,
                   "nv": 5 + cfg.nrv,
                   "transport": "EGLIB precision 1 (EGSE2, EGSLCT2, EGSDR1)" if eg else "fitted mixture-averaged (tranfit)",
                   "chemistry": ("Strang: 2 x BDF (DVODE MF=22) half-steps per step, 9 species / 12 reactions"
                                 if chem else "off"),
                   "chem_rhs": (("generated for the mechanism" if g.lib.izem_gpu_chem_generated() else
                                 "mechanism tables") if chem else None),
                   "l2": "inputs larger than L2 (state %.2f GB)" % (host["v"].nbytes / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "autotuned_threads_per_block": {k: v["chosen"] for k, v in tuning.items()},
                   **({"options": options} if options else {})},
        "e2e": {"value": e2e_value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "ms_per_step": e2e_s * 1e3 / e2e_steps,
                "copy_ms_per_step": t_copy * 1e3 / e2e_steps},
        "roofline": rl_chem if rl_chem else rl,
        "roofline_euler_face": rl if rl_chem else None,
        "dominant_kernel": {"name": dom_name, "launches": dom_n, "ms": dom_ms},
        "instrumented_ms_per_step": ms_instr / args.steps,
        "newton": {"max_iterations": newton_it, "unconverged_solves": newton_unconv, "itmax": 200,
                   "note": "prim_inv_var solves of the timed steps; each iterates until the reference's "
                           "stopping test holds or itmax"},
        "kernel_ms": {k: round(v[1], 3) for k, v in sorted(kt.items(), key=lambda kv: -kv[1][1])},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if mlp is not None:
        res["mlp_chem"] = mlp
    g.close()
    return res


def run_mlp_chem(args, g, stp, ncell, world):
    """The same reacting step with the learned chemistry (IZEM_CHEM_MLP).
    Two networks are trained on the GPU on 2^20 of the flow's own window
    reactors (half step scaled by 10**U[-0.05, 0.05]; three quarters of them
    first advanced by the FP64 integrator over up to 16 half steps, so the
    set covers the radical growth of the following steps), labelled by the
    FP64 BDF integrator; they learn the increment minus the explicit one,
    dt f(y0), which the gated step adds back.  The gate's tolerance scale is calibrated on 2^17
    held-out window reactors for a 0.8 % error target; rejected cells go to
    BDF.  Accuracy: after the timed steps, the same steps are replayed from
    the same state, and every chemistry half step is also integrated by BDF
    from the state the surrogate step starts from; the |dT| error over the
    window is reported against the largest BDF increment of that half step."""
    from phd_gb300.izem import TimeLoop
    from phd_gb300.mech import h2_mechanism
    from phd_gb300.surrogate import calibrate_flow_gate, flow_reactors, label, train_on
    mech = h2_mechanism()
    _, dt = g.timestep(DTmax=stp.DTmax, dtmin=stp.dtmin)
    age = 16.0
    t0 = time.perf_counter()
    X, Yt, E = label(mech, *flow_reactors(g, mech, 0.5 * dt, n_max=1 << 20, spread=0.05, seed=5, age=age),
                     explicit=True)
    held = flow_reactors(g, mech, 0.5 * dt, n_max=1 << 17, spread=0.05, seed=6, age=age)
    t_label = time.perf_counter() - t0
    t0 = time.perf_counter()
    epochs = 60
    nets = train_on(X, Yt, epochs=epochs, batch=4096, E=E)
    t_train = time.perf_counter() - t0
    gate, calib = calibrate_flow_gate(nets, mech, X, Yt, held, target=0.008)
    g.set_surrogate(nets[0], nets[1], gate=gate)
    mstp = make_stepper(g, True, mode=1)
    mstp.dtmin, mstp.DTmax = stp.dtmin, stp.DTmax
    mstp.step()
    g.synchronize()
    st_timed = g.download()
    loop0 = (mstp.dtmin, mstp.DTmax, mstp.time)
    barrier(world)
    steps = max(1, args.steps)
    mstp.log.clear()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        g.timer_start()
        for _ in range(steps):
            mstp.step()
        ms = g.timer_stop()
    ms = max_over_ranks(ms, world)
    lg = np.array(mstp.log, dtype=np.float64).reshape(-1, 5)

    # accuracy replay of the timed steps
    class Checked(TimeLoop):
        def __init__(self):
            super().__init__(g, True, chem_mode=1)
            self.rows = []

        def chem(self, dt_half):
            s0 = g.download()
            T0 = s0["T"].copy()
            g.reaction_selec(dt_half, mode=0)
            dref = (g.download()["T"] - T0) * g.adi.t_ref
            g.upload(**s0)
            d = g.reaction_selec(dt_half, mode=1)
            sst = g.surrogate_stats()
            dgot = (g.download()["T"] - T0) * g.adi.t_ref
            err = np.abs(dgot - dref)
            scale = float(np.abs(dref).max())
            self.rows.append({"max_dT_K": scale, "max_err_frac": float(err.max()) / scale if scale > 0 else None,
                              "rms_err_frac": float(np.sqrt((err ** 2).mean())) / scale if scale > 0 else None,
                              "fallback_frac": sst["fallback"] / max(1, sst["cells"])})
            return d

    g.upload(**st_timed)
    chk = Checked()
    chk.dtmin, chk.DTmax, chk.time = loop0
    for _ in range(steps):
        chk.step()
    errs = [r["max_err_frac"] for r in chk.rows if r["max_err_frac"] is not None]
    return {"value": world * ncell * steps / (ms * 1e-3) / 1e6, "unit": "Mcell-steps/s", "steps": steps,
            "ms_per_step": ms / steps,
            "timed_half_steps": {"n": int(len(lg)),
                                 "fallback_frac": (lg[:, 2] / np.maximum(lg[:, 1], 1)).round(4).tolist(),
                                 "ms": lg[:, 3].round(2).tolist(),
                                 "network_ms": lg[:, 4].round(2).tolist()},
            "accuracy_replay": {"half_steps": chk.rows, "max_err_frac_over_states": max(errs) if errs else None},
            "training": {"samples": int(len(X)), "networks": 2, "epochs": epochs, "aged_half_steps_max": age,
                         "target": "increment minus dt f(y0)",
                         "label_s": t_label, "train_s": t_train},
            "gate": gate_json(gate), "gate_calibration": calib, "clocks": clk.summary()}


def run_batch(args):
    """Batched stiff chemistry: args.cells independent constant-volume H2/air
    reactors (T ~ U[800,2400] K, p ~ U[1,10] atm, phi ~ U[0.3,3], progress
    c ~ U[0,1], dt log-uniform in [1e-8,1e-6] s), one BDF integration per cell
    per step, arrays resident on the device; e2e adds the host copies."""
    import torch
    from phd_gb300 import ics
    from phd_gb300.izem import chem_autotune_device, psr_batch_device, psr_batch
    from phd_gb300.mech import h2_mechanism
    mech = h2_mechanism()
    n = args.cells
    T, rho, Y, dt = ics.batched_reactors(n)
    dev = {k: torch.from_numpy(a).to("cuda:0") for k, a in (("T", T), ("rho", rho), ("Y", Y), ("dt", dt))}
    T0, Y0 = dev["T"].clone(), dev["Y"].clone()
    tuning = chem_autotune_device(mech, n, dev["T"], dev["rho"], dev["Y"], dev["dt"])
    ist = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    nst = torch.zeros(n, dtype=torch.int32, device="cuda:0")

    def step():
        dev["T"].copy_(T0)
        dev["Y"].copy_(Y0)
        torch.cuda.synchronize()
        return psr_batch_device(mech, n, dev["T"], dev["rho"], dev["Y"], dev["dt"], ist, nst)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        kms = [step() for _ in range(args.steps)]
        torch.cuda.synchronize()
    ms = float(np.sum(kms))
    steps_per_cell = nst.double().mean().item()
    t0 = time.perf_counter()
    Th, Yh = T.copy(), Y.copy()
    psr_batch(mech, Th, rho.copy(), Yh, dt.copy())
    e2e_s = time.perf_counter() - t0
    bytes_cell = 8 * (2 * 9 + 3) + 8 * (9 + 1)
    return {
        "metric": "batched stiff chemistry Mcells/s (FP64 BDF, DVODE MF=22, 9 species / 12 reactions)",
        "value": n * args.steps / (ms * 1e-3) / 1e6, "unit": "Mcells/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64 20261203)",
        "config": {"workload": "independent H2/air reactors", "cells": n, "mean_bdf_steps": steps_per_cell,
                   "autotuned_kernel_variant": tuning,
                   "max_bdf_steps": int(nst.max().item()), "l2": "inputs larger than L2" if n * bytes_cell > 129e6
                   else "inputs smaller than L2 (%d B)" % (n * bytes_cell)},
        "e2e": {"value": n / e2e_s / 1e6, "unit": "Mcells/s", "h2d_bytes_per_step": n * 8 * 12,
                "d2h_bytes_per_step": n * 8 * 10},
        "gpu_launches": args.steps, "clocks": clk.summary(),
    }


def run_surrogate(args):
    """Learned chemistry on independent reactors: two networks trained on the
    GPU on args.train reactors of the batched-chemistry distribution
    (labelled by the FP64 BDF integrator), then the gated surrogate step --
    tensor-core inference, error gate, BDF on the rejected cells -- on
    args.cells reactors of the same distribution drawn with another seed,
    against the BDF step on all of them.  Arrays resident on the device."""
    import torch
    from phd_gb300 import ics
    from phd_gb300.izem import chem_autotune_device, psr_batch_device
    from phd_gb300.mech import h2_mechanism
    from phd_gb300.surrogate import DEFAULT_GATE, STRICT_GATE, calibrate_cap, train_ensemble
    gate = STRICT_GATE if args.gate == "strict" else DEFAULT_GATE
    mech = h2_mechanism()
    t0 = time.perf_counter()
    nets = train_ensemble(mech, n=args.train, seed=31, epochs=args.epochs)
    t_train = time.perf_counter() - t0
    calib = None
    if args.gate == "calibrated":   # the dT cap chosen on 2^20 held-out labelled reactors
        gate, calib = calibrate_cap(nets, mech, DEFAULT_GATE)
    n = args.cells
    T = torch.empty(n, dtype=torch.float64, device="cuda:0")
    rho, dt = torch.empty_like(T), torch.empty_like(T)
    Y = torch.empty((n, 9), dtype=torch.float64, device="cuda:0")
    chunk = 1 << 22
    for c0 in range(0, n, chunk):
        c1 = min(n, c0 + chunk)
        Tc, rc, Yc, dc = ics.batched_reactors(c1 - c0, seed=20270101 + c0 // chunk)
        T[c0:c1].copy_(torch.from_numpy(Tc))
        rho[c0:c1].copy_(torch.from_numpy(rc))
        Y[c0:c1].copy_(torch.from_numpy(Yc))
        dt[c0:c1].copy_(torch.from_numpy(dc))
    T0, Y0 = T.clone(), Y.clone()

    def reset():
        T.copy_(T0)
        Y.copy_(Y0)
        torch.cuda.synchronize()

    tuning = chem_autotune_device(mech, n, T, rho, Y, dt)
    reset()
    psr_batch_device(mech, n, T, rho, Y, dt)   # warm-up, and the FP64 reference increments
    dT_ref_d = T - T0
    dT_ref = dT_ref_d.cpu().numpy()
    reset()
    bdf_ms = psr_batch_device(mech, n, T, rho, Y, dt)
    for _ in range(args.warmup):
        reset()
        nets[0].chem_step_device(mech, n, T, rho, Y, dt, gate, partner=nets[1])
    runs = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            reset()
            runs.append(nets[0].chem_step_device(mech, n, T, rho, Y, dt, gate, partner=nets[1]))
    err = np.abs((T - T0).cpu().numpy() - dT_ref)
    scale = float(np.abs(dT_ref).max())
    # accepted cells (not in the last step's fallback list) against their
    # temperature increment
    dgot = T - T0
    err_d = (dgot - dT_ref_d).abs()
    acc = torch.ones(n, dtype=torch.bool, device="cuda:0")
    acc[torch.from_numpy(nets[0].fallback_cells().astype(np.int64)).to("cuda:0")] = False
    # per-cell error of the accepted cells relative to their own FP64
    # increment, over the cells whose increment is at least 1 K and 10 K
    ref_abs = dT_ref_d.abs()
    rel_own = {}
    for thr in (1.0, 10.0):
        sel = acc & (ref_abs >= thr)
        rel = (err_d[sel] / ref_abs[sel]).cpu().numpy()
        rel_own["dT_ref_ge_%gK" % thr] = {
            "cells_frac": float(sel.sum().item()) / n,
            "median": float(np.median(rel)) if rel.size else None,
            "p99": float(np.percentile(rel, 99)) if rel.size else None,
            "max": float(rel.max()) if rel.size else None}
    by_dT = []
    for cap in (5.0, 10.0, 20.0, 50.0, 100.0, 200.0, 400.0, 800.0):
        keep = acc & (dgot.abs() <= cap)
        by_dT.append({"accepted_dT_le_K": cap, "cells_above_frac": float((acc & ~keep).sum().item()) / n,
                      "max_err_K": float(err_d[keep].max().item()) if bool(keep.any()) else 0.0})
    ms = float(np.mean([r["ms"] for r in runs]))
    ms_net = float(np.mean([r["ms_mlp"] for r in runs]))
    flop = 2.0 * 2 * 202240 * n     # two networks, 202,240 MACs per row
    tflops = flop / (ms_net * 1e-3) / 1e12
    peak = 1932.2
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peak = float(json.load(f).get("bf16_tflops", peak))
    return {
        "metric": "learned-chemistry step Mcells/s (gated BF16 tensor-core MLP + FP64 BDF fallback)",
        "value": n / (ms * 1e-3) / 1e6, "unit": "Mcells/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 network, f64 integrator", "data": "synthetic (seeded PCG64)",
        "config": {"workload": "independent H2/air reactors (batched-chemistry distribution)", "cells": n,
                   "training": {"samples": args.train, "epochs": args.epochs, "networks": 2, "seconds": t_train},
                   "gate": {"name": args.gate, "values": gate_json(gate), "calibration": calib},
                   "autotuned_kernel_variant": tuning,
                   "l2": "inputs larger than L2"},
        "bdf": {"value": n / (bdf_ms * 1e-3) / 1e6, "unit": "Mcells/s", "ms": bdf_ms},
        "speedup_vs_bdf": bdf_ms / ms,
        "fallback_frac": float(np.mean([r["fallback"] for r in runs])) / n,
        "max_dT_err_K": float(err.max()), "max_dT_K": scale, "max_dT_err_frac": float(err.max()) / scale,
        "rms_dT_err_K": float(np.sqrt((err ** 2).mean())),
        "accepted_cells": int(acc.sum().item()), "error_by_accepted_dT": by_dT,
        "accepted_err_rel_to_own_dT": rel_own,
        "roofline": {"bound": "tensor", "kernel": "k_mlp_tc (two networks, with the feature kernel)",
                     "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                     "traffic": None, "network_ms": ms_net},
        # per 2^20-reactor chunk: 2 feature kernels, 2 tensor-core networks, the gate; one BDF fallback launch
        "gpu_launches": args.steps * (5 * ((n + (1 << 20) - 1) >> 20) + 1), "clocks": clk.summary(),
    }


def run_field_surrogate(args, steps=None, warmup=None):
    """Learned chemistry on a reacting field: two networks trained on the GPU
    on args.train reactors of the batched-chemistry distribution (labelled
    by the FP64 BDF integrator), the gate's dT cap and absolute dT
    tolerances calibrated on 2^20 held-out ones taken over the field's step
    (surrogate.calibrate_cap), then inference on a
    512 x 256 x 256 field
    (phd_gb300.ics.reacting_field: the same distribution laid out as smooth
    seeded fields, one chemistry step of args.field_dt seconds, by default
    3e-7 s) through the library's
    field chemistry step (reaction_selec, IZEM_CHEM_MLP: tensor-core
    networks, error gate, BDF on the rejected cells), against the same step
    with BDF on every cell (IZEM_CHEM_BDF).  State resident on the device;
    each timed step starts from the same state (re-uploaded outside the
    timed region)."""
    from phd_gb300 import ics
    from phd_gb300.izem import IzemGPU, chem_autotune_device, metrics_dscalar
    from phd_gb300.mech import h2_mechanism
    from phd_gb300.surrogate import (ABS_SCALE_LADDER, CAP_LADDER_FINE, DEFAULT_GATE, STRICT_GATE, calibrate_cap,
                                     reaction_window, train_ensemble)
    import torch
    steps = steps if steps is not None else args.steps
    warmup = warmup if warmup is not None else args.warmup
    gate = STRICT_GATE if args.gate == "strict" else DEFAULT_GATE
    mech = h2_mechanism()
    t0 = time.perf_counter()
    nets = train_ensemble(mech, n=args.train, seed=31, epochs=args.epochs)
    t_train = time.perf_counter() - t0
    calib = None
    if args.gate == "calibrated":   # the dT cap for this field's step, on 2^20 held-out reactors over it
        gate, calib = calibrate_cap(nets, mech, DEFAULT_GATE, dt_s=args.field_dt, caps=CAP_LADDER_FINE,
                                    abs_scales=ABS_SCALE_LADDER)
    t0 = time.perf_counter()
    nx, ny, nz = args.field_size
    cfg, thd, adi, dxi, st, info = ics.reacting_field(nx, ny, nz, dt_s=args.field_dt, lib_dscalar=metrics_dscalar)
    t_ic = time.perf_counter() - t0
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st)
    del st
    g.finalize_ic()
    g.set_mechanism(mech)
    dt = info["dt_s"] / info["time_ref"]
    st0 = g.download()
    nrv = cfg.nrv
    win = reaction_window(cfg)
    # the register-budget variant of the chemistry kernels, tuned on 2^20 window reactors
    vw = st0["v"][win]
    Tw = st0["T"][win] * adi.t_ref
    nsamp = min(1 << 20, Tw.size)
    pick = np.random.Generator(np.random.PCG64(17)).choice(Tw.size, nsamp, replace=False)
    rho_s = vw[..., 0].reshape(-1)[pick] * adi.rho_ref * 1e-3
    Y_s = np.stack([vw[..., 5 + k].reshape(-1)[pick] for k in range(nrv)], axis=1) / (rho_s / (adi.rho_ref * 1e-3))[:, None]
    dev = [torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")
           for a in (Tw.reshape(-1)[pick], rho_s, Y_s, np.full(nsamp, info["dt_s"]))]
    tuning = chem_autotune_device(mech, nsamp, *dev)
    del vw, dev
    T0 = st0["T"][win].copy()
    # BDF on every window cell (the FP64 reference increments)
    g.synchronize()
    g.timer_start()
    g.reaction_selec(dt, mode=0)
    bdf_ms = g.timer_stop()
    bdf_stats = g.chem_stats()
    dT_ref = (g.download()["T"][win] - T0) * adi.t_ref
    g.set_surrogate(nets[0], nets[1], gate=gate)
    for _ in range(warmup):
        g.upload(**st0)
        g.reaction_selec(dt, mode=1)
    runs = []
    with ClockSampler(0) as clk:
        for _ in range(steps):
            g.upload(**st0)
            g.synchronize()
            g.timer_start()
            g.reaction_selec(dt, mode=1)
            ms = g.timer_stop()
            sst = g.surrogate_stats()
            runs.append({"ms": ms, "fallback": sst["fallback"], "cells": sst["cells"], "ms_network": sst["ms_network"]})
    dT = (g.download()["T"][win] - T0) * adi.t_ref
    g.close()
    err = np.abs(dT - dT_ref)
    scale = float(np.abs(dT_ref).max())
    ref_abs = np.abs(dT_ref)
    rel_own = {}
    for thr in (1.0, 10.0):
        sel = ref_abs >= thr
        rel = err[sel] / ref_abs[sel]
        rel_own["dT_ref_ge_%gK" % thr] = {
            "cells_frac": float(sel.mean()),
            "median": float(np.median(rel)) if rel.size else None,
            "p99": float(np.percentile(rel, 99)) if rel.size else None,
            "max": float(rel.max()) if rel.size else None}
    ncell = int(T0.size)
    ms = float(np.mean([r["ms"] for r in runs]))
    ms_net = float(np.mean([r["ms_network"] for r in runs]))
    flop = 2.0 * 2 * 202240 * ncell     # two networks, 202,240 MACs per row
    tflops = flop / (ms_net * 1e-3) / 1e12 if ms_net > 0 else None
    peak = 1932.2
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peak = float(json.load(f).get("bf16_tflops", peak))
    return {
        "metric": "learned-chemistry field step Mcells/s (gated BF16 tensor-core MLP + FP64 BDF fallback)",
        "value": ncell / (ms * 1e-3) / 1e6, "unit": "Mcells/s", "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network, f64 integrator", "data": "synthetic (seeded PCG64)",
        "config": {"workload": info["name"], "grid": [nx, ny, nz], "window_cells": ncell, "dt_s": info["dt_s"],
                   "training": {"samples": args.train, "epochs": args.epochs, "networks": 2, "seconds": t_train,
                                "distribution": "independent reactors of the batched-chemistry distribution"},
                   "gate": {"name": args.gate, "values": gate_json(gate), "calibration": calib},
                   "autotuned_kernel_variant": tuning, "initial_field_s": t_ic,
                   "l2": "inputs larger than L2"},
        "bdf": {"value": ncell / (bdf_ms * 1e-3) / 1e6, "unit": "Mcells/s", "ms": bdf_ms, "stats": bdf_stats},
        "speedup_vs_bdf": bdf_ms / ms,
        "fallback_frac": float(np.mean([r["fallback"] / max(1, r["cells"]) for r in runs])),
        "max_dT_err_K": float(err.max()), "max_dT_K": scale,
        "max_dT_err_frac": float(err.max()) / scale if scale > 0 else None,
        "rms_dT_err_K": float(np.sqrt((err ** 2).mean())),
        "err_rel_to_own_dT": rel_own,
        "roofline": {"bound": "tensor", "kernel": "k_mlp_tc (two networks, with the feature kernel)",
                     "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": tflops / peak if tflops else None, "traffic": None, "network_ms": ms_net},
        "clocks": clk.summary(),
    }


def run_jet(args, steps=None, warmup=None):
    """The reacting LES jet: the 512 x 512 x 256 planar H2/air jet
    (phd_gb300.ics.jet_les: 2 mm slot of H2/N2 at 300 m/s into 1200 K air
    at 10 m/s, 1 atm, 2 % seeded fluctuations at the inflow and in the
    initial field), WENO5 + EGLIB viscous fluxes with the Smagorinsky
    closure (MU_SGS_FACTOR 0.17), RK3 stages captured in a CUDA graph, the
    jet faces, Strang chemistry.  `steps` driver steps are timed with BDF on
    every cell, then the same number from the same state with the learned
    chemistry: two networks trained on 2^20 of the jet's own window
    reactors (aged by the integrator over up to 16 half steps, half steps
    scaled by 10**U[-0.3, 0.3]; the networks
    learn the increment minus dt f(y0)), then retrained with 2^19 more
    reactors that the gated surrogate itself advanced over one or two half
    steps (labelled by BDF), the gate calibrated on 2^17 held-out ones for a
    0.8 % error target, rejected cells by BDF."""
    from phd_gb300 import ics
    from phd_gb300.izem import IzemGPU, metrics_dscalar
    from phd_gb300.mech import h2_mechanism
    from phd_gb300.surrogate import calibrate_flow_gate, flow_reactors, label, train_on
    from phd_gb300.thd import eglib_link, load_species
    steps = steps if steps is not None else args.steps
    warmup = warmup if warmup is not None else args.warmup
    t0 = time.perf_counter()
    nx, ny, nz = args.jet_size
    cfg, thd, adi, dxi, st, info = ics.jet_les(nx, ny, nz, lib_dscalar=metrics_dscalar)
    t_ic = time.perf_counter() - t0
    cfg.eglib, cfg.reaction = 1, 1
    mech = h2_mechanism()
    g = IzemGPU(cfg, thd, adi)
    g.set_eglib(eglib_link(load_species("h2air9")))
    g.set_grid(*dxi)
    g.upload(**st)
    del st
    g.set_coords(*info["coords"], info["lx"])
    g.set_jet(info["jet"])
    g.set_les(mu_sgs_factor=0.17)
    g.finalize_ic()
    g.set_mechanism(mech)
    ncell = nx * ny * nz
    stp = make_stepper(g, True)
    for _ in range(warmup):
        stp.step()
    g.synchronize()
    st0 = g.download()
    loop0 = (stp.dtmin, stp.DTmax, stp.time)
    g.newton_stats(reset=True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        g.timer_start()
        for _ in range(steps):
            stp.step()
        ms_bdf = g.timer_stop()
    newton = g.newton_stats()
    # the learned chemistry from the same state
    g.upload(**st0)
    _, dt = g.timestep(DTmax=loop0[1], dtmin=loop0[0])
    t0 = time.perf_counter()
    # the jet's time step drifts as the flow develops: half steps within a
    # factor 2 of the current one
    X, Yt, E = label(mech, *flow_reactors(g, mech, 0.5 * dt, n_max=1 << 20, spread=0.3, seed=5, age=16.0),
                     explicit=True)
    held = flow_reactors(g, mech, 0.5 * dt, n_max=1 << 17, spread=0.3, seed=6, age=16.0)
    nets = train_on(X, Yt, epochs=42, batch=4096, E=E)
    gate, calib = calibrate_flow_gate(nets, mech, X, Yt, held, target=0.008)
    # one more round on the states the gated surrogate itself produces: 2^19
    # other window reactors advanced by it over one half step (and half of
    # them over a second), labelled by BDF and added to the training set
    R = flow_reactors(g, mech, 0.5 * dt, n_max=1 << 19, spread=0.3, seed=7, age=16.0)
    T1, rho1, Y1, dt1 = [np.ascontiguousarray(a.copy()) for a in R]
    nets[0].chem_step(mech, T1, rho1, Y1, dt1, gate, partner=nets[1])
    h = len(T1) // 2
    T2, rho2, Y2, dt2 = [np.ascontiguousarray(a[h:].copy()) for a in (T1, rho1, Y1, dt1)]
    nets[0].chem_step(mech, T2, rho2, Y2, dt2, gate, partner=nets[1])
    Xa, Yta, Ea = label(mech, np.concatenate([T1[:h], T2]), np.concatenate([rho1[:h], rho2]),
                        np.ascontiguousarray(np.concatenate([Y1[:h], Y2])), np.concatenate([dt1[:h], dt2]),
                        explicit=True)
    X, Yt, E = np.concatenate([X, Xa]), np.concatenate([Yt, Yta]), np.concatenate([E, Ea])
    nets = train_on(X, Yt, epochs=42, batch=4096, E=E)
    gate, calib = calibrate_flow_gate(nets, mech, X, Yt, held, target=0.008)
    t_train = time.perf_counter() - t0
    g.set_surrogate(nets[0], nets[1], gate=gate)
    g.upload(**st0)
    mstp = make_stepper(g, True, mode=1)
    mstp.dtmin, mstp.DTmax, mstp.time = loop0
    g.timer_start()
    for _ in range(steps):
        mstp.step()
    ms_mlp = g.timer_stop()
    lg = np.array(mstp.log, dtype=np.float64).reshape(-1, 5)
    g.close()
    return {"metric": "reacting LES jet Mcell-steps/s (learned chemistry with FP64 fallback; BDF beside it)",
            "value": ncell * steps / (ms_mlp * 1e-3) / 1e6, "unit": "Mcell-steps/s", "steps": steps,
            "warmup": warmup, "ms_per_step": ms_mlp / steps,
            "bdf": {"value": ncell * steps / (ms_bdf * 1e-3) / 1e6, "ms_per_step": ms_bdf / steps,
                    "clocks": clk.summary(), "newton": {"max_iterations": newton[0], "unconverged_solves": newton[1]}},
            "surrogate_half_steps": {"fallback_frac": (lg[:, 2] / np.maximum(lg[:, 1], 1)).round(4).tolist(),
                                     "dt_over_trained": (lg[:, 0] / (0.5 * dt)).round(4).tolist(),
                                     "ms": lg[:, 3].round(2).tolist(), "network_ms": lg[:, 4].round(2).tolist()},
            "gate_calibration": calib, "training_s": t_train, "initial_field_s": t_ic,
            "config": {"workload": info["name"] + " (WENO5 + EGLIB + Smagorinsky 0.17 + RK3 graph + Strang chemistry)",
                       "cells": ncell, "grid_m": info["dx_m"], "jet_width_m": info["width_m"],
                       "note": "timed steps are a sample of the 100-step run; throughput is per step"}}


def c4_summary(args):
    """The learned-chemistry workload on the 512 x 256 x 256 reacting field
    (--workload field) at its configured size -- two networks trained on
    4 M reactors of the batched-chemistry distribution labelled by the FP64
    integrator, calibrated gate -- condensed for the default line: speed-up
    over BDF on every cell, fallback, errors."""
    import copy
    a = copy.copy(args)
    a.train, a.epochs, a.gate = 1 << 22, 24, "calibrated"
    a.field_size, a.field_dt = [512, 256, 256], 3e-7
    r = run_field_surrogate(a, steps=max(1, min(args.steps, 3)), warmup=1)
    keys = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "bdf", "speedup_vs_bdf", "fallback_frac",
            "max_dT_err_K", "max_dT_K", "max_dT_err_frac", "rms_dT_err_K", "err_rel_to_own_dT", "roofline", "clocks")
    out = {k: r[k] for k in keys}
    c = r["config"]
    out["config"] = {"workload": c["workload"], "window_cells": c["window_cells"], "dt_s": c["dt_s"],
                     "training": c["training"], "gate": c["gate"]["values"]}
    return out


def gate_json(gate):
    """Gate values for the JSON line: an infinite dT cap (no cap) as null."""
    return [float(x) if np.isfinite(x) else None for x in gate]


def workload_note(chem, eg):
    return " (WENO5 + %s viscous fluxes + RK3%s)" % ("EGLIB precision-1" if eg else "fitted-transport",
                                                       " + Strang BDF chemistry" if chem else ", no chemistry")
TRAFFIC_PER_LAUNCH = {}


def pin(a):
    try:
        import torch
        t = torch.empty(a.shape[::-1], dtype=torch.float64 if a.dtype == np.float64 else torch.uint8).pin_memory()
        b = t.numpy().T
        b[...] = a
        return b
    except Exception:
        return np.asfortranarray(a)


def cpu_baseline(args, steps=2):
    """The oracle (C++ restatement of the reference, OpenMP) on a 64x64x32
    block of the same workload (the full layer's grid spacing), all host
    threads, stepped as the reference driver steps (TimeLoop's sequence)."""
    import oracle
    from phd_gb300 import ics
    nx, ny, nz = 64, 64, 32
    if args.workload == "tgv":
        cfg, thd, adi, dxi, st, info = ics.tgv(48, lib_dscalar=oracle.metrics_dscalar)
        nx = ny = nz = 48
    else:
        cfg, thd, adi, dxi, st, info = ics.mixing_layer_block(nx, ny, nz, lib_dscalar=oracle.metrics_dscalar)
    eg = args.workload == "mix" and args.transport == "eglib"
    chem = args.workload == "mix" and not args.no_chem
    cfg.reaction = 1 if chem else 0
    if eg:
        from phd_gb300.thd import eglib_link, load_species
        cfg.eglib = 1
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    if eg:
        orc.set_eglib(eglib_link(load_species("h2air9")))
    orc.finalize_ic(st)
    mech = None
    if chem:
        from phd_gb300.mech import h2_mechanism
        mech = h2_mechanism()

    loop = {"dtmin": 1.0, "DTmax": 0.0}

    def step():
        _, dt = orc.timestep(st, DTmax=loop["DTmax"], dtmin=loop["dtmin"])
        if chem:
            orc.chem_step(st, mech, 0.5 * dt)
        orc.rk3(st, dt)
        if chem:
            loop["DTmax"] = orc.chem_step(st, mech, 0.5 * dt)
        loop["dtmin"] = dt

    step()   # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    s = time.perf_counter() - t0
    cores = os.cpu_count()
    return {"value": nx * ny * nz * steps / s / 1e6, "unit": "Mcell-steps/s", "cores": cores, "kind": "port",
            "sample": "%d steps of a %dx%dx%d sub-block of the same workload, OpenMP over pencils, %d threads"
                      % (steps, nx, ny, nz, cores)}


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mix", choices=["mix", "tgv", "batch", "surrogate", "field", "jet"])
    ap.add_argument("--cells", type=int, default=None,
                    help="reactors of the batch (default 2^20) and surrogate (default 512*256*256) workloads")
    ap.add_argument("--train", type=int, default=1 << 22, help="training reactors of the surrogate workload")
    ap.add_argument("--epochs", type=int, default=24, help="training epochs of the surrogate workload")
    ap.add_argument("--gate", default="calibrated", choices=["calibrated", "default", "strict"],
                    help="surrogate error gate: the default tolerances with a dT cap calibrated on held-out "
                         "reactors, the default tolerances alone, or tighter ones")
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=128)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-chem", action="store_true", help="mixing layer without the chemistry half-steps")
    ap.add_argument("--no-mlp", action="store_true", help="skip the learned-chemistry leg of the reacting step")
    ap.add_argument("--field-size", type=int, nargs=3, default=[512, 256, 256],
                    help="grid of the learned-chemistry reacting field workload")
    ap.add_argument("--field-dt", type=float, default=3e-7,
                    help="chemistry step [s] of the reacting field workload (the training range is 1e-8 .. 1e-6)")
    ap.add_argument("--jet-size", type=int, nargs=3, default=[512, 512, 256],
                    help="grid of the reacting LES jet workload")
    ap.add_argument("--no-jet", action="store_true",
                    help="skip the reacting LES jet (512 x 512 x 256) in the default line")
    ap.add_argument("--no-c4", action="store_true",
                    help="skip the learned-chemistry workload on the 512 x 256 x 256 reacting field in the "
                         "default line")
    ap.add_argument("--les", type=float, default=None,
                    help="mixing layer with the Smagorinsky closure (EGLIB) at this MU_SGS_FACTOR")
    ap.add_argument("--dvodesimp", action="store_true", help="mixing layer with the dvodesimp chemistry skip")
    ap.add_argument("--vis-dt", action="store_true", help="mixing layer with the Fourier time-step criteria")
    ap.add_argument("--chem-variant", type=int, default=None,
                    help="pin the register-budget variant of the chemistry kernels (0..4) instead of autotuning it")
    ap.add_argument("--transport", default="eglib", choices=["eglib", "fitted"],
                    help="viscous transport of the mixing layer (EGLIB precision 1 or the tranfit fits)")
    args = ap.parse_args()
    if args.cells is None:
        args.cells = 512 * 256 * 256 if args.workload == "surrogate" else 1 << 20
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        if rank == 0:
            cb = cpu_baseline(args, steps=max(1, args.steps // 2))
            line = {"impl": "reference", "metric": "reacting RHS Mcell-steps/s, FP64 plain vs MLP-chem (<=1% dT err) on 1 GB300",
                    "value": cb["value"], "unit": cb["unit"], "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                    "higher_is_better": True, "dtype": "f64", "data": "synthetic",
                    "config": {"workload": "H2/air temporal mixing layer (sub-block)"
                               + workload_note(args.workload == "mix" and not args.no_chem,
                                               args.workload == "mix" and args.transport == "eglib")},
                    "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0,
                                                "d2h_bytes_per_step": 0},
                    "note": "C++ restatement of the reference Fortran (no Fortran compiler on either host)"}
            print(json.dumps(line))
        return
    if args.impl == "ours":
        from phd_gb300.build import build_gpu
        if rank == 0:
            build_gpu()
        barrier(world)
        if world > 1:
            # one replica per GPU: restrict this process to its local device
            local = int(os.environ.get("LOCAL_RANK", "0"))
            vis = os.environ.get("CUDA_VISIBLE_DEVICES")
            devs = vis.split(",") if vis else [str(q) for q in range(world)]
            os.environ["CUDA_VISIBLE_DEVICES"] = devs[local % len(devs)]
    if args.workload in ("batch", "surrogate", "field", "jet"):
        if rank == 0:
            run = {"batch": run_batch, "surrogate": run_surrogate, "field": run_field_surrogate,
                   "jet": run_jet}[args.workload]
            print(json.dumps(run(args)))
        return
    res = run_gpu(args, rank, world)
    if rank == 0:
        if args.workload == "mix" and not args.no_c4:
            res["surrogate_c4"] = c4_summary(args)
        if args.workload == "mix" and not args.no_jet:
            res["reacting_jet_les"] = run_jet(args, steps=2, warmup=3)
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(res))


if __name__ == "__main__":
    main()
