"""Benchmark: zone-cycles/s of the GPU MHD stage update on one GB300.

Workload (one "step" = one full VL2 cycle, both stages, over the whole mesh): decaying
MHD turbulence, 256^3 periodic unit box as 512 MeshBlocks of 32^3, rho = 1, plasma
beta = 1 with uniform B along x, seeded solenoidal velocity with power in |k| in [1,4]
at rms Mach 1, gamma = 5/3, VL2 + PPM + HLLD.  Synthetic inputs with those shapes.

The headline ``value`` is the FP32 pipeline (FP32 reconstruction / Riemann / divergence
with a compensated conserved update, FP64 CT and time step); the plain FP64 GPU path
is timed on the same inputs beside it.  ``e2e`` runs the same cycles through the C ABI
with the state uploaded from and downloaded to pinned host memory every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With torchrun (N > 1) every rank advances its own replica of the mesh on its own GPU
(the path has no cross-GPU exchange on one-GPU hosts: replicas only).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("zone-cycles/s on 1 GB300: FP32+learned c2p vs plain FP64 GPU at equal L1 "
          "error")
NX, NB, NG = (256, 256, 256), (8, 8, 8), 3
BYTES_PER_ZONE_CYCLE = {"fp32": 260.0, "fp64": 320.0}  # algorithmic HBM bytes
ACC_CYCLES = 100  # cycles run by both paths for the FP32-vs-FP64 comparison (the
                  # workload's 100 steps): per-variable L1 and energy spectra
PROFILE_CYCLES = 3

# Dominant kernel of the FP32 cycle: the stage-2 x1 sweep (PPM + HLLD), the largest single
# launch.  Algorithmic bytes per interior zone: W (5) and the two transverse cell-centred
# field components read, 5 divergence words written (FP32), the x1 face field read (FP64),
# two face EMFs and the CT weight written (FP32): 7*4 + 5*4 + 8 + 3*4 = 68 B.
DOMINANT = "flux_x1"
DOMINANT_STAGE = 2
DOMINANT_BYTES_PER_ZONE = 68.0
# DRAM bytes per interior zone of that launch from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, 128^3 case, 2,097,152 zones: 128.0 MB + 46.8 MB), scaled by zones
DOMINANT_TRAFFIC_PER_ZONE = (128.020224e6 + 46.763776e6) / 2097152
# warp instructions per interior zone of that launch (ncu smsp__inst_executed.sum at 128^3)
DOMINANT_INST_PER_ZONE = 153832579.0 / 2097152
GB300_SMSP = 152 * 4


def workload_config(nx=NX, nb=NB):
    return {"workload": "decaying MHD turbulence %dx%dx%d periodic as %d MeshBlocks of "
                        "%dx%dx%d, VL2 + PPM + HLLD, gamma 5/3, beta 1, rms Mach 1" % (
                            nx + (nb[0] * nb[1] * nb[2],) + tuple(nx[d] // nb[d]
                                                               for d in range(3))),
            "zones": nx[0] * nx[1] * nx[2], "meshblocks": nb[0] * nb[1] * nb[2],
            "reconstruction": "PPM (stage 1 donor cell)", "riemann": "HLLD",
            "integrator": "vl2", "cfl": 0.3,
            "precision": "FP32 bulk + Kahan conserved update, FP64 CT and dt",
            "l2": "inputs larger than L2 (0.56 GB per FP32 state register)"}


def make_ic(nx=NX, nb=NB, ng=NG, seed=20261204):
    from athena_gb300.mesh import MeshSpec
    from athena_gb300 import pgen
    mesh = MeshSpec(nx, nb, ng)
    gu, f1, f2, f3 = pgen.turbulence(nx, seed=seed, mach=1.0, beta=1.0)
    u = mesh.scatter_cells(gu)
    b1, b2, b3 = mesh.scatter_faces(f1, f2, f3)
    return mesh, (u, b1, b2, b3)


# ------------------------------------------------------------------------------------
def energy_spectra(mesh, w, bcc, kmax):
    """Shell-averaged kinetic and magnetic energy spectra of a periodic state:
    E_K(k) = sum over |k'| in [k - 1/2, k + 1/2) of |FFT(sqrt(rho) v)|^2 / 2 and
    E_M(k) the same of the cell-centred field (FFT normalised by the cell count),
    k = 1..kmax in units of the box wavenumber.  w, bcc: per-block primitives and
    cell-centred field with ghosts.  Evaluated with torch's FFT on the device (analysis of
    the outputs, not part of the timed path)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    gw = torch.from_numpy(mesh.gather_cells(w)).to(dev)
    gb = torch.from_numpy(mesh.gather_cells(bcc)).to(dev)
    n3, n2, n1 = gw.shape[1:]
    ncell = n1 * n2 * n3
    k1 = torch.fft.fftfreq(n1, d=1.0 / n1, device=dev, dtype=torch.float64)
    k2 = torch.fft.fftfreq(n2, d=1.0 / n2, device=dev, dtype=torch.float64)
    k3 = torch.fft.fftfreq(n3, d=1.0 / n3, device=dev, dtype=torch.float64)
    kk = torch.sqrt(k3[:, None, None] ** 2 + k2[None, :, None] ** 2 + k1[None, None, :] ** 2)
    shell = torch.round(kk).to(torch.int64).ravel()

    def spec(fields):
        power = torch.zeros(n3 * n2 * n1, dtype=torch.float64, device=dev)
        for f in fields:
            fk = torch.fft.fftn(f) / ncell
            power += 0.5 * (fk.real ** 2 + fk.imag ** 2).ravel()
        e = torch.bincount(shell, weights=power, minlength=kmax + 1)
        return e[1:kmax + 1].cpu().numpy()
    sq = torch.sqrt(gw[0])
    ek = spec([sq * gw[1], sq * gw[2], sq * gw[3]])
    em = spec([gb[0], gb[1], gb[2]])
    return ek, em


# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        # one nvidia-smi process in loop mode (-lms): a sample every 25 ms without the
        # start-up cost of a process per sample
        try:
            self._p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        for line in self._p.stdout:
            if self._stop.is_set():
                break
            line = line.strip()
            if line:
                self.samples.append([x.strip() for x in line.split(",")])

    def __enter__(self):
        self._p = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._p is not None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------------
def time_device_cycles(g, stream, steps, warmup):
    """Cycles timed with CUDA events on the library's stream (inputs resident)."""
    import torch
    g.cycle(warmup)
    g.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        s.record(stream)
        g.cycle(steps)
        e.record(stream)
    e.synchronize()
    return s.elapsed_time(e) / 1e3


def link_ceiling(dev, nbytes, reps=3):
    """The host link's ceiling for the e2e copies: one plain cudaMemcpyAsync (torch copy_)
    of a pinned host buffer of nbytes to the device and back, CUDA events, best of reps."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    h.fill_(1.0)
    d = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
    out = {}
    for name, (dst, src) in (("h2d_gbs", (d, h)), ("d2h_gbs", (h, d))):
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        out[name] = nbytes / best / 1e9
    out["bytes"] = nbytes
    out["how"] = "one cudaMemcpyAsync of a pinned host buffer each way, CUDA events"
    del h, d
    return out


def run_gpu(args, rank, world, local_rank):
    global NX, NB
    NX = (args.nx,) * 3
    NB = (args.nx // 32,) * 3
    import torch
    import torch.distributed as dist
    from athena_gb300 import build
    from athena_gb300.runtime import COPY_INTERIOR, COPY_WHOLE, StageUpdate
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    mesh, ic = make_ic(NX, NB)
    zones = mesh.nx[0] * mesh.nx[1] * mesh.nx[2]
    stream = torch.cuda.Stream(device=dev)
    res = {}
    for prec in ("fp32", "fp64"):
        g = StageUpdate(mesh, 5.0 / 3.0, xorder=3, rsolver="hlld", precision=prec, cfl=0.3)
        g.set_stream(stream.cuda_stream)
        g.set_state(*ic)
        g.initialize()
        if prec == "fp32":  # sweep tiling picked by the autotuner (state left unchanged)
            res["tiling"] = dict(zip(("seg_x2", "seg_x3"), g.autotune(cycles=2)))
            res["tiling"]["x3_staging"] = "tma_bulk" if g.x3_staging() else "cp_async"
        steps = args.steps if prec == "fp32" else max(3, min(args.steps, 10))
        sampler = ClockSampler(local_rank) if prec == "fp32" else None
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        if sampler:
            with sampler:
                dt = time_device_cycles(g, stream, steps, args.warmup)
        else:
            dt = time_device_cycles(g, stream, steps, args.warmup)
        torch.cuda.synchronize()
        if world > 1:
            t = torch.tensor([dt], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        res[prec] = {"seconds": dt, "steps": steps, "value": world * zones * steps / dt,
                     "ms_per_step": dt / steps * 1e3}
        if prec == "fp32":  # |div B| after the timed cycles (the reference's diagnostic)
            s_, m_, c_ = g.divb()
            res["divb"] = {"max": m_, "mean": s_ / max(c_, 1), "cells": c_,
                           "after_cycles": args.warmup + steps + 2}
        # accuracy: the same number of cycles from the same initial state in each path
        g.set_state(*ic)
        g.set_clock(0.0, 1.7976931348623157e308)
        g.initialize()
        g.cycle(ACC_CYCLES)
        res["u_" + prec] = mesh.interior(g.state()[0])
        w_acc, bcc_acc = g.prim()
        res["spec_" + prec] = energy_spectra(mesh, w_acc, bcc_acc, NX[0] // 2)
        del w_acc, bcc_acc
        if prec == "fp64":
            res["profile64"] = g.profile_cycle()
        else:
            res["clocks"] = sampler.summary()
            g.launch_count(reset=True)
            g.cycle(1)
            g.synchronize()
            res["launches_per_step"] = g.launch_count()
            # per-kernel CUDA-event profile (non-graph cycles on the library's stream),
            # averaged over PROFILE_CYCLES cycles
            profs = [g.profile_cycle() for _ in range(PROFILE_CYCLES)]
            res["profile32"] = [(profs[0][q][0],
                                 sum(p[q][1] for p in profs) / len(profs))
                                for q in range(len(profs[0]))]
            # e2e through the C ABI with pinned host buffers
            pinned = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
                      for a in ic]
            for p, a in zip(pinned, ic):
                p[...] = a
            pinned_out = [torch.empty(a.shape, dtype=torch.float64,
                                      pin_memory=True).numpy() for a in ic]
            ebytes = sum(p.nbytes for p in pinned)
            e_steps = max(2, min(args.steps, 10))
            # the faster host-copy mode of the library on this machine (chunked DMA over
            # several streams, or conversion kernels on the pinned arrays), by one timed
            # upload + download of each
            # upload + download of each; and the copies of each block's x2/x3 interior with
            # whole x1 rows (COPY_INTERIOR: initialize() recomputes the ghost zones)
            mode_ms = {}
            for name, extent, mode in (("whole/dma", COPY_WHOLE, 0),
                                       ("whole/link", COPY_WHOLE, 1),
                                       ("interior/dma", COPY_INTERIOR, 0)):
                g.set_copy_extent(extent)
                g.set_host_copy(mode)
                g.set_state(*pinned)
                g.state(out=pinned_out)
                t0 = time.perf_counter()
                g.set_state(*pinned)
                g.state(out=pinned_out)
                mode_ms[name] = (time.perf_counter() - t0) * 1e3
            host_mode = min(mode_ms, key=mode_ms.get)
            extent = COPY_INTERIOR if host_mode.startswith("interior") else COPY_WHOLE
            g.set_copy_extent(extent)
            g.set_host_copy(1 if host_mode == "whole/link" else 0)
            cbytes = state_copy_bytes(mesh, extent)
            for _ in range(2):
                g.set_state(*pinned)
                g.initialize()
                g.cycle(1)
                out = g.state(out=pinned_out)
            torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
            t0 = time.perf_counter()
            step_ms = []
            for _ in range(e_steps):
                ts = time.perf_counter()
                g.set_state(*pinned)    # host -> device (pinned) every step
                g.initialize()          # W(U), ghosts and the time step of that state
                g.cycle(1)
                out = g.state(out=pinned_out)   # device -> host (pinned) every step
                step_ms.append((time.perf_counter() - ts) * 1e3)  # the download syncs
            torch.cuda.synchronize()
            te = time.perf_counter() - t0
            if world > 1:
                t = torch.tensor([te], device=dev)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                te = float(t.item())
            res["e2e"] = {"value": world * zones * e_steps / te, "unit": "zone-cycles/s",
                          "h2d_bytes_per_step": cbytes, "d2h_bytes_per_step": cbytes,
                          "steps": e_steps, "ms_per_step": te / e_steps * 1e3,
                          "host_copy_mode": host_mode, "whole_state_bytes": ebytes,
                          "step_ms": {"min": min(step_ms), "median": float(np.median(step_ms)),
                                      "max": max(step_ms),
                                      "all": [round(x, 2) for x in step_ms]},
                          "upload_download_ms_by_mode": mode_ms,
                          "link_ceiling": link_ceiling(dev, ebytes)}
        g.close()
    res["linear_wave_l1"] = run_linear_wave()
    if not args.no_amr:
        res["amr_blast"] = run_amr_blast(stream, cpu=not args.no_cpu_baseline)
    if not args.no_learned:
        res["learned_c2p"], net = run_learned_c2p()
        if not args.no_sr:
            res["sr_kh"] = run_sr_kh(args.nx, stream, net)
    return mesh, res


LEARNED_CELLS = 1 << 24


def run_learned_c2p(reps=5):
    """Learned con2prim in isolation: 2^24 independent SR-MHD cells (gamma 4/3, Lorentz
    factor in [1,10], sigma in [1e-2,1e2], rho in [1e-4,1], p/rho in [1e-3,10], all
    log-uniform, isotropic v and B).  The network is trained here on 2^20 solver-made
    pairs; the plain solve starts from the pressure floor (an isolated cell has no
    previous pressure), the learned one from the BF16 network (tcgen05 tensor cores, and
    for comparison warp-level mma.sync) refined in FP32, both finished by the reference's
    FP64 iteration (two warp-coherent launches each)."""
    import torch
    from athena_gb300 import pgen
    from athena_gb300.learned_c2p import LearnedC2P, MODE_LEARNED_FP32, MODE_PLAIN, WARP_MMA
    net = LearnedC2P(4.0 / 3.0, seed=0)
    t0 = time.perf_counter()
    feats, targ = net.solver_pairs(1 << 20, 101)
    net.set_standardization(feats, targ)
    hist = net.train(feats, targ, steps=8000, batch=4096, lr=2.0e-3, seed=101)
    t_train = time.perf_counter() - t0
    w, bcc, u = pgen.sr_isolated_cells(LEARNED_CELLS, seed=777)
    cons, b = net.to_dev(u), net.to_dev(bcc)
    del w, bcc, u
    out = {"workload": "2^24 independent SR-MHD cells, gamma 4/3, Lorentz factor "
                       "log-uniform [1,10], sigma [1e-2,1e2], rho [1e-4,1], p/rho "
                       "[1e-3,10], isotropic v and B (synthetic, seeded)",
           "cells": LEARNED_CELLS,
           "training": {"pairs": feats.shape[0], "steps": 8000, "batch": 4096,
                        "seconds": t_train, "loss_first": float(hist[:10].mean()),
                        "loss_last": float(hist[-100:].mean())}}
    stream = torch.cuda.current_stream()
    for name, mode in (("plain", MODE_PLAIN), ("learned", MODE_LEARNED_FP32),
                       ("learned_warp_mma", MODE_LEARNED_FP32 | WARP_MMA)):
        ts = []
        for rep in range(reps + 2):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            prim, it, it32, fb = net.solve(cons, b, mode, want_iters32=True)
            s1.record(stream)
            s1.synchronize()
            if rep >= 2:
                ts.append(s0.elapsed_time(s1))
        it = it.cpu().numpy()
        ms = float(np.median(ts))
        out[name] = {"ms": ms, "cells_per_s": LEARNED_CELLS / (ms * 1e-3),
                     "mean_fp64_passes": float(it[it >= 0].mean()),
                     "unconverged": int((it < 0).sum())}
        if mode & 0xff == MODE_LEARNED_FP32:
            out[name]["mean_fp32_passes"] = float(it32.float().mean().item())
            out[name]["fallbacks"] = fb
    out["speedup"] = out["plain"]["ms"] / out["learned"]["ms"]
    out["passes_ratio"] = out["learned"]["mean_fp64_passes"] / out["plain"]["mean_fp64_passes"]
    return out, net


def run_linear_wave():
    """Linear-wave accuracy of the FP32 and FP64 paths: the oblique fast wave (VL2 + PLM +
    HLLD) for one period on 64x32x32 (one MeshBlock, the reference's config-1 case, and on
    128x64x64 with 8 MeshBlocks) at the reference's amplitude 1e-6, and on 64x32x32 at
    amplitude 1e-3; RMS L1 error against the initial state (linear_wave.cpp's error
    routine, restated in pgen.LinearWave.l1_errors)."""
    from athena_gb300 import pgen
    from athena_gb300.mesh import MeshSpec
    from athena_gb300.runtime import StageUpdate
    out = {}
    for nx, nb, amp in (((64, 32, 32), (1, 1, 1), 1.0e-6), ((128, 64, 64), (2, 2, 2), 1.0e-6),
                        ((64, 32, 32), (1, 1, 1), 1.0e-3)):
        mesh = MeshSpec(nx, nb, 2, (0.0, 0.0, 0.0), (3.0, 1.5, 1.5))
        lw = pgen.LinearWave(mesh, gamma=1.666666666666667, amp=amp)
        ic = lw.generate()
        row = {}
        for prec in ("fp64", "fp32"):
            g = StageUpdate(mesh, lw.gam, xorder=2, rsolver="hlld", precision=prec,
                            tlim=lw.period())
            g.set_state(*ic)
            g.initialize()
            ncyc = g.run_until(lw.period())
            u = g.state()[0]
            _, bcc = g.prim()
            row[prec] = lw.l1_errors(u, bcc)[0]
            row["cycles_" + prec] = ncyc
            g.close()
        row["ratio_fp32_vs_fp64"] = row["fp32"] / row["fp64"]
        out["%dx%dx%d_amp%g" % (nx + (amp,))] = row
    return out


SR_CYCLES = {"fp32": 10, "fp64": 3}
SR_ACC_CYCLES = 5


def run_sr_kh(n, stream, net):
    """Relativistic Kelvin-Helmholtz shear layer (the full SR step workload): n^3 periodic
    box as (n/32)^3 MeshBlocks, gamma 4/3, v_x = +-0.5c with tanh width 0.01, rho 1 / 0.1,
    p = 1, uniform B_x with sigma 0.1, seeded 1e-3 velocity noise, VL2 + PLM + HLLE.
    Zone-cycles/s of the FP32 and FP64 SR stage paths (CUDA events, state resident), their
    relative L1 difference after SR_ACC_CYCLES cycles, and the same step with the LLF and
    HLLD solvers in place of HLLE.  Inside the stage each start of the
    FP64 con2prim solve is timed (the stale pressure, that pressure refined in FP32, the
    network evaluated on tcgen05 in the W(U) kernel and refined in FP32) with its mean FP64
    passes, fallbacks and unconverged cells from the run statistics, also for the first
    W(U) without stale primitives (as after a restart).  The con2prim start study solves
    the conserved state of one cycle per cell with the isolated-cell entry point from the
    previous cycle's pressure, that pressure refined in FP32, and the network."""
    import torch
    from athena_gb300 import pgen
    from athena_gb300.learned_c2p import MODE_LEARNED_FP32, MODE_PLAIN, MODE_REFINED
    from athena_gb300.mesh import MeshSpec
    from athena_gb300.runtime import StageUpdate
    nx, nb = (n,) * 3, (n // 32,) * 3
    mesh = MeshSpec(nx, nb, 2)
    gam = 4.0 / 3.0
    gw, f1, f2, f3 = pgen.sr_kelvin_helmholtz(nx, seed=20261204)
    gu = pgen.sr_prim_to_cons(gw, pgen.cell_centered(f1, f2, f3), gam)
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    w0 = mesh.scatter_cells(gw)
    del gu, gw
    zones = n ** 3
    out = {"workload": "relativistic Kelvin-Helmholtz %d^3 periodic as %d MeshBlocks of "
                       "32^3, gamma 4/3, shear +-0.5c, sigma 0.1, VL2 + PLM + HLLE" %
                       (n, nb[0] * nb[1] * nb[2])}
    finals = {}
    wzero = np.zeros_like(w0)
    for prec in ("fp32", "fp64"):
        g = StageUpdate(mesh, gam, xorder=2, rsolver="hlle", precision=prec, cfl=0.3,
                        relativistic=True)
        g.set_stream(stream.cuda_stream)
        # every start of the FP64 solve inside the stage: the default first (FP32 path: the
        # stale pressure refined in FP32; FP64 path: the stale pressure, the reference's)
        starts = ("refined", "network", "stale") if prec == "fp32" else ("stale", "network")
        by_start, cold = {}, {}
        for start in starts:
            g.set_c2p_start(start, net.params if start == "network" else None)
            # the first W(U) with no stale primitives (w = 0, as after a restart, whose
            # file holds U and B only): the stale start is the pressure floor
            g.set_state(*ic)
            g.set_prim(wzero)
            g.initialize()
            st = g.stats(reset=True)
            cold[start] = {"mean_fp64_passes": st["sr_passes"] / max(st["sr_cells"], 1),
                           "unconverged": st["sr_unconverged"],
                           "fallbacks": st["sr_fallbacks"]}
            # the timed run from the initial primitives
            g.set_state(*ic)
            g.set_prim(w0)
            g.set_clock(0.0, 1.7976931348623157e308)
            g.initialize()
            g.stats(reset=True)
            t = time_device_cycles(g, stream, SR_CYCLES[prec], 3)
            st = g.stats(reset=True)
            by_start[start] = {"value": zones * SR_CYCLES[prec] / t, "unit": "zone-cycles/s",
                               "ms_per_step": t / SR_CYCLES[prec] * 1e3,
                               "mean_fp64_passes": st["sr_passes"] / max(st["sr_cells"], 1),
                               "unconverged": st["sr_unconverged"],
                               "fallbacks": st["sr_fallbacks"], "net_error": st["net_error"]}
        out[prec] = dict(by_start[starts[0]], steps=SR_CYCLES[prec], start=starts[0])
        out[prec]["in_stage_starts"] = by_start
        out[prec]["first_c2p_without_stale_primitives"] = cold
        g.set_c2p_start(starts[0])
        g.set_state(*ic)
        g.set_prim(w0)
        g.set_clock(0.0, 1.7976931348623157e308)
        g.initialize()
        g.cycle(SR_ACC_CYCLES - 1)
        if prec == "fp64":
            w_prev, _ = g.prim()
        g.cycle(1)
        finals[prec] = mesh.interior(g.state()[0])
        if prec == "fp64":
            u_new = g.state()[0]
            _, bcc_new = g.prim()
        g.close()
    out["speedup_fp32_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    # the same workload with each relativistic Riemann solver (default con2prim start)
    out["by_solver"] = {"hlle": {p: {"value": out[p]["value"],
                                     "ms_per_step": out[p]["ms_per_step"]}
                                 for p in ("fp32", "fp64")}}
    for rs in ("llf", "hlld"):
        out["by_solver"][rs] = {}
        for prec in ("fp32", "fp64"):
            g = StageUpdate(mesh, gam, xorder=2, rsolver=rs, precision=prec, cfl=0.3,
                            relativistic=True)
            g.set_stream(stream.cuda_stream)
            g.set_state(*ic)
            g.set_prim(w0)
            g.set_clock(0.0, 1.7976931348623157e308)
            g.initialize()
            t = time_device_cycles(g, stream, SR_CYCLES[prec], 3)
            st = g.stats()
            out["by_solver"][rs][prec] = {"value": zones * SR_CYCLES[prec] / t,
                                          "ms_per_step": t / SR_CYCLES[prec] * 1e3,
                                          "unconverged": st["sr_unconverged"]}
            g.close()
    l1 = l1_rel(finals["fp32"], finals["fp64"])
    out["l1_rel_fp32_vs_fp64"] = {"cycles": SR_ACC_CYCLES, "d": l1[0], "m1": l1[1],
                                  "m2": l1[2], "m3": l1[3], "e": l1[4]}
    # con2prim start study on the interior cells of cycle SR_ACC_CYCLES
    cons = np.ascontiguousarray(np.moveaxis(mesh.interior(u_new), 1, -1).reshape(-1, 5))
    bcc = np.ascontiguousarray(np.moveaxis(mesh.interior(bcc_new), 1, -1).reshape(-1, 3))
    pprev = np.ascontiguousarray(np.moveaxis(mesh.interior(w_prev), 1, -1)
                                 .reshape(-1, 5)[:, 4])
    dc, db, dp = net.to_dev(cons), net.to_dev(bcc), net.to_dev(pprev)
    study = {"cells": int(cons.shape[0])}
    for name, mode, guess in (("previous_pressure", MODE_PLAIN, dp),
                              ("previous_pressure_fp32_refined", MODE_REFINED, dp),
                              ("learned", MODE_LEARNED_FP32, dp)):
        ts = []
        for rep in range(4):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record()
            prim, it, _, fb = net.solve(dc, db, mode, pgas_guess=guess)
            s1.record()
            s1.synchronize()
            ts.append(s0.elapsed_time(s1))
        it = it.cpu().numpy()
        study[name] = {"mean_fp64_passes": float(it[it >= 0].mean()),
                       "unconverged": int((it < 0).sum()), "ms": float(np.median(ts[1:])),
                       "fallbacks": fb}
    out["c2p_start_study"] = study
    return out


AMR_ROOT = 160        # root grid cells per direction (10^3 MeshBlocks of 16^3)
AMR_THR = 0.3        # pressure-gradient threshold of the blast refinement condition
AMR_WARM = {"fp32": (5, 30), "fp64": (3, 10)}   # warm-up and timed cycles
AMR_ACC_CYCLES = 12


def run_amr_blast(stream, cpu=True):
    """Adaptive MHD blast (3 refinement levels, 16^3 MeshBlocks): unit cube
    [-0.5, 0.5]^3 with a 128^3 root grid, rho 1, p 0.1 and p 10 for r < 0.1,
    B = (1,1,1)/sqrt(2), gamma 5/3, VL2 + PLM + HLLE, CFL 0.3, refinement on the blast's
    pressure-gradient condition (thr AMR_THR, derefine_count 10) checked every cycle.
    Zone-cycles/s by the reference's count (the blocks of each cycle times 16^3), timed by
    the host clock around whole cycles: the CUDA-graph stages, the refinement measure,
    the flags and tree update (native host code) and every regrid; the stages alone are
    timed with CUDA events on the final mesh."""
    import time
    import torch
    from athena_gb300 import pgen
    from athena_gb300.adaptive import AdaptiveStageUpdate
    from athena_gb300.meshtree import MultiLevelMesh
    b = 1.0 / np.sqrt(2.0)

    def ic(m):
        return pgen.blast_blocks(m, 5.0 / 3.0, radius=0.1, pamb=0.1, prat=100.0,
                                 bfield=(b, b, b))
    out = {"workload": "adaptive MHD blast, 3 levels of 16^3 MeshBlocks on a %d^3 root "
                       "grid, VL2 + PLM + HLLE, thr %g" % (AMR_ROOT, AMR_THR)}
    for prec in ("fp32", "fp64"):
        warm, cyc = AMR_WARM[prec]
        mesh0 = MultiLevelMesh((AMR_ROOT,) * 3, (AMR_ROOT // 16,) * 3, 2, (-.5,) * 3,
                               (.5,) * 3)
        run = AdaptiveStageUpdate(mesh0, ic, 3, AMR_THR, 10, gamma=5.0 / 3.0, xorder=2,
                                  rsolver="hlle", precision=prec, cfl=0.3)
        run.su.set_stream(stream.cuda_stream)
        run.initialize()
        nb_init = run.mesh.nblocks
        run.cycle(warm)
        torch.cuda.synchronize()
        r0, tr0 = run.regrids, run.t_refine
        zc, nbs = 0, []
        t0 = time.perf_counter()
        for _ in range(cyc):
            nbs.append(run.mesh.nblocks)
            zc += run.mesh.nblocks * 16 ** 3
            run.cycle(1)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        out[prec] = {"value": zc / t, "unit": "zone-cycles/s", "cycles": cyc,
                     "ms_per_cycle": t / cyc * 1e3, "blocks_initial": nb_init,
                     "blocks_min": min(nbs), "blocks_max": max(nbs),
                     "levels": [int(v) for v in np.bincount(run.mesh.levels)[
                         run.mesh.tree.root_level:]],
                     "regrids": run.regrids - r0,
                     "refine_step_s": run.t_refine - tr0,
                     # every main-loop regrid of the run (warm-up included): the whole
                     # refinement step, device data movement and re-initialisation
                     "regrid_ms": [round(v, 2) for v in run.regrid_ms]}
        # the stages alone (CUDA graph replays) on the final mesh
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        run.su.cycle(2)
        ev0.record(stream)
        run.su.cycle(5)
        ev1.record(stream)
        ev1.synchronize()
        out[prec]["stages_ms_per_cycle"] = ev0.elapsed_time(ev1) / 5
        out[prec]["stages_blocks"] = run.mesh.nblocks
        run.close()
    out["speedup_fp32_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    # accuracy: FP32 against FP64 after AMR_ACC_CYCLES cycles from the same start
    finals = {}
    for prec in ("fp32", "fp64"):
        mesh0 = MultiLevelMesh((AMR_ROOT,) * 3, (AMR_ROOT // 16,) * 3, 2, (-.5,) * 3,
                               (.5,) * 3)
        run = AdaptiveStageUpdate(mesh0, ic, 3, AMR_THR, 10, gamma=5.0 / 3.0, xorder=2,
                                  rsolver="hlle", precision=prec, cfl=0.3)
        run.initialize()
        run.cycle(AMR_ACC_CYCLES)
        finals[prec] = ([(l.level, l.lx1, l.lx2, l.lx3) for l in run.mesh.locs],
                        run.mesh.interior(run.state()[0]))
        run.close()
    if finals["fp32"][0] == finals["fp64"][0]:
        l1 = l1_rel(finals["fp32"][1], finals["fp64"][1])
        out["l1_rel_fp32_vs_fp64"] = {"cycles": AMR_ACC_CYCLES, "d": l1[0], "m1": l1[1],
                                      "m2": l1[2], "m3": l1[3], "e": l1[4]}
    else:
        out["l1_rel_fp32_vs_fp64"] = {"cycles": AMR_ACC_CYCLES,
                                      "note": "the FP32 and FP64 runs refined differently"}
    if cpu:
        out["cpu_baseline"] = amr_cpu_baseline(ic)
    return out


def amr_profile_cycle(precision="fp32", warm=2):
    """One cycle of the adaptive blast without the CUDA graph, every kernel timed with CUDA
    events, between cudaProfilerStart and cudaProfilerStop (for ncu
    --profile-from-start off); returns per-kernel launches and milliseconds."""
    import torch
    from athena_gb300 import pgen
    from athena_gb300.adaptive import AdaptiveStageUpdate
    from athena_gb300.meshtree import MultiLevelMesh
    b = 1.0 / np.sqrt(2.0)
    mesh0 = MultiLevelMesh((AMR_ROOT,) * 3, (AMR_ROOT // 16,) * 3, 2, (-.5,) * 3, (.5,) * 3)
    run = AdaptiveStageUpdate(
        mesh0, lambda m: pgen.blast_blocks(m, 5.0 / 3.0, radius=0.1, pamb=0.1, prat=100.0,
                                           bfield=(b, b, b)),
        3, AMR_THR, 10, gamma=5.0 / 3.0, xorder=2, rsolver="hlle", precision=precision,
        cfl=0.3)
    run.initialize()
    run.cycle(warm)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    prof = run.su.profile_cycle()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    agg = {}
    for name, ms in prof:
        n, t = agg.get(name, (0, 0.0))
        agg[name] = (n + 1, t + ms)
    out = {"workload": "adaptive blast %s, %d blocks" % (precision, run.mesh.nblocks),
           "cycle_ms": sum(ms for _, ms in prof),
           "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in agg.items()}}
    run.close()
    return out


def x3_staging_cycles(n=128):
    """One cycle (per-kernel CUDA events, no graph) of the n^3 turbulence workload in FP32
    with each staging of the x3 sweep: per-thread cp.async, then TMA bulk copies."""
    from athena_gb300 import build
    from athena_gb300.runtime import StageUpdate
    build.build()
    mesh, ic = make_ic((n,) * 3, (n // 32,) * 3)
    g = StageUpdate(mesh, 5.0 / 3.0, xorder=3, rsolver="hlld", precision="fp32", cfl=0.3)
    g.set_state(*ic)
    g.initialize()
    out = {}
    for bulk in (0, 1):
        g.set_x3_staging(bulk)
        prof = g.profile_cycle()
        out["tma_bulk" if bulk else "cp_async"] = [ms for name, ms in prof
                                                   if name == "flux_x3_update"]
    st = g.stats()
    g.close()
    if st["sweep_timeout"]:
        raise RuntimeError("a bulk-copy wait timed out")
    return out


def amr_cpu_baseline(ic, threads=None):
    """The oracle (C port of the reference algorithm, FP64, OpenMP over MeshBlocks) on the
    host cores: the adaptive initial loop, then one timed cycle with its refinement step
    (a bounded sample of the adaptive blast workload)."""
    import time
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amr_run
    from athena_gb300.meshtree import MultiLevelMesh
    threads = threads or os.cpu_count()
    mesh0 = MultiLevelMesh((AMR_ROOT,) * 3, (AMR_ROOT // 16,) * 3, 2, (-.5,) * 3, (.5,) * 3)
    amr, om = amr_run.initialize(mesh0, ic, 3, AMR_THR, 10, gamma=5.0 / 3.0, xorder=2,
                                 rsolver="hlle", cfl=0.3, threads=threads)
    zones = amr.mesh.nblocks * 16 ** 3
    t0 = time.perf_counter()
    om = amr_run.cycle(amr, om, AMR_THR)
    t = time.perf_counter() - t0
    return {"value": zones / t, "unit": "zone-cycles/s", "cores": threads, "kind": "port",
            "sample": "1 cycle (with its refinement step) of the %d-block mesh after the "
                      "adaptive initial loop" % (zones // 16 ** 3)}


def state_copy_bytes(mesh, extent):
    """Bytes one upload (or download) of U and the three face arrays moves: whole
    arrays, or (COPY_INTERIOR) per block the own x2/x3 range with whole x1 rows."""
    from athena_gb300.runtime import COPY_WHOLE
    c1, c2, c3 = mesh.nc
    if extent == COPY_WHOLE:
        n = 5 * c3 * c2 * c1 + c3 * c2 * (c1 + 1) + c3 * (c2 + 1) * c1 + (c3 + 1) * c2 * c1
    else:
        n1, n2, n3 = mesh.bx
        n = 5 * n3 * n2 * c1 + n3 * n2 * (c1 + 1) + n3 * (n2 + 1) * c1 + (n3 + 1) * n2 * c1
    return 8 * n * mesh.nblocks


def l1_rel(a, b):
    return [float(np.abs(a[:, n] - b[:, n]).mean() / np.abs(b[:, n]).mean())
            for n in range(a.shape[1])]


def cpu_baseline(mesh_ic, cycles=2, threads=None):
    """The oracle (C port of the reference algorithm, FP64, OpenMP over MeshBlocks) on the
    host cores: `cycles` full cycles of the same 256^3 workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    mesh, ic = mesh_ic
    threads = threads or os.cpu_count()
    om = oracle.OracleMesh(mesh, 5.0 / 3.0, xorder=3, rsolver="hlld", cfl=0.3,
                           threads=threads)
    om.set_state(*ic)
    om.initialize()
    t0 = time.perf_counter()
    om.cycle(cycles)
    dt = time.perf_counter() - t0
    zones = mesh.nx[0] * mesh.nx[1] * mesh.nx[2]
    return {"value": zones * cycles / dt, "unit": "zone-cycles/s", "cores": threads,
            "kind": "port", "sample": "%d full VL2 cycles of the 256^3 workload, FP64, "
                                      "%d OpenMP threads" % (cycles, threads)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the isolated learned-con2prim and the SR measurements")
    ap.add_argument("--no-sr", action="store_true",
                    help="skip the relativistic Kelvin-Helmholtz measurement")
    ap.add_argument("--no-amr", action="store_true",
                    help="skip the adaptive blast measurement")
    ap.add_argument("--nx", type=int, default=256,
                    help="cells per direction (MeshBlocks of 32^3); 256 is the workload")
    ap.add_argument("--amr-profile-cycle", action="store_true",
                    help="only: one profiled cycle of the adaptive blast (FP32)")
    ap.add_argument("--x3-staging-cycles", action="store_true",
                    help="only: one non-graph FP32 cycle of the 128^3 workload with each x3 "
                         "staging (per-thread cp.async, TMA bulk copies), for ncu")
    args = ap.parse_args()
    if args.amr_profile_cycle:
        from athena_gb300 import build
        build.build()
        print(json.dumps(amr_profile_cycle()))
        return
    if args.x3_staging_cycles:
        print(json.dumps(x3_staging_cycles()))
        return
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))

    if args.impl == "reference":
        if rank != 0:
            return
        mesh_ic = make_ic()
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        mesh, ic = mesh_ic
        threads = os.cpu_count()
        om = oracle.OracleMesh(mesh, 5.0 / 3.0, xorder=3, rsolver="hlld", cfl=0.3,
                               threads=threads)
        om.set_state(*ic)
        om.initialize()
        om.cycle(args.warmup)
        t0 = time.perf_counter()
        om.cycle(args.steps)
        dt = time.perf_counter() - t0
        zones = NX[0] * NX[1] * NX[2]
        v = zones * args.steps / dt
        line = {"metric": METRIC, "value": v, "unit": "zone-cycles/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "impl": "reference",
                "config": workload_config(),
                "cpu_baseline": {"value": v, "unit": "zone-cycles/s", "cores": threads,
                                 "kind": "port",
                                 "sample": "each step one full VL2 cycle of the 256^3 "
                                           "workload, FP64, %d OpenMP threads" % threads},
                "e2e": {"value": v, "unit": "zone-cycles/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    mesh, res = run_gpu(args, rank, world, local_rank)
    line_config = workload_config(NX, NB)
    if "tiling" in res:
        line_config["sweep_tiling_autotuned"] = res["tiling"]
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    zones = mesh.nx[0] * mesh.nx[1] * mesh.nx[2]
    r32, r64 = res["fp32"], res["fp64"]
    peak, peak_kind = measured_peaks()
    # the whole VL2 cycle (CUDA graph of all stage kernels) as one unit
    cycle_achieved = (BYTES_PER_ZONE_CYCLE["fp32"] * zones /
                      (r32["seconds"] / r32["steps"]) / 1e9)
    # the dominant kernel: its CUDA-event duration in the profiled cycles
    dom = [ms for name, ms in res["profile32"] if name == DOMINANT]
    dom_ms = dom[DOMINANT_STAGE - 1]
    dom_bytes = DOMINANT_BYTES_PER_ZONE * zones
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    sm_hz = (res["clocks"].get("sm_mhz") or 2070.0) * 1e6
    l1 = l1_rel(res["u_fp32"], res["u_fp64"])
    # energy spectra after ACC_CYCLES cycles: the largest relative difference over the
    # resolved band (k <= N/8, i.e. at least 8 cells per wavelength) and over all k
    (ek32, em32), (ek64, em64) = res["spec_fp32"], res["spec_fp64"]
    kres = NX[0] // 8
    spectra = {"cycles": ACC_CYCLES, "k": "1..%d" % (NX[0] // 2),
               "resolved_band": "1..%d" % kres,
               "max_rel_diff_kinetic_resolved": float(np.max(np.abs(ek32[:kres] / ek64[:kres] - 1))),
               "max_rel_diff_magnetic_resolved": float(np.max(np.abs(em32[:kres] / em64[:kres] - 1))),
               "max_rel_diff_kinetic_all": float(np.max(np.abs(ek32 / ek64 - 1))),
               "max_rel_diff_magnetic_all": float(np.max(np.abs(em32 / em64 - 1))),
               "E_kinetic_fp64": [float(v) for v in ek64[:16]],
               "E_magnetic_fp64": [float(v) for v in em64[:16]]}
    line = {"metric": METRIC, "value": r32["value"], "unit": "zone-cycles/s",
            "n_gpus": world, "steps": r32["steps"], "warmup": args.warmup,
            "ms_per_step": r32["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": line_config,
            "fp64_gpu": {"value": r64["value"], "ms_per_step": r64["ms_per_step"],
                         "steps": r64["steps"]},
            "speedup_fp32_vs_fp64_gpu": r32["value"] / r64["value"],
            "l1_rel_fp32_vs_fp64": {"cycles": ACC_CYCLES, "d": l1[0], "m1": l1[1],
                                    "m2": l1[2], "m3": l1[3], "e": l1[4]},
            "energy_spectra_fp32_vs_fp64": spectra,
            "divb": res.get("divb"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": DOMINANT_TRAFFIC_PER_ZONE * zones,
                         "kernel": "flux_x1_kernel<float, PPM, HLLD> (stage 2)",
                         "launch_ms": dom_ms, "bytes_per_launch": dom_bytes,
                         "traffic_source": "ncu dram bytes of the 128^3 launch, scaled by "
                                           "zones",
                         "limiter": "instruction issue (FP32/ALU), not HBM",
                         "issue_frac": DOMINANT_INST_PER_ZONE * zones /
                                       (GB300_SMSP * sm_hz * dom_ms * 1e-3),
                         "peak_kind": peak_kind,
                         "cycle": {"achieved": cycle_achieved,
                                   "frac": cycle_achieved / peak,
                                   "bytes_per_zone_cycle": BYTES_PER_ZONE_CYCLE["fp32"],
                                   "kernels": res["launches_per_step"]}},
            "e2e": res["e2e"], "gpu_launches": res["launches_per_step"] * r32["steps"],
            "clocks": res["clocks"],
            "kernel_ms_fp32": res["profile32"], "kernel_ms_fp64": res["profile64"]}
    if "learned_c2p" in res:
        line["learned_c2p"] = res["learned_c2p"]
    if "sr_kh" in res:
        line["sr_kh"] = res["sr_kh"]
    if "linear_wave_l1" in res:
        line["linear_wave_l1"] = res["linear_wave_l1"]
    if "amr_blast" in res:
        line["amr_blast"] = res["amr_blast"]
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline((mesh, make_ic(NX, NB)[1]))
        # like for like: the plain FP64 GPU path against the FP64 CPU baseline
        line["fp64_gpu"]["vs_cpu_baseline"] = r64["value"] / line["cpu_baseline"]["value"]
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
