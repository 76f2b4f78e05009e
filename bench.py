#!/usr/bin/env python3
"""Benchmark of the GB300 FIREBALL Harris assembly hot path.

One step = one pass of the path over one structure: the neighbor maps
(driver_neighbors), the 2c + 3c H/S assembly (assemble_S, assemble_T,
assemble_vna_2c, assemble_vna_3c) and the force derivatives with the force
reduction (Dassemble_S/T/vna_2c/vna_3c, build_forces).  The assembly and
force kernels run as one CUDA graph launch per step, with launch shapes
picked by the library's autotuner.  The density matrices the solver would
supply are seeded synthetic blocks.

Default workload: SiC4096, the 4,096-atom zincblende SiC cell (8x8x8 cells,
a = 4.36 A, N(0, 0.1 A) jitter, sp3, rc = 5.0 bohr), synthetic Gaussian-
polynomial Fdata, every kernel in FP64 (--prec fp64).  The same step with
the double-float three-center kernels, its agreement with the FP64 result
and with the oracle, the table vs MLP-3c comparison, the DOGS, vnl, Ewald,
McWEDA and Bloch-sum steps, and the Si512, C/H/O 1536 and 256-structure
batch workloads at both precisions ride along as extra keys of the line.

--workload batch256: 256 independent Si / SiC structures of 32..512 atoms in
one batch (one neighbor build + one graph launch per step), compared with
the same 256 structures assembled one after another through the
single-structure calls.

  value  neighbor blocks/s with inputs resident in HBM (device timing, CUDA
         events on the library's stream, L2 flushed between steps)
  e2e    the same metric through the C ABI with host buffers: positions and
         density matrices copied in from pinned memory, S, T, vna, vnao
         blocks and ftot copied out, every step

--impl reference times the CPU restatement of the reference algorithm
(oracle/, OpenMP on all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "thunder-master_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = ("H/S assembly ms/step & neighbor blocks/s: table vs MLP-3c, 1 GB300, |ΔH|<1e-5 Ha")
UNIT = "neighbor blocks/s"
WORKLOADS = {
    "si512": "Si512: 4x4x4 diamond Si, a=5.43 A, N(0,0.15 A) jitter, sp3, rc=5.0 bohr; neighbors + 2c + 3c "
             "H/S + forces, FP64",
    "si64": "Si64: 2x2x2 diamond Si, a=5.43 A, N(0,0.05 A) jitter, sp3, rc=5.0 bohr; neighbors + 2c + 3c H/S "
            "+ forces, FP64",
    "cho1536": "C/H/O 1536 atoms (1:2:1), 24 A box, dmin 1.0 A, rc C 4.5 / O 4.0 / H 4.0 bohr; neighbors + "
               "2c + 3c H/S + forces, FP64",
    "sic4096": "SiC4096: 8x8x8 zincblende SiC, a=4.36 A, N(0,0.1 A) jitter, sp3, rc=5.0 bohr; neighbors + 2c "
               "+ 3c H/S + forces, FP64",
    "batch256": "256 independent structures, 32..512 atoms (seeded), diamond Si (a=5.43 A) or zincblende SiC "
                "(a=4.36 A), N(0,0.1 A) jitter, 0-5% vacancies, sp3, rc=5.0 bohr; one batch: neighbors + 2c + 3c "
                "H/S + forces",
}


def fdata_root():
    return os.environ.get("FBGPU_FDATA_ROOT") or os.path.join(ROOT, "_fdata")


def load_workload(name):
    from fbgpu import synth
    path = synth.fdata_dir_for(name, root=fdata_root())
    st = synth.structure_for(name)
    nZ = [s.nZ for s in synth.species_for(name)]
    return path, nZ, st


def denmat_fast(neighn, neigh_j0, neigh_back0, blk_off, norb_of, seed=42):
    from fbgpu import synth
    return synth.symmetric_denmat(neighn, neigh_j0, neigh_back0, blk_off, norb_of, seed)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # the raw samples go to FBGPU_CLOCKS_DIR (default: the system temp dir)
        import tempfile
        out = os.environ.get("FBGPU_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, "clocks_rank%d.csv" % device)

    @classmethod
    def warm(cls, device):
        """One query ahead of every sampler: the first nvidia-smi start of a
        process (binary and NVML state loaded cold) is the slow one."""
        try:
            subprocess.run(["nvidia-smi", "-i", str(device), "--query-gpu=" + cls.FIELDS,
                            "--format=csv,noheader,nounits"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                           timeout=60)
        except (OSError, subprocess.SubprocessError):
            pass

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # nvidia-smi's start-up (a cold process start, NVML initialisation and
        # its first queries) stalls the driver for several milliseconds: wait
        # for its second sample so that the start-up falls before the timed
        # region, not inside it (measured: one end-to-end step 4.5 ms slower
        # otherwise)
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None:
            with open(self.path) as f:
                if f.read().count("\n") >= 2:
                    break
            time.sleep(0.02)

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        if sm:
            out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# algorithmic work per unit
# ---------------------------------------------------------------------------
# Executed FP64 FLOPs per sp3 x sp3 triplet of the FP64 force kernel
# (2 DFMA + DADD + DMUL: 1,912 + 64 + 334 thread instructions, ncu on
# SiC4096, profiles/k_dassemble_3c_sic4096.md; the divisions and square roots
# are DFMA sequences and count in DFMA)
FP64_FLOP_PER_TRIPLET = 2 * 1911.959 + 64.0 + 333.996


def flops_dassemble_3c(nme, prec="df"):
    """FP64 FLOPs per triplet of the force kernel: the FP64 kernel's executed
    count (ncu), about 3,500 of them the interpolation (Legendre sums first at
    each of the 16 stencil nodes, 4 + 3 FMA per node and element, then the x
    contractions along each stencil row, 3 FMA per node, and the row's y
    weights, 4 FMA per row).  The double-float kernel runs the same
    formulation on the FP32 pipe; this count is its "FP64-equivalent" work."""
    return FP64_FLOP_PER_TRIPLET * (nme / 10.0)


def flops_assemble_3c(nme):
    return 2.0 * (5 * 16 * nme + 5 * nme) + 600.0


def bytes_dassemble_3c(T, P, N, nb_per_pair, table_bytes):
    # triplet list (6 int32 per triplet), rho blocks once per pair, positions,
    # three per-atom force vectors written, tables once
    return T * 24 + P * nb_per_pair * 8 + N * 24 + 3 * N * 24 + table_bytes


def tuned_shapes(ctx, fbgpu, autotune):
    """Autotune the assembly and force kernels on the current system (or keep
    the default shapes); returns the chosen shapes for the JSON line."""
    if autotune:
        ctx.autotune(fbgpu.FB_ALL | fbgpu.FB_FORCES, reps=2)
    return {k: ctx.get_launch(k) for k in fbgpu.TUNABLE}


# Executed FP32 work of the double-float three-center kernels per sp3 x sp3
# triplet (2 FFMA + FADD + FMUL thread instructions: the force kernel
# 6,417 + 19,682 + 2,149, ncu on SiC4096; the value kernel on Si512, the count
# per triplet does not depend on the system size), and the DRAM bytes per
# triplet of one launch (ncu on SiC4096, where the launch's working set
# exceeds what L2 keeps between launches) (profiles/): the df formulation's
# arithmetic is what the FP32 pipe must execute.
DF_FP32_FLOP = {"dassemble_3c": 2 * 6416.868 + 19681.613 + 2148.956, "assemble_3c": 16284.0}
# DRAM read + write bytes per triplet of one force-kernel launch, ncu on
# SiC4096 (profiles/k_dassemble_3c_sic4096.md, 159.30 MB per launch;
# profiles/k_dassemble_3c_df_sic4096.md, 159.65 MB; means of three launches),
# over 5,125,854 triplets
DRAM_BYTES_PER_TRIPLET = {"fp64": 159.295317e6 / 5125854, "df": 159.650645e6 / 5125854}
TRAFFIC_SOURCE = {"fp64": "profiles/k_dassemble_3c_sic4096.md", "df": "profiles/k_dassemble_3c_df_sic4096.md"}


def roofline_for(ctx, ktimes, T, P, natoms, nZ, steps, prec="df", sm_mhz=None):
    """Roofline of the dominant kernel from its CUDA-event launch times.
    Double-float kernels run on the FP32 pipe: achieved = executed FP32
    FLOPs per launch / launch time against the FP32 FFMA peak probed in the
    same run.  FP64 kernels: the algorithmic FP64 FLOPs against the DFMA
    peak.  The FP64-equivalent rate (algorithmic FLOPs of the FP64
    formulation) and the HBM view are reported beside it."""
    dom = max(ktimes, key=lambda k: ktimes[k][0])
    dom_ms = ktimes[dom][0] / max(1, ktimes[dom][1])
    from fbgpu import synth
    nme = len(synth.make_munu_3c([0, 1], [0, 1])[0])
    fl64 = {"dassemble_3c": T * flops_dassemble_3c(nme, prec), "assemble_3c": T * flops_assemble_3c(nme)}.get(dom)
    if fl64 is None:
        return None
    fp64_peak = ctx.probe_fp64()
    ach64 = fl64 / (dom_ms * 1e-3) / 1e12
    table_bytes = 8 * 31 * 31 * 5 * nme * len(nZ) ** 3
    by = bytes_dassemble_3c(T, P, natoms, 16, table_bytes)
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        hbm_peak = json.load(f)["hbm_gbs"]
    hbm = {"achieved": round(by / (dom_ms * 1e-3) / 1e9, 3), "peak": hbm_peak, "unit": "GB/s",
           "frac": round(by / (dom_ms * 1e-3) / 1e9 / hbm_peak, 6), "bytes_per_launch": by,
           "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)"}
    if prec == "df":
        fp32_peak = ctx.probe_fp32()
        fl32 = T * DF_FP32_FLOP[dom]
        ach = fl32 / (dom_ms * 1e-3) / 1e12
        return {"bound": "fp32", "kernel": dom, "achieved": round(ach, 4), "peak": round(fp32_peak, 4),
                "unit": "TFLOP/s", "frac": round(ach / fp32_peak, 4),
                "traffic": round(T * DRAM_BYTES_PER_TRIPLET["df"]) if dom == "dassemble_3c" else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on SiC4096 (%s), "
                                  "scaled by triplets" % TRAFFIC_SOURCE["df"],
                "peak_source": "of measured: fb_probe_fp32 FFMA chains in this run",
                "flops_per_launch": fl32,
                "flops_source": "executed FP32 FLOPs of the double-float kernel (2 FFMA + FADD + FMUL per "
                                "triplet, ncu on SiC4096)",
                "avg_launch_ms": round(dom_ms, 4),
                "fp64_equivalent": {"algorithmic_flops_per_launch": fl64, "achieved": round(ach64, 4),
                                    "fp64_peak": round(fp64_peak, 4), "unit": "TFLOP/s",
                                    "ratio_to_fp64_peak": round(ach64 / fp64_peak, 4)},
                "hbm": hbm}
    # The FP64 pipe executes 2 lanes per SM per clock (an FMA counting as 2
    # FLOP): its rate at the clock sampled under load is the peak.  The
    # DFMA-chain probe is reported beside it; it reaches about 84 % of that
    # rate, below what this kernel's mix of DFMA, DMUL and DADD issues.
    import torch
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    pipe_peak = 4.0 * nsm * (sm_mhz or 2070.0) * 1e6 / 1e12
    return {"bound": "fp64", "kernel": dom, "achieved": round(ach64, 4), "peak": round(pipe_peak, 4),
            "unit": "TFLOP/s", "frac": round(ach64 / pipe_peak, 4),
            "traffic": round(T * DRAM_BYTES_PER_TRIPLET["fp64"]) if dom == "dassemble_3c" else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on SiC4096 (%s), "
                              "scaled by triplets" % TRAFFIC_SOURCE["fp64"],
            "flops_source": "executed FP64 FLOPs per sp3 x sp3 triplet (2 DFMA + DADD + DMUL, ncu on SiC4096, "
                            "profiles/k_dassemble_3c_sic4096.md) x triplets",
            "peak_source": "FP64 pipe rate: 2 lanes per SM per clock x %d SMs x %.0f MHz (median SM clock sampled "
                           "during the timed region), FMA as 2 FLOP; no FP64 figure in MEASURED_PEAKS.json"
                           % (nsm, sm_mhz or 2070.0),
            "probe": {"value": round(fp64_peak, 4), "unit": "TFLOP/s", "frac": round(ach64 / fp64_peak, 4),
                      "what": "fb_probe_fp64: 16 independent DFMA chains per thread, 64 warps per SM, in this run"},
            "flops_per_launch": fl64, "avg_launch_ms": round(dom_ms, 4), "hbm": hbm}


P_HARTREE = 14.39975 / 0.529177          # eV (P_eq2 / P_abohr)
HA_PER_BOHR = P_HARTREE / 0.529177       # eV/Angstrom per Ha/bohr


def mlp_compare(ctx, fbgpu, torch, stream, flush, ws, local, d_rho, d_cape, P, T, steps, epochs, tol_ha=1e-5):
    """Table vs MLP-3c on the current system: train the surrogate on the GPU
    (2^22 samples of the FP64 table interpolator), validate it per bin, then
    time the assembly + force step with the table path, the gated MLP path
    (|dH| <= tol_ha in the worst case) and the ungated MLP path, and measure
    each one's errors against the table path (which equals the FP64 oracle
    to 1e-10 eV)."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.mlp_init(seed=2026)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = ctx.mlp_train(nsamples=1 << 22, epochs=epochs, batch=4096, lr=2e-3, seed=7)
    train_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    max_bin_err = ctx.mlp_validate(samples_per_bin=64, seed=11)
    val_s = time.perf_counter() - t0
    bins = ctx.mlp_bin_errors()
    used = bins[bins > 0]
    what = fbgpu.FB_ALL | fbgpu.FB_FORCES
    timed = make_timer(torch, ctx, stream, flush, ws, local)

    def step():
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.assemble_graph(what)

    def run(mode, tol=None):
        info = {}
        if mode == fbgpu.FB_MLP_GATED:
            tau, cov = ctx.mlp_gate(tol)
            info.update(tol_ha=tol, tau_table_units=tau, coverage=round(cov, 6))
        else:
            ctx.mlp_set_mode(mode)
        for _ in range(2):
            step()
        ms, launches = timed(step, steps)
        out = {k: ctx.blocks(k) for k in ("S", "vna")}
        out["ftot"] = ctx.forces("ftot")
        info.update(ms_per_step=round(ms / steps, 4), value=round(P * steps / (ms * 1e-3), 1),
                    gpu_launches_per_step=launches // steps, triplets_to_network=ctx.mlp_routed()[0])
        return info, out

    table, ref = run(fbgpu.FB_MLP_OFF)
    res = {"table": table}
    for name, mode, tol, engine in (("mlp_gated", fbgpu.FB_MLP_GATED, tol_ha, fbgpu.FB_MLP_ENGINE_TC),
                                    ("mlp_all", fbgpu.FB_MLP_ALL, None, fbgpu.FB_MLP_ENGINE_TC),
                                    ("mlp_all_mma_sync", fbgpu.FB_MLP_ALL, None, fbgpu.FB_MLP_ENGINE_MMA)):
        ctx.mlp_set_engine(engine)
        info, out = run(mode, tol)
        info["engine"] = "tcgen05 (TMEM)" if engine == fbgpu.FB_MLP_ENGINE_TC else "mma.sync"
        dH = (out["vna"] - ref["vna"]) / P_HARTREE
        dS = out["S"] - ref["S"]
        dF = (out["ftot"] - ref["ftot"]) / HA_PER_BOHR
        info.update(max_abs_dH_ha=float(np.abs(dH).max()), rms_dH_ha=float(np.sqrt(np.mean(dH * dH))),
                    max_abs_dS=float(np.abs(dS).max()), rms_dS=float(np.sqrt(np.mean(dS * dS))),
                    max_abs_dF_ha_per_bohr=float(np.abs(dF).max()),
                    rms_dF_ha_per_bohr=float(np.sqrt(np.mean(dF * dF))),
                    speedup_vs_table=round(table["ms_per_step"] / info["ms_per_step"], 4))
        res[name] = info
    # per-kernel device times of the ungated MLP path through the separate calls
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_TC)
    ctx.mlp_set_mode(fbgpu.FB_MLP_ALL)

    def kstep():
        ctx.assemble(fbgpu.FB_ALL)
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.Dassemble(fbgpu.FB_ALL)
    kstep()
    timed(kstep, steps, timing=True)
    res["mlp_all"]["kernels_ms_per_step"] = {k: round(v[0] / steps, 4) for k, v in ctx.timing().items() if v[1]}
    ctx.set_timing(False)
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)
    res["training"] = {"samples": 1 << 22, "epochs": epochs, "batch": 4096, "seconds": round(train_s, 2),
                       "loss_first_last": [float(hist[0]), float(hist[-1])],
                       "validation_seconds": round(val_s, 2), "bins": int(len(used)),
                       "bin_error_table_units": {"max": float(max_bin_err), "median": float(np.median(used)),
                                                 "p10": float(np.quantile(used, 0.1))}}
    res["network"] = "3 inputs (each a BF16 hi/lo pair) + 16-float species-triple embedding, 3 x 128 SiLU, " \
                     "50 Legendre coefficients; BF16 weights, FP32 accumulation; evaluated on tcgen05 " \
                     "(UMMA 128xNx16, TMEM accumulators), trained with mma.sync m16n8k16 GEMMs"
    return res


PREC_NAME = {0: "fp64", 1: "df"}


def measure_single(args, ctx, fbgpu, torch, stream, flush, ws, local, st, NB, rho, cape, d_rho, d_cape, prec,
                   steps, warmup, e2e=True, clocks=False, autotune=True):
    """Time one step of the path on the structure already on ctx, at one
    precision of the three-center kernels: the device step (inputs in HBM),
    the end-to-end step through the C ABI with pinned host buffers, and the
    separate calls with per-kernel CUDA-event timing.  Returns the timings
    and the step's outputs (S, T, vna, vnao, ftot)."""
    ctx.set_precision(prec)
    ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
    shapes = tuned_shapes(ctx, fbgpu, autotune)
    step_what = fbgpu.FB_ALL | fbgpu.FB_FORCES

    def device_step():
        ctx.driver_neighbors()
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.assemble_graph(step_what)

    def kernel_step():
        # the same work through the separate calls, for per-kernel timing
        ctx.driver_neighbors()
        ctx.assemble(fbgpu.FB_ALL)
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.Dassemble(fbgpu.FB_ALL)

    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    h_pos = pin(3 * st.natoms)
    h_pos[:] = st.ratom.ravel()
    h_rho, h_cape = pin(NB), pin(NB)
    h_rho[:] = rho
    h_cape[:] = cape
    h_out = [pin(NB) for _ in range(4)]
    h_f = pin(3 * st.natoms)

    import ctypes as C
    ptrs = [C.c_void_p(a.ctypes.data) for a in (h_pos, h_rho, h_cape, *h_out, h_f)]

    def e2e_step():
        # one call: positions and density matrices in, S, T, vna, vnao and
        # ftot out, the copies overlapped with the kernels (fb_step_forces)
        ctx._check(ctx.L.fb_step_forces(ctx.h, *ptrs))

    def e2e_calls_step():
        # the same through the separate calls (each copy synchronous)
        ctx.update_positions(h_pos)
        ctx.driver_neighbors()
        ctx.set_denmat(h_rho, h_cape)
        ctx.assemble_graph(step_what)
        for key, buf in zip(("S", "T", "vna", "vnao"), h_out):
            ctx._check(ctx.L.fb_get_blocks(ctx.h, fbgpu.BLOCK[key], buf))
        ctx._check(ctx.L.fb_get_forces(ctx.h, fbgpu.FORCE["ftot"], h_f))

    timed = make_timer(torch, ctx, stream, flush, ws, local)
    for _ in range(warmup):
        device_step()
        if e2e:
            e2e_step()
            e2e_calls_step()
        kernel_step()
    sampler = ClockSampler(local) if clocks else None
    if sampler:
        sampler.start()
    ms, launches = timed(device_step, steps)
    if e2e:
        e2e_step()  # (one more untimed step right before the timed ones)
    ms_e2e = timed(e2e_step, steps)[0] if e2e else None
    ms_e2e_calls = timed(e2e_calls_step, steps)[0] if e2e else None
    clk = sampler.stop() if sampler else None
    out = {k: ctx.blocks(k) for k in ("S", "T", "vna", "vnao")}
    out["ftot"] = ctx.forces("ftot")
    ms_k, _ = timed(kernel_step, steps, timing=True)
    ktimes = ctx.timing()
    ctx.set_timing(False)
    return {"ms": ms, "ms_e2e": ms_e2e, "ms_e2e_calls": ms_e2e_calls, "launches": launches, "ktimes": ktimes,
            "ms_k": ms_k, "clocks": clk, "shapes": shapes, "out": out, "prec": PREC_NAME[prec]}


def max_abs_diffs(a, b):
    """Largest |a - b| per output: blocks in eV, ftot in eV/Angstrom."""
    return {k: float(np.abs(a[k] - b[k]).max()) for k in ("S", "T", "vna", "vnao", "ftot")}


def run_gpu(args):
    import torch
    import fbgpu
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    ClockSampler.warm(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.workload == "batch256":
        return run_batch(args, torch, fbgpu, ws, rank, local)
    path, nZ, st = load_workload(args.workload)
    ctx = fbgpu.Context(local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, NB = ctx.driver_neighbors()
    nbm = ctx.neighbors()
    norb_of = np.array([ctx.norb_species[k - 1] for k in st.imass])
    rho, cape = denmat_fast(nbm["neighn"], nbm["neigh_j"] - 1, nbm["neigh_back"] - 1, nbm["blk_off"], norb_of)
    d_rho = torch.from_numpy(rho).to(f"cuda:{local}")
    d_cape = torch.from_numpy(cape).to(f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    prec_main = fbgpu.FB_PREC_FP64 if args.prec == "fp64" else fbgpu.FB_PREC_DF
    prec_other = fbgpu.FB_PREC_DF if prec_main == fbgpu.FB_PREC_FP64 else fbgpu.FB_PREC_FP64
    common = (args, ctx, fbgpu, torch, stream, flush, ws, local, st, NB, rho, cape, d_rho, d_cape)
    m = measure_single(*common, prec_main, args.steps, args.warmup, e2e=True, clocks=True,
                       autotune=not args.no_autotune)
    o = measure_single(*common, prec_other, args.steps, max(3, min(args.warmup, 3)), e2e=True,
                       autotune=not args.no_autotune)
    ctx.set_precision(prec_main)

    per_step = m["ms"] / args.steps
    value = ws * P * args.steps / (m["ms"] * 1e-3)
    e2e_value = ws * P * args.steps / (m["ms_e2e"] * 1e-3)
    h2d = 3 * st.natoms * 8 + 2 * NB * 8
    d2h = 4 * NB * 8 + 3 * st.natoms * 8
    roof = roofline_for(ctx, m["ktimes"], T, P, st.natoms, nZ, args.steps, m["prec"],
                        (m["clocks"] or {}).get("sm_mhz"))
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if m["prec"] == "fp64" else "f64 (three-center: double-float f32x2)",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "natoms": st.natoms, "pairs": P, "triplets": T,
                   "three_center_arithmetic": "fp64" if m["prec"] == "fp64" else "double-float (FP32 pipe)",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "flushed between steps (256 MiB write)", "forces": True,
                   "step": "fb_neighbors + one CUDA graph launch (assembly + forces)",
                   "launch_shapes": m["shapes"], "autotuned": not args.no_autotune},
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(m["ms_e2e"] / args.steps, 4),
                "how": "fb_step_forces: positions and rho/cape in from pinned host memory, S, T, vna, vnao and "
                       "ftot out, every step, the copies overlapped with the kernels",
                "separate_calls": {"value": round(ws * P * args.steps / (m["ms_e2e_calls"] * 1e-3), 1),
                                   "ms_per_step": round(m["ms_e2e_calls"] / args.steps, 4),
                                   "how": "fb_update_positions, fb_neighbors, fb_set_denmat, fb_assemble_graph, "
                                          "fb_get_blocks x 4, fb_get_forces (each copy synchronous)"}},
        "gpu_launches": m["launches"],
        "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in m["ktimes"].items() if v[1]},
        "separate_calls_ms_per_step": round(m["ms_k"] / args.steps, 4),
        "roofline": roof,
        "clocks": m["clocks"],
    }
    # the same step with the other precision of the three-center kernels
    line["double_float" if o["prec"] == "df" else "fp64_path"] = {
        "what": ("three-center kernels in double-float (f32 pairs, 48-bit significand) on the FP32 pipe; every "
                 "data-selecting decision in FP64") if o["prec"] == "df" else "every kernel in FP64",
        "ms_per_step": round(o["ms"] / args.steps, 4), "value": round(ws * P * args.steps / (o["ms"] * 1e-3), 1),
        "unit": UNIT, "e2e": {"value": round(ws * P * args.steps / (o["ms_e2e"] * 1e-3), 1),
                              "ms_per_step": round(o["ms_e2e"] / args.steps, 4)},
        "speedup_vs_headline": round(m["ms"] / o["ms"], 4),
        "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in o["ktimes"].items() if v[1]},
        "roofline": roofline_for(ctx, o["ktimes"], T, P, st.natoms, nZ, args.steps, o["prec"],
                                 (m["clocks"] or {}).get("sm_mhz")),
        "launch_shapes": o["shapes"],
        "max_abs_diff_vs_headline": max_abs_diffs(o["out"], m["out"])}
    legs = set(args.legs.split(",")) if args.legs != "none" else set()
    if rank == 0:
        if "bloch" in legs:
            line["bloch"] = bloch_measure(ctx, torch, stream, local)
        if "solve" in legs:
            line["solve_k"] = solve_measure(args, fbgpu, torch, stream, local)
        if "dogs" in legs:
            line["dogs"] = dogs_measure(args, fbgpu, torch, stream, flush, ws, local, st, nZ, no_cpu=args.no_cpu)
        if "vnl" in legs:
            line["vnl"] = vnl_measure(args, fbgpu, torch, stream, flush, local, path, st, nZ, no_cpu=args.no_cpu)
        if "vxc" in legs:
            line["vxc"] = vxc_measure(args, fbgpu, torch, stream, flush, local, st, nZ, no_cpu=args.no_cpu)
    if args.mlp_epochs > 0:
        ctx.set_precision(prec_main)
        line["mlp3c"] = mlp_compare(ctx, fbgpu, torch, stream, flush, ws, local, d_rho, d_cape, P, T,
                                    args.steps, args.mlp_epochs)
    if rank == 0 and args.extra_workloads and args.extra_workloads != "none":
        line["workloads"] = {}
        for name in args.extra_workloads.split(","):
            if name and name != args.workload:
                line["workloads"][name] = (measure_batch_extra(args, torch, fbgpu, local) if name == "batch256"
                                           else measure_other_workload(args, name, fbgpu, torch, stream, flush,
                                                                       local))
    if rank == 0 and not args.no_cpu:
        cb, ref = cpu_baseline(args.workload, path, nZ, st, P, keep=True)
        line["cpu_baseline"] = cb
        if ref is not None:
            line["parity_vs_oracle"] = {
                "what": "max |GPU - oracle| in this run, same structure and density matrices (eV, eV/Angstrom)",
                m["prec"]: max_abs_diffs(m["out"], ref), o["prec"]: max_abs_diffs(o["out"], ref),
                "max_abs_ftot_ev_per_A": float(np.abs(ref["ftot"]).max()),
                "tolerance": "blocks 1e-10 eV; forces 1e-10 of the largest component (the reference algorithm "
                             "built with and without FMA contraction differs by ~1e-11 of it)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def measure_other_workload(args, name, fbgpu, torch, stream, flush, local):
    """Device step of another single-structure workload at both precisions
    (neighbors + one graph launch of assembly and forces)."""
    path, nZ, st = load_workload(name)
    ctx = fbgpu.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, NB = ctx.driver_neighbors()
    nbm = ctx.neighbors()
    norb_of = np.array([ctx.norb_species[k - 1] for k in st.imass])
    rho, cape = denmat_fast(nbm["neighn"], nbm["neigh_j"] - 1, nbm["neigh_back"] - 1, nbm["blk_off"], norb_of)
    d_rho = torch.from_numpy(rho).to(f"cuda:{local}")
    d_cape = torch.from_numpy(cape).to(f"cuda:{local}")
    out = {"workload": WORKLOADS[name], "natoms": st.natoms, "pairs": P, "triplets": T}
    res = {}
    for prec in (fbgpu.FB_PREC_FP64, fbgpu.FB_PREC_DF):
        r = measure_single(args, ctx, fbgpu, torch, stream, flush, 1, local, st, NB, rho, cape, d_rho, d_cape,
                           prec, args.steps, 3, e2e=False, autotune=not args.no_autotune)
        res[r["prec"]] = r
        out[r["prec"]] = {"ms_per_step": round(r["ms"] / args.steps, 4),
                          "value": round(P * args.steps / (r["ms"] * 1e-3), 1), "unit": UNIT,
                          "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in r["ktimes"].items()
                                                  if v[1]}}
    out["df_max_abs_diff_vs_fp64"] = max_abs_diffs(res["df"]["out"], res["fp64"]["out"])
    ctx.close()
    return out


def bloch_measure(ctx, torch, stream, local, reps=5):
    """Bloch sums of the assembled blocks into dense complex H(k) and S(k)
    at one general k-point (h.SOLVESH/M_kspace_Lowdin.f90), on the device."""
    import fbgpu
    ctx.assemble(fbgpu.FB_ALL)
    n = int(ctx.L.fb_norbitals(ctx.h))
    hk = torch.empty((n, n), dtype=torch.complex128, device=f"cuda:{local}")
    sk = torch.empty((n, n), dtype=torch.complex128, device=f"cuda:{local}")
    k = np.array([[0.11, -0.23, 0.31]])
    ctx.bloch_device(k, hk.data_ptr(), sk.data_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        ctx.bloch_device(k, hk.data_ptr(), sk.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = 2 * n * n * 16
    herm = float((hk - hk.conj().T).abs().max().item())
    del hk, sk
    return {"what": "dense complex H(k) = T + vna + vnao and S(k) at one k-point (Bloch sums of the blocks)",
            "norbitals": n, "ms": round(ms, 4), "bytes_written": nbytes,
            "hbm_gbs": round(nbytes / (ms * 1e-3) / 1e9, 1), "hermiticity_max_abs": herm}


def solve_measure(args, fbgpu, torch, stream, local, name="si512", nk=2):
    """The k-point Lowdin solver (kspace_Lowdin: Bloch sums, eigenpairs of
    S(k), S^-1/2, eigenpairs of S^-1/2 H S^-1/2, c = S^-1/2 c_Lowdin) on
    Si512 (2,048 orbitals), per k-point, and its agreement with the
    oracle's numpy restatement on the oracle's Bloch sums."""
    path, nZ, st = load_workload(name)
    ctx = fbgpu.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.assemble(fbgpu.FB_ALL)
    n = int(ctx.L.fb_norbitals(ctx.h))
    kpts = np.array([[0.11, -0.23, 0.31], [0.0, 0.0, 0.0]])[:nk]
    c = torch.empty((nk, n, n, 2), dtype=torch.float64, device=f"cuda:{local}")
    ctx.solve_k(kpts[:1], c_ptr=c.data_ptr())  # workspace + library load
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eig, dropped = ctx.solve_k(kpts, c_ptr=c.data_ptr())
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / nk
    out = {"what": "kspace_Lowdin per k-point on %s: Bloch sums + zheevd(S) + Lowdin S^-1/2 + zheevd(S^-1/2 H "
                   "S^-1/2) + c = S^-1/2 c_L (cuSOLVER / cuBLAS FP64, own kernels for the sums and scaling)" % name,
           "norbitals": n, "kpoints": nk, "ms_per_kpoint": round(dt * 1e3, 2),
           "dropped_overlap_eigenvalues": [int(x) for x in dropped]}
    del c
    ctx.close()
    if not args.no_cpu:
        from oracle import lowdin
        from oracle import oracle as orc
        s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice, threads=os.cpu_count() or 1).neighbors()
        S, T, vb, vbo = s.assemble()
        t0 = time.perf_counter()
        err = 0.0
        for k in range(nk):
            eps = lowdin.solve_k(s.bloch(kpts[k:k + 1], T + vb + vbo)[0], s.bloch(kpts[k:k + 1], S)[0])[0]
            err = max(err, float(np.abs(eps - eig[k]).max()))
        out["max_abs_deig_ev"] = err
        out["cpu_numpy_s_per_kpoint"] = round((time.perf_counter() - t0) / nk, 3)
    return out


def dogs_measure(args, fbgpu, torch, stream, flush, ws, local, st, nZ, no_cpu=False):
    """The DOGS step (charge-weighted vna, M_assemble_*_DOGS.f90 and
    M_Dassemble_*_DOGS.f90) on the same structure with seeded shell charges:
    fb_neighbors + one graph launch of the value and force pass (FP64
    kernels), its agreement with the oracle's DOGS restatement, and the
    oracle's time for the same step on one host core."""
    from fbgpu import synth
    path = synth.fdata_dir_for(args.workload, root=fdata_root(), dogs=True)
    ctx = fbgpu.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, NB = ctx.driver_neighbors()
    nbm = ctx.neighbors()
    norb_of = np.array([ctx.norb_species[k - 1] for k in st.imass])
    rho, cape = denmat_fast(nbm["neighn"], nbm["neigh_j"] - 1, nbm["neigh_back"] - 1, nbm["blk_off"], norb_of)
    dq = np.random.default_rng(5).uniform(-0.3, 0.3, (st.natoms, 3))
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(dq)
    d_rho = torch.from_numpy(rho).to(f"cuda:{local}")
    d_cape = torch.from_numpy(cape).to(f"cuda:{local}")
    what = fbgpu.FB_ALL | fbgpu.FB_FORCES
    ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
    shapes = tuned_shapes(ctx, fbgpu, not args.no_autotune)

    def step():
        ctx.driver_neighbors()
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.assemble_graph(what)

    timed = make_timer(torch, ctx, stream, flush, 1, local)
    for _ in range(max(3, args.warmup)):
        step()
    ms, launches = timed(step, args.steps)
    ms_k, _ = timed(lambda: (ctx.driver_neighbors(), ctx.assemble(fbgpu.FB_ALL),
                             ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr()),
                             ctx.Dassemble(fbgpu.FB_ALL)), args.steps, timing=True)
    ktimes = ctx.timing()
    ctx.set_timing(False)
    out = {"what": "DOGS value + force pass (charged-shell sub-cells, smoothed monopoles), FP64 kernels, "
                   "shell charges U(-0.3, 0.3) seeded",
           "ms_per_step": round(ms / args.steps, 4), "value": round(P * args.steps / (ms * 1e-3), 1),
           "unit": UNIT, "gpu_launches_per_step": launches // max(1, args.steps),
           "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in ktimes.items() if v[1]},
           "launch_shapes": shapes}
    # the Ewald terms (matrix + ewaldsr + ewaldlr) on top of the DOGS value pass
    ctx.assemble(fbgpu.FB_ALL)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.assemble(fbgpu.FB_EWALD)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        ctx.assemble(fbgpu.FB_EWALD)
    e1.record(stream)
    torch.cuda.synchronize()
    out["ewald"] = {"what": "DOGS Ewald: N x N matrix (reciprocal + screened lattice sums), ewaldsr, ewaldlr",
                    "ms": round(e0.elapsed_time(e1) / args.steps, 4)}
    ctx.set_timing(True)
    ctx.assemble(fbgpu.FB_EWALD)
    torch.cuda.synchronize()
    out["ewald"]["kernels_ms"] = {k: round(v[0], 4) for k, v in ctx.timing().items() if v[1]}
    ctx.set_timing(False)
    ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
    ctx.Dassemble(fbgpu.FB_EWALD)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        ctx.Dassemble(fbgpu.FB_EWALD)
    e1.record(stream)
    torch.cuda.synchronize()
    out["ewald"]["force_ms"] = round(e0.elapsed_time(e1) / args.steps, 4)
    ctx.set_timing(True)
    ctx.Dassemble(fbgpu.FB_EWALD)
    torch.cuda.synchronize()
    out["ewald"]["force_kernels_ms"] = {k: round(v[0], 4) for k, v in ctx.timing().items() if v[1]}
    ctx.set_timing(False)
    out["ewald"]["force_what"] = ("dewald + Ewald energy force, ewaldsr (pair + three-center) and ewaldlr forces, "
                                  "build_forces terms")
    ew_gpu = ctx.ewald()
    sr_gpu, lr_gpu = ctx.blocks("ewaldsr"), ctx.blocks("ewaldlr")
    # the same Ewald passes with the FP64 lattice and reciprocal sums
    ctx.set_precision(fbgpu.FB_PREC_FP64)
    ctx.assemble(fbgpu.FB_EWALD)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.assemble(fbgpu.FB_EWALD)
    e1.record(stream)
    torch.cuda.synchronize()
    out["ewald"]["fp64_ms"] = round(e0.elapsed_time(e1), 4)
    out["ewald"]["fp64_max_abs_dewald_matrix_vs_df"] = float(np.abs(ctx.ewald() - ew_gpu).max())
    e0.record(stream)
    ctx.Dassemble(fbgpu.FB_EWALD)
    e1.record(stream)
    torch.cuda.synchronize()
    out["ewald"]["fp64_force_ms"] = round(e0.elapsed_time(e1), 4)
    ctx.set_precision(fbgpu.FB_PREC_DF)
    # agreement with the oracle and the oracle's single-core time
    got = {k: ctx.blocks(k) for k in ("vna", "vnao")}
    ctx.set_denmat(rho, cape)
    ctx.Dassemble()
    f_gpu = ctx.forces("ftot")
    ctx.close()
    if no_cpu or st.natoms > 1024:
        out["cpu_oracle"] = "not run (single-core oracle bounded to systems of at most 1024 atoms)"
    else:
        from oracle import oracle as orc
        fd = orc.Fdata(path, nZ)
        t0 = time.perf_counter()
        s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
        ref = s.assemble_dogs(dq)
        d = s.dassemble_dogs(rho, cape, dq)
        t = time.perf_counter() - t0
        out["max_abs_dvna_ev"] = float(max(np.abs(got["vna"] - ref[2]).max(), np.abs(got["vnao"] - ref[3]).max()))
        t0 = time.perf_counter()
        ew, sr, lr = s.assemble_ewald(dq)
        out["ewald"]["cpu_oracle_s"] = round(time.perf_counter() - t0, 3)
        out["ewald"]["max_abs_dewald"] = float(np.abs(ew_gpu - ew).max())
        out["ewald"]["max_abs_dsr_lr_ev"] = float(max(np.abs(sr_gpu - sr).max(), np.abs(lr_gpu - lr).max()))
        out["max_abs_dftot_ev_per_A"] = float(np.abs(f_gpu - d["ftot"]).max())
        out["cpu_oracle"] = {"value": round(P / t, 1), "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "1 DOGS step (neighbors + value + force pass), %.3f s" % t}
    return out


def vnl_measure(args, fbgpu, torch, stream, flush, local, path, st, nZ, no_cpu=False):
    """The non-local pseudopotential step on the same structure: the PP maps
    (driver_neighbors_PP), svnl + vnl 2c/3c and the vnl force pass as one
    graph launch, with a seeded density over the PPp pairs; its agreement
    with the oracle and the oracle's time for the same step on one core."""
    ctx = fbgpu.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    sz = ctx.driver_neighbors_PP()
    rho_pp = np.random.default_rng(11).normal(0.0, 0.1, sz["nvnl"])
    d_rho = torch.from_numpy(rho_pp).to(f"cuda:{local}")
    ctx.set_denmat_pp_device(d_rho.data_ptr())
    what = fbgpu.FB_VNL | fbgpu.FB_FORCES

    def step():
        ctx.driver_neighbors_PP()
        ctx.set_denmat_pp_device(d_rho.data_ptr())
        ctx.assemble_graph(what)

    timed = make_timer(torch, ctx, stream, flush, 1, local)
    for _ in range(max(3, args.warmup)):
        step()
    ms, launches = timed(step, args.steps)
    ms_k, _ = timed(lambda: (ctx.driver_neighbors_PP(), ctx.set_denmat_pp_device(d_rho.data_ptr()),
                             ctx.assemble(fbgpu.FB_VNL), ctx.Dassemble(fbgpu.FB_VNL2C | fbgpu.FB_VNL3C)),
                    args.steps, timing=True)
    kt = ctx.timing()
    ctx.set_timing(False)
    out = {"what": "vnl: PP/PPx/PPp maps + common triplets, svnl, vnl 2c + 3c, vnl forces (FP64)",
           "sizes": sz, "ms_per_step": round(ms / args.steps, 4),
           "value": round(sz["nppp"] * args.steps / (ms * 1e-3), 1), "unit": "vnl blocks (PPp pairs)/s",
           "gpu_launches_per_step": launches // max(1, args.steps),
           "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in kt.items() if v[1]}}
    vnl = ctx.blocks("vnl")
    ctx.set_denmat_pp(rho_pp)
    ctx.Dassemble(fbgpu.FB_VNL2C | fbgpu.FB_VNL3C)
    f_gpu = ctx.forces("ftot")
    ctx.close()
    if no_cpu or st.natoms > 1024:
        out["cpu_oracle"] = "not run (single-core oracle bounded to systems of at most 1024 atoms)"
    else:
        from oracle import oracle as orc
        fd = orc.Fdata(path, nZ)
        t0 = time.perf_counter()
        s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors().neighbors_pp()
        _, vref = s.assemble_pp()
        d = s.dassemble_pp(rho_pp)
        t = time.perf_counter() - t0
        out["max_abs_dvnl_ev"] = float(np.abs(vnl - vref).max())
        out["max_abs_dftot_ev_per_A"] = float(np.abs(f_gpu - d["ftot_vnl"]).max())
        out["cpu_oracle"] = {"value": round(s.nppp / t, 1), "unit": "vnl blocks (PPp pairs)/s", "cores": 1,
                             "kind": "port", "sample": "1 vnl step (maps + value + force pass), %.3f s" % t}
    return out


def vxc_measure(args, fbgpu, torch, stream, flush, local, st, nZ, no_cpu=False):
    """The McWEDA exchange-correlation step (Harris) on the same structure,
    with the Fdata set that carries the McWEDA tables: neighbors, then the
    overlap, the input densities (2c + 3c) and the vxc blocks as one graph
    launch; its agreement with the oracle and the oracle's time for the
    same step on one core."""
    from fbgpu import synth
    path = synth.fdata_dir_for(args.workload, root=fdata_root(), vxc=True)
    ctx = fbgpu.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, _ = ctx.driver_neighbors()
    what = fbgpu.FB_S | fbgpu.FB_VXC

    def step():
        ctx.driver_neighbors()
        ctx.assemble_graph(what)

    timed = make_timer(torch, ctx, stream, flush, 1, local)
    for _ in range(max(3, args.warmup)):
        step()
    ms, launches = timed(step, args.steps)
    timed(lambda: (ctx.driver_neighbors(), ctx.assemble(what)), args.steps, timing=True)
    kt = ctx.timing()
    ctx.set_timing(False)
    out = {"what": "McWEDA vxc (Harris): overlap, rho_in / rho_bond and weighted densities (2c + 3c), "
                   "Ceperley-Alder SN terms, vxc_bond; FP64 (three-center densities double-float)",
           "ms_per_step": round(ms / args.steps, 4), "value": round(P * args.steps / (ms * 1e-3), 1),
           "unit": "neighbor blocks/s", "gpu_launches_per_step": launches // max(1, args.steps),
           "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in kt.items() if v[1]}}
    vxc = ctx.blocks("vxc")
    # the force pass too (Dassemble_vxc with the S, T and vna force terms of
    # build_forces), with a seeded density matrix, as one graph
    nb = ctx.nblock
    rng = np.random.default_rng(7)
    d_rho = torch.from_numpy(rng.normal(0.0, 0.1, nb)).to(f"cuda:{local}")
    d_cape = torch.from_numpy(rng.normal(0.0, 0.05, nb)).to(f"cuda:{local}")
    ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
    whatf = fbgpu.FB_ALL | fbgpu.FB_VXC | fbgpu.FB_FORCES

    def stepf():
        ctx.driver_neighbors()
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.assemble_graph(whatf)

    for _ in range(max(3, args.warmup)):
        stepf()
    msf, lf = timed(stepf, args.steps)
    timed(lambda: (ctx.driver_neighbors(), ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr()),
                   ctx.assemble(fbgpu.FB_ALL | fbgpu.FB_VXC),
                   ctx.Dassemble(fbgpu.FB_ALL | fbgpu.FB_VXC)), args.steps, timing=True)
    ktf = ctx.timing()
    ctx.set_timing(False)
    out["with_forces"] = {"what": "Harris S, T, vna + McWEDA vxc, value and force pass (Dassemble_vxc and the "
                                  "build_forces terms), one graph",
                          "ms_per_step": round(msf / args.steps, 4),
                          "value": round(P * args.steps / (msf * 1e-3), 1), "unit": "neighbor blocks/s",
                          "gpu_launches_per_step": lf // max(1, args.steps),
                          "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in ktf.items() if v[1]}}
    ctx.close()
    if no_cpu or st.natoms > 1024:
        out["cpu_oracle"] = "not run (single-core oracle bounded to systems of at most 1024 atoms)"
    else:
        from oracle import oracle as orc
        fd = orc.Fdata(path, nZ)
        t0 = time.perf_counter()
        s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
        ref = s.assemble_vxc()
        t = time.perf_counter() - t0
        out["max_abs_dvxc_ev"] = float(np.abs(vxc - ref["vxc"]).max())
        out["cpu_oracle"] = {"value": round(s.npairs / t, 1), "unit": "neighbor blocks/s", "cores": 1,
                             "kind": "port", "sample": "1 vxc step (neighbors + overlap + densities + vxc), %.3f s" % t}
    return out


def make_timer(torch, ctx, stream, flush, ws, local):
    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed(step, nsteps, timing=False):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        barrier()
        if timing:
            ctx.set_timing(True)
        l0 = ctx.kernel_launches()
        for k in range(nsteps):
            with torch.cuda.stream(stream):
                flush.zero_()
            evs[k][0].record(stream)
            step()
            evs[k][1].record(stream)
        barrier()
        launches = ctx.kernel_launches() - l0
        ms = sum(a.elapsed_time(b) for a, b in evs)
        if ws > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, launches
    return timed


def batch_inputs(structs, ctx, fbgpu):
    """Seeded symmetric density matrices of a batch (global numbering)."""
    nbm = ctx.neighbors()
    off = ctx.batch_offsets()
    sid = np.repeat(np.arange(len(structs)), np.diff(off["atom"]))
    owner = np.repeat(np.arange(len(nbm["neighn"])), nbm["neighn"])
    jg = nbm["neigh_j"] - 1 + off["atom"][sid[owner]]
    imass = np.concatenate([st.imass for st in structs])
    norb_of = np.array([ctx.norb_species[k - 1] for k in imass])
    return denmat_fast(nbm["neighn"], jg, nbm["neigh_back"] - 1, nbm["blk_off"], norb_of)


def measure_batch(args, torch, fbgpu, ws, local, prec, steps, warmup, e2e=True, clocks=False, seq_steps=3):
    """Config 4: 256 structures of uneven size in one batch (one neighbor
    build + one graph launch per step), against the same structures
    assembled one at a time through the single-structure calls."""
    from fbgpu import synth
    path = synth.fdata_dir_for("batch256", root=fdata_root())
    nZ = [s.nZ for s in synth.species_for("batch256")]
    structs = synth.batch_structures(256)
    ctx = fbgpu.Context(local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    ctx.read_Fdata(path, nZ)
    ctx.set_precision(prec)
    ctx.set_batch([(st.ratom, st.imass, st.lattice, 0) for st in structs])
    P, T, NB = ctx.driver_neighbors()
    off = ctx.batch_offsets()
    rho, cape = batch_inputs(structs, ctx, fbgpu)
    dev = f"cuda:{local}"
    d_rho = torch.from_numpy(rho).to(dev)
    d_cape = torch.from_numpy(cape).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
    shapes = tuned_shapes(ctx, fbgpu, not args.no_autotune)
    step_what = fbgpu.FB_ALL | fbgpu.FB_FORCES
    natoms = int(off["atom"][-1])

    def batch_step():
        ctx.driver_neighbors()
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.assemble_graph(step_what)

    # the same structures one at a time through the single-structure calls
    seq = fbgpu.Context(local)
    seq.set_stream(stream.cuda_stream)
    seq.read_Fdata(path, nZ)
    seq.set_precision(prec)
    bo = off["block"]

    def sequential_step():
        for k, st in enumerate(structs):
            seq.set_structure(st.ratom, st.imass, st.lattice)
            seq.driver_neighbors()
            seq.assemble(fbgpu.FB_ALL)
            seq.set_denmat_device(d_rho.data_ptr() + 8 * int(bo[k]), d_cape.data_ptr() + 8 * int(bo[k]))
            seq.Dassemble(fbgpu.FB_ALL)

    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    h_pos = pin(3 * natoms)
    h_pos[:] = np.concatenate([st.ratom.ravel() for st in structs])
    h_rho, h_cape = pin(NB), pin(NB)
    h_rho[:] = rho
    h_cape[:] = cape
    h_out = [pin(NB) for _ in range(4)]
    h_f = pin(3 * natoms)

    import ctypes as C
    ptrs = [C.c_void_p(a.ctypes.data) for a in (h_pos, h_rho, h_cape, *h_out, h_f)]

    def e2e_step():
        ctx._check(ctx.L.fb_step_forces(ctx.h, *ptrs))

    timed = make_timer(torch, ctx, stream, flush, ws, local)
    for _ in range(warmup):
        batch_step()
        if e2e:
            e2e_step()
    sequential_step()
    sampler = ClockSampler(local) if clocks else None
    if sampler:
        sampler.start()
    ms, launches = timed(batch_step, steps)
    ms_e2e = timed(e2e_step, steps)[0] if e2e else None
    clk = sampler.stop() if sampler else None
    ftot_batch = ctx.forces("ftot")
    ms_seq, seq_launches = make_timer(torch, seq, stream, flush, ws, local)(sequential_step, seq_steps)
    # the last structure of the sequential pass against its slice of the batch
    last = len(structs) - 1
    f_last = seq.forces("ftot")
    seq_diff = float(np.abs(f_last - ftot_batch[3 * int(off["atom"][last]):3 * int(off["atom"][last + 1])]).max())

    def kernel_step():
        ctx.driver_neighbors()
        ctx.assemble(fbgpu.FB_ALL)
        ctx.set_denmat_device(d_rho.data_ptr(), d_cape.data_ptr())
        ctx.Dassemble(fbgpu.FB_ALL)
    kernel_step()
    ms_k, _ = timed(kernel_step, steps, timing=True)
    ktimes = ctx.timing()
    ctx.set_timing(False)
    roof = roofline_for(ctx, ktimes, T, P, natoms, nZ, steps, PREC_NAME[prec])
    sizes = np.diff(off["atom"])
    seq.close()
    ctx.close()
    return {"structs": structs, "path": path, "nZ": nZ, "P": P, "T": T, "NB": NB, "natoms": natoms,
            "sizes": sizes, "ms": ms, "ms_e2e": ms_e2e, "launches": launches, "clocks": clk, "shapes": shapes,
            "ms_seq": ms_seq, "seq_steps": seq_steps, "seq_launches": seq_launches, "ktimes": ktimes,
            "ms_k": ms_k, "roofline": roof, "seq_vs_batch_max_abs_dftot": seq_diff, "prec": PREC_NAME[prec],
            "ftot": ftot_batch}


def measure_batch_extra(args, torch, fbgpu, local):
    """The batch configuration as an extra key of the single-structure
    line, at both precisions."""
    out = {"workload": WORKLOADS["batch256"]}
    ft = {}
    for prec in (fbgpu.FB_PREC_FP64, fbgpu.FB_PREC_DF):
        r = measure_batch(args, torch, fbgpu, 1, local, prec, args.steps, 3, e2e=False)
        out.update(structures=256, natoms=r["natoms"], pairs=r["P"], triplets=r["T"],
                   atoms_min_max=[int(r["sizes"].min()), int(r["sizes"].max())])
        ft[r["prec"]] = r["ftot"]
        per = r["ms"] / args.steps
        seq = r["ms_seq"] / r["seq_steps"]
        out[r["prec"]] = {"batch_ms_per_step": round(per, 4),
                          "value": round(r["P"] * args.steps / (r["ms"] * 1e-3), 1), "unit": UNIT,
                          "sequential_ms_per_step": round(seq, 4), "batch_speedup": round(seq / per, 3),
                          "sequential_launches_per_step": r["seq_launches"] // r["seq_steps"],
                          "batch_launches_per_step": r["launches"] // args.steps,
                          "last_structure_sequential_vs_batch_max_abs_dftot": r["seq_vs_batch_max_abs_dftot"],
                          "launch_shapes": r["shapes"]}
    out["df_max_abs_dftot_vs_fp64"] = float(np.abs(ft["df"] - ft["fp64"]).max())
    return out


def run_batch(args, torch, fbgpu, ws, rank, local):
    """Config: 256 structures of uneven size in one batch, against the same
    structures assembled one at a time."""
    prec = fbgpu.FB_PREC_FP64 if args.prec == "fp64" else fbgpu.FB_PREC_DF
    r = measure_batch(args, torch, fbgpu, ws, local, prec, args.steps, args.warmup, e2e=True, clocks=True,
                      seq_steps=max(1, min(args.steps, 3)))
    P, T, NB, natoms = r["P"], r["T"], r["NB"], r["natoms"]
    h2d = 3 * natoms * 8 + 2 * NB * 8
    d2h = 4 * NB * 8 + 3 * natoms * 8
    per_step = r["ms"] / args.steps
    ms_seq, seq_steps = r["ms_seq"], r["seq_steps"]
    line = {
        "metric": METRIC, "value": round(ws * P * args.steps / (r["ms"] * 1e-3), 1), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if r["prec"] == "fp64" else "f64 (three-center: double-float f32x2)", "data": "synthetic",
        "config": {"workload": WORKLOADS["batch256"], "structures": len(r["structs"]), "natoms": natoms,
                   "atoms_min_max": [int(r["sizes"].min()), int(r["sizes"].max())], "pairs": P, "triplets": T,
                   "three_center_arithmetic": "double-float (FP32 pipe)" if r["prec"] == "df" else "fp64",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 and flushed between steps (256 MiB write)", "forces": True,
                   "step": "fb_neighbors over the batch + one CUDA graph launch (assembly + forces)",
                   "launch_shapes": r["shapes"], "autotuned": not args.no_autotune},
        "e2e": {"value": round(ws * P * args.steps / (r["ms_e2e"] * 1e-3), 1), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(r["ms_e2e"] / args.steps, 4)},
        "sequential": {"ms_per_step": round(ms_seq / seq_steps, 4),
                       "value": round(P * seq_steps / (ms_seq * 1e-3), 1), "unit": UNIT,
                       "gpu_launches_per_step": r["seq_launches"] // seq_steps,
                       "how": "the 256 structures one after another: fb_set_structure + fb_neighbors + "
                              "fb_assemble + fb_dassemble each (device-resident density matrices)",
                       "batch_speedup": round((ms_seq / seq_steps) / per_step, 3),
                       "last_structure_max_abs_dftot_vs_batch": r["seq_vs_batch_max_abs_dftot"]},
        "gpu_launches": r["launches"],
        "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in r["ktimes"].items() if v[1]},
        "separate_calls_ms_per_step": round(r["ms_k"] / args.steps, 4),
        "roofline": r["roofline"],
        "clocks": r["clocks"],
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_batch(r["path"], r["nZ"], r["structs"], P)
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_baseline_batch(path, nZ, structs, P_total, nsample=16):
    """The oracle on a bounded sample of the batch (the first nsample
    structures), scaled to blocks/s."""
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    fd = orc.Fdata(path, nZ)
    t_tot, p_tot = 0.0, 0
    for st in structs[:nsample]:
        t0 = time.perf_counter()
        s = orc.System(fd, st.ratom, st.imass, st.lattice, threads=cores).neighbors()
        s.assemble()
        t1 = time.perf_counter()
        norb = np.array([fd.norb(int(k)) for k in st.imass])
        rho, cape = denmat_fast(np.diff(s.pair_off), s.neigh_j[:s.npairs], s.neigh_back[:s.npairs], s.blk_off, norb)
        t2 = time.perf_counter()
        s.dassemble(rho, cape)
        t3 = time.perf_counter()
        t_tot += (t1 - t0) + (t3 - t2)
        p_tot += s.npairs
    return {"value": round(p_tot / t_tot, 1), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "the first %d of the 256 structures (%d pairs), neighbors + 2c + 3c assembly + forces, "
                      "%.3f s" % (nsample, p_tot, t_tot)}


def cpu_baseline(workload, path, nZ, st, P_expect=None, steps=1, keep=False):
    """The oracle (C restatement, OpenMP on every host core) on one full step
    of the same workload: neighbors, 2c + 3c assembly, forces.  keep: also
    return the last step's S, T, vna, vnao and ftot (same density matrices
    as the GPU step: the same generator over bit-identical neighbor maps)."""
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    fd = orc.Fdata(path, nZ)
    times = []
    P = None
    ref = None
    for _ in range(steps):
        t0 = time.perf_counter()
        s = orc.System(fd, st.ratom, st.imass, st.lattice, threads=cores).neighbors()
        blocks = s.assemble()
        t1 = time.perf_counter()
        norb = np.array([fd.norb(int(k)) for k in st.imass])
        rho, cape = denmat_fast(np.diff(s.pair_off), s.neigh_j[:s.npairs], s.neigh_back[:s.npairs], s.blk_off, norb)
        t2 = time.perf_counter()
        d = s.dassemble(rho, cape)
        t3 = time.perf_counter()
        times.append((t1 - t0) + (t3 - t2))
        P = s.npairs
        if keep:
            ref = dict(zip(("S", "T", "vna", "vnao"), blocks))
            ref["ftot"] = d["ftot"]
    t = float(np.median(times))
    rec = {"value": round(P / t, 1), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "%d full step(s) of the same workload (neighbors + 2c + 3c assembly + forces), median "
                     "%.3f s/step" % (steps, t)}
    return (rec, ref) if keep else rec


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    if args.workload == "batch256":
        return run_reference_batch(args, ws)
    path, nZ, st = load_workload(args.workload)
    cb = None
    for _ in range(args.warmup):
        cpu_baseline(args.workload, path, nZ, st)
    t0 = time.perf_counter()
    cb = cpu_baseline(args.workload, path, nZ, st, steps=args.steps)
    wall = time.perf_counter() - t0
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * wall / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "natoms": st.natoms},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_batch(args, ws):
    from fbgpu import synth
    path = synth.fdata_dir_for("batch256", root=fdata_root())
    nZ = [s.nZ for s in synth.species_for("batch256")]
    structs = synth.batch_structures(256)
    for _ in range(min(args.warmup, 1)):
        cpu_baseline_batch(path, nZ, structs, None, nsample=2)
    t0 = time.perf_counter()
    cbs = [cpu_baseline_batch(path, nZ, structs, None) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    cb = cbs[-1]
    cb["value"] = round(float(np.median([c["value"] for c in cbs])), 1)
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * wall / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS["batch256"], "structures": 256},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fbgpu", choices=["fbgpu", "reference"])
    ap.add_argument("--workload", default="sic4096", choices=sorted(WORKLOADS))
    ap.add_argument("--extra-workloads", default="si512,cho1536,batch256",
                    help="comma-separated workloads also measured (both precisions) as extra keys of the line")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline measurement")
    ap.add_argument("--legs", default="bloch,solve,dogs,vnl,vxc",
                    help="extra measurements on the same structure (comma list, or none)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--mlp-epochs", type=int, default=12,
                    help="train the MLP-3c surrogate this many epochs over 2^22 samples and compare it with the "
                         "table path (0: skip)")
    ap.add_argument("--prec", default="fp64", choices=["df", "fp64"],
                    help="three-center arithmetic of the headline: FP64 (default) or double-float on the FP32 pipe "
                         "(the other one is measured too, as an extra key)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
