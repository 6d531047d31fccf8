#!/usr/bin/env python
"""Benchmark of the batched acoustic FWI gradient (forward + checkpoints,
L2 misfit, adjoint with recompute and fused correlation, shot sum) on GB300.

Default workload: 64 shots on a 2001 x 801 layered model (h = 10 m), 50-300
receivers and 2000-4000 time steps per shot, 8 Hz Ricker, checkpoint period
50 (the batched configuration of the benchmark set).  One "step" is one full
gradient of all shots.  Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}]

--impl reference times the reference's CPU algorithm (the C++ restatement in
oracle/, OpenMP on all host cores; Julia is not available to run
SeismicWaves.jl itself) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gpts/s & shots/s fwd+adjoint gradient, batched vs plain, % of HBM roofline"
UNIT = "Gpts/s"


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="acoustic2d_2001x801")
    p.add_argument("--shots", type=int, default=0, help="override the number of shots (0 = workload's)")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-sample-nt", type=int, default=400)
    p.add_argument("--nt", type=int, default=0, help="cap every shot's time steps (small profiling cases)")
    p.add_argument("--tz", type=int, default=0, help="stencil tile height (0 = library heuristic)")
    p.add_argument("--variant", type=int, default=-1, help="2D stencil variant (-1 = library default)")
    p.add_argument("--no-autotune", action="store_true",
                   help="skip the autotuner (it runs by default unless --tz or --variant is given)")
    p.add_argument("--forward-only", action="store_true", help="time the batched forward instead of the gradient")
    p.add_argument("--bf16", type=int, default=0, help="acoustic snapshot_bf16 (0 FP32, 1 BF16 recompute buffer, "
                                                      "2 also BF16 checkpoints)")
    p.add_argument("--no-parity", action="store_true", help="skip the FP64-oracle error of the benchmark's shortest shot")
    p.add_argument("--check-freq", type=int, default=0, help="override the checkpoint period (small profiling cases)")
    p.add_argument("--precision", type=int, default=0,
                   help="1: compensated (double-FP32) forward passes of the acoustic CD / VD gradient")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the full-length 3D and elastic gradients that the default run times after the headline")
    return p.parse_args()


def max_over_ranks(t: float, dist=None, device=None) -> float:
    """The slowest rank's time (the job's time): all-reduce MAX over the process
    group, or t itself when running alone."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return t
    import torch

    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(units_per_rank: float, steps: int, world: int, t: float) -> float:
    """Whole-job throughput of `world` replicas that each process `units_per_rank`
    per step for `steps` steps in (max-over-ranks) time t."""
    return units_per_rank * steps * world / t


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _workload(name, shots, nt_cap=0, check_freq=0):
    import __graft_entry__

    sw = __graft_entry__.load_package()
    from seismicwaves_gb300 import configs

    w = configs.WORKLOADS[name]()
    if shots:
        w.shots = w.shots[:shots]
    if nt_cap:
        for s in w.shots:
            s.nt = min(s.nt, nt_cap)
    if check_freq:
        w.check_freq = check_freq
    return sw, w


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "yes", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- GPU driver
def _cap(arr, nt_cap):
    """Cap every shot's time steps (short autotuning trials)."""
    if nt_cap:
        for st in arr:
            st.nt = min(st.nt, nt_cap)


def _tune_tz(R, w, kind, candidates):
    """Band height of a variable-density or elastic simulation from capped gradient trials (2 K + 2 steps)."""
    from seismicwaves_gb300 import tune

    setter = R.lib.sw_acoustic_vd_set_tuning if kind == "vd" else R.lib.sw_elastic_set_tuning
    idx = list(range(len(w.shots)))
    cap = 2 * w.check_freq + 2
    t0 = time.perf_counter()
    tz, timings = tune.autotune_tz((kind, w.name, len(idx)), lambda t: R.ctx.check(setter(R.h, t), "set_tuning"),
                                   lambda: R.gradient_device(idx, cap), candidates)
    return tz, {"tz": tz, "trial_ms": {str(t): round(x * 1e3, 3) for t, x in timings.items()},
                "tuning_s": round(time.perf_counter() - t0, 2),
                "what": f"band height from batched gradients capped at {cap} steps, best of 2 per candidate"}


class GradientRun:
    """The workload's shots as C-ABI structs over device (or pinned host) buffers."""

    def __init__(self, sw, w, device, on_device=True, bf16=0, precision=0):
        import torch

        L = sw._lib
        self.sw, self.w, self.L, self.torch = sw, w, L, torch
        self.dev = torch.device("cuda", device)
        self.ctx = L.Context(device)
        self.lib = self.ctx.lib
        nd = w.vp.ndim
        prm = L.SwAcousticParams()
        prm.ndim = nd
        for d in range(nd):
            prm.n[d], prm.h[d] = w.vp.shape[d], w.h[d]
        prm.dt, prm.halo, prm.rcoef, prm.freetop = w.dt, w.halo, 1e-4, int(w.freetop)
        gp = L.SwGradParams()
        gp.check_freq = w.check_freq
        gp.snapshot_bf16 = bf16
        self.h = ctypes.c_void_p()
        self.ctx.check(self.lib.sw_wavesim_create(self.ctx.h, ctypes.byref(prm), 1, ctypes.byref(gp),
                                                  ctypes.byref(self.h)), "sw_wavesim_create")
        if precision:  # compensated forward passes
            self.ctx.check(self.lib.sw_wavesim_set_precision(self.h, precision), "sw_wavesim_set_precision")
        self.hf = ctypes.c_void_p()
        self.ctx.check(self.lib.sw_wavesim_create(self.ctx.h, ctypes.byref(prm), 0, None, ctypes.byref(self.hf)),
                       "sw_wavesim_create")
        self.stream = torch.cuda.ExternalStream(self.ctx.stream, device=self.dev)
        vmax = float(np.max(w.vp))  # init_bdc!: max of the simulated model
        self.host = []
        for s in w.shots:
            si = sw.nearest_grid_points(s.src_pos, w.h)
            ri = sw.nearest_grid_points(s.rec_pos, w.h)
            tf = sw.scale_srctf(s.stf(w.dt), si, w.vp, w.h, w.dt)
            parts = []
            for d in range(nd):
                parts += L.cpml_coefficients(vmax, w.dt, w.halo, 1e-4, w.h[d], s.f0, w.freetop and d == nd - 1)
            cp = np.concatenate(parts).astype(np.float32)
            if precision:  # the FP64 coefficients of the compensated forward
                p64 = []
                for d in range(nd):
                    p64 += L.cpml_coefficients64(vmax, w.dt, w.halo, 1e-4, w.h[d], s.f0, w.freetop and d == nd - 1)
                self.host.append((si, ri, tf, cp, np.concatenate(p64)))
            else:
                self.host.append((si, ri, tf, cp))
        self.precision = precision
        # device-resident inputs and outputs
        t = torch
        self.vp_d = t.from_numpy(np.ascontiguousarray(w.vp.ravel(order="F"), dtype=np.float32)).to(self.dev)
        self.vpo_d = t.from_numpy(np.ascontiguousarray(w.vp_observed.ravel(order="F"), dtype=np.float32)).to(self.dev)
        self.tf_d = [t.from_numpy(np.ascontiguousarray(h[2].ravel(order="F"))).to(self.dev) for h in self.host]
        self.tr_d = [t.zeros(s.nt * h[1].shape[0], dtype=t.float32, device=self.dev) for s, h in zip(w.shots, self.host)]
        self.obs_d = [t.zeros_like(x) for x in self.tr_d]
        self.grad_d = t.zeros(int(np.prod(w.vp.shape)), dtype=t.float64, device=self.dev)
        self.mis_d = t.zeros(1, dtype=t.float64, device=self.dev)

    def structs(self, idx, tf, tr, obs):
        arr = (self.L.SwAcousticShot * len(idx))()
        for k, i in enumerate(idx):
            si, ri, _, cp = self.host[i][:4]
            st = arr[k]
            st.nt, st.nsrc, st.nrec = self.w.shots[i].nt, si.shape[0], ri.shape[0]
            st.src_idx, st.rec_idx, st.cpml = si.ctypes.data, ri.ctypes.data, cp.ctypes.data
            if len(self.host[i]) > 4:
                st.cpml64 = self.host[i][4].ctypes.data
            st.srctf, st.traces = tf[i], tr[i]
            if obs is not None:
                st.observed = obs[i]
        return arr

    def make_observed(self):
        """Observed data: a forward run on the perturbed model."""
        self.ctx.check(self.lib.sw_wavesim_set_vp(self.hf, self.vpo_d.data_ptr(), 1), "set_vp")
        idx = list(range(len(self.w.shots)))
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.obs_d], None)
        self.ctx.check(self.lib.sw_acoustic_forward(self.hf, len(idx), arr, 1), "observed forward")
        self.lib.sw_wavesim_destroy(self.hf)
        if self.precision:  # the compensated forward takes the FP64 model
            self.vp64 = np.asfortranarray(self.w.vp, dtype=np.float64)
            self.ctx.check(self.lib.sw_wavesim_set_vp64(self.h, self.vp64.ctypes.data, 0), "set_vp64")
        else:
            self.ctx.check(self.lib.sw_wavesim_set_vp(self.h, self.vp_d.data_ptr(), 1), "set_vp")

    def forward_device(self, idx):
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.tr_d], None)
        self.ctx.check(self.lib.sw_acoustic_forward(self.h, len(idx), arr, 1), "sw_acoustic_forward")

    def gradient_device(self, idx):
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.tr_d],
                           [x.data_ptr() for x in self.obs_d])
        self.ctx.check(self.lib.sw_acoustic_gradient(self.h, len(idx), arr, 1, self.grad_d.data_ptr(),
                                                      self.mis_d.data_ptr()), "sw_acoustic_gradient")

    def setup_host(self):
        """Pinned host copies of the per-step inputs and outputs (end-to-end leg)."""
        t = self.torch
        if getattr(self, "precision", 0):  # FP64 model for the compensated forward
            self.vp_h = t.from_numpy(np.ascontiguousarray(self.w.vp.ravel(order="F"), dtype=np.float64)).pin_memory()
        else:
            self.vp_h = self.vp_d.cpu().pin_memory()
        self.tf_h = [x.cpu().pin_memory() for x in self.tf_d]
        self.obs_h = [x.cpu().pin_memory() for x in self.obs_d]
        self.tr_h = [t.zeros(x.numel(), dtype=t.float32).pin_memory() for x in self.tr_d]
        self.grad_h = t.zeros(self.grad_d.numel(), dtype=t.float64).pin_memory()
        self.mis_h = t.zeros(1, dtype=t.float64).pin_memory()
        h2d = (self.vp_h.numel() * self.vp_h.element_size() + sum(x.numel() * 4 for x in self.tf_h)
               + sum(x.numel() * 4 for x in self.obs_h))
        d2h = sum(x.numel() * 4 for x in self.tr_h) + self.grad_h.numel() * 8 + 8
        return h2d, d2h

    def gradient_host(self):
        idx = list(range(len(self.w.shots)))
        if getattr(self, "precision", 0):
            self.ctx.check(self.lib.sw_wavesim_set_vp64(self.h, self.vp_h.data_ptr(), 0), "set_vp64")
        else:
            self.ctx.check(self.lib.sw_wavesim_set_vp(self.h, self.vp_h.data_ptr(), 0), "set_vp")
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_h], [x.data_ptr() for x in self.tr_h],
                           [x.data_ptr() for x in self.obs_h])
        self.ctx.check(self.lib.sw_acoustic_gradient(self.h, len(idx), arr, 0, self.grad_h.data_ptr(),
                                                      self.mis_h.data_ptr()), "sw_acoustic_gradient")

    def timed(self, fn, n):
        t = self.torch
        a, b = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        t.cuda.synchronize(self.dev)
        a.record(self.stream)
        for _ in range(n):
            fn()
        b.record(self.stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3


class ElasticRun:
    """The elastic workload's shots as C-ABI structs over device (or pinned host) buffers."""

    def __init__(self, sw, w, device):
        import torch

        L = sw._lib
        E = sys.modules[sw.__name__ + ".elastic"]
        self.sw, self.w, self.L, self.torch, self.E = sw, w, L, torch, E
        self.dev = torch.device("cuda", device)
        self.ctx = L.Context(device)
        self.lib = self.ctx.lib
        nx, nz = w.lam.shape
        prm = L.SwElasticParams()
        prm.n[0], prm.n[1] = nx, nz
        prm.h[0], prm.h[1] = w.h
        prm.dt, prm.halo, prm.rcoef, prm.freetop = w.dt, w.halo, 1e-4, int(w.freetop)
        gp = L.SwGradParams()
        gp.check_freq = w.check_freq
        self.h = ctypes.c_void_p()
        self.ctx.check(self.lib.sw_elastic_create(self.ctx.h, ctypes.byref(prm), 1, ctypes.byref(gp),
                                                  ctypes.byref(self.h)), "sw_elastic_create")
        self.stream = torch.cuda.ExternalStream(self.ctx.stream, device=self.dev)
        vmax = float(np.max(w.vp))
        hx, hz = w.h
        self.host = []
        for s in w.shots:
            sp = lambda pos, sh, mir: E.spread_positions((nx, nz), w.h, pos, shift=sh, mirror=mir)  # noqa: E731
            src = [sp(s.src_pos, (0.0, 0.0), True), sp(s.src_pos, (hx / 2, hz / 2), True)]
            rec = [sp(s.rec_pos, (hx / 2, 0.0), False), sp(s.rec_pos, (0.0, hz / 2), False)]
            tabs = [[E._table(src[t]) for t in range(2)], [E._table(rec[t]) for t in range(2)]]
            tf = (s.stf(w.dt) / (hx * hz)).astype(np.float32)
            parts = []
            for d in range(2):
                parts += L.cpml_coefficients(vmax, w.dt, w.halo, 1e-4, w.h[d], s.f0, w.freetop and d == 1)
            cp = np.concatenate(parts).astype(np.float32)
            self.host.append((tabs, tf, cp))
        self.mt = np.ascontiguousarray(np.array(w.momtens, dtype=np.float32).reshape(1, 3))
        t = torch
        self.tf_d = [t.from_numpy(np.ascontiguousarray(h[1].ravel(order="F"))).to(self.dev) for h in self.host]
        self.tr_d = [t.zeros(s.nt * 2 * s.rec_pos.shape[0], dtype=t.float32, device=self.dev) for s in w.shots]
        self.obs_d = [t.zeros_like(x) for x in self.tr_d]
        self.grad_d = t.zeros(3 * nx * nz, dtype=t.float64, device=self.dev)
        self.mis_d = t.zeros(1, dtype=t.float64, device=self.dev)

    def set_material(self, lam, mu, rho):
        arrs = [np.asfortranarray(a, dtype=np.float32) for a in (lam, mu, rho)]
        self.ctx.check(self.lib.sw_elastic_set_material(self.h, *(a.ctypes.data for a in arrs)), "set_material")

    def structs(self, idx, tf, tr, obs):
        arr = (self.L.SwElasticShot * len(idx))()
        for k, i in enumerate(idx):
            tabs, _, cp = self.host[i]
            s = self.w.shots[i]
            st = arr[k]
            st.nt, st.kind, st.nsrc, st.nrec = s.nt, 0, 1, s.rec_pos.shape[0]
            st.srctf, st.traces, st.cpml, st.momtens = tf[i], tr[i], cp.ctypes.data, self.mt.ctypes.data
            for t in range(2):
                for (off, ij, coef), tgt in ((tabs[0][t], st.src[t]), (tabs[1][t], st.rec[t])):
                    tgt.offsets, tgt.ij, tgt.coef = off.ctypes.data, ij.ctypes.data, coef.ctypes.data
            if obs is not None:
                st.observed = obs[i]
        return arr

    def make_observed(self):
        self.set_material(*self.w.observed_model)
        idx = list(range(len(self.w.shots)))
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.obs_d], None)
        self.ctx.check(self.lib.sw_elastic_forward(self.h, len(idx), arr, 1), "observed forward")
        self.set_material(self.w.lam, self.w.mu, self.w.rho)

    def gradient_device(self, idx, nt_cap=0):
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.tr_d],
                           [x.data_ptr() for x in self.obs_d])
        _cap(arr, nt_cap)
        n = self.grad_d.numel() // 3
        p = self.grad_d.data_ptr()
        self.ctx.check(self.lib.sw_elastic_gradient(self.h, len(idx), arr, 1, p, p + 8 * n, p + 16 * n,
                                                     self.mis_d.data_ptr()), "sw_elastic_gradient")

    def setup_host(self):
        t = self.torch
        self.tf_h = [x.cpu().pin_memory() for x in self.tf_d]
        self.obs_h = [x.cpu().pin_memory() for x in self.obs_d]
        self.tr_h = [t.zeros(x.numel(), dtype=t.float32).pin_memory() for x in self.tr_d]
        self.grad_h = t.zeros(self.grad_d.numel(), dtype=t.float64).pin_memory()
        self.mis_h = t.zeros(1, dtype=t.float64).pin_memory()
        h2d = sum(x.numel() * 4 for x in self.tf_h) + sum(x.numel() * 4 for x in self.obs_h)
        d2h = sum(x.numel() * 4 for x in self.tr_h) + self.grad_h.numel() * 8 + 8
        return h2d, d2h

    def gradient_host(self):
        idx = list(range(len(self.w.shots)))
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_h], [x.data_ptr() for x in self.tr_h],
                           [x.data_ptr() for x in self.obs_h])
        n = self.grad_h.numel() // 3
        p = self.grad_h.data_ptr()
        self.ctx.check(self.lib.sw_elastic_gradient(self.h, len(idx), arr, 0, p, p + 8 * n, p + 16 * n,
                                                     self.mis_h.data_ptr()), "sw_elastic_gradient")

    timed = GradientRun.timed


class VDRun(GradientRun):
    """The variable-density workload's shots as C-ABI structs (sw_acoustic_vd_*)."""

    def __init__(self, sw, w, device, precision=0):
        import torch

        L = sw._lib
        V = sys.modules[sw.__name__ + ".vd"]
        self.sw, self.w, self.L, self.torch = sw, w, L, torch
        self.dev = torch.device("cuda", device)
        self.ctx = L.Context(device)
        self.lib = self.ctx.lib
        prm = L.SwAcousticParams()
        prm.ndim = 2
        for d in range(2):
            prm.n[d], prm.h[d] = w.vp.shape[d], w.h[d]
        prm.n[2], prm.h[2] = 1, 1.0
        prm.dt, prm.halo, prm.rcoef, prm.freetop = w.dt, w.halo, 1e-4, int(w.freetop)
        gp = L.SwGradParams()
        gp.check_freq = w.check_freq
        self.h = ctypes.c_void_p()
        self.ctx.check(self.lib.sw_acoustic_vd_create(self.ctx.h, ctypes.byref(prm), 0, 1, ctypes.byref(gp),
                                                      ctypes.byref(self.h)), "sw_acoustic_vd_create")
        if precision:  # compensated forward passes
            self.ctx.check(self.lib.sw_acoustic_vd_set_precision(self.h, precision), "sw_acoustic_vd_set_precision")
        self.stream = torch.cuda.ExternalStream(self.ctx.stream, device=self.dev)
        vmax = float(np.max(w.vp))
        self.host = []
        for s in w.shots:
            si = sw.nearest_grid_points(s.src_pos, w.h)
            ri = sw.nearest_grid_points(s.rec_pos, w.h)
            tf = V.scale_srctf_vd(s.stf(w.dt), si, w.vp, w.rho, w.h, w.dt)
            parts = []
            for d in range(2):
                parts += L.cpml_coefficients(vmax, w.dt, w.halo, 1e-4, w.h[d], s.f0, w.freetop and d == 1)
            self.host.append((si, ri, tf, np.concatenate(parts).astype(np.float32)))
        t = torch
        self.tf_d = [t.from_numpy(np.ascontiguousarray(h[2].ravel(order="F"))).to(self.dev) for h in self.host]
        self.tr_d = [t.zeros(s.nt * h[1].shape[0], dtype=t.float32, device=self.dev) for s, h in zip(w.shots, self.host)]
        self.obs_d = [t.zeros_like(x) for x in self.tr_d]
        self.grad_d = t.zeros(2 * int(np.prod(w.vp.shape)), dtype=t.float64, device=self.dev)
        self.mis_d = t.zeros(1, dtype=t.float64, device=self.dev)

    def set_material(self, vp, rho):
        a = [np.asfortranarray(x, dtype=np.float32) for x in (vp, rho)]
        self.ctx.check(self.lib.sw_acoustic_vd_set_material(self.h, a[0].ctypes.data, a[1].ctypes.data),
                       "sw_acoustic_vd_set_material")

    def make_observed(self):
        self.set_material(self.w.vp_observed, self.w.rho_observed)
        idx = list(range(len(self.w.shots)))
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.obs_d], None)
        self.ctx.check(self.lib.sw_acoustic_vd_forward(self.h, len(idx), arr, 1), "observed forward")
        self.set_material(self.w.vp, self.w.rho)

    def gradient_device(self, idx, nt_cap=0):
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_d], [x.data_ptr() for x in self.tr_d],
                           [x.data_ptr() for x in self.obs_d])
        _cap(arr, nt_cap)
        n = self.grad_d.numel() // 2
        p = self.grad_d.data_ptr()
        self.ctx.check(self.lib.sw_acoustic_vd_gradient(self.h, len(idx), arr, 1, p, p + 8 * n,
                                                         self.mis_d.data_ptr()), "sw_acoustic_vd_gradient")

    def setup_host(self):
        t = self.torch
        self.tf_h = [x.cpu().pin_memory() for x in self.tf_d]
        self.obs_h = [x.cpu().pin_memory() for x in self.obs_d]
        self.tr_h = [t.zeros(x.numel(), dtype=t.float32).pin_memory() for x in self.tr_d]
        self.grad_h = t.zeros(self.grad_d.numel(), dtype=t.float64).pin_memory()
        self.mis_h = t.zeros(1, dtype=t.float64).pin_memory()
        h2d = sum(x.numel() * 4 for x in self.tf_h) + sum(x.numel() * 4 for x in self.obs_h)
        d2h = sum(x.numel() * 4 for x in self.tr_h) + self.grad_h.numel() * 8 + 8
        return h2d, d2h

    def gradient_host(self):
        idx = list(range(len(self.w.shots)))
        arr = self.structs(idx, [x.data_ptr() for x in self.tf_h], [x.data_ptr() for x in self.tr_h],
                           [x.data_ptr() for x in self.obs_h])
        n = self.grad_h.numel() // 2
        p = self.grad_h.data_ptr()
        self.ctx.check(self.lib.sw_acoustic_vd_gradient(self.h, len(idx), arr, 0, p, p + 8 * n,
                                                         self.mis_h.data_ptr()), "sw_acoustic_vd_gradient")


def _vd_cpu_baseline(sw, w, nt_sample):
    import oracle

    V = sys.modules[sw.__name__ + ".vd"]
    nt_sample = _sample_nt(w, nt_sample)
    s = w.shots[0]
    si = sw.nearest_grid_points(s.src_pos, w.h)
    ri = sw.nearest_grid_points(s.rec_pos, w.h)
    tf = V.scale_srctf_vd(s.stf(w.dt)[:nt_sample], si, w.vp, w.rho, w.h, w.dt).astype(np.float64)
    cp = oracle.cpml_blocks(w.vp, w.h, w.dt, w.halo, 1e-4, s.f0, w.freetop)
    obs = np.zeros((nt_sample, ri.shape[0]))
    threads = os.cpu_count() or 1
    K = min(w.check_freq, nt_sample - 1)
    t0 = time.perf_counter()
    oracle.vd_gradient(w.vp, w.rho, w.h, w.dt, w.halo, cp, tf, si, ri, obs, check_freq=K, nthreads=threads)
    dt = time.perf_counter() - t0
    nx, nz = w.vp.shape
    sample = (f"one shot of {w.name}, {nt_sample} time steps, checkpoint period {K}, "
              "FP64 gradient (forward + recompute + adjoint)")
    return float(nx * nz) * nt_sample / dt / 1e9, threads, sample, dt


VD_KINDS = {0: "k_vd_p + k_vd_v forward", 4: "k_vd_p + k_vd_v recompute (writes slots)",
            1: "k_vd_v + k_vd_p<corr> adjoint with fused correlation"}


def measure_vd(a, name="acoustic_vd2d_2001x801", shots=0, nt_cap=0, steps=None, warmup=None, plain=True, cpu=True,
               device=0):
    """Batched variable-density gradient: Gpts/s, shots/s, e2e, plain per-shot path, roofline of the dominant kind."""
    import torch

    steps = a.steps if steps is None else steps
    warmup = a.warmup if warmup is None else warmup
    sw, w = _workload(name, shots, nt_cap)
    R = VDRun(sw, w, device, precision=a.precision)
    tuned, tz = None, a.tz or 8
    if a.tz:
        R.ctx.check(R.lib.sw_acoustic_vd_set_tuning(R.h, a.tz), "sw_acoustic_vd_set_tuning")
    R.make_observed()
    if not (a.tz or a.no_autotune):
        tz, tuned = _tune_tz(R, w, "vd", (8, 16, 32))
    nshots = len(w.shots)
    allidx = list(range(nshots))
    pts = float(w.point_steps())
    for _ in range(warmup):
        R.gradient_device(allidx)
    torch.cuda.synchronize(R.dev)
    clocks = ClockSampler(device)
    clocks.start()
    t_dev = R.timed(lambda: R.gradient_device(allidx), steps)
    clk = clocks.stop()
    R.ctx.profile(True)
    R.timed(lambda: R.gradient_device(allidx), 1)
    R.ctx.profile(False)
    prof = {k: R.ctx.profile_read(k) for k in range(6)}
    kernels_per_call = sum(R.ctx.profile_kernels(k) for k in range(6))
    h2d, d2h = R.setup_host()
    R.gradient_host()
    t_e2e = R.timed(R.gradient_host, steps)
    pl = None
    if plain:
        R.gradient_device([0])
        t_plain = R.timed(lambda: [R.gradient_device([i]) for i in allidx], 1)
        pl = {"value": pts / t_plain / 1e9, "unit": UNIT, "shots_per_s": nshots / t_plain,
              "ms_per_step": t_plain * 1e3, "what": "same kernels, one shot per call"}
    dom = max(VD_KINDS, key=lambda k: prof[k][0])
    ms_tot, launches, bytes_tot = prof[dom]
    achieved = bytes_tot / (ms_tot / 1e3) / 1e9 if ms_tot > 0 else None
    peak, peak_kind = _peak()
    traffic_per_shot = _traffic_from_profiles("k_vd_v + k_vd_p<corr> adjoint", w.name) if dom == 1 else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None,
            "traffic": traffic_per_shot * nshots if traffic_per_shot else None,
            "algorithmic_bytes_per_launch": bytes_tot / max(launches, 1),
            "avg_launch_us": ms_tot * 1e3 / max(launches, 1), "launches": launches, "kernel": VD_KINDS[dom],
            "peak_kind": peak_kind,
            "kernels": {VD_KINDS[k]: {"ms": prof[k][0], "launches": prof[k][1],
                                      "GB_per_s": (prof[k][2] / (prof[k][0] / 1e3) / 1e9) if prof[k][0] else None}
                        for k in VD_KINDS},
            "other_kernels_ms": {"sources and receivers": prof[2][0], "misfit, flushes, reduction": prof[3][0]}}
    out = {"metric": METRIC, "value": pts * steps / t_dev / 1e9, "unit": UNIT, "n_gpus": 1, "steps": steps,
           "warmup": warmup, "ms_per_step": t_dev * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": w.name, "grid": list(w.vp.shape), "h_m": w.h[0], "shots": nshots,
                      "nt": max(s.nt for s in w.shots), "check_freq": w.check_freq, "halo": w.halo,
                      "tz": tz, "tuning": tuned,
                      "cache": "inputs larger than L2 (each step streams several GB of wavefield state)",
                      "precision": "fp32 wavefields and stencil, fp32 sums over one checkpoint window, "
                                   "fp64 window totals, misfit and shot sum"
                                   + ("; compensated double-fp32 forward passes" if a.precision else "")},
           "shots_per_s": nshots * steps / t_dev, "plain": pl,
           "batched_vs_plain": (nshots * steps / t_dev / pl["shots_per_s"]) if pl else None,
           "clocks": clk,
           "e2e": {"value": pts * steps / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h},
           "gpu_launches": kernels_per_call * steps, "roofline": roof}
    if cpu:
        import oracle

        oracle.load()
        v, threads, sample, _ = _vd_cpu_baseline(sw, w, a.cpu_sample_nt)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    R.lib.sw_acoustic_vd_destroy(R.h)
    return out


def _elastic_cpu_baseline(sw, w, nt_sample):
    import oracle

    nt_sample = _sample_nt(w, nt_sample)
    E = sys.modules[sw.__name__ + ".elastic"]
    s = w.shots[0]
    nx, nz = w.lam.shape
    hx, hz = w.h
    sp = lambda pos, sh, mir: E.spread_positions((nx, nz), w.h, pos, shift=sh, mirror=mir)  # noqa: E731
    shot = dict(kind="mt", srctf=s.stf(w.dt)[:nt_sample] / (hx * hz), momtens=np.array([w.momtens]),
                src_tables=[sp(s.src_pos, (0.0, 0.0), True), sp(s.src_pos, (hx / 2, hz / 2), True)],
                rec_tables=[sp(s.rec_pos, (hx / 2, 0.0), False), sp(s.rec_pos, (0.0, hz / 2), False)])
    cp = oracle.cpml_blocks(w.vp, w.h, w.dt, w.halo, 1e-4, s.f0, w.freetop)
    obs = np.zeros((nt_sample, 2, s.rec_pos.shape[0]))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.elastic_gradient(w.lam, w.mu, w.rho, w.h, w.dt, w.halo, w.freetop, cp, shot, obs,
                            check_freq=min(w.check_freq, nt_sample - 1), nthreads=threads)
    dt = time.perf_counter() - t0
    pts = float(nx * nz) * nt_sample
    sample = (f"one shot of {w.name}, {nt_sample} time steps, checkpoint period "
              f"{min(w.check_freq, nt_sample - 1)}, FP64 gradient (forward + recompute + adjoint)")
    return pts / dt / 1e9, threads, sample, dt


def _peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def _traffic_ratio_from_profiles(kind, workload):
    """DRAM bytes over algorithmic bytes of the `kind` stencil launches
    (forward / recompute / adjoint) in an ncu capture summary under profiles/
    (a smaller case of the same workload; the ratio carries over to the full
    launch because both grow with the active points per launch)."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        txt = f.read_text()
        if f"workload: {workload}" not in txt:
            continue
        for line in txt.splitlines():
            if line.startswith(f"traffic_over_algorithmic[{kind}]:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def _one_step_model_bytes(w):
    """Bytes one gradient must move with one time step per launch in FP32: per
    interior point-step 16 (forward: R/W p, d) + 16 (K-1)/K (recompute) +
    4 + 4 (write / read D) + 16 (adjoint) + 8 (correlation RMW); per strip cell
    and axis 16 per pass (R/W psi, xi, three passes); checkpoints 2 fields x
    4 B written and read every K steps; fact once per launch (negligible)."""
    nd = w.vp.ndim
    n = w.vp.shape
    pts = float(np.prod([k - 2 for k in n]))
    strip = 0.0
    for d in range(nd):
        wd = sum(1 for x in range(1, n[d] - 1) if x < w.halo or x >= n[d] - w.halo)
        strip += wd * pts / (n[d] - 2)
    K = w.check_freq
    per_pt = 16 + 16 * (K - 1) / K + 8 + 16 + 8 + 16.0 / K
    per_strip = 16 * (2 + (K - 1) / K)
    steps = float(sum(s.nt for s in w.shots))
    return steps * (pts * per_pt + strip * per_strip)


def _traffic_from_profiles(kernel, workload):
    """DRAM bytes per launch and per shot of `kernel` from an ncu capture summary in profiles/."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        txt = f.read_text()
        if f"kernel: {kernel}\n" in txt and f"workload: {workload}" in txt:
            for line in txt.splitlines():
                if line.startswith("dram_bytes_per_launch_per_shot:"):
                    try:
                        return float(line.split(":", 1)[1].split()[0])
                    except ValueError:
                        return None
    return None


def _sample_nt(w, nt_sample):
    """CPU sample length: the requested steps, fewer on large grids (about 2e9 point-steps at most)."""
    return int(max(20, min(nt_sample, 2e9 // max(w.gridpoints, 1))))


# Error bars of the FP32 path against the FP64 oracle (relative L2 of traces
# and gradient, relative misfit).
PARITY_BARS = {"traces_rel_l2": 1e-5, "misfit_rel": 1e-6, "gradient_rel_l2": 1e-5}


def _parity_2d(R, sw, w):
    """Error of one benchmark shot against the FP64 oracle, outside the timed
    region: the shortest shot of the workload at its full record length, one
    GPU gradient call (same device inputs as the benchmark, observed data of
    the perturbed model) against the oracle's forward + misfit + adjoint
    gradient with the same checkpoint period on the same inputs."""
    import oracle

    oracle.load()
    idx = min(range(len(w.shots)), key=lambda i: w.shots[i].nt)
    s = w.shots[idx]
    R.gradient_device([idx])
    R.torch.cuda.synchronize(R.dev)
    si, ri = R.host[idx][:2]
    nrec = ri.shape[0]
    g = R.grad_d.cpu().numpy().reshape(w.vp.shape, order="F")
    mis = float(R.mis_d.item())
    tr = R.tr_d[idx].cpu().numpy().reshape(nrec, s.nt).T
    obs = R.obs_d[idx].cpu().numpy().reshape(nrec, s.nt).T.astype(np.float64)
    tf = sw.scale_srctf(s.stf(w.dt), si, w.vp, w.h, w.dt).astype(np.float64)
    cp = oracle.cpml_blocks(w.vp, w.h, w.dt, w.halo, 1e-4, s.f0, w.freetop)
    t0 = time.perf_counter()
    gref, mref, tref = oracle.acoustic_gradient(w.vp, w.h, w.dt, w.halo, cp, tf, si, ri, obs,
                                                check_freq=w.check_freq, nthreads=os.cpu_count() or 1)
    t_oracle = time.perf_counter() - t0

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))

    errs = {"traces_rel_l2": rel(tr, tref), "misfit_rel": abs(mis - mref) / abs(mref),
            "gradient_rel_l2": rel(g, gref)}
    return {"shot": idx, "nt": s.nt, "receivers": nrec, **errs, "bars": PARITY_BARS,
            "within_bars": {k: errs[k] <= PARITY_BARS[k] for k in errs},
            "oracle": "FP64 C++ restatement of the reference's CD path (oracle/), same inputs",
            "oracle_s": round(t_oracle, 2)}


def _cpu_baseline(sw, w, nt_sample):
    import oracle

    nt_sample = _sample_nt(w, nt_sample)
    s = w.shots[0]
    si = sw.nearest_grid_points(s.src_pos, w.h)
    ri = sw.nearest_grid_points(s.rec_pos, w.h)
    stf = s.stf(w.dt)[:nt_sample]
    tf = sw.scale_srctf(stf, si, w.vp, w.h, w.dt).astype(np.float64)
    cp = oracle.cpml_blocks(w.vp, w.h, w.dt, w.halo, 1e-4, s.f0, w.freetop)
    obs = np.zeros((nt_sample, ri.shape[0]))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.acoustic_gradient(w.vp, w.h, w.dt, w.halo, cp, tf, si, ri, obs,
                             check_freq=min(w.check_freq, nt_sample - 1), nthreads=threads)
    dt = time.perf_counter() - t0
    pts = float(np.prod(w.vp.shape)) * nt_sample
    sample = (f"one shot of {w.name}, {nt_sample} time steps, checkpoint period "
              f"{min(w.check_freq, nt_sample - 1)}, FP64 gradient (forward + recompute + adjoint)")
    return pts / dt / 1e9, threads, sample, dt


def run_reference(a):
    rank, world, _ = _dist()
    if rank != 0:
        return
    sw, w = _workload(a.workload, a.shots, a.nt)
    import oracle

    oracle.load()
    base = _cpu_baseline
    if a.workload.startswith("acoustic_vd"):
        base = _vd_cpu_baseline
    elif a.workload.startswith("elastic"):
        base = _elastic_cpu_baseline
    vals = []
    for i in range(a.warmup + a.steps):
        v, threads, sample, dt = base(sw, w, a.cpu_sample_nt)
        if i >= a.warmup:
            vals.append((v, dt))
    value = statistics.mean(v for v, _ in vals)
    ms = statistics.mean(d for _, d in vals) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _extra_acoustic3d(a, device):
    """The 3D workload at full size and length (16 shots of 400^3, nt 2000,
    K = 100, FP16 recompute buffer with per-tile exponents): one warm-up
    gradient (with the per-kernel event timing: direct launches), one timed
    (CUDA graph); Gpts/s, shots/s and the stencil kinds' bandwidth."""
    import torch

    sw, w = _workload("acoustic3d_400", 0, 0)
    R = GradientRun(sw, w, device, bf16=3)
    R.make_observed()
    idx = list(range(len(w.shots)))
    tuned = None
    if not a.no_autotune:
        from seismicwaves_gb300 import tune

        arr = R.structs(idx, [x.data_ptr() for x in R.tf_d], [x.data_ptr() for x in R.tr_d], None)
        t0 = time.perf_counter()
        r = tune.autotune(R.ctx, R.h, (w.vp.shape, w.halo), arr, len(idx), 3, steps=12, on_device=1)
        tuned = {"variant": r["variant"], "tz": r["tz"], "tuning_s": round(time.perf_counter() - t0, 2),
                 "trial_ms": {"/".join(map(str, k)): round(t * 1e3, 3) for k, t in r["trial_s"].items()},
                 "what": "batched forwards of 12 steps, best of 2 per candidate"}
    R.ctx.profile(True)  # the warm-up gradient, timed per kernel kind
    R.gradient_device(idx)
    torch.cuda.synchronize(R.dev)
    R.ctx.profile(False)
    prof = {k: R.ctx.profile_read(k) for k in (0, 1, 4)}
    clocks = ClockSampler(device)
    clocks.start()
    t = R.timed(lambda: R.gradient_device(idx), 1)
    clk = clocks.stop()
    pts = float(w.point_steps())
    peak, _ = _peak()
    k3 = "k_ac3d_inner + k_ac3d_zslab + k_ac3d_yslab"
    names = {0: f"{k3} <1> forward", 4: f"{k3} <1> recompute", 1: f"{k3} <2> adjoint + correlation"}
    kern = {names[k]: {"ms": prof[k][0], "GB_per_s": prof[k][2] / (prof[k][0] / 1e3) / 1e9 if prof[k][0] else None,
                       "frac": prof[k][2] / (prof[k][0] / 1e3) / 1e9 / peak if prof[k][0] else None}
            for k in prof}
    out = {"workload": w.name, "grid": list(w.vp.shape), "shots": len(w.shots), "nt": max(s.nt for s in w.shots),
           "check_freq": w.check_freq, "buffer": "fp16 recompute buffer, exponent per row and 128-point tile",
           "value": pts / t / 1e9, "unit": UNIT,
           "ms_per_step": t * 1e3, "shots_per_s": len(w.shots) / t, "steps": 1, "warmup": 1, "kernels": kern,
           "clocks": clk, "tuning": tuned}
    R.lib.sw_wavesim_destroy(R.h)
    return out


def _extras(a, device):
    """Full-length gradients of the 3D and elastic workloads, timed after the
    headline (its device memory released first)."""
    import gc

    import torch

    out = {}
    gc.collect()
    torch.cuda.empty_cache()
    e = measure_elastic(a, "elastic2d_1200x600", steps=1, warmup=2, plain=False, cpu=False, device=device)
    out["elastic2d_1200x600"] = {k: e[k] for k in ("value", "unit", "ms_per_step", "shots_per_s", "steps", "warmup",
                                                    "config", "clocks")}
    out["elastic2d_1200x600"]["roofline"] = {k: e["roofline"][k] for k in ("kernel", "achieved", "frac", "kernels")}
    gc.collect()
    torch.cuda.empty_cache()
    out["acoustic3d_400"] = _extra_acoustic3d(a, device)
    return out


def run_gb300(a):
    import torch

    rank, world, local = _dist()
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    sw, w = _workload(a.workload, a.shots, a.nt, a.check_freq)
    R = GradientRun(sw, w, local, bf16=a.bf16, precision=a.precision)
    if a.tz or a.variant >= 0:
        R.ctx.check(R.lib.sw_wavesim_set_tuning(R.h, a.tz, max(a.variant, 0)), "sw_wavesim_set_tuning")
    R.make_observed()
    tuned = None
    veff = a.variant
    if not (a.no_autotune or a.tz or a.variant >= 0):
        from seismicwaves_gb300 import tune

        allidx0 = list(range(len(w.shots)))
        arr = R.structs(allidx0, [x.data_ptr() for x in R.tf_d], [x.data_ptr() for x in R.tr_d],
                        [x.data_ptr() for x in R.obs_d])
        t0 = time.perf_counter()
        r = tune.autotune(R.ctx, R.h, (w.vp.shape, w.halo), arr, len(allidx0), w.vp.ndim, on_device=1,
                          gradient_out=(R.grad_d.data_ptr(), R.mis_d.data_ptr()), check_freq=w.check_freq)
        veff = r["variant"]
        bands = r["band_heights"]
        tuned = {"variant": r["variant"], "tz": r["tz"],
                 "band_heights": dict(zip(("forward", "recompute", "adjoint"), bands)) if bands else None,
                 "trial_ms": {"/".join(map(str, k)): round(t * 1e3, 3) for k, t in r["trial_s"].items()},
                 "per_kind_ms": {f"{v}/{tz}": {n: round(x, 3) for n, x in d.items()}
                                 for (v, tz), d in r["per_kind_ms"].items()},
                 "band_ms": {str(tz): {n: round(x, 3) for n, x in d.items()} for tz, d in r["band_ms"].items()},
                 "tuning_s": round(time.perf_counter() - t0, 2),
                 "what": "trials: batched gradients of the workload's shots capped at 2 K + 2 steps; each "
                         "candidate's best of 2 timed trials, per-kind ms from one event-timed trial; then "
                         "each stencil kind's band height from its own time"}
    nshots = len(w.shots)
    allidx = list(range(nshots))
    pts = float(w.point_steps())
    if a.forward_only:
        for _ in range(a.warmup):
            R.forward_device(allidx)
        clocks = ClockSampler(local)
        clocks.start()
        t_f = R.timed(lambda: R.forward_device(allidx), a.steps)
        clk = clocks.stop()
        R.ctx.profile(True)
        R.timed(lambda: R.forward_device(allidx), 1)
        R.ctx.profile(False)
        ms, nl, by = R.ctx.profile_read(0)
        peak, peak_kind = _peak()
        if rank == 0:
            print(json.dumps({"mode": "forward", "value": pts * a.steps / t_f / 1e9, "unit": UNIT,
                              "ms_per_step": t_f * 1e3 / a.steps, "steps": a.steps, "warmup": a.warmup,
                              "config": {"workload": w.name, "shots": nshots, "nt": max(s.nt for s in w.shots)},
                              "clocks": clk, "stencil": {"ms": ms, "launches": nl, "GB_per_s": by / (ms / 1e3) / 1e9,
                                                         "frac": by / (ms / 1e3) / 1e9 / peak, "peak": peak,
                                                         "peak_kind": peak_kind}}), flush=True)
        return

    def barrier():
        torch.cuda.synchronize(R.dev)
        if dist:
            dist.barrier()

    # warm-up (also allocates all device memory once and captures the CUDA graph)
    for _ in range(a.warmup):
        R.gradient_device(allidx)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t_dev = R.timed(lambda: R.gradient_device(allidx), a.steps)
    clk = clocks.stop()
    # one more gradient with per-kernel CUDA-event timing (direct launches) for the roofline
    R.ctx.profile(True)
    t_prof = R.timed(lambda: R.gradient_device(allidx), 1)
    R.ctx.profile(False)
    prof = {k: R.ctx.profile_read(k) for k in range(5)}
    kernels_per_call = sum(R.ctx.profile_kernels(k) for k in range(5))
    t_dev = max_over_ranks(t_dev, dist, R.dev)
    barrier()
    value = whole_job_rate(pts, a.steps, world, t_dev) / 1e9
    shots_per_s = whole_job_rate(nshots, a.steps, world, t_dev)

    # end to end through the C ABI with pinned host buffers (inputs up, gradient/traces down, every step)
    h2d, d2h = R.setup_host()
    R.gradient_host()
    t_e2e = max_over_ranks(R.timed(R.gradient_host, a.steps), dist, R.dev)
    e2e = whole_job_rate(pts, a.steps, world, t_e2e) / 1e9

    # plain per-shot path: the same library, one shot per call, with the library's own launch
    # shapes for a single shot (the batch's tuning does not carry over)
    plain = None
    if not a.no_plain:
        if tuned:
            R.ctx.check(R.lib.sw_wavesim_set_tuning(R.h, 0, 0), "sw_wavesim_set_tuning")
            R.ctx.check(R.lib.sw_wavesim_set_band_heights(R.h, 0, 0, 0), "sw_wavesim_set_band_heights")
        R.gradient_device([0])
        t_plain = R.timed(lambda: [R.gradient_device([i]) for i in allidx], 1)
        plain = {"value": pts / t_plain / 1e9, "unit": UNIT, "shots_per_s": nshots / t_plain,
                 "ms_per_step": t_plain * 1e3,
                 "what": "same kernels, one shot per call, the library's default launch shapes for one shot"}

    parity = None
    if rank == 0 and not a.no_parity and w.vp.ndim == 2:
        parity = _parity_2d(R, sw, w)
    if rank != 0:
        return
    # roofline of the dominant kernel (largest total time among the stencil kinds)
    nd = w.vp.ndim
    # 2D, 4-warp one-step stencil: the x strips run as extra blocks unless variant bit 18 is set
    xs = nd == 2 and not (veff >= 0 and veff & (262144 | 512 | 3))

    def kname(m):
        if nd == 3:
            return f"k_ac3d_inner + k_ac3d_zslab + k_ac3d_yslab<{m}>"
        return f"k_ac2d_step<{m}, XS> (x strips as extra blocks)" if xs else f"k_ac2d_step<{m}>"

    if nd == 2 and veff >= 0 and (veff & 256) and nshots >= 4:
        adj, adj_what = "k_ac2d_adj_grp", "adjoint + correlation (4 shots per block, Kahan sums)"
    elif nd == 2:
        adj, adj_what = kname(3), "adjoint + correlation (plain FP32 sums, FP64 flush every 32 steps)"
    else:
        adj, adj_what = kname(2), "adjoint + correlation (Kahan sums)"
    two = "k_ac2d_pair (two steps per launch) / " if (nd == 2 and veff >= 0 and veff & 1024) else ""
    kinds = {0: (f"{two}{kname('0/1')} forward", kname(1), "forward"),
             4: (f"{two}{kname(1)} recompute (writes D)", kname(1), "recompute"),
             1: (f"{two}{adj} {adj_what}", adj, "adjoint")}
    dom = max(kinds, key=lambda k: prof[k][0])
    ms_tot, launches, bytes_tot = prof[dom]
    achieved = bytes_tot / (ms_tot / 1e3) / 1e9 if ms_tot > 0 else None
    peak, peak_kind = _peak()
    algo_per_launch = bytes_tot / max(launches, 1)
    ratio = _traffic_ratio_from_profiles(kinds[dom][2], w.name)
    # whole gradient: the stencil kinds' algorithmic bytes over the timed step,
    # and the same step against the one-step-per-launch byte model of the path
    step_s = t_dev / a.steps
    kern_bytes = sum(prof[k][2] for k in kinds)
    model_bytes = _one_step_model_bytes(w)
    whole = {"kernel_bytes_per_step": kern_bytes, "frac": kern_bytes / step_s / 1e9 / peak,
             "one_step_model_bytes_per_step": model_bytes,
             "frac_vs_one_step_model": model_bytes / step_s / 1e9 / peak,
             "what": "frac: the kernels' own algorithmic bytes per gradient / ms_per_step / peak; "
                     "frac_vs_one_step_model: bytes a one-step-per-launch gradient must move (FP32 state, "
                     "K-step recompute, D buffer, correlation; strips and checkpoints) / ms_per_step / peak"}
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None,
            "traffic": ratio * algo_per_launch if ratio else None,
            "traffic_over_algorithmic": ratio,
            "kernel": kinds[dom][0], "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": bytes_tot / max(launches, 1),
            "avg_launch_us": ms_tot * 1e3 / max(launches, 1),
            "launches": launches,
            "kernels": {kinds[k][0]: {"ms": prof[k][0], "launches": prof[k][1],
                                      "GB_per_s": (prof[k][2] / (prof[k][0] / 1e3) / 1e9) if prof[k][0] else None}
                        for k in kinds}}
    if plain:  # the plain path moves at least the batch's stencil bytes (it re-reads `fact` per shot)
        plain["hbm_frac_lower_bound"] = kern_bytes / (plain["ms_per_step"] / 1e3) / 1e9 / peak
    # kernels per gradient (a profiled step may launch several) x timed gradients
    total_launches = kernels_per_call * a.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": t_dev * 1e3 / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "grid": list(w.vp.shape), "h_m": w.h[0], "shots": nshots,
                       "nt_range": [min(s.nt for s in w.shots), max(s.nt for s in w.shots)],
                       "receivers_range": [min(s.rec_pos.shape[0] for s in w.shots),
                                           max(s.rec_pos.shape[0] for s in w.shots)],
                       "check_freq": w.check_freq, "halo": w.halo,
                       "cache": "inputs larger than L2 (each step streams tens of GB of wavefield state)",
                       "precision": "fp32 wavefields and stencil, "
                                    + ("fp32 correlation sums flushed to fp64 every 32 steps"
                                       if (nd == 2 and not (veff >= 0 and (veff & 256)))
                                       else "Kahan fp32 correlation")
                                    + ", fp64 misfit and shot sum"
                                    + (", compensated double-fp32 forward passes" if a.precision else "")
                                    + (", bf16 recompute buffer" if a.bf16 >= 1 else "")
                                    + (", bf16 checkpoints" if a.bf16 >= 2 else ""),
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU, all shots batched"},
            "shots_per_s": shots_per_s,
            "plain": plain,
            "batched_vs_plain": (shots_per_s / plain["shots_per_s"]) if plain else None,
            "clocks": clk,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": total_launches,
            "roofline": roof,
            "whole_gradient": whole,
            "parity": parity,
            "tuning": tuned or {"tz": a.tz, "variant": a.variant},
            "launch": "CUDA graph per batch (captured in the warm-up, replayed in the timed steps)",
            "profiled_step_ms": t_prof * 1e3}
    if not a.no_cpu:
        import oracle

        oracle.load()
        v, threads, sample, _ = _cpu_baseline(sw, w, a.cpu_sample_nt)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    if not a.no_extras and world == 1 and a.workload == "acoustic2d_2001x801" and not (a.shots or a.nt):
        R.lib.sw_wavesim_destroy(R.h)
        del R
        line["extras"] = _extras(a, local)
    print(json.dumps(line), flush=True)


ELASTIC_KINDS = {0: "k_el_stress + k_el_disp forward", 4: "k_el_stress + k_el_disp recompute (writes slots)",
                 1: "k_el_stress + k_el_disp adjoint", 5: "k_el_corr4 gradient correlation"}


def measure_elastic(a, name="elastic2d_1200x600", shots=0, nt_cap=0, steps=None, warmup=None, plain=True,
                    cpu=True, device=0):
    """Batched elastic gradient: Gpts/s, shots/s, e2e, plain per-shot path, roofline of the dominant kind."""
    import torch

    steps = a.steps if steps is None else steps
    warmup = a.warmup if warmup is None else warmup
    sw, w = _workload(name, shots, nt_cap)
    R = ElasticRun(sw, w, device)
    tuned, tz = None, a.tz or 8
    if a.tz:
        R.ctx.check(R.lib.sw_elastic_set_tuning(R.h, a.tz), "sw_elastic_set_tuning")
    R.make_observed()
    if not (a.tz or a.no_autotune):
        tz, tuned = _tune_tz(R, w, "elastic", (8, 16, 32, 72, 136))
    nshots = len(w.shots)
    allidx = list(range(nshots))
    pts = float(w.point_steps())
    for _ in range(warmup):
        R.gradient_device(allidx)
    torch.cuda.synchronize(R.dev)
    clocks = ClockSampler(device)
    clocks.start()
    t_dev = R.timed(lambda: R.gradient_device(allidx), steps)
    clk = clocks.stop()
    R.ctx.profile(True)
    R.timed(lambda: R.gradient_device(allidx), 1)
    R.ctx.profile(False)
    prof = {k: R.ctx.profile_read(k) for k in range(6)}
    kernels_per_call = sum(R.ctx.profile_kernels(k) for k in range(6))
    h2d, d2h = R.setup_host()
    R.gradient_host()
    t_e2e = R.timed(R.gradient_host, steps)
    pl = None
    if plain:
        R.gradient_device([0])
        t_plain = R.timed(lambda: [R.gradient_device([i]) for i in allidx], 1)
        pl = {"value": pts / t_plain / 1e9, "unit": UNIT, "shots_per_s": nshots / t_plain,
              "ms_per_step": t_plain * 1e3, "what": "same kernels, one shot per call"}
    dom = max(ELASTIC_KINDS, key=lambda k: prof[k][0])
    ms_tot, launches, bytes_tot = prof[dom]
    achieved = bytes_tot / (ms_tot / 1e3) / 1e9 if ms_tot > 0 else None
    peak, peak_kind = _peak()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "traffic": None, "kernel": ELASTIC_KINDS[dom],
            "peak_kind": peak_kind,
            "kernels": {ELASTIC_KINDS[k]: {"ms": prof[k][0], "launches": prof[k][1],
                                           "GB_per_s": (prof[k][2] / (prof[k][0] / 1e3) / 1e9) if prof[k][0] else None}
                        for k in ELASTIC_KINDS},
            "other_kernels_ms": {"sources and receivers": prof[2][0], "misfit, scales, reduction": prof[3][0]}}
    out = {"metric": METRIC, "value": pts * steps / t_dev / 1e9, "unit": UNIT, "n_gpus": 1, "steps": steps,
           "warmup": warmup, "ms_per_step": t_dev * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": w.name, "grid": list(w.lam.shape), "h_m": w.h[0], "shots": nshots,
                      "nt": max(s.nt for s in w.shots), "receivers": w.shots[0].rec_pos.shape[0],
                      "check_freq": w.check_freq, "halo": w.halo, "sources": "explosive moment tensor, sinc spread",
                      "tz": tz, "tuning": tuned,
                      "cache": "inputs larger than L2 (each step streams several GB of wavefield state)",
                      "precision": "fp32 wavefields and stencil, Kahan fp32 correlation, fp64 misfit and shot sum"},
           "shots_per_s": nshots * steps / t_dev, "plain": pl,
           "batched_vs_plain": (nshots * steps / t_dev / pl["shots_per_s"]) if pl else None,
           "clocks": clk,
           "e2e": {"value": pts * steps / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h},
           "gpu_launches": kernels_per_call * steps, "roofline": roof}
    if cpu:
        import oracle

        oracle.load()
        v, threads, sample, _ = _elastic_cpu_baseline(sw, w, a.cpu_sample_nt)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    R.lib.sw_elastic_destroy(R.h)
    return out


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
        return
    try:
        if a.workload.startswith("acoustic_vd"):
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps(measure_vd(a, a.workload, a.shots, a.nt, plain=not a.no_plain,
                                            cpu=not a.no_cpu)), flush=True)
            return
        if a.workload.startswith("elastic"):
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps(measure_elastic(a, a.workload, a.shots, a.nt, plain=not a.no_plain,
                                                 cpu=not a.no_cpu)), flush=True)
            return
        run_gb300(a)
    finally:
        if int(os.environ.get("WORLD_SIZE", "1")) > 1:
            import torch.distributed as dist

            if dist.is_initialized():
                dist.destroy_process_group()


if __name__ == "__main__":
    main()
