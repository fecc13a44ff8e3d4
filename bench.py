"""Benchmark of the GB300 PBD step: particle-steps/s on the 1M-particle fluid workloads.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]
                    [--leg headline|contacts|batched|batched_frames|solids|adjoint|adjoint_physics|dense|render]

Our arm (default): the headline workload fluid_1m -- 100^3 = 1,000,000 fluid particles in a
128^3-cell domain (seed 2), kernel radius 1, 4 solver iterations, vorticity 5e-4, XSPH 0.01,
FP32 -- and beside it fluid_1m_dense, the same particles in the density regime of the
reference's config.txt (poly6 width 4.1, spiky width 3.5, two cell shells, lambda eps 1e-4,
~125 neighbours per particle), whose density constraint acts; its interior density error is
reported.  For each: `value` is particle-steps/s with the state resident in HBM (K frames
replayed as CUDA graphs, CUDA events on the launching stream); `e2e` drives the
reference-facing C ABI with host buffers each frame (pbd_clear + pbd_add_particles from pinned
memory, then pbd_step_readback: one frame and the final positions and velocities back into
pinned memory), copies inside the timed region.  The roofline entry is for the dominant
kernel, timed with CUDA event pairs around each launch (pbd_profile_frames) over K frames.

Reference arm (--impl reference): the reference step has no CPU implementation and its CUDA
code does not build with CUDA 13, so the arm times the oracle's FP32 OpenMP C
transliteration of the reference kernels on all host cores: the same workload, W untimed
frames, then exactly K timed frames -- the frames our arm times.  It never loads libpbd.so
(its parameters are config.txt's values filled in Python).

Under torchrun (N > 1) every rank steps its own replica of the workload ("replicas only":
the step has no exchange); value = particles x frames of all ranks / max rank time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pbd-simulation-framework-cuda_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s (plain 1M-particle PBD step)"
UNIT = "particle-steps/s"
L2_BYTES = 129 * 2 ** 20
DENSE = "fluid_1m_dense"
# interior particles of the density error: list length >= this share of the workload's bulk
# list length (the 90th percentile after the warm-up), kernel support clear of the walls
INTERIOR_SHARE = 0.9


def algorithmic_bytes_per_particle_step(iterations=4, passes=3, vort_visc=True):
    """B = 328 + 16 P + 88 I (vorticity and XSPH on) or 200 + 16 P + 88 I (off):
    each per-particle array read or written once per data-dependent pass, FP32 float4 state."""
    return (328 if vort_visc else 200) + 16 * passes + 88 * iterations


# per-particle algorithmic bytes of one launch of each kernel
KERNEL_BYTES = {
    "predict_key": 84,      # read x, v, f_ext (48), write v, p*, key (36)
    "onesweep_pass": 16,    # read key + value, write key + value
    "reorder_cells": 112,   # read perm, key (8), gather x, p*, v (48), write (48), cell writes (8)
    "lambda": 20,           # read p* (16), write lambda (4)
    "delta": 68,            # read p*, lambda, x (36), write p*, x (32); +16 for v on the last pass
    "omega": 48,            # read p*, v (32), write omega (16)
    "vort_visc": 80,        # read p*, v, omega (48), write f_ext, v (32)
    "update": 64,
}
# the same passes over the stored lists (full or near) do the same algorithmic work
for _k in ("lambda", "delta", "omega", "vort_visc"):
    KERNEL_BYTES[_k + "_list"] = KERNEL_BYTES[_k]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, dev):
    """The largest of a per-rank value over the job (the slowest replica's time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(particles_per_rank, frames, world, seconds):
    """Particle-steps/s of the whole job: every rank steps its own replica, the job takes as long
    as its slowest rank."""
    return particles_per_rank * frames * world / seconds


def build_workload(pbd, scenes, name, base=None):
    return scenes.workload(name, pbd, base=base)


def workload_config(name, params, n, world):
    """The bench line's `config`: the same dict for our arm and the reference arm."""
    w_set = n * (16 * 3 + 16 * 3 + 4 + 16 + 16 * 2) + 2 * params.max_grid * 4
    return {"workload": name, "particles": n, "domain_cells": int(round(params.bounds_max[0] + 1.5)),
            "solver_iterations": int(params.solver_iterations), "vorticity": float(params.e_vorticity),
            "xsph_viscosity": float(params.c_viscosity), "rest_density": float(params.rest_density),
            "lambda_epsilon": float(params.lambda_epsilon), "kernel_width_poly": float(params.kernel_width_poly),
            "kernel_width_spiky": float(params.kernel_width_spiky),
            "kernel_width_neighbours": int(params.kernel_width_neighbours), "parallelism": f"replicas x{world}",
            "l2": f"working set {w_set / 2**20:.0f} MiB > L2 {L2_BYTES / 2**20:.0f} MiB (no flush)"}


def bench_out_dir():
    d = os.environ.get("PBD_BENCH_OUT")
    if not d:
        import tempfile
        d = os.path.join(tempfile.gettempdir(), "pbd_bench")
    os.makedirs(d, exist_ok=True)
    return d


_REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}


class NvmlApi:
    """The three NVML reads the clock record needs (libnvidia-ml through ctypes; reads only)."""

    class _Pci(ctypes.Structure):
        _fields_ = [("busIdLegacy", ctypes.c_char * 16), ("domain", ctypes.c_uint), ("bus", ctypes.c_uint),
                    ("device", ctypes.c_uint), ("pciDeviceId", ctypes.c_uint), ("pciSubSystemId", ctypes.c_uint),
                    ("busId", ctypes.c_char * 32)]

    def __init__(self, pci):
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        count = ctypes.c_uint()
        self.lib.nvmlDeviceGetCount_v2(ctypes.byref(count))
        self.h = None
        for k in range(count.value):
            h = ctypes.c_void_p()
            if self.lib.nvmlDeviceGetHandleByIndex_v2(k, ctypes.byref(h)) != 0:
                continue
            info = NvmlApi._Pci()
            if self.lib.nvmlDeviceGetPciInfo_v3(h, ctypes.byref(info)) == 0 and \
                    (info.domain, info.bus, info.device) == tuple(pci):
                self.h = h
                break
        if self.h is None:
            raise RuntimeError("no NVML device with the CUDA device's PCI address")
        try:
            self._reasons = self.lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self._reasons = self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sm_mhz(self):
        v = ctypes.c_uint()
        return v.value if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(v)) == 0 else None

    def sm_max_mhz(self):
        v = ctypes.c_uint()
        return v.value if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(v)) == 0 else None

    def reasons(self):
        v = ctypes.c_ulonglong()
        return v.value if self._reasons(self.h, ctypes.byref(v)) == 0 else 0

    def close(self):
        self.lib.nvmlShutdown()


class NvmlClocks:
    """SM clock and clock-event reasons sampled every `period` s by a thread while the timed
    region runs (entering takes one sample first, so every sample counted lies in the region)."""

    def __init__(self, api, period=0.002):
        self.api = api
        self.period = period
        self.samples = []
        self.stop = threading.Event()
        self.thread = None
        self.max_mhz = None

    def _sample(self):
        self.samples.append((self.api.sm_mhz(), self.api.reasons()))

    def _run(self):
        while not self.stop.is_set():
            self._sample()
            self.stop.wait(self.period)

    def __enter__(self):
        self.max_mhz = self.api.sm_max_mhz()
        self.api.sm_mhz()
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.thread.join(timeout=5)
        self._sample()

    def summary(self):
        sms = [m for m, _ in self.samples if m is not None]
        reasons = set()
        for _, bits in self.samples:
            for name, b in _REASON_BITS.items():
                if bits & b:
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sms)) if sms else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(reasons), "samples": len(sms), "source": f"nvml every {self.period * 1e3:.0f} ms"}


def clock_sampler(torch, local):
    """NVML sampling of the CUDA device `local`, else nvidia-smi's."""
    try:
        pr = torch.cuda.get_device_properties(local)
        return NvmlClocks(NvmlApi((pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)))
    except Exception:  # noqa: BLE001
        return ClockSampler(local)


class ClockSampler:
    """nvidia-smi samples (every 50 ms) during the timed region: entering waits for the first
    sample, which is left out of the summary, so every sample counted was taken inside the
    region.  The fallback when NVML cannot be loaded."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.skip = 0
        # PBD_BENCH_OUT keeps the samples (and the autotuner's cache) in a folder of the caller's
        # choosing; by default they go to a temporary folder
        self.path = os.path.join(bench_out_dir(), f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
            with open(self.path) as f:
                self.skip = len(f.readlines())
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path).readlines()[self.skip:]:
                f = [t.strip() for t in line.split(",")]
                if len(f) < 7:
                    continue
                try:
                    sms.append(float(f[0]))
                    mx = float(f[1])
                except ValueError:
                    continue
                for k, nm in enumerate(names):
                    if f[3 + k].lower().startswith("active"):
                        reasons.add(nm)
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sms)) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms), "source": "nvidia-smi every 50 ms"}


def oracle_params(scenes, name):
    """The workload's parameters and lattice for the CPU oracle, without the library."""
    import pbd   # the Params structure only: pbd.py loads libpbd.so on first use, never here
    return scenes.workload(name, pbd, base=scenes.config_txt_params(pbd.Params))


def cpu_baseline(name, max_seconds, threads=None):
    """FP32 OpenMP transliteration of the reference step (oracle build), timed on host cores over
    a bounded sample: frames after one untimed frame until `max_seconds` have passed."""
    import scenes
    from oracle import oracle as orc_mod
    params, pos, vel, w = oracle_params(scenes, name)
    if threads:
        orc_mod.set_threads(threads)
    cores = orc_mod.max_threads()
    o = orc_mod.Oracle(params, len(pos), "f32")
    o.add_particles(pos, vel)
    o.step(1)   # first frame (page faults of the list) outside the sample
    frames, t0 = 0, time.perf_counter()
    while True:
        o.step(1)
        frames += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or frames >= 1000:
            break
    o.close()
    rate = len(pos) * frames / el
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{name}: {len(pos)} particles x {frames} frames (after 1 untimed), {el:.1f} s, FP32 OpenMP"}


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_batched(torch, pbd, scenes, stream, sh, frames):
    """256 seeded dam-break scenes (4K-65K particles, rest density 900-1100, |g| 8-11, domains
    32-96 cells): scenes/s advanced as one batch vs the same scenes stepped one by one."""
    sl = scenes.batched_scenes()
    shared = scenes.workload_params(pbd, 64, 1000.0)
    shared.lambda_epsilon = 0.1
    descs = [pbd.scene_desc(sc["n"], sc["rest_density"], sc["gravity"], sc["box"]) for sc in sl]
    total = sum(sc["n"] for sc in sl)
    tune_cache = os.environ.get("PBD_TUNE_CACHE", os.path.join(bench_out_dir(), "autotune.jsonl"))
    os.makedirs(os.path.dirname(tune_cache), exist_ok=True)
    with pbd.Batch(shared, descs) as tb:            # tuning copy: the autotuner advances frames
        for k, sc in enumerate(sl):
            tb.add_particles(k, sc["pos"], sc["vel"])
        block = tb.autotune(tune_cache, stream=sh)
        stream.synchronize()
        tb.sync()
    b = pbd.Batch(shared, descs)
    for k, sc in enumerate(sl):
        b.add_particles(k, sc["pos"], sc["vel"])
    b.autotune(tune_cache, stream=sh)              # served from the cache: no frames consumed
    b.step(3, stream=sh)
    stream.synchronize()
    e0, e1 = _events(torch)
    torch.cuda.synchronize()
    e0.record(stream)
    b.step(frames, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    b.sync()
    ms_batch = e0.elapsed_time(e1) / frames
    launches = b.launches_per_step()
    # the same frames' kernels one by one (direct launches, an event pair around each): what the
    # graph's frame costs beyond its kernels is the room a persistent kernel could win back
    prof = b.profile(frames, stream=sh)
    b.sync()
    kernel_sum = sum(v[1] for v in prof.values()) / frames
    b.close()
    sims = []
    for sc in sl:
        p = shared.copy()
        p.rest_density = sc["rest_density"]
        p.gravity = sc["gravity"]
        for a in range(3):
            p.bounds_min[a] = 1.5
            p.bounds_max[a] = sc["box"] - 1.5
        x = pbd.Sim(p, sc["n"])
        x.add_particles(sc["pos"], sc["vel"])
        sims.append(x)
    for x in sims:
        x.step(3, stream=sh)
    one_frames = max(5, frames // 4)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(one_frames):
        for x in sims:
            x.step(1, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_one = e0.elapsed_time(e1) / one_frames
    for x in sims:
        x.sync()
        x.close()
    return {"workload": "batched_256", "scenes": len(sl), "particles": total, "frames": frames,
            "ms_per_frame": ms_batch, "scenes_per_s": len(sl) * 1e3 / ms_batch,
            "particle_steps_per_s": total * 1e3 / ms_batch, "launches_per_frame": launches,
            "neighbour_block": block, "kernel_ms_per_frame": {k: v[1] / frames for k, v in prof.items()},
            "kernel_sum_ms_per_frame": kernel_sum, "graph_minus_kernels_ms": ms_batch - kernel_sum,
            "one_by_one_ms_per_frame": ms_one,
            "one_by_one_scenes_per_s": len(sl) * 1e3 / ms_one, "speedup_vs_one_by_one": ms_one / ms_batch}


def run_solids(torch, pbd, scenes, stream, sh, frames):
    """64^3 fluid + 8 static solid boxes (65,536 solids), 128^3 domain: particle-steps/s."""
    pos, vel, w = scenes.solids_scene()
    p = scenes.workload_params(pbd, 128, 1000.0)
    p.lambda_epsilon = 0.1
    with pbd.Sim(p, len(pos)) as sim:
        sim.add_particles_mass(pos, vel, w)
        sim.step(3, stream=sh)
        stream.synchronize()
        e0, e1 = _events(torch)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(frames, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        sim.sync()
        ms = e0.elapsed_time(e1) / frames
        st = sim.state()
    solid_ids = np.nonzero(w == 0)[0]
    return {"workload": "solids_328k", "particles": len(pos), "solid_particles": int(len(solid_ids)), "frames": frames,
            "ms_per_frame": ms, "particle_steps_per_s": len(pos) * 1e3 / ms}


def run_adjoint(torch, pbd, scenes, stream, sh, frames=60, every=10, fd_check=True, short=(10, 5, 2),
                physics=False):
    """Differentiable dam break (65,536 particles, 60 frames x 4 iterations, checkpoints every
    10): device time of forward+adjoint against the forward alone, and the gradient of
    L = mean |x_final - target|^2 along a seeded direction of v0 and for rest density and eps,
    against central differences of the FP64 oracle (the step 1e-3, and a step near the FP32
    resolution of the parameter), at the full horizon and at a short one.  physics: the same
    scene with the fluid workload's vorticity confinement (5e-4) and XSPH viscosity (0.01), both
    differentiated (timing only)."""
    pos, vel, target = scenes.adjoint_dam_break()
    n = len(pos)
    p = scenes.workload_params(pbd, 72, 1000.0, vorticity=0.0005 if physics else 0.0, viscosity=0.01 if physics else 0.0)
    p.lambda_epsilon = 0.1
    p.flags &= ~pbd.FLAG_CELL_END_QUIRK
    p.flags |= pbd.FLAG_TRACK_IDS

    def dl_dx(state):
        g = np.zeros((n, 4), np.float32)
        g[:, :3] = 2.0 * (state["x"][:, :3] - target[state["ids"]]) / n
        return g

    def gradients(sim, horizon):
        sim.clear()
        sim.add_particles(pos, vel)
        sim.adjoint_forward(horizon, every, stream=sh)
        fin = sim.state()
        loss = float(np.mean(np.sum((fin["x"][:, :3] - target[fin["ids"]]) ** 2, axis=1)))
        gv, gx, gr, ge = sim.adjoint_backward(dl_dx(fin), stream=sh)
        return loss, gv, gr, ge

    e0, e1 = _events(torch)
    e2 = torch.cuda.Event(enable_timing=True)
    with pbd.Sim(p, n) as sim:
        loss, gv, gr, ge = gradients(sim, frames)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(frames, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_fwd = e0.elapsed_time(e1)
        g = dl_dx(sim.state())
        torch.cuda.synchronize()
        e0.record(stream)
        sim.adjoint_forward(frames, every, stream=sh)
        e2.record(stream)
        sim.adjoint_backward(g, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_adj = e0.elapsed_time(e1)
        ms_adj_fwd = e0.elapsed_time(e2)
        short_grads = [gradients(sim, h) for h in short] if fd_check else []
        sim.sync()
    out = {"workload": "adjoint_64k" + ("_vorticity_xsph" if physics else ""), "particles": n, "frames": frames,
           "iterations": p.solver_iterations,
           "checkpoint_every": every, "loss": loss, "forward_ms": ms_fwd, "forward_plus_adjoint_ms": ms_adj,
           "adjoint_forward_ms": ms_adj_fwd, "adjoint_backward_ms": ms_adj - ms_adj_fwd,
           "cost_ratio": ms_adj / ms_fwd, "dL_drest_density": gr, "dL_deps": ge,
           "dL_dv0_norm": float(np.linalg.norm(gv[:, :3]))}
    if fd_check:
        from oracle import oracle as orc_mod
        rng = np.random.default_rng(5)
        dirn = rng.normal(size=(n, 3))

        def oloss(prm, vel0, horizon):
            o = orc_mod.Oracle(prm, n, "f64")
            o.add_particles(pos, vel0)
            o.step(horizon)
            s2 = o.state()
            o.close()
            return float(np.mean(np.sum((s2["x"][:, :3] - target[s2["ids"]]) ** 2, axis=1)))

        def fd_param(field, h, horizon):
            pp, pm = p.copy(), p.copy()
            setattr(pp, field, getattr(p, field) + h)
            setattr(pm, field, getattr(p, field) - h)
            step = float(np.float32(getattr(pp, field))) - float(np.float32(getattr(pm, field)))   # FP32 fields
            return (oloss(pp, vel, horizon) - oloss(pm, vel, horizon)) / step

        def fd_v0(h, horizon, gvh):
            vp, vm = vel.copy(), vel.copy()
            vp[:, :3] += (h * dirn).astype(np.float32)
            vm[:, :3] -= (h * dirn).astype(np.float32)
            step = vp[:, :3].astype(np.float64) - vm[:, :3].astype(np.float64)
            return (oloss(p, vp, horizon) - oloss(p, vm, horizon)), float(np.sum(gvh[:, :3].astype(np.float64) * step))

        def rel(a, b):
            return abs(a - b) / max(abs(b), 1e-30)

        t0 = time.perf_counter()
        checks = {}
        for horizon, (lo, gvh, grh, geh) in ((frames, (loss, gv, gr, ge)), *zip(short, short_grads)):
            c = {"loss": lo}
            for name, field, ad, small in (("rest_density", "rest_density", grh, 1.25e-4), ("eps", "lambda_epsilon", geh, 1e-7)):
                for h in (1e-3, small):
                    fd = fd_param(field, h, horizon)
                    c[f"{name}@h={h:g}"] = {"adjoint": ad, "fd_fp64": fd, "rel": rel(ad, fd)}
            for h in (1e-3, 1e-6):
                fd, ad = fd_v0(h, horizon, gvh)
                c[f"v0_direction@h={h:g}"] = {"adjoint": ad, "fd_fp64": fd, "rel": rel(ad, fd)}
            # a check is conclusive only where the FP64 differences at the two steps agree with
            # each other (the loss is smooth there); beyond that horizon the dynamics are not
            ok = {}
            for name, steps in (("rest_density", (1e-3, 1.25e-4)), ("eps", (1e-3, 1e-7)), ("v0_direction", (1e-3, 1e-6))):
                a, b = (c[f"{name}@h={h:g}"]["fd_fp64"] / (h if name == "v0_direction" else 1.0) for h in steps)
                ok[name] = rel(a, b) < 0.1
            c["fd_steps_agree"] = ok
            # the 1e-3 target: the parameters against the step-1e-3 differences, dL/dv0 against the
            # small-step ones (its step-1e-3 differences are not converged: see fd_steps_agree's spread)
            c["within_1e-3"] = {"rest_density": c["rest_density@h=0.001"]["rel"] < 1e-3,
                                "eps": c["eps@h=0.001"]["rel"] < 1e-3,
                                "v0_direction": c["v0_direction@h=1e-06"]["rel"] < 1e-3}
            checks[f"{horizon}_frames"] = c
        out["gradient_check"] = checks
        met = [h for h in (frames, *short) if all(checks[f"{h}_frames"]["within_1e-3"].values())]
        out["largest_horizon_within_1e-3"] = max(met) if met else 0
        out["largest_horizon_within_1e-3_by_gradient"] = {
            name: max([h for h in (frames, *short) if checks[f"{h}_frames"]["within_1e-3"][name]] or [0])
            for name in ("rest_density", "eps", "v0_direction")}
        out["gradient_check_s"] = time.perf_counter() - t0
    return out


def run_contacts(torch, pbd, scenes, stream, sh, frames):
    """The large-fluid workload with collisionType 1 (contact constraints in batches of disjoint
    pairs, maxCollisionBatches 16): particle-steps/s."""
    params, pos, vel, _ = build_workload(pbd, scenes, "fluid_1m")
    params.collision_type = 1
    params.max_collision_batches = 16
    with pbd.Sim(params, len(pos)) as sim:
        sim.add_particles(pos, vel)
        sim.step(3, stream=sh)
        stream.synchronize()
        e0, e1 = _events(torch)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(frames, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        sim.sync()
        ms = e0.elapsed_time(e1) / frames
        prof = sim.profile(3, stream=sh)
        sim.sync()
    return {"workload": "fluid_1m, collisionType 1", "particles": len(pos), "frames": frames,
            "max_collision_batches": 16, "ms_per_frame": ms, "particle_steps_per_s": len(pos) * 1e3 / ms,
            "kernel_ms_per_frame": {k: v[1] / 3 for k, v in prof.items()}}


def run_render(torch, pbd, sim, stream, sh, reps=10):
    """Headless sprites of the simulation's current state at 1920 x 1080 (device time per image,
    no copies to the host; plus one call that also copies RGBA and depth back)."""
    cam = pbd.camera(eye=(230.0, 150.0, 250.0), center=(64.0, 30.0, 64.0), width=1920, height=1080)
    L = pbd.lib()
    sim.render(cam, stream=sh)                     # workspace + warm-up
    e0, e1 = _events(torch)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        pbd.check(L.pbd_render_sprites(sim.h, pbd.C.byref(cam), None, None, pbd.C.c_void_p(sh)))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    t0 = time.perf_counter()
    rgba, depth = sim.render(cam, stream=sh)
    ms_host = (time.perf_counter() - t0) * 1e3
    return {"width": 1920, "height": 1080, "particles": sim.n, "ms_per_image": ms,
            "sprites_per_s": sim.n * 1e3 / ms, "ms_with_host_copies": ms_host,
            "covered_pixel_fraction": float((depth < 1.0).mean())}


def run_reference(args):
    """The oracle's FP32 OpenMP port of the reference kernels on all host cores, the workload our
    arm times: W untimed frames, then exactly K timed frames (rank 0 only)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import scenes
    from oracle import oracle as orc_mod
    params, pos, vel, w = oracle_params(scenes, args.workload)
    n = len(pos)
    cores = orc_mod.max_threads()
    o = orc_mod.Oracle(params, n, "f32")
    o.add_particles(pos, vel)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    el = time.perf_counter() - t0
    o.close()
    value = job_throughput(n, args.steps, 1, el)
    sample = (f"{args.workload}: {n} particles, frames {args.warmup + 1}-{args.warmup + args.steps} "
              f"(after {args.warmup} untimed), {el:.1f} s, FP32 OpenMP")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice, SplitMix64)",
            "config": workload_config(args.workload, params, n, args.gpus),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:  # noqa: BLE001
        return {}


def traffic_of(name, kernel):
    """ncu DRAM bytes of one launch of `kernel` on workload `name` (profiles/traffic.json)."""
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        return t.get(name, {}).get(kernel)
    except Exception:  # noqa: BLE001
        return None


def measure_workload(torch, pbd, scenes, name, args, stream, sh, world, dev, local, extra=None, staged_compare=False):
    """value, e2e, clocks, roofline, per-kernel time and density error of one workload: W warm-up
    frames, K timed frames (graph replays, CUDA events), K profiled frames, then e2e over the
    same frames as the timed ones on a fresh simulation."""
    params, pos, vel, w = build_workload(pbd, scenes, name)
    n = len(pos)
    sim = pbd.Sim(params, n)
    sim.add_particles(pos, vel)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- warm-up (also records the CUDA graphs); the bulk list length for the interior
    sim.step(args.warmup, stream=sh)
    stream.synchronize()
    sim.sync()
    launches_per_step = sim.launches_per_step()
    _, cnt, _ = sim.neighbours(0)
    min_nb = int(INTERIOR_SHARE * np.percentile(cnt, 90))

    # ---- device-resident timing
    ev0, ev1 = _events(torch)
    with clock_sampler(torch, local) as clocks:
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        sim.step(args.steps, stream=sh)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    sim.sync()
    ms = ev0.elapsed_time(ev1)
    t_rank = max_over_ranks(ms / 1e3, world, dev)
    value = job_throughput(n, args.steps, world, t_rank)

    # ---- density constraint after the timed frames: all particles, and the interior ones
    _, derr_mean, derr_max = sim.density_error(stream=sh)
    margin = float(max(params.kernel_width_poly, 1.0))
    imean, imax, icount = sim.density_error_interior(min_nb, margin, stream=sh)
    density = {"mean": derr_mean, "max": derr_max, "interior_mean": imean, "interior_max": imax,
               "interior_particles": icount, "interior_rule": f"list length >= {min_nb} "
               f"({INTERIOR_SHARE} x the 90th percentile after the warm-up), more than {margin} inside every wall",
               "after_frames": args.warmup + args.steps}
    out_extra = extra(sim) if extra else {}

    # ---- per-kernel device time over the next K frames (direct launches)
    prof = sim.profile(args.steps, stream=sh)
    stream.synchronize()
    sim.sync()
    share = {k: v[1] for k, v in prof.items()}
    top = max(share, key=share.get)
    launches, total_ms = prof[top]
    per_launch_s = total_ms / launches / 1e3
    bytes_per = KERNEL_BYTES.get(top, 0) * n
    if top in ("delta", "delta_list"):
        # one of I delta launches also writes v: average the extra 16 B over the I launches
        bytes_per += 16 * n / params.solver_iterations
    achieved = bytes_per / per_launch_s / 1e9
    peaks = load_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    # ---- end to end through the reference-facing ABI with host buffers, over the same frames
    # of the run as the timed ones: a fresh simulation from the initial state, the same warm-up
    sim.close()
    sim = pbd.Sim(params, n)
    sim.add_particles(pos, vel)
    sim.step(args.warmup, stream=sh)
    stream.synchronize()
    sim.sync()
    e2e_steps = max(3, args.steps)
    hx = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
    hv = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
    st = sim.state()
    hx[:] = st["x"]
    hv[:] = st["v"]
    xp = hx.ctypes.data_as(pbd.C.POINTER(pbd.C.c_float))
    vp = hv.ctypes.data_as(pbd.C.POINTER(pbd.C.c_float))
    L = pbd.lib()
    # each frame: the state in from pinned host memory, one step, the state out to pinned host
    # memory (pbd_step_readback); the next frame's input is this frame's output
    src = [xp, vp]
    rx, rv = pbd.C.POINTER(pbd.C.c_float)(), pbd.C.POINTER(pbd.C.c_float)()

    def e2e_frame():
        pbd.check(L.pbd_clear(sim.h))
        pbd.check(L.pbd_add_particles(sim.h, n, src[0], src[1], None))
        pbd.check(L.pbd_step_readback(sim.h, 1, pbd.C.c_void_p(sh), pbd.C.byref(rx), pbd.C.byref(rv)))
        src[0], src[1] = rx, rv

    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_frame()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_value = job_throughput(n, e2e_steps, world, t_e2e)
    sim.sync()
    sim.close()

    staged = None
    if staged_compare:
        # the same K frames with the shared-memory-staged lambda and delta passes
        # (PBD_FLAG_STAGED_PASSES), on a fresh simulation after the same warm-up
        ps = params.copy()
        ps.flags |= pbd.FLAG_STAGED_PASSES
        with pbd.Sim(ps, n) as sim:
            sim.add_particles(pos, vel)
            sim.step(args.warmup, stream=sh)
            stream.synchronize()
            e0, e1 = _events(torch)
            torch.cuda.synchronize()
            e0.record(stream)
            sim.step(args.steps, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            sim.sync()
            sprof = sim.profile(args.steps, stream=sh)
            sim.sync()
        sms = e0.elapsed_time(e1) / args.steps
        staged = {"ms_per_step": sms, "value": n * 1e3 / sms, "vs_lists": (ms / args.steps) / sms,
                  "kernel_ms_per_frame": {k: v[1] / args.steps for k, v in sprof.items()}}

    bps = algorithmic_bytes_per_particle_step(params.solver_iterations, 3,
                                              bool(params.active & (pbd.ACTIVE["computeOmegas"] | pbd.ACTIVE["computeViscosity"])))
    return {
        "value": value, "ms_per_step": ms / args.steps, "particles": n,
        "config": workload_config(name, params, n, world),
        "clocks": clocks.summary(),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "frames": e2e_steps, "first_frame": args.warmup + 1},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic_of(name, top),
                     "algorithmic_bytes_per_launch": bytes_per, "launch_ms": per_launch_s * 1e3},
        "step_roofline": {"bytes_per_particle_step": bps, "achieved_gbs": bps * value / world / 1e9,
                          "frac": bps * value / world / 1e9 / peak},
        "kernel_ms_per_frame": {k: v[1] / args.steps for k, v in prof.items()},
        "density_error": density,
        **({"staged_passes": staged} if staged is not None else {}),
        **out_extra,
    }


def run_ours(args):
    import torch
    import pbd
    import scenes

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def render_of(sim):
        # headless sprites of the state after the timed frames
        try:
            return {"render": run_render(torch, pbd, sim, stream, sh)}
        except Exception as e:  # noqa: BLE001
            return {"render": {"error": f"{type(e).__name__}: {e}"}}

    head = measure_workload(torch, pbd, scenes, args.workload, args, stream, sh, world, dev, local, extra=render_of)

    def leg(fn, *a, **k):
        # a failing secondary leg is reported in the line instead of losing the headline number
        try:
            return fn(*a, **k)
        except Exception as e:  # noqa: BLE001
            return {"error": f"{type(e).__name__}: {e}"}

    dense = None
    if args.workload != DENSE:
        dense = leg(measure_workload, torch, pbd, scenes, DENSE, args, stream, sh, world, dev, local, staged_compare=True)
    batched = leg(run_batched, torch, pbd, scenes, stream, sh, frames=max(10, min(args.steps, 60)))
    solids = leg(run_solids, torch, pbd, scenes, stream, sh, frames=max(10, min(args.steps, 100)))
    adjoint = leg(run_adjoint, torch, pbd, scenes, stream, sh, fd_check=not args.no_fd_check)
    adjoint_physics = leg(run_adjoint, torch, pbd, scenes, stream, sh, fd_check=False, physics=True)
    contacts = leg(run_contacts, torch, pbd, scenes, stream, sh, frames=20)

    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice, SplitMix64)",
        "config": head["config"], "clocks": head["clocks"], "e2e": head["e2e"], "gpu_launches": head["gpu_launches"],
        "roofline": head["roofline"], "step_roofline": head["step_roofline"],
        "kernel_ms_per_frame": head["kernel_ms_per_frame"], "density_error": head["density_error"],
        "dense": dense, "batched": batched, "solids": solids, "adjoint": adjoint, "adjoint_physics": adjoint_physics,
        "contacts": contacts,
        "render": head.get("render"),
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_leg(args):
    """One secondary workload alone, e.g. as the target of a profiler."""
    import torch
    import pbd
    import scenes
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    if args.leg == "contacts":
        out = run_contacts(torch, pbd, scenes, stream, sh, frames=max(3, min(args.steps, 20)))
    elif args.leg == "batched":
        out = run_batched(torch, pbd, scenes, stream, sh, frames=max(10, min(args.steps, 60)))
    elif args.leg == "solids":
        out = run_solids(torch, pbd, scenes, stream, sh, frames=max(10, min(args.steps, 100)))
    elif args.leg == "headline":
        out = measure_workload(torch, pbd, scenes, args.workload, args, stream, sh, 1, torch.device("cuda", 0), 0)
    elif args.leg == "dense":
        out = measure_workload(torch, pbd, scenes, DENSE, args, stream, sh, 1, torch.device("cuda", 0), 0,
                               staged_compare=True)
    elif args.leg == "batched_frames":
        # the 256-scene batch alone: W + K frames (a profiler target; no tuning, no single scenes)
        sl = scenes.batched_scenes()
        shared = scenes.workload_params(pbd, 64, 1000.0)
        shared.lambda_epsilon = 0.1
        descs = [pbd.scene_desc(sc["n"], sc["rest_density"], sc["gravity"], sc["box"]) for sc in sl]
        with pbd.Batch(shared, descs) as b:
            for k, sc in enumerate(sl):
                b.add_particles(k, sc["pos"], sc["vel"])
            b.step(args.warmup + args.steps, stream=sh)
            b.sync()
        out = {"scenes": len(sl), "frames": args.warmup + args.steps}
    elif args.leg == "render":
        params, pos, vel, _ = build_workload(pbd, scenes, "fluid_1m")
        with pbd.Sim(params, len(pos)) as sim:
            sim.add_particles(pos, vel)
            sim.step(args.warmup + args.steps, stream=sh)
            out = run_render(torch, pbd, sim, stream, sh, reps=3)
    else:
        out = run_adjoint(torch, pbd, scenes, stream, sh, fd_check=not args.no_fd_check and args.leg == "adjoint",
                          physics=args.leg == "adjoint_physics")
    print(json.dumps({"leg": args.leg, **out}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fluid_1m")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-fd-check", action="store_true", help="skip the FP64 finite-difference check of the adjoint")
    ap.add_argument("--leg", choices=["headline", "contacts", "batched", "batched_frames", "solids", "adjoint",
                                      "adjoint_physics", "dense", "render"],
                    help="measure only this secondary workload and print its result (not the bench line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.leg:
        return run_leg(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
