#!/usr/bin/env python
"""Benchmark of the BP+EE energy-and-force path on GB300.

Default workload: one energy+force evaluation of the 24,000-atom open water
cube (8,000 H2O; elements H, O; 3 x 512 relu networks for energy and charge;
DSF/elu Coulomb + C6 vdW at 15 A), synthetic seeded inputs and random-init
weights. One step = one E+F (neighbour lists, descriptors, both networks
forward and backward, pair terms, forces).

  value     atom-steps/s of the fused-adjoint FP32 path with positions already
            in HBM (device pointers through the C ABI), CUDA events on the
            library's stream, L2 flushed between timed steps
  e2e       the same through the public API with host buffers: H2D of the
            positions and D2H of energies + forces inside the timed region
  plain_autograd  torch-op graph + torch.autograd.grad over the same lists
  bf16      the fused path with 1-pass BF16 network GEMMs
  roofline  network GEMMs (the dominant kernel) vs the measured BF16 peak
  cpu_baseline  the FP64 oracle on the host cores (one full E+F)

``--impl reference`` times the CPU implementation of the path (the oracle
port: the reference's TensorFlow graph cannot run here) on the same 24,000-atom
cube, one full E+F per step.
Multi-GPU runs are independent replicas (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

METRIC = "atom-steps/s E+F, fused adjoint vs plain autograd, 1 GB300; serve p50/p99 ms"
UNIT = "atom-steps/s"
# DRAM bytes of the six k_gemm launches of one evaluation (one ncu capture; the
# k_gemm summary under profiles/ gives the command and the per-launch figures)
GEMM_DRAM_BYTES_PER_STEP = 1_706_279_000
# Warp instructions per evaluation of the instruction-issue-bound kernels on
# this workload (smsp__inst_executed.sum, one ncu capture; the
# instruction-count summary under profiles/ gives the command). Their
# roofline is the issue rate: 4 warp instructions per clock per SM.
ISSUE_INST_PER_STEP = {"descriptors": {"k_desc_fwd": 114_775_011},
                       "adjoint_gather": {"k_desc_adj": 135_380_912, "k_force_gather": 11_101_129},
                       "pair_terms": {"k_coulomb": 213_111_838}}
WORKLOAD = ("water cube: 8,000 H2O = 24,000 atoms, open boundary, O on a 3.1 A lattice "
            "+-0.2 A jitter, single energy+force")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_ranks(ms, natoms, ws, device="cuda"):
    """Replicas over ws ranks (one per GPU, each timing the same workload on
    its own device): the step time is the maximum over ranks and the value
    counts every rank's atoms. Needs an initialised process group when ws > 1
    (NCCL on GPUs; gloo with device="cpu")."""
    if ws > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, ws * natoms / (ms / 1000.0)


def _peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        import tempfile
        self.f = os.path.join(tempfile.gettempdir(), f"tm_clocks_{os.getpid()}.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=open(self.f, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.f):
            parts = [t.strip() for t in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_workload(precision="fp32"):
    from tensormol_gb300 import systems
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS, descriptor_width
    w = systems.water_cube_24k(seed=1)
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    model = BPEEModel(eles, W, params=dict(PARAMS), precision=precision)
    return w, eles, W, model


def time_fused_device(model, w, steps, warmup, flush, torch):
    """value: device-resident positions, CUDA events on the library's stream."""
    s = model.system(w.x, w.Z, w.offsets)
    stream = torch.cuda.ExternalStream(int(model.ctx.stream or 0))
    x_dev = torch.tensor(w.x, dtype=torch.float64, device="cuda")
    E_dev = torch.zeros((1, 4), dtype=torch.float64, device="cuda")
    F_dev = torch.zeros((w.natoms, 3), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(warmup):
        s.energy_force_device(x_dev.data_ptr(), E_dev.data_ptr(), F_dev.data_ptr())
    torch.cuda.synchronize()
    l0 = model.ctx.launches
    times = []
    clocks = Clocks()
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
        s.energy_force_device(x_dev.data_ptr(), E_dev.data_ptr(), F_dev.data_ptr())
        with torch.cuda.stream(stream):
            b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    ck = clocks.stop()
    launches = (model.ctx.launches - l0)
    F = F_dev.cpu().numpy()
    E = E_dev.cpu().numpy()
    return s, times, launches, ck, E, F


def time_e2e(model, s, w, steps, warmup, torch):
    """e2e: host (pinned) positions in, energies + forces out, through the ABI."""
    import ctypes
    xh = torch.tensor(w.x, dtype=torch.float64).pin_memory()
    Eh = torch.zeros((1, 4), dtype=torch.float64).pin_memory()
    Fh = torch.zeros((w.natoms, 3), dtype=torch.float64).pin_memory()
    stream = torch.cuda.ExternalStream(int(model.ctx.stream or 0))
    lib = model.lib

    def call():
        model.ctx.check(lib.tm_energy_force(s.h, ctypes.c_void_p(xh.data_ptr()), 0,
                                            ctypes.c_void_p(Eh.data_ptr()), ctypes.c_void_p(Fh.data_ptr()),
                                            None, None, None))
    for _ in range(warmup):
        call()
    times = []
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        call()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return times, int(xh.numel() * 8), int((Eh.numel() + Fh.numel()) * 8)


def time_plain(model, W, w, steps, warmup, torch):
    from tensormol_gb300.plain import PlainAutograd
    s = model.system(w.x, w.Z, w.offsets)
    pl = PlainAutograd(model, W)
    x = torch.tensor(w.x, dtype=torch.float64, device="cuda")

    for _ in range(warmup):
        s.build_nlist()
        pl.prepare(s)
        pl.energy_force(x)
    torch.cuda.synchronize()
    times, t_lists, t_graph = [], [], []
    E = F = None
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        m = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        # lists: the library's build, exported to index tensors (as the
        # reference's graph is fed its lists by the host)
        s.build_nlist()
        pl.prepare(s)
        m.record()
        # the framework-op graph and torch.autograd.grad
        E, F = pl.energy_force(x)
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
        t_lists.append(a.elapsed_time(m))
        t_graph.append(m.elapsed_time(b))
    out = (E.cpu().numpy(), F.cpu().numpy())
    s.close()
    del pl
    torch.cuda.empty_cache()
    return times, out, t_lists, t_graph


def oracle_eval(w, eles, W):
    import torch
    torch.set_num_threads(os.cpu_count() or 1)
    from oracle import reference as orc
    from tensormol_gb300.params import PARAMS
    t0 = time.perf_counter()
    o = orc.OpenSystemOracle(orc.Model(eles, W, dict(PARAMS)), w.x, w.Z, w.offsets)
    ref = o.terms(w.x)
    return ref, time.perf_counter() - t0


def errors(E, F, ref, natoms):
    from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE
    dE = abs(float(np.ravel(E)[0]) - float(ref["Etotal"][0])) * EV_PER_HARTREE / natoms
    per_atom = np.abs(F - ref["force"]).max(1) / JOULEPERHARTREE * EV_PER_HARTREE
    return {"dE_per_atom_eV": dE, "max_dF_eV_per_A": float(per_atom.max()),
            "p999_dF_eV_per_A": float(np.quantile(per_atom, 0.999)),
            "frac_atoms_within_1e-4": float(np.mean(per_atom < 1e-4))}


def relu_decisions(model, w, eles, W, ref):
    """The fused FP32 path's relu decisions (sign of every hidden pre-activation,
    from the layer outputs of an energy-only evaluation) against the FP64
    oracle's: how many differ, and how close to the kink the differing units
    lie (|z| / sum|a||w| of the exact pre-activation)."""
    s = model.system(w.x, w.Z, w.offsets)
    s.energy_force(w.x, False)
    refined = s.refined_units()
    outs = [s.layer_outputs(l) for l in range(len(model.p["HiddenLayers"]))]
    s.close()
    Z = np.asarray(w.Z)
    rel, total = [], 0
    for ni, net in enumerate(("E", "Q")):
        for e in eles:
            idx = np.nonzero(Z == e)[0]
            h = ref["G"][idx]
            for li, (Wm, b) in enumerate(W[net][e][:-1]):
                Wm = np.asarray(Wm, np.float64)
                b = np.asarray(b, np.float64).reshape(-1)
                z = h @ Wm + b
                sc = np.abs(h) @ np.abs(Wm) + np.abs(b)
                o = outs[li][ni][idx]
                on = o != 0 if li == len(outs) - 1 else o > 0
                bad = on != (z > 0)
                rel.extend((np.abs(z[bad]) / sc[bad]).tolist())
                total += z.size
                h = np.maximum(z, 0.0)
    return {"units": total, "differing_from_fp64": len(rel),
            "max_rel_distance_of_differing": max(rel, default=0.0),
            "refined_in_fp64_class_arithmetic": refined}


def smooth_accuracy(w, eles, flush, torch):
    """Fused FP32 path vs the FP64 oracle with the smooth activation of the
    reference's released networks (sigmoid_with_param, alpha = 100): with relu
    the FP64 forces themselves jump by ~0.1 eV/A under 1e-6 A perturbations
    (units at their kink), so a max-abs bound is only meaningful here."""
    from tensormol_gb300 import systems
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS, descriptor_width
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    m = BPEEModel(eles, W, params=p, precision="fp32")
    s = m.system(w.x, w.Z, w.offsets)
    o = s.energy_force(w.x, True)
    s.close()
    m.close()
    torch.set_num_threads(os.cpu_count() or 1)
    from oracle import reference as orc
    ref = orc.OpenSystemOracle(orc.Model(eles, W, p), w.x, w.Z, w.offsets).terms(w.x)
    return errors(o["Etotal"], o["force"], ref, w.natoms)


def serve_specs(seed=4, nreq=160, nmin=10, nmax=5000):
    """Serving requests: half water clusters of N log-uniform in [nmin, nmax]
    atoms (round(N/3) molecules, as the 60-atom cluster is built), half
    random-walk CHNO molecules of 8-64 atoms (as the 512-molecule batch is
    built); 45 % ask
    for 50 NVE steps (0.5 fs, Maxwell-Boltzmann velocities at 300 K), 45 % for
    a geometry optimisation to fmax 0.05 eV/A (at most 200 FIRE steps), 10 %
    for one energy+force."""
    from tensormol_gb300 import systems
    rng = np.random.default_rng(seed)
    specs = []
    for q in range(nreq):
        n = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        if rng.uniform() < 0.5:
            w = systems.water(max(4, int(round(n / 3.0))), seed=1000 + q, spacing=3.1)
            x, Z = w.x, w.Z
        else:   # a CHNO molecule as in the 512-molecule batch (8-64 atoms)
            x, Z = systems.chno_molecule(np.random.default_rng(2000 + q), int(rng.integers(8, 65)))
        u = rng.uniform()
        kind = "md" if u < 0.45 else ("opt" if u < 0.9 else "ef")
        v = systems.maxwell_boltzmann(Z, 300.0, seed=5000 + q) if kind == "md" else None
        specs.append((Z, x, kind, v))
    return specs


def serve_requests(specs):
    from tensormol_gb300 import serve
    return [serve.Request(Z, x, kind=kind, nsteps=(200 if kind == "opt" else 50), v=v, fmax=0.05)
            for (Z, x, kind, v) in specs]


def box_snapshot_accuracy(W, box, lat, x0):
    """The 12,288-atom box at its initial positions: BF16 and FP32 networks
    against each other and against the FP64 oracle (27-image tessellation),
    the same relu networks as the MD runs."""
    from oracle import reference as orc
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS
    out = {}
    for prec in ("bf16", "fp32"):
        m = BPEEModel([1, 8], W, params=dict(PARAMS), precision=prec)
        s = m.system(x0, box.Z, None, lat)
        out[prec] = s.energy_force(x0, True)
        s.close()
        m.close()
    import torch
    torch.set_num_threads(os.cpu_count() or 1)
    ref = orc.PeriodicOracle(orc.Model([1, 8], W, dict(PARAMS)), x0, box.Z, lat).terms(x0)
    n = box.natoms
    return {"fp32_vs_fp64": errors(out["fp32"]["Etotal"], out["fp32"]["force"], ref, n),
            "bf16_vs_fp64": errors(out["bf16"]["Etotal"], out["bf16"]["force"], ref, n),
            "bf16_vs_fp32": errors(out["bf16"]["Etotal"], out["bf16"]["force"],
                                   {"Etotal": out["fp32"]["Etotal"], "force": out["fp32"]["force"]}, n),
            "snapshot": "initial positions (wrapped), relu networks with output layers scaled by 0.01"}


def time_md(model_fp32, torch, oracle=True):
    """The MD workloads: (1) the 60-atom cluster, one E+F then 100 NVE steps of
    0.5 fs, FP32 networks; (2) the 12,288-atom periodic box (49.7 A), 1,000 Nose-Hoover-chain
    (length 3) steps at 300 K, dt 0.5 fs, BF16 networks, 1.0 A neighbour skin,
    with an FP32-network run of the same steps beside it. Device-resident integrators (FP64 state);
    time from CUDA events on the library stream; drift = slope of the
    conserved quantity (least squares over the run)."""
    from tensormol_gb300 import md, systems
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS, descriptor_width
    out = {}
    stream = torch.cuda.ExternalStream(int(model_fp32.ctx.stream or 0))

    def timed(fn):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r = fn()
        b.record(stream)
        b.synchronize()
        return r, a.elapsed_time(b)

    # random-init networks are no physical potential: under them a cluster
    # heats up several-fold within 100 steps and a periodic box collapses
    # within 1,000 (energy falling, temperature rising without bound). For
    # stable runs the output layers are scaled by 0.01 (the networks still run
    # in full; the systems stay near their initial state)
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    for net in W:
        for e in W[net]:
            Wl, bl = W[net][e][-1]
            W[net][e][-1] = (0.01 * Wl, bl)

    w = systems.water_cluster_60(seed=0)
    m60 = BPEEModel([1, 8], W, params=dict(PARAMS), precision="fp32")
    s = m60.system(w.x, w.Z, w.offsets)
    s.energy_force(w.x, True)
    dyn = md.DeviceMD(s, "nve", dt=0.5, T=300.0)
    dyn.set_velocities(systems.maxwell_boltzmann(w.Z, 300.0, seed=11))
    dyn.run(5)
    log, ms = timed(lambda: dyn.run(100))
    t_fs = 0.5 * np.arange(100)
    slope = np.polyfit(t_fs, log[:, 2], 1)[0]                   # J/mol per fs
    out["water60_nve_100"] = {"ms_per_step": ms / 100, "atom_steps_per_s": 60 * 100 / (ms * 1e-3),
                              "conserved_drift_J_per_mol_per_ps": slope * 1e3,
                              "kinetic_J_per_mol": float(np.mean(log[:, 1]) * 60)}
    dyn.close()
    s.close()
    m60.close()

    box = systems.water_box_12k(seed=2)
    lat = np.eye(3) * 49.7
    x0 = box.x - 49.7 * np.floor(box.x / 49.7)
    v0 = systems.maxwell_boltzmann(box.Z, 300.0, seed=12)
    res = {}
    for prec in ("bf16", "fp32"):
        m = BPEEModel([1, 8], W, params=dict(PARAMS), precision=prec)
        s = m.system(x0, box.Z, None, lat)
        dyn = md.DeviceMD(s, "nhc", dt=0.5, T=300.0, chain=3)
        dyn.set_velocities(v0)
        dyn.run(3, skin=1.0)
        log, ms = timed(lambda: dyn.run(1000, skin=1.0))
        t_ns = 0.5e-6 * np.arange(1000)
        slope = np.polyfit(t_ns, log[:, 2], 1)[0]                 # J/mol per ns
        res[prec] = {"ms_per_step": ms / 1000, "atom_steps_per_s": box.natoms * 1000 / (ms * 1e-3),
                     "conserved_drift_kJ_per_mol_per_ns": slope / 1e3,
                     "conserved_drift_J_per_mol_per_atom_per_ns": slope / box.natoms,
                     "T_mean_K": float(np.mean(log[:, 3]))}
        dyn.close()
        s.close()
        m.close()
    out["waterbox12288_nhc3_1000"] = res
    if oracle:
        res["snapshot_accuracy"] = box_snapshot_accuracy(W, box, lat, x0)
    out["note"] = ("periodic box: 1.0 A skin lists (candidates rebuilt on displacement, exact "
                   "rows filtered every step); 60-atom cluster: a full build every step; drift is the "
                   "least-squares slope of the extended-system conserved energy over the run; "
                   "both systems' networks have their output layers scaled by 0.01 so that "
                   "the random-init potential neither heats the cluster several-fold nor "
                   "collapses the box")
    return out


def time_chno512(steps, flush, torch):
    """C3: 512 CHNO molecules of 8-64 atoms (seed 3) as one batch, one fused
    E+F per step with device-resident positions (FP32 networks, 4 elements,
    3 x 512); median of the CUDA-event times, L2 flushed before each step."""
    from tensormol_gb300 import systems
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS, descriptor_width
    eles = [1, 6, 7, 8]
    b = systems.chno_batch(nmol=512, seed=3)
    model = BPEEModel(eles, systems.random_weights(eles, descriptor_width(4), seed=7),
                      params=dict(PARAMS))
    s, times, _, _, _, _ = time_fused_device(model, b, max(steps, 20), 3, flush, torch)
    s.close()
    model.close()
    ms = float(np.median(times))
    return {"molecules": 512, "atoms": int(b.natoms), "ms_per_step": ms,
            "atom_steps_per_s": b.natoms / (ms / 1000.0)}


def _serve_point(serve, model, specs, lam, max_atoms, max_mols, seed=44):
    """One arrival-rate point: Poisson arrivals at lam requests/s of the
    requests in specs, served with continuous batching."""
    rng = np.random.default_rng(seed)
    reqs = serve_requests(specs)
    t = 0.0
    for r in reqs:
        t += rng.exponential(1.0 / lam)
        r.arrival = t
    srv = serve.Server(model, max_atoms, max_mols, admission="first_fit")
    wall = srv.run_arrivals(reqs)
    st = srv.stats(wall)
    lat = np.array([(r.t_done - r.t_submit) * 1e3 for r in reqs])
    info = np.array(srv.step_info, dtype=float)          # relayout?, layout ms, step ms, atoms
    split = {"relayout_step_fraction": float(info[:, 0].mean()),
             "layout_ms_p50": float(np.percentile(info[:, 1], 50)),
             "layout_ms_p99": float(np.percentile(info[:, 1], 99)),
             "compute_ms_p50": float(np.percentile(info[:, 2], 50)),
             "compute_ms_p99": float(np.percentile(info[:, 2], 99))}
    srv.close()
    return {"arrival_rate_per_s": lam, "requests": len(reqs),
            "atom_steps_per_s": st["atom_steps_per_s"],
            "p50_step_ms": st["p50_ms"], "p99_step_ms": st["p99_ms"],
            "p99_over_p50": st["p99_ms"] / st["p50_ms"],
            "mean_batch_atoms": st["mean_batch_atoms"],
            "request_latency_p50_ms": float(np.percentile(lat, 50)),
            "request_latency_p99_ms": float(np.percentile(lat, 99)),
            "step_split": split}


def time_serving(max_atoms=32768, max_mols=512, loads=(0.25, 0.5, 1.1, 1.5, 3.0),
                 rates=(10, 30, 100, 300, 1000, 2000)):
    """Offline: every request submitted at once, batches kept full. Online:
    Poisson arrivals (a) whose offered atom-steps/s is `load` x the offline
    rate, and (b) at absolute rates of 10 to 2,000 requests/s; step latency
    p50/p99 and achieved throughput under continuous batching (first-fit
    admission with bounded overtaking). One 4-element (H, C, N, O) model serves
    every request (3 x 512 networks, FP32 path). The device capacity that a
    150 GB HBM budget allows is reported; the timed server's batch is held to
    32,768 atoms, a latency bound (the step time grows with the batch atoms)."""
    from tensormol_gb300 import serve, systems
    from tensormol_gb300.model import BPEEModel
    from tensormol_gb300.params import PARAMS, descriptor_width
    eles = [1, 6, 7, 8]
    model = BPEEModel(eles, systems.random_weights(eles, descriptor_width(4), seed=7),
                      params=dict(PARAMS))
    budget = 150 * 10**9
    cap_budget = serve.Server.capacity_for_budget(model, budget, max_mols)
    warm = serve.Server(model, max_atoms, max_mols)
    for r in serve_requests(serve_specs(seed=9, nreq=8, nmax=2000)):
        warm.submit(r)
    warm.drain()
    warm.close()
    specs = serve_specs()
    off = serve.Server(model, max_atoms, max_mols, admission="first_fit")
    reqs = serve_requests(specs)
    t0 = time.perf_counter()
    for r in reqs:
        off.submit(r, now=t0)
    off.drain()
    t_off = time.perf_counter() - t0
    offline = off.stats(t_off)
    capacity_bytes = off.bytes
    off.close()
    work = offline["atom_steps"]
    rate = offline["atom_steps_per_s"]
    n_opt = sum(1 for r in reqs if r.kind == "opt")
    n_conv = sum(1 for r in reqs if r.kind == "opt" and r.converged)
    n_drop = sum(1 for r in reqs if r.error is not None)
    sweep = []
    for load in loads:
        e = _serve_point(serve, model, specs, load * rate / (work / len(specs)), max_atoms, max_mols)
        e["offered_load_vs_offline"] = load
        e["throughput_vs_offline"] = e["atom_steps_per_s"] / rate
        sweep.append(e)
    rate_sweep = []
    for lam in rates:
        # about 4 s of arrivals at low rates, the whole request set at high ones
        n = int(max(40, min(len(specs), lam * 4.0)))
        e = _serve_point(serve, model, specs[:n], float(lam), max_atoms, max_mols, seed=45)
        e["throughput_vs_offline"] = e["atom_steps_per_s"] / rate
        rate_sweep.append(e)
    model.close()
    online = next((e for e in sweep if e["throughput_vs_offline"] >= 0.8), sweep[-1])
    return {"requests": len(specs), "atom_steps": int(work),
            "kinds": {k: sum(1 for sp in specs if sp[2] == k) for k in ("md", "opt", "ef")},
            "opt_converged": f"{n_conv}/{n_opt}",
            "dropped_nonfinite": n_drop,
            "capacity": {"max_atoms": max_atoms, "max_mols": max_mols,
                         "device_bytes": capacity_bytes,
                         "hbm_budget_bytes": budget, "max_atoms_within_budget": cap_budget,
                         "note": "admission is against min(HBM-budget capacity, the 32,768-atom "
                                 "batch bound that keeps step latency bounded)"},
            "offline": {"atom_steps_per_s": rate, "p50_step_ms": offline["p50_ms"],
                        "p99_step_ms": offline["p99_ms"], "steps": offline["steps"]},
            # headline: the first load at which continuous batching reaches 80 % of
            # the offline rate (else the highest load)
            "online": online,
            "sweep": sweep,
            "rate_sweep": rate_sweep,
            "workload": "half water clusters of N log-uniform [10, 5000] atoms, half CHNO "
                        "molecules of 8-64 atoms; 45% 50-step NVE (dt 0.5 fs), 45% FIRE optimisation to "
                        "fmax 0.05 eV/A (<= 200 steps), 10% single E+F; Poisson arrivals"}


def run_reference(args):
    """CPU implementation of the path (the oracle port) on the same workload as
    the GPU arm: one full E+F of the 24,000-atom cube per step (lists, FP64
    descriptors, networks, pair terms, autograd forces), all host threads."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    import torch
    ncores = os.cpu_count() or 1
    torch.set_num_threads(ncores)
    from oracle import reference as orc
    from tensormol_gb300 import systems
    from tensormol_gb300.params import PARAMS, descriptor_width
    sample = systems.water_cube_24k(seed=1)   # the GPU arm's system
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    model = orc.Model(eles, W, dict(PARAMS))

    def step():
        o = orc.OpenSystemOracle(model, sample.x, sample.Z, sample.offsets)
        o.terms(sample.x)
    for _ in range(args.warmup):
        step()
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        t.append(time.perf_counter() - t0)
    ms = 1000.0 * sum(t) / len(t)
    val = sample.natoms / (ms / 1000.0)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "elements": [1, 8], "hidden": [512, 512, 512],
                       "activation": "relu"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": "one full E+F per step of the 24,000-atom cube (the "
                                       "GPU arm's workload), FP64 oracle (PyTorch-CPU autograd; "
                                       "C neighbour lists); the reference's TensorFlow graph "
                                       "cannot run without TensorFlow"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle leg")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--no-md", action="store_true", help="skip the MD workloads")
    ap.add_argument("--fused-only", action="store_true",
                    help="time only the device-resident fused E+F (for profiler launch lists)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    ws, rank, local = _dist()
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from tensormol_gb300 import _lib
    _lib.load(build_if_missing=True)
    from tensormol_gb300.model import Context, default_context  # noqa: F401
    import tensormol_gb300.model as tmm
    tmm._DEFAULT_CTX = Context(local)
    w, eles, W, model = build_workload("fp32")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > L2
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    s, times, launches, clocks, E, F = time_fused_device(model, w, args.steps, args.warmup, flush, torch)
    ms, value = aggregate_ranks(sum(times) / len(times), w.natoms, ws)
    if args.fused_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                              "gpu_launches": int(launches), "note": "fused E+F only"}))
        return 0
    # stage breakdown (one profiled evaluation)
    import ctypes
    # stage breakdown: CUDA events on the library's stream between the stages,
    # averaged over `steps` evaluations
    acc = np.zeros(7)
    for _ in range(args.steps):
        st = np.zeros(7, dtype=np.float32)
        model.ctx.check(model.lib.tm_energy_force_profile(s.h, 0, st.ctypes.data))
        acc += st
    stages = dict(zip(["nlist", "descriptors", "mlp_forward", "mlp_backward", "pair_terms",
                       "adjoint_gather", "total"], [float(v) / args.steps for v in acc]))
    # the six layer-GEMM launches alone (CUDA events around each launch; the
    # relu refinement launches between them excluded), averaged over `steps`
    gemm_launch_ms = np.zeros(6)
    for _ in range(args.steps):
        lm = np.zeros(6, dtype=np.float32)
        model.ctx.check(model.lib.tm_system_profile_layers(s.h, lm.ctypes.data))
        gemm_launch_ms += lm
    gemm_launch_ms /= args.steps
    counts = s.nlist_counts()
    e2e_t, h2d, d2h = time_e2e(model, s, w, args.steps, args.warmup, torch)
    e2e_ms = sum(e2e_t) / len(e2e_t)
    s.close()
    serving = None if args.no_serve else time_serving()
    md_runs = None if args.no_md else time_md(model, torch, oracle=not args.no_cpu)
    chno = time_chno512(args.steps, flush, torch)
    # BF16 variant
    _, _, _, model16 = build_workload("bf16")
    s16, t16, _, _, E16, F16 = time_fused_device(model16, w, args.steps, args.warmup, flush, torch)
    ms16 = sum(t16) / len(t16)
    s16.close()
    model16.close()
    plain = None
    if not args.no_plain:
        pt, (Ep, Fp), pls, plg = time_plain(model, W, w, max(2, min(args.steps, 3)), 2, torch)
        plain = {"ms_per_step": sum(pt) / len(pt), "lists_ms": sum(pls) / len(pls),
                 "autograd_graph_ms": sum(plg) / len(plg)}
        plain["value"] = w.natoms / (plain["ms_per_step"] / 1000.0)
        plain["speedup_fused_vs_plain"] = plain["ms_per_step"] / ms
        # the same lists in both arms: plain's graph + autograd against the
        # fused evaluation without its own list stage
        plain["speedup_fused_vs_plain_graph_only"] = plain["autograd_graph_ms"] / (ms - stages["nlist"])
    # roofline: the six network GEMM launches per E+F
    peak, hbm, src = _peaks()
    natoms = w.natoms
    D, H = 256, 512
    alg_flop = natoms * 2 * (2 * (D * H + 2 * H * H + H) + 2 * (H + 2 * H * H + H * D))
    gemm_ms = float(gemm_launch_ms.sum())
    achieved = alg_flop / (gemm_ms / 1000.0) / 1e12
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": GEMM_DRAM_BYTES_PER_STEP,
            # the FP32 mode's own bound: three TF32 passes at half the BF16 rate
            "frac_of_split_tf32_bound": achieved * 6.0 / peak,
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of the 6 k_gemm launches "
                            "of one evaluation, one ncu capture (k_gemm summary under profiles/); "
                            "algorithmic operand + output bytes are about 1.2 GB",
            "kernel": "k_gemm: 6 launches per E+F (3 forward, 3 backward; both networks per launch)",
            "launch_ms": [round(float(v), 4) for v in gemm_launch_ms],
            "algorithmic_flop_per_step": alg_flop,
            "note": (f"peak = {src} BF16 dense burst from MEASURED_PEAKS.json; FP32 mode executes "
                     "3 TF32 MMA passes (hi*hi + hi*lo + lo*hi) at half the BF16 rate, i.e. 6x the "
                     "BF16 tensor time for the same algorithmic FLOPs")}
    # the other stages against HBM (algorithmic bytes per evaluation from the
    # built lists: N atoms, P ordered pairs <= 4.6 A, T triples <= 3.1 A)
    N, P, T, Pee = natoms, counts["pairs"], counts["triples"], counts["ee_pairs"]
    Dd = 256
    stage_bytes = {"nlist": 24 * N + 4 * N + 4 * P + 8 * T + 4 * P + 4 * T,
                   "descriptors": 16 * N + 4 * P + 8 * T + 4 * N * Dd,
                   "adjoint_gather": 16 * N + 4 * P + 8 * T + 4 * N * Dd + 12 * N,
                   "pair_terms": 16 * N + 12 * N + 4 * N}
    stage_roof = {}
    for k_, b_ in stage_bytes.items():
        gbs = b_ / (stages[k_] * 1e-3) / 1e9
        stage_roof[k_] = {"bound": "hbm", "algorithmic_bytes": int(b_), "achieved_gbs": gbs,
                          "peak_gbs": hbm, "frac": gbs / hbm}
    stage_roof["pair_terms"]["pair_evaluations_per_s"] = 2 * Pee / (stages["pair_terms"] * 1e-3)
    # the same stages against the instruction issue rate (their bound)
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    issue_peak = 4.0 * nsm * mhz * 1e6   # warp instructions per second
    issue_roof = {}
    for k_, kern in ISSUE_INST_PER_STEP.items():
        inst = float(sum(kern.values()))
        if inst <= 0:
            continue
        ach = inst / (stages[k_] * 1e-3)
        issue_roof[k_] = {"bound": "issue", "warp_instructions": kern, "achieved": ach,
                          "peak": issue_peak, "unit": "warp inst/s", "frac": ach / issue_peak}
    stage_roof["counts"] = {"atoms": N, "pairs": P, "triples": T, "ee_pairs_i_lt_j": Pee}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "elements": eles, "hidden": [512, 512, 512],
                       "activation": "relu", "precision": "fp32 (3-pass split-TF32 tcgen05 GEMMs, "
                       "FP32 descriptors/adjoint/pair terms)", "l2": "flushed (256 MiB write) "
                       "before every timed step", "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                       "pairs": None},
            "e2e": {"value": ws * natoms / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches), "clocks": clocks, "stages_ms": stages, "roofline": roof,
            "stage_rooflines": stage_roof, "issue_rooflines": issue_roof,
            "bf16": {"value": natoms / (ms16 / 1000.0), "ms_per_step": ms16},
            "plain_autograd": plain,
            "serve": serving,
            "md": md_runs,
            "chno512": chno,
            "published_reference": {"value": 274.0, "unit": UNIT, "hardware": "2015 Core i7, 1 core",
                                    "source": "24,000 atoms / ~87.5 s read off doc/images/Timings.png"}}
    if not args.no_cpu and rank == 0:
        ref, t_cpu = oracle_eval(w, eles, W)
        line["cpu_baseline"] = {"value": natoms / t_cpu, "unit": UNIT, "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": "one full E+F of the 24,000-atom cube by the FP64 oracle "
                                          "(PyTorch-CPU float64 + autograd, C neighbour lists)"}
        acc = {"fused_fp32": errors(E, F, ref, natoms), "bf16": errors(E16, F16, ref, natoms)}
        if plain is not None:
            acc["plain_autograd"] = errors(Ep, Fp, ref, natoms)
        acc["activation"] = "relu"
        acc["relu_decisions"] = relu_decisions(model, w, eles, W, ref)
        acc["fused_fp32_sigmoid_with_param"] = smooth_accuracy(w, eles, flush, torch)
        line["accuracy_vs_fp64_oracle"] = acc
    if serving is not None:
        # last key of the line: the serving headline survives a tail of the output
        on = serving["online"]
        line["serve_summary"] = {
            "offered_load_vs_offline": on["offered_load_vs_offline"],
            "throughput_vs_offline": round(on["throughput_vs_offline"], 3),
            "p50_step_ms": round(on["p50_step_ms"], 3), "p99_step_ms": round(on["p99_step_ms"], 3),
            "p99_over_p50": round(on["p99_over_p50"], 3),
            "rates_per_s": [e["arrival_rate_per_s"] for e in serving["rate_sweep"]],
            "p99_over_p50_by_rate": [round(e["p99_over_p50"], 2) for e in serving["rate_sweep"]]}
    if ws > 1:
        torch.distributed.barrier()
    if rank == 0:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
