"""Benchmark of the lattice Boltzmann hot path on one GB300.

Default workload ("channel", the headline): D3Q19 channel flow past a sphere,
256x128x128 nodes, FP32 populations, tau = 0.55, x-periodic, uniform body
force gx = 1e-6, half-way bounce-back walls on the y and z faces, a voxelised
sphere of radius 16 centred at (64, 64, 64), equilibrium initialisation at
rho = 1.  A step is one lattice time step over all nodes; the metric is GLUPS
(lattice node updates per second, all nodes counted, as the reference counts
MLUPS in src/output.cpp:172).  The population state (1.28 GB for two sets)
is larger than L2, so every step streams from HBM.

Other workloads (--workload) measure the remaining configurations with the
same JSON line: "cavity" (D2Q9 lid-driven cavity 256x256, tau 0.6, lid 0.1).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

--impl reference times the reference algorithm on the host cores instead
(the OpenMP C restatement in oracle/, run with all host threads on the same
lattice): the reference itself is a CUDA/Qt desktop application with no CPU
path, and its kernels cannot be built on the GPU machine.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


class Workload:
    """One benchmark configuration: lattice, extents, physics, and the
    algorithmic bytes per lattice update of the kernel it times."""

    def __init__(self, name, lattice, size, tau, steps, bytes_per_lu, force=(0, 0, 0),
                 wall_u=(0, 0, 0), traffic=None, describe=None, G=0.0,
                 storage=0, rho_ref=0.0, dtype="f32"):
        self.name, self.lattice, self.size, self.tau = name, lattice, tuple(size), tau
        self.steps, self.bytes_per_lu, self.force, self.wall_u = steps, bytes_per_lu, force, wall_u
        self.traffic, self.describe = traffic, describe or {}
        self.G, self.storage, self.rho_ref, self.dtype = G, storage, rho_ref, dtype

    def initial_rho(self):
        """None (uniform rho = 1) or the seeded spinodal density field
        rho = 0.693 (1 + eps), eps ~ U[-0.01, 0.01] (numpy PCG64, seed 2024)."""
        if not self.name.startswith("spinodal"):
            return None
        rng = np.random.default_rng(2024)
        return (0.693 * (1 + rng.uniform(-0.01, 0.01, self.N))).astype(np.float32)

    @property
    def N(self):
        return int(np.prod(self.size))

    def flags(self):
        nx, ny, nz = self.size
        if self.name.startswith("channel"):
            fl = np.zeros((nz, ny, nx), np.uint8)
            fl[:, 0, :] = fl[:, -1, :] = 1
            fl[0, :, :] = fl[-1, :, :] = 1
            cx, cy, cz, r = 64, 64, 64, 16
            z, y, x = np.ogrid[0:nz, 0:ny, 0:nx]
            fl[(x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r] = 1
            return fl.reshape(-1)
        if self.name == "cavity":
            fl = np.zeros((ny, nx), np.uint8)
            fl[:, 0] = fl[:, -1] = fl[-1, :] = 1
            fl[0, :] = 3  # row 0 is the top wall (physical +y is row-1), moving with the lid
            return fl.reshape(-1)
        if self.name.startswith("spinodal"):
            return np.zeros(self.N, np.uint8)  # fully periodic
        raise ValueError(self.name)

    def config(self, n_gpus):
        c = {"workload": "%s_%s" % (self.name, "x".join(str(s) for s in self.size if s > 1)),
             "lattice": "D3Q19" if self.lattice == 19 else "D2Q9", "nodes": list(self.size),
             "tau": self.tau, "parallelism": "replicas" if n_gpus > 1 else "single"}
        c.update(self.describe)
        return c


WORKLOADS = {
    # 19x4 loads + 19x4 stores + 1 flag byte (moments only on the last step)
    "channel": Workload(
        "channel", 19, (256, 128, 128), 0.55, 20000, 2 * 19 * 4 + 1, force=(1e-6, 0, 0),
        # DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
        # of d3q19_fused_kernel, captured on this lattice with the caches left
        # as the previous step left them (ncu --cache-control none, mean of
        # two launches)
        traffic=578.4e6,
        describe={"body_force_x": 1e-6, "sphere": {"center": [64, 64, 64], "radius": 16},
                  "boundaries": "x periodic, half-way bounce-back on y/z faces and sphere",
                  "init": "equilibrium rho=1 u=0",
                  "l2": "state (1.28 GB) larger than L2"}),
    "cavity": Workload(
        "cavity", 9, (256, 256, 1), 0.6, 10000, 2 * 9 * 4 + 1, wall_u=(0.1, 0, 0),
        describe={"lid_velocity": 0.1, "boundaries": "half-way bounce-back box, moving top wall",
                  "init": "equilibrium rho=1 u=0",
                  "l2": "state (4.7 MB) fits L2: temporal blocks of 5 steps per launch "
                        "(32x14 tiles with their halo in shared memory), graph-replayed "
                        "programmatic dependent launches"}),
}
# the channel with 16-bit deviation storage (f_k - w_k * 1.0 kept in binary16 /
# bfloat16, FP32 arithmetic): 19x2 loads + 19x2 stores + 1 flag byte per update
for _st, _nm in [(1, "f16"), (2, "bf16")]:
    WORKLOADS["channel_" + _nm] = Workload(
        "channel_" + _nm, 19, (256, 128, 128), 0.55, 20000, 2 * 19 * 2 + 1,
        force=(1e-6, 0, 0), storage=_st, rho_ref=1.0, dtype=_nm,
        describe={"body_force_x": 1e-6, "sphere": {"center": [64, 64, 64], "radius": 16},
                  "boundaries": "x periodic, half-way bounce-back on y/z faces and sphere",
                  "init": "equilibrium rho=1 u=0", "storage": _nm,
                  "storage_offset": "f_k - w_k*1.0",
                  "l2": "state (0.64 GB) larger than L2"})
# D3Q19 Shan-Chen spinodal decomposition, 256^3 periodic, tau = 1, G = -5,
# psi = 1 - exp(-rho); algorithmic bytes/LU: populations read + written once,
# 152 (FP32) / 76 (16-bit deviation storage).  The default step (single pass,
# populations staged in shared memory) keeps psi on chip and reads no flags on
# this wall-free lattice; the two-pass step (--tuning 0x100) also writes and
# reads psi and reads the flags twice.
for _st, _nm, _b in [(0, "f32", 152), (1, "f16", 76), (2, "bf16", 76)]:
    WORKLOADS["spinodal" + ("" if _st == 0 else "_" + _nm)] = Workload(
        "spinodal" + ("" if _st == 0 else "_" + _nm), 19, (256, 256, 256), 1.0, 10000, _b,
        G=-5.0, storage=_st, rho_ref=0.693, dtype=_nm,
        describe={"G": -5.0, "psi": "1-exp(-rho)", "storage": _nm,
                  "storage_offset": "f_k - w_k*0.693" if _st else None,
                  "init": "rho=0.693(1+eps), eps~U[-0.01,0.01], seed 2024, u=0",
                  "boundaries": "periodic", "l2": "state larger than L2"})


ENSEMBLE = {"domains": 512, "steps": 5000, "seed": 4,
            # periodic domains read no flags: 9x4 loads + 9x4 stores, plus psi written
            # and read by the two-pass step (the single-pass tiles keep psi on chip)
            "bytes_per_lu": {"tiles": 2 * 9 * 4, "two_pass": 2 * 9 * 4 + 8}}


def run_ensemble(args, dist, ws, rank, local):
    """The batched ensemble: 512 independent periodic D2Q9 Shan-Chen droplet
    domains (sides uniform over the multiples of 32 in [64, 512], G ~
    U[-5.5, -4.5], one droplet of radius U[0.1, 0.3]*side, tau = 1),
    autotuned launch shape, CUDA-graph-replayed persistent launches.  Each
    droplet starts at the coexistence densities of its own G (liquid 1.49 ..
    2.31, vapour 0.25 .. 0.10): the fixed pair 2.0 / 0.1 is far from
    coexistence for G near -4.5 and those droplets blow up within 300 steps.
    GLUPS counts the nodes of all domains."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    select_device(pkg, ws, local)
    nx, ny, G, rho = pkg.droplet_ensemble(args.domains or ENSEMBLE["domains"],
                                          seed=ENSEMBLE["seed"])
    steps = args.steps if args.steps else ENSEMBLE["steps"]
    ens = pkg.Ensemble(nx, ny, G)
    if args.launch_shape:
        ens.set_launch(*args.launch_shape)
        shape = list(args.launch_shape)
    else:
        shape = ens.autotune(trial_steps=3)
    ens.init_equilibrium(rho)
    ens.step(max(args.warmup, 3))
    if dist:
        dist.barrier()
    n0 = ens.launches()
    with ClockSampler(local) as clk:
        ms = ens.time_steps(steps)
    launches = ens.launches() - n0
    mom = ens.moments()
    assert np.isfinite(mom[0]).all()
    ens.close()
    ms = dist_max(dist, ms)
    if rank != 0:
        return 0
    NT = int(np.sum(nx.astype(np.int64) * ny))
    peak, peak_kind = measured_peak()
    bytes_per_lu = ENSEMBLE["bytes_per_lu"]["tiles" if shape[0] == 0 else "two_pass"]
    achieved = bytes_per_lu * NT / (ms / steps * 1e-3) / 1e9
    line = {"metric": "GLUPS", "value": ws * NT * steps / (ms * 1e-3) / 1e9, "unit": "GLUPS",
            "n_gpus": ws, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "ensemble_512_d2q9_shan_chen_droplets", "domains": len(nx),
                       "droplet": "radius U[0.1,0.3]*side at the coexistence densities of "
                                  "its G (tanh interface, width 2)",
                       "deviation": "droplet densities: the Shan-Chen coexistence pair of each "
                                    "domain's G (liquid 1.49..2.31, vapour 0.25..0.10) instead "
                                    "of a fixed 2.0 / 0.1, whose droplets blow up within 300 "
                                    "steps for G near -4.5 (the oracle too)",
                       "total_nodes": NT, "sides": "multiples of 32 in [64, 512], seed %d"
                       % ENSEMBLE["seed"], "G": "U[-5.5,-4.5]", "tau": 1.0,
                       "psi": "1-exp(-rho)",
                       "launch_shape": ({("single_pass_tiles" if shape[1] <= 5 else
                                          "single_pass_warp_strips" if shape[1] <= 9 else
                                          "single_pass_warp_strips_smem_row_ring"):
                                         "32x%d" % {1: 8, 2: 8, 3: 16, 4: 16, 5: 32, 6: 32,
                                                    7: 32, 8: 64, 9: 16, 10: 32, 11: 64,
                                                    12: 16}[shape[1]],
                                         "shape": shape[1], "blocks_per_sm": shape[2]}
                                        if shape[0] == 0 else
                                        {"threads_x": shape[0], "rows_per_item": shape[1],
                                         "blocks_per_sm": shape[2]}),
                       "parallelism": "replicas" if ws > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "bytes_per_lu": bytes_per_lu, "traffic": None},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


CLOSURE = {"U0": 0.05, "Re": 1600.0, "fine": 512, "factors": (2, 4, 8, 16), "plain_only": (2,),
           "t_end": 10.0, "fine_every": 256, "train_snapshots": 16, "train_steps": 3000,
           "batch": 16384, "lr": 2e-3, "avg_radius": 1, "max_ke_error": 0.01}


def run_closure(args, dist, ws, rank, local):
    """Learned closure for the under-resolved Taylor-Green vortex (Re 1600,
    U0 = 0.05) over coarse grids 256^3 .. 32^3.  One fine 512^3 FP32 BGK run
    is Favre box-filtered onto every coarse grid (the reference kinetic
    energy every 256 fine steps; training data at 16 snapshots); a closure
    network is trained on the GPU for each of 128^3, 64^3 and 32^3 and its
    output scale calibrated on the first half of the trajectory; plain BGK
    runs on every grid.  value = the closure's speed-up over the plain FP32
    path at equal kinetic-energy error: the wall time of the cheapest plain
    run whose KE-decay error is at most the closure run's, divided by the
    closure run's -- the best such pair among the closure runs with a KE
    error of at most 1 % (every pair is listed)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    select_device(pkg, ws, local)
    C = pkg.closure
    cfg = dict(CLOSURE)
    nf = args.size[0] if args.size else cfg["fine"]
    factors = tuple(f for f in cfg["factors"] if nf // f >= 8)
    with ClockSampler(local) as clk:
        sw = C.resolution_sweep(nf, factors, U0=cfg["U0"], Re=cfg["Re"], t_end=cfg["t_end"],
                                fine_every=cfg["fine_every"],
                                train_snapshots=cfg["train_snapshots"],
                                train_steps=cfg["train_steps"], batch=cfg["batch"], lr=cfg["lr"],
                                avg_radius=cfg["avg_radius"], plain_only=cfg["plain_only"])
    if rank != 0:
        return 0
    pairs = C.speedup_at_equal_error(sw["runs"])
    best = C.headline(pairs, max_error=cfg["max_ke_error"])
    closure_runs = [r for r in sw["runs"] if r["kind"] == "closure"]
    c128 = next((r for r in closure_runs if r["n"] == nf // 4), None)
    best_run = next((r for r in closure_runs if best and r["n"] == best["closure_n"]), None)
    kfig = closure_kernel_figures(sw["runs"], best_run["n"] if best_run else nf // 4)
    line = {"metric": "closure_speedup_at_equal_ke_error",
            "value": best["speedup"] if best else None, "unit": "x", "n_gpus": ws,
            "steps": best_run["steps"] if best_run else None, "warmup": 0,
            "ms_per_step": 1e3 * best_run["seconds"] / best_run["steps"] if best_run else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+bf16", "data": "synthetic",
            "config": {"workload": "closure_tgv_re1600_fine%d" % nf, "U0": cfg["U0"],
                       "Re": cfg["Re"], "fine_nodes": nf ** 3,
                       "coarse_grids": [nf // f for f in factors],
                       "filter": "Favre box, factor = fine / coarse",
                       "convective_times": cfg["t_end"],
                       "mlp": "19-64-64-1 ReLU, BF16 tensor cores (tcgen05), FP32 accumulate",
                       "training": {"snapshots": cfg["train_snapshots"],
                                    "adam_steps": cfg["train_steps"], "batch": cfg["batch"],
                                    "target": "nu_t of the filtered sub-grid stress, both "
                                              "contractions averaged over 3^3 coarse cells",
                                    "inputs": "inputs never excited in the training data "
                                              "get zero first-layer weights",
                                    "output_scale": "fitted on the first half of the "
                                                    "trajectory from %s"
                                                    % list(C.CALIBRATION_SCALES)},
                       "ke_error": "RMS over the samples of E/E0 against the filtered fine run",
                       "headline": "best speed-up among closure runs with KE error <= %g"
                                   % cfg["max_ke_error"]},
            "roofline": kfig[0], "mlp_time": kfig[1],
            "closure": {"equal_error_pairs": pairs, "best": best, "runs": sw["runs"],
                        "fine_seconds": sw["fine_seconds"], "fine_steps": sw["fine_steps"],
                        "closure_128_vs_fine_run": (sw["fine_seconds"] / c128["seconds"])
                                                   if c128 else None},
            "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


FALLBACK_BF16_TFLOPS_SUSTAINED = 1700.0


def measured_tensor_peak():
    """Dense BF16 tensor throughput for a kernel timed inside a long run (the
    sustained figure)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops_sustained"]), "measured"
    except Exception:
        return FALLBACK_BF16_TFLOPS_SUSTAINED, "fallback"


# learned closure: 2 (19*64 + 64*64 + 64) FLOP of the network per cell
CLOSURE_FLOP_PER_CELL = 2 * (19 * 64 + 64 * 64 + 64)


def closure_kernel_figures(runs, n):
    """The closure step kernel on the n^3 grid: its time per step beside the
    plain step's on the same grid (the difference is the network's share),
    and its roofline: 153 algorithmic bytes per cell against HBM and the
    network's FLOP against the sustained BF16 tensor peak."""
    cl = next((r for r in runs if r["kind"] == "closure" and r["n"] == n), None)
    pl = next((r for r in runs if r["kind"] == "plain" and r["n"] == n), None)
    if cl is None:
        return None, None
    cells = n ** 3
    t_cl = cl["seconds"] / cl["steps"]
    hbm, hbm_kind = measured_peak()
    tc, tc_kind = measured_tensor_peak()
    gbs = 153.0 * cells / t_cl / 1e9
    tflops = CLOSURE_FLOP_PER_CELL * cells / t_cl / 1e12
    roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
            "peak_source": hbm_kind, "bytes_per_lu": 153, "traffic": None,
            "kernel": "d3q19_closure_tc_kernel", "grid": n,
            "tensor": {"achieved": tflops, "peak": tc, "unit": "TFLOP/s", "frac": tflops / tc,
                       "peak_source": tc_kind + " (sustained)",
                       "flop_per_cell": CLOSURE_FLOP_PER_CELL}}
    mlp = {"grid": n, "closure_ms_per_step": 1e3 * t_cl,
           "plain_ms_per_step": 1e3 * pl["seconds"] / pl["steps"] if pl else None}
    if pl:
        mlp["network_ms_per_step"] = mlp["closure_ms_per_step"] - mlp["plain_ms_per_step"]
        mlp["network_share_of_step"] = mlp["network_ms_per_step"] / mlp["closure_ms_per_step"]
    return roof, mlp


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            p = [s.strip() for s in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank, int(os.environ.get("LOCAL_RANK", "0"))


def dist_init(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend)
    return dist


def select_device(pkg, ws, local):
    """One process per GPU: this rank's library calls go to GPU `local`."""
    if ws > 1:
        rc = pkg.lib().lb_set_device(local)
        assert rc == 0, "lb_set_device(%d) failed" % local


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(wl, budget_s=15.0, max_steps=None, warmup=0):
    """The oracle's float port of the reference loop (swap streaming + collision,
    native boundary mode) on the workload's full lattice with all host threads,
    timed for a bounded number of steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lb_oracle as orc
    orc.lib()
    N = wl.N
    nx, ny, nz = wl.size
    flags = wl.flags()
    one = np.ones(N, np.float32)
    z = np.zeros(N, np.float32)
    tau_inv = np.float32(1 / wl.tau)
    F = tuple(np.float32(v) for v in wl.force)
    rho0 = wl.initial_rho()
    if rho0 is not None:
        one = rho0
    psi = np.zeros(N, np.float32) if wl.G != 0 else None
    if wl.lattice == 19:
        w = (np.float32(12 / 36), np.float32(2 / 36), np.float32(1 / 36))
        f = orc.d3q19_equilibrium(one, z, z, z, *w)
    else:
        w = (np.float32(16 / 36), np.float32(4 / 36), np.float32(1 / 36))
        f = orc.d2q9_equilibrium(one, z, z, *w)
    corr = orc.wall_correction(wl.lattice, wl.wall_u)
    steps = 0
    t0 = time.perf_counter()
    while True:
        if warmup and steps == warmup:
            steps, warmup, t0 = 0, 0, time.perf_counter()  # untimed warm-up done
        if wl.lattice == 19:
            orc.d3q19_stream_native(f, flags, corr, nx, ny, nz)
            orc.d3q19_collide_native(f, flags, None, nx, ny, nz, *w, tau_inv, F, G=wl.G, psi=psi)
        else:
            orc.d2q9_stream_native(f, flags, corr, nx, ny)
            orc.d2q9_collide_native(f, flags, None, nx, ny, *w, tau_inv, F[:2])
        steps += 1
        el = time.perf_counter() - t0
        if not warmup and (el >= budget_s or (max_steps and steps >= max_steps)):
            break
    return {"value": N * steps / el / 1e9, "unit": "GLUPS", "cores": orc.num_threads(),
            "kind": "port", "steps": steps, "seconds": el,
            "sample": "%d time steps of the full %s lattice (oracle/lb_oracle.c, float, OpenMP)"
                      % (steps, "x".join(str(s) for s in wl.size if s > 1))}


def run_reference(args, wl):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    budget = float(os.environ.get("LB_CPU_BUDGET_S", "60"))
    cb = cpu_baseline(wl, budget_s=budget, max_steps=args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": "GLUPS", "value": cb["value"], "unit": "GLUPS",
            "n_gpus": args.gpus, "steps": cb["steps"], "warmup": args.warmup,
            "ms_per_step": 1e3 * cb["seconds"] / cb["steps"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": wl.config(1),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="channel",
                    choices=sorted(WORKLOADS) + ["ensemble", "closure"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--parallelism", default="auto", choices=["auto", "replicas", "zslab"],
                    help="channel with N > 1 ranks: one z-slab of one lattice per rank (auto, "
                         "zslab) or independent replicas")
    ap.add_argument("--slabs", type=int, default=0,
                    help="channel, one rank: cut the lattice into this many z-slabs stepped "
                         "as one group on the GPU")
    ap.add_argument("--no-f16", action="store_true",
                    help="channel: skip the 16-bit storage figure beside the FP32 one")
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--tuning", type=lambda v: int(v, 0), default=0,
                    help="lb_config.tuning (0 = the library's default)")
    ap.add_argument("--graph-steps", type=int, default=64)
    ap.add_argument("--domains", type=int, default=None,
                    help="ensemble: number of domains (profiling of a smaller case only)")
    ap.add_argument("--launch-shape", type=int, nargs=3, default=None,
                    metavar=("THREADS_X", "ROWS", "BLOCKS_PER_SM"),
                    help="ensemble: this launch shape instead of the autotuner's pick")
    ap.add_argument("--size", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="other lattice extents (profiling of a smaller case only)")
    args = ap.parse_args()
    if args.workload in ("ensemble", "closure"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the CPU leg is measured on "
                              "the channel workload only"}))
            return 0
        ws, rank, local = dist_env()
        run = run_ensemble if args.workload == "ensemble" else run_closure
        return run(args, dist_init(ws, "gloo"), ws, rank, local)
    wl = WORKLOADS[args.workload]
    if args.size:
        wl.size = tuple(args.size)
        wl.traffic = None
    if args.steps is None:
        args.steps = wl.steps
    if args.impl == "reference":
        return run_reference(args, wl)
    args.warmup = max(args.warmup, 3)

    ws, rank, local = dist_env()
    if wl.name.startswith("channel") and (args.parallelism == "zslab" or args.slabs > 1 or
                                          (args.parallelism == "auto" and ws > 1)):
        return run_zslab(args, wl, ws, rank, local)
    dist = dist_init(ws, "gloo")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    select_device(pkg, ws, local)
    L = pkg.lib()
    N = wl.N
    nx, ny, nz = wl.size
    flags = wl.flags()

    # ------------------------------------------------ device-resident throughput
    lat = pkg.Lattice(wl.lattice, nx, ny, nz, tau_inv=np.float32(1 / wl.tau),
                      force=tuple(np.float32(v) for v in wl.force), wall_u=wl.wall_u,
                      graph_steps=args.graph_steps, tuning=args.tuning, G=wl.G,
                      storage=wl.storage, rho_ref=wl.rho_ref)
    lat.set_flags(flags)
    lat.init_equilibrium(wl.initial_rho())
    lat.step(args.warmup)
    lat.synchronize()
    if dist:
        dist.barrier()
    n0 = lat.launches()
    with ClockSampler(local) as clk:
        ms = lat.time_steps(args.steps)
    launches = lat.launches() - n0
    ms = dist_max(dist, ms)
    glups = ws * N * args.steps / (ms * 1e-3) / 1e9
    mom = lat.moments()
    assert np.isfinite(mom[0]).all() and np.isfinite(mom[1]).all()
    lat.close()

    # ------------------------- the same lattice with 16-bit deviation storage
    f16 = None
    if wl.name == "channel" and not args.no_f16:
        f16 = measure_f16(pkg, wl, flags, args, ws, dist, glups)

    # ------------------------------------------------ end to end through the C ABI
    e2e = e2e_dropin = None
    if args.e2e_steps > 0 and wl.name == "channel":
        e2e = measure_e2e(pkg, L, wl, flags, args.e2e_steps, ws, dist)
        e2e_dropin = measure_e2e_dropin(pkg, L, wl, flags, max(200, args.e2e_steps // 4))

    if rank != 0:
        return 0
    peak, peak_kind = measured_peak()
    kern_ms = ms / args.steps
    achieved = wl.bytes_per_lu * N / (kern_ms * 1e-3) / 1e9
    line = {
        "metric": "GLUPS", "value": glups, "unit": "GLUPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
        "data": "synthetic", "config": wl.config(ws),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_lu": wl.bytes_per_lu, "traffic": wl.traffic},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    # the same rate counted over fluid nodes only (wall nodes move no data)
    n_fluid = int(np.count_nonzero((flags & 1) == 0))
    line["fluid_nodes"] = n_fluid
    line["fluid_glups"] = glups * n_fluid / N
    if f16:
        line["fp16_storage"] = f16
    if e2e:
        line["e2e"] = e2e
    if e2e_dropin:
        line["e2e_dropin"] = e2e_dropin
    if not args.no_cpu_baseline and ws == 1:
        cb = cpu_baseline(wl, budget_s=float(os.environ.get("LB_CPU_BUDGET_S", "12")))
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line))
    return 0


def channel_flags(nx, ny, nz, spheres):
    """y/z walls and one sphere of radius 16 at (64, 64, 64 + 128 s) for each
    s < spheres (the channel of every 128 planes)."""
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = 1
    fl[0, :, :] = fl[-1, :, :] = 1
    z, y, x = np.ogrid[0:nz, 0:ny, 0:nx]
    for sp in range(spheres):
        fl[(x - 64) ** 2 + (y - 64) ** 2 + (z - 64 - 128 * sp) ** 2 <= 16 * 16] = 1
    return fl.reshape(-1)


def run_zslab(args, wl, ws, rank, local):
    """The channel cut into z-slabs (include/lbgb300.h part 7).  One rank:
    the 256x128x128 lattice in --slabs slabs stepped as one group on the GPU
    (faces moved by device copies, the interior planes of each slab on a
    second stream).  N ranks (one per GPU): a 256x128x(128 N) channel with a
    sphere in every 128 planes, rank r holding planes 128 r .. 128 r + 127
    and exchanging its two faces with its z-neighbours over NCCL every step
    (weak scaling: 128 planes per GPU)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    S = pkg.slab
    nx, ny, nz1 = wl.size
    nzg = nz1 * ws
    flags = channel_flags(nx, ny, nzg, max(1, nzg // 128))
    P = nx * ny
    kw = dict(tau_inv=np.float32(1 / wl.tau), force=tuple(np.float32(v) for v in wl.force),
              storage=wl.storage, rho_ref=wl.rho_ref)
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        select_device(pkg, ws, local)
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        bounds = [(rank * nz1, nz1)]
    else:
        bounds = S.slab_bounds(nzg, max(1, args.slabs))
    slabs = []
    for z0, nz in bounds:
        sl = S.Slab(nx, ny, nzg, z0, nz, **kw)
        sl.set_flags(np.ascontiguousarray(flags.reshape(nzg, P)[sl.planes()].reshape(-1)))
        sl.init_equilibrium(None)
        slabs.append(sl)
    n0 = sum(sl.launches() for sl in slabs)
    if ws > 1:
        import torch
        sr = S.SlabRank(slabs[0], S.SlabExchange(dist, rank, ws))
        sr.step(max(args.warmup, 3))
        slabs[0].synchronize()
        dist.barrier()
        n0 = slabs[0].launches()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            t0.record(sr.stream)
            sr.step(args.steps)
            t1.record(sr.stream)
            t1.synchronize()
        ms = t0.elapsed_time(t1)
        ms = dist_max(dist, ms)
    else:
        grp = S.SlabGroup(slabs)
        grp.step(max(args.warmup, 3))
        grp.synchronize()
        n0 = grp.launches()
        with ClockSampler(local) as clk:
            ms = grp.time_steps(args.steps)
    launches = sum(sl.launches() for sl in slabs) - n0
    mom = slabs[0].moments()
    assert np.isfinite(slabs[0].own(mom[0])).all()
    face_bytes = slabs[0].face_bytes
    for sl in slabs:
        sl.close()
    if rank != 0:
        return 0
    N = nx * ny * nzg
    peak, peak_kind = measured_peak()
    achieved = wl.bytes_per_lu * N / ws / (ms / args.steps * 1e-3) / 1e9
    cfg = wl.config(ws)
    cfg.update({"workload": "%s_zslab_%dx%dx%d" % (wl.name, nx, ny, nzg),
                "nodes": [nx, ny, nzg], "parallelism": "zslab",
                "slabs": len(bounds) if ws == 1 else ws,
                "slab_planes": [nz for _, nz in bounds] if ws == 1 else nz1,
                "exchange": "device copies between the slabs of one GPU" if ws == 1 else
                            "NCCL send/recv of the two faces with the z-neighbours",
                "exchange_bytes_per_slab_step": 2 * face_bytes,
                "spheres": "radius 16 at (64, 64, 64 + 128 s)"})
    line = {"metric": "GLUPS", "value": N * args.steps / (ms * 1e-3) / 1e9, "unit": "GLUPS",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic", "config": cfg,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "bytes_per_lu": wl.bytes_per_lu, "traffic": None},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def measure_f16(pkg, wl, flags, args, ws, dist, glups_f32):
    """The headline lattice again with populations stored as binary16
    deviations f_k - w_k (FP32 arithmetic), same physics, steps and timing:
    the "FP16-store vs FP32" figure of the metric.  Its roofline counts
    19 x 2 loads + 19 x 2 stores + 1 flag byte = 77 B per update."""
    nx, ny, nz = wl.size
    lat = pkg.Lattice(wl.lattice, nx, ny, nz, tau_inv=np.float32(1 / wl.tau),
                      force=tuple(np.float32(v) for v in wl.force), wall_u=wl.wall_u,
                      graph_steps=args.graph_steps, tuning=args.tuning, storage=1, rho_ref=1.0)
    lat.set_flags(flags)
    lat.init_equilibrium(None)
    lat.step(args.warmup)
    lat.synchronize()
    if dist:
        dist.barrier()
    n0 = lat.launches()
    ms = lat.time_steps(args.steps)
    launches = lat.launches() - n0
    assert np.isfinite(lat.moments()[0]).all()
    lat.close()
    ms = dist_max(dist, ms)
    glups = ws * wl.N * args.steps / (ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    achieved = 77 * wl.N / (ms / args.steps * 1e-3) / 1e9
    return {"value": glups, "unit": "GLUPS", "ms_per_step": ms / args.steps,
            "vs_fp32": glups / glups_f32, "storage": "binary16 f_k - w_k*1.0, FP32 arithmetic",
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "bytes_per_lu": 77}}


def solid_bound_d3q19(solid, nx, ny, nz):
    """The reference's solid_bound rule (src/simulation_d3q19.cu:167-204): a
    solid node whose 18 neighbours are all solid, for x in 1 .. nx-2 only,
    y and z periodic."""
    s = solid.reshape(nz, ny, nx).astype(bool)
    sb = s.copy()
    for cz in (-1, 0, 1):
        for cy in (-1, 0, 1):
            for cx in (-1, 0, 1):
                if abs(cx) + abs(cy) + abs(cz) in (1, 2):
                    sb &= np.roll(s, (-cz, -cy, -cx), (0, 1, 2))
    sb[:, :, 0] = sb[:, :, -1] = False
    return sb.reshape(-1).astype(np.uint8)


def measure_e2e_dropin(pkg, L, wl, flags, steps, fused=True):
    """The reference's own host sequence through the drop-in entry points, on
    the headline lattice in the reference's semantics: lb_run_lbm_d3q19 runs,
    per step, streaming_d3q19, collision_d3q19 into the plot buffer (Zou-He
    velocity inlet u = 0 at x = 0 and pressure outlet rho = 1 at x = nx-1,
    full-way bounce-back walls and sphere), read_value_3d at the cursor and a
    16-byte device-to-host copy (queued in stream order), as
    SimulationD3Q19::runLBM does
    (src/simulation_d3q19.cu:350-430).  tau = 0.8: at 0.55 the reference's
    own Zou-He faces grow a disturbance on this geometry (the oracle, the
    reference compiled for the host, does the same).  Timed with host
    buffers: the populations uploaded from pinned memory, the run, and the
    moment fields read back."""
    import ctypes as C
    nx, ny, nz = wl.size
    N = wl.N
    solid = (flags & 1).astype(np.uint8)
    sb = solid_bound_d3q19(solid, nx, ny, nz)
    dd = pkg.DeviceData(19, nx, ny, nz, plot=True)
    dd.set_solid(solid, sb)
    hp = C.c_void_p()
    assert L.lb_malloc_host(C.byref(hp), 4 * 19 * N) == 0
    f_host = np.frombuffer((C.c_float * (19 * N)).from_address(hp.value), np.float32).reshape(19, N)
    for k in range(19):
        f_host[k] = pkg.W3[0] if k == 0 else (pkg.W3[1] if k <= 6 else pkg.W3[2])
    mp = C.c_void_p()
    assert L.lb_malloc_host(C.byref(mp), 4 * 4 * N) == 0
    m_host = np.frombuffer((C.c_float * (4 * N)).from_address(mp.value), np.float32).reshape(4, N)
    vp = C.c_void_p()
    assert L.lb_malloc_host(C.byref(vp), 16) == 0
    prm = pkg.abi.lb_run_params_d3q19()
    prm.w0, prm.w1, prm.w7 = (float(w) for w in pkg.W3)
    prm.tau_inv, prm.rho_out = np.float32(1 / 0.8), 1.0
    prm.cursor[0], prm.cursor[1], prm.cursor[2] = nx // 2, ny // 3, nz // 2
    L.lb_abi_set_mode(pkg.abi.LB_ABI_FUSED if fused else pkg.abi.LB_ABI_STANDALONE)

    def run(n):
        for k, name in enumerate(dd.s.POP):
            assert L.lb_memcpy_h2d(C.c_void_p(getattr(dd.s, name)),
                                   C.c_void_p(hp.value + 4 * k * N), 4 * N) == 0
        rc = L.lb_run_lbm_d3q19(dd.ptr(), C.c_void_p(dd.plot), C.byref(prm), n, vp)
        assert rc == 0, L.lb_abi_last_error()
        for i, name in enumerate(("rho", "ux", "uy", "uz")):
            assert L.lb_memcpy_d2h(C.c_void_p(mp.value + 4 * i * N),
                                   C.c_void_p(getattr(dd.s, name)), 4 * N) == 0

    run(3)
    launches_before = None
    t0 = time.perf_counter()
    run(steps)
    el = time.perf_counter() - t0
    assert np.isfinite(m_host[0]).all()
    L.lb_abi_release_d3q19(dd.ptr())
    L.lb_abi_set_mode(pkg.abi.LB_ABI_STANDALONE)
    dd.close()
    for p_ in (hp, mp, vp):
        L.lb_free_host(p_)
    del launches_before
    return {"value": N * steps / el / 1e9, "unit": "GLUPS", "steps": steps,
            "h2d_bytes_per_step": 4 * 19 * N / steps, "d2h_bytes_per_step": (16 * steps + 16 * N) / steps,
            "mode": "fused" if fused else "standalone",
            "path": "lb_run_lbm_d3q19: per step streaming_d3q19 + collision_d3q19 (plot buffer) "
                    "+ read_value_3d + a 16-byte copy to pinned host memory in stream order "
                    "(one host wait after the last step); the "
                    "reference's semantics (Zou-He x faces, full-way bounce-back), tau 0.8",
            "bytes_per_lu": 185 if fused else 330}


def measure_e2e(pkg, L, wl, flags, steps, ws, dist):
    """End to end through the library's C ABI with host buffers: the initial
    populations are uploaded from pinned host memory (lb_set_populations),
    then lb_run_probe runs the reference's per-step host pattern (a step,
    then the read_value-style cursor value delivered to host memory -- here
    written by every step's kernel into mapped page-locked memory, so the
    steps replay from CUDA graphs without a host round trip between them),
    and the final rho and u fields are read back into pinned host memory --
    all inside the timed region.  Same workload and physics as the
    device-resident number."""
    import ctypes as C
    N = wl.N
    nx, ny, nz = wl.size
    pinned_ptrs = []

    def pinned(shape, dtype):
        """numpy view of page-locked host memory (cudaMallocHost via the library)"""
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        assert L.lb_malloc_host(C.byref(p), n) == 0, "lb_malloc_host failed"
        pinned_ptrs.append(p)
        buf = (C.c_uint8 * n).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    w = pkg.W3 if wl.lattice == 19 else pkg.W2
    Q = wl.lattice
    f_host = pinned((Q, N), np.float32)
    for k in range(Q):  # equilibrium at rho = 1, u = 0 is w_k
        f_host[k] = w[0] if k == 0 else (w[1] if k <= (6 if Q == 19 else 4) else w[2])
    out_fields = [pinned((N,), np.float32) for _ in range(4)]
    value = pinned((4,), np.float32)
    lat = pkg.Lattice(wl.lattice, nx, ny, nz, tau_inv=np.float32(1 / wl.tau),
                      force=tuple(np.float32(v) for v in wl.force), wall_u=wl.wall_u)
    lat.set_flags(flags)
    cx, cy, cz = nx // 2, ny // 3, nz // 2
    vp = value.ctypes.data_as(C.c_void_p)
    # warm-up
    assert L.lb_set_populations(lat.h, f_host.ctypes.data_as(C.c_void_p)) == 0
    assert L.lb_run_probe(lat.h, 3, cx, cy, cz, vp) == 0
    lat.synchronize()
    if dist:
        dist.barrier()
    n0 = lat.launches()
    t0 = time.perf_counter()
    rc1 = L.lb_set_populations(lat.h, f_host.ctypes.data_as(C.c_void_p))
    rc2 = L.lb_run_probe(lat.h, steps, cx, cy, cz, vp)
    rc3 = L.lb_get_moments(lat.h, *[a.ctypes.data_as(C.c_void_p) for a in out_fields])
    el = time.perf_counter() - t0
    assert rc1 == rc2 == rc3 == 0, L.lb_error(lat.h)
    launches = lat.launches() - n0
    el = dist_max(dist, el)
    assert np.isfinite(out_fields[0]).all() and np.isfinite(value).all()
    lat.close()
    for p in pinned_ptrs:
        L.lb_free_host(p)
    h2d = 4 * Q * N
    d2h = 16 * steps + 4 * 4 * N
    return {"value": ws * N * steps / el / 1e9, "unit": "GLUPS",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "steps": steps, "gpu_launches": launches,
            "path": "lb_set_populations + lb_run_probe (every step's kernel writes the cursor's "
                    "16 bytes into mapped pinned host memory; graph-replayed steps) + "
                    "lb_get_moments, pinned host buffers, wall clock"}


if __name__ == "__main__":
    sys.exit(main())
