"""Benchmark of the D3Q19 fused collide+stream hot path on one GB300.

Workload (the channel-flow-past-a-sphere case): D3Q19, 256x128x128 nodes,
FP32 populations, tau = 0.55, x-periodic, uniform body force gx = 1e-6,
half-way bounce-back walls on the y and z faces, a voxelised sphere of radius
16 centred at (64, 64, 64), equilibrium initialisation at rho = 1.  A step is
one lattice time step over all nodes; the metric is GLUPS (lattice node
updates per second, all nodes counted, as the reference counts MLUPS in
src/output.cpp:172).  The population state (1.28 GB for two sets) is larger
than L2, so every step streams from HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores instead
(the OpenMP C restatement in oracle/, run with all host threads on the same
lattice): the reference itself is a CUDA/Qt desktop application with no CPU
path, and its kernels cannot be built on the GPU machine.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ = 256, 128, 128
TAU = 0.55
GX = 1e-6
SPHERE = (64, 64, 64, 16)
# algorithmic bytes per lattice update of the fused kernel: 19 loads + 19
# stores of 4 bytes + 1 flag byte (moments are written on the last step only)
BYTES_PER_LU = 2 * 19 * 4 + 1
# DRAM bytes per launch of the fused kernel (dram__bytes_read.sum +
# dram__bytes_write.sum) from the ncu capture summarised in
# profiles/d3q19_fused_channel_256x128x128.md (captured at 128^3 and scaled
# by the node count to this lattice)
NCU_TRAFFIC_PER_LAUNCH = 522.1e6
FALLBACK_HBM_GBS = 6800.0


def channel_flags():
    fl = np.zeros((NZ, NY, NX), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = 1
    fl[0, :, :] = fl[-1, :, :] = 1
    cx, cy, cz, r = SPHERE
    z, y, x = np.ogrid[0:NZ, 0:NY, 0:NX]
    fl[(x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r] = 1
    return fl.reshape(-1)


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

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
        self.out = ""
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


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(budget_s=15.0, max_steps=None):
    """The oracle's float port of the reference loop, native mode, on the full
    lattice with all host threads, timed for a bounded number of steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lb_oracle as orc
    orc.lib()
    N = NX * NY * NZ
    flags = channel_flags()
    one = np.ones(N, np.float32)
    z = np.zeros(N, np.float32)
    w = (np.float32(12 / 36), np.float32(2 / 36), np.float32(1 / 36))
    f = orc.d3q19_equilibrium(one, z, z, z, *w)
    corr = np.zeros(19, np.float32)
    tau_inv = np.float32(1 / TAU)
    F = (np.float32(GX), np.float32(0), np.float32(0))
    steps = 0
    t0 = time.perf_counter()
    while True:
        orc.d3q19_stream_native(f, flags, corr, NX, NY, NZ)
        orc.d3q19_collide_native(f, flags, None, NX, NY, NZ, *w, tau_inv, F)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_steps and steps >= max_steps):
            break
    return {"value": N * steps / el / 1e9, "unit": "GLUPS", "cores": orc.num_threads(),
            "kind": "port", "steps": steps, "seconds": el,
            "sample": "%d time steps of the full %dx%dx%d lattice (oracle/lb_oracle.c, float, "
                      "OpenMP)" % (steps, NX, NY, NZ)}


def config_block(n_gpus):
    return {"workload": "d3q19_channel_sphere_256x128x128", "lattice": "D3Q19",
            "nodes": [NX, NY, NZ], "tau": TAU, "body_force_x": GX,
            "sphere": {"center": SPHERE[:3], "radius": SPHERE[3]},
            "boundaries": "x periodic, half-way bounce-back on y/z faces and sphere",
            "init": "equilibrium rho=1 u=0", "l2": "state (1.28 GB) larger than L2",
            "parallelism": "replicas" if n_gpus > 1 else "single"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    budget = float(os.environ.get("LB_CPU_BUDGET_S", "60"))
    cb = cpu_baseline(budget_s=budget, max_steps=args.steps)
    line = {"impl": "reference", "metric": "GLUPS", "value": cb["value"], "unit": "GLUPS",
            "n_gpus": args.gpus, "steps": cb["steps"], "warmup": 0,
            "ms_per_step": 1e3 * cb["seconds"] / cb["steps"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(1),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--tuning", type=lambda v: int(v, 0), default=0,
                    help="lb_config.tuning (0 = the library's default)")
    ap.add_argument("--size", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="other lattice extents (profiling of a smaller case only)")
    args = ap.parse_args()
    if args.size:
        global NX, NY, NZ
        NX, NY, NZ = args.size
    if args.impl == "reference":
        return run_reference(args)
    args.warmup = max(args.warmup, 3)

    ws, rank, local = dist_env()
    dist = dist_init(ws, "gloo")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    L = pkg.lib()
    N = NX * NY * NZ
    flags = channel_flags()

    # ------------------------------------------------ device-resident throughput
    lat = pkg.Lattice(19, NX, NY, NZ, tau_inv=np.float32(1 / TAU),
                      force=(np.float32(GX), 0, 0), graph_steps=64, tuning=args.tuning)
    lat.set_flags(flags)
    lat.init_equilibrium()
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
    rho, ux, uy, uz = lat.moments()
    assert np.isfinite(rho).all() and np.isfinite(ux).all()
    lat.close()

    # ------------------------------------------------ end to end through the C ABI
    # the reference's per-step host sequence (streaming_d3q19, collision_d3q19,
    # read_value_3d, 16-byte probe copy) in fused mode, driven by the library's
    # native host loop, with the initial state uploaded from pinned host memory
    # and the final moment fields read back inside the timed region
    e2e = None
    if args.e2e_steps > 0:
        e2e = measure_e2e(pkg, L, flags, args.e2e_steps, ws, dist)

    if rank != 0:
        return 0
    peak, peak_kind = measured_peak()
    kern_ms = ms / args.steps
    achieved = BYTES_PER_LU * N / (kern_ms * 1e-3) / 1e9
    line = {
        "metric": "GLUPS", "value": glups, "unit": "GLUPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config_block(ws),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_lu": BYTES_PER_LU,
                     "traffic": NCU_TRAFFIC_PER_LAUNCH},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline and ws == 1:
        cb = cpu_baseline(budget_s=float(os.environ.get("LB_CPU_BUDGET_S", "12")))
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line))
    return 0


def measure_e2e(pkg, L, flags, steps, ws, dist):
    import ctypes as C
    N = NX * NY * NZ
    pinned_ptrs = []

    def pinned(shape, dtype):
        """numpy view of page-locked host memory (cudaMallocHost via the library)"""
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        assert L.lb_malloc_host(C.byref(p), n) == 0, "lb_malloc_host failed"
        pinned_ptrs.append(p)
        buf = (C.c_uint8 * n).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    w = pkg.W3
    # inputs in pinned memory: equilibrium populations at rho = 1, u = 0 (= w_k) and walls
    f_host = pinned((19, N), np.float32)
    for k in range(19):
        f_host[k] = w[0] if k == 0 else (w[1] if k <= 6 else w[2])
    solid = pinned((N,), np.uint8)
    solid[:] = flags & 1
    sb = pinned((N,), np.uint8)
    sb[:] = 0
    out_fields = [pinned((N,), np.float32) for _ in range(4)]
    dd = pkg.DeviceData(19, NX, NY, NZ)
    assert L.lb_abi_set_mode(pkg.abi.LB_ABI_FUSED) == 0
    params = pkg.abi.lb_run_params_d3q19(w[0], w[1], w[2], np.float32(1 / TAU), 0.0, 0.0, 0.0,
                                         1.0, (C.c_int * 3)(NX // 2, NY // 2, NZ // 2))
    value = np.zeros(4, np.float32)
    # warm-up (allocates the library's second population set)
    dd.upload(f_host)
    dd.set_solid(solid, sb)
    assert L.lb_run_lbm_d3q19(dd.ptr(), C.c_void_p(dd.plot), C.byref(params), 3,
                              value.ctypes.data_as(C.c_void_p)) == 0
    L.lb_device_synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    dd.upload(f_host)
    dd.set_solid(solid, sb)
    rc = L.lb_run_lbm_d3q19(dd.ptr(), C.c_void_p(dd.plot), C.byref(params), steps,
                            value.ctypes.data_as(C.c_void_p))
    for name, dst in zip(("rho", "ux", "uy", "uz"), out_fields):
        L.lb_memcpy_d2h(dst.ctypes.data_as(C.c_void_p), C.c_void_p(getattr(dd.s, name)), 4 * N)
    L.lb_device_synchronize()
    el = time.perf_counter() - t0
    assert rc == 0, L.lb_abi_last_error()
    el = dist_max(dist, el)
    L.lb_abi_set_mode(pkg.abi.LB_ABI_STANDALONE)
    assert np.isfinite(out_fields[0]).all()
    dd.close()
    for p in pinned_ptrs:
        L.lb_free_host(p)
    h2d = 19 * 4 * N + 2 * N
    d2h = 16 * steps + 4 * 4 * N
    return {"value": ws * N * steps / el / 1e9, "unit": "GLUPS",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "steps": steps, "path": "reference entry points (fused mode) via lb_run_lbm_d3q19",
            "physics": "reference semantics on the same lattice and walls"}


if __name__ == "__main__":
    sys.exit(main())
