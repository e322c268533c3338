"""Benchmark of the nekBench hot path on GB300: axhelm GDOF/s and PCG time to 1e-8.

One "step" is one axhelm application (FP64, BK/Poisson, N=7) over the
E = 64^3 = 262144-element perturbed box (134M local nodes; 9.7 GB of operands
per step, far larger than L2, so no flush is needed between steps).  The JSON
line also carries the PCG comparison (plain FP64 Jacobi-PCG vs FP32-inner
mixed precision with FP64 refinement, with and without the learned
preconditioner) to a true FP64 relative residual of 1e-8.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU axhelm (the oracle's restatement,
bit-identical to axhelm/kernel/CPU/axhelm.c) on the host cores with all threads.
Multi-GPU (torchrun): every rank runs the same per-GPU workload on its own
elements (weak scaling, no collective on the data path); timing is the max
over ranks.
"""
from __future__ import annotations

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

METRIC = "axhelm GDOF/s & PCG time-to-1e-8 (mixed+learned vs plain FP64) at N=7, 1 GB300"
N_ORDER = 7
V100_PUBLISHED_GDOFS = 7.41742  # axhelm/readme.md:25,31 (V100, BK, N=7)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=64, help="elements per direction (E = n^3)")
    p.add_argument("--pcg-n", type=int, default=64, help="elements per direction of the PCG runs")
    p.add_argument("--no-pcg", action="store_true")
    p.add_argument("--no-learned", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    return p.parse_args()


# ------------------------------------------------------------------ distributed helpers
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend, rank=rank, world_size=ws)
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.index)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline
class CpuAxhelm:
    """The reference's CPU axhelm (axhelm/kernel/CPU/axhelm.c restated in
    oracle/cpu_axhelm.c with the order fixed at compile time and the
    reference's -O3, as the reference builds it; OpenMP over elements, all host
    threads; within a few per cent of the compiled reference on the same cores)
    on a bounded sample of the workload: n_el elements of the same N=7
    perturbed box."""

    def __init__(self, n_el=4096):
        import oracle as O
        self.O = O
        self.m = O.BoxMesh(N_ORDER, 16, 16, max(1, n_el // 256), perturb=0.1, seed=1)
        self.q = O.uniform(self.m.Nlocal, 1, 3, -1, 1)
        self.Aq = np.zeros(self.m.Nlocal)

    def apply(self):
        m = self.m
        self.O.cpu_axhelm(N_ORDER + 1, True, m.E, m.Nlocal, m.ggeo, m.D, None, self.q, self.Aq)

    def rate(self, seconds):
        self.apply()  # warm-up
        reps, t0 = 0, time.perf_counter()
        while True:
            self.apply()
            reps += 1
            el = time.perf_counter() - t0
            if el >= seconds:
                break
        per = el / reps
        return {"value": self.m.E * N_ORDER ** 3 / per / 1e9, "unit": "GDOF/s",
                "cores": self.O.omp_threads(), "kind": "port",
                "sample": f"{reps} applications of FP64 BK axhelm on {self.m.E} elements (N=7, "
                          f"{self.m.Nlocal} nodes) of the same perturbed box in {el:.1f} s, "
                          f"compile-time order, -O3, OpenMP over elements"}


def run_reference(args, rank, ws):
    if rank != 0:
        return
    import oracle as O
    O.build()
    cpu = CpuAxhelm()
    for _ in range(args.warmup):
        cpu.apply()
    per_step = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu.apply()
        per_step.append(time.perf_counter() - t0)
    med = float(np.median(per_step))
    v = cpu.m.E * N_ORDER ** 3 / med / 1e9
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "GDOF/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": med * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"axhelm FP64 BK (Poisson), N=7, bounded sample of {cpu.m.E} "
                                   f"elements of the perturbed box per step, host cores", "N": N_ORDER},
            "cpu_baseline": {"value": v, "unit": "GDOF/s", "cores": O.omp_threads(), "kind": "port",
                             "sample": f"{args.steps} timed applications on {cpu.m.E} elements "
                                       f"({cpu.m.Nlocal} nodes), median"},
            "e2e": {"value": v, "unit": "GDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def time_axhelm(nb, torch, Nq, flags, prec, E, L, g, D, lam, q, Aq, steps, warmup, stream):
    for _ in range(warmup):
        nb.axhelm(Nq, flags, prec, E, L, g, D, lam, q, Aq, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        nb.axhelm(Nq, flags, prec, E, L, g, D, lam, q, Aq, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


class HostPipeline:
    """End-to-end axhelm on host buffers: the element range is cut into chunks;
    chunk c's q is copied in (stream 1), operated on through nekb_axhelm
    (stream 2) and its Aq copied back (stream 3), so copies in both directions
    overlap the compute of other chunks.  Per-chunk events keep the reuse of
    the device buffers across steps ordered."""

    def __init__(self, nb, torch, Nq, flags, prec, E, g, D, q_dev, A_dev, hq, hA, chunks=8):
        self.nb, self.torch = nb, torch
        self.Nq, self.flags, self.prec, self.E = Nq, flags, prec, E
        self.g, self.D, self.q, self.A, self.hq, self.hA = g, D, q_dev, A_dev, hq, hA
        self.Np = Nq ** 3
        self.bounds = [(E * c // chunks, E * (c + 1) // chunks) for c in range(chunks)]
        self.s_in, self.s_cmp, self.s_out = (torch.cuda.Stream() for _ in range(3))
        self.done_cmp = [None] * chunks
        self.done_out = [None] * chunks
        self.launches = 0

    def step(self):
        torch, nb, Np = self.torch, self.nb, self.Np
        for c, (e0, e1) in enumerate(self.bounds):
            n0, n1 = e0 * Np, e1 * Np
            if self.done_cmp[c] is not None:
                self.s_in.wait_event(self.done_cmp[c])  # previous step read q[c]
            with torch.cuda.stream(self.s_in):
                self.q[n0:n1].copy_(self.hq[n0:n1], non_blocking=True)
            ev_in = torch.cuda.Event()
            ev_in.record(self.s_in)
            self.s_cmp.wait_event(ev_in)
            if self.done_out[c] is not None:
                self.s_cmp.wait_event(self.done_out[c])  # previous step copied A[c] out
            nb.axhelm(self.Nq, self.flags, self.prec, e1 - e0, (e1 - e0) * Np,
                      self.g + e0 * 7 * Np * 8, self.D, None, self.q[n0:n1], self.A[n0:n1],
                      stream=self.s_cmp.cuda_stream)
            self.launches += 1
            ev_c = torch.cuda.Event()
            ev_c.record(self.s_cmp)
            self.done_cmp[c] = ev_c
            self.s_out.wait_event(ev_c)
            with torch.cuda.stream(self.s_out):
                self.hA[n0:n1].copy_(self.A[n0:n1], non_blocking=True)
            ev_o = torch.cuda.Event()
            ev_o.record(self.s_out)
            self.done_out[c] = ev_o

    def sync(self):
        for s in (self.s_in, self.s_cmp, self.s_out):
            s.synchronize()


def load_profile_traffic():
    path = os.path.join(ROOT, "profiles", "axhelm_fp64_bk_n7.md")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.startswith("dram_bytes_per_launch_full:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return float(json.load(open(path))["bf16_tflops"])
    return 1900.0


def pcg_comparison(nb, torch, dev, n, learned, names=None):
    """Three solvers on the same problem to true FP64 relative residual 1e-8
    (`names`: only these runs)."""
    import oracle as O
    bp = nb.BP(N_ORDER, n, n, n, perturb=0.1, seed=5)
    L = bp.Nlocal
    lam = torch.empty(2 * L, dtype=torch.float64, device=dev)
    nb.fill_uniform(lam[:L], 5, 1, 0.5, 1.5)
    nb.fill_uniform(lam[L:], 5, 2, 0.5, 2.0)
    f = torch.empty(L, dtype=torch.float64, device=dev)
    nb.fill_uniform(f, 5, 3, -1.0, 1.0)
    bp.ogs.gather_scatter_many(f)
    torch.cuda.synchronize()
    out = {"workload": f"N=7, E={n}^3={bp.E} perturbed box, Dirichlet, lambda0~U[0.5,1.5], "
                       f"lambda1~U[0.5,2.0], f~U[-1,1] assembled; stop at true FP64 "
                       f"relative residual 1e-8", "E": bp.E, "unknowns_local": L}
    runs = [("fp64_jacobi", dict(solver=nb.SOLVER_FP64)),
            ("fp64_split_jacobi", dict(solver=nb.SOLVER_FP64_SPLIT)),
            ("mixed_fp32_trilinear", dict(solver=nb.SOLVER_MIXED, inner_precision=nb.FP32_TRILINEAR)),
            ("mixed_fp32", dict(solver=nb.SOLVER_MIXED, inner_precision=nb.FP32)),
            ("mixed_bf16", dict(solver=nb.SOLVER_MIXED, inner_precision=nb.BF16))]
    net = None
    if learned:
        net = learned_net(nb, torch, dev)
        if net is not None:
            runs.append(("mixed_learned", dict(solver=nb.SOLVER_MIXED, inner_precision=nb.FP32,
                                               precond=nb.PRECOND_LEARNED, net=net)))
    if names is not None:
        runs = [rk for rk in runs if rk[0] in names]
    r, x = torch.empty_like(f), torch.empty_like(f)
    for name, kw in runs:
        # a 20-iteration warm-up on the same buffers instantiates the solver's
        # CUDA graphs and lower-precision copies; then one timed solve
        r.copy_(f)
        x.zero_()
        bp.pcg(lam, r, x, 1e-8, 20, **kw)
        r.copy_(f)
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = bp.pcg(lam, r, x, 1e-8, 20000, **kw)
        torch.cuda.synchronize()
        st["wall_s"] = time.perf_counter() - t0
        out[name] = {k: st[k] for k in ("iterations", "outer_iterations", "status",
                                         "true_rel_res", "elapsed_s", "wall_s")}
    base = out["fp64_jacobi"]["elapsed_s"]
    for name, _ in runs[1:]:
        out[name]["speedup_vs_fp64"] = base / out[name]["elapsed_s"]
    bp.free()
    del bp
    return out


# FP64 instructions per node of the even-odd BK operator at N=7 (transforms 2 x 3,
# pair sums 5 x 6, geometric factors 9, final sum 2)
EO_FP64_OPS_PER_NODE = 47

NET_FLOP_PER_ELEMENT = 2 * 27 * 512 * (16 + 16 * 16 + 16)  # 3 layers of 3x3x3 convs, C=16, Nq=8


def time_net(nb, torch, dev, E, fp32_subset=8):
    """Learned-preconditioner inference (one application over E elements):
    tensor-core kernel on all E elements, FP32-core kernel on E/8 (scaled)."""
    net = nb.Net(8, 16, 3, seed=1)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    x = torch.randn(E * 512, device=dev, generator=g)
    out = torch.empty_like(x)
    res = {}
    for name, mode, Et in (("tensor_core", nb.NET_TENSOR, E), ("tensor_core_tcgen05", nb.NET_TENSOR_TC5, E),
                           ("tensor_core_mma_sync", nb.NET_TENSOR_SYNC, E),
                           ("fp32_cores", nb.NET_FP32, E // fp32_subset)):
        net.inference = mode
        for _ in range(3):
            net.forward(x, out, Et)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            net.forward(x, out, Et)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5 * (E / Et)
        res[name] = {"ms_per_application": ms, "elements": E, "timed_elements": Et,
                     "tflops": E * NET_FLOP_PER_ELEMENT / (ms * 1e-3) / 1e12}
    return res


def nekbone_bp5(nb, torch, dev):
    """The reference's nekBone BP5 case (nekBone/readme.md:24-53): periodic
    unperturbed [-1,1]^3 box 16x16x32, N=7, Poisson (BK), COPY preconditioner,
    zero-mean rhs/solution.  Correctness check to tol 1e-6 (published: maxError
    1.02763e-07 in 78 iterations) and 5000 fixed FP64 iterations timed
    (published V100: 2.09109 GDOF/s/iter)."""
    import math
    bp = nb.BP(N_ORDER, 16, 16, 32, periodic=True, dirichlet=False, perturb=0.0, box=(-1.0, 1.0))
    L = bp.Nlocal
    X, Y, Z = (bp.device_array(c, L, torch.float64) for c in "xyz")
    JW = bp.device_array("ggeo", 7 * L, torch.float64).view(bp.E, 7, bp.Np)[:, 0, :].reshape(-1)
    exact = torch.cos(math.pi * X) * torch.cos(math.pi * Y) * torch.cos(math.pi * Z)
    f = (3 * math.pi ** 2) * JW * exact
    bp.ogs.gather_scatter_many(f)
    r, x = f.clone(), torch.zeros_like(f)
    kw = dict(precond=nb.PRECOND_COPY, bk=True, zero_mean=True)
    st = bp.pcg(None, r, x, 1e-6, 1000, **kw)
    err = float((x - exact).abs().max())
    r.copy_(f)
    x.zero_()
    bp.pcg(None, r, x, 0.0, 50, fixed_iterations=True, **kw)  # graphs, warm clocks
    r.copy_(f)
    x.zero_()
    st2 = bp.pcg(None, r, x, 0.0, 5000, fixed_iterations=True, **kw)
    out = {"workload": "nekBone BP5: N=7, E=16x16x32=8192 periodic [-1,1]^3, BK, COPY, FP64",
           "check_iterations": st["iterations"], "check_max_error": err,
           "published_check": {"iterations": 78, "max_error": 1.02763e-07},
           "fixed_iterations": st2["iterations"], "elapsed_s": st2["elapsed_s"],
           "gdofs_per_iter": st2["iterations"] * bp.E * N_ORDER ** 3 / st2["elapsed_s"] / 1e9,
           "published_v100_gdofs_per_iter": 2.09109}
    bp.free()
    return out


def cpu_pcg_reference(pcg, n_gpu, seconds=2.0, n=16, gpu_same=None):
    """The reference's CPU path for the PCG (the oracle's OpenMP restatement:
    the CPU baseline axhelm, gather-scatter and vector kernels as OpenMP loops
    over all host threads) on the same problem class as the GPU solves (N=7
    perturbed box, lambda0~U[0.5,1.5], lambda1~U[0.5,2.0], Dirichlet, Jacobi)
    at E=n^3: fixed FP64 iterations (about `seconds` of CPU work) for the
    per-iteration time, and one whole solve to 1e-8, measured, beside the GPU
    solvers' measured times on the same problem (`gpu_same`).  The time to
    1e-8 at the GPU's size is only projected: the per-iteration time scaled by
    the element ratio, times the GPU FP64 solve's iterations."""
    import oracle as O
    m = O.BoxMesh(N_ORDER, n, n, n, perturb=0.1, seed=5)
    L = m.Nlocal
    lam = np.concatenate([O.uniform(L, 5, 1, 0.5, 1.5), O.uniform(L, 5, 2, 0.5, 2.0)])
    bp = O.BP(m, lam)
    f = O.gs_many_add(bp.Ng, bp.offs, bp.gids, O.uniform(L, 5, 3, -1.0, 1.0))
    f[m.maskIds] = 0.0
    r, x = f.copy(), np.zeros(L)
    t0 = time.perf_counter()
    _, setup = bp.pcg_omp(r, x, 0.0, 5, fixed=True)
    per = max((time.perf_counter() - t0 - setup) / 5, 1e-6)
    k = int(min(200, max(10, seconds / per)))
    r, x = f.copy(), np.zeros(L)
    t0 = time.perf_counter()
    it, setup = bp.pcg_omp(r, x, 0.0, k, fixed=True)
    el = time.perf_counter() - t0 - setup
    per = el / it
    out = {"kind": "port", "cores": O.omp_threads(),
           "sample": f"{it} fixed FP64 Jacobi-PCG iterations on E={n}^3={m.E} elements ({L} local "
                     f"nodes) of the same problem class, OpenMP over all host threads",
           "seconds_per_iteration": per,
           "gdofs_per_iter": m.E * N_ORDER ** 3 / per / 1e9,
           "setup_s": setup}
    r, x = f.copy(), np.zeros(L)
    t0 = time.perf_counter()
    it_full, setup_full = bp.pcg_omp(r, x, 1e-8, 20000)
    full = time.perf_counter() - t0 - setup_full
    out["measured_to_1e-8"] = {"E": m.E, "iterations": it_full, "seconds": full,
                               "note": "whole CPU solve on all host threads, measured"}
    if gpu_same:
        out["measured_to_1e-8"]["gpu_same_problem"] = {
            k2: {"iterations": v["iterations"], "seconds": v["elapsed_s"],
                 "cpu_over_gpu": full / v["elapsed_s"]}
            for k2, v in gpu_same.items() if isinstance(v, dict) and "elapsed_s" in v}
    fp64 = (pcg or {}).get("fp64_jacobi")
    if fp64:
        proj = per * (n_gpu ** 3 / m.E) * fp64["iterations"]
        out["projected_time_to_1e-8_s"] = proj
        out["projection"] = (f"per-iteration time x (E={n_gpu}^3 / E={n}^3) x the GPU FP64 "
                             f"solve's {fp64['iterations']} iterations")
        out["gpu_speedup"] = {k2: proj / v["elapsed_s"] for k2, v in pcg.items()
                              if isinstance(v, dict) and "elapsed_s" in v}
    return out


def dot_adv(nb, torch, dev, E, peak_bw, fp64_peak):
    """The dot and adv benchmark kernels at N=7.  dot: weightedInnerProduct2_v0
    partials over E elements (3 arrays of E*512 doubles, larger than L2) timed
    alone (CUDA events) and as the reference driver times a call (kernel, copy
    of the partials to the host, host sum; dot/main.cpp:27-48).  adv:
    advCubatureHex3D_v0 with cubN=11 on 8192 elements, FP64-pipe bound."""
    from nekbench_gb300 import adv as advmod
    out = {}
    L = E * 512
    arrs = [torch.empty(L, dtype=torch.float64, device=dev) for _ in range(3)]
    for s, t in enumerate(arrs):
        nb.fill_uniform(t, 1, 10 + s, 0.0, 1.0)
    nblk = nb.dot_num_blocks(L)
    tmp = torch.empty(nblk, dtype=torch.float64, device=dev)
    host = torch.empty(nblk, dtype=torch.float64, pin_memory=True)
    for _ in range(3):
        nb.dot_partials(0, L, *arrs, tmp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        nb.dot_partials(0, L, *arrs, tmp)
    e1.record()
    torch.cuda.synchronize()
    kern = e0.elapsed_time(e1) * 1e-3 / 20
    t0 = time.perf_counter()
    for _ in range(10):
        nb.dot_partials(0, L, *arrs, tmp)
        host.copy_(tmp)
        float(np.cumsum(host.numpy())[-1])
    call = (time.perf_counter() - t0) / 10
    out["dot"] = {"workload": f"weightedInnerProduct2_v0, N=7, E={E} ({L} nodes), blockSize 256",
                  "kernel_ms": kern * 1e3, "kernel_gbs": 24 * L / kern / 1e9,
                  "hbm_frac": 24 * L / kern / 1e9 / peak_bw,
                  "reference_call_ms": call * 1e3, "reference_call_gbs": 24 * L / call / 1e9,
                  "gdofs": E * 343 / kern / 1e9}
    del arrs, tmp, host
    Nq, cq, Ea = 8, 12, 8192
    g = torch.Generator(device=dev).manual_seed(5)
    r = lambda n: torch.rand(n, dtype=torch.float64, device=dev, generator=g)  # noqa: E731
    vgeo, cub, D, I, U = r(12 * Ea * 512), r(12 * Ea * cq ** 3), r(cq * cq), r(Nq * cq), r(3 * Ea * 512)
    NU = torch.empty_like(U)
    for _ in range(3):
        nb.adv_cubature(Nq, cq, Ea, vgeo, cub, D, I, Ea * 512, U, NU)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(5):
        nb.adv_cubature(Nq, cq, Ea, vgeo, cub, D, I, Ea * 512, U, NU)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / 5
    NUs = torch.empty_like(U)
    for _ in range(3):
        nb.adv_cubature(Nq, cq, Ea, vgeo, cub, D, I, Ea * 512, U, NUs, nb.FP64_SPLIT)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(5):
        nb.adv_cubature(Nq, cq, Ea, vgeo, cub, D, I, Ea * 512, U, NUs, nb.FP64_SPLIT)
    e1.record()
    torch.cuda.synchronize()
    ts = e0.elapsed_time(e1) * 1e-3 / 5
    split_diff = float((NUs - NU).abs().max() / NU.abs().max())
    tflops = advmod.flops(Nq, cq) * Ea / t / 1e12
    out["adv"] = {"workload": "advCubatureHex3D_v0, N=7, cubN=11, E=8192, FP64",
                  "ms": t * 1e3, "gdofs": Ea * 343 / t / 1e9, "fp64_tflops": tflops,
                  "fp64_peak_tflops_measured": fp64_peak, "fp64_frac": tflops / fp64_peak,
                  "gbs": advmod.bytes_moved(Nq, cq) * Ea / t / 1e9,
                  "flops_per_element": advmod.flops(Nq, cq),
                  "bytes_per_element": advmod.bytes_moved(Nq, cq),
                  "fp64_split": {"ms": ts * 1e3, "gdofs": Ea * 343 / ts / 1e9,
                                 "speedup_vs_fp64": t / ts,
                                 "max_rel_diff_to_fp64": split_diff}}
    del vgeo, cub, U, NU, NUs
    torch.cuda.empty_cache()
    return out


def learned_net(nb, torch, dev):
    path = os.path.join(ROOT, "nekbench_gb300", "weights", "precond_n7_c16.bin")
    if not os.path.exists(path) or not hasattr(nb, "Net"):
        return None
    return nb.Net.load(path)


def run_gpu(args, rank, ws, local):
    import torch

    import nekbench_gb300 as nb
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    n = args.n
    Nq = N_ORDER + 1
    bp = nb.BP(N_ORDER, n, n, n, perturb=0.1, seed=1, stream=stream.cuda_stream)
    E, L = bp.E, bp.Nlocal
    g, D = bp.ptr("ggeo"), bp.ptr("D")
    q = torch.empty(L, dtype=torch.float64, device=dev)
    nb.fill_uniform(q, 1, 3, -1.0, 1.0, stream=stream.cuda_stream)
    Aq = torch.empty_like(q)
    torch.cuda.synchronize()

    # ---- device-resident timing (inputs already in HBM)
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_axhelm(nb, torch, Nq, nb.AX_BK, nb.FP64, E, L, g, D, None, q, Aq, args.steps,
                         args.warmup, stream)
    torch.cuda.synchronize()
    barrier(ws)
    ms = max_over_ranks(ms, ws)
    gdofs = ws * E * N_ORDER ** 3 / (ms * 1e-3) / 1e9

    # ---- end to end through the C ABI with host buffers (q in, Aq out)
    hq = torch.empty(L, dtype=torch.float64, pin_memory=True)
    hq.copy_(q.cpu())
    hA = torch.empty(L, dtype=torch.float64, pin_memory=True)
    e2e_steps = max(8, min(args.steps, 32))
    pipe = HostPipeline(nb, torch, Nq, nb.AX_BK, nb.FP64, E, g, D, q, Aq, hq, hA)
    for _ in range(2):
        pipe.step()
    pipe.sync()
    torch.cuda.synchronize()
    barrier(ws)
    # the pipeline runs continuously; a step ends when its last chunk's Aq has
    # reached host memory (an event on the copy-out stream)
    t0 = time.perf_counter()
    ends = []
    for _ in range(e2e_steps):
        pipe.step()
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(pipe.s_out)
        ends.append(ev)
    pipe.sync()
    e2e_wall_s = (time.perf_counter() - t0) / e2e_steps
    intervals = [ends[i].elapsed_time(ends[i + 1]) * 1e-3 for i in range(len(ends) - 1)]
    # value: the MEAN steady-state step (first to last copy-out event over the
    # steps between them); the median is reported beside it
    e2e_s = float(np.mean(intervals))
    e2e_median_s = float(np.median(intervals))
    # the chunked host-fed result equals one device-resident application, bit for bit
    nb.axhelm(Nq, nb.AX_BK, nb.FP64, E, L, g, D, None, q, Aq, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e2e_exact = bool(torch.equal(hA, Aq.cpu()))
    e2e_s = max_over_ranks(e2e_s, ws)
    e2e_median_s = max_over_ranks(e2e_median_s, ws)
    e2e_gdofs = ws * E * N_ORDER ** 3 / e2e_s / 1e9

    # ---- roofline of the dominant kernel (FP64 BK axhelm)
    alg_bytes = 9 * 8 * L  # (2 + 7) words per node: q, Aq, 7 ggeo (axhelm/main.cpp:162)
    alg_flops = (12 * Nq + 15) * L  # axhelm/main.cpp:165-166
    peak_bw, peak_src = measured_peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    fp64_peak = nb.peak_fma(True)
    traffic = load_profile_traffic()
    # the binding roof is GB300's FP64 pipe (the HBM time is an eighth of the
    # FP64 time): achieved = the reference's flop count ((12 Nq + 15) per node,
    # axhelm/main.cpp:165-166) per launch over the launch time, against the
    # FP64 FMA rate measured on this GPU by the library's own peak kernel (no
    # FP64 figure is in the measured-peaks file).  The even-odd kernel issues
    # 47 FP64 instructions per node where the direct sums need 59, so its rate
    # by the reference's count can pass the FP64 peak.
    alg_tflops = alg_flops / (ms * 1e-3) / 1e12
    roofline = {"bound": "fp64", "achieved": alg_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": alg_tflops / fp64_peak, "traffic": traffic,
                "peak_source": "measured FP64 FMA rate of this GPU (nekb_peak_fma, FMA = 2 flop)",
                "fp64_instructions_per_node": EO_FP64_OPS_PER_NODE,
                # FP64 instructions issued per second over the pipe's instruction rate
                "fp64_pipe_frac": EO_FP64_OPS_PER_NODE * L / (ms * 1e-3) / (fp64_peak * 1e12 / 2),
                "hbm": {"achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                        "frac": achieved / peak_bw, "peak_source": peak_src}}

    # ---- other precisions of the operator (same mesh, same step definition)
    variants = {}
    Df = bp.ptr("Df")
    q32 = q.float()
    A32 = torch.empty_like(q32)
    lam64 = torch.empty(2 * L, dtype=torch.float64, device=dev)
    nb.fill_uniform(lam64[:L], 1, 1, 0.5, 1.5, stream=stream.cuda_stream)
    nb.fill_uniform(lam64[L:], 1, 2, 0.5, 2.0, stream=stream.cuda_stream)
    lam32 = lam64.float()
    lambf = lam32.to(torch.bfloat16)
    gf, gb, tri = bp.ptr("ggeo_f"), bp.ptr("ggeo_bf"), bp.ptr("trilinear")
    torch.cuda.synchronize()
    for name, flags, prec, gg, DD, la, qq, aa, bpn in [
            ("fp64_helmholtz", 0, nb.FP64, g, D, lam64, q, Aq, 88),
            ("fp64_split_bk", nb.AX_BK, nb.FP64_SPLIT, g, D, None, q, Aq, 72),
            ("fp64_split_helmholtz", 0, nb.FP64_SPLIT, g, D, lam64, q, Aq, 88),
            ("fp32_bk", nb.AX_BK, nb.FP32, gf, Df, None, q32, A32, 36),
            ("fp32_helmholtz", 0, nb.FP32, gf, Df, lam32, q32, A32, 44),
            ("bf16_helmholtz", 0, nb.BF16, gb, Df, lambf, q32, A32, 26),
            ("fp32_trilinear_bk", nb.AX_BK, nb.FP32_TRILINEAR, tri, Df, None, q32, A32, 8),
            ("fp32_trilinear_helmholtz", 0, nb.FP32_TRILINEAR, tri, Df, lam32, q32, A32, 16)]:
        t = time_axhelm(nb, torch, Nq, flags, prec, E, L, gg, DD, la, qq, aa, 10, 3, stream)
        variants[name] = {"ms": t, "gdofs": E * N_ORDER ** 3 / (t * 1e-3) / 1e9,
                          "alg_gbs": bpn * L / (t * 1e-3) / 1e9,
                          "hbm_frac": bpn * L / (t * 1e-3) / 1e9 / peak_bw}
    del q32, A32, lam32, lambf, lam64
    bp.free()
    del bp
    torch.cuda.empty_cache()

    pcg = pcg_small = None
    if not args.no_pcg:
        pcg = pcg_comparison(nb, torch, dev, args.pcg_n, not args.no_learned)
        pcg_small = pcg_comparison(nb, torch, dev, 16, False,
                                   names=("fp64_jacobi", "fp64_split_jacobi", "mixed_fp32"))
    bp5 = None if args.no_pcg else nekbone_bp5(nb, torch, dev)
    net_cost = time_net(nb, torch, dev, E)
    for v in net_cost.values():
        v["bf16_peak_tflops"] = measured_bf16()
        v["frac_of_bf16_peak"] = v["tflops"] / v["bf16_peak_tflops"]

    benchmarks = dot_adv(nb, torch, dev, E, peak_bw, fp64_peak)

    cpu = CpuAxhelm().rate(args.cpu_seconds) if (rank == 0 and ws == 1) else None
    if pcg is not None and rank == 0 and ws == 1:
        try:
            pcg["cpu_reference_fp64_jacobi"] = cpu_pcg_reference(pcg, args.pcg_n,
                                                                 gpu_same=pcg_small)
        except Exception as exc:  # a failed baseline must not cost the bench line
            pcg["cpu_reference_fp64_jacobi"] = {"error": f"{type(exc).__name__}: {exc}"}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": gdofs, "unit": "GDOF/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"axhelm FP64 BK (Poisson) N=7 on E={n}^3={E} perturbed trilinear "
                               f"box elements per GPU ({L} local nodes, {alg_bytes / 1e9:.1f} GB "
                               f"per step)", "N": N_ORDER, "E_per_gpu": E,
                   "l2": "inputs larger than L2 (no flush needed)",
                   "parallelism": f"replicas x{ws} (element-parallel, no collective)"},
        "e2e": {"value": e2e_gdofs, "unit": "GDOF/s", "h2d_bytes_per_step": 8 * L,
                "d2h_bytes_per_step": 8 * L,
                "note": "nekb_axhelm through the C ABI on 8 element chunks per step; each "
                        "chunk's q copied from pinned host memory and its Aq copied back on "
                        "separate streams, overlapping the other chunks' compute; geometry "
                        "resident; value from the mean steady-state step (intervals between "
                        "the steps' last copy-out events, averaged over all steps)",
                "median_step_gdofs": ws * E * N_ORDER ** 3 / e2e_median_s / 1e9,
                "wall_clock_gdofs": ws * E * N_ORDER ** 3 / e2e_wall_s / 1e9,
                "steps": e2e_steps, "bit_identical_to_device_result": e2e_exact},
        "gpu_launches": args.steps,
        "roofline": roofline,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "variants": variants,
        "pcg": pcg,
        "nekbone_bp5": bp5,
        "learned_preconditioner_inference": net_cost,
        "dot_and_adv_benchmarks": benchmarks,
        "reference_published": {"v100_axhelm_gdofs": V100_PUBLISHED_GDOFS},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, ws, local = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
    else:
        run_gpu(args, rank, ws, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
