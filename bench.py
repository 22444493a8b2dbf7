#!/usr/bin/env python
"""Benchmark of the boundary-integral hot path: GMRES solves/s of the Stokes system
(SOLVEI, stokesbubb.f:294-415) on the 64-drop workload, FP32-refined vs plain FP64.

Workload: 64 seeded drops, radii U[0.5, 1], r(theta) = r (1 + 0.05 cos 2 theta) at equal
arclength, centres in [-20, 20]^2 with gaps > 0.2, 512 nodes each (N = 32,768 nodes,
65,536 unknowns). One step = one Stokes GMRES solve to ||b - A x|| / ||b|| <= 1e-10,
geometry and right-hand side resident in HBM. The plain FP64 solve starts from x0 = b (the
reference's settings); the FP32-refined solve is iterative refinement from x = 0 (its
first residual is b itself and costs no apply).
The right-hand side is SETVELF's surface-tension term -dz/(2 |dz|) (stokesbubb.f:55-57),
computed from the geometry EXTRACTDAT produced on the GPU.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs N independent replicas (one per GPU; the path has no data exchange), and
value is the aggregate over ranks. `--impl reference` times the reference algorithm
(the per-level CADAPDR FMM and SLATEC GMRES, restated in C) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GMRES solves/s and FMM Mpts/s, FP32-refined vs FP64 on GPU at 1e-10 rel err"
WORKLOAD = "many_drops_64x512"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    # profilers that do not descend into CUDA graphs see every kernel with "off"
    ap.add_argument("--graphs", default="on", choices=["on", "off"])
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload():
    from electricbubbles_gb300 import configs
    return configs.many_drops()


# ---------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # wait (up to 5 s) for the first sample, so that sampling covers the timed region
            t_end = time.time() + 5.0
            while time.time() < t_end and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------
# reference arm / CPU baseline: the reference algorithm restated in C, on host cores
# ---------------------------------------------------------------------------------
def cpu_reference_solves(cfg, nsolves, nthreads):
    """Times `nsolves` Stokes solves of the reference algorithm (CADAPDR per-level FMM,
    LEVMAX = 7, TOL = 1e-13, and SLATEC GMRES) with nthreads OpenMP threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    ex = O.extractdat(cfg.nd, cfg.rku())
    g = O.Geometry.from_extract(cfg.nd, ex)
    rhs = surface_tension_rhs(ex["dz"], ex["dsda"])
    times, infos = [], []
    for _ in range(nsolves):
        t0 = time.perf_counter()
        x, info = O.solvei(g, rhs, mode=1, nthreads=nthreads)  # 1: CADAPDR restatement
        times.append(time.perf_counter() - t0)
        infos.append(info)
    return times, infos, x


def surface_tension_rhs(dz, dsda):
    import numpy as np
    zn = -0.5 * dz / dsda
    return np.ascontiguousarray(zn).view(np.float64).copy()


def run_reference(args, rank, world):
    if rank != 0:
        return
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = workload()
    nthreads = O.max_threads()
    if args.warmup > 0:
        cpu_reference_solves(cfg, 1, nthreads)
    times, infos, _ = cpu_reference_solves(cfg, args.steps, nthreads)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded drops)",
        "config": {"workload": WORKLOAD, "nodes": cfg.nbk, "unknowns": 2 * cfg.nbk,
                   "solver": "CADAPDR per-level FMM (LEVMAX=7, TOL=1e-13) + SLATEC GMRES, C restatement",
                   "gmres_tol": 1e-10, "threads": nthreads},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
                         "sample": "%d full Stokes solves of the 64x512 workload" % args.steps},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gmres_iters": [i["iters"] for i in infos],
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------
def run_gpu(args, rank, world, local):
    import numpy as np
    import torch
    from electricbubbles_gb300 import configs
    from electricbubbles_gb300.api import Context

    dist = world > 1
    if dist:
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    cfg = workload()
    graphs = 1 if args.graphs == "on" else -1
    ctx = Context(device=local, graphs=graphs)
    ctx.set_stream(stream.cuda_stream)
    geo = ctx.extractdat(cfg.nd, cfg.rku())          # EXTRACTDAT on the GPU (set-up)
    rhs_h = surface_tension_rhs(geo["dz"], geo["dsda"])
    n = rhs_h.shape[0]
    rhs = torch.from_numpy(rhs_h).to(dev)
    x = torch.empty_like(rhs)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(max(args.steps, 1))]

    def timed(mode, steps, warmup, c=None):
        c = c or ctx
        for _ in range(warmup):
            c.solvei(rhs, mode, out=x)
        torch.cuda.synchronize()
        if dist:
            td.barrier()
        infos = []
        t0 = time.perf_counter()
        l0 = c.launch_count()
        for s in range(steps):
            flush.zero_()
            ev[s][0].record(stream)
            _, info = c.solvei(rhs, mode, out=x)
            ev[s][1].record(stream)
            infos.append(info)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        timed.launches = c.launch_count() - l0
        dev_ms = sum(a.elapsed_time(b) for a, b in ev[:steps])
        if dist:
            t = torch.tensor([dev_ms], device=dev)
            td.all_reduce(t, op=td.ReduceOp.MAX)
            dev_ms = float(t.item())
        return dev_ms, wall, infos

    # plain FP64 and refined solves (the refined one is the headline); the clocks are
    # sampled over all the timed solves
    clocks = ClockSampler(local)
    clocks.start()
    ms64, _, inf64 = timed("fp64", args.steps, args.warmup)
    x64 = x.clone()
    # the same FP64 solves with the double-float FP64-class operators (df64 = 1)
    ctx_df = Context(device=local, df64=1, graphs=graphs)
    ctx_df.set_stream(stream.cuda_stream)
    ctx_df.extractdat(cfg.nd, cfg.rku())
    ms64_df, _, _ = timed("fp64", args.steps, args.warmup, ctx_df)
    ms32, wall32, inf32 = timed("fp32_refined", args.steps, args.warmup)
    clk = clocks.stop()
    launches = timed.launches
    rel_diff = float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64))

    # Laplace solves (SOLVE_LAPL, laplace.f:335-425) on the same geometry, GETBCs' -2 Re z
    rl = torch.from_numpy(np.ascontiguousarray(-2.0 * np.ascontiguousarray(geo["z"]).real)).to(dev)
    xl = torch.empty_like(rl)
    lap = {}
    for mode in ("fp64", "fp32_refined"):
        for _ in range(args.warmup):
            ctx.solve_lapl(rl, mode, out=xl)
        torch.cuda.synchronize()
        ea0, ea1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea0.record(stream)
        for _ in range(args.steps):
            _, linfo = ctx.solve_lapl(rl, mode, out=xl)
        ea1.record(stream)
        torch.cuda.synchronize()
        lap[mode + "_solves_per_s"] = world * args.steps / (ea0.elapsed_time(ea1) * 1e-3)
        lap[mode + "_info"] = linfo
    # the same solves right-preconditioned by the deflation of each drop's constant
    # density (eb_opts.lap_deflate): same system and stopping test, fewer iterations
    ctx_ld = Context(device=local, graphs=graphs, lap_deflate=1)
    ctx_ld.set_stream(stream.cuda_stream)
    ctx_ld.extractdat(cfg.nd, cfg.rku())
    for mode in ("fp64", "fp32_refined"):
        for _ in range(args.warmup):
            ctx_ld.solve_lapl(rl, mode, out=xl)
        torch.cuda.synchronize()
        ea0, ea1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea0.record(stream)
        for _ in range(args.steps):
            _, linfo = ctx_ld.solve_lapl(rl, mode, out=xl)
        ea1.record(stream)
        torch.cuda.synchronize()
        lap["deflated_" + mode + "_solves_per_s"] = world * args.steps / (ea0.elapsed_time(ea1) * 1e-3)
        lap["deflated_" + mode + "_info"] = linfo

    # wall-bounded flow (zbond != 0): 64 drops x 512 nodes above the wall y = 0, every
    # Stokes sum with the images across it; solves as above, and the operator with and
    # without the images on the same geometry
    wcfg = configs.wall_drops(k=64, n=512, seed=12, box=24.0)
    ctx_w = Context(device=local, graphs=graphs)
    ctx_w.set_stream(stream.cuda_stream)
    ctx_w.set_wall(1)
    wgeo = ctx_w.extractdat(wcfg.nd, wcfg.rku())
    wrhs = torch.from_numpy(surface_tension_rhs(wgeo["dz"], wgeo["dsda"])).to(dev)
    wx = torch.empty_like(wrhs)
    wall = {"workload": wcfg.name + " above the wall y = 0", "nodes": wcfg.nbk}
    for mode in ("fp64", "fp32_refined"):
        for _ in range(args.warmup):
            ctx_w.solvei(wrhs, mode, out=wx)
        torch.cuda.synchronize()
        ew0, ew1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ew0.record(stream)
        for _ in range(args.steps):
            _, winfo = ctx_w.solvei(wrhs, mode, out=wx)
        ew1.record(stream)
        torch.cuda.synchronize()
        wall[mode + "_solves_per_s"] = world * args.steps / (ew0.elapsed_time(ew1) * 1e-3)
        wall[mode + "_info"] = winfo
    wu = torch.randn(2 * wcfg.nbk, dtype=torch.float64, device=dev)
    wy = torch.empty_like(wu)
    for iw in (1, 0):
        ctx_w.set_wall(iw)
        for prec in ("fp64", "fp32"):
            for _ in range(3):
                ctx_w.fasmvp(wu, prec, out=wy)
            torch.cuda.synchronize()
            ew0, ew1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ew0.record(stream)
            for _ in range(10):
                ctx_w.fasmvp(wu, prec, out=wy)
            ew1.record(stream)
            torch.cuda.synchronize()
            wall["apply_us_%s_%s" % (prec, "wall" if iw else "free")] = ew0.elapsed_time(ew1) * 100.0
    ctx_w.close()

    # FMM Mpts/s: single Stokes operator applies, FP64 and FP32
    u = torch.randn(n, dtype=torch.float64, device=dev)
    y = torch.empty_like(u)
    mpts = {}
    for prec in ("fp64", "fp32"):
        for _ in range(3):
            ctx.fasmvp(u, prec, out=y)
        reps = 10
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(reps):
            flush.zero_()
            e0.record(stream)
            ctx.fasmvp(u, prec, out=y)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        mpts[prec] = cfg.nbk / (tot / reps * 1e-3) / 1e6

    # per-kernel live CUDA-event timing of the near-field (P2P + L2P) and M2L kernels of
    # both operator precisions; algorithmic flops per launch from the tree actually built:
    # 40 per near-field pair, 8 p e per point per level of L2P, 2 * 8 p^2 per M2L pair
    tree = ctx.tree_info()
    fp64_peak = ctx.measure_fp64_peak()
    fp32_peak = ctx.measure_fp32_peak()
    levels_l2p = max(tree["levels"] - 1, 1)
    kern = {}

    def kentry(ms, nl, flops):
        return {"avg_launch_ms": ms / nl, "flops_per_launch": flops,
                "achieved_tflops": flops / (ms / nl * 1e-3) / 1e12}

    near_pair_flops = 40.0 * tree["u_pairs"]
    for c, prec, p_ord, arith in ((ctx, "fp32", 20, "fp32"), (ctx_df, "fp64", 44, "df"),
                                  (ctx, "fp64", 44, "native")):
        c.set_profiling(True)
        for _ in range(10):
            c.fasmvp(u, prec, out=y)
        nl, leaf_ms = c.kernel_time(0)
        nm, m2l_ms = c.kernel_time(1)
        nn, near_ms = c.kernel_time(2)
        c.set_profiling(False)
        m2l_flops = 2 * 8.0 * p_ord * p_ord * tree["v_pairs"]
        if arith == "fp32":
            # the far field evaluates the locals of min(levels - 1, 6) levels at every node
            far_flops = 8.0 * p_ord * 2 * tree["npoints"] * min(levels_l2p, 6)
            kern["k_near32<2>"] = kentry(near_ms, nn, near_pair_flops)
            kern["k_far32<2>"] = kentry(leaf_ms, nl, far_flops)
            kern["k_m2l_f32p<2, 20>"] = kentry(m2l_ms, nm, m2l_flops)
        elif arith == "df":
            kern["k_leaf_df<2>"] = kentry(leaf_ms, nl, near_pair_flops + 8.0 * p_ord * 2 * tree["npoints"])
            kern["k_m2l_df<2>"] = kentry(m2l_ms, nm, m2l_flops)
        else:
            kern["k_leaf64<2>"] = kentry(leaf_ms, nl, near_pair_flops + 8.0 * p_ord * 2 * tree["npoints"])
            kern["k_m2l<double, 2>"] = kentry(m2l_ms, nm, m2l_flops)
    ctx_df.close()
    # the FP32 M2L on the tensor cores (tcgen05, 3xTF32) against the CUDA-core M2L
    ctx_tc = Context(device=local, graphs=graphs, m2l_tc=1)
    ctx_tc.set_stream(stream.cuda_stream)
    ctx_tc.extractdat(cfg.nd, cfg.rku())
    ctx_tc.set_profiling(True)
    for _ in range(10):
        ctx_tc.fasmvp(u, "fp32", out=y)
    ntc, tc_ms = ctx_tc.kernel_time(1)
    ctx_tc.set_profiling(False)
    kern["k_m2l_tc<2> (tcgen05)"] = kentry(tc_ms, ntc, 2 * 8.0 * 20 * 20 * tree["v_pairs"])
    ms_tc, _, _ = timed("fp32_refined", args.steps, args.warmup, ctx_tc)
    m2l_ab = {"k_m2l_f32p_us": 1e3 * kern["k_m2l_f32p<2, 20>"]["avg_launch_ms"],
              "k_m2l_tc_us": 1e3 * tc_ms / max(ntc, 1),
              "refined_solves_per_s_tc": world * args.steps / (ms_tc * 1e-3),
              "kept": "CUDA-core k_m2l_f32p (eb_opts.m2l_tc off by default)"}
    ctx_tc.close()
    for name, k in kern.items():
        if name in ("k_leaf64<2>", "k_m2l<double, 2>"):
            k["peak_tflops"] = fp64_peak
            k["frac_of_fp64_peak"] = k["achieved_tflops"] / fp64_peak
            continue
        k["peak_tflops"] = fp32_peak
        k["frac_of_fp32_peak"] = k["achieved_tflops"] / fp32_peak
        if "df" in name:
            # double-float kernels do FP64-class arithmetic on the FP32 pipes
            k["frac_of_fp64_peak"] = k["achieved_tflops"] / fp64_peak
    dom = kern["k_near32<2>"]

    # end to end through the C ABI with host buffers: geometry + rhs in, solution out
    zh = torch.from_numpy(np.ascontiguousarray(geo["z"]).view(np.float64).copy()).pin_memory()
    dzh = torch.from_numpy(np.ascontiguousarray(geo["dz"]).view(np.float64).copy()).pin_memory()
    dsh = torch.from_numpy(geo["dsda"].copy()).pin_memory()
    kah = torch.from_numpy(geo["kappa"].copy()).pin_memory()
    zkh = torch.from_numpy(np.ascontiguousarray(geo["zk"]).view(np.float64).copy()).pin_memory()
    rhh = torch.from_numpy(rhs_h.copy()).pin_memory()
    xh = torch.empty_like(rhh).pin_memory()
    lib, h = ctx._lib, ctx._h
    nd = np.ascontiguousarray(cfg.nd, dtype=np.int32)
    import ctypes
    from electricbubbles_gb300._lib import SolveInfo, check

    def e2e_step():
        check("eb_set_geometry", lib.eb_set_geometry(h, cfg.k, nd.ctypes.data, zh.data_ptr(), dzh.data_ptr(),
                                                      dsh.data_ptr(), kah.data_ptr(), zkh.data_ptr(), 0))
        info = SolveInfo()
        check("eb_stokes_solve", lib.eb_stokes_solve(h, n, rhh.data_ptr(), xh.data_ptr(), 1,
                                                      ctypes.byref(info), 0))

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = 0.0
    for s in range(args.steps):
        flush.zero_()
        ev[s][0].record(stream)
        e2e_step()  # returns with the solution in host memory
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    e2e_ms = sum(a.elapsed_time(b) for a, b in ev[:args.steps])
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        e2e_ms = float(t.item())
    h2d = 8 * (zh.numel() + dzh.numel() + dsh.numel() + kah.numel() + zkh.numel() + rhh.numel()) + 4 * cfg.k
    d2h = 8 * xh.numel()

    # RK2 steps (F twice: EXTRACTDAT, Laplace solve, DtN, SETVELF, Stokes solve,
    # INTERFACENEW, EQUIT/FILTER) with the state resident on the GPU
    def rk_rate(c, mode, steps, e0=0.5, cx=None):
        cx = cx or ctx
        y0 = torch.from_numpy(c.rku()).to(dev)
        y = y0.clone()
        cx.rk2(c.nd, 1e-3, y, e0=e0, mode=mode)
        torch.cuda.synchronize()
        e0_, e1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0_.record(stream)
        for _ in range(steps):
            info = cx.rk2(c.nd, 1e-3, y, e0=e0, mode=mode)
        e1_.record(stream)
        torch.cuda.synchronize()
        return steps / (e0_.elapsed_time(e1_) * 1e-3), info

    rk = {}
    for mode in ("fp64", "fp32_refined"):
        r, info = rk_rate(cfg, mode, 3)
        rk[WORKLOAD + "/" + mode] = {"steps_per_s": r, "last_step": info}
        r, info = rk_rate(cfg, mode, 3, cx=ctx_ld)
        rk[WORKLOAD + "/" + mode + "/lap_deflate"] = {"steps_per_s": r, "last_step": info}
    single = configs.single_drop(256)
    for mode in ("fp64", "fp32_refined"):
        r, info = rk_rate(single, mode, 100)
        rk["single_drop_n256/" + mode] = {"steps_per_s": r, "last_step": info, "steps": 100}

    # the single drop (N = 256, E0 = 0.5): plain FP64 Stokes and Laplace solves/s and
    # F-evaluations/s (the RK right-hand side: EXTRACTDAT, both solves, DtN, SETVELF,
    # INTERFACENEW, EQUIT), with the small-problem direct sums (the default below 1,024
    # points) and with the FMM at every size
    def single_rates(cx, reps=50):
        sg = cx.extractdat(single.nd, single.rku())
        srhs = torch.from_numpy(surface_tension_rhs(sg["dz"], sg["dsda"])).to(dev)
        srl = torch.from_numpy(np.ascontiguousarray(-2.0 * np.ascontiguousarray(sg["z"]).real)).to(dev)
        sx, sxl = torch.empty_like(srhs), torch.empty_like(srl)
        sy = torch.from_numpy(single.rku()).to(dev)
        sd = torch.empty_like(sy)
        out = {}
        for lab, fn in (("stokes_solves_per_s", lambda: cx.solvei(srhs, "fp64", out=sx)),
                        ("laplace_solves_per_s", lambda: cx.solve_lapl(srl, "fp64", out=sxl)),
                        ("f_evals_per_s", lambda: cx.f(single.nd, sy, e0=0.5, mode="fp64", out=sd))):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0_, e1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0_.record(stream)
            for _ in range(reps):
                fn()
            e1_.record(stream)
            torch.cuda.synchronize()
            out[lab] = reps / (e0_.elapsed_time(e1_) * 1e-3)
        return out
    single_fp64 = {"workload": "single_drop_n256 (E0 = 0.5, plain FP64)"}
    for lab, dm in (("direct", 0), ("fmm", -1)):
        cx = Context(device=local, graphs=graphs, direct_max=dm)
        cx.set_stream(stream.cuda_stream)
        single_fp64[lab] = single_rates(cx)
        cx.close()

    # the 256 independent single-drop simulations of uneven sizes (N log-uniform in
    # [128, 4096], E0 U[0.1, 1], seed 4) as one batch in one context: every kernel
    # launch covers all simulations, GMRES per simulation; 50 FP32-refined RK2 steps
    # (dt = 1e-3), timed on the device after one untimed step
    sims = configs.uneven_simulations()
    bnd = np.concatenate([sm.nd for sm in sims])
    be0 = np.array([sm.params["E0"] for sm in sims])
    by = torch.from_numpy(np.concatenate([sm.rku() for sm in sims])).to(dev)
    bctx = Context(device=local, graphs=graphs)
    bctx.set_stream(stream.cuda_stream)
    bctx.batch_define([sm.k for sm in sims], be0)
    uneven_steps = 50
    binfo = bctx.rk2(bnd, 1e-3, by, mode="fp32_refined")
    # leaf sizes picked for this forest by the autotuner (FP32 operator timed per
    # candidate), once, before the timed steps; every later stage's tree uses them
    btune = bctx.autotune()
    binfo = bctx.rk2(bnd, 1e-3, by, mode="fp32_refined")
    torch.cuda.synchronize()
    ea_, eb2_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ea_.record(stream)
    l0 = bctx.launch_count()
    for _ in range(uneven_steps):
        binfo = bctx.rk2(bnd, 1e-3, by, mode="fp32_refined")
    eb2_.record(stream)
    torch.cuda.synchronize()
    bms = ea_.elapsed_time(eb2_)
    uneven = {"workload": "uneven_simulations_256 (N log-uniform in [128, 4096], seed 4)",
              "simulations": len(sims), "nodes": int(bnd.sum()), "steps": uneven_steps, "mode": "fp32_refined",
              "batched": "one context, one launch per kernel for all simulations, GMRES per simulation",
              "ms_per_step": bms / uneven_steps,
              "sim_steps_per_s": len(sims) * uneven_steps / (bms * 1e-3),
              "launches_per_step": (bctx.launch_count() - l0) / uneven_steps,
              "last_step": binfo, "tree": bctx.tree_info(),
              "autotuned": {"leaf64": btune["leaf64"], "leaf_cap": btune["leaf_cap"],
                            "fp32_apply_us": {"%d/%d" % (c["leaf64"], c["leaf_cap"]): round(c["apply_us"], 1)
                                              for c in btune["candidates"]}}}
    bctx.close()

    # the gradient workload (16 drops x 512, radii U[0.6, 1], seed 5): J = the summed
    # Taylor deformation (L - B)/(L + B) after 50 RK2 steps (dt = 1e-3, E0 = 0.5, plain
    # FP64, GMRES 1e-10), and dJ/dy0, dJ/dE0, dJ/dcap by reverse mode (checkpointed states,
    # hand-written adjoint kernels, transposed solves); wall time of the whole gradient,
    # host state. Checked against central differences (step 1e-4) of the forward steps
    # along E0 and along a smooth node displacement (drop modes 1 to 5).
    gcfg = configs.gradient_drops()
    gsteps, gdt, ge0 = 50, 1e-3, 0.5
    gctx = Context(device=local, graphs=graphs)
    gctx.set_stream(stream.cuda_stream)
    gy0 = gcfg.rku()
    gctx.rk2_gradient(gcfg.nd, gdt, gy0, 1, e0=ge0)  # warm-up (allocations, graphs)
    torch.cuda.synchronize()
    t0g = time.perf_counter()
    grad = gctx.rk2_gradient(gcfg.nd, gdt, gy0, gsteps, e0=ge0)
    torch.cuda.synchronize()
    grad_s = time.perf_counter() - t0g

    def g_loss(yv, e):
        yv = yv.copy()
        for _ in range(gsteps):
            gctx.rk2(gcfg.nd, gdt, yv, e0=e)
        return gctx.deformation(gcfg.nd, yv, grad=False)[0]

    t0f = time.perf_counter()
    g_loss(gy0, ge0)
    fwd_s = time.perf_counter() - t0f
    hfd = 1e-4
    fd_e0 = (g_loss(gy0, ge0 + hfd) - g_loss(gy0, ge0 - hfd)) / (2 * hfd)
    grng = np.random.default_rng(96)
    dz_ = np.zeros(gcfg.nbk, complex)
    for b in range(gcfg.k):
        th = 2 * np.pi * np.arange(512) / 512
        for m in range(1, 6):
            ca, cb = grng.standard_normal(2) + 1j * grng.standard_normal(2)
            dz_[512 * b:512 * (b + 1)] += ca * np.exp(1j * m * th) + cb * np.exp(-1j * m * th)
    gd = np.stack([dz_.real, dz_.imag], 1).reshape(-1)
    gd /= np.linalg.norm(gd)
    fd_dir = (g_loss(gy0 + hfd * gd, ge0) - g_loss(gy0 - hfd * gd, ge0)) / (2 * hfd)
    ad_dir = float(grad["y0"] @ gd)
    # the same gradient with FP32-refined forward and transposed solves
    gctx.rk2_gradient(gcfg.nd, gdt, gy0, 1, e0=ge0, mode="fp32_refined")
    torch.cuda.synchronize()
    t0g = time.perf_counter()
    grad32 = gctx.rk2_gradient(gcfg.nd, gdt, gy0, gsteps, e0=ge0, mode="fp32_refined")
    torch.cuda.synchronize()
    grad32_s = time.perf_counter() - t0g
    gradient = {"workload": "gradient_drops_16x512 (seed 5), 50 RK2 steps, dt 1e-3, E0 0.5, plain FP64, GMRES 1e-10",
                "loss": "sum over drops of (L - B)/(L + B)", "J": grad["J"],
                "gradient_wall_s": grad_s, "forward_wall_s": fwd_s, "gradient_over_forward": grad_s / fwd_s,
                "dJ_dE0": grad["e0"], "dJ_dcap": grad["cap"], "dJ_dy0_norm": float(np.linalg.norm(grad["y0"])),
                "fd_check_h": hfd,
                "dJ_dE0_vs_central_difference_rel": abs(grad["e0"] - fd_e0) / abs(fd_e0),
                "smooth_direction_vs_central_difference_rel": abs(ad_dir - fd_dir) / abs(fd_dir),
                "solves": grad["info"],
                "fp32_refined": {"gradient_wall_s": grad32_s,
                                 "dJ_dy0_rel_vs_fp64": float(np.linalg.norm(grad32["y0"] - grad["y0"])
                                                             / np.linalg.norm(grad["y0"])),
                                 "dJ_dE0_rel_vs_fp64": abs(grad32["e0"] - grad["e0"]) / abs(grad["e0"])}}
    gctx.close()

    # the 1,024 x 1,024 workload (N = 1,048,576): FMM Mpts/s and one full solve per mode
    big = configs.large_drops()
    gb = ctx.extractdat(big.nd, big.rku())
    ub = torch.randn(2 * big.nbk, dtype=torch.float64, device=dev)
    yb = torch.empty_like(ub)
    large = {"workload": "large_drops_1024x1024", "nodes": big.nbk, "tree": ctx.tree_info()}
    ea, eb_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for prec in ("fp64", "fp32"):
        ctx.fasmvp(ub, prec, out=yb)
        torch.cuda.synchronize()
        ea.record(stream)
        for _ in range(3):
            ctx.fasmvp(ub, prec, out=yb)
        eb_.record(stream)
        torch.cuda.synchronize()
        large["fmm_mpts_per_s_" + prec] = big.nbk / (ea.elapsed_time(eb_) / 3 * 1e-3) / 1e6
    # the FP32 kernels at this size (near and far field, M2L; timed in profiling mode, where
    # the near field runs on the main stream) against the FP32 peak: where the 64 x 512
    # kernels are latency-bound, these fill the GPU
    btree = large["tree"]
    ctx.set_profiling(True)
    for _ in range(3):
        ctx.fasmvp(ub, "fp32", out=yb)
    nl, leaf_ms = ctx.kernel_time(0)
    nm, m2l_ms = ctx.kernel_time(1)
    nn, near_ms = ctx.kernel_time(2)
    ctx.set_profiling(False)
    bkern = {"k_near32<2>": kentry(near_ms, nn, 40.0 * btree["u_pairs"]),
             "k_far32<2>": kentry(leaf_ms, nl, 8.0 * 20 * 2 * btree["npoints"] * min(max(btree["levels"] - 1, 1), 6)),
             "k_m2l_f32p<2, 20>": kentry(m2l_ms, nm, 2 * 8.0 * 20 * 20 * btree["v_pairs"])}
    for v in bkern.values():
        v["frac_of_fp32_peak"] = v["achieved_tflops"] / fp32_peak
    large["kernels_fp32"] = bkern
    rb = torch.from_numpy(surface_tension_rhs(gb["dz"], gb["dsda"])).to(dev)
    xb = torch.empty_like(rb)
    for mode in ("fp64", "fp32_refined"):
        ea.record(stream)
        _, info = ctx.solvei(rb, mode, out=xb)
        eb_.record(stream)
        torch.cuda.synchronize()
        large["solve_ms_" + mode] = ea.elapsed_time(eb_)
        large["solve_info_" + mode] = info
    # the Laplace solve (GETBCs' -2 Re z) on the 1,024 drops: each drop adds one small,
    # distinct eigenvalue to FASMVP_LAP, more than the MAXL = 100 Krylov vectors of a
    # GMRES cycle resolve; with the per-drop deflation (eb_opts.lap_deflate) it converges
    rlb = torch.from_numpy(np.ascontiguousarray(-2.0 * np.ascontiguousarray(gb["z"]).real)).to(dev)
    xlb = torch.empty_like(rlb)
    ctx_ldb = Context(device=local, graphs=graphs, lap_deflate=1)
    ctx_ldb.set_stream(stream.cuda_stream)
    ctx_ldb.extractdat(big.nd, big.rku())
    for lab, cx in (("laplace_refined", ctx), ("laplace_refined_deflated", ctx_ldb)):
        ea.record(stream)
        _, info = cx.solve_lapl(rlb, "fp32_refined", out=xlb)
        eb_.record(stream)
        torch.cuda.synchronize()
        large[lab + "_ms"] = ea.elapsed_time(eb_)
        large[lab + "_info"] = info
    ctx_ldb.close()

    cpu = None
    if rank == 0:
        ncores = os.cpu_count() or 1
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as O
            ncores = O.max_threads()
            times, _, xr = cpu_reference_solves(cfg, 2, ncores)
            # the reference is serial: one solve on one thread as well
            times1, _, _ = cpu_reference_solves(cfg, 1, 1)
            # Laplace: SOLVE_LAPL with the restated DAPIF2 FMM (NAPB 30, TOL 1e-11)
            exo = O.extractdat(cfg.nd, cfg.rku())
            go = O.Geometry.from_extract(cfg.nd, exo)
            t0l = time.perf_counter()
            O.solve_lapl(go, -2.0 * exo["z"].real, nthreads=ncores, mode=1)
            lap_cpu = 1.0 / (time.perf_counter() - t0l)
            # the GPU solutions' true residuals against the exact operator (direct sums)
            rhs_np = rhs.cpu().numpy()
            exact = {}
            for lab, xs in (("fp32_refined", x), ("fp64", x64)):
                xv = xs.cpu().numpy()
                res = rhs_np - O.fasmvp(go, xv, 0, ncores)
                exact[lab] = float(np.linalg.norm(res) / np.linalg.norm(rhs_np))
            cpu = {"value": 2 / sum(times), "unit": "solves/s", "cores": ncores, "kind": "port",
                   "gpu_true_residual_vs_direct_sum": exact,
                   "sample": "2 full Stokes solves of the 64x512 workload with the restated "
                             "CADAPDR FMM + SLATEC GMRES",
                   "value_1thread": 1 / sum(times1),
                   "laplace_solves_per_s": lap_cpu,
                   "laplace_solver": "SOLVE_LAPL with the restated DAPIF2 FMM (NAPB 30, TOL 1e-11)",
                   "gpu_vs_cpu_solution_rel": float(np.linalg.norm(x.cpu().numpy() - xr) / np.linalg.norm(xr))}
        except Exception as exc:  # the baseline must not hide the GPU result
            cpu = {"value": None, "unit": "solves/s", "cores": ncores, "kind": "port",
                   "sample": "failed: %s" % exc}

    value = world * args.steps / (ms32 * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 inner operator, f64 residual/Arnoldi (refined)",
        "data": "synthetic (seeded drops; surface-tension right-hand side)",
        "config": {"workload": WORKLOAD, "nodes": cfg.nbk, "unknowns": n, "drops": cfg.k,
                   "solve": "fp32_refined GMRES-IR from x = 0 (FP32 inner GMRES, double-float FP64-class "
                            "residuals), tol 1e-10", "parallelism": "replicas",
                   "l2": "256 MiB write between timed steps (outside the step's CUDA events)"},
        "fp64_solves_per_s": world * args.steps / (ms64 * 1e-3),
        "fp64_solve": "plain GMRES from x0 = b, native FP64 operators throughout (the default plain path)",
        "fp64df_solves_per_s": world * args.steps / (ms64_df * 1e-3),
        "refined_speedup_vs_fp64": ms64 / ms32,
        "refined_speedup_vs_fp64df": ms64_df / ms32,
        "fmm_mpts_per_s": mpts,
        "solve_info": {"fp64": inf64[-1], "fp32_refined": inf32[-1]},
        "accuracy": {"refined_vs_fp64_rel_l2": rel_diff, "refined_true_residual": inf32[-1]["err"]},
        "tree": tree,
        "roofline": {"kernel": "k_near32<2> (FP32 near field P2P over the U lists, 40 flop per "
                               "target-source pair; with k_m2l_f32p<2, 20> and k_p2m_chunks<2> the largest "
                               "kernels of the refined solve)", "bound": "fp32",
                     "achieved": dom["achieved_tflops"], "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": dom["achieved_tflops"] / fp32_peak,
                     # DRAM bytes of one k_near32<2> launch of this workload (ncu
                     # dram__bytes_read.sum + dram__bytes_write.sum: 1,381,632 + 0)
                     "traffic": 1381632 if WORKLOAD == "many_drops_64x512" else None,
                     "traffic_unit": "bytes per launch (ncu capture of this workload)",
                     "peak_source": "measured in-run FP32 FMA chain (MEASURED_PEAKS.json has no FP32 "
                                    "CUDA-core figure)",
                     "flops_per_launch": dom["flops_per_launch"], "avg_launch_ms": dom["avg_launch_ms"]},
        "kernels": kern,
        "m2l_tensor_ab": m2l_ab,
        "laplace": lap,
        "wall": wall,
        "peaks_measured_in_run": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak},
        "cpu_baseline": cpu,
        "e2e": {"value": world * args.steps / (e2e_ms * 1e-3), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "includes": "eb_set_geometry (copy + tree build) and eb_stokes_solve from pinned host buffers"},
        "clocks": clk,
        "gpu_launches": launches,
        "rk2": rk,
        "single_drop": single_fp64,
        "uneven": uneven,
        "gradient": gradient,
        "large": large,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        td.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    from electricbubbles_gb300 import build
    build.build()
    run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
