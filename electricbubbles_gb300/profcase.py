"""A short run of every stage of the hot path, for kernel profilers.

    python -m electricbubbles_gb300.profcase [stage ...]

Stages (all by default), on the 64-drop x 512-node workload unless named otherwise:
  tree     geometry install: EXTRACTDAT and the adaptive tree build
  solve    one FP32-refined Stokes solve with the GMRES loop driven from the host, so
           that every kernel is its own launch (the Arnoldi, FP32 and double-float
           operator kernels)
  apply    ten FP32 Stokes operator applies, then ten double-float ones
  rk2      one FP32-refined RK2 step (the spectral kernels, SETVELF, EQUIT, both solves)
  batch    one FP32-refined RK2 step of 64 of the uneven simulations as one batch
  wall     one FP32-refined Stokes solve (host loop) of 64 drops x 512 nodes above the
           wall y = 0: the image lists, mirrored multipoles and reflected near field
  lapsolve one FP32-refined Laplace solve (host loop) with the per-drop deflation
           (eb_opts.lap_deflate): k_deflate and the one-pass inner Arnoldi kernels
  single   one plain FP64 RK2 step of the single 256-node drop (direct sums: at most
           1,024 points)
  batchloop one FP32-refined RK2 step of 64 of the uneven simulations as one batch with
           the GMRES loops driven from the host (the batched Arnoldi kernels as launches)
  vjp      one adjoint of F (eb_rk_f_vjp) on the 16-drop x 512-node gradient workload,
           plain FP64 with the GMRES loops driven from the host: the stage's forward rerun,
           the transposed solves and the adjoint kernels

Each stage runs once; the device holds well under 1 GB. Prints "ok" at the end.
"""
import sys

import numpy as np

from . import configs
from .api import Context


def _tree(ctx, cfg):
    return ctx.extractdat(cfg.nd, cfg.rku())


def stage_tree():
    ctx = Context(graphs=-1)
    _tree(ctx, configs.many_drops())


def stage_solve():
    cfg = configs.many_drops()
    ctx = Context(graphs=-1)
    g = _tree(ctx, cfg)
    rhs = np.ascontiguousarray(-0.5 * g["dz"] / g["dsda"]).view(np.float64).copy()
    ctx.solvei(rhs, "fp32_refined")


def stage_apply():
    cfg = configs.many_drops()
    rng = np.random.default_rng(5)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    for prec, df64 in (("fp32", 0), ("fp64", 1)):
        ctx = Context(graphs=-1, df64=df64)
        _tree(ctx, cfg)
        for _ in range(10):
            ctx.stokes_sum(dens, -1, prec)
        ctx.close()


def stage_rk2():
    cfg = configs.many_drops()
    ctx = Context(graphs=-1)
    ctx.rk2(cfg.nd, 1e-3, cfg.rku(), e0=0.5, mode="fp32_refined")


def stage_batch():
    sims = configs.uneven_simulations()[:64]
    ctx = Context()
    ctx.batch_define([s.k for s in sims], np.array([s.params["E0"] for s in sims]))
    nd = np.concatenate([s.nd for s in sims])
    y = np.concatenate([s.rku() for s in sims])
    ctx.rk2(nd, 1e-3, y, mode="fp32_refined")


def stage_wall():
    cfg = configs.wall_drops(k=64, n=512, seed=12, box=24.0)
    ctx = Context(graphs=-1)
    ctx.set_wall(1)
    g = _tree(ctx, cfg)
    rhs = np.ascontiguousarray(-0.5 * g["dz"] / g["dsda"]).view(np.float64).copy()
    ctx.solvei(rhs, "fp32_refined")


def stage_lapsolve():
    cfg = configs.many_drops()
    ctx = Context(graphs=-1, lap_deflate=1)
    g = _tree(ctx, cfg)
    ctx.solve_lapl(-2.0 * np.asarray(g["z"]).real, "fp32_refined")


def stage_single():
    cfg = configs.single_drop(256)
    ctx = Context()
    y = cfg.rku()
    ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, mode="fp64")


def stage_batchloop():
    sims = configs.uneven_simulations()[:64]
    ctx = Context(graphs=-1)
    ctx.batch_define([s.k for s in sims], np.array([s.params["E0"] for s in sims]))
    nd = np.concatenate([s.nd for s in sims])
    y = np.concatenate([s.rku() for s in sims])
    ctx.rk2(nd, 1e-3, y, mode="fp32_refined")


def stage_vjp():
    cfg = configs.gradient_drops()
    ctx = Context(graphs=-1)
    v = np.random.default_rng(1).standard_normal(2 * cfg.nbk)
    ctx.f_vjp(cfg.nd, cfg.rku(), v, e0=0.5)
    ctx.close()


STAGES = {"tree": stage_tree, "solve": stage_solve, "apply": stage_apply, "rk2": stage_rk2,
          "batch": stage_batch, "wall": stage_wall, "lapsolve": stage_lapsolve, "single": stage_single,
          "batchloop": stage_batchloop, "vjp": stage_vjp}


def main(argv):
    for name in argv or list(STAGES):
        STAGES[name]()
    print("ok")


if __name__ == "__main__":
    main(sys.argv[1:])
