// Autotuner of the tree's leaf sizes for the installed geometry.
//
// No counterpart in the reference, whose leaf rule is fixed (LEVMAX = 7 levels in
// CADAPDR, cadapdrop.f:252-346; NAPB = 30 points per box in DAPIF2, dapif1.f:1165-1255).
// The best leaf size depends on how the nodes are spread (drop sizes, spacing, uneven
// simulations in one batch): each candidate (mean points per leaf of the uniform floor,
// maximum points per leaf below it) is installed, the FP32 Stokes operator (the inner
// operator of the refined solver, which does nearly all of its applies) is timed with
// CUDA events, and the fastest candidate is kept.
#include <algorithm>
#include <cfloat>

#include "eb_internal.h"

namespace {
const int kCand[][2] = {{24, 48}, {32, 48}, {32, 64}, {40, 80}, {48, 96}, {32, 96}};
constexpr int kNCand = sizeof(kCand) / sizeof(kCand[0]);
constexpr int kWarm = 2, kReps = 5;
}  // namespace

int eb_autotune(eb_ctx* ctx, eb_tune_info* info) {
  if (!ctx) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const int n = 2 * ctx->nbk;
  DevBuf x, y;
  EB_TRY(x.ensure(sizeof(double) * (size_t)n));
  EB_TRY(y.ensure(sizeof(double) * (size_t)n));
  // a smooth unit density on every node: its FP32 apply costs what any density costs
  EB_CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(double) * (size_t)n, s));
  eb_tune_info out{};
  double best = DBL_MAX;
  int bi = 0;
  for (int c = 0; c < kNCand && c < EB_TUNE_MAX; ++c) {
    ctx->opts.leaf64 = kCand[c][0];
    ctx->opts.leaf_cap = kCand[c][1];
    EB_TRY(eb_geom_tree(ctx));
    for (int r = 0; r < kWarm; ++r) EB_TRY(eb_stokes_matvec_dev(ctx, x.as<double>(), y.as<double>(), EB_FP32));
    EB_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
    for (int r = 0; r < kReps; ++r) EB_TRY(eb_stokes_matvec_dev(ctx, x.as<double>(), y.as<double>(), EB_FP32));
    EB_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
    EB_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    EB_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    const double us = 1e3 * ms / kReps;
    out.leaf_target[c] = kCand[c][0];
    out.leaf_cap_cand[c] = kCand[c][1];
    out.apply_us[c] = us;
    out.ncand = c + 1;
    if (us < best) {
      best = us;
      bi = c;
    }
  }
  ctx->opts.leaf64 = kCand[bi][0];
  ctx->opts.leaf_cap = kCand[bi][1];
  EB_TRY(eb_geom_tree(ctx));
  out.leaf64 = kCand[bi][0];
  out.leaf_cap = kCand[bi][1];
  if (info) *info = out;
  return eb_check_launch(ctx, "autotune");
}
