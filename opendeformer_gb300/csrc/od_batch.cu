// Batched stepping of many scenes on one GPU (no reference counterpart: the
// reference steps one Simulator at a time, core/simulator.h:21-22).
//
// A batch advances every scene by the same Newmark step sequence as
// od_step (the full-order restatement of linearNewmark.cpp:27-30, 57-79)
// with a fixed number of launches per step whatever the number of scenes:
// each multi-scene kernel takes a table of per-scene device views
// (SceneDev) and a tile list (one CTA per tile, a tile being a contiguous
// range of one scene's elements, DOFs, block rows or values); the linear
// solves of all scenes run in one mixed-precision system (MixedSys) whose
// inner FP32 PCG is a single cooperative launch with per-scene step lengths
// and convergence.  Scenes keep their own device state, so a scene can be
// stepped alone (od_step) or in any batch between calls.
#include <cmath>
#include <vector>

#include "od_internal.h"

namespace od {

enum NmOp { NM_PREDICT = 0, NM_STAGE, NM_RESIDUAL, NM_ZERO_DV, NM_ADD, NM_CORRECT };

// Newmark vector operations of od_step on 256 padded DOFs of one scene
__global__ void nm_batch_kernel(int op, int n_sc, const int* __restrict__ prefix, const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int i = (blockIdx.x - prefix[s]) * 256 + threadIdx.x;
  if (i >= D.n_pad) return;
  if (op == NM_ZERO_DV) {
    D.dv[i] = 0.0;
    return;
  }
  if (i >= D.dofs) return;
  switch (op) {
    case NM_PREDICT:
      D.dp[i] = D.d[i] + D.h * D.v[i] + D.c_ad * D.a[i];
      D.vp[i] = D.v[i] + D.c_av * D.a[i];
      break;
    case NM_STAGE: {
      const double ai = D.a[i];
      D.u[D.free_pos[i]] = D.dp[i] + D.bh2 * ai;
      const double vk = D.vp[i] + D.gh * ai;
      D.tmp[i] = D.alpha_m * vk + ai;
      D.tmp2[i] = vk;
      break;
    }
    case NM_RESIDUAL:
      D.rhs[i] = D.fext[i] - D.fint[i] - D.rhs[i];
      break;
    case NM_ADD:
      D.a[i] += D.dv[i];
      break;
    case NM_CORRECT:
      D.d[i] = D.dp[i] + D.bh2 * D.a[i];
      D.v[i] = D.vp[i] + D.gh * D.a[i];
      D.u[D.free_pos[i]] = D.d[i];
      break;
  }
}

struct Batch {
  Ctx* ctx = nullptr;
  std::vector<Scene*> sc;
  std::vector<SceneDev> sd_host;
  SceneDev* sd = nullptr;
  int* dirs = nullptr;  // all tile-directory prefixes in one allocation
  TileDir zero_k, zero_f, corot, inv, plastic, expand, rows, dof;
  std::vector<TileDir> scatter;  // per colour
  TileDir gather{nullptr, -1, 256};  // gathered assembly (tiles -1: some scene has no lists)
  MixedSys* mix = nullptr;
  int newton = 1, precond = OD_PRECOND_BLOCK_JACOBI;
  std::vector<od_solver_params> prm;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool stepped = false;  // a Newton system of the last step is on the device
};

static void batch_free(Batch* b) {
  if (!b) return;
  cudaFree(b->sd);
  cudaFree(b->dirs);
  mixed_free(b->mix);
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  delete b;
}

static SceneDev scene_dev(const Scene* s) {
  SceneDev D{};
  const od_integrator_params& p = s->ip;
  D.n_tets = s->n_tets;
  D.dofs = s->dofs;
  D.nb = s->bsr.nb;
  D.n_pad = s->pcg.n_pad;
  D.nvals = s->nvals;
  D.nnzb = s->bsr.nnzb;
  D.kind = s->mat.kind;
  D.thr = s->mat.threshold;
  D.lambda = s->lambda;
  D.mu = s->mu;
  D.yield = s->mat.yield_criterion;
  D.creep = s->mat.creep_ratio;
  D.max_plastic = s->mat.max_plastic_strain;
  D.plastic = s->plastic;
  D.tets = s->tets;
  D.X = s->X;
  D.u = s->u;
  D.pre = s->pre;
  D.emap = s->emap;
  D.gdof = s->gdof;
  D.color_off = s->color_off_dev;
  D.gat_kptr = s->gat_kptr;
  D.gat_ksrc = s->gat_ksrc;
  D.gat_fptr = s->gat_fptr;
  D.gat_fsrc = s->gat_fsrc;
  D.K = s->K;
  D.fint = s->fint;
  D.stage_k = s->stage_k;
  D.stage_f = s->stage_f;
  D.M = s->M;
  D.fext = s->fext;
  D.row_ptr = s->bsr.row_ptr;
  D.col = s->bsr.col;
  D.desc_kind = s->bsr.desc_kind;
  D.desc_off = s->bsr.desc_off;
  D.gen = s->bsr.gen;
  D.A64 = s->A64;
  D.free_pos = s->free_pos;
  D.d = s->d;
  D.v = s->v;
  D.a = s->a;
  D.dp = s->dp;
  D.vp = s->vp;
  D.dv = s->dv;
  D.rhs = s->rhs;
  D.tmp = s->tmp;
  D.tmp2 = s->tmp2;
  const double h = p.dt;
  D.h = h;
  D.bh2 = p.nm_beta * h * h;
  D.gh = p.nm_gamma * h;
  D.c_ad = (0.5 - p.nm_beta) * h * h;
  D.c_av = (1.0 - p.nm_gamma) * h;
  D.alpha_m = p.alpha_m;
  D.beta_k = p.beta_k;
  return D;
}

static int ceil_div(long long n, int d) { return (int)((n + d - 1) / d); }

// the tile directories of every multi-scene kernel: O(scenes) host work
static od_status batch_build(Batch* B) {
  const int n = (int)B->sc.size();
  int max_colors = 0;
  for (const Scene* s : B->sc) max_colors = std::max(max_colors, (int)s->color_off.size() - 1);
  const int n_dirs = 9 + max_colors;
  bool gathered = true;
  for (const Scene* s : B->sc) gathered = gathered && (s->gat_kptr || s->n_tets == 0);
  std::vector<int> pre((size_t)n_dirs * (n + 1), 0);
  auto P = [&](int d) { return pre.data() + (size_t)d * (n + 1); };
  for (int i = 0; i < n; i++) {
    const Scene* s = B->sc[i];
    B->sd_host.push_back(scene_dev(s));
    const int kind = s->mat.kind;
    const bool corot = kind == OD_MATERIAL_COROTATIONAL, plastic = kind == OD_MATERIAL_COROTATIONAL_PLASTIC;
    const int et = ceil_div(s->n_tets, 128);
    const int counts[8] = {ceil_div(s->nvals, kZeroTileValues), ceil_div(s->pcg.n_pad, kZeroTileValues),
                           corot ? et : 0, corot || plastic ? 0 : et, plastic ? et : 0,
                           ceil_div(9LL * s->bsr.nnzb, kExpandTile), ceil_div(s->bsr.nb, kBatchRows),
                           ceil_div(s->pcg.n_pad, 256)};
    for (int d = 0; d < 8; d++) P(d)[i + 1] = P(d)[i] + counts[d];
    P(8)[i + 1] = P(8)[i] + (s->gat_kptr ? ceil_div((long long)s->nvals + s->pcg.n_pad, 256) : 0);
    for (int c = 0; c < max_colors; c++) {
      const int cnt = c + 1 < (int)s->color_off.size() ? s->color_off[c + 1] - s->color_off[c] : 0;
      P(9 + c)[i + 1] = P(9 + c)[i] + ceil_div(90LL * cnt, 256);
    }
  }
  OD_CUDA(cudaMalloc(&B->dirs, sizeof(int) * pre.size()));
  OD_CUDA(cudaMemcpy(B->dirs, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice));
  auto dir = [&](int d, int size) { return TileDir{B->dirs + (size_t)d * (n + 1), P(d)[n], size}; };
  B->zero_k = dir(0, kZeroTileValues);
  B->zero_f = dir(1, kZeroTileValues);
  B->corot = dir(2, 128);
  B->inv = dir(3, 128);
  B->plastic = dir(4, 128);
  B->expand = dir(5, kExpandTile);
  B->rows = dir(6, kBatchRows);
  B->dof = dir(7, 256);
  for (int c = 0; c < max_colors; c++) B->scatter.push_back(dir(9 + c, 256));
  if (gathered) B->gather = dir(8, 256);
  OD_CUDA(cudaMalloc(&B->sd, sizeof(SceneDev) * std::max(1, n)));
  OD_CUDA(cudaMemcpy(B->sd, B->sd_host.data(), sizeof(SceneDev) * n, cudaMemcpyHostToDevice));
  std::vector<const double*> rhs;
  std::vector<double*> dv;
  for (Scene* s : B->sc) {
    rhs.push_back(s->rhs);
    dv.push_back(s->dv);
  }
  OD_TRY(mixed_build(B->ctx, B->sc, rhs, dv, &B->mix));
  OD_CUDA(cudaEventCreate(&B->ev[0]));
  OD_CUDA(cudaEventCreate(&B->ev[1]));
  return OD_OK;
}

static od_status nm_op(Batch* B, int op) {
  if (B->dof.tiles <= 0) return OD_OK;
  B->ctx->launches++;
  nm_batch_kernel<<<B->dof.tiles, 256, 0, B->ctx->stream>>>(op, (int)B->sc.size(), B->dof.prefix, B->sd);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

static od_status batch_step(Batch* B, std::vector<od_step_stats>& acc) {
  Ctx* ctx = B->ctx;
  for (Scene* s : B->sc) {
    if (s->sched_freq > 0.0) {
      const double t = s->time + s->ip.dt;
      OD_TRY(launch_loads(s, s->has_body ? s->load_body : nullptr, s->n_trac,
                          std::sin(2.0 * 3.14159265358979323846 * s->sched_freq * t + s->sched_phase)));
    }
  }
  OD_TRY(nm_op(B, NM_PREDICT));
  std::vector<od_solve_stats> ss;
  for (int it = 0; it < B->newton; it++) {
    OD_TRY(nm_op(B, NM_STAGE));
    const int n = (int)B->sc.size();
    OD_TRY(launch_eval_batch(ctx, n, B->sd, B->zero_k, B->zero_f, B->corot, B->inv, B->plastic, B->scatter, B->gather));
    OD_TRY(launch_spmv_lower_batch(ctx, n, B->sd, B->rows));
    OD_TRY(nm_op(B, NM_RESIDUAL));
    OD_TRY(launch_expand_batch(ctx, n, B->sd, B->expand));
    OD_TRY(nm_op(B, NM_ZERO_DV));
    OD_TRY(mixed_solve(ctx, B->mix, B->precond, B->prm, ss, true));
    OD_TRY(nm_op(B, NM_ADD));
    for (size_t i = 0; i < B->sc.size(); i++) {
      od_step_stats& a = acc[i];
      a.pcg_iterations += ss[i].iterations;
      a.solves += 1;
      a.max_rel_residual = std::max(a.max_rel_residual, ss[i].rel_residual);
      if (ss[i].status != OD_OK && a.status == OD_OK) a.status = ss[i].status;
    }
  }
  OD_TRY(nm_op(B, NM_CORRECT));
  for (size_t i = 0; i < B->sc.size(); i++) {
    acc[i].steps++;
    B->sc[i]->time += B->sc[i]->ip.dt;
  }
  B->stepped = true;
  return OD_OK;
}

// Autotuner of the inner solve's tile shapes: the last Newton system of the
// batch (matrices and right-hand sides still on the device) is solved again
// with every candidate -- ring-kernel piece size and consumer warps x
// partition slice cost --
// from a zero correction, each timed with CUDA events on the context stream
// (best of `repeats`); the scenes' state is not touched (the corrections
// are scratch between steps) and the scenes' iteration history, which
// weights the partition, is put back after every solve.  The fastest
// candidate stays set.
static od_status batch_autotune(Batch* B, int repeats, od_tune_report* rep) {
  Ctx* ctx = B->ctx;
  MixedSys* m = B->mix;
  std::vector<double> hist;
  for (Scene* s : B->sc) hist.push_back(s->mix_iters_last);
  auto restore = [&] {
    for (size_t i = 0; i < B->sc.size(); i++) B->sc[i]->mix_iters_last = hist[i];
  };
  const int shapes[5][2] = {{12, 12}, {16, 12}, {20, 12}, {12, 15}, {16, 15}};   // piece steps, consumer warps
  const double costs[4] = {2.0, 4.0, 8.0, 16.0};
  const int def_ps = m->piece_steps, def_nw = m->ring_warps;   // the shape set before tuning
  const double def_cost = m->slice_cost;
  od_tune_report r{};
  r.best_ms = 1e300;
  std::vector<od_solve_stats> ss;
  for (int pi = 0; pi < 5; pi++)
    for (int ci = 0; ci < 4; ci++) {
      OD_TRY(mixed_retune(m, shapes[pi][0], shapes[pi][1], costs[ci]));
      float best = 1e30f;
      int iters = 0;
      for (int rr = 0; rr < std::max(1, repeats); rr++) {
        OD_TRY(nm_op(B, NM_ZERO_DV));
        OD_CUDA(cudaEventRecord(B->ev[0], ctx->stream));
        OD_TRY(mixed_solve(ctx, m, B->precond, B->prm, ss, true));
        OD_CUDA(cudaEventRecord(B->ev[1], ctx->stream));
        OD_CUDA(cudaEventSynchronize(B->ev[1]));
        restore();
        float ms = 0.f;
        OD_CUDA(cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]));
        best = std::min(best, ms);
        iters = 0;
        for (const od_solve_stats& x : ss) iters += x.iterations;
      }
      r.candidates++;
      if (shapes[pi][0] == def_ps && shapes[pi][1] == def_nw && costs[ci] == def_cost) {
        r.default_ms = best;
        r.default_iters = iters;
      }
      if (best < r.best_ms) {
        r.best_ms = best;
        r.best_iters = iters;
        r.best.piece_steps = shapes[pi][0];
        r.best.consumer_warps = shapes[pi][1];
        r.best.slice_cost = costs[ci];
      }
    }
  OD_TRY(nm_op(B, NM_ZERO_DV));
  OD_TRY(mixed_retune(m, r.best.piece_steps, r.best.consumer_warps, r.best.slice_cost));
  if (rep) *rep = r;
  return OD_OK;
}

}  // namespace od

using namespace od;

struct od_batch {
  Batch* b;
};

#define OD_BATCH_ARG(cond, msg) \
  do {                          \
    if (!(cond)) {              \
      set_error(msg);           \
      return OD_ERR_INVALID_ARG; \
    }                           \
  } while (0)

extern "C" od_status od_batch_create(od_ctx* ctx, int n_scenes, od_scene* const* scenes, od_batch** out) {
  OD_BATCH_ARG(ctx && out && (n_scenes == 0 || scenes), "od_batch_create: NULL argument");
  OD_BATCH_ARG(n_scenes > 0, "od_batch_create: empty batch");
  *out = nullptr;
  Batch* B = new Batch();
  B->ctx = &ctx->c;
  for (int i = 0; i < n_scenes; i++) {
    if (!scenes[i]) { delete B; set_error("od_batch_create: NULL scene"); return OD_ERR_INVALID_ARG; }
    Scene* s = &scenes[i]->s;
    const char* why = nullptr;
    if (s->ctx != B->ctx) why = "a scene belongs to another context";
    else if (!s->has_integrator || s->ip.kind != OD_INTEGRATOR_NEWMARK) why = "every scene needs a Newmark integrator";
    else if (s->ip.solver.precision != OD_PRECISION_MIXED) why = "every scene needs the mixed-precision solver";
    else if (s->ip.solver.precond >= OD_PRECOND_IC0)
      why = "batched scenes use the none, Jacobi or block-Jacobi preconditioner (mixed IC(0) steps alone)";
    else if (s->has_damping) why = "scenes with external damping cannot be batched";
    else if (i > 0 && s->ip.newton_iters != B->sc[0]->ip.newton_iters) why = "scenes differ in Newton iterations";
    else if (i > 0 && s->ip.solver.precond != B->sc[0]->ip.solver.precond) why = "scenes differ in preconditioner";
    for (Scene* o : B->sc)
      if (o == s) why = "a scene appears twice";
    if (why) {
      delete B;
      set_error(std::string("od_batch_create: ") + why);
      return OD_ERR_INVALID_ARG;
    }
    B->sc.push_back(s);
    B->prm.push_back(s->ip.solver);
  }
  B->newton = std::max(1, B->sc[0]->ip.newton_iters);
  B->precond = B->sc[0]->ip.solver.precond;
  OD_CUDA(cudaSetDevice(B->ctx->device));
  od_status st = batch_build(B);
  if (st != OD_OK) {
    batch_free(B);
    return st;
  }
  od_batch* h = new od_batch{B};
  *out = h;
  return OD_OK;
}

extern "C" od_status od_batch_destroy(od_batch* batch) {
  if (!batch) return OD_OK;
  cudaSetDevice(batch->b->ctx->device);
  batch_free(batch->b);
  delete batch;
  return OD_OK;
}

extern "C" od_status od_batch_get_tuning(od_batch* batch, od_mixed_tuning* out) {
  OD_BATCH_ARG(batch && out, "od_batch_get_tuning: NULL argument");
  out->piece_steps = batch->b->mix->piece_steps;
  out->consumer_warps = batch->b->mix->ring_warps;
  out->slice_cost = batch->b->mix->slice_cost;
  return OD_OK;
}

extern "C" od_status od_batch_set_tuning(od_batch* batch, const od_mixed_tuning* t) {
  OD_BATCH_ARG(batch && t, "od_batch_set_tuning: NULL argument");
  OD_CUDA(cudaSetDevice(batch->b->ctx->device));
  return mixed_retune(batch->b->mix, t->piece_steps, t->consumer_warps, t->slice_cost);
}

extern "C" od_status od_batch_autotune(od_batch* batch, int repeats, od_tune_report* report) {
  OD_BATCH_ARG(batch, "od_batch_autotune: batch is NULL");
  OD_BATCH_ARG(batch->b->stepped, "od_batch_autotune: step the batch once first (it tunes on the last system)");
  OD_BATCH_ARG(repeats >= 1 && repeats <= 16, "od_batch_autotune: repeats must be in 1..16");
  OD_CUDA(cudaSetDevice(batch->b->ctx->device));
  return batch_autotune(batch->b, repeats, report);
}

extern "C" od_status od_batch_step(od_batch* batch, int n_steps, od_step_stats* stats) {
  OD_BATCH_ARG(batch, "od_batch_step: batch is NULL");
  OD_BATCH_ARG(n_steps >= 0, "od_batch_step: negative step count");
  Batch* B = batch->b;
  Ctx* ctx = B->ctx;
  OD_CUDA(cudaSetDevice(ctx->device));
  std::vector<od_step_stats> acc(B->sc.size(), od_step_stats{});
  OD_CUDA(cudaEventRecord(B->ev[0], ctx->stream));
  od_status st = OD_OK;
  for (int k = 0; k < n_steps && st == OD_OK; k++) st = batch_step(B, acc);
  cudaEventRecord(B->ev[1], ctx->stream);
  ctx->host_syncs++;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess && st == OD_OK) st = cuda_fail(e, "od_batch_step");
  float ms = 0.f;
  if (st == OD_OK) cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]);
  if (stats)
    for (size_t i = 0; i < acc.size(); i++) {
      stats[i] = acc[i];
      stats[i].device_ms = ms;
      if (st != OD_OK && stats[i].status == OD_OK) stats[i].status = st;
    }
  return st;
}
