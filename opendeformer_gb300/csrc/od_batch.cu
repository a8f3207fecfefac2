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

// Newmark vector operations of od_step on a tile of padded DOFs of one scene
__global__ void nm_batch_kernel(int op, const Tile* __restrict__ tiles, const SceneDev* __restrict__ sd) {
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev& D = sd[tl.scene];
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
  Tile* tiles = nullptr;  // all tile lists in one allocation
  int n_zero = 0, n_corot = 0, n_inv = 0, n_exp = 0, n_rows = 0, n_dof = 0;
  Tile *t_zero = nullptr, *t_corot = nullptr, *t_inv = nullptr, *t_scat = nullptr, *t_exp = nullptr,
       *t_rows = nullptr, *t_dof = nullptr;
  std::vector<int> scat_off;
  MixedSys* mix = nullptr;
  int newton = 1, precond = OD_PRECOND_BLOCK_JACOBI;
  std::vector<od_solver_params> prm;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

static void batch_free(Batch* b) {
  if (!b) return;
  cudaFree(b->sd);
  cudaFree(b->tiles);
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
  D.tets = s->tets;
  D.X = s->X;
  D.u = s->u;
  D.pre = s->pre;
  D.emap = s->emap;
  D.gdof = s->gdof;
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

static void chunk(std::vector<Tile>& out, int scene, int n, int step, int aux = 0, int aux2 = 0) {
  for (int b = 0; b < n; b += step) out.push_back(Tile{scene, b, std::min(n, b + step), aux, aux2});
}

static od_status batch_build(Batch* B) {
  const int n = (int)B->sc.size();
  std::vector<Tile> zero, corot, inv, scat, exp, rows, dof;
  int max_colors = 0;
  for (int i = 0; i < n; i++) {
    const Scene* s = B->sc[i];
    B->sd_host.push_back(scene_dev(s));
    chunk(zero, i, s->nvals, 4096, 0);
    chunk(zero, i, s->pcg.n_pad, 4096, 1);
    chunk(s->mat.kind == OD_MATERIAL_COROTATIONAL ? corot : inv, i, s->n_tets, 128);
    chunk(exp, i, 9 * s->bsr.nnzb, 2048);
    chunk(rows, i, s->bsr.nb, kBatchRows);
    chunk(dof, i, s->pcg.n_pad, 256);
    max_colors = std::max(max_colors, (int)s->color_off.size() - 1);
  }
  B->scat_off.assign(1, 0);
  for (int c = 0; c < max_colors; c++) {
    for (int i = 0; i < n; i++) {
      const Scene* s = B->sc[i];
      if (c + 1 >= (int)s->color_off.size()) continue;
      const int e0 = s->color_off[c], cnt = s->color_off[c + 1] - e0;
      if (cnt <= 0) continue;
      for (int t = 0; t < 90 * cnt; t += 256) scat.push_back(Tile{i, t, std::min(90 * cnt, t + 256), e0, cnt});
    }
    B->scat_off.push_back((int)scat.size());
  }
  B->n_zero = (int)zero.size();
  B->n_corot = (int)corot.size();
  B->n_inv = (int)inv.size();
  B->n_exp = (int)exp.size();
  B->n_rows = (int)rows.size();
  B->n_dof = (int)dof.size();
  std::vector<Tile> all;
  for (auto* v : {&zero, &corot, &inv, &scat, &exp, &rows, &dof}) all.insert(all.end(), v->begin(), v->end());
  OD_CUDA(cudaMalloc(&B->tiles, sizeof(Tile) * std::max<size_t>(1, all.size())));
  if (!all.empty()) OD_CUDA(cudaMemcpy(B->tiles, all.data(), sizeof(Tile) * all.size(), cudaMemcpyHostToDevice));
  Tile* p = B->tiles;
  B->t_zero = p; p += zero.size();
  B->t_corot = p; p += corot.size();
  B->t_inv = p; p += inv.size();
  B->t_scat = p; p += scat.size();
  B->t_exp = p; p += exp.size();
  B->t_rows = p; p += rows.size();
  B->t_dof = p;
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
  if (B->n_dof <= 0) return OD_OK;
  B->ctx->launches++;
  nm_batch_kernel<<<B->n_dof, 256, 0, B->ctx->stream>>>(op, B->t_dof, B->sd);
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
    OD_TRY(launch_eval_batch(ctx, B->sd, B->t_zero, B->n_zero, B->t_corot, B->n_corot, B->t_inv, B->n_inv,
                             B->t_scat, B->scat_off));
    OD_TRY(launch_spmv_lower_batch(ctx, B->sd, B->t_rows, B->n_rows));
    OD_TRY(nm_op(B, NM_RESIDUAL));
    OD_TRY(launch_expand_batch(ctx, B->sd, B->t_exp, B->n_exp));
    OD_TRY(nm_op(B, NM_ZERO_DV));
    OD_TRY(mixed_solve(ctx, B->mix, B->precond, B->prm, ss));
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
