// Serving many simulation scenes on one GPU (od_server_*, include/od_gb300.h).
//
// No reference counterpart: the reference steps one Simulator at a time
// (core/simulator.h:21-22).  Step requests (one Newmark step of one scene,
// with that request's time step, body force and surface traction) queue per
// scene.  Every tick takes the oldest request of each scene with one pending
// (oldest first, at most max_batch), sets each request's integrator time
// step and loads, and steps the resident ones together: one od_batch step
// (batched servers) or od_step scene by scene (the plain path).  Requests
// that arrive meanwhile join a later tick (continuous batching at step
// granularity).
//
// Residency: scenes live on the device while a byte budget allows.  A tick
// that meets a request of a scene that is not resident evicts the least
// recently used resident scenes it does not step itself (each to a host
// checkpoint, od_scene_save) until the newcomer's estimated bytes fit, and
// hands the newcomer to the admission workers: host threads, each with a
// context (and stream) of its own, that build scenes -- mesh analysis,
// pattern, element maps, device arrays, integrator, checkpoint restore --
// in parallel while the tick's device work runs.  Scenes the workers
// finished join the next tick.  With admission_thread = 0 the tick builds
// them itself before stepping.
//
// Threads: the caller's thread owns the server and its context; the worker
// only creates scenes in its own context and passes them over a locked
// queue (the caller's thread then adopts them into its context).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "od_internal.h"

using namespace od;

namespace {

using clock_type = std::chrono::steady_clock;

struct Request {
  long long ticket;
  od_step_request r;
};

struct Slot {
  // the scene as registered (host copies, read-only after od_server_add_scene)
  std::vector<double> X;
  std::vector<int> tets, facets, cdofs, load_facets;
  od_material mat{};
  od_integrator_params integ{};
  // residency (caller's thread)
  enum { kCold = 0, kBuilding = 1, kResident = 2 } state = kCold;
  od_scene* scene = nullptr;
  long long bytes = 0;            // device bytes while resident (estimate while building)
  long long last_use = 0;         // LRU stamp
  std::vector<unsigned char> blob;  // checkpoint while evicted (written by the caller's thread,
  bool has_blob = false;            //  read by the worker only while the slot is building)
  std::deque<Request> queue;
  // the resident scene's load layout: set once per residency by a full
  // od_scene_set_loads; later requests only change the values
  bool loads_ready = false;
  bool trac_on = false;
};

struct Built {
  int sid;
  od_scene* scene;
  od_status st;
  std::string err;
};

}  // namespace

struct od_server {
  od_ctx* ctx = nullptr;
  od_server_config cfg{};
  long long budget = 0, used = 0;
  double bytes_per_tet = 2600.0;   // estimate of a newcomer's device bytes, raised to the largest seen
  std::vector<Slot> slots;
  long long next_ticket = 1, stamp = 0;
  clock_type::time_point t0;
  od_server_stats stats{};
  // admission workers, each with a context of its own
  std::vector<od_ctx*> wctx;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int> todo;           // slots to build (locked)
  std::vector<Built> done;        // built scenes not yet adopted (locked)
  bool stop = false;              // (locked)
  double worker_s = 0.0;          // (locked)
};

namespace {

double now_s(const od_server* sv) {
  return std::chrono::duration<double>(clock_type::now() - sv->t0).count();
}

// Builds slot sid's scene in context c: scene, integrator, restored state.
od_status build_scene(od_ctx* c, Slot& sl, od_scene** out) {
  od_scene* sc = nullptr;
  od_status st = od_scene_create(c, (int)(sl.X.size() / 3), sl.X.data(), (int)(sl.tets.size() / 4), sl.tets.data(),
                                 (int)(sl.facets.size() / 3), sl.facets.data(), (int)sl.cdofs.size(),
                                 sl.cdofs.empty() ? nullptr : sl.cdofs.data(), &sl.mat, &sc);
  if (st == OD_OK) st = od_integrator_setup(sc, &sl.integ);
  if (st == OD_OK && sl.has_blob) st = od_scene_load(sc, sl.blob.data(), sl.blob.size());
  if (st == OD_OK) st = od_ctx_synchronize(c);
  if (st != OD_OK) {
    od_scene_destroy(sc);
    return st;
  }
  *out = sc;
  return OD_OK;
}

void worker_main(od_server* sv, od_ctx* wctx) {
  for (;;) {
    int sid = -1;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv.wait(lk, [&] { return sv->stop || !sv->todo.empty(); });
      if (sv->stop) return;
      sid = sv->todo.front();
      sv->todo.pop_front();
    }
    const auto t = clock_type::now();
    Built b{sid, nullptr, OD_OK, std::string()};
    b.st = build_scene(wctx, sv->slots[sid], &b.scene);
    if (b.st != OD_OK) b.err = od_last_error();
    const double dt = std::chrono::duration<double>(clock_type::now() - t).count();
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->done.push_back(std::move(b));
    sv->worker_s += dt;
  }
}

// A scene built in another context moves to the server's: its stream work
// is finished (build_scene synchronised it) and every later call runs on the
// server's stream.
void adopt(od_server* sv, Slot& sl, od_scene* sc) {
  sc->s.ctx = &sv->ctx->c;
  sl.scene = sc;
  sl.state = Slot::kResident;
  sl.loads_ready = false;
  sl.has_blob = false;
  sl.blob.clear();
  sl.blob.shrink_to_fit();
  od_scene_info info{};
  if (od_scene_get_info(sc, &info) == OD_OK && info.device_bytes > 0) {
    sv->used += info.device_bytes - sl.bytes;
    sl.bytes = info.device_bytes;
  }
}

od_status evict(od_server* sv, Slot& sl) {
  size_t n = 0;
  OD_TRY(od_scene_save(sl.scene, nullptr, &n));
  sl.blob.resize(n);
  OD_TRY(od_scene_save(sl.scene, sl.blob.data(), &n));
  sl.has_blob = true;
  od_scene_destroy(sl.scene);
  sl.scene = nullptr;
  sl.state = Slot::kCold;
  sv->used -= sl.bytes;
  sv->stats.evictions++;
  return OD_OK;
}

// Evicts least-recently-used resident scenes outside `keep` until `need`
// more bytes fit the budget; false if it cannot.
od_status make_room(od_server* sv, long long need, const std::vector<char>& keep, bool* ok) {
  *ok = true;
  while (sv->used + need > sv->budget) {
    int victim = -1;
    for (int i = 0; i < (int)sv->slots.size(); i++) {
      const Slot& s = sv->slots[i];
      if (s.state != Slot::kResident || keep[i]) continue;
      if (victim < 0 || s.last_use < sv->slots[victim].last_use) victim = i;
    }
    if (victim < 0) {
      *ok = false;
      return OD_OK;
    }
    OD_TRY(evict(sv, sv->slots[victim]));
  }
  return OD_OK;
}

od_status collect_built(od_server* sv) {
  std::vector<Built> got;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    got.swap(sv->done);
  }
  od_status rc = OD_OK;
  for (Built& b : got) {
    Slot& sl = sv->slots[b.sid];
    if (b.st != OD_OK) {
      sl.state = Slot::kCold;
      sv->used -= sl.bytes;
      sl.bytes = 0;
      if (rc == OD_OK) {
        set_error("od_server: building scene " + std::to_string(b.sid) + " failed: " + b.err);
        rc = b.st;
      }
      continue;
    }
    if (sl.has_blob) sv->stats.restores++;
    adopt(sv, sl, b.scene);
    sv->stats.admissions++;
  }
  return rc;
}

// the request's time step and loads on its (resident) scene
od_status apply_request(Slot& sl, const od_step_request& r) {
  od_integrator_params p = sl.integ;
  p.dt = r.dt;
  OD_TRY(od_integrator_update(sl.scene, &p));
  const int nlf = (int)sl.load_facets.size();
  const bool trac = nlf > 0 && (r.traction[0] != 0.0 || r.traction[1] != 0.0 || r.traction[2] != 0.0);
  if (sl.loads_ready && sl.trac_on == trac)   // same facets: new values on the device only
    return scene_set_uniform_loads(&sl.scene->s, r.body, trac ? r.traction : nullptr);
  OD_TRY(od_scene_set_loads(sl.scene, r.body, trac ? 1 : 0, trac ? r.traction : nullptr, trac ? &nlf : nullptr,
                            trac ? sl.load_facets.data() : nullptr));
  sl.loads_ready = true;
  sl.trac_on = trac;
  return OD_OK;
}

}  // namespace

extern "C" {

od_status od_server_create(od_ctx* ctx, const od_server_config* cfg, od_server** out) {
  OD_CHECK_ARG(ctx && cfg && out, "od_server_create: NULL argument");
  OD_CHECK_ARG(cfg->max_batch >= 0, "od_server_create: max_batch must be >= 0");
  OD_CHECK_ARG(cfg->admission_thread >= 0 && cfg->admission_thread <= 64,
               "od_server_create: admission threads must be in 0..64");
  od_server* sv = new (std::nothrow) od_server();
  if (!sv) return OD_ERR_OUT_OF_MEMORY;
  sv->ctx = ctx;
  sv->cfg = *cfg;
  sv->t0 = clock_type::now();
  if (cfg->budget_bytes > 0) {
    sv->budget = cfg->budget_bytes;
  } else {
    size_t fr = 0, tot = 0;
    cudaSetDevice(ctx->c.device);
    cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) { delete sv; return cuda_fail(e, "cudaMemGetInfo"); }
    sv->budget = std::max(0LL, (long long)fr - std::max(0LL, cfg->reserve_bytes));
  }
  for (int k = 0; k < cfg->admission_thread; k++) {
    od_ctx* w = nullptr;
    od_status st = od_ctx_create(ctx->c.device, &w);
    if (st == OD_OK) {
      try {
        sv->workers.emplace_back(worker_main, sv, w);
        sv->wctx.push_back(w);
      } catch (...) {
        od_ctx_destroy(w);
        st = OD_ERR_INTERNAL;
        set_error("od_server_create: cannot start an admission thread");
      }
    }
    if (st != OD_OK) {
      od_server_destroy(sv);
      return st;
    }
  }
  *out = sv;
  return OD_OK;
}

od_status od_server_destroy(od_server* sv) {
  if (!sv) return OD_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv.notify_all();
  for (std::thread& t : sv->workers)
    if (t.joinable()) t.join();
  for (Built& b : sv->done) od_scene_destroy(b.scene);
  for (Slot& s : sv->slots) od_scene_destroy(s.scene);
  for (od_ctx* w : sv->wctx) od_ctx_destroy(w);
  delete sv;
  return OD_OK;
}

od_status od_server_add_scene(od_server* sv, const od_scene_spec* spec, int* scene_id) {
  OD_CHECK_ARG(sv && spec && scene_id, "od_server_add_scene: NULL argument");
  OD_CHECK_ARG(spec->n_nodes > 0 && spec->X && spec->n_tets > 0 && spec->tets,
               "od_server_add_scene: need nodes and elements");
  OD_CHECK_ARG(spec->n_facets >= 0 && (spec->n_facets == 0 || spec->facets), "od_server_add_scene: bad facets");
  OD_CHECK_ARG(spec->n_cdofs >= 0 && (spec->n_cdofs == 0 || spec->cdofs), "od_server_add_scene: bad constraints");
  OD_CHECK_ARG(spec->n_load_facets >= 0 && (spec->n_load_facets == 0 || spec->load_facets),
               "od_server_add_scene: bad load facets");
  OD_CHECK_ARG(spec->integrator.kind == OD_INTEGRATOR_NEWMARK, "od_server_add_scene: scenes step with Newmark");
  for (int k = 0; k < spec->n_load_facets; k++)
    OD_CHECK_ARG(spec->load_facets[k] >= 0 && spec->load_facets[k] < spec->n_facets,
                 "od_server_add_scene: load facet out of range");
  // the worker reads slots while building: registration only while no
  // scene is being built (the slot vector must not move)
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    OD_CHECK_ARG(sv->todo.empty(), "od_server_add_scene: register scenes before submitting requests");
  }
  for (const Slot& s : sv->slots)
    OD_CHECK_ARG(s.state != Slot::kBuilding, "od_server_add_scene: register scenes before submitting requests");
  Slot sl;
  sl.X.assign(spec->X, spec->X + 3 * (size_t)spec->n_nodes);
  sl.tets.assign(spec->tets, spec->tets + 4 * (size_t)spec->n_tets);
  if (spec->n_facets) sl.facets.assign(spec->facets, spec->facets + 3 * (size_t)spec->n_facets);
  if (spec->n_cdofs) sl.cdofs.assign(spec->cdofs, spec->cdofs + spec->n_cdofs);
  if (spec->n_load_facets) sl.load_facets.assign(spec->load_facets, spec->load_facets + spec->n_load_facets);
  sl.mat = spec->material;
  sl.integ = spec->integrator;
  sv->slots.push_back(std::move(sl));
  *scene_id = (int)sv->slots.size() - 1;
  return OD_OK;
}

od_status od_server_now(od_server* sv, double* t) {
  OD_CHECK_ARG(sv && t, "od_server_now: NULL argument");
  *t = now_s(sv);
  return OD_OK;
}

od_status od_server_submit(od_server* sv, const od_step_request* req, long long* ticket) {
  OD_CHECK_ARG(sv && req, "od_server_submit: NULL argument");
  OD_CHECK_ARG(req->scene >= 0 && req->scene < (int)sv->slots.size(), "od_server_submit: no such scene");
  OD_CHECK_ARG(req->dt > 0.0, "od_server_submit: dt must be positive");
  Request r{sv->next_ticket++, *req};
  sv->slots[req->scene].queue.push_back(r);
  if (ticket) *ticket = r.ticket;
  return OD_OK;
}

od_status od_server_pending(od_server* sv, long long* pending) {
  OD_CHECK_ARG(sv && pending, "od_server_pending: NULL argument");
  long long n = 0;
  for (const Slot& s : sv->slots) n += (long long)s.queue.size();
  *pending = n;
  return OD_OK;
}

od_status od_server_warm(od_server* sv, int n, const int* scene_ids, int* admitted) {
  OD_CHECK_ARG(sv && admitted && (n == 0 || scene_ids), "od_server_warm: NULL argument");
  *admitted = 0;
  for (int k = 0; k < n; k++) {
    const int sid = scene_ids[k];
    OD_CHECK_ARG(sid >= 0 && sid < (int)sv->slots.size(), "od_server_warm: no such scene");
    Slot& sl = sv->slots[sid];
    if (sl.state != Slot::kCold) continue;
    const long long est = (long long)(sv->bytes_per_tet * (double)(sl.tets.size() / 4));
    if (sv->used + est > sv->budget) break;
    od_scene* sc = nullptr;
    sl.bytes = est;
    sv->used += est;
    od_status st = build_scene(sv->ctx, sl, &sc);
    if (st != OD_OK) {
      sv->used -= est;
      sl.bytes = 0;
      return st;
    }
    adopt(sv, sl, sc);
    sl.last_use = ++sv->stamp;
    sv->stats.admissions++;
    (*admitted)++;
  }
  return OD_OK;
}

od_status od_server_tick(od_server* sv, int capacity, od_step_result* results, int* n_results) {
  OD_CHECK_ARG(sv && n_results && (capacity == 0 || results), "od_server_tick: NULL argument");
  *n_results = 0;
  const auto tk0 = clock_type::now();
  OD_TRY(collect_built(sv));
  const double now = now_s(sv);
  // heads: oldest pending request of every scene that has one, oldest first
  std::vector<std::pair<double, int>> heads;
  for (int i = 0; i < (int)sv->slots.size(); i++) {
    const Slot& s = sv->slots[i];
    if (!s.queue.empty() && s.queue.front().r.arrival <= now) heads.push_back({s.queue.front().r.arrival, i});
  }
  std::sort(heads.begin(), heads.end());
  int limit = (int)heads.size();
  if (sv->cfg.max_batch > 0) limit = std::min(limit, sv->cfg.max_batch);
  limit = std::min(limit, capacity);
  std::vector<char> keep(sv->slots.size(), 0);
  for (int k = 0; k < limit; k++) keep[heads[k].second] = 1;
  // admission: newcomers go to the worker (or are built here)
  std::vector<int> step_ids;
  for (int k = 0; k < limit; k++) {
    const int sid = heads[k].second;
    Slot& sl = sv->slots[sid];
    if (sl.state == Slot::kResident) {
      step_ids.push_back(sid);
      continue;
    }
    if (sl.state == Slot::kBuilding) continue;
    const long long est = (long long)(sv->bytes_per_tet * (double)(sl.tets.size() / 4));
    bool ok = false;
    OD_TRY(make_room(sv, est, keep, &ok));
    if (!ok) {
      sv->stats.deferred++;
      continue;
    }
    sl.bytes = est;
    sv->used += est;
    if (!sv->workers.empty()) {
      sl.state = Slot::kBuilding;
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->todo.push_back(sid);
      }
      sv->cv.notify_one();
    } else {
      od_scene* sc = nullptr;
      od_status st = build_scene(sv->ctx, sl, &sc);
      if (st != OD_OK) {
        sv->used -= est;
        sl.bytes = 0;
        return st;
      }
      if (sl.has_blob) sv->stats.restores++;
      adopt(sv, sl, sc);
      sv->stats.admissions++;
      step_ids.push_back(sid);
    }
  }
  const auto tk1 = clock_type::now();
  sv->stats.s_admit += std::chrono::duration<double>(tk1 - tk0).count();
  if (step_ids.empty()) return OD_OK;
  // the requests' parameters and loads
  std::vector<Request> reqs;
  std::vector<od_scene*> scenes;
  for (int sid : step_ids) {
    Slot& sl = sv->slots[sid];
    reqs.push_back(sl.queue.front());
    sl.queue.pop_front();
    OD_TRY(apply_request(sl, reqs.back().r));
    scenes.push_back(sl.scene);
    sl.last_use = ++sv->stamp;
  }
  const auto tk2 = clock_type::now();
  sv->stats.s_loads += std::chrono::duration<double>(tk2 - tk1).count();
  std::vector<od_step_stats> st(scenes.size());
  od_status fail = OD_OK;   // a step that failed as a call: its requests come back with that status
  if (sv->cfg.batched) {
    od_batch* b = nullptr;
    const auto tb0 = clock_type::now();
    fail = od_batch_create(sv->ctx, (int)scenes.size(), scenes.data(), &b);
    const auto tb1 = clock_type::now();
    if (fail == OD_OK) {
      fail = od_batch_step(b, 1, st.data());
      const auto tb2 = clock_type::now();
      od_batch_destroy(b);
      sv->stats.s_build += std::chrono::duration<double>(clock_type::now() - tb2).count();
    }
    sv->stats.s_build += std::chrono::duration<double>(tb1 - tb0).count();
  } else {
    for (size_t k = 0; k < scenes.size() && fail == OD_OK; k++) {
      const od_status rc = od_step(scenes[k], 1, &st[k]);
      if (rc != OD_OK && rc != OD_ERR_NOT_CONVERGED && rc != OD_ERR_NAN) fail = rc;
      else if (rc != OD_OK && st[k].status == OD_OK) st[k].status = rc;
    }
  }
  if (fail != OD_OK) {
    const std::string why = od_last_error();
    for (size_t k = 0; k < reqs.size(); k++) {
      od_step_result& r = results[k];
      r.ticket = reqs[k].ticket;
      r.scene = reqs[k].r.scene;
      r.status = fail;
      r.pcg_iterations = 0;
      r.arrival = reqs[k].r.arrival;
      r.done = now_s(sv);
    }
    *n_results = (int)reqs.size();
    set_error("od_server_tick: " + why);
    return fail;
  }
  const auto tk3 = clock_type::now();
  sv->stats.s_step += std::chrono::duration<double>(tk3 - tk2).count();
  if (sv->cfg.batched) {
    if (!st.empty()) sv->stats.s_device += 1e-3 * st[0].device_ms;   // one event pair around the batch step
  } else {
    for (const od_step_stats& x : st) sv->stats.s_device += 1e-3 * x.device_ms;
  }
  const double t_done = now_s(sv);
  for (size_t k = 0; k < reqs.size(); k++) {
    od_step_result& r = results[k];
    r.ticket = reqs[k].ticket;
    r.scene = reqs[k].r.scene;
    r.status = st[k].status;
    r.pcg_iterations = st[k].pcg_iterations;
    r.arrival = reqs[k].r.arrival;
    r.done = t_done;
  }
  *n_results = (int)reqs.size();
  // device bytes now include each scene's FP32 system: correct the budget
  for (int sid : step_ids) {
    Slot& sl = sv->slots[sid];
    od_scene_info info{};
    if (od_scene_get_info(sl.scene, &info) == OD_OK && info.device_bytes > 0) {
      sv->used += info.device_bytes - sl.bytes;
      sl.bytes = info.device_bytes;
      sv->bytes_per_tet = std::max(sv->bytes_per_tet, (double)info.device_bytes / (double)(sl.tets.size() / 4));
    }
  }
  bool ok = true;
  OD_TRY(make_room(sv, 0, std::vector<char>(sv->slots.size(), 0), &ok));   // an estimate fell short
  sv->stats.ticks++;
  sv->stats.steps += (long long)reqs.size();
  return OD_OK;
}

od_status od_server_get_scene(od_server* sv, int scene_id, od_scene** out) {
  OD_CHECK_ARG(sv && out, "od_server_get_scene: NULL argument");
  OD_CHECK_ARG(scene_id >= 0 && scene_id < (int)sv->slots.size(), "od_server_get_scene: no such scene");
  Slot& sl = sv->slots[scene_id];
  while (sl.state == Slot::kBuilding) {   // wait for the worker's copy
    OD_TRY(collect_built(sv));
    if (sl.state == Slot::kBuilding) std::this_thread::sleep_for(std::chrono::milliseconds(1));
  }
  if (sl.state == Slot::kCold) {
    std::vector<char> keep(sv->slots.size(), 0);
    keep[scene_id] = 1;
    const long long est = (long long)(sv->bytes_per_tet * (double)(sl.tets.size() / 4));
    bool ok = false;
    OD_TRY(make_room(sv, est, keep, &ok));
    if (!ok) {
      set_error("od_server_get_scene: the scene does not fit the budget");
      return OD_ERR_OUT_OF_MEMORY;
    }
    od_scene* sc = nullptr;
    sl.bytes = est;
    sv->used += est;
    od_status st = build_scene(sv->ctx, sl, &sc);
    if (st != OD_OK) {
      sv->used -= est;
      sl.bytes = 0;
      return st;
    }
    if (sl.has_blob) sv->stats.restores++;
    adopt(sv, sl, sc);
    sv->stats.admissions++;
  }
  sl.last_use = ++sv->stamp;
  *out = sl.scene;
  return OD_OK;
}

od_status od_server_get_stats(od_server* sv, od_server_stats* out) {
  OD_CHECK_ARG(sv && out, "od_server_get_stats: NULL argument");
  *out = sv->stats;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    out->s_worker = sv->worker_s;
  }
  long long n = 0;
  for (const Slot& s : sv->slots) n += s.state == Slot::kResident ? 1 : 0;
  out->resident = n;
  out->resident_bytes = sv->used;
  out->budget_bytes = sv->budget;
  return OD_OK;
}

}  // extern "C"
