// lbm_server.cu - a request loop that keeps many solves resident on one GPU
// and advances them together (continuous batching).  No counterpart in the
// reference, which runs one box per MPI job.
//
// A request names a box (grid, wall axis, particles, precision), its seeded
// initial state and a number of steps.  One host thread (started by
// lbm_server_create) runs the loop:
//
//   admit    queued requests, first come first served with skip-ahead over
//            requests that do not fit, while the HBM budget (lbm_footprint of
//            every resident context) and the slot count allow; each gets its
//            own context, initial field (lbm_init_spectral) and particles
//            (lbm_init_particles) on its own stream;
//   group    resident FP32 boxes that a batch can hold and that are at the
//            same step phase into lbm_batches (rebuilt when membership
//            changes); others step on their own streams;
//   advance  every group and every standalone box by one chunk of steps
//            (even, so that boxes admitted later meet the batch at phase 0;
//            a box with an odd number of steps takes its last step alone);
//   retire   finished boxes: a deterministic summary of the final state
//            (lbm_summary), then the context is destroyed and its HBM
//            returned.
//
// A box's arithmetic does not depend on which other boxes share its batch or
// on how its steps are cut into chunks, so a request gives the same bits
// alone and in any mix.  Walls normal to y or z are served by relabelling
// the axes so that the wall axis is the engine's x (the reference channel's
// wall axis, C/streaming.f90:175-187); the summary's momentum is mapped back.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lbm_internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

// batches stepped side by side on their own streams (regroup)
constexpr int kConcurrent = 3;

struct Job {
  int64_t id = 0;
  lbm_request req{};
  lbm_result res{};
  lbm_ctx* ctx = nullptr;
  uint64_t bytes = 0;
  int remaining = 0;
  bool batchable = false;
  int internal_axis[3] = {0, 1, 2};  // external axis of internal x, y, z
  lbm_ctx* kept = nullptr;           // finished context held for lbm_server_take
};

}  // namespace

struct lbm_server {
  uint64_t budget = 0, used = 0;
  int max_active = 0, chunk = 0;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  std::vector<Job*> active;
  int64_t next_id = 1;
  bool stop = false;
  std::thread loop;
  // loop-thread state
  std::vector<lbm_batch*> batches;
  std::vector<std::vector<Job*>> batch_members;
  bool membership_changed = true;
  int64_t rebuilds = 0, chunks = 0, done = 0, failed = 0;
  double busy_s = 0.0;
  // loop-thread seconds spent admitting (context set-up), regrouping and
  // retiring (summary and context destruction)
  double admit_s = 0.0, regroup_s = 0.0, retire_s = 0.0;
};

namespace {

double now_s(const lbm_server* s) {
  return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

// engine config for a request: the wall axis becomes the engine's x
bool make_config(const lbm_request& r, lbm_config* cfg, int axis_of[3]) {
  const int ext[3] = {r.nx, r.ny, r.nz};
  int order[3] = {0, 1, 2};
  if (r.wall_axis == 1) { order[0] = 1; order[1] = 0; order[2] = 2; }
  if (r.wall_axis == 2) { order[0] = 2; order[1] = 0; order[2] = 1; }
  for (int i = 0; i < 3; ++i) axis_of[i] = order[i];
  const int preset = r.wall_axis >= 0 ? LBM_PRESET_CHANNEL : LBM_PRESET_BOX;
  if (lbm_config_init(cfg, preset, ext[order[0]], ext[order[1]], ext[order[2]], r.npart, r.rad,
                      r.rhopart) != LBM_OK)
    return false;
  cfg->precision = r.precision;
  if (r.mrt_type > 0) cfg->mrt_type = r.mrt_type;
  return true;
}

void finish(lbm_server* s, Job* j, int err) {
  if (err == LBM_OK) {
    double out[6];
    err = lbm_summary(j->ctx, out);
    if (err == LBM_OK) {
      j->res.summary[0] = out[0];
      for (int i = 0; i < 3; ++i) j->res.summary[1 + j->internal_axis[i]] = out[1 + i];
      j->res.summary[4] = out[4];
      j->res.summary[5] = out[5];
    }
  }
  const bool keep = err == LBM_OK && j->req.keep_state;
  if (keep)
    j->kept = j->ctx;  // stays resident (and counted) until taken
  else
    lbm_destroy(j->ctx);
  j->ctx = nullptr;
  std::lock_guard<std::mutex> lk(s->mu);
  if (!keep) s->used -= j->bytes;
  j->res.t_done = now_s(s);
  j->res.state = err == LBM_OK ? LBM_REQ_DONE : LBM_REQ_FAILED;
  j->res.error = err;
  if (err == LBM_OK) ++s->done; else ++s->failed;
  s->active.erase(std::find(s->active.begin(), s->active.end(), j));
  s->membership_changed = true;
  s->cv_done.notify_all();
}

// create and initialise the context of an admitted job (loop thread)
int start_job(lbm_server* s, Job* j) {
  lbm_config cfg;
  if (!make_config(j->req, &cfg, j->internal_axis)) return LBM_ERR_ARG;
  int rc = lbm_create(&cfg, &j->ctx);
  if (rc) return rc;
  if ((rc = lbm_init_spectral(j->ctx, j->req.k0, j->req.u_rms, j->req.seed))) return rc;
  if ((rc = lbm_macrovar(j->ctx))) return rc;
  if (j->req.npart > 0 &&
      (rc = lbm_init_particles(j->ctx, j->req.npart, (int)(j->req.seed % 2147483646ull) + 1, 0)))
    return rc;
  if ((rc = lbm_synchronize(j->ctx))) return rc;
  // stochastic forcing rotates its tables with the step count, so boxes
  // admitted at different steps could not share a batch's step phase: they
  // step alone (concurrently, each on its own stream)
  j->batchable = cfg.precision == LBM_PREC_F32 && cfg.nx % 4 == 0 && cfg.nx <= 128 &&
                 cfg.forcing != LBM_FORCING_STOCHASTIC;
  j->remaining = j->req.nsteps;
  return LBM_OK;
}

double secs_since(Clock::time_point t) {
  return std::chrono::duration<double>(Clock::now() - t).count();
}

void admit(lbm_server* s) {
  const auto t0 = Clock::now();
  struct Tally {
    lbm_server* s;
    Clock::time_point t0;
    ~Tally() { s->admit_s += secs_since(t0); }
  } tally{s, t0};
  std::vector<Job*> take;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    int looked = 0;
    for (auto it = s->queue.begin(); it != s->queue.end() && looked < 64;) {
      if ((int)(s->active.size() + take.size()) >= s->max_active) break;
      Job* j = s->jobs[*it].get();
      ++looked;
      if (s->used + j->bytes <= s->budget) {
        s->used += j->bytes;
        take.push_back(j);
        it = s->queue.erase(it);
      } else {
        ++it;
      }
    }
  }
  for (Job* j : take) {
    j->res.t_start = now_s(s);
    j->res.state = LBM_REQ_RUNNING;
    const int rc = start_job(s, j);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->active.push_back(j);
      s->membership_changed = true;
    }
    if (rc) finish(s, j, rc);
  }
}

// batches of phase-compatible FP32 boxes; everything else steps alone
void regroup(lbm_server* s) {
  const auto t0 = Clock::now();
  for (lbm_batch* b : s->batches) lbm_batch_destroy(b);
  s->batches.clear();
  s->batch_members.clear();
  std::vector<Job*> cand;
  for (Job* j : s->active)
    if (j->batchable && j->remaining >= 2 && j->res.steps_done % 2 == 0) cand.push_back(j);
  // group by boundary and forcing kind (all are at phase 0 at a chunk
  // boundary: admitted at phase 0, advanced by even chunks)
  std::map<std::pair<int, int>, std::vector<Job*>> groups;
  for (Job* j : cand) {
    const int wall = j->req.wall_axis >= 0 ? 1 : 0;
    groups[{wall, 0}].push_back(j);
  }
  for (auto& kv : groups) {
    // up to kConcurrent batches of about equal node counts per group: each
    // batch has its own stream, so one batch's particle kernels overlap
    // another's stream + collide kernel
    std::vector<Job*> jobs = kv.second;
    std::sort(jobs.begin(), jobs.end(), [](const Job* a, const Job* b) {
      return (int64_t)a->req.nx * a->req.ny * a->req.nz > (int64_t)b->req.nx * b->req.ny * b->req.nz;
    });
    const int parts = std::max(1, std::min<int>(kConcurrent, (int)jobs.size() / 2));
    std::vector<std::vector<Job*>> part(parts);
    std::vector<int64_t> load(parts, 0);
    for (Job* j : jobs) {
      const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      part[g].push_back(j);
      load[g] += (int64_t)j->req.nx * j->req.ny * j->req.nz;
    }
    for (auto& members : part) {
      if (members.empty()) continue;
      std::vector<lbm_ctx*> ctxs;
      for (Job* j : members) ctxs.push_back(j->ctx);
      lbm_batch* b = nullptr;
      if (lbm_batch_create(ctxs.data(), (int)ctxs.size(), &b) == LBM_OK) {
        s->batches.push_back(b);
        s->batch_members.push_back(members);
      } else {
        for (Job* j : members) j->batchable = false;
      }
    }
  }
  ++s->rebuilds;
  s->membership_changed = false;
  s->regroup_s += secs_since(t0);
}

void advance(lbm_server* s) {
  // chunk: even, at most the smallest even remainder of a batched box
  int k = s->chunk;
  bool any_batched = false;
  for (auto& m : s->batch_members)
    for (Job* j : m) {
      any_batched = true;
      k = std::min(k, j->remaining & ~1);
    }
  if (!any_batched) k = s->chunk;
  if (k < 2) k = 2;
  std::vector<Job*> solo;
  for (Job* j : s->active) {
    bool in = false;
    for (auto& m : s->batch_members) in |= std::find(m.begin(), m.end(), j) != m.end();
    if (!in) solo.push_back(j);
  }
  const size_t resident_before = s->active.size();
  const auto w0 = Clock::now();
  std::vector<int> batch_rc(s->batches.size());
  for (size_t g = 0; g < s->batches.size(); ++g)
    batch_rc[g] = lbm_batch_step(s->batches[g], k, k >= 12 ? 1 : 0);
  std::vector<int> solo_steps(solo.size()), solo_rc(solo.size());
  for (size_t i = 0; i < solo.size(); ++i) {
    solo_steps[i] = std::min(k, solo[i]->remaining);
    solo_rc[i] = lbm_step(solo[i]->ctx, solo_steps[i]);
  }
  // while the chunk runs, bring in new requests (their set-up runs on
  // their own streams); they join at the next regrouping
  admit(s);
  std::vector<std::pair<Job*, int>> finished;
  for (size_t g = 0; g < s->batches.size(); ++g) {
    const int rcw = lbm_batch_wait(s->batches[g]);
    const int rcb = batch_rc[g] ? batch_rc[g] : rcw;
    for (Job* j : s->batch_members[g]) {
      // each box's own errors (a particle overlap, ...) end only that box
      const int rc = rcb ? rcb : lbm_synchronize(j->ctx);
      j->remaining -= k;
      j->res.steps_done += k;
      j->res.batched = 1;
      if (rc) finished.push_back({j, rc});
      else if (j->remaining <= 1) s->membership_changed = true;  // leaves the batch
    }
  }
  for (size_t i = 0; i < solo.size(); ++i) {
    const int rcs = lbm_synchronize(solo[i]->ctx);
    const int rc = solo_rc[i] ? solo_rc[i] : rcs;
    solo[i]->remaining -= solo_steps[i];
    solo[i]->res.steps_done += solo_steps[i];
    if (rc) finished.push_back({solo[i], rc});
  }
  s->busy_s += std::chrono::duration<double>(Clock::now() - w0).count();
  ++s->chunks;
  std::vector<Job*> done;
  for (size_t i = 0; i < resident_before && i < s->active.size(); ++i)
    if (s->active[i]->remaining <= 0) done.push_back(s->active[i]);
  const auto t_retire = Clock::now();
  if (!done.empty() || !finished.empty()) {
    // a finished box leaves its batch before its context goes away
    for (lbm_batch* b : s->batches) lbm_batch_destroy(b);
    s->batches.clear();
    s->batch_members.clear();
    s->membership_changed = true;
  }
  for (auto& f : finished)
    if (std::find(done.begin(), done.end(), f.first) == done.end()) finish(s, f.first, f.second);
  for (Job* j : done) {
    bool failed = false;
    for (auto& f : finished) failed |= f.first == j;
    if (!failed) finish(s, j, LBM_OK);
  }
  s->retire_s += secs_since(t_retire);
}

void run_loop(lbm_server* s) {
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] {
        return s->stop || !s->queue.empty() || !s->active.empty();
      });
      if (s->stop) break;
    }
    admit(s);
    bool have;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      have = !s->active.empty();
    }
    if (!have) continue;
    if (s->membership_changed) regroup(s);
    advance(s);
  }
  for (lbm_batch* b : s->batches) lbm_batch_destroy(b);
  s->batches.clear();
  for (Job* j : std::vector<Job*>(s->active)) finish(s, j, LBM_ERR_STATE);
}

}  // namespace

extern "C" {

int lbm_server_create(uint64_t hbm_budget, int max_active, int chunk_steps, lbm_server** out) {
  if (!out || hbm_budget == 0 || max_active < 1 || chunk_steps < 2) return LBM_ERR_ARG;
  lbm_server* s = new lbm_server();
  s->budget = hbm_budget;
  s->max_active = max_active;
  s->chunk = chunk_steps & ~1;
  s->t0 = Clock::now();
  s->loop = std::thread(run_loop, s);
  *out = s;
  return LBM_OK;
}

int lbm_server_submit(lbm_server* s, const lbm_request* r, int64_t* id) {
  if (!s || !r || !id) return LBM_ERR_ARG;
  if (r->nx < 8 || r->ny < 8 || r->nz < 8 || r->wall_axis < -1 || r->wall_axis > 2 ||
      r->nsteps < 1 || r->npart < 0 || r->mrt_type < 0 || r->mrt_type > 3 ||
      (r->precision != LBM_PREC_F32 && r->precision != LBM_PREC_F64))
    return LBM_ERR_ARG;
  auto j = std::make_unique<Job>();
  j->req = *r;
  lbm_config cfg;
  if (!make_config(*r, &cfg, j->internal_axis)) return LBM_ERR_ARG;
  if (lbm_footprint(&cfg, &j->bytes) != LBM_OK) return LBM_ERR_ARG;
  // statistics and initial-field scratch are transient; keep headroom for the latter
  j->bytes += (uint64_t)cfg.nx * cfg.ny * cfg.nz * 3 * 8 * 2;
  std::lock_guard<std::mutex> lk(s->mu);
  if (j->bytes > s->budget) return LBM_ERR_NOMEM;
  j->id = s->next_id++;
  j->res.id = j->id;
  j->res.state = LBM_REQ_QUEUED;
  j->res.t_submit = now_s(s);
  *id = j->id;
  s->queue.push_back(j->id);
  s->jobs[j->id] = std::move(j);
  s->cv_work.notify_all();
  return LBM_OK;
}

int lbm_server_result(lbm_server* s, int64_t id, lbm_result* out) {
  if (!s || !out) return LBM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return LBM_ERR_ARG;
  *out = it->second->res;
  return LBM_OK;
}

int lbm_server_wait(lbm_server* s, int64_t id, double timeout_s) {
  if (!s) return LBM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return LBM_ERR_ARG;
  Job* j = it->second.get();
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    return j->res.state == LBM_REQ_DONE || j->res.state == LBM_REQ_FAILED;
  });
  return ok ? LBM_OK : LBM_ERR_TIMEOUT;
}

int lbm_server_stats(lbm_server* s, double* out) {
  if (!s || !out) return LBM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = (double)(s->next_id - 1);
  out[1] = (double)s->done;
  out[2] = (double)s->failed;
  out[3] = (double)s->active.size();
  out[4] = (double)s->queue.size();
  out[5] = (double)s->used;
  out[6] = (double)s->rebuilds;
  out[7] = (double)s->chunks;
  out[8] = s->busy_s;
  out[10] = s->admit_s;
  out[11] = s->regroup_s;
  out[12] = s->retire_s;
  out[9] = now_s(s);
  return LBM_OK;
}

int lbm_server_take(lbm_server* s, int64_t id, lbm_ctx** out) {
  if (!s || !out) return LBM_ERR_ARG;
  *out = nullptr;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return LBM_ERR_ARG;
  Job* j = it->second.get();
  if (j->res.state != LBM_REQ_DONE || !j->kept) return LBM_ERR_STATE;
  *out = j->kept;
  j->kept = nullptr;
  s->used -= j->bytes;
  s->cv_work.notify_all();
  return LBM_OK;
}

int lbm_server_destroy(lbm_server* s) {
  if (!s) return LBM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->loop.joinable()) s->loop.join();
  for (auto& kv : s->jobs)
    if (kv.second->kept) lbm_destroy(kv.second->kept);
  delete s;
  return LBM_OK;
}

}  // extern "C"
