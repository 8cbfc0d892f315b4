// mpm_serve.cu -- serving runtime over the batched step (C ABI in
// include/mpm3d_gpu.h, mpm_serve_*).
//
// One server thread owns the device batch. Client threads only touch the
// ticket table and the submission queue under the server mutex; staging a
// scene (deck -> host set-up and input copy) runs on the client thread.
//
// Server loop:
//   1. admit queued scenes -- in submission order, or least work first --
//      while the estimated device bytes of the resident scenes stay within the
//      budget (and their particles within the optional cap);
//   2. hand the batch to the device loop (mpm_batch_run_loop): one graph
//      launch in which the device repeats steps until a resident scene takes
//      its last step or, once chunk_steps steps are taken, a submission has
//      raised the batch's interrupt flag (a page-locked word the device reads
//      once per two steps);
//   3. read every resident scene's progress in one copy, snapshot the fields
//      of the finished ones, retire them and wake their waiters.
// The launch shape autotuner times every candidate (particle block, node
// block, scatter blocks per SM) on one frozen composition -- the first whose
// scenes all have the steps for the sweep left -- two rounds in opposite
// orders (a launch shape changes no result), and keeps the fastest per
// particle-step.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mpm3d_gpu.h"
#include "mpm_batch_host.h"

using mpm::BatchProgress;
using mpm::HostScene;

namespace {

using Clock = std::chrono::steady_clock;

// steps a device loop may take at most (it ends earlier when a scene
// finishes or, after chunk_steps steps, when a submission arrives)
constexpr int kLoopBudget = 1 << 20;

double ms_since(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

enum TicketState { T_QUEUED, T_RESIDENT, T_DONE, T_FAILED };

struct Ticket {
  int64_t id = 0;
  TicketState state = T_QUEUED;
  int code = MPM_OK;
  std::string err;
  HostScene* scene = nullptr;  // owned while queued
  long long bytes = 0, np = 0;
  int steps = 0;
  uint32_t mask = 0;
  int scene_id = -1;
  Clock::time_point t_submit, t_admit, t_done;
  double scalars[MPM_NSCALARS] = {};
  std::map<int, std::vector<double>> fields;
};

struct Tune {
  int pb, nb, sb;           // particle block, node block, scatter blocks per SM
  double ms = 0, work = 0;  // accumulated time and particle-steps
};

}  // namespace

struct mpm_server {
  mpm_serve_config cfg{};
  mpm_batch* batch = nullptr;
  std::thread thr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::deque<int64_t> queue;
  std::map<int64_t, Ticket*> tickets;
  std::map<int, int64_t> by_scene;  // resident scene id -> ticket
  int64_t next_ticket = 1;
  long long resident_bytes = 0, peak_bytes = 0, resident_particles = 0;
  // statistics
  long long submitted = 0, finished = 0, chunks = 0;
  double particle_steps = 0, busy_ms = 0;
  int pb = 256, nb = 256, sb = 64;
  std::vector<Tune> tune;
  bool tuned = false;
  std::string err;
};

namespace {

int serr(mpm_server* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return code;
}

// fail every ticket that is resident (after a batch error) -- caller holds mu
void fail_resident(mpm_server* s, int code, const std::string& msg) {
  for (auto& kv : s->by_scene) {
    auto it = s->tickets.find(kv.second);
    if (it == s->tickets.end()) continue;
    Ticket* t = it->second;
    t->state = T_FAILED;
    t->code = code;
    t->err = msg;
    t->t_done = Clock::now();
  }
  s->by_scene.clear();
  s->resident_bytes = 0;
  s->resident_particles = 0;
}

// The admission decision (see mpm_serve_plan). Candidates are taken in
// submission order (FIFO) or least work (particles x steps, ties by
// submission order) first; admission stops at the first candidate that does
// not fit the scene cap, the particle cap (a lone scene is always admitted)
// or the byte budget. With nothing resident, a candidate over the byte budget
// can never run: it is rejected and the next one is tried.
int serve_plan(const mpm_serve_config& cfg, int n, const int64_t* np, const int* steps, const int64_t* bytes,
               int rs, int64_t rp, int64_t rb, int* admit, int* reject, int* nreject) {
  std::vector<char> taken((size_t)n, 0);
  int na = 0, nr = 0;
  const int max_scenes = cfg.max_scenes > 0 ? cfg.max_scenes : 4096;
  for (;;) {
    int pick = -1;
    for (int k = 0; k < n; ++k) {
      if (taken[k]) continue;
      if (pick < 0) {
        pick = k;
        if (cfg.policy != MPM_SERVE_SHORTEST) break;
        continue;
      }
      if ((double)np[k] * steps[k] < (double)np[pick] * steps[pick]) pick = k;
    }
    if (pick < 0) break;
    if (rs >= max_scenes) break;
    if (cfg.max_resident_particles > 0 && rs > 0 && rp + np[pick] > cfg.max_resident_particles) break;
    if (cfg.hbm_budget_bytes > 0 && rb + bytes[pick] > cfg.hbm_budget_bytes) {
      if (rs > 0) break;
      taken[pick] = 1;
      reject[nr++] = pick;
      continue;
    }
    taken[pick] = 1;
    admit[na++] = pick;
    rs += 1;
    rp += np[pick];
    rb += bytes[pick];
  }
  *nreject = nr;
  return na;
}

void serve_loop(mpm_server* s) {
  cudaSetDevice(s->cfg.device);
  std::vector<BatchProgress> prog;
  std::vector<int> retire;
  for (;;) {
    // 1. admission (under the lock: the queue and tickets are shared)
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        if (s->stop) return;
        if (!s->queue.empty()) {
          const int nq = (int)s->queue.size();
          std::vector<int64_t> qnp(nq), qbytes(nq);
          std::vector<int> qsteps(nq), admit(nq), reject(nq);
          std::vector<int64_t> ids(s->queue.begin(), s->queue.end());
          for (int k = 0; k < nq; ++k) {
            const Ticket* t = s->tickets[ids[k]];
            qnp[k] = t->np;
            qsteps[k] = t->steps;
            qbytes[k] = t->bytes;
          }
          int nrej = 0;
          const int nadm = serve_plan(s->cfg, nq, qnp.data(), qsteps.data(), qbytes.data(), (int)s->by_scene.size(),
                                      s->resident_particles, s->resident_bytes, admit.data(), reject.data(), &nrej);
          for (int k = 0; k < nrej; ++k) {  // can never fit: fail them rather than block the queue
            Ticket* t = s->tickets[ids[reject[k]]];
            t->state = T_FAILED;
            t->code = MPM_ERR_OOM;
            t->err = "scene needs more device memory than the serving budget";
            t->t_done = Clock::now();
            delete t->scene;
            t->scene = nullptr;
          }
          for (int k = 0; k < nadm; ++k) {
            Ticket* t = s->tickets[ids[admit[k]]];
            int id = -1;
            mpm::batch_insert(s->batch, t->scene, &id);
            t->scene = nullptr;  // the batch owns it now
            t->scene_id = id;
            t->state = T_RESIDENT;
            t->t_admit = Clock::now();
            s->by_scene[id] = t->id;
            s->resident_bytes += t->bytes;
            s->resident_particles += t->np;
            s->peak_bytes = std::max(s->peak_bytes, s->resident_bytes);
          }
          if (nadm || nrej) {
            std::vector<char> gone(nq, 0);
            for (int k = 0; k < nadm; ++k) gone[admit[k]] = 1;
            for (int k = 0; k < nrej; ++k) gone[reject[k]] = 1;
            s->queue.clear();
            for (int k = 0; k < nq; ++k)
              if (!gone[k]) s->queue.push_back(ids[k]);
            if (nrej) s->cv_done.notify_all();
          }
        }
        if (!s->by_scene.empty()) break;
        s->cv_work.wait(lk);
      }
    }
    // 2. the device loop (server thread only touches the batch): the device
    // steps the batch until a resident scene takes its last step, the step
    // budget is spent, or a submission interrupts it
    int r = mpm_batch_commit(s->batch);
    std::vector<BatchProgress> before;
    if (r == MPM_OK) r = mpm::batch_progress(s->batch, before);
    auto work_since = [&](const std::vector<BatchProgress>& a, const std::vector<BatchProgress>& b2) {
      double w = 0;  // particle-steps taken between two progress reads (parked scenes take none)
      for (const BatchProgress& q : b2)
        for (const BatchProgress& p0 : a)
          if (p0.id == q.id) w += (double)q.np * std::max(0, q.istep - p0.istep);
      return w;
    };
    if (r == MPM_OK && s->cfg.autotune && !s->tuned) {
      // every candidate timed on this one composition (no admission or
      // retirement between the trials), two rounds in opposite orders; only
      // when every resident scene has the steps for the whole sweep left
      const int per = 2;
      int left = 1 << 30;
      for (const BatchProgress& q : before) left = std::min(left, q.target - q.istep);
      if (left >= (int)(2 * per * s->tune.size() + 1)) {
        for (int round = 0; round < 2 && r == MPM_OK; ++round)
          for (size_t n = 0; n < s->tune.size() && r == MPM_OK; ++n) {
            Tune& c = s->tune[round ? s->tune.size() - 1 - n : n];
            r = mpm_batch_set_blocks(s->batch, c.pb, c.nb);
            if (r == MPM_OK) r = mpm_batch_set_option(s->batch, MPM_BATCH_SCATTER_BLOCKS, c.sb);
            std::vector<BatchProgress> a, z;
            if (r == MPM_OK) r = mpm::batch_progress(s->batch, a);
            double tms = 0;
            if (r == MPM_OK) r = mpm_batch_time_steps(s->batch, per, 1, &tms);
            if (r == MPM_OK) r = mpm::batch_progress(s->batch, z);
            if (r == MPM_OK) {
              const double w = work_since(a, z);
              c.ms += tms;
              c.work += w;
              std::lock_guard<std::mutex> lk(s->mu);
              s->particle_steps += w;
              s->busy_ms += tms;
            }
          }
        if (r == MPM_OK) {
          const Tune* best = &s->tune[0];
          for (auto& c : s->tune)
            if (c.work > 0 && (best->work <= 0 || c.ms / c.work < best->ms / best->work)) best = &c;
          s->pb = best->pb;
          s->nb = best->nb;
          s->sb = best->sb;
          s->tuned = true;
          r = mpm_batch_set_blocks(s->batch, s->pb, s->nb);
          if (r == MPM_OK) r = mpm_batch_set_option(s->batch, MPM_BATCH_SCATTER_BLOCKS, s->sb);
        }
        if (r == MPM_OK) r = mpm::batch_progress(s->batch, before);
      }
    }
    // submissions are admitted at most every chunk_steps steps: the loop
    // honours their interrupt only after that many steps
    int taken = 0;
    Clock::time_point t0 = Clock::now();
    if (r == MPM_OK) r = mpm_batch_set_option(s->batch, MPM_BATCH_LOOP_MIN_STEPS, s->cfg.chunk_steps);
    if (r == MPM_OK) r = mpm_batch_run_loop(s->batch, kLoopBudget, &taken);
    const double ms = ms_since(t0, Clock::now());
    if (r == MPM_OK) r = mpm::batch_progress(s->batch, prog);
    const double work = r == MPM_OK ? work_since(before, prog) : 0.0;
    // 3. retirement
    retire.clear();
    std::vector<Ticket*> done;
    if (r == MPM_OK) {
      for (const BatchProgress& q : prog)
        if (q.istep >= q.target) retire.push_back(q.id);
      std::vector<Ticket*> owners;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        for (int id : retire) owners.push_back(s->tickets[s->by_scene[id]]);
      }
      for (size_t i = 0; i < retire.size() && r == MPM_OK; ++i) {
        Ticket* t = owners[i];
        r = mpm_batch_scene_scalars(s->batch, retire[i], t->scalars);
        for (int f = 1; f <= 25 && r == MPM_OK; ++f)
          if (t->mask & (1u << f)) {
            int nc = mpm_field_components(f);
            std::vector<double> buf((size_t)(nc * t->np));
            r = mpm_batch_scene_download(s->batch, retire[i], f, buf.data());
            if (r == MPM_OK) t->fields[f].swap(buf);
          }
        if (r == MPM_OK) r = mpm_batch_remove(s->batch, retire[i]);
        if (r == MPM_OK) done.push_back(t);
      }
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (r == MPM_OK) {
        s->chunks++;
        s->particle_steps += work;
        s->busy_ms += ms;
        Clock::time_point now = Clock::now();
        for (Ticket* t : done) {
          t->state = T_DONE;
          t->t_done = now;
          s->by_scene.erase(t->scene_id);
          s->resident_bytes -= t->bytes;
          s->resident_particles -= t->np;
          s->finished++;
        }
      } else {
        std::string msg = mpm_batch_last_error(s->batch);
        fail_resident(s, r, msg);
        // start over with an empty batch
        mpm_batch_destroy(s->batch);
        s->batch = nullptr;
        if (mpm_batch_create(s->cfg.device, &s->batch) != MPM_OK) {
          s->stop = true;
          s->err = "batch lost after error: " + msg;
        } else {
          mpm_batch_set_blocks(s->batch, s->pb, s->nb);
          mpm_batch_set_option(s->batch, MPM_BATCH_SCATTER_BLOCKS, s->sb);
        }
      }
    }
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

int mpm_serve_create(const mpm_serve_config* cfg, mpm_server** out) {
  if (!out) return MPM_ERR_ARG;
  *out = nullptr;
  mpm_server* s = new mpm_server();
  if (cfg) s->cfg = *cfg;
  if (s->cfg.device < 0) cudaGetDevice(&s->cfg.device);
  if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 25;
  if (s->cfg.max_scenes <= 0) s->cfg.max_scenes = 4096;
  int r = mpm_batch_create(s->cfg.device, &s->batch);
  if (r) {
    delete s;
    return r;
  }
  if (s->cfg.hbm_budget_bytes <= 0) {
    size_t fr = 0, tot = 0;
    cudaSetDevice(s->cfg.device);
    cudaMemGetInfo(&fr, &tot);
    // resident scenes' estimates; the batch holds two arenas of the layout
    // (current and spare, with headroom), so about 2.5x this is in use
    s->cfg.hbm_budget_bytes = (int64_t)(0.35 * (double)fr);
  }
  if (s->cfg.autotune) {
    const int blk[2] = {256, 512}, sbs[3] = {8, 32, 64};
    for (int a : blk)
      for (int b2 : blk)
        for (int c : sbs) s->tune.push_back(Tune{a, b2, c});
  }
  s->thr = std::thread(serve_loop, s);
  *out = s;
  return MPM_OK;
}

void mpm_serve_destroy(mpm_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->thr.joinable()) s->thr.join();
  if (s->batch) mpm_batch_destroy(s->batch);
  for (auto& kv : s->tickets) {
    delete kv.second->scene;
    delete kv.second;
  }
  delete s;
}

const char* mpm_serve_last_error(const mpm_server* s) { return s ? s->err.c_str() : "null server"; }

int mpm_serve_submit(mpm_server* s, const mpm_deck* d, int steps, uint32_t field_mask, int64_t* ticket) {
  if (!s || !d || !ticket || steps < 1) return serr(s, MPM_ERR_ARG, "bad argument");
  Clock::time_point t0 = Clock::now();
  std::string err;
  int code = MPM_OK;
  HostScene* h = mpm::scene_stage(d, steps, err, &code);
  if (!h) return serr(s, code, "%s", err.c_str());
  Ticket* t = new Ticket();
  t->scene = h;
  t->bytes = mpm::scene_device_bytes(h);
  t->np = mpm::scene_np(h);
  t->steps = steps;
  t->mask = field_mask;
  t->t_submit = t0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete h;
      delete t;
      return serr(s, MPM_ERR_STATE, "server stopped: %s", s->err.c_str());
    }
    t->id = s->next_ticket++;
    s->tickets[t->id] = t;
    s->queue.push_back(t->id);
    s->submitted++;
    *ticket = t->id;
    // a running device loop returns at its next test, so that the server
    // can admit the scene (the flag is a page-locked word, no CUDA call)
    if (s->batch) mpm_batch_interrupt(s->batch);
  }
  s->cv_work.notify_all();
  return MPM_OK;
}

int mpm_serve_wait(mpm_server* s, int64_t ticket, int timeout_ms) {
  if (!s) return MPM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return serr(s, MPM_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Ticket* t = it->second;
  auto ready = [&] { return t->state == T_DONE || t->state == T_FAILED || s->stop; };
  if (timeout_ms < 0)
    s->cv_done.wait(lk, ready);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  if (t->state == T_DONE) return MPM_OK;
  if (t->state == T_FAILED) return serr(s, t->code, "%s", t->err.c_str());
  if (s->stop) return serr(s, MPM_ERR_STATE, "server stopped: %s", s->err.c_str());
  return MPM_ERR_TIMEOUT;
}

int mpm_serve_result(mpm_server* s, int64_t ticket, double* scalars16, double* times_ms3) {
  if (!s) return MPM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return serr(s, MPM_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Ticket* t = it->second;
  if (t->state == T_FAILED) return serr(s, t->code, "%s", t->err.c_str());
  if (t->state != T_DONE) return serr(s, MPM_ERR_STATE, "ticket %lld has not finished", (long long)ticket);
  if (scalars16) memcpy(scalars16, t->scalars, sizeof t->scalars);
  if (times_ms3) {
    times_ms3[0] = ms_since(t->t_submit, t->t_admit);
    times_ms3[1] = ms_since(t->t_admit, t->t_done);
    times_ms3[2] = ms_since(t->t_submit, t->t_done);
  }
  return MPM_OK;
}

int mpm_serve_field(mpm_server* s, int64_t ticket, int field, double* out) {
  if (!s || !out) return MPM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return serr(s, MPM_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Ticket* t = it->second;
  if (t->state != T_DONE) return serr(s, MPM_ERR_STATE, "ticket %lld has not finished", (long long)ticket);
  auto f = t->fields.find(field);
  if (f == t->fields.end()) return serr(s, MPM_ERR_ARG, "field %d was not requested at submission", field);
  memcpy(out, f->second.data(), sizeof(double) * f->second.size());
  return MPM_OK;
}

int mpm_serve_release(mpm_server* s, int64_t ticket) {
  if (!s) return MPM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return serr(s, MPM_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  Ticket* t = it->second;
  if (t->state == T_QUEUED || t->state == T_RESIDENT)
    return serr(s, MPM_ERR_STATE, "ticket %lld is still running", (long long)ticket);
  delete t;
  s->tickets.erase(it);
  return MPM_OK;
}

int mpm_serve_launch_shape(mpm_server* s, int* particle_block, int* node_block, int* scatter_blocks) {
  if (!s || !particle_block || !node_block || !scatter_blocks) return MPM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  *particle_block = s->pb;
  *node_block = s->nb;
  *scatter_blocks = s->sb;
  return s->tuned ? MPM_OK : MPM_ERR_STATE;
}

int mpm_serve_stats(mpm_server* s, double* o) {
  if (!s || !o) return MPM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  o[0] = (double)s->submitted;
  o[1] = (double)s->finished;
  o[2] = (double)s->queue.size();
  o[3] = (double)s->by_scene.size();
  o[4] = (double)s->chunks;
  o[5] = s->particle_steps;
  o[6] = s->busy_ms;
  o[7] = s->pb;
  o[8] = s->nb;
  o[9] = (double)s->peak_bytes;
  return MPM_OK;
}

int mpm_serve_plan(const mpm_serve_config* cfg, int nqueued, const int64_t* np, const int* steps,
                   const int64_t* bytes, int resident_scenes, int64_t resident_particles, int64_t resident_bytes,
                   int* admit, int* reject, int* nreject) {
  if (!cfg || nqueued < 0 || (nqueued > 0 && (!np || !steps || !bytes || !admit || !reject)) || !nreject)
    return -MPM_ERR_ARG;
  return serve_plan(*cfg, nqueued, np, steps, bytes, resident_scenes, resident_particles, resident_bytes, admit,
                    reject, nreject);
}

int mpm_serve_drain(mpm_server* s, int timeout_ms) {
  if (!s) return MPM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto idle = [&] { return (s->queue.empty() && s->by_scene.empty()) || s->stop; };
  if (timeout_ms < 0)
    s->cv_done.wait(lk, idle);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle))
    return MPM_ERR_TIMEOUT;
  if (s->stop && !(s->queue.empty() && s->by_scene.empty()))
    return serr(s, MPM_ERR_STATE, "server stopped: %s", s->err.c_str());
  return MPM_OK;
}

}  // extern "C"
