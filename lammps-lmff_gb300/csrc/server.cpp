// Serving many independent requests on one device: a submission queue, admission
// under a device-memory budget, and continuous batching.
//
// No counterpart in the reference, which runs one simulation per process.  A request
// is one system: a single point (forces, energies, virial) or an NVE run of nsteps.
// Two worker threads, each owning one engine cloned from the caller's, run
// concurrently on the device (the engines have their own streams):
//   * single points admitted since the last iteration are evaluated together, one
//     batched launch per kernel (lmff_batch_set + lmff_batch_compute);
//   * NVE requests with the same dt form one resident multi-system batch that advances
//     md_chunk_steps at a time through lmff_run_nve (CUDA-graph steps).  Requests join
//     and leave only at chunk boundaries; a chunk ends early at the first request's
//     last step, so every request stops exactly at its nsteps.  When the membership
//     changes the state of the continuing requests is read back and the batch re-formed.
// Each system's neighbours, bins, force sums and reductions are its own (the batch is
// a concatenation of independent systems), so a single point is bitwise the same alone
// and in any mix.  An NVE run in a batch rebuilds its list whenever any member needs
// one, so it equals the run alone up to summation order.
// A batch that fails (for example one system with more than three intralayer
// neighbours) is retried one request at a time, so the error lands only on the
// request that caused it.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "lmff_gb300.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Job {
  int64_t ticket = 0;
  // inputs, copied at submission
  int natoms = 0;
  std::vector<double> x, v;
  std::vector<double> x0, v0;   // submitted state of an NVE request (restart after a failed batch)
  std::vector<int> type;
  std::vector<int64_t> mol;
  double lo[3], hi[3];
  int periodic[3];
  int nsteps = 0;
  double dt = 0.0;
  // caller-owned outputs
  double *f_out = nullptr, *x_out = nullptr, *v_out = nullptr;
  lmff_result *res = nullptr;
  // progress
  double bytes = 0.0;
  double t_submit = 0.0, t_done = 0.0;
  int steps_done = 0;
  bool solo = false;     // run alone (after a failed batch)
  bool done = false;
  int status = LMFF_OK;
  std::string err;

  lmff_system_desc desc() const {
    lmff_system_desc d;
    memset(&d, 0, sizeof d);
    d.natoms = natoms;
    d.x = x.data();
    d.type = type.data();
    d.mol = mol.data();
    d.v = v.empty() ? nullptr : v.data();
    for (int k = 0; k < 3; k++) {
      d.lo[k] = lo[k];
      d.hi[k] = hi[k];
      d.periodic[k] = periodic[k];
    }
    return d;
  }
};

}  // namespace

struct lmff_server {
  lmff_server_config cfg;
  lmff_engine *pt = nullptr;   // single points
  lmff_engine *md = nullptr;   // resident NVE batch
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> queue;        // submitted, not admitted
  std::vector<Job *> points;      // admitted single points
  std::vector<Job *> md_active;   // admitted NVE requests
  std::vector<Job *> resident;    // current members of md's batch, in batch order
  bool resident_synced = true;    // the members' host x, v hold the device state
  std::unordered_map<int64_t, Job *> jobs;
  int64_t next_ticket = 1;
  double admitted_bytes = 0.0;
  double bytes_per_atom = 4096.0;
  bool stop = false;
  std::thread w_points, w_md;
  lmff_server_stats st;
  std::vector<double> pt_f;                 // points worker: batch forces
  std::vector<double> md_x, md_v, md_f;     // NVE worker: batch state read back
};

namespace {

thread_local std::string g_server_err;

// device bytes per atom a batch like the engine's current one needs
double engine_bytes_per_atom(lmff_engine *e) {
  lmff_stats s;
  if (lmff_get_stats(e, &s) != LMFF_OK || s.natoms <= 0) return 0.0;
  return s.bytes_per_atom_need;
}

void finish(lmff_server *s, Job *j, int status, const std::string &err) {
  std::lock_guard<std::mutex> lk(s->mu);
  j->status = status;
  j->err = err;
  j->done = true;
  j->t_done = now_s();
  s->admitted_bytes -= j->bytes;
  if (status == LMFF_OK) s->st.completed++;
  else s->st.failed++;
  s->cv_done.notify_all();
  s->cv_work.notify_all();   // budget released: queued requests may be admitted
}

// FIFO admission while the budget holds (called with the lock held)
void admit(lmff_server *s) {
  while (!s->queue.empty()) {
    Job *j = s->queue.front();
    if (s->admitted_bytes + j->bytes > s->cfg.hbm_budget_bytes && s->admitted_bytes > 0.0) break;
    s->queue.pop_front();
    s->admitted_bytes += j->bytes;
    s->st.max_admitted_bytes = std::max(s->st.max_admitted_bytes, s->admitted_bytes);
    if (j->nsteps > 0) s->md_active.push_back(j);
    else s->points.push_back(j);
  }
}

// one batched evaluation of single points; on failure, each alone
void run_points(lmff_server *s, std::vector<Job *> &batch) {
  std::vector<lmff_system_desc> descs;
  int64_t total = 0;
  for (Job *j : batch) {
    descs.push_back(j->desc());
    total += j->natoms;
  }
  s->pt_f.resize(3 * (size_t)total);
  std::vector<lmff_result> res(batch.size());
  int rc = lmff_batch_set(s->pt, (int)descs.size(), descs.data());
  if (rc == LMFF_OK) rc = lmff_batch_compute(s->pt, s->pt_f.data(), res.data());
  if (rc != LMFF_OK) {
    std::string err = lmff_last_error(s->pt);
    if (batch.size() == 1) {
      finish(s, batch[0], rc, err);
      return;
    }
    for (Job *j : batch) {
      std::vector<Job *> one{j};
      run_points(s, one);
    }
    return;
  }
  double bpa = engine_bytes_per_atom(s->pt);
  size_t o = 0;
  for (size_t k = 0; k < batch.size(); k++) {
    Job *j = batch[k];
    if (j->f_out) memcpy(j->f_out, &s->pt_f[3 * o], sizeof(double) * 3 * j->natoms);
    if (j->res) *j->res = res[k];
    o += j->natoms;
    finish(s, j, LMFF_OK, "");
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->st.point_batches++;
  s->st.point_systems += (int64_t)batch.size();
  s->bytes_per_atom = std::max(s->bytes_per_atom, bpa);
}

// copy the device state of the batch members back into their host x, v
int sync_resident(lmff_server *s) {
  if (s->resident_synced || s->resident.empty()) return LMFF_OK;
  int64_t total = 0;
  for (Job *j : s->resident) total += j->natoms;
  s->md_x.resize(3 * (size_t)total);
  s->md_v.resize(3 * (size_t)total);
  s->md_f.resize(3 * (size_t)total);
  int rc = lmff_download(s->md, s->md_x.data(), s->md_v.data(), s->md_f.data());
  if (rc) return rc;
  size_t o = 0;
  for (Job *j : s->resident) {
    size_t b = 3 * o, nb = 3 * (size_t)j->natoms;
    std::copy(s->md_x.begin() + b, s->md_x.begin() + b + nb, j->x.begin());
    if (j->v.empty()) j->v.assign(nb, 0.0);
    std::copy(s->md_v.begin() + b, s->md_v.begin() + b + nb, j->v.begin());
    o += j->natoms;
  }
  s->resident_synced = true;
  return LMFF_OK;
}

// members of the next NVE chunk: the oldest request's dt; solo requests run alone
std::vector<Job *> pick_md(lmff_server *s) {
  std::vector<Job *> out;
  if (s->md_active.empty()) return out;
  Job *head = s->md_active.front();
  if (head->solo) {
    out.push_back(head);
    return out;
  }
  int64_t atoms = 0;
  for (Job *j : s->md_active) {
    if (j->solo || j->dt != head->dt) continue;
    if (!out.empty() && atoms + j->natoms > s->cfg.max_batch_atoms) break;
    out.push_back(j);
    atoms += j->natoms;
  }
  return out;
}

void drop_active(lmff_server *s, Job *j) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->md_active.erase(std::remove(s->md_active.begin(), s->md_active.end(), j), s->md_active.end());
}

// isolate a failed batch: restart every member alone from its submitted state
void isolate(lmff_server *s, const std::vector<Job *> &members, int rc, const std::string &err) {
  if (members.size() == 1) {
    drop_active(s, members[0]);
    finish(s, members[0], rc, err);
    return;
  }
  for (Job *j : members) {
    j->solo = true;
    j->steps_done = 0;
    j->x = j->x0;   // restart from the submitted positions and velocities
    j->v = j->v0;
  }
}

void run_md_chunk(lmff_server *s) {
  std::vector<Job *> members;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    members = pick_md(s);
  }
  if (members.empty()) return;
  int rc = LMFF_OK;
  if (members != s->resident) {
    rc = sync_resident(s);
    if (rc) {
      std::string err = lmff_last_error(s->md);
      std::vector<Job *> old = s->resident;
      s->resident.clear();
      s->resident_synced = true;
      isolate(s, old, rc, err);
      return;
    }
    std::vector<lmff_system_desc> descs;
    for (Job *j : members) descs.push_back(j->desc());
    rc = lmff_batch_set(s->md, (int)descs.size(), descs.data());
    if (rc) {
      std::string err = lmff_last_error(s->md);
      s->resident.clear();
      isolate(s, members, rc, err);
      return;
    }
    s->resident = members;
    s->resident_synced = true;
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.md_reforms++;
  }
  int chunk = s->cfg.md_chunk_steps;
  for (Job *j : members) chunk = std::min(chunk, j->nsteps - j->steps_done);
  lmff_thermo th[2];
  // the chunk's last step evaluates energies and virials of every member
  rc = lmff_run_nve(s->md, chunk, members[0]->dt, chunk, th);
  if (rc) {
    std::string err = lmff_last_error(s->md);
    s->resident.clear();
    s->resident_synced = true;
    isolate(s, members, rc, err);
    return;
  }
  s->resident_synced = false;
  bool any_done = false;
  for (Job *j : members) {
    j->steps_done += chunk;
    any_done = any_done || j->steps_done >= j->nsteps;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.md_chunks++;
    s->st.md_steps += chunk;
  }
  if (!any_done) return;
  std::vector<lmff_result> res(members.size());
  rc = lmff_batch_results(s->md, (int)members.size(), res.data());
  if (rc == LMFF_OK) rc = sync_resident(s);
  if (rc) {
    std::string err = lmff_last_error(s->md);
    s->resident.clear();
    s->resident_synced = true;
    isolate(s, members, rc, err);
    return;
  }
  double bpa = engine_bytes_per_atom(s->md);
  size_t o = 0;
  std::vector<Job *> keep;
  for (size_t k = 0; k < members.size(); k++) {
    Job *j = members[k];
    size_t b = 3 * o, nb = 3 * (size_t)j->natoms;
    o += j->natoms;
    if (j->steps_done < j->nsteps) {
      keep.push_back(j);
      continue;
    }
    if (j->x_out) memcpy(j->x_out, j->x.data(), sizeof(double) * nb);
    if (j->v_out) memcpy(j->v_out, j->v.data(), sizeof(double) * nb);
    if (j->f_out) memcpy(j->f_out, &s->md_f[b], sizeof(double) * nb);
    if (j->res) *j->res = res[k];
    drop_active(s, j);
    finish(s, j, LMFF_OK, "");
  }
  // the survivors' host state is current; the next chunk re-forms without them
  s->resident.clear();
  s->resident_synced = true;
  std::lock_guard<std::mutex> lk(s->mu);
  s->bytes_per_atom = std::max(s->bytes_per_atom, bpa);
}

// single points: one batched evaluation of everything admitted, then again
void points_main(lmff_server *s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    admit(s);
    if (s->points.empty()) {
      if (s->stop && s->queue.empty()) break;
      s->cv_work.wait(lk);
      continue;
    }
    std::vector<Job *> pts;
    int64_t atoms = 0;
    size_t k = 0;
    for (; k < s->points.size(); k++) {
      Job *j = s->points[k];
      if (!pts.empty() && atoms + j->natoms > s->cfg.max_batch_atoms) break;
      pts.push_back(j);
      atoms += j->natoms;
    }
    s->points.erase(s->points.begin(), s->points.begin() + k);
    lk.unlock();
    double t0 = now_s();
    run_points(s, pts);
    double t1 = now_s();
    lk.lock();
    s->st.busy_s += t1 - t0;
  }
}

// NVE requests: one chunk of the resident batch at a time
void md_main(lmff_server *s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    admit(s);
    if (s->md_active.empty()) {
      if (s->stop && s->queue.empty()) break;
      s->cv_work.wait(lk);
      continue;
    }
    lk.unlock();
    double t0 = now_s();
    run_md_chunk(s);
    double t1 = now_s();
    lk.lock();
    s->st.busy_s += t1 - t0;
  }
}

}  // namespace

extern "C" {

int lmff_server_create(lmff_server **out, const lmff_engine *proto, const lmff_server_config *cfg) {
  if (!out || !proto) return LMFF_EINVAL;
  *out = nullptr;
  lmff_server *s = new (std::nothrow) lmff_server;
  if (!s) return LMFF_ENOMEM;
  memset(&s->cfg, 0, sizeof s->cfg);
  if (cfg) s->cfg = *cfg;
  if (s->cfg.hbm_budget_bytes <= 0) s->cfg.hbm_budget_bytes = 64e9;
  if (s->cfg.max_batch_atoms <= 0) s->cfg.max_batch_atoms = 8 << 20;
  if (s->cfg.md_chunk_steps <= 0) s->cfg.md_chunk_steps = 20;
  if (s->cfg.bytes_per_atom > 0) s->bytes_per_atom = s->cfg.bytes_per_atom;
  memset(&s->st, 0, sizeof s->st);
  int rc = lmff_clone(proto, &s->pt);
  if (rc == LMFF_OK) rc = lmff_clone(proto, &s->md);
  if (rc != LMFF_OK) {
    if (s->pt) lmff_destroy(s->pt);
    delete s;
    return rc;
  }
  s->w_points = std::thread(points_main, s);
  s->w_md = std::thread(md_main, s);
  *out = s;
  return LMFF_OK;
}

}  // extern "C"

namespace {

// validated copy of a request (no lock held)
int make_job(const lmff_request *r, Job **out) {
  *out = nullptr;
  if (!r || r->natoms <= 0 || !r->x || !r->type || r->nsteps < 0 || (r->nsteps > 0 && !(r->dt > 0.0))) {
    g_server_err = "request needs natoms > 0, x, type, nsteps >= 0 and dt > 0 for NVE";
    return LMFF_EINVAL;
  }
  Job *j = new (std::nothrow) Job;
  if (!j) return LMFF_ENOMEM;
  size_t n3 = 3 * (size_t)r->natoms;
  j->natoms = r->natoms;
  j->x.assign(r->x, r->x + n3);
  if (r->v) j->v.assign(r->v, r->v + n3);
  j->type.assign(r->type, r->type + r->natoms);
  if (r->mol) j->mol.assign(r->mol, r->mol + r->natoms);
  else j->mol.assign(r->natoms, 0);
  for (int k = 0; k < 3; k++) {
    j->lo[k] = r->lo[k];
    j->hi[k] = r->hi[k];
    j->periodic[k] = r->periodic[k];
  }
  j->nsteps = r->nsteps;
  j->dt = r->dt;
  j->f_out = r->f_out;
  j->x_out = r->x_out;
  j->v_out = r->v_out;
  j->res = r->res;
  if (j->nsteps > 0) {
    j->x0 = j->x;
    j->v0 = j->v;
  }
  *out = j;
  return LMFF_OK;
}

// queues jobs atomically: a worker iteration sees all of them or none
int enqueue(lmff_server *s, std::vector<Job *> &js, int64_t *tickets) {
  std::lock_guard<std::mutex> lk(s->mu);
  for (Job *j : js) {
    j->bytes = s->bytes_per_atom * j->natoms;
    if (j->bytes > s->cfg.hbm_budget_bytes) {
      g_server_err = "request of " + std::to_string(j->natoms) + " atoms exceeds the device-memory budget";
      for (Job *k : js) delete k;
      return LMFF_ENOMEM;
    }
  }
  double t = now_s();
  for (size_t k = 0; k < js.size(); k++) {
    Job *j = js[k];
    j->ticket = s->next_ticket++;
    j->t_submit = t;
    s->jobs[j->ticket] = j;
    s->queue.push_back(j);
    s->st.submitted++;
    tickets[k] = j->ticket;
  }
  s->cv_work.notify_all();
  return LMFF_OK;
}

}  // namespace

extern "C" {

int lmff_server_submit(lmff_server *s, const lmff_request *r, int64_t *ticket) {
  return lmff_server_submit_many(s, 1, r, ticket);
}

int lmff_server_submit_many(lmff_server *s, int nreq, const lmff_request *reqs, int64_t *tickets) {
  if (!s || nreq < 1 || !reqs || !tickets) return LMFF_EINVAL;
  for (int k = 0; k < nreq; k++) tickets[k] = 0;
  std::vector<Job *> js;
  for (int k = 0; k < nreq; k++) {
    Job *j = nullptr;
    int rc = make_job(&reqs[k], &j);
    if (rc) {
      for (Job *q : js) delete q;
      return rc;
    }
    js.push_back(j);
  }
  return enqueue(s, js, tickets);
}

int lmff_server_wait(lmff_server *s, int64_t ticket, double timeout_s, double *latency_s) {
  if (!s) return LMFF_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) {
    g_server_err = "unknown or already collected ticket";
    return LMFF_EINVAL;
  }
  Job *j = it->second;
  auto ready = [&] { return j->done; };
  if (timeout_s < 0) s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return LMFF_PENDING;
  if (latency_s) *latency_s = j->t_done - j->t_submit;
  int rc = j->status;
  g_server_err = j->err;
  s->jobs.erase(it);
  delete j;
  return rc;
}

int lmff_server_get_stats(lmff_server *s, lmff_server_stats *out) {
  if (!s || !out) return LMFF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->st;
  out->queued = (int64_t)s->queue.size();
  out->active = (int64_t)(s->points.size() + s->md_active.size());
  out->admitted_bytes = s->admitted_bytes;
  out->bytes_per_atom = s->bytes_per_atom;
  return LMFF_OK;
}

const char *lmff_server_last_error(void) { return g_server_err.c_str(); }

void lmff_server_destroy(lmff_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->w_points.joinable()) s->w_points.join();
  if (s->w_md.joinable()) s->w_md.join();
  for (auto &kv : s->jobs) delete kv.second;
  lmff_destroy(s->pt);
  lmff_destroy(s->md);
  delete s;
}

}  // extern "C"
