// Request server: stationary CD solves of differing meshes and coefficients,
// served concurrently on one GPU (the served form of
// ConvectionDiffusion<d>::assemble() + solve(), src/System/
// ConvectionDiffusion.C:112-281, run once per request).
//
// Design:
//  * n_slots workers, each with its own cdg_context (stream + reduction
//    scratch); requests on different slots overlap on the device;
//  * a mesh class (dim, order, n, levels) has one host hierarchy (mesh, DOF
//    map, TStructure: built once) and a pool of device-resident problem
//    instances (CSR matrices, multigrid hierarchy, Krylov state, captured
//    iteration graph) that are reused by later requests of the class;
//  * admission: a queued request starts when a slot is free and its instance
//    is idle in the pool or a new one fits the HBM budget; idle instances
//    are evicted least recently used first to make room.  Requests that do
//    not fit wait; smaller ones behind them may start (continuous batching),
//    unless the head of the queue has waited longer than kHeadPatience;
//  * batching per launch: a small request the batched solver takes (batch.cu:
//    mixed precision, V-cycle, up to kBatchMaxDofs DOFs) is assembled and
//    prepared on its slot's stream, then handed to the batcher thread and
//    the slot moves on; the batcher solves everything handed over since its
//    last launch in one launch (one block per request, each stopping on its
//    own convergence test), copies the solutions out and completes the jobs.
//    Requests handed over while a launch runs go into the next one.
//    CDG_SERVER_BATCH=0 at server creation keeps every request on its slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace cdg {
namespace {

using Clock = std::chrono::steady_clock;
constexpr double kHeadPatience = 2.0;   // seconds before the queue head blocks others
constexpr int kBatchers = 4;            // batched launches in flight
constexpr int kServerPrioDofs = 20000;  // requests up to this size run on high-priority
                                        // streams (CDG_SERVER_PRIORITY=0: none)
// requests batched per launch up to this size (CDG_SERVER_BATCH_DOFS
// overrides, at most the batched solver's kBatchMaxDofs).  Measured on GB300
// (200 requests of the served mix, saturated, 8 slots): 597 solves/s without
// batching, 638 with this cap, 424 with 5000 -- a block solves a 4225-DOF
// request in 5 ms against 1.7 ms for the stream-level solver, and at these
// arrival rates a launch holds about one small request, so only requests the
// block solves faster than the stream path (about 2000 DOFs and below) gain
constexpr int kServerBatchDofs = 2500;

struct ClassKey {
  int dim, order, n, levels;
  bool operator<(const ClassKey& o) const {
    return std::tie(dim, order, n, levels) < std::tie(o.dim, o.order, o.n, o.levels);
  }
};

struct MeshClass {
  std::mutex build;                   // one builder at a time
  cdg_hierarchy* h = nullptr;
  long long bytes = 0;                // estimated device bytes of one instance
  int ndof = 0;
};

struct Instance {
  ClassKey key;
  cdg_problem* p = nullptr;
  long long bytes = 0;
  bool busy = false;
  int last_slot = -1;
  unsigned long long last_used = 0;
};

struct Instance;

struct Job {
  long long ticket = 0;
  cdg_request req{};
  ClassKey key{};
  double* out = nullptr;
  Clock::time_point submit, start, done;
  bool finished = false;
  cdg_result res{};
  // handed to the batcher: the instance, and the end of its preparation on
  // the slot's stream
  Instance* inst = nullptr;
  cudaEvent_t ready = nullptr;
  int inline_coarse = 0;   // coarse block inverted inside the batch
};

struct Slot {
  int id = 0;
  cdg_context* ctx = nullptr;
  cdg_context* hi = nullptr;   // the same slot's high-priority stream (small requests)
  std::thread th;
};

// cells per direction n = roots * 2^nref with roots 1 or 3
bool split_n(int n, int* roots, int* nref) {
  for (int r : {1, 3}) {
    if (n % r) continue;
    int m = n / r, k = 0;
    while (m > 1 && m % 2 == 0) { m /= 2; ++k; }
    if (m == 1) { *roots = r; *nref = k; return true; }
  }
  return false;
}

// levels down to a coarsest grid of 3 or 4 cells per direction
int default_levels(int roots, int nref) {
  if (roots == 3) return nref + 1;
  return std::max(1, nref - 1);
}

long long estimate_bytes(const cdg_hierarchy* h, int n_levels, int restart) {
  long long b = 0;
  int info[6];
  for (int l = 0; l < n_levels; ++l) {
    cdg_hierarchy_level_info(h, l, info);
    const long long ncells = info[0], nloc = info[1], ndof = info[2], nnz = info[4],
                    nv = info[5];
    b += nnz * 16 + ncells * nloc * nloc * 4 + ncells * nloc * 16 + ndof * 112 +
         ncells * nv * 3 * 8;
    b += ndof >= 32768 ? nnz * 17 + ndof * 8 : 0;   // sliced ELLPACK copy
    b += (l + 1 < n_levels) ? ndof * 24 * 16 : 0;   // transfer matrices
  }
  cdg_hierarchy_level_info(h, 0, info);
  b += (long long)(2 * restart + 3) * info[2] * 8;
  return b + b / 8 + (2 << 20);
}

// before the hierarchy exists: the same estimate from the structured sizes
long long estimate_bytes_unbuilt(const ClassKey& k, int restart) {
  long long b = 0;
  int n = k.n;
  for (int l = 0; l < k.levels; ++l, n /= 2) {
    const long long m = (long long)k.order * n + 1;
    const long long ndof = k.dim == 2 ? m * m : m * m * m;
    const long long band = k.dim == 2 ? (2LL * k.order + 1) * (2LL * k.order + 1)
                                      : (2LL * k.order + 1) * (2LL * k.order + 1) * (2LL * k.order + 1);
    const long long nloc = k.dim == 2 ? (k.order + 1LL) * (k.order + 1) : (k.order + 1LL) * (k.order + 1) * (k.order + 1);
    const long long ncells = k.dim == 2 ? (long long)n * n : (long long)n * n * n;
    b += ndof * band * 16 + ncells * nloc * nloc * 4 + ncells * nloc * 16 + ndof * 112 +
         ncells * 8 * 3 * 8 + ndof * 24 * 16;
    b += ndof >= 32768 ? ndof * band * 17 + ndof * 8 : 0;   // sliced ELLPACK copy
  }
  const long long m = (long long)k.order * k.n + 1;
  b += (long long)(2 * restart + 3) * (k.dim == 2 ? m * m : m * m * m) * 8;
  return b + b / 8 + (2 << 20);
}

}  // namespace
}  // namespace cdg

using namespace cdg;

struct cdg_server {
  int device = 0;
  long long budget = 0, used = 0;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  // batching per launch: kBatchers threads, each with its own stream, take
  // whatever has been handed over when they are free (a long launch does not
  // hold back the next one)
  bool batch = true;
  bool prio = true;
  int batch_max_dofs = kServerBatchDofs;
  std::vector<cdg_context*> bctx;
  std::vector<std::thread> batchers;
  std::condition_variable cv_batch;
  std::deque<Job*> bq;
  long long batches = 0, batched = 0;
  std::unordered_map<long long, std::unique_ptr<Job>> jobs;
  std::map<ClassKey, std::unique_ptr<MeshClass>> classes;
  std::vector<std::unique_ptr<Instance>> pool;
  bool stop = false;
  long long next_ticket = 1;
  unsigned long long tick = 0;
  long long submitted = 0, completed = 0, failed = 0, running = 0, evictions = 0,
            peak_running = 0;
};

namespace {

MeshClass* get_class(cdg_server* s, const ClassKey& k) {
  auto it = s->classes.find(k);
  if (it == s->classes.end())
    it = s->classes.emplace(k, std::unique_ptr<MeshClass>(new MeshClass())).first;
  return it->second.get();
}

// under s->mu: an idle instance of the class (prefer one last used on this
// slot), or nullptr
Instance* find_idle(cdg_server* s, const ClassKey& k, int slot) {
  Instance* best = nullptr;
  for (auto& u : s->pool) {
    Instance* in = u.get();
    if (in->busy || in->key < k || k < in->key) continue;
    if (!best || (in->last_slot == slot && best->last_slot != slot)) best = in;
  }
  return best;
}

// under s->mu: remove idle instances (least recently used first) until
// `need` more bytes fit; returns the instances to destroy outside the lock
bool make_room(cdg_server* s, long long need, std::vector<Instance*>* victims) {
  long long idle = 0;
  for (auto& u : s->pool)
    if (!u->busy) idle += u->bytes;
  if (s->used - idle + need > s->budget) return false;   // evict nothing in vain
  while (s->used + need > s->budget) {
    Instance* lru = nullptr;
    for (auto& u : s->pool)
      if (!u->busy && (!lru || u->last_used < lru->last_used)) lru = u.get();
    if (!lru) return false;
    s->used -= lru->bytes;
    s->evictions++;
    for (auto it = s->pool.begin(); it != s->pool.end(); ++it)
      if (it->get() == lru) {
        victims->push_back(it->release());
        s->pool.erase(it);
        break;
      }
  }
  return true;
}

void destroy_instances(cdg_context* ctx, std::vector<Instance*>& v) {
  for (Instance* in : v) {
    // idle: its last work finished before it returned to the pool; bind it to
    // this worker's (idle) stream so destroy waits on nothing else
    in->p->ctx = ctx;
    cdg_problem_destroy(in->p);
    delete in;
  }
  v.clear();
}

// the batcher takes the job (assembled and prepared): 1 handed over, 0 run
// here, < 0 an error
int run_job(cdg_server* s, Slot* slot, Job* job, Instance* inst) {
  cdg_problem* p = inst->p;
  // the problem's work goes to this slot's stream; small requests to its
  // high-priority one
  cdg_context* ctx = s->prio && p->lev[0].ndof <= kServerPrioDofs ? slot->hi : slot->ctx;
  p->ctx = ctx;
  CDG_TRY(cdg_problem_set_solution(p, nullptr));
  CDG_TRY(cdg_problem_assemble(p, &job->req.a));
  if (s->batch && p->lev[0].ndof <= s->batch_max_dofs && batch_eligible(p, job->req.s, nullptr)) {
    CDG_TRY(batch_prepare(ctx, p, job->req.s, &job->inline_coarse));
    if (!job->ready) CDG_CUDA(cudaEventCreateWithFlags(&job->ready, cudaEventDisableTiming));
    CDG_CUDA(cudaEventRecord(job->ready, ctx->stream));
    job->inst = inst;
    return 1;
  }
  int rc = cdg_problem_solve(p, &job->req.s, &job->res.stats);
  if (rc != CDG_OK) return rc;
  return cdg_problem_get_solution(p, job->out);
}

// completes a job under s->mu
void finish_job(cdg_server* s, Job* job, Instance* inst, int slot_id, int rc) {
  job->res.status = rc;
  job->res.slot = slot_id;
  if (inst) {
    inst->busy = false;
    inst->last_slot = slot_id;
    inst->last_used = ++s->tick;
  }
  job->done = Clock::now();
  job->res.queue_seconds = std::chrono::duration<double>(job->start - job->submit).count();
  job->res.latency_seconds = std::chrono::duration<double>(job->done - job->submit).count();
  job->finished = true;
  s->running--;
  s->completed++;
  if (rc != CDG_OK) s->failed++;
}

// the batcher: one launch over every job handed over since the last one
void batcher(cdg_server* s, int id) {
  cudaSetDevice(s->device);
  cdg_context* bctx = s->bctx[id];
  std::vector<Job*> jobs;
  std::vector<cdg_problem*> probs;
  std::vector<cdg_solver_params> params;
  std::vector<int> inl;
  std::vector<BatchResult> res;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    while (s->bq.empty() && !s->stop) s->cv_batch.wait_for(lk, std::chrono::milliseconds(50));
    if (s->bq.empty()) break;   // stopping with nothing handed over
    jobs.assign(s->bq.begin(), s->bq.end());
    s->bq.clear();
    lk.unlock();
    cudaStream_t st = bctx->stream;
    probs.clear();
    params.clear();
    inl.clear();
    for (Job* j : jobs) {
      cudaStreamWaitEvent(st, j->ready, 0);
      probs.push_back(j->inst->p);
      params.push_back(j->req.s);
      inl.push_back(j->inline_coarse);
    }
    res.assign(jobs.size(), BatchResult{CDG_OK, 0, 0.0, 0.0});
    const auto t0 = Clock::now();
    int rc = batch_launch(bctx, probs.data(), params.data(), inl.data(), (int)jobs.size(),
                          res.data());
    for (size_t q = 0; q < jobs.size() && rc == CDG_OK; ++q) {
      const DevLevel& F = jobs[q]->inst->p->lev[0];
      if (cudaMemcpyAsync(jobs[q]->out, F.sol, (size_t)F.ndof * sizeof(double),
                          cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = CDG_ERR_CUDA;
    }
    if (rc == CDG_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = CDG_ERR_CUDA;
    const double secs = std::chrono::duration<double>(Clock::now() - t0).count();
    lk.lock();
    for (size_t q = 0; q < jobs.size(); ++q) {
      Job* j = jobs[q];
      j->res.stats.iterations = res[q].iterations;
      j->res.stats.residual = res[q].residual;
      j->res.stats.initial_residual = res[q].initial;
      j->res.stats.seconds = secs;
      finish_job(s, j, j->inst, (int)s->slots.size(), rc != CDG_OK ? rc : res[q].status);
    }
    s->batches++;
    s->batched += (long long)jobs.size();
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

void worker(cdg_server* s, Slot* slot) {
  cudaSetDevice(s->device);
  std::vector<Instance*> victims;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    Job* job = nullptr;
    Instance* inst = nullptr;
    long long reserve = 0;
    while (!s->stop) {
      // the first queued request that can start now
      const auto now = Clock::now();
      for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        Job* j = *it;
        MeshClass* mc = get_class(s, j->key);
        Instance* in = find_idle(s, j->key, slot->id);
        long long need = 0;
        if (!in) {
          need = mc->h ? mc->bytes
                       : estimate_bytes_unbuilt(j->key, std::max(1, j->req.s.gmres_restart));
          if (!make_room(s, need, &victims)) {
            // does not fit yet; a long-waiting head blocks the others
            if (it == s->queue.begin() &&
                std::chrono::duration<double>(now - j->submit).count() > kHeadPatience)
              break;
            continue;
          }
        }
        job = j;
        inst = in;
        reserve = need;
        s->queue.erase(it);
        break;
      }
      if (job) break;
      if (!victims.empty()) {
        lk.unlock();
        destroy_instances(slot->ctx, victims);
        lk.lock();
        continue;
      }
      s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
    }
    if (!job) break;   // stopping
    if (inst) {
      inst->busy = true;
    }
    s->used += reserve;
    s->running++;
    s->peak_running = std::max(s->peak_running, s->running);
    job->start = Clock::now();
    lk.unlock();
    if (!victims.empty()) destroy_instances(slot->ctx, victims);

    int rc = CDG_OK;
    bool own = false;   // instance created for this job
    if (!inst) {
      MeshClass* mc;
      {
        std::lock_guard<std::mutex> g(s->mu);
        mc = get_class(s, job->key);
      }
      {
        std::lock_guard<std::mutex> g(mc->build);
        if (!mc->h) {
          int roots = 1, nref = 0;
          split_n(job->req.n, &roots, &nref);
          // numbering, patterns (and, at instance creation, transfers and the
          // sliced operator) built on this slot's GPU; CDG_SERVER_HOST_SETUP=1
          // builds the hierarchy on the host
          if (getenv("CDG_SERVER_HOST_SETUP"))
            rc = cdg_hierarchy_create(job->req.dim, job->req.order, roots, nref,
                                      job->key.levels, job->req.a.neumann_mask, &mc->h);
          else
            rc = cdg_hierarchy_create_device(slot->ctx, job->req.dim, job->req.order, roots,
                                             nref, job->key.levels, job->req.a.neumann_mask,
                                             &mc->h);
          if (rc == CDG_OK) {
            mc->bytes = estimate_bytes(mc->h, job->key.levels,
                                       std::max(1, job->req.s.gmres_restart));
            int info[6];
            cdg_hierarchy_level_info(mc->h, 0, info);
            mc->ndof = info[2];
          } else {
            mc->h = nullptr;
          }
        }
      }
      if (rc == CDG_OK) {
        std::unique_ptr<Instance> in(new Instance());
        in->key = job->key;
        in->bytes = mc->bytes;
        rc = cdg_problem_create(slot->ctx, mc->h, &in->p);
        if (rc == CDG_OK) {
          in->busy = true;
          inst = in.get();
          own = true;
          std::lock_guard<std::mutex> g(s->mu);
          // the reservation made at admission becomes the instance's size
          s->used += in->bytes - reserve;
          s->pool.push_back(std::move(in));
        } else {
          std::lock_guard<std::mutex> g(s->mu);
          s->used -= reserve;
        }
      } else {
        std::lock_guard<std::mutex> g(s->mu);
        s->used -= reserve;
      }
    }
    (void)own;
    if (rc == CDG_OK) rc = run_job(s, slot, job, inst);
    lk.lock();
    if (rc == 1) {
      // handed to the batcher, which completes it
      s->bq.push_back(job);
      s->cv_batch.notify_one();
      continue;
    }
    finish_job(s, job, inst, slot->id, rc);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int cdg_request_ndof(const cdg_request* r, int* ndof) {
  int roots = 1, nref = 0;
  if (!r || !ndof || (r->dim != 2 && r->dim != 3) || (r->order != 1 && r->order != 2) ||
      r->n < 2 || !split_n(r->n, &roots, &nref)) {
    set_error("request: dim 2/3, order 1/2, n = roots * 2^k with roots 1 or 3");
    return CDG_ERR_ARG;
  }
  long long m = (long long)r->order * r->n + 1, v = m * m * (r->dim == 3 ? m : 1);
  if (v > 2000000000LL) { set_error("request too large"); return CDG_ERR_LIMIT; }
  *ndof = (int)v;
  return CDG_OK;
}

int cdg_server_create(int device, int n_slots, long long budget, cdg_server** out) {
  if (!out || n_slots < 1 || n_slots > 64) { set_error("n_slots must be in [1, 64]"); return CDG_ERR_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device");
    return CDG_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) { set_error("bad device %d", device); return CDG_ERR_ARG; }
  std::unique_ptr<cdg_server> s(new cdg_server());
  s->device = device;
  CDG_CUDA(cudaSetDevice(device));
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    CDG_CUDA(cudaMemGetInfo(&fr, &tot));
    budget = (long long)(fr * 0.8);
  }
  s->budget = budget;
  {
    const char* e = getenv("CDG_SERVER_BATCH");
    s->batch = !(e && e[0] == '0');
  }
  {
    const char* e = getenv("CDG_SERVER_PRIORITY");
    s->prio = !(e && e[0] == '0');
  }
  if (s->batch) {
    const char* e = getenv("CDG_SERVER_BATCH_DOFS");
    if (e) s->batch_max_dofs = std::min(atoi(e), kBatchMaxDofs);
    for (int i = 0; i < kBatchers; ++i) {
      cdg_context* c = nullptr;
      int rc = cdg_context_create(device, &c);
      if (rc == CDG_OK && s->prio) rc = cdg_context_high_priority(c);
      if (rc != CDG_OK) {
        if (c) cdg_context_destroy(c);
        for (cdg_context* x : s->bctx) cdg_context_destroy(x);
        return rc;
      }
      s->bctx.push_back(c);
    }
  }
  for (int i = 0; i < n_slots; ++i) {
    std::unique_ptr<Slot> sl(new Slot());
    sl->id = i;
    int rc = cdg_context_create(device, &sl->ctx);
    if (rc == CDG_OK) rc = cdg_context_create(device, &sl->hi);
    if (rc == CDG_OK && s->prio) rc = cdg_context_high_priority(sl->hi);
    if (rc != CDG_OK) {
      if (sl->ctx) cdg_context_destroy(sl->ctx);
      if (sl->hi) cdg_context_destroy(sl->hi);
      for (auto& x : s->slots) {
        cdg_context_destroy(x->ctx);
        cdg_context_destroy(x->hi);
      }
      for (cdg_context* x : s->bctx) cdg_context_destroy(x);
      return rc;
    }
    s->slots.push_back(std::move(sl));
  }
  cdg_server* raw = s.release();
  for (auto& sl : raw->slots) sl->th = std::thread(worker, raw, sl.get());
  for (int i = 0; i < (int)raw->bctx.size(); ++i) raw->batchers.emplace_back(batcher, raw, i);
  *out = raw;
  return CDG_OK;
}

int cdg_server_destroy(cdg_server* s) {
  if (!s) return CDG_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& sl : s->slots)
    if (sl->th.joinable()) sl->th.join();
  // the batcher finishes what the workers handed over, then stops
  s->cv_batch.notify_all();
  for (auto& t : s->batchers)
    if (t.joinable()) t.join();
  cudaSetDevice(s->device);
  for (auto& in : s->pool) {
    in->p->ctx = s->slots[0]->ctx;
    cdg_problem_destroy(in->p);
  }
  for (auto& kv : s->classes)
    if (kv.second->h) cdg_hierarchy_destroy(kv.second->h);
  for (auto& sl : s->slots) {
    cdg_context_destroy(sl->ctx);
    cdg_context_destroy(sl->hi);
  }
  for (cdg_context* x : s->bctx) cdg_context_destroy(x);
  for (auto& kv : s->jobs)
    if (kv.second->ready) cudaEventDestroy(kv.second->ready);
  delete s;
  return CDG_OK;
}

int cdg_server_submit(cdg_server* s, const cdg_request* r, double* out, long long* ticket) {
  if (!s || !r || !out || !ticket) { set_error("null argument"); return CDG_ERR_ARG; }
  int ndof = 0;
  CDG_TRY(cdg_request_ndof(r, &ndof));
  int roots = 1, nref = 0;
  split_n(r->n, &roots, &nref);
  std::unique_ptr<Job> j(new Job());
  j->req = *r;
  int levels = r->s.preconditioner == 2 ? r->s.multigrid_n_levels : 1;
  if (r->s.preconditioner == 2 && levels <= 0) levels = default_levels(roots, nref);
  if (levels > nref + 1) { set_error("too many multigrid levels for n = %d", r->n); return CDG_ERR_ARG; }
  if (r->s.preconditioner == 2) j->req.s.multigrid_n_levels = levels;
  j->key = ClassKey{r->dim, r->order, r->n, levels};
  j->out = out;
  j->res.ndof = ndof;
  j->submit = Clock::now();
  std::lock_guard<std::mutex> g(s->mu);
  j->ticket = s->next_ticket++;
  *ticket = j->ticket;
  s->queue.push_back(j.get());
  s->jobs.emplace(j->ticket, std::move(j));
  s->submitted++;
  s->cv_work.notify_one();
  return CDG_OK;
}

int cdg_server_wait(cdg_server* s, long long ticket, double timeout, cdg_result* res) {
  if (!s || !res) { set_error("null argument"); return CDG_ERR_ARG; }
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) { set_error("unknown ticket %lld", ticket); return CDG_ERR_ARG; }
  Job* j = it->second.get();
  auto pred = [&] { return j->finished; };
  if (timeout < 0)
    s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout), pred))
    return 1;
  *res = j->res;
  if (j->ready) cudaEventDestroy(j->ready);
  s->jobs.erase(it);
  return CDG_OK;
}

int cdg_server_counters(cdg_server* s, long long* c) {
  if (!s || !c) { set_error("null argument"); return CDG_ERR_ARG; }
  std::lock_guard<std::mutex> g(s->mu);
  long long resident = 0;
  for (auto& in : s->pool) resident += in->bytes;
  c[0] = s->submitted;
  c[1] = s->completed;
  c[2] = s->failed;
  c[3] = (long long)s->queue.size();
  c[4] = s->running;
  c[5] = (long long)s->pool.size();
  c[6] = resident;
  c[7] = s->evictions;
  c[8] = s->budget;
  c[9] = s->peak_running;
  long long launches = 0;
  for (auto& sl : s->slots)
    launches += cdg_context_launch_count(sl->ctx) + cdg_context_launch_count(sl->hi);
  for (cdg_context* x : s->bctx) launches += cdg_context_launch_count(x);
  c[10] = launches;
  c[11] = (long long)s->classes.size();
  return CDG_OK;
}

int cdg_server_batch_counters(cdg_server* s, long long* c) {
  if (!s || !c) { set_error("null argument"); return CDG_ERR_ARG; }
  std::lock_guard<std::mutex> g(s->mu);
  c[0] = s->batches;
  c[1] = s->batched;
  c[2] = s->batch ? 1 : 0;
  return CDG_OK;
}

}  // extern "C"
