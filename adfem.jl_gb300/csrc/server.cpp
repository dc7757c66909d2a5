// Serving loop of libadfem_gpu (C ABI in include/adfem_gpu.h, adfem_server_*).
//
// The reference holds a single global mesh (deps/MFEM/API.cpp:6-10) and serves one
// caller; this runtime serves a stream of independent solve requests:
//  * a FIFO queue; worker threads (one CUDA stream each) take the next request as soon
//    as they are free, so small and large requests run concurrently on the GPU and a
//    finished request is replaced immediately (continuous batching at request level);
//  * resident systems per (mesh, kind): operator pattern, sliced-ELL copies, solver
//    vectors and the CUDA graphs captured by their solver stay on the device and are
//    reused by later requests on the same mesh; several instances of one (mesh, kind)
//    serve concurrent requests; the last solution of an instance is kept for warm starts;
//  * HBM admission: resident systems and worker buffers are counted against a budget;
//    idle systems are evicted least-recently-used when a new one does not fit; a request
//    that does not fit even into an empty server is rejected with ADFEM_ERR_BUSY (never
//    an abort), one that fits later waits in the queue;
//  * packing: the solves of small mixed-precision requests (at most pack_max_dof DOFs)
//    are handed to a packer thread that solves all waiting ones in one graph-captured
//    launch, one thread block per system (pack.cu); packs grow with the load;
//  * per-request status and timings; p50/p99 of the completed requests.
// A request runs its own kernels with grids and reduction orders fixed by its own sizes
// (a packed request: its own thread block), so its results do not depend on the other
// requests in flight.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "adfem_internal.h"
#include "solver.cuh"

using Clock = std::chrono::steady_clock;

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
  long long ticket = 0;
  adfem_request req{};
  Clock::time_point t_submit, t_start;
  adfem_response resp{};
  bool done = false;
};

struct Resident {
  adfem_system* sys = nullptr;
  const adfem_mesh* mesh = nullptr;
  int kind = 0;
  size_t bytes = 0;
  bool busy = false;
  uint64_t last_use = 0;
  bool bd_set = false;
  std::vector<long long> bd;   // Dirichlet DOFs currently imposed
  std::vector<double> bdval;
  adfem::DevBuf uprev;         // last solution (warm starts)
  bool uprev_valid = false;
};

// A solve handed to the packer: forward (u from the system's rhs) or adjoint (lam
// from g); the worker waits for done.
struct PackTicket {
  adfem_system* sys = nullptr;
  double* out = nullptr;
  const double* g = nullptr;
  bool adjoint = false;
  bool warm = false;
  adfem_solver_opts opts{};
  adfem_solver_stats stats{};
  int status = ADFEM_OK;
  std::string msg;
  bool done = false;
};

struct Worker {
  cudaStream_t stream = nullptr;
  adfem::DevBuf in[4], u, g, lam, grad;
  std::vector<double> hg;      // host dL/du of the misfit
  size_t bytes() const {
    size_t b = u.bytes + g.bytes + lam.bytes + grad.bytes;
    for (const auto& d : in) b += d.bytes;
    return b;
  }
};

constexpr int kPackers = 4;  // packer threads (concurrent packed launches)
// Default packing threshold: up to ~4k DOFs a system solved by one thread block is about
// as fast as the whole-GPU solver even alone, and packs of many run at a fraction of the
// per-solve cost; larger systems are faster on the whole GPU unless many are packed.
constexpr int kPackDefaultDof = 16384;

int ndof_of(const adfem::Mesh* m, int kind) { return (int)(kind == ADFEM_SYS_ELASTICITY ? 2 * m->nv : m->nv); }

// Device bytes of a resident system before it exists (admission): per stored operator
// entry 8+8+4 (scaled FP64 standard and difference forms, FP32) + 8+4 (banded path
// copies) + 2+2 (column deltas) = 36 B with 15% padding; per DOF ~210 B of solver and
// Dirichlet vectors; per element ~96 B of element scratch and Gauss-point staging.
size_t estimate_system_bytes(const adfem::Mesh* m, int kind) {
  const double ndof = (double)ndof_of(m, kind);
  const double nnz = (double)m->nnz * (kind == ADFEM_SYS_ELASTICITY ? 4.0 : 1.0);
  const double b = 36.0 * 1.15 * nnz + 210.0 * ndof + 96.0 * (double)m->ne + 64.0 * 1024;
  return (size_t)b;
}

// Worker buffers a request needs (inputs at Gauss points, u, g, lambda, gradient).
size_t estimate_worker_bytes(const adfem::Mesh* m, int kind) {
  const size_t ng = 3 * (size_t)m->ne, nd = (size_t)ndof_of(m, kind);
  return sizeof(double) * ((kind == ADFEM_SYS_ELASTICITY ? 4 : 2) * ng + 3 * nd + ng);
}

}  // namespace

struct adfem_server {
  adfem_server_config cfg{};
  size_t budget = 0;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work;  // queue non-empty or stopping
  std::condition_variable cv_done;  // a request finished (memory may have been freed)
  std::deque<std::shared_ptr<Job>> queue;
  std::unordered_map<long long, std::shared_ptr<Job>> jobs;
  long long next_ticket = 1;
  bool stopping = false;
  bool stopping_packer = false;
  int running = 0;
  std::vector<std::thread> threads;
  std::vector<std::unique_ptr<Resident>> residents;
  std::vector<std::unique_ptr<Worker>> workers;
  // packer
  int pack_max_dof = 0, pack_max = 0;
  std::deque<PackTicket*> pack_queue;
  std::condition_variable cv_pack;       // pack queue non-empty or stopping
  std::condition_variable cv_pack_done;  // a ticket finished
  struct Packer {
    std::thread th;
    cudaStream_t stream = nullptr;
    adfem::PackSlot* slot = nullptr;
  };
  std::vector<Packer> packers;
  long long packs = 0, packed_requests = 0;
  size_t used = 0;  // resident systems + worker buffers
  uint64_t tick = 0;
  std::vector<double> lat, qlat;
  long long submitted = 0, completed = 0, rejected = 0, timeouts = 0, failed = 0;
  long long hits = 0, misses = 0, evictions = 0;

  // ---- helpers (mu held)
  void finish(const std::shared_ptr<Job>& job, int status) {
    const auto t = Clock::now();
    job->resp.status = status;
    job->resp.total_ms = ms_between(job->t_submit, t);
    if (job->t_start.time_since_epoch().count() != 0) job->resp.run_ms = ms_between(job->t_start, t);
    if (status == ADFEM_OK) {
      completed++;
      lat.push_back(job->resp.total_ms);
      qlat.push_back(job->resp.queue_ms);
    } else if (status == ADFEM_ERR_TIMEOUT) {
      timeouts++;
    } else if (status == ADFEM_ERR_BUSY) {
      rejected++;
    } else {
      failed++;
    }
    job->done = true;
    cv_done.notify_all();
  }
  Resident* find_free(const adfem_mesh* mesh, int kind) {
    for (auto& r : residents)
      if (!r->busy && r->sys && r->mesh == mesh && r->kind == kind) return r.get();
    return nullptr;
  }
  bool evict_one_idle() {
    int best = -1;
    for (int i = 0; i < (int)residents.size(); i++)
      if (!residents[i]->busy && residents[i]->sys &&
          (best < 0 || residents[i]->last_use < residents[best]->last_use))
        best = i;
    if (best < 0) return false;
    used -= residents[best]->bytes;
    adfem_system_destroy(residents[best]->sys);
    residents.erase(residents.begin() + best);
    evictions++;
    return true;
  }
  bool any_busy() const {
    for (auto& r : residents)
      if (r->busy) return true;
    return false;
  }
  void run_worker(int wid);
  void run_packer(int pid);
  int pack_solve(PackTicket& t);
  int run_job(Worker& W, Resident& R, Job& job);
};

// Hand a solve to the packer and wait for it (the worker's stream work before it must
// be complete).
int adfem_server::pack_solve(PackTicket& t) {
  {
    std::lock_guard<std::mutex> lk(mu);
    pack_queue.push_back(&t);
  }
  cv_pack.notify_one();
  std::unique_lock<std::mutex> lk(mu);
  cv_pack_done.wait(lk, [&] { return t.done; });
  if (t.status != ADFEM_OK) return adfem::fail(t.status, t.msg);
  return ADFEM_OK;
}

void adfem_server::run_packer(int pid) {
  cudaSetDevice(device);
  Packer& P = packers[pid];
  std::vector<PackTicket*> batch;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_pack.wait(lk, [&] { return stopping_packer || !pack_queue.empty(); });
      if (pack_queue.empty()) break;
      batch.clear();
      while (!pack_queue.empty() && (int)batch.size() < pack_max) {
        batch.push_back(pack_queue.front());
        pack_queue.pop_front();
      }
    }
    // one launch for the forward solves, one for the adjoint solves
    for (int adj = 0; adj < 2; adj++) {
      std::vector<PackTicket*> grp;
      for (PackTicket* t : batch)
        if (t->adjoint == (adj == 1)) grp.push_back(t);
      if (grp.empty()) continue;
      std::vector<adfem_system*> sys;
      std::vector<double*> out;
      std::vector<const double*> g;
      std::vector<adfem_solver_stats> st(grp.size());
      adfem_solver_opts o = grp[0]->opts;
      for (PackTicket* t : grp) {
        sys.push_back(t->sys);
        out.push_back(t->out);
        g.push_back(t->g);
      }
      // warm starts and tolerances are per request: split the group where they differ
      size_t i0 = 0;
      while (i0 < grp.size()) {
        size_t i1 = i0 + 1;
        while (i1 < grp.size() && grp[i1]->warm == grp[i0]->warm && grp[i1]->opts.rtol == grp[i0]->opts.rtol &&
               grp[i1]->opts.max_iter == grp[i0]->opts.max_iter)
          i1++;
        o = grp[i0]->opts;
        o.warm_start = grp[i0]->warm ? 1 : 0;
        const int cnt = (int)(i1 - i0);
        const int r = adfem::system_solve_packed(sys.data() + i0, cnt, out.data() + i0, g.data() + i0, &o,
                                                 st.data() + i0, P.stream, adj == 1, P.slot);
        const std::string msg = r == ADFEM_OK ? std::string() : std::string(adfem_last_error());
        std::lock_guard<std::mutex> lk(mu);
        packs++;
        packed_requests += adj ? 0 : cnt;
        for (size_t i = i0; i < i1; i++) {
          grp[i]->stats = st[i];
          // a failed pack call reports per-system statuses; a setup failure applies to all
          grp[i]->status = r == ADFEM_OK ? ADFEM_OK : (st[i].status != ADFEM_OK ? st[i].status : r);
          grp[i]->msg = msg;
          grp[i]->done = true;
        }
        i0 = i1;
      }
    }
    cv_pack_done.notify_all();
  }
}

// ---------------------------------------------------------------------------
int adfem_server::run_job(Worker& W, Resident& R, Job& job) {
  const adfem_request& q = job.req;
  const adfem::Mesh* m = adfem::mesh_of(q.mesh);
  const int kind = q.kind;
  const size_t ng = 3 * (size_t)m->ne;
  const size_t nd = (size_t)ndof_of(m, kind);
  const int nin = kind == ADFEM_SYS_ELASTICITY ? 4 : 2;
  // worker buffers (growth is counted against the budget)
  {
    const size_t before = W.bytes();
    for (int i = 0; i < nin; i++) ADFEM_TRY(W.in[i].alloc(sizeof(double) * ng));
    ADFEM_TRY(W.u.alloc(sizeof(double) * nd));
    if (q.nobs > 0) {
      ADFEM_TRY(W.g.alloc(sizeof(double) * nd));
      ADFEM_TRY(W.lam.alloc(sizeof(double) * nd));
      ADFEM_TRY(W.grad.alloc(sizeof(double) * ng));
    }
    const size_t after = W.bytes();
    if (after != before) {
      std::lock_guard<std::mutex> lk(mu);
      used += after - before;
    }
  }
  cudaStream_t st = W.stream;
  for (int i = 0; i < nin; i++)
    ADFEM_CUDA(cudaMemcpyAsync(W.in[i].p, q.in[i], sizeof(double) * ng, cudaMemcpyHostToDevice, st));
  // Dirichlet data: re-imposed only when it differs from what this instance holds
  const bool same_bd = R.bd_set && R.bd.size() == (size_t)q.nbd &&
                       std::equal(R.bd.begin(), R.bd.end(), q.bd) &&
                       (q.bdval ? (R.bdval.size() == (size_t)q.nbd && std::equal(R.bdval.begin(), R.bdval.end(), q.bdval))
                                : R.bdval.empty());
  if (!same_bd) {
    ADFEM_TRY(adfem_system_set_dirichlet(R.sys, q.bd, q.nbd, q.bdval));
    R.bd.assign(q.bd, q.bd + q.nbd);
    if (q.bdval) R.bdval.assign(q.bdval, q.bdval + q.nbd);
    else R.bdval.clear();
    R.bd_set = true;
    R.uprev_valid = false;
  }
  if (kind == ADFEM_SYS_POISSON)
    ADFEM_TRY(adfem_system_assemble_poisson_d(R.sys, W.in[0].as<double>(), W.in[1].as<double>(), st));
  else
    ADFEM_TRY(adfem_system_assemble_elasticity_d(R.sys, W.in[0].as<double>(), W.in[1].as<double>(),
                                                 W.in[2].as<double>(), W.in[3].as<double>(), st));
  adfem_solver_opts o = cfg.opts;
  if (q.precision >= 0) o.precision = q.precision;
  o.warm_start = 0;
  if (q.warm_start && R.uprev_valid) {
    ADFEM_CUDA(cudaMemcpyAsync(W.u.p, R.uprev.p, sizeof(double) * nd, cudaMemcpyDeviceToDevice, st));
    o.warm_start = 1;
  }
  const bool packed = pack_max_dof > 0 && o.precision == ADFEM_PREC_MIXED && (long long)nd <= pack_max_dof;
  adfem_solver_stats fs{};
  if (packed) {
    ADFEM_CUDA(cudaStreamSynchronize(st));  // assembly and the warm-start copy are done
    PackTicket t;
    t.sys = R.sys;
    t.out = W.u.as<double>();
    t.warm = o.warm_start != 0;
    t.opts = o;
    ADFEM_TRY(pack_solve(t));
    fs = t.stats;
    job.resp.packed = 1;
  } else {
    ADFEM_TRY(adfem_system_solve_d(R.sys, W.u.as<double>(), &o, &fs, st));
  }
  job.resp.iterations = fs.iterations;
  job.resp.relres = fs.relres;
  if (R.uprev.bytes < sizeof(double) * nd) {
    const size_t before = R.uprev.bytes;
    ADFEM_TRY(R.uprev.alloc(sizeof(double) * nd));
    std::lock_guard<std::mutex> lk(mu);
    used += R.uprev.bytes - before;
    R.bytes += R.uprev.bytes - before;
  }
  ADFEM_CUDA(cudaMemcpyAsync(R.uprev.p, W.u.p, sizeof(double) * nd, cudaMemcpyDeviceToDevice, st));
  R.uprev_valid = true;
  ADFEM_CUDA(cudaMemcpyAsync(q.u, W.u.p, sizeof(double) * nd, cudaMemcpyDeviceToHost, st));
  ADFEM_CUDA(cudaStreamSynchronize(st));
  if (q.nobs > 0) {
    // misfit L = sum (u[obs] - uobs)^2 and dL/du on the host (obs is a small subset)
    W.hg.assign(nd, 0.0);
    double loss = 0.0;
    for (long long k = 0; k < q.nobs; k++) {
      const long long i = q.obs[k] - 1;
      const double d = q.u[i] - q.uobs[k];
      loss += d * d;
      W.hg[i] += 2.0 * d;
    }
    job.resp.loss = loss;
    ADFEM_CUDA(cudaMemcpyAsync(W.g.p, W.hg.data(), sizeof(double) * nd, cudaMemcpyHostToDevice, st));
    adfem_solver_stats as{};
    if (packed) {
      ADFEM_CUDA(cudaStreamSynchronize(st));
      PackTicket t;
      t.sys = R.sys;
      t.out = W.lam.as<double>();
      t.g = W.g.as<double>();
      t.adjoint = true;
      t.opts = o;
      t.opts.warm_start = 0;
      ADFEM_TRY(pack_solve(t));
      as = t.stats;
    } else {
      ADFEM_TRY(adfem_system_adjoint_d(R.sys, W.g.as<double>(), W.lam.as<double>(), &o, &as, st));
    }
    job.resp.adjoint_iterations = as.iterations;
    if (kind == ADFEM_SYS_POISSON)
      ADFEM_TRY(adfem_system_grad_kappa_d(R.sys, W.u.as<double>(), W.lam.as<double>(), W.grad.as<double>(), st));
    else
      ADFEM_TRY(adfem_system_grad_E_d(R.sys, W.u.as<double>(), W.lam.as<double>(), W.in[0].as<double>(),
                                      W.in[1].as<double>(), W.grad.as<double>(), st));
    ADFEM_CUDA(cudaMemcpyAsync(q.grad, W.grad.p, sizeof(double) * ng, cudaMemcpyDeviceToHost, st));
    ADFEM_CUDA(cudaStreamSynchronize(st));
  }
  return ADFEM_OK;
}

void adfem_server::run_worker(int wid) {
  cudaSetDevice(device);
  Worker& W = *workers[wid];
  for (;;) {
    std::shared_ptr<Job> job;
    Resident* R = nullptr;
    bool create = false;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stopping || !queue.empty(); });
      if (queue.empty()) break;  // stopping, nothing left
      job = queue.front();
      queue.pop_front();
      const auto now = Clock::now();
      if (job->req.deadline_ms > 0.0 && ms_between(job->t_submit, now) > job->req.deadline_ms) {
        std::snprintf(job->resp.message, sizeof(job->resp.message), "deadline passed before the request started");
        finish(job, ADFEM_ERR_TIMEOUT);
        continue;
      }
      R = find_free(job->req.mesh, job->req.kind);
      if (R) {
        hits++;
      } else {
        const adfem::Mesh* m = adfem::mesh_of(job->req.mesh);
        const size_t est = estimate_system_bytes(m, job->req.kind);
        while (used + est > budget && evict_one_idle()) {
        }
        if (used + est > budget) {
          if (running == 0 && !any_busy()) {
            std::snprintf(job->resp.message, sizeof(job->resp.message), "does not fit the HBM budget");
            finish(job, ADFEM_ERR_BUSY);
            continue;
          }
          // wait for running requests to release memory, then try again
          queue.push_front(job);
          cv_done.wait(lk);
          continue;
        }
        misses++;
        residents.push_back(std::make_unique<Resident>());
        R = residents.back().get();
        R->mesh = job->req.mesh;
        R->kind = job->req.kind;
        R->bytes = est;
        used += est;
        create = true;
      }
      R->busy = true;
      running++;
      job->t_start = now;
      job->resp.queue_ms = ms_between(job->t_submit, now);
    }
    int status = ADFEM_OK;
    if (create) {
      status = adfem_system_create(const_cast<adfem_mesh*>(R->mesh), R->kind, &R->sys);
      std::lock_guard<std::mutex> lk(mu);
      if (status == ADFEM_OK) {
        const size_t actual = adfem::system_device_bytes(R->sys);
        used = used - R->bytes + actual;
        R->bytes = actual;
      }
    }
    if (status == ADFEM_OK) status = run_job(W, *R, *job);
    if (status != ADFEM_OK) std::snprintf(job->resp.message, sizeof(job->resp.message), "%s", adfem_last_error());
    {
      std::lock_guard<std::mutex> lk(mu);
      running--;
      R->busy = false;
      R->last_use = ++tick;
      if (!R->sys) {  // creation failed: drop the placeholder
        used -= R->bytes;
        residents.erase(std::find_if(residents.begin(), residents.end(),
                                     [&](const std::unique_ptr<Resident>& p) { return p.get() == R; }));
      }
      finish(job, status);
    }
  }
  cudaStreamSynchronize(W.stream);
}

// ---------------------------------------------------------------------------
extern "C" {

void adfem_server_config_default(adfem_server_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->hbm_budget_bytes = 0;
  cfg->workers = 8;
  cfg->max_queue = 65536;
  adfem_solver_opts_default(&cfg->opts);
  cfg->pack_max_dof = 0;
  cfg->pack_max = 0;
}

int adfem_server_create(const adfem_server_config* cfg, adfem_server** out) {
  ADFEM_RANGE("adfem_server_create");
  if (!out) return adfem::fail(ADFEM_ERR_INVALID, "null argument");
  *out = nullptr;
  auto S = std::make_unique<adfem_server>();
  adfem_server_config_default(&S->cfg);
  if (cfg) S->cfg = *cfg;
  if (S->cfg.workers <= 0) S->cfg.workers = 8;
  if (S->cfg.workers > 256) return adfem::fail(ADFEM_ERR_INVALID, "server: at most 256 workers");
  if (S->cfg.max_queue <= 0) S->cfg.max_queue = 65536;
  S->pack_max_dof = std::min(S->cfg.pack_max_dof == 0 ? kPackDefaultDof : std::max(S->cfg.pack_max_dof, 0),
                             adfem::pack_rows_limit());
  S->pack_max = S->cfg.pack_max <= 0 ? 64 : std::min(S->cfg.pack_max, adfem::kPackMaxSystems);
  ADFEM_CUDA(cudaGetDevice(&S->device));
  size_t freeb = 0, total = 0;
  ADFEM_CUDA(cudaMemGetInfo(&freeb, &total));
  S->budget = S->cfg.hbm_budget_bytes > 0 ? (size_t)S->cfg.hbm_budget_bytes : (size_t)(0.8 * (double)freeb);
  for (int i = 0; i < S->cfg.workers; i++) {
    auto W = std::make_unique<Worker>();
    ADFEM_CUDA(cudaStreamCreateWithFlags(&W->stream, cudaStreamNonBlocking));
    S->workers.push_back(std::move(W));
  }
  // packers: several packs run at once (a pack lasts as long as its largest system)
  const int npack = S->pack_max_dof > 0 ? kPackers : 0;
  S->packers.resize(npack);
  for (auto& P : S->packers) {
    ADFEM_CUDA(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
    P.slot = adfem::pack_slot_create();
  }
  adfem_server* s = S.get();
  for (int i = 0; i < npack; i++) s->packers[i].th = std::thread([s, i] { s->run_packer(i); });
  for (int i = 0; i < s->cfg.workers; i++) s->threads.emplace_back([s, i] { s->run_worker(i); });
  *out = S.release();
  return ADFEM_OK;
}

int adfem_server_destroy(adfem_server* srv) {
  ADFEM_RANGE("adfem_server_destroy");
  if (!srv) return ADFEM_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stopping = true;
  }
  srv->cv_work.notify_all();
  srv->cv_done.notify_all();
  for (auto& t : srv->threads) t.join();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stopping_packer = true;
  }
  srv->cv_pack.notify_all();
  for (auto& P : srv->packers) {
    if (P.th.joinable()) P.th.join();
    if (P.stream) cudaStreamDestroy(P.stream);
    adfem::pack_slot_destroy(P.slot);
  }
  for (auto& r : srv->residents)
    if (r->sys) adfem_system_destroy(r->sys);
  srv->residents.clear();
  for (auto& w : srv->workers)
    if (w->stream) cudaStreamDestroy(w->stream);
  delete srv;
  return ADFEM_OK;
}

int adfem_server_submit(adfem_server* srv, const adfem_request* req, long long* ticket) {
  ADFEM_RANGE("adfem_server_submit");
  if (!srv || !req || !ticket) return adfem::fail(ADFEM_ERR_INVALID, "null argument");
  const adfem::Mesh* m = adfem::mesh_of(req->mesh);
  if (!m) return adfem::fail(ADFEM_ERR_INVALID, "server: request without a mesh");
  if (req->kind != ADFEM_SYS_POISSON && req->kind != ADFEM_SYS_ELASTICITY)
    return adfem::fail(ADFEM_ERR_INVALID, "server: unknown request kind");
  const int nin = req->kind == ADFEM_SYS_ELASTICITY ? 4 : 2;
  for (int i = 0; i < nin; i++)
    if (!req->in[i]) return adfem::fail(ADFEM_ERR_INVALID, "server: missing input field");
  if (!req->u || req->nbd < 0 || (req->nbd > 0 && !req->bd) || req->nobs < 0)
    return adfem::fail(ADFEM_ERR_INVALID, "server: bad output or Dirichlet arguments");
  const long long nd = ndof_of(m, req->kind);
  if (req->nobs > 0) {
    if (!req->obs || !req->uobs || !req->grad) return adfem::fail(ADFEM_ERR_INVALID, "server: observations need obs, uobs, grad");
    for (long long k = 0; k < req->nobs; k++)
      if (req->obs[k] < 1 || req->obs[k] > nd) return adfem::fail(ADFEM_ERR_INVALID, "server: observation id out of range");
  }
  if (req->precision != -1 && req->precision != ADFEM_PREC_FP64 && req->precision != ADFEM_PREC_MIXED)
    return adfem::fail(ADFEM_ERR_INVALID, "server: unknown precision");
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->stopping) return adfem::fail(ADFEM_ERR_INVALID, "server: shutting down");
  const size_t need = estimate_system_bytes(m, req->kind) + estimate_worker_bytes(m, req->kind);
  if (need > srv->budget) {
    srv->rejected++;
    return adfem::fail(ADFEM_ERR_BUSY, "server: request needs ~" + std::to_string(need >> 20) +
                                           " MiB, more than the HBM budget of " +
                                           std::to_string(srv->budget >> 20) + " MiB");
  }
  if ((int)srv->queue.size() >= srv->cfg.max_queue) {
    srv->rejected++;
    return adfem::fail(ADFEM_ERR_BUSY, "server: queue full");
  }
  auto job = std::make_shared<Job>();
  job->ticket = srv->next_ticket++;
  job->req = *req;
  job->t_submit = Clock::now();
  srv->queue.push_back(job);
  srv->jobs[job->ticket] = job;
  srv->submitted++;
  *ticket = job->ticket;
  srv->cv_work.notify_one();
  return ADFEM_OK;
}

int adfem_server_wait(adfem_server* srv, long long ticket, double timeout_ms, adfem_response* resp) {
  ADFEM_RANGE("adfem_server_wait");
  if (!srv) return adfem::fail(ADFEM_ERR_INVALID, "null argument");
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(ticket);
  if (it == srv->jobs.end()) return adfem::fail(ADFEM_ERR_INVALID, "server: unknown ticket");
  std::shared_ptr<Job> job = it->second;
  if (timeout_ms < 0.0) {
    srv->cv_done.wait(lk, [&] { return job->done; });
  } else if (!job->done) {
    srv->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), [&] { return job->done; });
  }
  if (!job->done) return adfem::fail(ADFEM_ERR_TIMEOUT, "server: request still running");
  if (resp) *resp = job->resp;
  srv->jobs.erase(ticket);
  return ADFEM_OK;
}

static double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  const size_t k = std::min(v.size() - 1, (size_t)std::floor(p * (double)(v.size() - 1) + 0.5));
  std::nth_element(v.begin(), v.begin() + k, v.end());
  return v[k];
}

int adfem_server_get_stats(adfem_server* srv, adfem_server_stats* out) {
  ADFEM_RANGE("adfem_server_get_stats");
  if (!srv || !out) return adfem::fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = srv->submitted;
  out->completed = srv->completed;
  out->rejected = srv->rejected;
  out->timeouts = srv->timeouts;
  out->failed = srv->failed;
  out->cache_hits = srv->hits;
  out->cache_misses = srv->misses;
  out->evictions = srv->evictions;
  out->resident_systems = (long long)srv->residents.size();
  out->device_bytes = (long long)srv->used;
  out->p50_ms = percentile(srv->lat, 0.50);
  out->p99_ms = percentile(srv->lat, 0.99);
  out->p50_queue_ms = percentile(srv->qlat, 0.50);
  out->p99_queue_ms = percentile(srv->qlat, 0.99);
  double s = 0.0, mx = 0.0;
  for (double v : srv->lat) {
    s += v;
    mx = std::max(mx, v);
  }
  out->mean_ms = srv->lat.empty() ? 0.0 : s / (double)srv->lat.size();
  out->max_ms = mx;
  out->packs = srv->packs;
  out->packed_requests = srv->packed_requests;
  return ADFEM_OK;
}

int adfem_server_reset_stats(adfem_server* srv) {
  ADFEM_RANGE("adfem_server_reset_stats");
  if (!srv) return adfem::fail(ADFEM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->lat.clear();
  srv->qlat.clear();
  srv->submitted = srv->completed = srv->rejected = srv->timeouts = srv->failed = 0;
  srv->hits = srv->misses = srv->evictions = 0;
  srv->packs = srv->packed_requests = 0;
  return ADFEM_OK;
}

}  // extern "C"
