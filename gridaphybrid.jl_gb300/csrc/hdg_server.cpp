// hdg_server.cpp -- the serving loop: HDG solves of different meshes, orders
// and coefficient fields, admitted as worker slots and HBM budget free up and
// run concurrently, each on its own stream.
//
// Threads: `slots` workers share one queue.  A worker takes the first request
// in priority order that fits in the budget -- requests that have waited
// kAgeMs in arrival order, then the others shortest estimated work first (the
// first in that order may be passed by others at most kMaxBypass times when
// it does not fit, after which admission waits for it) -- reuses an idle
// resident mesh of the same shape when there is one (connectivity, pattern
// and every device buffer stay on the GPU between requests), solves through
// the same entry points as a single-problem caller, and posts the response.
// Idle meshes are evicted least-recently-used when the budget is short.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hdg_internal.h"
#include "hdg_kernels.h"

namespace hdg {

namespace {

struct Shape {
  int nk, nfd, ni, nf, n;
};

Shape shape_of(int D, int k) {
  Shape s{};
  const int k1 = k + 1;
  s.nk = D == 2 ? k1 * k1 : k1 * k1 * k1;
  s.nfd = D == 2 ? k1 : k1 * k1;
  s.ni = (D + 1) * s.nk;
  s.nf = 2 * D * s.nfd;
  s.n = s.ni + s.nf;
  return s;
}

}  // namespace

bool shape_supported(int D, int k, int precision, int solver, size_t smem_optin, std::string &why) {
  if (D < 2 || D > 3 || k < 1 || k > kMaxK) {
    why = "D must be 2 or 3 and 1 <= k <= 4";
    return false;
  }
  const Shape s = shape_of(D, k);
  const size_t avail = smem_optin > 1024 ? smem_optin - 1024 : 0;
  switch (precision) {
    case HDG_PREC_FP64:
      if ((size_t)s.n * (s.n + 1) * sizeof(double) > avail && !l2block_supported(false, D, k)) {
        why = "the FP64 cell block exceeds shared memory";
        return false;
      }
      break;
    case HDG_PREC_FP32_REFINED:
      if (condense_mixed_smem(s.ni, s.nf) > avail) {
        why = "the FP32 cell block exceeds shared memory";
        return false;
      }
      break;
    case HDG_PREC_FF_BLOCK:
      if (!ffblock_supported(D, k) && !l2block_supported(false, D, k)) {
        why = "block elimination is built for D=2, k<=3 and D=3, k<=3";
        return false;
      }
      break;
    default:
      why = "unknown precision";
      return false;
  }
  if (precision != HDG_PREC_FP64 && !cellop_supported(2 * D, s.nfd)) {
    why = "no unassembled FP32 operator for this facet size";
    return false;
  }
  if (solver == HDG_SOLVER_PCG && !pcg_supports_nfd(s.nfd)) {
    why = "no PCG kernel for this facet size";
    return false;
  }
  if (solver != HDG_SOLVER_PCG && solver != HDG_SOLVER_DIRECT) {
    why = "unknown solver";
    return false;
  }
  return true;
}

double footprint_bound(int D, int n, int k, int precision, int solver) {
  const Shape s = shape_of(D, k);
  const double nd1 = std::pow((double)n, D - 1);
  const double ncells = nd1 * n;
  const double nfacets = D * nd1 * (n + 1);
  const double nbnd = 2.0 * D * nd1;
  const double nbr = nfacets - nbnd;
  const double nfree = nbr * s.nfd;
  const int nl = 2 * D;
  const double nblocks = nbr * (2 * nl - 1);
  const double nnz = nblocks * s.nfd * s.nfd;
  const bool fast = precision != HDG_PREC_FP64;
  // cell blocks condensed by the L2-panel block elimination (FP64 too large
  // for the shared-memory LU, or float-float beyond the shared-memory kernel)
  const bool l2block = l2block_supported(false, D, k) &&
                       (fast ? !ffblock_supported(D, k) : (double)s.n * (s.n + 1) * 8.0 > 227.0 * 1024 - 1024);
  double b = 0.0;
  // mesh and Dirichlet data
  b += ncells * (D + D * D) * 8.0 + ncells * nl * 4.0 + nfacets * s.nfd * 4.0 + nfacets * 2 * 4.0 + ncells * 8.0 +
       nbnd * s.nfd * 8.0;
  // pattern and block maps
  b += (nfree + 1) * 8.0 + nnz * 4.0 + nbr * 4 * 4.0 + nblocks * 20.0 + ncells * 4.0 + ncells * nl * 4.0;
  // cell blocks (not kept by the L2-panel kernel, which integrates each cell
  // into its slot), condensed blocks, recovery factors, CSR values and rhs
  const double blocks = l2block ? 0.0 : (double)s.n * s.n * 8 + s.n * 8;
  b += ncells * (blocks + (double)s.nf * s.nf * 8 + 2.0 * s.nf * 8 + 4) + nnz * 8 + nfree * 8;
  b += fast || l2block ? 8.0 * ncells * s.ni * (s.nf + 1) : 8.0 * ncells * s.ni * (s.n + 1);
  if (precision == HDG_PREC_FF_BLOCK) b += ncells * 360.0;  // per-cell panel and integration coefficients
  if (l2block)  // per-CTA slots (one CTA per SM): panels Y, Z and the cell block; per-cell factors
    b += 160.0 * 8.0 * ((double)s.ni * (s.nf + 1) * 2 + (double)s.n * s.n + s.n) + ncells * 1056.0;
  if (fast) b += ncells * cellop_rec(nl, s.nfd) * 4.0;
  // skeleton solve
  if (solver == HDG_SOLVER_DIRECT) {
    b += nfree * (nfree + 1) * 8.0 + ncells * 4.0 + nfree * 8.0;
  } else {
    b += 6 * nfree * 8.0 + nbr * s.nfd * s.nfd * 8.0;
    // the inner frame's scaling W (FP64), inner vectors, products by block row
    if (fast) b += nbr * s.nfd * s.nfd * 8.0 + 5 * nfree * 4.0 + 2 * nfree * 4.0;
  }
  // recovery and error norms
  b += ncells * s.ni * 8.0 + 2 * ncells * 8.0;
  // tables, scalars, partials and allocation granularity
  return b * 1.02 + 48.0 * (1 << 20);
}

}  // namespace hdg

using namespace hdg;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxBypass = 8;
// admission order: requests that have waited this long first (in arrival
// order), then the rest shortest estimated work first
constexpr double kAgeMs = 1000.0;
// resident meshes that are idle may hold at most this share of the budget
constexpr double kIdleShare = 0.5;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// A resident mesh: its own context (stream) and problem.
struct Resident {
  hdg_context *ctx = nullptr;
  hdg_problem *pb = nullptr;
  int D = 0, n = 0, k = 0;
  double bytes = 0.0;  // charged against the budget while resident
  unsigned long long last_use = 0;
};

struct Job {
  long long ticket = 0;
  hdg_request req{};
  std::vector<double> kappa;
  double footprint = 0.0;
  double work = 0.0;  // estimated device work: cells x (cell block size)^2
  Clock::time_point t_submit;
  int bypassed = 0;
};

}  // namespace

struct hdg_server {
  int device = 0;
  double budget = 0.0;
  size_t smem_optin = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job> queue;
  std::deque<hdg_response> done;
  std::vector<std::unique_ptr<Resident>> idle;  // resident meshes not in use
  std::vector<std::thread> workers;
  double in_use = 0.0, peak = 0.0, busy_ms = 0.0;
  long long next_ticket = 1;
  long long submitted = 0, completed = 0, failed = 0;
  int running = 0, max_running = 0;
  long long mesh_hits = 0, mesh_misses = 0, evictions = 0, retries = 0;
  unsigned long long clock = 0;
  bool stop = false;
  std::string err;

  int fail(int code, const char *msg) {
    std::lock_guard<std::mutex> g(mu);
    err = msg;
    return code;
  }

  static void destroy_resident(Resident *r) {
    if (r->pb) hdg_problem_destroy(r->pb);
    if (r->ctx) hdg_context_destroy(r->ctx);
    r->pb = nullptr;
    r->ctx = nullptr;
  }

  // With mu held: bytes that evicting idle meshes (except `keep`) could free.
  double evictable(const Resident *keep) const {
    double s = 0.0;
    for (const auto &r : idle)
      if (r.get() != keep) s += r->bytes;
    return s;
  }

  // With mu held: picks the next admissible job; moves it to `job`, and the
  // resident mesh to reuse (or null) to `res`; evicted meshes go to `trash`.
  bool admit(Job &job, std::unique_ptr<Resident> &res, std::vector<std::unique_ptr<Resident>> &trash) {
    // priority order: aged requests in arrival order, then shortest work first
    const Clock::time_point now = Clock::now();
    std::vector<size_t> order(queue.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    auto aged = [&](size_t i) { return ms_between(queue[i].t_submit, now) >= kAgeMs; };
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
      const bool ax = aged(x), ay = aged(y);
      if (ax != ay) return ax;
      if (ax) return x < y;
      return queue[x].work < queue[y].work;
    });
    for (size_t oi = 0; oi < order.size(); ++oi) {
      const size_t qi = order[oi];
      Job &j = queue[qi];
      const hdg_request &q = j.req;
      int match = -1;
      for (size_t i = 0; i < idle.size(); ++i)
        if (idle[i]->D == q.D && idle[i]->n == q.n && idle[i]->k == q.k &&
            (match < 0 || idle[i]->last_use > idle[(size_t)match]->last_use))
          match = (int)i;
      const Resident *keep = match >= 0 ? idle[(size_t)match].get() : nullptr;
      // a reused mesh is already charged; only growth beyond it is new
      const double need = std::max(0.0, j.footprint - (keep ? keep->bytes : 0.0));
      if (in_use + need > budget && in_use + need - evictable(keep) > budget) {
        if (oi == 0 && ++j.bypassed > kMaxBypass) return false;  // the first in order waits for memory
        continue;
      }
      // evict least-recently-used idle meshes until the job fits
      while (in_use + need > budget) {
        size_t victim = idle.size();
        for (size_t i = 0; i < idle.size(); ++i)
          if (idle[i].get() != keep && (victim == idle.size() || idle[i]->last_use < idle[victim]->last_use))
            victim = i;
        if (victim == idle.size()) break;
        in_use -= idle[victim]->bytes;
        trash.push_back(std::move(idle[victim]));
        idle.erase(idle.begin() + (long)victim);
        ++evictions;
        match = -1;
        for (size_t i = 0; i < idle.size(); ++i)
          if (idle[i].get() == keep) match = (int)i;
      }
      if (match >= 0) {
        res = std::move(idle[(size_t)match]);
        idle.erase(idle.begin() + match);
        ++mesh_hits;
      } else {
        ++mesh_misses;
      }
      in_use += need;
      peak = std::max(peak, in_use);
      job = std::move(j);
      queue.erase(queue.begin() + (long)qi);
      return true;
    }
    return false;
  }

  void worker(int slot) {
    cudaSetDevice(device);
    for (;;) {
      Job job;
      std::unique_ptr<Resident> res;
      std::vector<std::unique_ptr<Resident>> trash;
      {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
          if (stop) return;
          if (!queue.empty() && admit(job, res, trash)) break;
          cv_work.wait(lk);
        }
        ++running;
        max_running = std::max(max_running, running);
      }
      for (auto &t : trash) destroy_resident(t.get());
      trash.clear();
      const double charged = job.footprint - (res ? std::min(job.footprint, res->bytes) : 0.0) +
                             (res ? res->bytes : 0.0);
      hdg_response r{};
      r.ticket = job.ticket;
      r.slot = slot;
      r.footprint_bytes = job.footprint;
      r.reused_mesh = res ? 1 : 0;
      const Clock::time_point t_start = Clock::now();
      r.queue_ms = ms_between(job.t_submit, t_start);
      int rc = run(job, res, r);
      if (rc == HDG_ERR_NOMEM) {
        // The device ran out of memory below the admission budget: freed
        // blocks that the memory pool keeps, or other users of the GPU.  Give
        // the memory of the failed attempt and of every idle mesh back, return
        // the pool's unused memory to the device, and run the request once more.
        if (res) destroy_resident(res.get());
        res.reset();
        {
          std::lock_guard<std::mutex> g(mu);
          for (auto &m : idle) {
            in_use -= m->bytes;
            trash.push_back(std::move(m));
            ++evictions;
          }
          idle.clear();
          ++retries;
        }
        for (auto &t : trash) destroy_resident(t.get());
        trash.clear();
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
          cudaDeviceSynchronize();
          cudaMemPoolTrimTo(pool, 0);
        }
        cudaGetLastError();
        r = hdg_response{};
        r.ticket = job.ticket;
        r.slot = slot;
        r.footprint_bytes = job.footprint;
        r.queue_ms = ms_between(job.t_submit, t_start);
        rc = run(job, res, r);
      }
      const Clock::time_point t_end = Clock::now();
      r.status = rc;
      if (rc != HDG_OK && res && res->ctx) {  // before a failed request's mesh (and context) goes
        std::strncpy(r.message, hdg_last_error(res->ctx), sizeof(r.message) - 1);
        r.message[sizeof(r.message) - 1] = '\0';
      }
      r.run_ms = ms_between(t_start, t_end);
      r.latency_ms = ms_between(job.t_submit, t_end);
      {
        std::lock_guard<std::mutex> g(mu);
        in_use -= charged;  // the job's reservation, including the reused mesh's bytes
        if (res && res->pb && rc == HDG_OK) {
          double actual = 0.0;
          hdg_problem_device_bytes(res->pb, &actual);
          res->bytes = std::max(actual, 0.0);
          res->last_use = ++clock;
          in_use += res->bytes;
          peak = std::max(peak, in_use);
          idle.push_back(std::move(res));
          // keep the idle meshes within their share of the budget (LRU out)
          double idle_bytes = evictable(nullptr);
          while (idle_bytes > kIdleShare * budget && idle.size() > 1) {
            size_t victim = 0;
            for (size_t i = 1; i < idle.size(); ++i)
              if (idle[i]->last_use < idle[victim]->last_use) victim = i;
            idle_bytes -= idle[victim]->bytes;
            in_use -= idle[victim]->bytes;
            trash.push_back(std::move(idle[victim]));
            idle.erase(idle.begin() + (long)victim);
            ++evictions;
          }
        }
        --running;
        ++completed;
        if (rc != HDG_OK) ++failed;
        busy_ms += r.run_ms;
        done.push_back(r);
      }
      if (res) destroy_resident(res.get());  // a failed request does not keep its mesh
      for (auto &t : trash) destroy_resident(t.get());
      trash.clear();
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }

  int run(const Job &job, std::unique_ptr<Resident> &res, hdg_response &r) {
    const hdg_request &q = job.req;
    int rc;
    if (!res) {
      res.reset(new Resident());
      res->D = q.D;
      res->n = q.n;
      res->k = q.k;
      if ((rc = hdg_context_create(device, &res->ctx))) return rc;
      const int cells[3] = {q.n, q.n, q.n};
      const double dom[6] = {0, 1, 0, 1, 0, 1};
      if ((rc = hdg_problem_create_cartesian(res->ctx, q.D, cells, dom, q.k, &res->pb))) return rc;
    }
    hdg_problem *pb = res->pb;
    if ((rc = hdg_set_darcy(pb, q.stab_mode, q.tau, q.problem))) return rc;
    std::vector<double> ones;
    const double *kap = job.kappa.empty() ? nullptr : job.kappa.data();
    if (!kap) {
      ones.assign((size_t)pb->mesh.ncells, 1.0);
      kap = ones.data();
    }
    double stats[7] = {0};
    if ((rc = hdg_solve(pb, q.precision, q.solver, q.rtol, q.maxit, kap, q.solution, stats))) return rc;
    r.iters = (int)stats[0];
    r.relres = stats[1];
    if ((rc = hdg_l2_errors(pb, &r.err_flux, &r.err_pressure))) return rc;
    return HDG_OK;
  }
};

extern "C" {

int hdg_server_create(int device, int slots, double hbm_budget_bytes, hdg_server **out) {
  if (!out || slots < 1 || slots > 64) return HDG_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HDG_ERR_NODEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HDG_ERR_NODEVICE;
  if (prop.major * 10 + prop.minor < 100) return HDG_ERR_NODEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return HDG_ERR_CUDA;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return HDG_ERR_CUDA;
  hdg_server *s = new (std::nothrow) hdg_server();
  if (!s) return HDG_ERR_NOMEM;
  s->device = device;
  s->smem_optin = prop.sharedMemPerBlockOptin;
  s->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : 0.85 * (double)free_b;
  for (int i = 0; i < slots; ++i) s->workers.emplace_back([s, i] { s->worker(i); });
  *out = s;
  return HDG_OK;
}

int hdg_server_destroy(hdg_server *s) {
  if (!s) return HDG_ERR_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (Job &j : s->queue) {
      hdg_response r{};
      r.ticket = j.ticket;
      r.status = HDG_ERR_STATE;
      s->done.push_back(r);
    }
    s->queue.clear();
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &r : s->idle) hdg_server::destroy_resident(r.get());
  delete s;
  return HDG_OK;
}

int hdg_server_submit(hdg_server *s, const hdg_request *req, long long *ticket) {
  if (!s || !req) return HDG_ERR_INVALID;
  std::string why;
  if (!shape_supported(req->D, req->k, req->precision, req->solver, s->smem_optin, why))
    return s->fail(HDG_ERR_INVALID, why.c_str());
  if (req->n < 1 || req->n > 4096 || !(req->rtol > 0.0) || req->maxit < 1 || !(req->tau > 0.0))
    return s->fail(HDG_ERR_INVALID, "bad request parameters");
  Job j;
  j.req = *req;
  j.req.kappa = nullptr;
  const double ncells = std::pow((double)req->n, req->D);
  if (ncells > 2.0e8) return s->fail(HDG_ERR_INVALID, "mesh too large");
  if (req->kappa) j.kappa.assign(req->kappa, req->kappa + (size_t)ncells);
  j.footprint = footprint_bound(req->D, req->n, req->k, req->precision, req->solver);
  {
    const double nb = std::pow(req->k + 1.0, req->D) * (req->D + 1) + 2.0 * req->D * std::pow(req->k + 1.0, req->D - 1);
    j.work = ncells * nb * nb;
  }
  if (j.footprint > s->budget) return s->fail(HDG_ERR_INVALID, "request larger than the HBM budget");
  j.t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return HDG_ERR_STATE;
    j.ticket = s->next_ticket++;
    if (ticket) *ticket = j.ticket;
    ++s->submitted;
    s->queue.push_back(std::move(j));
  }
  s->cv_work.notify_one();
  return HDG_OK;
}

int hdg_server_poll(hdg_server *s, hdg_response *out, int max, double timeout_ms, int *count) {
  if (!s || !count || (max > 0 && !out)) return HDG_ERR_INVALID;
  *count = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && timeout_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), [s] { return !s->done.empty(); });
  int c = 0;
  while (c < max && !s->done.empty()) {
    out[c++] = s->done.front();
    s->done.pop_front();
  }
  *count = c;
  return HDG_OK;
}

int hdg_server_drain(hdg_server *s, double timeout_ms) {
  if (!s) return HDG_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms),
                                      [s] { return s->queue.empty() && s->running == 0; });
  return ok ? HDG_OK : HDG_ERR_NOT_CONVERGED;
}

int hdg_server_stats(hdg_server *s, double *st) {
  if (!s || !st) return HDG_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  st[0] = (double)s->submitted;
  st[1] = (double)s->completed;
  st[2] = (double)s->failed;
  st[3] = (double)s->running;
  st[4] = (double)s->queue.size();
  st[5] = s->in_use;
  st[6] = s->budget;
  st[7] = s->peak;
  st[8] = (double)s->mesh_hits;
  st[9] = (double)s->mesh_misses;
  st[10] = (double)s->evictions;
  st[11] = (double)s->max_running;
  st[12] = s->busy_ms;
  st[13] = (double)s->retries;
  return HDG_OK;
}

const char *hdg_server_last_error(hdg_server *s) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> g(s->mu);
  return s->err.c_str();
}

}  // extern "C"
