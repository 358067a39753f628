// Continuous-batching server over a solved model (host runtime, C++).
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fgb_internal.h"
#include "fgb_model.h"

namespace fgb {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long id;
  int n;
  double cell[9];
  std::vector<double> pos;
  std::vector<int> species;
  long long bytes;
  Clock::time_point t_submit, t_done;
  int passed_over = 0;   // batches admitted past this request
  bool done = false;
  int status = FGB_OK;
  std::string error;
  double energy = 0, stress[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> forces, var;
};

// Device bytes per atom of the prediction pipeline for this model (the
// workspace buffers of predict.cu, neighbour arrays at up to 128 neighbours
// per atom, and the widest per-species GEMM rows).
long long footprint_per_atom(const fgb_model_s *m) {
  const B2Params &p = m->b2;
  long long mmax = 1;
  for (int c : m->h_counts) mmax = std::max<long long>(mmax, c);
  long long b = 8LL * p.n_A + 3 * 8LL * p.n_d + 16LL * mmax + 8 * 16;
  b += 128LL * (8 + 32 + 4 + 4 + 32 + 8 + 24);   // pairs: keys, rel, j, shift, twin, grads
  b += 9LL * 2 * (p.n_d + mmax) + 8LL * mmax;     // tensor-core slices and K rows
  return b;
}

// Page-locked host staging buffer of a worker: host<->device copies of a
// batch's inputs and results run asynchronously on the worker's stream
// (from pageable memory they would be staged and synchronous).
template <typename T>
struct Pinned {
  T *p = nullptr;
  size_t n = 0;
  int ensure(size_t want) {
    if (want <= n) return FGB_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (cudaHostAlloc((void **)&p, sizeof(T) * want, cudaHostAllocDefault) !=
        cudaSuccess) {
      p = nullptr;
      set_error("serving: page-locked staging buffer of %zu bytes",
                sizeof(T) * want);
      return FGB_ENOMEM;
    }
    n = want;
    return FGB_OK;
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// A queued request passed over this many times (because it did not fit the
// memory left while later, smaller ones did) blocks the requests behind it
// until it is admitted.
constexpr int kMaxPassOvers = 4;

}  // namespace
}  // namespace fgb

using namespace fgb;

struct fgb_server_s {
  std::vector<fgb_model_s *> replicas;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::map<long long, std::unique_ptr<Request>> all;
  long long next_id = 1, in_flight_bytes = 0, budget = 0, bytes_per_atom = 0;
  long long completed = 0, batches = 0;
  int max_structures = 64, want = 0xF, precision = 0, device = 0;
  double cutoff = 0;
  bool stop = false;
};


// Admission: scan the queue in arrival order and take every request that
// fits the memory budget left (in-flight bytes of all workers) until the
// batch holds max_structures; a request that does not fit is passed over,
// at most kMaxPassOvers times, after which nothing behind it is taken
// before it.  Returns the batch's bytes (0: nothing fits now).
static long long admit(fgb_server_s *s, std::vector<Request *> &batch) {
  long long bytes = 0;
  bool blocked = false;
  for (auto it = s->queue.begin();
       it != s->queue.end() && (int)batch.size() < s->max_structures;) {
    Request *r = *it;
    if (s->in_flight_bytes + bytes + r->bytes <= s->budget) {
      bytes += r->bytes;
      batch.push_back(r);
      it = s->queue.erase(it);
      continue;
    }
    if (r->passed_over >= kMaxPassOvers) blocked = true;
    if (blocked) break;
    ++it;
  }
  if (!batch.empty())
    for (Request *r : s->queue) {
      if (r->t_submit > batch.back()->t_submit) break;
      r->passed_over++;
    }
  return bytes;
}

static bool any_fits(const fgb_server_s *s) {
  for (const Request *r : s->queue) {
    if (s->in_flight_bytes + r->bytes <= s->budget) return true;
    if (r->passed_over >= kMaxPassOvers) return false;
  }
  return false;
}

static void worker_loop(fgb_server_s *s, int w) {
  cudaSetDevice(s->device);
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  fgb_model_s *m = s->replicas[w];
  std::vector<int> offsets;
  std::vector<double> cells;
  Pinned<double> pos, energy, forces, stress, var;
  Pinned<int> species;
  for (;;) {
    std::vector<Request *> batch;
    long long bytes = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || any_fits(s); });
      if (s->stop) break;
      bytes = admit(s, batch);
      if (batch.empty()) continue;
      s->in_flight_bytes += bytes;
      s->batches++;
    }
    const int S = (int)batch.size();
    offsets.assign(S + 1, 0);
    for (int k = 0; k < S; k++) offsets[k + 1] = offsets[k] + batch[k]->n;
    const int N = offsets[S];
    int rc = FGB_OK;
    if ((rc = pos.ensure(3 * (size_t)N + 1)) ||
        (rc = species.ensure((size_t)N + 1)) ||
        (rc = energy.ensure((size_t)S + 1)) ||
        (rc = forces.ensure(3 * (size_t)N + 1)) ||
        (rc = stress.ensure(6 * (size_t)S + 1)) ||
        (rc = var.ensure((size_t)N + 1))) {
    } else {
      cells.resize(9 * S);
      for (int k = 0; k < S; k++) {
        std::copy(batch[k]->cell, batch[k]->cell + 9, cells.begin() + 9 * k);
        std::copy(batch[k]->pos.begin(), batch[k]->pos.end(),
                  pos.p + 3 * (size_t)offsets[k]);
        std::copy(batch[k]->species.begin(), batch[k]->species.end(),
                  species.p + offsets[k]);
      }
      std::fill(energy.p, energy.p + S, 0.0);
      std::fill(stress.p, stress.p + 6 * (size_t)S, 0.0);
      rc = fgb_predict_host(m, S, offsets.data(), cells.data(), pos.p,
                            species.p, s->cutoff, s->want, s->precision,
                            energy.p, forces.p, stress.p, var.p, st);
    }
    std::string err = rc ? fgb_last_error() : "";
    {
      std::lock_guard<std::mutex> lk(s->mu);
      auto now = Clock::now();
      for (int k = 0; k < S; k++) {
        Request *r = batch[k];
        r->status = rc;
        r->error = err;
        if (!rc) {
          r->energy = energy.p[k];
          std::copy(stress.p + 6 * k, stress.p + 6 * k + 6, r->stress);
          r->forces.assign(forces.p + 3 * (size_t)offsets[k],
                           forces.p + 3 * (size_t)offsets[k + 1]);
          r->var.assign(var.p + offsets[k], var.p + offsets[k + 1]);
        }
        r->t_done = now;
        r->done = true;
        s->completed++;
      }
      s->in_flight_bytes -= bytes;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  cudaStreamDestroy(st);
}

extern "C" int fgb_serve_start(fgb_server_t *out, fgb_model_t model,
                               int n_workers, long long memory_budget_bytes,
                               int max_structures, double cutoff, int want,
                               int precision) {
  if (!out || !model || n_workers < 1 || n_workers > 16 ||
      memory_budget_bytes <= 0 || max_structures < 1 || !(cutoff > 0)) {
    set_error("fgb_serve_start: invalid arguments");
    return FGB_EINVAL;
  }
  if (!model->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  fgb_server_s *s = new fgb_server_s();
  cudaGetDevice(&s->device);
  s->budget = memory_budget_bytes;
  s->bytes_per_atom = footprint_per_atom(model);
  s->max_structures = max_structures;
  s->cutoff = cutoff;
  s->want = want;
  s->precision = precision;
  for (int w = 0; w < n_workers; w++) {
    int rc = FGB_OK;
    fgb_model_s *m = model_replicate(model, rc);
    if (!m) {
      for (auto *r : s->replicas) delete r;
      delete s;
      return rc;
    }
    s->replicas.push_back(m);
  }
  for (int w = 0; w < n_workers; w++)
    s->workers.emplace_back(worker_loop, s, w);
  *out = s;
  return FGB_OK;
}

extern "C" int fgb_serve_submit(fgb_server_t s, int n_atoms,
                                const double *h_cell, const double *h_positions,
                                const int *h_species, long long *request_id) {
  if (!s || n_atoms < 0 || !h_cell || (n_atoms && (!h_positions || !h_species)) ||
      !request_id) {
    set_error("fgb_serve_submit: invalid arguments");
    return FGB_EINVAL;
  }
  long long bytes = std::max<long long>(1, n_atoms) * s->bytes_per_atom;
  if (bytes > s->budget) {
    set_error("fgb_serve_submit: a %d-atom structure needs %lld bytes, more "
              "than the %lld-byte memory budget", n_atoms, bytes, s->budget);
    return FGB_EINVAL;
  }
  std::unique_ptr<Request> r(new Request());
  r->n = n_atoms;
  std::copy(h_cell, h_cell + 9, r->cell);
  r->pos.assign(h_positions, h_positions + 3 * (size_t)n_atoms);
  r->species.assign(h_species, h_species + n_atoms);
  r->bytes = bytes;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) { set_error("fgb_serve_submit: server stopped"); return FGB_EINVAL; }
    r->id = s->next_id++;
    *request_id = r->id;
    s->queue.push_back(r.get());
    s->all[r->id] = std::move(r);
  }
  s->cv_work.notify_one();
  return FGB_OK;
}

extern "C" int fgb_serve_poll(fgb_server_t s, long long request_id, int *done,
                              double *h_energy, double *h_forces,
                              double *h_stress, double *h_local_var,
                              double *latency_ms) {
  if (!s || !done) { set_error("fgb_serve_poll: invalid arguments"); return FGB_EINVAL; }
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(request_id);
    if (it == s->all.end()) { set_error("fgb_serve_poll: unknown request %lld", request_id); return FGB_EINVAL; }
    if (!it->second->done) { *done = 0; return FGB_OK; }
    r = std::move(it->second);
    s->all.erase(it);
  }
  *done = 1;
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (r->status) {
    set_error("%s", r->error.c_str());
    return r->status;
  }
  if (h_energy) *h_energy = r->energy;
  if (h_stress) std::copy(r->stress, r->stress + 6, h_stress);
  if (h_forces) std::copy(r->forces.begin(), r->forces.end(), h_forces);
  if (h_local_var) std::copy(r->var.begin(), r->var.end(), h_local_var);
  return FGB_OK;
}

extern "C" int fgb_serve_stats(fgb_server_t s, long long *completed,
                               long long *batches, long long *bytes_per_atom) {
  if (!s) { set_error("fgb_serve_stats: null server"); return FGB_EINVAL; }
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (batches) *batches = s->batches;
  if (bytes_per_atom) *bytes_per_atom = s->bytes_per_atom;
  return FGB_OK;
}

extern "C" int fgb_serve_stop(fgb_server_t s) {
  if (!s) return FGB_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto *m : s->replicas) delete m;
  delete s;
  return FGB_OK;
}
