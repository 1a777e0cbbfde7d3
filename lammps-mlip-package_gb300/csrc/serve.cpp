// Serving loop: energy + force + stress requests for periodic structures of
// different sizes, evaluated by continuous batching on one GPU.
//
// Requests are queued by mlipg_server_submit (any thread).  One worker
// thread admits queued requests in arrival order while their estimated
// device footprint fits the memory budget, groups them by precision into
// batches of at most `max_batch_atoms` atoms (a separate, smaller cap for
// FP64 batches: an FP64 evaluation costs some twenty times a mixed one of
// the same size, and one long FP64 batch would hold every request queued
// behind it; a precision whose batch is full stops taking requests while
// the other one keeps being admitted in arrival order), builds the image-coded
// neighbour lists and launches each batch (one persistent launch over all
// its cells) on the stream of that precision's handle.  Batches stay
// resident on the device (positions, lists, outputs) until their results
// are copied out; requests that arrive while others are on the GPU are
// admitted as soon as budget frees and queue behind them on the stream, and
// FP64 and mixed batches run on two streams concurrently; batch buffers come
// from the stream-ordered pool, so nothing synchronises the device.  A
// request's energy is reduced per cell in a fixed order and does not depend
// on which other requests share its batch; forces and virial agree with a
// lone evaluation to the rounding of the force accumulation.  Waits have
// deadlines (MLIPG_ETIMEDOUT).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/mlipg.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long ticket;
  int natoms;
  int precision;
  double lattice[9];
  std::vector<double> x;
  std::vector<int> elements;
  Clock::time_point t_submit, t_done;
  size_t est_bytes = 0;
  bool done = false;
  int status = MLIPG_OK;
  double energy = 0;
  double virial[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> forces;
};

struct InFlight {
  mlipg_batch* batch = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<std::shared_ptr<Request>> reqs;
  size_t bytes = 0;
};

// default cap of FP64 batches (atoms); mlipg_server_set_batch_atoms changes it
constexpr int kDefaultFp64BatchAtoms = 8192;

size_t estimate_bytes(int natoms, double cutoff) {
  // positions/forces/energies/virials per atom + ~density * sphere neighbours
  const double nbar = 0.1 * 4.18879 * cutoff * cutoff * cutoff;   // generous density 0.1/A^3
  return (size_t)natoms * (128 + (size_t)(8 * nbar)) + 256;
}

}  // namespace

struct mlipg_server {
  mlipg_handle* h[2] = {nullptr, nullptr};   // FP64, mixed
  size_t budget = 0;
  int max_batch_atoms[2] = {0, 0};            // FP64, mixed
  double cutoff = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<long long, std::shared_ptr<Request>> all;
  std::vector<InFlight> inflight;
  size_t used = 0;
  long long next_ticket = 1;
  bool stop = false;
  std::thread worker;
  // statistics
  std::vector<double> latencies_ms;
  long long atoms_done = 0, batches = 0;
  Clock::time_point t_first, t_last;
  bool have_first = false;
  int worker_error = MLIPG_OK;
  int device = 0;
};

static void fulfil(mlipg_server* s, InFlight& f, int rc) {
  std::vector<double> e(f.reqs.size()), v(6 * f.reqs.size());
  int natoms = 0;
  mlipg_batch_sizes(f.batch, &natoms, nullptr);
  std::vector<double> forces((size_t)natoms * 3);
  if (rc == MLIPG_OK) rc = mlipg_batch_results(f.batch, e.data(), forces.data(), v.data());
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lock(s->mu);
  size_t off = 0;
  for (size_t k = 0; k < f.reqs.size(); ++k) {
    Request& r = *f.reqs[k];
    r.status = rc;
    r.energy = e[k];
    for (int q = 0; q < 6; ++q) r.virial[q] = v[6 * k + q];
    r.forces.assign(forces.begin() + off, forces.begin() + off + 3 * (size_t)r.natoms);
    off += 3 * (size_t)r.natoms;
    r.t_done = now;
    r.done = true;
    s->latencies_ms.push_back(
        std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count());
    s->atoms_done += r.natoms;
    s->t_last = now;
  }
  s->used -= f.bytes;
  s->batches++;
  s->cv_done.notify_all();
  s->cv_work.notify_all();
}

static void worker_loop(mlipg_server* s) {
  cudaSetDevice(s->device);   // the handles live on the creating thread's device
  while (true) {
    // 1. admission: arrival order, budget, per-precision batch size cap
    std::vector<std::shared_ptr<Request>> take[2];
    size_t take_bytes[2] = {0, 0};
    {
      std::unique_lock<std::mutex> lock(s->mu);
      if (s->queue.empty() && s->inflight.empty()) {
        if (s->stop) return;
        s->cv_work.wait_for(lock, std::chrono::milliseconds(2));
        continue;
      }
      // arrival order; the budget is shared (a request that does not fit stops
      // all admission, an oversized one runs alone), the batch caps are per
      // precision (a full batch closes its precision only)
      int atoms[2] = {0, 0};
      bool closed[2] = {false, false};
      for (auto it = s->queue.begin(); it != s->queue.end() && !(closed[0] && closed[1]);) {
        auto& r = *it;
        const int p = r->precision == MLIPG_PREC_FP64 ? 0 : 1;
        if (closed[p]) {
          ++it;
          continue;
        }
        const bool fits = s->used + take_bytes[0] + take_bytes[1] + r->est_bytes <= s->budget;
        const bool alone = s->inflight.empty() && take[0].empty() && take[1].empty();
        if (!fits && !alone) break;   // wait for memory; an oversized request runs alone
        if (!take[p].empty() && atoms[p] + r->natoms > s->max_batch_atoms[p]) {
          closed[p] = true;
          ++it;
          continue;
        }
        atoms[p] += r->natoms;
        take_bytes[p] += r->est_bytes;
        take[p].push_back(r);
        it = s->queue.erase(it);
      }
      s->used += take_bytes[0] + take_bytes[1];
    }
    // 2. build + launch the admitted batches (host work overlaps the GPU)
    for (int p = 0; p < 2; ++p) {
      if (take[p].empty()) continue;
      std::vector<int> n;
      std::vector<double> lat, x;
      std::vector<int> el;
      for (auto& r : take[p]) {
        n.push_back(r->natoms);
        lat.insert(lat.end(), r->lattice, r->lattice + 9);
        x.insert(x.end(), r->x.begin(), r->x.end());
        el.insert(el.end(), r->elements.begin(), r->elements.end());
      }
      InFlight f;
      f.reqs = take[p];
      f.bytes = take_bytes[p];
      int rc = mlipg_batch_create(s->h[p], (int)n.size(), n.data(), lat.data(), x.data(),
                                  el.data(), &f.batch);
      if (rc == MLIPG_OK) rc = mlipg_batch_launch(f.batch);
      if (rc == MLIPG_OK &&
          (cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming) != cudaSuccess ||
           cudaEventRecord(f.done, static_cast<cudaStream_t>(mlipg_stream(s->h[p]))) !=
               cudaSuccess))
        rc = MLIPG_ECUDA;
      if (rc != MLIPG_OK) {
        if (f.batch) fulfil(s, f, rc);
        else {
          std::lock_guard<std::mutex> lock(s->mu);
          for (auto& r : f.reqs) {
            r->status = rc;
            r->done = true;
          }
          s->used -= f.bytes;
          s->cv_done.notify_all();
        }
        if (f.batch) mlipg_batch_destroy(f.batch);
        if (f.done) cudaEventDestroy(f.done);
        continue;
      }
      std::lock_guard<std::mutex> lock(s->mu);
      s->inflight.push_back(std::move(f));
    }
    // 3. retire finished batches
    std::vector<InFlight> finished;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      for (size_t k = 0; k < s->inflight.size();) {
        const cudaError_t q = cudaEventQuery(s->inflight[k].done);
        if (q == cudaSuccess || (q != cudaErrorNotReady)) {
          finished.push_back(std::move(s->inflight[k]));
          s->inflight.erase(s->inflight.begin() + k);
        } else {
          ++k;
        }
      }
    }
    for (auto& f : finished) {
      fulfil(s, f, MLIPG_OK);
      mlipg_batch_destroy(f.batch);
      cudaEventDestroy(f.done);
    }
    if (finished.empty() && take[0].empty() && take[1].empty())
      std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

extern "C" int mlipg_server_create(const char* potential_path, size_t device_budget_bytes,
                                   int max_batch_atoms, mlipg_server** out) {
  if (!potential_path || !out || device_budget_bytes == 0 || max_batch_atoms <= 0)
    return MLIPG_EINVAL;
  *out = nullptr;
  mlipg_server* s = new mlipg_server();
  cudaGetDevice(&s->device);
  for (int p = 0; p < 2; ++p) {
    const int rc = mlipg_create(potential_path, p == 0 ? MLIPG_PREC_FP64 : MLIPG_PREC_MIXED,
                                &s->h[p]);
    if (rc != MLIPG_OK || !mlipg_stream(s->h[p])) {
      for (auto* h : s->h) mlipg_destroy(h);
      delete s;
      return rc != MLIPG_OK ? rc : MLIPG_ENOGPU;
    }
  }
  s->budget = device_budget_bytes;
  s->max_batch_atoms[1] = max_batch_atoms;
  s->max_batch_atoms[0] = std::min(max_batch_atoms, kDefaultFp64BatchAtoms);
  s->cutoff = mlipg_cutoff(s->h[0]);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return MLIPG_OK;
}

extern "C" int mlipg_server_set_batch_atoms(mlipg_server* s, int precision, int max_atoms) {
  if (!s || max_atoms <= 0 || (precision != MLIPG_PREC_FP64 && precision != MLIPG_PREC_MIXED))
    return MLIPG_EINVAL;
  std::lock_guard<std::mutex> lock(s->mu);
  s->max_batch_atoms[precision == MLIPG_PREC_FP64 ? 0 : 1] = max_atoms;
  return MLIPG_OK;
}

extern "C" int mlipg_server_submit(mlipg_server* s, int natoms, const double* lattice9,
                                   const double* x, const int* elements, int precision,
                                   long long* ticket) {
  if (!s || natoms <= 0 || !lattice9 || !x || !elements || !ticket ||
      (precision != MLIPG_PREC_FP64 && precision != MLIPG_PREC_MIXED))
    return MLIPG_EINVAL;
  auto r = std::make_shared<Request>();
  r->natoms = natoms;
  r->precision = precision;
  std::memcpy(r->lattice, lattice9, sizeof r->lattice);
  r->x.assign(x, x + 3 * (size_t)natoms);
  r->elements.assign(elements, elements + natoms);
  r->est_bytes = estimate_bytes(natoms, s->cutoff);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->all[r->ticket] = r;
    s->queue.push_back(r);
    if (!s->have_first) {
      s->t_first = r->t_submit;
      s->have_first = true;
    }
  }
  s->cv_work.notify_one();
  return MLIPG_OK;
}

extern "C" int mlipg_server_wait(mlipg_server* s, long long ticket, int timeout_ms,
                                 double* energy, double* forces, double* virial6) {
  if (!s) return MLIPG_EINVAL;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return MLIPG_EINVAL;
  auto r = it->second;
  const bool ok = s->cv_done.wait_for(lock, std::chrono::milliseconds(std::max(timeout_ms, 0)),
                                      [&] { return r->done; });
  if (!ok) return MLIPG_ETIMEDOUT;
  if (r->status != MLIPG_OK) return r->status;
  if (energy) *energy = r->energy;
  if (virial6) std::memcpy(virial6, r->virial, sizeof r->virial);
  if (forces) std::memcpy(forces, r->forces.data(), r->forces.size() * sizeof(double));
  s->all.erase(it);
  return MLIPG_OK;
}

// out8: completed requests, p50 latency (ms), p99 latency (ms), atom-steps/s
// over first submit .. last completion, batches launched, device bytes in
// use, queued requests, requests in flight
extern "C" int mlipg_server_stats(mlipg_server* s, double* out8) {
  if (!s || !out8) return MLIPG_EINVAL;
  std::lock_guard<std::mutex> lock(s->mu);
  std::vector<double> l = s->latencies_ms;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    const size_t k = std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5));
    return l[k];
  };
  const double span =
      s->have_first ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0.0;
  size_t infl = 0;
  for (auto& f : s->inflight) infl += f.reqs.size();
  out8[0] = (double)l.size();
  out8[1] = pct(0.50);
  out8[2] = pct(0.99);
  out8[3] = span > 0 ? s->atoms_done / span : 0.0;
  out8[4] = (double)s->batches;
  out8[5] = (double)s->used;
  out8[6] = (double)s->queue.size();
  out8[7] = (double)infl;
  return MLIPG_OK;
}

extern "C" void mlipg_server_destroy(mlipg_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& f : s->inflight) {
    mlipg_batch_destroy(f.batch);
    cudaEventDestroy(f.done);
  }
  for (auto* h : s->h) mlipg_destroy(h);
  delete s;
}
