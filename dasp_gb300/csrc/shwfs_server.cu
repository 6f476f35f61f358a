// Serving loop: continuous batching of WFS-frame requests from many
// simulated AO systems on one GPU (shwfs_server_* in include/shwfs.h).
//
// One dispatcher thread owns every engine handle (handles are not
// thread-safe); callers only touch mutex-protected queues.  Each pass of the
// dispatcher
//   1. admits waiting systems, in arrival order, while their estimated device
//      footprint fits the HBM budget (the estimate is replaced by the handle's
//      real footprint once created);
//   2. retires finished frames (CUDA event query), copies their centroids to
//      the caller and records the latency;
//   3. launches every released request whose system is idle while fewer than
//      max_inflight frames are on the device, each system on its own stream.
// Requests of one system run in submission order (its integration state is
// sequential); requests of different systems overlap on the device.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/shwfs.h"
#include "engine_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id;
  const float* phs;
  bool phsDev;
  float* out;
  double release;
};

struct System {
  int id = 0;
  shwfs_init init{};
  int form = 0;
  int64_t estimate = 0, bytes = 0;
  bool admitted = false, failed = false, removing = false;
  std::string error;
  shwfs_handle* h = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  float* d_phs = nullptr;   // staging for host phases
  float* d_cents = nullptr;
  float* d_bimg = nullptr;
  float* h_cents = nullptr;  // pinned
  int* h_status = nullptr;   // pinned
  size_t nphs = 0, ncents = 0, nbimg = 0;
  std::deque<Request> queue;
  bool busy = false;
  Request cur{};
  int curReadout = 0;
};

int64_t numel(const shwfs_array& a) {
  int64_t n = 1;
  for (int i = 0; i < a.ndim; i++) n *= a.shape[i];
  return a.data ? n : 0;
}

// device bytes a system will hold, from its init (before the engine exists)
int64_t estimate_bytes(const shwfs_init& in, int form, int integMode) {
  const int64_t ns = in.nsubaps, p = in.phasesize, m = in.nimg;
  const int64_t phs = numel(in.phs), P = in.spotpsf.data ? in.spotpsf.shape[in.spotpsf.ndim - 1] : 0;
  const int64_t npsf = in.spotpsf.data ? (in.spotpsf.ndim == 4 ? ns : 1) : 0;
  int64_t b = 0;
  b += phs * 4;                                  // phase staging
  b += ns * 2 * 4 + ns * m * m * 4;              // cents, bimg
  b += ns * p * p * 4;                           // pupil
  b += npsf * P * P * 4 + npsf * P * (P / 2 + 1) * 8;  // PSFs and spectra
  b += ns * 64 + (int64_t)in.fftsize * 64 + 65536;     // lists, tables, small buffers
  if (in.skybrightnessArr.data) b += ns * m * m * 4;
  if (in.centWeight.data) b += numel(in.centWeight) * 4;
  if (form != SHWFS_FORM_FP32) b += 4 << 20;     // GEMM-DFT constants
  if (integMode == SHWFS_INTEG_PHYSICAL) b += 2 * ns * m * m * 4;  // sub-exposure and exposure sum
  return b;
}

}  // namespace

struct shwfs_server {
  shwfs_server_config cfg{};
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  std::vector<std::unique_ptr<System>> systems;  // index = id
  std::deque<shwfs_completion> done;
  int64_t used = 0;
  int inflight = 0;
  uint64_t nextReq = 1, submitted = 0, completed = 0;
  bool stop = false;
  bool wake = false;
  std::thread worker;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // ---- dispatcher-thread helpers (called with mu released unless noted) ----
  void release_system(System& s) {
    if (s.h) shwfs_free(s.h);
    s.h = nullptr;
    if (s.ev) cudaEventDestroy(s.ev);
    if (s.st) cudaStreamDestroy(s.st);
    if (s.d_phs) cudaFree(s.d_phs);
    if (s.d_cents) cudaFree(s.d_cents);
    if (s.d_bimg) cudaFree(s.d_bimg);
    if (s.h_cents) cudaFreeHost(s.h_cents);
    if (s.h_status) cudaFreeHost(s.h_status);
    s.ev = nullptr;
    s.st = nullptr;
    s.d_phs = s.d_cents = s.d_bimg = s.h_cents = nullptr;
    s.h_status = nullptr;
  }

  // create the engine of an admitted system; false (with s.error) on failure
  bool create_system(System& s) {
    s.nphs = (size_t)numel(s.init.phs);
    s.ncents = (size_t)s.init.nsubaps * 2;
    s.nbimg = (size_t)s.init.nsubaps * s.init.nimg * s.init.nimg;
    auto cuda_ok = [&](cudaError_t e, const char* what) {
      if (e == cudaSuccess) return true;
      s.error = std::string(what) + ": " + cudaGetErrorString(e);
      return false;
    };
    if (!cuda_ok(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking), "stream")) return false;
    if (!cuda_ok(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming), "event")) return false;
    if (!cuda_ok(cudaMalloc((void**)&s.d_phs, s.nphs * 4), "phase buffer")) return false;
    if (!cuda_ok(cudaMalloc((void**)&s.d_cents, s.ncents * 4), "cents buffer")) return false;
    if (!cuda_ok(cudaMalloc((void**)&s.d_bimg, s.nbimg * 4), "bimg buffer")) return false;
    if (!cuda_ok(cudaMemset(s.d_phs, 0, s.nphs * 4), "memset")) return false;
    if (!cuda_ok(cudaMallocHost((void**)&s.h_cents, s.ncents * 4), "pinned cents")) return false;
    if (!cuda_ok(cudaMallocHost((void**)&s.h_status, sizeof(int)), "pinned status")) return false;
    shwfs_init in = s.init;
    in.phs.data = s.d_phs;
    in.phs.on_device = 1;
    in.cents.data = s.d_cents;
    in.cents.on_device = 1;
    in.bimg.data = s.d_bimg;
    in.bimg.on_device = 1;
    if (shwfs_initialise(&in, &s.h) != SHWFS_OK) {
      s.error = shwfs_last_error();
      return false;
    }
    if (s.form != SHWFS_FORM_FP32) {
      shwfs_value v{};
      v.kind = SHWFS_VAL_INT;
      v.ival = s.form;
      if (shwfs_update(s.h, SHWFS_FORM, &v) != SHWFS_OK) {
        s.error = shwfs_last_error();
        return false;
      }
    }
    if (cfg.integration_mode != SHWFS_INTEG_COMPAT) {
      shwfs_value v{};
      v.kind = SHWFS_VAL_INT;
      v.ival = cfg.integration_mode;
      if (shwfs_update(s.h, SHWFS_INTEGMODE, &v) != SHWFS_OK) {
        s.error = shwfs_last_error();
        return false;
      }
    }
    s.bytes = shwfs::engine_device_bytes(s.h) + (int64_t)(s.nphs + s.ncents + s.nbimg) * 4;
    return true;
  }

  void complete(System& s, int status, int readout, double release) {
    shwfs_completion c{};
    c.request = s.cur.id;
    c.system = s.id;
    c.status = status;
    c.readout = readout;
    c.done_s = now();
    c.latency_s = c.done_s - release;
    std::lock_guard<std::mutex> lk(mu);
    done.push_back(c);
    completed++;
    cv.notify_all();
  }

  void run_loop() {
    cudaSetDevice(cfg.device);
    while (true) {
      bool progress = false;
      std::vector<System*> admitNow, toRemove;
      // the systems of this pass: add_system may grow `systems` (and move its
      // storage) at any time, so the pass walks a copy of the pointers taken
      // under the lock; each System stays where it is until the server goes
      std::vector<System*> snap;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (stop) break;
        wake = false;
        snap.reserve(systems.size());
        for (auto& sp : systems) snap.push_back(sp.get());
        // 1. admission in arrival order, against the budget
        for (auto& sp : systems) {
          System& s = *sp;
          if (s.admitted || s.failed || s.removing) continue;
          if (used + s.estimate > cfg.hbm_budget_bytes) break;  // keep arrival order
          used += s.estimate;
          s.admitted = true;
          admitNow.push_back(&s);
        }
        for (auto& sp : systems)
          if (sp->removing && sp->admitted && !sp->busy && !sp->failed) toRemove.push_back(sp.get());
      }
      for (System* s : admitNow) {
        const bool ok = create_system(*s);
        std::deque<Request> dropped;
        {
          std::lock_guard<std::mutex> lk(mu);
          used -= s->estimate;
          if (ok) {
            used += s->bytes;
          } else {
            s->failed = true;
            s->admitted = false;
            dropped.swap(s->queue);
          }
        }
        if (!ok) {
          release_system(*s);
          // its queued frames complete with the creation failure
          for (const Request& r : dropped) {
            s->cur = r;
            complete(*s, SHWFS_ERR_CUDA, 0, r.release);
          }
        }
        progress = true;
      }
      for (System* s : toRemove) {
        release_system(*s);
        std::lock_guard<std::mutex> lk(mu);
        used -= s->bytes;
        s->admitted = false;
        s->failed = true;  // gone for good
        progress = true;
      }
      // 2. retire finished frames
      for (System* sp : snap) {
        System& s = *sp;
        if (!s.busy) continue;
        const cudaError_t q = cudaEventQuery(s.ev);
        if (q == cudaErrorNotReady) continue;
        int status = SHWFS_OK;
        if (q != cudaSuccess) {
          status = SHWFS_ERR_CUDA;
        } else if (s.curReadout) {
          if (*s.h_status & 2) status = SHWFS_ERR_STATE;
          if (s.cur.out) memcpy(s.cur.out, s.h_cents, s.ncents * 4);
        }
        s.busy = false;
        {
          std::lock_guard<std::mutex> lk(mu);
          inflight--;
        }
        complete(s, status, s.curReadout, s.cur.release);
        progress = true;
      }
      // 3. launch released requests of idle systems
      const double tnow = now();
      for (System* sp : snap) {
        System& s = *sp;
        Request r{};
        {
          std::lock_guard<std::mutex> lk(mu);
          if (!s.admitted || s.busy || s.failed || s.queue.empty() || inflight >= cfg.max_inflight) continue;
          if (s.queue.front().release > tnow) continue;
          r = s.queue.front();
          s.queue.pop_front();
          inflight++;
        }
        s.cur = r;
        s.busy = true;
        const float* ph = r.phs;
        int status = SHWFS_OK;
        if (!r.phsDev) {
          if (cudaMemcpyAsync(s.d_phs, r.phs, s.nphs * 4, cudaMemcpyHostToDevice, s.st) != cudaSuccess)
            status = SHWFS_ERR_CUDA;
          ph = s.d_phs;
        }
        if (status == SHWFS_OK && shwfs::engine_frame(s.h, ph, s.st, &s.curReadout) != SHWFS_OK) status = SHWFS_ERR_CUDA;
        if (status == SHWFS_OK && s.curReadout) {
          if (cudaMemcpyAsync(s.h_cents, s.d_cents, s.ncents * 4, cudaMemcpyDeviceToHost, s.st) != cudaSuccess ||
              cudaMemcpyAsync(s.h_status, shwfs::engine_status_ptr(s.h), sizeof(int), cudaMemcpyDeviceToHost,
                              s.st) != cudaSuccess)
            status = SHWFS_ERR_CUDA;
        }
        if (status == SHWFS_OK && cudaEventRecord(s.ev, s.st) != cudaSuccess) status = SHWFS_ERR_CUDA;
        if (status != SHWFS_OK) {
          s.busy = false;
          {
            std::lock_guard<std::mutex> lk(mu);
            inflight--;
          }
          complete(s, status, 0, r.release);
        }
        progress = true;
      }
      if (!progress) {
        std::unique_lock<std::mutex> lk(mu);
        if (!stop && !wake) cv.wait_for(lk, std::chrono::microseconds(inflight > 0 ? 5 : 200));
      }
    }
    // drain: wait for frames on the device, then free everything
    std::vector<System*> all;
    {
      std::lock_guard<std::mutex> lk(mu);
      for (auto& sp : systems) all.push_back(sp.get());
    }
    for (System* sp : all) {
      if (sp->st) cudaStreamSynchronize(sp->st);
      release_system(*sp);
    }
  }
};

extern "C" {

shwfs_status shwfs_server_create(const shwfs_server_config* cfg, shwfs_server** out) {
  if (!cfg || !out || cfg->hbm_budget_bytes <= 0 || cfg->max_inflight < 1)
    return shwfs::engine_fail(SHWFS_ERR_INVALID, "server needs a positive HBM budget and max_inflight >= 1");
  if (cfg->integration_mode != SHWFS_INTEG_COMPAT && cfg->integration_mode != SHWFS_INTEG_PHYSICAL)
    return shwfs::engine_fail(SHWFS_ERR_INVALID, "unknown integration mode");
  shwfs_server* s = new shwfs_server;
  s->cfg = *cfg;
  s->t0 = Clock::now();
  s->worker = std::thread([s] { s->run_loop(); });
  *out = s;
  return SHWFS_OK;
}

shwfs_status shwfs_server_add_system(shwfs_server* s, const shwfs_init* init, int form, int* system) {
  if (!s || !init || !system || form < SHWFS_FORM_FP32 || form > SHWFS_FORM_TF32)
    return shwfs::engine_fail(SHWFS_ERR_INVALID, "bad add_system arguments");
  if (!init->phs.data || !init->cents.data || !init->bimg.data)
    return shwfs::engine_fail(SHWFS_ERR_INVALID, "phs, cents and bimg must give the system's shapes");
  auto sys = std::make_unique<System>();
  sys->init = *init;
  sys->form = form;
  sys->estimate = estimate_bytes(*init, form, s->cfg.integration_mode);
  std::lock_guard<std::mutex> lk(s->mu);
  if (sys->estimate > s->cfg.hbm_budget_bytes)
    return shwfs::engine_fail(SHWFS_ERR_NOMEM, "system needs more device memory than the whole HBM budget");
  sys->id = (int)s->systems.size();
  *system = sys->id;
  s->systems.push_back(std::move(sys));
  s->wake = true;
  s->cv.notify_all();
  return SHWFS_OK;
}

shwfs_status shwfs_server_remove_system(shwfs_server* s, int system) {
  if (!s) return SHWFS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (system < 0 || system >= (int)s->systems.size()) return SHWFS_ERR_INVALID;
  System& sys = *s->systems[system];
  sys.removing = true;
  // frames still queued will not run: each completes with SHWFS_ERR_STATE so
  // that every submitted request is reported exactly once
  const double t = s->now();
  for (const auto& r : sys.queue) {
    shwfs_completion c{};
    c.request = r.id;
    c.system = sys.id;
    c.status = SHWFS_ERR_STATE;
    c.readout = 0;
    c.done_s = t;
    c.latency_s = t - r.release;
    s->done.push_back(c);
    s->completed++;
  }
  sys.queue.clear();
  if (!sys.admitted) sys.failed = true;
  s->wake = true;
  s->cv.notify_all();
  return SHWFS_OK;
}

shwfs_status shwfs_server_submit(shwfs_server* s, int system, const float* phs, int phs_on_device, float* out_cents,
                                 double release_s, uint64_t* request) {
  if (!s || !phs) return shwfs::engine_fail(SHWFS_ERR_INVALID, "null server or phase");
  std::lock_guard<std::mutex> lk(s->mu);
  if (system < 0 || system >= (int)s->systems.size()) return shwfs::engine_fail(SHWFS_ERR_INVALID, "no such system");
  System& sys = *s->systems[system];
  if (sys.removing) return shwfs::engine_fail(SHWFS_ERR_STATE, "system is being removed");
  if (sys.failed)
    return shwfs::engine_fail(SHWFS_ERR_STATE, ("system could not be started: " + sys.error).c_str());
  Request r{};
  r.id = s->nextReq++;
  r.phs = phs;
  r.phsDev = phs_on_device != 0;
  r.out = out_cents;
  r.release = release_s > 0 ? release_s : s->now();
  sys.queue.push_back(r);
  s->submitted++;
  if (request) *request = r.id;
  s->wake = true;
  s->cv.notify_all();
  return SHWFS_OK;
}

shwfs_status shwfs_server_poll(shwfs_server* s, shwfs_completion* out, int max, int* n) {
  if (!s || !n || (max > 0 && !out)) return SHWFS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  int k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return SHWFS_OK;
}

shwfs_status shwfs_server_get_stats(shwfs_server* s, shwfs_server_stats* st) {
  if (!s || !st) return SHWFS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(st, 0, sizeof(*st));
  for (auto& sp : s->systems) {
    st->systems++;
    if (sp->admitted) st->admitted++;
    else if (!sp->failed && !sp->removing) st->pending++;
  }
  st->used_bytes = s->used;
  st->budget_bytes = s->cfg.hbm_budget_bytes;
  st->inflight = s->inflight;
  st->submitted = s->submitted;
  st->completed = s->completed;
  return SHWFS_OK;
}

double shwfs_server_clock(shwfs_server* s) { return s ? s->now() : 0.0; }

shwfs_status shwfs_server_destroy(shwfs_server* s) {
  if (!s) return SHWFS_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  delete s;
  return SHWFS_OK;
}

}  // extern "C"
