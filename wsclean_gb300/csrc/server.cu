// Request server: continuous batching of inversion / prediction requests on
// one GPU.
//
// Takes the place of GriddingTaskManager / ThreadedScheduler on this path
// (scheduling/griddingtaskmanager.cpp:26-103, threadedscheduler.cpp:12-228),
// which hand gridding tasks to a pool of CPU threads.  Here `max_active` worker
// threads each run one request at a time on gridders that own their own CUDA
// streams, so admitted requests overlap on the device; a request's failure is
// returned to whoever waits for it, as the threaded scheduler forwards a
// task's exception to its caller.
//
// Admission: the queue is scanned in arrival order.  A request whose session
// is running (or has an earlier request still queued) is passed over without
// holding back the ones behind it; otherwise the first request whose device
// memory does not fit stops the scan for every request that would need new
// memory, so a large request is not overtaken indefinitely.  With nothing
// running, the first eligible request is admitted whatever its size.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "wgpu_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Ticket {
  wgpu_request_t req;
  uint64_t id = 0;
  double bytes = 0;  // estimated device memory of the request
  double need = 0;   // memory charged at admission (0 for a resident session)
  Clock::time_point submitted, started, finished;
  int status = WGPU_OK;
  std::string error;
  bool done = false;
  bool held = false;  // passed over at least once for lack of device memory
};

struct Session {
  wgpu_gridder_t *g = nullptr;
  bool bound = false;
  bool busy = false;
  size_t n_rows = 0, n_chan = 0;  // shape of the bound set
  double bytes = 0;  // device memory held between requests
  ~Session() {
    if (g) wgpu_gridder_destroy(g);
  }
};

// Device bytes a request needs: the sorted records, permutation, keys and
// inputs (about 64 B per sample), uvw, the w-plane batch with its column
// buffers, the image buffers, the bucket offsets, and a fixed allowance.
double estimate_bytes(const wgpu_request_t &r, double plane_budget) {
  double fmin = 1e300, fmax = 0;
  for (size_t c = 0; c < r.n_chan; ++c) {
    fmin = std::min(fmin, r.freq[c]);
    fmax = std::max(fmax, r.freq[c]);
  }
  double w_min = 0, w_max = 0;
  for (size_t i = 0; i < r.n_rows; ++i) {
    const double w = r.uvw[3 * i + 2];
    const double a = w * fmin / wgpu::kSpeedOfLight, b = w * fmax / wgpu::kSpeedOfLight;
    w_min = std::min(w_min, std::min(a, b));
    w_max = std::max(w_max, std::max(a, b));
  }
  wgpu_plan_request_t q;
  std::memset(&q, 0, sizeof(q));
  q.width = (int64_t)r.width_t;
  q.height = (int64_t)r.height_t;
  q.dl = r.pixel_size_x;
  q.dm = r.pixel_size_y;
  q.l_shift = r.l_shift;
  q.m_shift = r.m_shift;
  q.epsilon = r.epsilon;
  q.w_min = w_min;
  q.w_max = w_max;
  q.n_vis = (int64_t)(r.n_rows * r.n_chan);
  q.memory_budget_bytes = plane_budget;
  const wgpu_plan_t p = wgpu::make_plan(q);
  const double n = (double)r.n_rows * (double)r.n_chan;
  const double spill = (double)(p.support - 1) * (2.0 * p.tile + p.support - 1) /
                       ((double)p.tile * p.tile);
  const double planes = (double)p.plane_batch * 8.0 * (double)p.nu * (double)p.nv * (1.0 + spill);
  const double rows = (double)p.plane_batch * 8.0 * (double)p.nv * (double)((p.width + 31) / 32 * 32);
  const double img = 40.0 * (double)r.width * (double)r.height;
  const double keys = 4.0 * (double)(p.nu / p.tile) * (double)(p.nv / p.tile) * 4.0 * (double)p.n_planes;
  return 64.0 * n + 24.0 * (double)r.n_rows + planes + rows + img + keys + 64e6;
}

}  // namespace

struct wgpu_server {
  double budget = 0;
  double plane_budget = 0;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv;       // queue, memory or session state changed
  std::condition_variable done_cv;  // a request finished
  std::deque<std::shared_ptr<Ticket>> queue;
  std::map<uint64_t, std::shared_ptr<Ticket>> tickets;
  std::map<uint64_t, std::shared_ptr<Session>> sessions;
  double used = 0, peak_used = 0;
  int running = 0, peak_running = 0;
  uint64_t next_id = 1;
  bool stopping = false;
  std::vector<std::thread> workers;
  uint64_t completed = 0, failed = 0, held_for_memory = 0;
  double vis_done = 0;
  Clock::time_point first_submit, last_finish;
  bool any_submit = false;

  // Next admissible request (caller holds mu); null if none.
  std::shared_ptr<Ticket> pick() {
    std::set<uint64_t> blocked;  // sessions with an earlier request waiting
    bool memory_blocked = false;
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      const auto &t = *it;
      const uint64_t sid = t->req.session;
      double need = t->bytes;
      if (sid != 0) {
        auto s = sessions.find(sid);
        const bool busy = s != sessions.end() && s->second->busy;
        if (busy || blocked.count(sid)) {
          blocked.insert(sid);
          continue;
        }
        if (s != sessions.end() && s->second->bound) need = 0;
      }
      const bool fits = used + need <= budget || running == 0;
      if (need > 0 && (memory_blocked || !fits)) {
        memory_blocked = true;
        if (!t->held) {
          t->held = true;
          ++held_for_memory;
        }
        if (sid != 0) blocked.insert(sid);
        continue;
      }
      auto picked = t;
      picked->need = need;
      queue.erase(it);
      return picked;
    }
    return nullptr;
  }

  void run_worker();
  void execute(Ticket &t);
};

void wgpu_server::execute(Ticket &t) {
  const wgpu_request_t &r = t.req;
  auto check = [](int st) {
    if (st != WGPU_OK) throw wgpu::Error(st, wgpu_last_error());
  };
  // precision as WGriddingMSGridder::MakeGridder picks it
  // (wgridder/wgriddingmsgridder.cpp:41-54)
  const int prec = r.epsilon <= 1.01e-5 ? 8 : 4;
  auto create = [&](wgpu_gridder_t **g) {
    check(wgpu_gridder_create(r.width, r.height, r.width_t, r.height_t, r.pixel_size_x,
                              r.pixel_size_y, r.l_shift, r.m_shift, 1, r.epsilon, 0, 0, prec, g));
    check(wgpu_gridder_set_plane_budget(*g, plane_budget));
  };
  std::unique_ptr<wgpu_gridder_t, void (*)(wgpu_gridder_t *)> own(nullptr, wgpu_gridder_destroy);
  wgpu_gridder_t *g = nullptr;
  std::shared_ptr<Session> sess;
  if (r.session != 0) {
    {
      std::lock_guard<std::mutex> lock(mu);
      sess = sessions[r.session];
    }
    if (!sess->bound) {
      if (!sess->g) create(&sess->g);
      const int st = wgpu_gridder_bind(sess->g, r.n_rows, r.n_chan, r.uvw, r.freq, r.mask);
      if (st != WGPU_OK) {
        const std::string msg = wgpu_last_error();
        wgpu_gridder_destroy(sess->g);
        sess->g = nullptr;
        throw wgpu::Error(st, msg);
      }
      sess->bound = true;
      sess->n_rows = r.n_rows;
      sess->n_chan = r.n_chan;
    } else if (r.n_rows != sess->n_rows || r.n_chan != sess->n_chan) {
      throw wgpu::Error(WGPU_ERR_INVALID, "request shape differs from its session's bound set");
    }
    g = sess->g;
  } else {
    wgpu_gridder_t *tmp = nullptr;
    create(&tmp);
    own.reset(tmp);
    g = tmp;
  }
  if (r.kind == WGPU_REQUEST_INVERT) {
    check(wgpu_gridder_initialize_inversion(g));
    if (r.session != 0) {
      check(wgpu_gridder_invert_bound(g, r.vis));
    } else if (r.mask) {
      throw wgpu::Error(WGPU_ERR_INVALID, "a sample mask needs a session (bound set)");
    } else {
      check(wgpu_gridder_add_inversion_data(g, r.n_rows, r.n_chan, r.uvw, r.freq, r.vis));
    }
    check(wgpu_gridder_finalize_image(g, r.image_factor));
    if (r.image_out) check(wgpu_gridder_real_image(g, r.image_out));
  } else {
    check(wgpu_gridder_initialize_prediction(g, r.model));
    if (r.session != 0) {
      check(wgpu_gridder_predict_bound(g, r.vis_out));
    } else if (r.mask) {
      check(wgpu_gridder_predict_visibilities_masked(g, r.n_rows, r.n_chan, r.uvw, r.freq,
                                                     r.mask, r.vis_out));
    } else {
      check(wgpu_gridder_predict_visibilities(g, r.n_rows, r.n_chan, r.uvw, r.freq, r.vis_out));
    }
  }
}

void wgpu_server::run_worker() {
  cudaSetDevice(device);
  for (;;) {
    std::shared_ptr<Ticket> t;
    std::shared_ptr<Session> sess;
    {
      std::unique_lock<std::mutex> lock(mu);
      cv.wait(lock, [&] { return (t = pick()) != nullptr || (stopping && queue.empty()); });
      if (!t) return;
      used += t->need;
      ++running;
      peak_used = std::max(peak_used, used);
      peak_running = std::max(peak_running, running);
      if (t->req.session != 0) {
        auto &s = sessions[t->req.session];
        if (!s) s = std::make_shared<Session>();
        s->busy = true;
        sess = s;
      }
      t->started = Clock::now();
    }
    try {
      execute(*t);
      t->status = WGPU_OK;
    } catch (const wgpu::Error &e) {
      t->status = e.status;
      t->error = e.what();
    } catch (const std::bad_alloc &) {
      t->status = WGPU_ERR_NOMEM;
      t->error = "host allocation failed";
    } catch (const std::exception &e) {
      t->status = WGPU_ERR_INVALID;
      t->error = e.what();
    }
    {
      std::lock_guard<std::mutex> lock(mu);
      --running;
      if (sess) {
        sess->busy = false;
        if (sess->bound)
          sess->bytes += t->need;  // stays resident until the session closes
        else
          used -= t->need;
      } else {
        used -= t->need;
      }
      t->finished = Clock::now();
      t->done = true;
      last_finish = t->finished;
      if (t->status == WGPU_OK) {
        ++completed;
        vis_done += (double)t->req.n_rows * (double)t->req.n_chan;
      } else {
        ++failed;
      }
    }
    done_cv.notify_all();
    cv.notify_all();
  }
}

extern "C" {

int wgpu_server_create(double device_bytes, int max_active, double plane_budget_bytes,
                       wgpu_server_t **server) {
  if (!server || max_active < 1 || max_active > 64 || !(device_bytes > 0) ||
      !(plane_budget_bytes >= 0))
    return wgpu::report_failure(WGPU_ERR_INVALID, "invalid server arguments");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return wgpu::report_failure(WGPU_ERR_CUDA, "no usable CUDA device");
  }
  auto *s = new wgpu_server();
  s->budget = device_bytes;
  s->plane_budget =
      plane_budget_bytes > 0 ? plane_budget_bytes : device_bytes / (2.0 * max_active);
  cudaGetDevice(&s->device);
  for (int i = 0; i < max_active; ++i) s->workers.emplace_back([s] { s->run_worker(); });
  wgpu::clear_failure();
  *server = s;
  return WGPU_OK;
}

int wgpu_server_submit(wgpu_server_t *s, const wgpu_request_t *req, uint64_t *ticket) {
  if (!s || !req || !ticket) return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  if (req->kind != WGPU_REQUEST_INVERT && req->kind != WGPU_REQUEST_PREDICT)
    return wgpu::report_failure(WGPU_ERR_INVALID, "unknown request kind");
  if (!req->uvw || !req->freq || req->n_rows == 0 || req->n_chan == 0)
    return wgpu::report_failure(WGPU_ERR_INVALID, "request without visibilities");
  if (req->kind == WGPU_REQUEST_INVERT && !req->vis)
    return wgpu::report_failure(WGPU_ERR_INVALID, "inversion request without visibilities");
  if (req->kind == WGPU_REQUEST_PREDICT && (!req->model || !req->vis_out))
    return wgpu::report_failure(WGPU_ERR_INVALID, "prediction request without model or output");
  auto t = std::make_shared<Ticket>();
  t->req = *req;
  try {
    t->bytes = estimate_bytes(*req, s->plane_budget);
  } catch (const wgpu::Error &e) {
    return wgpu::report_failure(e.status, e.what());
  }
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) return wgpu::report_failure(WGPU_ERR_STATE, "server is stopping");
    t->id = s->next_id++;
    t->submitted = Clock::now();
    if (!s->any_submit) {
      s->first_submit = t->submitted;
      s->any_submit = true;
    }
    s->tickets[t->id] = t;
    s->queue.push_back(t);
  }
  s->cv.notify_all();
  *ticket = t->id;
  wgpu::clear_failure();
  return WGPU_OK;
}

int wgpu_server_wait(wgpu_server_t *s, uint64_t ticket, double *latency_ms, double *queue_ms) {
  if (!s) return wgpu::report_failure(WGPU_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return wgpu::report_failure(WGPU_ERR_INVALID, "unknown ticket");
  std::shared_ptr<Ticket> t = it->second;
  s->done_cv.wait(lock, [&] { return t->done; });
  using Ms = std::chrono::duration<double, std::milli>;
  if (latency_ms) *latency_ms = Ms(t->finished - t->submitted).count();
  if (queue_ms) *queue_ms = Ms(t->started - t->submitted).count();
  s->tickets.erase(ticket);
  if (t->status != WGPU_OK) return wgpu::report_failure(t->status, t->error);
  wgpu::clear_failure();
  return WGPU_OK;
}

int wgpu_server_close_session(wgpu_server_t *s, uint64_t session) {
  if (!s) return wgpu::report_failure(WGPU_ERR_INVALID, "null server");
  std::shared_ptr<Session> victim;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->sessions.find(session);
    if (it == s->sessions.end()) return WGPU_OK;
    bool queued = false;
    for (const auto &t : s->queue) queued = queued || t->req.session == session;
    if (it->second->busy || queued)
      return wgpu::report_failure(WGPU_ERR_STATE, "session has requests queued or running");
    s->used -= it->second->bytes;
    victim = it->second;
    s->sessions.erase(it);
  }
  victim.reset();  // destroys the gridder outside the lock
  s->cv.notify_all();
  wgpu::clear_failure();
  return WGPU_OK;
}

int wgpu_server_stats(wgpu_server_t *s, wgpu_server_stats_t *out) {
  if (!s || !out) return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = s->queue.size();
  out->running = (uint64_t)s->running;
  out->peak_running = (uint64_t)s->peak_running;
  out->device_bytes_in_use = s->used;
  out->peak_device_bytes = s->peak_used;
  out->visibilities = s->vis_done;
  out->held_for_memory = s->held_for_memory;
  out->elapsed_s =
      s->any_submit && s->completed + s->failed > 0
          ? std::chrono::duration<double>(s->last_finish - s->first_submit).count()
          : 0.0;
  return WGPU_OK;
}

void wgpu_server_destroy(wgpu_server_t *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stopping = true;
  }
  s->cv.notify_all();
  for (auto &w : s->workers) w.join();
  delete s;
}

}  // extern "C"
