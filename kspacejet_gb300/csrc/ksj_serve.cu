// ksj_serve.cu -- the request loop behind include/ksj_serve.h (host code).
//
// One scheduler thread owns every CUDA object.  Its loop:
//   1. admit: while the oldest pending request fits (a free slot, and the
//      device bytes of admitted requests plus its own <= the cap), stage its
//      inputs through the slot's pinned buffer, enqueue copy-in, the
//      ksj_gpu_gridding_adjoint call and copy-out on the slot's stream, and
//      record the slot's completion event;
//   2. retire: every slot whose event has completed copies its result to the
//      caller's buffer, records the latency and frees its bytes and slot;
//   3. otherwise sleep briefly on the submit condition variable.
// Slots keep their device workspace, input, output and pinned staging
// buffers between requests (grow-only), so steady state allocates nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ksj_gpu.h"
#include "ksj_serve.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Ticket {
  uint64_t id = 0;
  ksj_serve_request req{};
  Clock::time_point submitted;
  uint64_t bytes = 0;
  ksj_gpu_status result = KSJ_GPU_OK;
  bool done = false;
};

struct Buffer {
  void* p = nullptr;
  size_t cap = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Buffer kspace, traj, out, workspace;  // device
  Buffer pin_in, pin_out;               // pinned host staging
  Ticket* busy = nullptr;
};

struct Trajectory {
  void* d = nullptr;
  size_t bytes = 0;
  cudaEvent_t ready = nullptr;
};

bool ensure_device(Buffer& b, size_t bytes) {
  if (b.cap >= bytes) return true;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b.cap = bytes;
  return true;
}

bool ensure_pinned(Buffer& b, size_t bytes) {
  if (b.cap >= bytes) return true;
  if (b.p) cudaFreeHost(b.p);
  b.p = nullptr;
  b.cap = 0;
  if (cudaMallocHost(&b.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b.cap = bytes;
  return true;
}

ksj_gpu_gridding_desc make_desc(const ksj_serve_request& r) {
  ksj_gpu_gridding_desc d{};
  d.struct_size = sizeof(d);
  d.kernel = KSJ_GPU_KERNEL_KAISER_BESSEL;
  d.image_rows = d.image_cols = r.image;
  d.grid_rows = d.grid_cols = r.grid;
  d.kernel_width = r.kernel_width;
  d.row_origin = d.col_origin = (r.image - 1) / 2.0;
  d.channels = r.channels;
  d.samples = r.samples;
  d.frames = 1;
  d.dcf_mode = r.dcf_mode;
  d.output = r.output == KSJ_SERVE_OUTPUT_RSS ? KSJ_GPU_OUTPUT_RSS : KSJ_GPU_OUTPUT_COIL_MAJOR;
  d.sample_format = KSJ_GPU_SAMPLES_CF32;
  return d;
}

size_t out_bytes(const ksj_serve_request& r) {
  const size_t px = static_cast<size_t>(r.image) * r.image;
  return r.output == KSJ_SERVE_OUTPUT_RSS ? px * 4 : px * r.channels * 8;
}

}  // namespace

struct ksj_serve {
  ksj_serve_config cfg{};
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<Ticket*> pending;
  std::unordered_map<uint64_t, Ticket*> tickets;
  std::vector<Slot> slots;
  std::unordered_map<uint64_t, Trajectory> trajectories;  // scheduler thread only
  uint64_t next_id = 1;
  uint64_t in_flight_bytes = 0;  // scheduler thread only
  bool stop = false;
  bool init_ok = false;
  std::thread worker;
  // statistics (under mu)
  uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, samples_done = 0;
  std::vector<double> latencies_ms;
  Clock::time_point first_submit, last_done;
  bool any_submit = false;
  uint64_t peak_bytes = 0;
  uint32_t peak_in_flight = 0;

  void run();
  bool launch(Slot& slot, Ticket* t);
  void retire(Slot& slot);
};

bool ksj_serve::launch(Slot& slot, Ticket* t) {
  const ksj_serve_request& r = t->req;
  const ksj_gpu_gridding_desc d = make_desc(r);
  const size_t ws = ksj_gpu_gridding_workspace_bytes(&d);
  const size_t kb = static_cast<size_t>(r.channels) * r.samples * 8;
  const size_t tb = static_cast<size_t>(r.samples) * 8;
  const size_t ob = out_bytes(r);
  if (ws == 0 || !ensure_device(slot.kspace, kb) || !ensure_device(slot.out, ob) ||
      !ensure_device(slot.workspace, ws) ||
      (!(r.flags & KSJ_SERVE_HOST_PINNED) && !ensure_pinned(slot.pin_in, kb + tb)) ||
      !ensure_pinned(slot.pin_out, ob + 16))
    return false;
  // inputs: pinned callers are copied by DMA directly; pageable ones are
  // staged through the slot's pinned buffer.  Trajectories with an id stay
  // resident and later requests wait on their upload event.
  const bool pinned = (r.flags & KSJ_SERVE_HOST_PINNED) != 0;
  const void* k_src = r.kspace;
  const void* t_src = r.trajectory;
  if (!pinned) {
    std::memcpy(slot.pin_in.p, r.kspace, kb);
    k_src = slot.pin_in.p;
    t_src = static_cast<char*>(slot.pin_in.p) + kb;
  }
  if (cudaMemcpyAsync(slot.kspace.p, k_src, kb, cudaMemcpyHostToDevice, slot.stream) != cudaSuccess) return false;
  const float* d_traj = nullptr;
  if (r.trajectory_id != 0) {
    auto it = trajectories.find(r.trajectory_id);
    if (it == trajectories.end()) {
      Trajectory tr{};
      tr.bytes = tb;
      if (cudaMalloc(&tr.d, tb) != cudaSuccess ||
          cudaEventCreateWithFlags(&tr.ready, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      if (!pinned) std::memcpy(const_cast<void*>(t_src), r.trajectory, tb);
      if (cudaMemcpyAsync(tr.d, t_src, tb, cudaMemcpyHostToDevice, slot.stream) != cudaSuccess ||
          cudaEventRecord(tr.ready, slot.stream) != cudaSuccess)
        return false;
      it = trajectories.emplace(r.trajectory_id, tr).first;
    } else if (it->second.bytes != tb || cudaStreamWaitEvent(slot.stream, it->second.ready, 0) != cudaSuccess) {
      return false;  // an id names one trajectory: a different sample count is an error
    }
    d_traj = static_cast<const float*>(it->second.d);
  } else {
    if (!ensure_device(slot.traj, tb)) return false;
    if (!pinned) std::memcpy(const_cast<void*>(t_src), r.trajectory, tb);
    if (cudaMemcpyAsync(slot.traj.p, t_src, tb, cudaMemcpyHostToDevice, slot.stream) != cudaSuccess) return false;
    d_traj = static_cast<const float*>(slot.traj.p);
  }
  if (ksj_gpu_gridding_adjoint(&d, nullptr, slot.kspace.p, d_traj, nullptr, slot.out.p, slot.workspace.p,
                               slot.workspace.cap, slot.stream) != KSJ_GPU_OK)
    return false;
  // result, then the device check flags (first word of the workspace) behind it
  void* out_dst = pinned ? r.out : slot.pin_out.p;
  if (cudaMemcpyAsync(out_dst, slot.out.p, ob, cudaMemcpyDeviceToHost, slot.stream) != cudaSuccess ||
      cudaMemcpyAsync(static_cast<char*>(slot.pin_out.p) + ob, slot.workspace.p, 4, cudaMemcpyDeviceToHost,
                      slot.stream) != cudaSuccess ||
      cudaEventRecord(slot.done, slot.stream) != cudaSuccess)
    return false;
  slot.busy = t;
  return true;
}

void ksj_serve::retire(Slot& slot) {
  Ticket* t = slot.busy;
  slot.busy = nullptr;
  uint32_t flags = 0;
  const size_t ob = out_bytes(t->req);
  std::memcpy(&flags, static_cast<const char*>(slot.pin_out.p) + ob, sizeof(flags));
  if (!(t->req.flags & KSJ_SERVE_HOST_PINNED)) std::memcpy(t->req.out, slot.pin_out.p, ob);
  const auto now = Clock::now();
  in_flight_bytes -= t->bytes;
  std::lock_guard<std::mutex> lock(mu);
  t->result = flags == 0 ? KSJ_GPU_OK : KSJ_GPU_ERROR_NONFINITE_INPUT;
  t->done = true;
  if (t->result == KSJ_GPU_OK) {
    ++completed;
    samples_done += static_cast<uint64_t>(t->req.channels) * t->req.samples;
  } else {
    ++failed;
  }
  latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - t->submitted).count());
  last_done = now;
  done_cv.notify_all();
}

void ksj_serve::run() {
  if (cudaSetDevice(cfg.device) != cudaSuccess) return;
  slots.resize(cfg.slots);
  for (Slot& s : slots) {
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess)
      return;
  }
  {
    std::lock_guard<std::mutex> lock(mu);
    init_ok = true;
  }
  done_cv.notify_all();
  for (;;) {
    bool progressed = false;
    // retire finished slots
    for (Slot& s : slots) {
      if (s.busy != nullptr && cudaEventQuery(s.done) == cudaSuccess) {
        retire(s);
        progressed = true;
      }
    }
    // admit in arrival order
    for (;;) {
      Ticket* t = nullptr;
      Slot* free_slot = nullptr;
      for (Slot& s : slots)
        if (s.busy == nullptr) {
          free_slot = &s;
          break;
        }
      {
        std::lock_guard<std::mutex> lock(mu);
        if (free_slot == nullptr || pending.empty()) break;
        if (in_flight_bytes + pending.front()->bytes > cfg.device_memory_cap) break;
        t = pending.front();
        pending.pop_front();
      }
      in_flight_bytes += t->bytes;
      if (!launch(*free_slot, t)) {
        free_slot->busy = nullptr;
        in_flight_bytes -= t->bytes;
        cudaStreamSynchronize(free_slot->stream);
        std::lock_guard<std::mutex> lock(mu);
        t->result = KSJ_GPU_ERROR_CUDA;
        t->done = true;
        ++failed;
        done_cv.notify_all();
      } else {
        uint32_t n = 0;
        for (Slot& s : slots) n += s.busy != nullptr;
        std::lock_guard<std::mutex> lock(mu);
        peak_bytes = std::max(peak_bytes, in_flight_bytes);
        peak_in_flight = std::max(peak_in_flight, n);
      }
      progressed = true;
    }
    bool busy = false;
    for (Slot& s : slots) busy |= s.busy != nullptr;
    std::unique_lock<std::mutex> lock(mu);
    if (stop && pending.empty() && !busy) break;
    if (!progressed) work_cv.wait_for(lock, std::chrono::microseconds(busy ? 20 : 2000));
  }
  for (Slot& s : slots) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    for (Buffer* b : {&s.kspace, &s.traj, &s.out, &s.workspace})
      if (b->p) cudaFree(b->p);
    for (Buffer* b : {&s.pin_in, &s.pin_out})
      if (b->p) cudaFreeHost(b->p);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (auto& kv : trajectories) {
    cudaFree(kv.second.d);
    cudaEventDestroy(kv.second.ready);
  }
}

extern "C" ksj_gpu_status ksj_serve_create(const ksj_serve_config* config, ksj_serve** out) {
  if (config == nullptr || out == nullptr || config->struct_size < sizeof(ksj_serve_config) || config->slots == 0 ||
      config->slots > 64 || config->device_memory_cap == 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  auto* s = new (std::nothrow) ksj_serve{};
  if (s == nullptr) return KSJ_GPU_ERROR_OUT_OF_MEMORY;
  s->cfg = *config;
  s->worker = std::thread([s] { s->run(); });
  {
    std::unique_lock<std::mutex> lock(s->mu);
    s->done_cv.wait_for(lock, std::chrono::seconds(30), [s] { return s->init_ok; });
    if (!s->init_ok) {
      s->stop = true;
      lock.unlock();
      s->work_cv.notify_all();
      s->worker.join();
      delete s;
      return KSJ_GPU_ERROR_CUDA;
    }
  }
  *out = s;
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_serve_submit(ksj_serve* s, const ksj_serve_request* r, uint64_t* out_ticket) {
  if (s == nullptr || r == nullptr || out_ticket == nullptr || r->struct_size < sizeof(ksj_serve_request))
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const ksj_gpu_gridding_desc d = make_desc(*r);
  const size_t ws = ksj_gpu_gridding_workspace_bytes(&d);
  const uint64_t kb = uint64_t{r->channels} * r->samples * 8;
  const uint64_t bytes = ws + kb + uint64_t{r->samples} * 8 + out_bytes(*r);
  std::lock_guard<std::mutex> lock(s->mu);
  if (ws == 0 || r->kspace == nullptr || r->trajectory == nullptr || r->out == nullptr ||
      (r->output != KSJ_SERVE_OUTPUT_RSS && r->output != KSJ_SERVE_OUTPUT_COIL_MAJOR) || r->channels > s->cfg.max_channels ||
      kb > s->cfg.max_frame_bytes || out_bytes(*r) > s->cfg.max_image_bytes || bytes > s->cfg.device_memory_cap) {
    ++s->rejected;
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  }
  auto* t = new (std::nothrow) Ticket{};
  if (t == nullptr) return KSJ_GPU_ERROR_OUT_OF_MEMORY;
  t->id = s->next_id++;
  t->req = *r;
  t->submitted = Clock::now();
  t->bytes = bytes;
  if (!s->any_submit) {
    s->first_submit = t->submitted;
    s->any_submit = true;
  }
  ++s->submitted;
  s->tickets[t->id] = t;
  s->pending.push_back(t);
  *out_ticket = t->id;
  s->work_cv.notify_all();
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_serve_wait(ksj_serve* s, uint64_t ticket, uint32_t timeout_ms, ksj_gpu_status* result) {
  if (s == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  Ticket* t = it->second;
  auto pred = [t] { return t->done; };
  if (timeout_ms == 0) s->done_cv.wait(lock, pred);
  else if (!s->done_cv.wait_for(lock, std::chrono::milliseconds(timeout_ms), pred)) return KSJ_GPU_ERROR_UNSUPPORTED;
  if (result) *result = t->result;
  s->tickets.erase(it);
  delete t;
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_serve_drain(ksj_serve* s) {
  if (s == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(s->mu);
  s->done_cv.wait(lock, [s] {
    for (auto& kv : s->tickets)
      if (!kv.second->done) return false;
    return true;
  });
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_serve_get_stats(ksj_serve* s, ksj_serve_stats* out) {
  if (s == nullptr || out == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  *out = {};
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->failed = s->failed;
  out->gridded_samples = s->samples_done;
  out->wall_seconds =
      s->any_submit && !s->latencies_ms.empty() ? std::chrono::duration<double>(s->last_done - s->first_submit).count()
                                                : 0.0;
  if (!s->latencies_ms.empty()) {
    std::vector<double> v = s->latencies_ms;
    std::sort(v.begin(), v.end());
    auto q = [&v](double p) {
      const size_t i = static_cast<size_t>(p * static_cast<double>(v.size() - 1) + 0.5);
      return v[std::min(i, v.size() - 1)];
    };
    out->latency_p50_ms = q(0.50);
    out->latency_p99_ms = q(0.99);
    out->latency_max_ms = v.back();
  }
  out->peak_device_bytes = s->peak_bytes;
  out->peak_in_flight = s->peak_in_flight;
  return KSJ_GPU_OK;
}

extern "C" void ksj_serve_reset_stats(ksj_serve* s) {
  if (s == nullptr) return;
  std::lock_guard<std::mutex> lock(s->mu);
  s->submitted = s->completed = s->rejected = s->failed = s->samples_done = 0;
  s->latencies_ms.clear();
  s->any_submit = false;
  s->peak_bytes = 0;
  s->peak_in_flight = 0;
}

extern "C" void ksj_serve_destroy(ksj_serve* s) {
  if (s == nullptr) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->tickets) delete kv.second;
  for (Ticket* t : s->pending)
    if (s->tickets.find(t->id) == s->tickets.end()) delete t;
  delete s;
}
