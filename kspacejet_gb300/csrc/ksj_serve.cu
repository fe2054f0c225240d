// ksj_serve.cu -- the request loop behind include/ksj_serve.h (host code).
//
// One scheduler thread owns every CUDA object.  Its loop:
//   1. retire: every slot whose completion event has fired hands each request
//      of its batch its result (copied from staging when the caller's buffer
//      is pageable) and its own check flags, records the latency and frees
//      the slot and its bytes;
//   2. admit: while a slot is free, the oldest pending request opens a batch
//      and the pending requests of the same class (grid, image, kernel width,
//      DCF mode, output form) join it in arrival order, up to the batch's
//      frame limit and as long as the device bytes of everything in flight
//      stay within the cap; the batch is copied in (each request's k-space
//      into its frame of a padded [frame][channel][sample] block, cached
//      trajectories device to device), reconstructed by ONE ragged call
//      (ksj_gpu_gridding_adjoint_ragged: per-frame coil and sample counts,
//      padding never read) and copied out, all on the slot's stream;
//   3. otherwise wait briefly on the submit condition variable.
// Requests that arrive while batches are on the GPU queue up and leave in
// the next batch of their class as soon as a slot frees (continuous
// batching); several slots keep several batches in flight.  Slots keep
// their device and pinned buffers between batches (grow-only), so steady
// state allocates nothing.  A request's frame of a ragged call is
// byte-identical to the same reconstruction made alone, so a result does
// not depend on its batch-mates.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "ksj_gpu.h"
#include "ksj_serve.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t kDefaultBatchFrames = 32;

struct Ticket {
  uint64_t id = 0;
  ksj_serve_request req{};
  Clock::time_point submitted;
  uint64_t bytes = 0;  // device bytes of this request alone (admission of a single request)
  ksj_gpu_status result = KSJ_GPU_OK;
  bool done = false;
};

struct Buffer {
  void* p = nullptr;
  size_t cap = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr, copied = nullptr, computed = nullptr, done = nullptr;  // timing events of a batch
  cudaStream_t copy2 = nullptr;     // second input-copy stream (every other request), for a second copy engine
  cudaEvent_t copy2_done = nullptr;
  Buffer kspace, out, workspace, counts;  // device: copied inputs (packed), images, workspace, per-frame table
  Buffer pin_in, pin_out, pin_meta;             // pinned host: pageable inputs, pageable outputs, counts + flags
  std::vector<Ticket*> batch;                    // in frame order; empty = free
  std::vector<size_t> out_staged;                // per request: offset in pin_out, or SIZE_MAX (direct)
  const uint32_t* flags = nullptr;               // per-frame check flags, in pin_meta
  uint64_t bytes = 0;
  uint32_t frames = 0;
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

// Requests of one class share a ragged call.  With a coil split, requests
// of at most `split` coils batch apart from larger ones: a ragged call's
// per-frame work (the coil lines of the transforms, the lanes of the
// gridding) follows its largest coil count.
using ClassKey = std::tuple<uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, bool>;
ClassKey class_of(const ksj_serve_request& r, uint32_t split) {
  return {r.grid, r.image, r.kernel_width, r.dcf_mode, r.output, split != 0 && r.channels <= split};
}

ksj_gpu_gridding_desc make_desc(const ksj_serve_request& r, uint32_t frames, uint32_t channels, uint32_t samples) {
  ksj_gpu_gridding_desc d{};
  d.struct_size = sizeof(d);
  d.kernel = KSJ_GPU_KERNEL_KAISER_BESSEL;
  d.image_rows = d.image_cols = r.image;
  d.grid_rows = d.grid_cols = r.grid;
  d.kernel_width = r.kernel_width;
  d.row_origin = d.col_origin = (r.image - 1) / 2.0;
  d.channels = channels;
  d.samples = samples;
  d.frames = frames;
  d.dcf_mode = r.dcf_mode;
  d.output = r.output == KSJ_SERVE_OUTPUT_RSS ? KSJ_GPU_OUTPUT_RSS : KSJ_GPU_OUTPUT_COIL_MAJOR;
  d.sample_format = KSJ_GPU_SAMPLES_CF32;
  return d;
}

size_t pixels_of(const ksj_serve_request& r) { return static_cast<size_t>(r.image) * r.image; }

// bytes of one frame of a call's output with `channels` coils
size_t frame_out_bytes(const ksj_serve_request& r, uint32_t channels) {
  return r.output == KSJ_SERVE_OUTPUT_RSS ? pixels_of(r) * 4 : pixels_of(r) * channels * 8;
}

// bytes the caller receives
size_t out_bytes(const ksj_serve_request& r) { return frame_out_bytes(r, r.channels); }

// Device bytes of a ragged call over `frames` frames of at most `channels`
// coils and `samples` samples (0 on a bad shape).
uint64_t batch_bytes(const ksj_serve_request& r, uint32_t frames, uint32_t channels, uint32_t samples) {
  const ksj_gpu_gridding_desc d = make_desc(r, frames, channels, samples);
  const size_t ws = ksj_gpu_gridding_workspace_bytes(&d);
  if (ws == 0) return 0;
  return ws + uint64_t{frames} * channels * samples * 8 + uint64_t{frames} * samples * 8 +
         uint64_t{frames} * frame_out_bytes(r, channels) + uint64_t{frames} * 28;
}

}  // namespace

struct ksj_serve {
  ksj_serve_config cfg{};
  uint32_t max_batch = kDefaultBatchFrames;
  bool in_place = false;  // read page-locked inputs in place instead of copying them
  uint32_t coil_split = 0;  // requests of at most this many coils batch apart (0: no split)
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
  uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, samples_done = 0, batches = 0, batched_frames = 0;
  double copy_in_ms = 0.0, compute_ms = 0.0, copy_out_ms = 0.0;
  std::vector<double> latencies_ms;
  Clock::time_point first_submit, last_done;
  bool any_submit = false;
  uint64_t peak_bytes = 0;
  uint32_t peak_in_flight = 0;

  void run();
  bool launch(Slot& slot, const std::vector<Ticket*>& batch, uint32_t channels, uint32_t samples);
  void retire(Slot& slot);
  void fail_batch(const std::vector<Ticket*>& batch, ksj_gpu_status status);
};

// The device-readable address of host or device memory `p` (page-locked,
// mapped host memory or device memory), or null when the device cannot read
// it (pageable host memory).
const void* device_address(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  if (a.type == cudaMemoryTypeHost && a.devicePointer != nullptr) return a.devicePointer;
  return nullptr;
}

bool ksj_serve::launch(Slot& slot, const std::vector<Ticket*>& batch, uint32_t cmax, uint32_t mmax) {
  const ksj_serve_request& r0 = batch.front()->req;
  const uint32_t nf = static_cast<uint32_t>(batch.size());
  const ksj_gpu_gridding_desc d = make_desc(r0, nf, cmax, mmax);
  const size_t ws = ksj_gpu_gridding_workspace_bytes(&d);
  const size_t flags_at = ksj_gpu_gridding_frame_flags_offset(&d);
  const size_t frame_o = frame_out_bytes(r0, cmax);
  // where each request's inputs are read from: in place (mapped page-locked
  // memory, when the loop reads inputs in place), through the slot's
  // page-locked staging (pageable memory), and copied to the slot's device
  // buffer unless read in place
  std::vector<const void*> k_dev(nf, nullptr), t_dev(nf, nullptr);
  size_t stage_in = 0, stage_out = 0, packed = 0;
  for (uint32_t f = 0; f < nf; ++f) {
    const ksj_serve_request& r = batch[f]->req;
    const size_t kb = size_t{r.channels} * r.samples * 8, tb = size_t{r.samples} * 8;
    if (in_place) {
      k_dev[f] = device_address(r.kspace);
      if (r.trajectory_id == 0) t_dev[f] = device_address(r.trajectory);
    }
    if (k_dev[f] == nullptr) stage_in += kb;
    if (r.trajectory_id == 0 && t_dev[f] == nullptr) stage_in += tb;
    if (!in_place) packed += kb + tb;
    if (!(r.flags & KSJ_SERVE_HOST_PINNED)) stage_out += out_bytes(r);
  }
  const size_t meta_bytes = size_t{nf} * (4 + 4 + 8 + 8 + 4) + 16;
  if (ws == 0 || !ensure_device(slot.kspace, packed + 16) || !ensure_device(slot.out, nf * frame_o) ||
      !ensure_device(slot.workspace, ws) || !ensure_device(slot.counts, meta_bytes) ||
      !ensure_pinned(slot.pin_in, stage_in + 16) || !ensure_pinned(slot.pin_out, stage_out + 16) ||
      !ensure_pinned(slot.pin_meta, meta_bytes))
    return false;
  // per frame: coils, samples, k-space address, trajectory address (then,
  // after the call, the frame's check flags)
  uint32_t* counts = static_cast<uint32_t*>(slot.pin_meta.p);
  uint64_t* addr = reinterpret_cast<uint64_t*>(static_cast<char*>(slot.pin_meta.p) + ((size_t{nf} * 8 + 15) & ~size_t{15}));
  uint32_t* flags = reinterpret_cast<uint32_t*>(addr + 2 * nf);
  // the requests' input copies alternate between the slot's stream and a
  // second copy stream (which first waits for the slot's earlier work), so
  // two copy engines carry them; the reconstruction waits for both
  if (cudaEventRecord(slot.start, slot.stream) != cudaSuccess ||
      cudaStreamWaitEvent(slot.copy2, slot.start, 0) != cudaSuccess)
    return false;
  char* stage = static_cast<char*>(slot.pin_in.p);
  char* dev = static_cast<char*>(slot.kspace.p);
  cudaStream_t cs = slot.stream;
  auto place = [&](const void* src, size_t bytes, const void* in_place_addr) -> const void* {
    if (in_place_addr != nullptr) return in_place_addr;
    const void* from = src;
    if (device_address(src) == nullptr) {  // pageable: through the page-locked staging
      std::memcpy(stage, src, bytes);
      from = stage;
      stage += (bytes + 15) & ~size_t{15};
      if (in_place) return device_address(from);
    }
    if (cudaMemcpyAsync(dev, from, bytes, cudaMemcpyHostToDevice, cs) != cudaSuccess) return nullptr;
    const void* at = dev;
    dev += (bytes + 255) & ~size_t{255};
    return at;
  };
  for (uint32_t f = 0; f < nf; ++f) {
    const ksj_serve_request& r = batch[f]->req;
    const size_t kb = size_t{r.channels} * r.samples * 8, tb = size_t{r.samples} * 8;
    counts[f] = r.channels;
    counts[nf + f] = r.samples;
    cs = (f & 1) ? slot.copy2 : slot.stream;
    const void* k_at = place(r.kspace, kb, k_dev[f]);
    if (k_at == nullptr) return false;
    const void* t_at = nullptr;
    if (r.trajectory_id != 0) {
      auto it = trajectories.find(r.trajectory_id);
      if (it == trajectories.end()) {
        Trajectory tr{};
        tr.bytes = tb;
        if (cudaMalloc(&tr.d, tb) != cudaSuccess ||
            cudaEventCreateWithFlags(&tr.ready, cudaEventDisableTiming) != cudaSuccess) {
          cudaGetLastError();
          if (tr.d) cudaFree(tr.d);
          return false;
        }
        if (cudaMemcpyAsync(tr.d, r.trajectory, tb, cudaMemcpyHostToDevice, slot.stream) != cudaSuccess ||
            cudaEventRecord(tr.ready, slot.stream) != cudaSuccess)
          return false;
        it = trajectories.emplace(r.trajectory_id, tr).first;
      } else if (it->second.bytes != tb || cudaStreamWaitEvent(slot.stream, it->second.ready, 0) != cudaSuccess) {
        return false;  // an id names one trajectory: a different sample count is an error
      }
      t_at = it->second.d;
    } else {
      t_at = place(r.trajectory, tb, t_dev[f]);
    }
    if (t_at == nullptr) return false;
    addr[f] = reinterpret_cast<uint64_t>(k_at);
    addr[nf + f] = reinterpret_cast<uint64_t>(t_at);
  }
  const size_t addr_off = reinterpret_cast<char*>(addr) - static_cast<char*>(slot.pin_meta.p);
  if (cudaEventRecord(slot.copy2_done, slot.copy2) != cudaSuccess ||
      cudaStreamWaitEvent(slot.stream, slot.copy2_done, 0) != cudaSuccess ||
      cudaMemcpyAsync(slot.counts.p, slot.pin_meta.p, addr_off + size_t{nf} * 16, cudaMemcpyHostToDevice,
                      slot.stream) != cudaSuccess)
    return false;
  const uint32_t* d_counts = static_cast<const uint32_t*>(slot.counts.p);
  const uint64_t* d_addr = reinterpret_cast<const uint64_t*>(static_cast<const char*>(slot.counts.p) + addr_off);
  if (cudaEventRecord(slot.copied, slot.stream) != cudaSuccess ||
      ksj_gpu_gridding_adjoint_ragged(&d, nullptr, d_counts, d_counts + nf, d_addr, d_addr + nf, slot.out.p,
                                      slot.workspace.p, slot.workspace.cap, slot.stream) != KSJ_GPU_OK ||
      cudaEventRecord(slot.computed, slot.stream) != cudaSuccess)
    return false;
  // results (a coil-major frame's first `channels` coils are contiguous),
  // then every frame's check flags
  slot.out_staged.assign(nf, SIZE_MAX);
  char* ostage = static_cast<char*>(slot.pin_out.p);
  size_t ooff = 0;
  for (uint32_t f = 0; f < nf; ++f) {
    const ksj_serve_request& r = batch[f]->req;
    const size_t ob = out_bytes(r);
    void* dst = r.out;
    if (!(r.flags & KSJ_SERVE_HOST_PINNED)) {
      dst = ostage + ooff;
      slot.out_staged[f] = ooff;
      ooff += ob;
    }
    if (cudaMemcpyAsync(dst, static_cast<const char*>(slot.out.p) + f * frame_o, ob, cudaMemcpyDeviceToHost,
                        slot.stream) != cudaSuccess)
      return false;
  }
  if (cudaMemcpyAsync(flags, static_cast<const char*>(slot.workspace.p) + flags_at, size_t{nf} * 4,
                      cudaMemcpyDeviceToHost, slot.stream) != cudaSuccess ||
      cudaEventRecord(slot.done, slot.stream) != cudaSuccess)
    return false;
  slot.flags = flags;
  slot.batch = batch;
  slot.frames = nf;
  return true;
}

void ksj_serve::fail_batch(const std::vector<Ticket*>& batch, ksj_gpu_status status) {
  std::lock_guard<std::mutex> lock(mu);
  for (Ticket* t : batch) {
    t->result = status;
    t->done = true;
    ++failed;
  }
  done_cv.notify_all();
}

void ksj_serve::retire(Slot& slot) {
  const uint32_t nf = slot.frames;
  const auto now = Clock::now();
  for (uint32_t f = 0; f < nf; ++f) {
    Ticket* t = slot.batch[f];
    if (slot.out_staged[f] != SIZE_MAX)
      std::memcpy(t->req.out, static_cast<const char*>(slot.pin_out.p) + slot.out_staged[f], out_bytes(t->req));
  }
  in_flight_bytes -= slot.bytes;
  float t_in = 0.0f, t_run = 0.0f, t_out = 0.0f;
  cudaEventElapsedTime(&t_in, slot.start, slot.copied);
  cudaEventElapsedTime(&t_run, slot.copied, slot.computed);
  cudaEventElapsedTime(&t_out, slot.computed, slot.done);
  std::lock_guard<std::mutex> lock(mu);
  copy_in_ms += t_in;
  compute_ms += t_run;
  copy_out_ms += t_out;
  for (uint32_t f = 0; f < nf; ++f) {
    Ticket* t = slot.batch[f];
    t->result = slot.flags[f] == 0 ? KSJ_GPU_OK : KSJ_GPU_ERROR_NONFINITE_INPUT;
    t->done = true;
    if (t->result == KSJ_GPU_OK) {
      ++completed;
      samples_done += static_cast<uint64_t>(t->req.channels) * t->req.samples;
    } else {
      ++failed;
    }
    latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - t->submitted).count());
  }
  ++batches;
  batched_frames += nf;
  last_done = now;
  slot.batch.clear();
  slot.bytes = 0;
  slot.frames = 0;
  done_cv.notify_all();
}

void ksj_serve::run() {
  if (cudaSetDevice(cfg.device) != cudaSuccess) return;
  slots.resize(cfg.slots);
  for (Slot& s : slots) {
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s.copy2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s.copy2_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&s.start) != cudaSuccess || cudaEventCreate(&s.copied) != cudaSuccess ||
        cudaEventCreate(&s.computed) != cudaSuccess || cudaEventCreate(&s.done) != cudaSuccess)
      return;
  }
  {
    std::lock_guard<std::mutex> lock(mu);
    init_ok = true;
  }
  done_cv.notify_all();
  for (;;) {
    bool progressed = false;
    for (Slot& s : slots) {
      if (!s.batch.empty() && cudaEventQuery(s.done) == cudaSuccess) {
        retire(s);
        progressed = true;
      }
    }
    // admit: one batch per free slot
    for (;;) {
      Slot* free_slot = nullptr;
      for (Slot& s : slots)
        if (s.batch.empty()) {
          free_slot = &s;
          break;
        }
      std::vector<Ticket*> batch;
      uint32_t cmax = 0, mmax = 0;
      uint64_t bytes = 0;
      {
        std::lock_guard<std::mutex> lock(mu);
        if (free_slot == nullptr || pending.empty()) break;
        const ksj_serve_request& head = pending.front()->req;
        const ClassKey key = class_of(head, coil_split);
        // the head first, then its class's later requests in arrival order,
        // while the batch stays within its frame limit and the device cap
        for (auto it = pending.begin(); it != pending.end() && batch.size() < max_batch; ++it) {
          const ksj_serve_request& r = (*it)->req;
          if (class_of(r, coil_split) != key) continue;
          const uint32_t c = std::max(cmax, r.channels), m = std::max(mmax, r.samples);
          const uint64_t b = batch_bytes(head, static_cast<uint32_t>(batch.size() + 1), c, m);
          if (b == 0 || in_flight_bytes + b > cfg.device_memory_cap) {
            if (batch.empty()) break;  // the head waits for bytes to free
            continue;
          }
          batch.push_back(*it);
          cmax = c;
          mmax = m;
          bytes = b;
        }
        if (batch.empty()) break;
        for (Ticket* t : batch) pending.erase(std::find(pending.begin(), pending.end(), t));
      }
      in_flight_bytes += bytes;
      free_slot->bytes = bytes;
      if (!launch(*free_slot, batch, cmax, mmax)) {
        free_slot->batch.clear();
        in_flight_bytes -= bytes;
        free_slot->bytes = 0;
        cudaStreamSynchronize(free_slot->stream);
        cudaStreamSynchronize(free_slot->copy2);
        cudaGetLastError();
        fail_batch(batch, KSJ_GPU_ERROR_CUDA);
      } else {
        uint32_t n = 0;
        for (Slot& s : slots) n += s.batch.empty() ? 0u : static_cast<uint32_t>(s.batch.size());
        std::lock_guard<std::mutex> lock(mu);
        peak_bytes = std::max(peak_bytes, in_flight_bytes);
        peak_in_flight = std::max(peak_in_flight, n);
      }
      progressed = true;
    }
    bool busy = false;
    for (Slot& s : slots) busy |= !s.batch.empty();
    std::unique_lock<std::mutex> lock(mu);
    if (stop && pending.empty() && !busy) break;
    if (!progressed) work_cv.wait_for(lock, std::chrono::microseconds(busy ? 20 : 2000));
  }
  for (Slot& s : slots) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    for (Buffer* b : {&s.kspace, &s.out, &s.workspace, &s.counts})
      if (b->p) cudaFree(b->p);
    for (Buffer* b : {&s.pin_in, &s.pin_out, &s.pin_meta})
      if (b->p) cudaFreeHost(b->p);
    if (s.copy2) cudaStreamSynchronize(s.copy2);
    for (cudaEvent_t e : {s.start, s.copied, s.computed, s.done, s.copy2_done})
      if (e) cudaEventDestroy(e);
    if (s.stream) cudaStreamDestroy(s.stream);
    if (s.copy2) cudaStreamDestroy(s.copy2);
  }
  for (auto& kv : trajectories) {
    cudaFree(kv.second.d);
    cudaEventDestroy(kv.second.ready);
  }
}

extern "C" ksj_gpu_status ksj_serve_create(const ksj_serve_config* config, ksj_serve** out) {
  constexpr size_t kBaseConfig = offsetof(ksj_serve_config, max_batch_frames);
  if (config == nullptr || out == nullptr || config->struct_size < kBaseConfig || config->slots == 0 ||
      config->slots > 64 || config->device_memory_cap == 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  auto* s = new (std::nothrow) ksj_serve{};
  if (s == nullptr) return KSJ_GPU_ERROR_OUT_OF_MEMORY;
  std::memcpy(&s->cfg, config, std::min<size_t>(config->struct_size, sizeof(ksj_serve_config)));
  s->cfg.struct_size = sizeof(ksj_serve_config);
  if (config->struct_size >= offsetof(ksj_serve_config, max_batch_frames) + sizeof(uint32_t) &&
      config->max_batch_frames != 0)
    s->max_batch = std::min<uint32_t>(config->max_batch_frames, 1024);
  if (config->struct_size >= offsetof(ksj_serve_config, read_inputs_in_place) + sizeof(uint32_t))
    s->in_place = config->read_inputs_in_place != 0;
  if (config->struct_size >= offsetof(ksj_serve_config, coil_split) + sizeof(uint32_t))
    s->coil_split = config->coil_split;
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
  const uint64_t kb = uint64_t{r->channels} * r->samples * 8;
  const uint64_t bytes = r->channels && r->samples ? batch_bytes(*r, 1, r->channels, r->samples) : 0;
  std::lock_guard<std::mutex> lock(s->mu);
  if (bytes == 0 || r->kspace == nullptr || r->trajectory == nullptr || r->out == nullptr ||
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
  out->batches = s->batches;
  out->batched_frames = s->batched_frames;
  out->copy_in_ms = s->copy_in_ms;
  out->compute_ms = s->compute_ms;
  out->copy_out_ms = s->copy_out_ms;
  return KSJ_GPU_OK;
}

extern "C" void ksj_serve_reset_stats(ksj_serve* s) {
  if (s == nullptr) return;
  std::lock_guard<std::mutex> lock(s->mu);
  s->submitted = s->completed = s->rejected = s->failed = s->samples_done = 0;
  s->batches = s->batched_frames = 0;
  s->copy_in_ms = s->compute_ms = s->copy_out_ms = 0.0;
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
