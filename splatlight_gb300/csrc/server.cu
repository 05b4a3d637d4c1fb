// Request server: continuous batching of render requests over resident scenes.  Requests (scene, RenderFrame, eye,
// light-intensity scale) arrive from any thread; a worker thread admits them by footprint into the next batch of a
// free pipeline (an sl_batch with its own stream and buffers, so batches overlap on the device), launches the
// batch's captured chain, copies each image into a pinned result slot, and hands results back through poll().
// Memory is bounded everywhere: device buffers per pipeline are sized once for the admission limits (slots, tiles,
// pixels per batch; a request larger than an empty batch is refused at submit), and the pinned host result slots
// are a fixed pool (a batch waits for free slots; the caller releases a slot after reading its image).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sl_batch.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  uint64_t tag = 0;
  uint32_t scene = 0;
  sl_render_frame frame;
  float eye[3] = {0, 0, 0};
  float light_scale = 1.0f;
  uint64_t slots = 0, tiles = 0, pixels = 0;
  double t_submit = 0.0, t_start = 0.0;
  uint32_t result_slot = 0;
  uint32_t batch_views = 0;
};

struct Pipe {
  sl_batch* b = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  sl::DevBuf out;           // device images of the batch
  std::vector<Req> reqs;
  std::vector<uint32_t> scene_of_view;
  std::vector<sl_render_frame> frames;
  std::vector<float> eyes, scales;
  uint64_t slots = 0, tiles = 0;
  bool busy = false, replayed = false;
  int attempts = 0;
};

}  // namespace

struct sl_server {
  int device = 0;
  std::vector<sl_renderer*> scenes;
  std::vector<sl_lighting*> lights;
  sl_server_options opt{};
  std::vector<Pipe> pipes;
  // pinned result slots
  float* arena = nullptr;
  uint64_t slot_floats = 0;
  std::vector<uint32_t> free_slots;
  // per result slot: kSlotFree, kSlotBusy (a batch writes it), kSlotReady (its result waits in the queue),
  // kSlotDelivered (handed out by poll; only this state may be released)
  std::vector<uint8_t> slot_state;
  // queues
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req> pending;
  std::deque<sl_server_result> results;
  std::thread worker;
  bool stop = false;
  Clock::time_point epoch;
  // statistics
  uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, batches = 0, batch_views = 0, replays = 0;
  uint64_t reshaded = 0;  // views re-run with every blended splat shaded (radiance above the coverage allowance)
  uint64_t relaunches = 0;  // batches launched again (entries beyond the capacity class, or a re-shade)
  uint64_t device_bytes = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - epoch).count(); }
};

namespace sl {
namespace {

enum : uint8_t { kSlotFree = 0, kSlotBusy = 1, kSlotReady = 2, kSlotDelivered = 3 };

uint64_t footprint_slots(const sl_renderer* r, const sl_render_frame& f) {
  return ((uint64_t)r->count + 1u + (uint32_t)f.palette[3][1] + 255) & ~255ull;
}

// Moves requests from the pending queue into pipe p's next batch while they fit (FIFO: the first request that does
// not fit ends the batch, so no request waits behind later ones forever).  Called with the lock held.
void form_batch(sl_server* S, Pipe& p) {
  p.reqs.clear();
  uint64_t slots = 0, tiles = 0, pixels = 0;
  while (!S->pending.empty() && p.reqs.size() < S->opt.max_views && !S->free_slots.empty()) {
    const Req& q = S->pending.front();
    if (slots + q.slots > S->opt.max_slots || tiles + q.tiles > S->opt.max_tiles ||
        pixels + q.pixels > S->opt.max_pixels)
      break;
    slots += q.slots;
    tiles += q.tiles;
    pixels += q.pixels;
    Req r = q;
    S->pending.pop_front();
    r.result_slot = S->free_slots.back();
    S->free_slots.pop_back();
    S->slot_state[r.result_slot] = kSlotBusy;
    p.reqs.push_back(r);
  }
}

int launch(sl_server* S, Pipe& p) {
  const uint32_t n = (uint32_t)p.reqs.size();
  p.scene_of_view.resize(n);
  p.frames.resize(n);
  p.eyes.resize(3 * n);
  p.scales.resize(n);
  for (uint32_t v = 0; v < n; v++) {
    p.scene_of_view[v] = p.reqs[v].scene;
    p.frames[v] = p.reqs[v].frame;
    for (int c = 0; c < 3; c++) p.eyes[3 * v + c] = p.reqs[v].eye[c];
    p.scales[v] = p.reqs[v].light_scale;
  }
  uint64_t slots, tiles, pix;
  int rc = batch_layout(p.b, p.scene_of_view.data(), p.frames.data(), n, &slots, &tiles, &pix);
  if (rc) return rc;
  rc = batch_fit(p.b, slots, tiles);
  if (rc) return rc;
  p.slots = slots;
  p.tiles = tiles;
  rc = batch_launch(p.b, p.scene_of_view.data(), p.frames.data(), p.eyes.data(), p.scales.data(), n,
                    p.out.as<float>(), slots, tiles, p.s, &p.replayed);
  if (rc) return rc;
  // each image into its pinned result slot
  for (uint32_t v = 0; v < n; v++) {
    const uint64_t off = p.b->offsets[v];
    const uint64_t bytes = 4ull * sizeof(float) * p.reqs[v].pixels;
    cudaError_t e = cudaMemcpyAsync(S->arena + (uint64_t)p.reqs[v].result_slot * S->slot_floats,
                                    p.out.as<float>() + off, bytes, cudaMemcpyDeviceToHost, p.s);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
  }
  cudaError_t e = cudaEventRecord(p.done, p.s);
  if (e != cudaSuccess) return cuda_fail(e, "batch event");
  const double t = S->now();
  for (Req& r : p.reqs) {
    r.t_start = t;
    r.batch_views = n;
  }
  p.busy = true;
  return SL_OK;
}

void fail_batch(sl_server* S, Pipe& p, int code) {
  std::lock_guard<std::mutex> lk(S->mu);
  const double t = S->now();
  for (const Req& r : p.reqs) {
    sl_server_result res{};
    res.tag = r.tag;
    res.status = code;
    res.t_submit = r.t_submit;
    res.t_start = r.t_start;
    res.t_done = t;
    res.image = nullptr;
    S->slot_state[r.result_slot] = kSlotFree;
    S->free_slots.push_back(r.result_slot);
    S->results.push_back(res);
    S->failed++;
  }
  p.reqs.clear();
  p.busy = false;
  S->cv.notify_all();
}

// After pipe p's event completed: the overflow retry, or the results.
void complete(sl_server* S, Pipe& p) {
  bool retry = false;
  int rc = batch_finish(p.b, (uint32_t)p.reqs.size(), p.slots, p.tiles, p.replayed, nullptr, nullptr, &retry);
  if (rc == SL_OK && retry && ++p.attempts < 3) {
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->relaunches++;
    }
    p.busy = false;
    rc = launch(S, p);
    if (rc == SL_OK) return;
  }
  if (rc != SL_OK || retry) {
    fail_batch(S, p, rc != SL_OK ? rc : SL_ERR_OVERFLOW);
    return;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  const double t = S->now();
  for (const Req& r : p.reqs) {
    sl_server_result res{};
    res.tag = r.tag;
    res.status = SL_OK;
    res.batch_views = r.batch_views;
    res.width = (uint32_t)r.frame.viewport[0];
    res.height = (uint32_t)r.frame.viewport[1];
    res.result_slot = r.result_slot;
    res.t_submit = r.t_submit;
    res.t_start = r.t_start;
    res.t_done = t;
    res.image = S->arena + (uint64_t)r.result_slot * S->slot_floats;
    S->slot_state[r.result_slot] = kSlotReady;
    S->results.push_back(res);
    S->completed++;
  }
  S->batches++;
  S->batch_views += p.reqs.size();
  if (p.replayed) S->replays++;
  for (uint8_t f : p.b->shade_blended) S->reshaded += f;
  p.reqs.clear();
  p.busy = false;
  S->cv.notify_all();
}

void worker_loop(sl_server* S) {
  cudaSetDevice(S->device);
  for (;;) {
    bool progressed = false;
    for (Pipe& p : S->pipes) {
      if (p.busy) {
        cudaError_t q = cudaEventQuery(p.done);
        if (q == cudaSuccess) {
          complete(S, p);
          progressed = true;
        } else if (q != cudaErrorNotReady) {
          fail_batch(S, p, cuda_fail(q, "batch"));
          progressed = true;
        }
      }
    }
    for (Pipe& p : S->pipes) {
      if (p.busy) continue;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        form_batch(S, p);
      }
      if (p.reqs.empty()) continue;
      p.attempts = 0;
      batch_begin(p.b, (uint32_t)p.reqs.size());
      int rc = launch(S, p);
      if (rc) fail_batch(S, p, rc);
      progressed = true;
    }
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->stop) {
      bool idle = true;
      for (Pipe& p : S->pipes) idle = idle && !p.busy;
      if (idle) break;
    }
    if (!progressed) {
      bool any_busy = false;
      for (Pipe& p : S->pipes) any_busy = any_busy || p.busy;
      // nothing to do: sleep until a request arrives (or poll the device again shortly while batches run)
      S->cv.wait_for(lk, std::chrono::microseconds(any_busy ? 20 : 2000));
    }
  }
  // requests never admitted: cancelled
  std::lock_guard<std::mutex> lk(S->mu);
  const double t = S->now();
  while (!S->pending.empty()) {
    const Req& r = S->pending.front();
    sl_server_result res{};
    res.tag = r.tag;
    res.status = SL_ERR_CANCELLED;
    res.t_submit = r.t_submit;
    res.t_done = t;
    S->results.push_back(res);
    S->pending.pop_front();
  }
  S->cv.notify_all();
}

}  // namespace
}  // namespace sl

using namespace sl;

extern "C" {

int sl_server_create(sl_renderer* const* renderers, sl_lighting* const* lightings, uint32_t n_scenes,
                     const sl_server_options* opt, sl_server** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (!renderers || n_scenes == 0) return fail(SL_ERR_INVALID_ARG, "no scenes");
  sl_server_options o{};
  if (opt) o = *opt;
  if (!o.max_views) o.max_views = 64;
  if (!o.pipelines) o.pipelines = 2;
  if (!o.max_slots) o.max_slots = 32ull << 20;
  if (!o.max_tiles) o.max_tiles = 1u << 19;
  if (!o.max_pixels) o.max_pixels = 32ull << 20;
  if (!o.max_view_pixels) o.max_view_pixels = 1920ull * 1080ull;
  if (!o.result_slots) o.result_slots = 2 * o.max_views;
  if (!o.tile_w) {
    o.tile_w = 16;
    o.tile_h = 16;
  }
  if (o.pipelines > 8 || o.max_views > 256 || o.max_view_pixels > o.max_pixels)
    return fail(SL_ERR_INVALID_ARG, "server options out of range");
  // device footprint of the pipelines: per slot (keys x2, values x2, order, record, rect, coverage mark) 73 B,
  // per tile entry (keys x2, values x2) 16 B at 2 entries per slot to start, per tile 28 B, per pixel 16 B
  const uint64_t per_pipe = 73ull * o.max_slots + 32ull * o.max_slots + 28ull * o.max_tiles + 16ull * o.max_pixels;
  uint64_t scene_bytes = 0;
  for (uint32_t k = 0; k < n_scenes; k++) {
    if (!renderers[k]) return fail(SL_ERR_INVALID_ARG, "null renderer");
    scene_bytes += renderers[k]->gaussians.bytes + renderers[k]->emitters.bytes;
  }
  if (o.hbm_budget_bytes && per_pipe * o.pipelines > o.hbm_budget_bytes)
    return fail(SL_ERR_ADMISSION, "the pipelines' buffers (" + std::to_string(per_pipe * o.pipelines) +
                                      " B) exceed the device-memory budget");
  sl_server* S = new sl_server();
  S->device = renderers[0]->device;
  cudaSetDevice(S->device);
  S->scenes.assign(renderers, renderers + n_scenes);
  S->lights.assign(n_scenes, nullptr);
  if (lightings)
    for (uint32_t k = 0; k < n_scenes; k++) S->lights[k] = lightings[k];
  S->opt = o;
  S->epoch = Clock::now();
  S->slot_floats = 4ull * o.max_view_pixels;
  cudaError_t e = cudaMallocHost((void**)&S->arena, sizeof(float) * S->slot_floats * o.result_slots);
  if (e != cudaSuccess) {
    delete S;
    return cuda_fail(e, "pinned result slots");
  }
  for (uint32_t k = o.result_slots; k > 0; k--) S->free_slots.push_back(k - 1);
  S->slot_state.assign(o.result_slots, kSlotFree);
  S->pipes.resize(o.pipelines);
  int rc = SL_OK;
  for (Pipe& p : S->pipes) {
    sl_batch_options bo{};
    bo.max_views = o.max_views;
    bo.max_slots = o.max_slots;
    bo.max_tiles = o.max_tiles;
    bo.tile_w = o.tile_w;
    bo.tile_h = o.tile_h;
    rc = sl_batch_create(renderers, lightings, n_scenes, &bo, &p.b);
    if (rc) break;
    if ((e = cudaStreamCreateWithFlags(&p.s, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&p.done, cudaEventDisableTiming)) != cudaSuccess ||
        (e = p.out.ensure(16ull * o.max_pixels)) != cudaSuccess) {
      rc = cuda_fail(e, "server pipeline");
      break;
    }
  }
  if (rc) {
    sl_server_destroy(S);
    return rc;
  }
  S->device_bytes = per_pipe * o.pipelines + scene_bytes;
  S->worker = std::thread(worker_loop, S);
  *out = S;
  return SL_OK;
}

int sl_server_submit(sl_server* S, const sl_server_request* req, uint64_t tag) {
  if (!S || !req) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (req->scene >= S->scenes.size()) return fail(SL_ERR_INVALID_ARG, "no such scene");
  sl_renderer* r = S->scenes[req->scene];
  int rc = check_frame(&req->frame, r->count, r->n_emitters);
  if (rc) return rc;
  if (!(req->light_scale >= 0.0f) || !(req->light_scale < 1e30f)) return fail(SL_ERR_INVALID_ARG, "bad light scale");
  Req q;
  q.tag = tag;
  q.scene = req->scene;
  q.frame = req->frame;
  for (int c = 0; c < 3; c++) q.eye[c] = req->eye[c];
  q.light_scale = req->light_scale;
  const uint32_t W = (uint32_t)req->frame.viewport[0], H = (uint32_t)req->frame.viewport[1];
  q.slots = footprint_slots(r, req->frame);
  q.tiles = (uint64_t)((W + S->opt.tile_w - 1) / S->opt.tile_w) * ((H + S->opt.tile_h - 1) / S->opt.tile_h);
  q.pixels = (uint64_t)W * H;
  if (q.slots > S->opt.max_slots || q.tiles > S->opt.max_tiles || q.pixels > S->opt.max_view_pixels) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->rejected++;
    return fail(SL_ERR_ADMISSION, "the request's footprint exceeds an empty batch (slots " +
                                      std::to_string(q.slots) + ", tiles " + std::to_string(q.tiles) + ", pixels " +
                                      std::to_string(q.pixels) + ")");
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return fail(SL_ERR_CANCELLED, "the server is shutting down");
    if (S->opt.max_pending && S->pending.size() >= S->opt.max_pending) {
      S->rejected++;
      return fail(SL_ERR_ADMISSION, "the pending queue is full (" + std::to_string(S->opt.max_pending) + ")");
    }
    q.t_submit = S->now();
    S->pending.push_back(q);
    S->submitted++;
  }
  S->cv.notify_all();
  return SL_OK;
}

int sl_server_poll(sl_server* S, sl_server_result* out, uint32_t cap, uint32_t* n_out, uint32_t wait_us) {
  if (!S || !n_out || (cap && !out)) return fail(SL_ERR_INVALID_ARG, "null argument");
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->results.empty() && wait_us)
    S->cv.wait_for(lk, std::chrono::microseconds(wait_us), [S] { return !S->results.empty(); });
  uint32_t n = 0;
  while (n < cap && !S->results.empty()) {
    const sl_server_result& res = S->results.front();
    if (res.status == SL_OK) S->slot_state[res.result_slot] = kSlotDelivered;
    out[n++] = res;
    S->results.pop_front();
  }
  *n_out = n;
  return SL_OK;
}

int sl_server_release(sl_server* S, uint32_t result_slot) {
  if (!S) return fail(SL_ERR_INVALID_ARG, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (result_slot >= S->opt.result_slots) return fail(SL_ERR_INVALID_ARG, "no such result slot");
  const uint8_t st = S->slot_state[result_slot];
  if (st != kSlotDelivered)
    return fail(SL_ERR_INVALID_ARG, st == kSlotFree ? "result slot released twice (or never handed out)"
                                                    : "result slot not yet handed out by sl_server_poll");
  S->slot_state[result_slot] = kSlotFree;
  S->free_slots.push_back(result_slot);
  S->cv.notify_all();
  return SL_OK;
}

int sl_server_get_stats(sl_server* S, sl_server_stats* st) {
  if (!S || !st) return fail(SL_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  memset(st, 0, sizeof(*st));
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->rejected = S->rejected;
  st->failed = S->failed;
  st->batches = S->batches;
  st->batch_views = S->batch_views;
  st->graph_replays = S->replays;
  st->pending = S->pending.size();
  st->device_bytes = S->device_bytes;
  st->free_result_slots = S->free_slots.size();
  st->reshaded_views = S->reshaded;
  st->relaunches = S->relaunches;
  return SL_OK;
}

int sl_server_destroy(sl_server* S) {
  if (!S) return SL_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->device);
  for (Pipe& p : S->pipes) {
    if (p.s) cudaStreamSynchronize(p.s);
    if (p.b) sl_batch_destroy(p.b);
    if (p.done) cudaEventDestroy(p.done);
    if (p.s) cudaStreamDestroy(p.s);
    p.out.release();
  }
  if (S->arena) cudaFreeHost(S->arena);
  delete S;
  return SL_OK;
}

}  // extern "C"
