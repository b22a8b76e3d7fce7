// bcx_serve.cpp -- continuous-batching request server for sort_by_key,
// exclusive_scan and reduce.
//
// The reference has no serving layer: a caller issues one algorithm call at a
// time on a queue and blocks on each result (e.g. reduce into a host pointer,
// reduce.hpp:225).  This server accepts requests from any thread while
// earlier ones are on the GPU:
//   * a scheduler thread admits requests in arrival order whenever a slot
//     (a CUDA stream) is free, the device's free memory (measured at each
//     admission: the driver's free bytes plus what the stream-ordered pool
//     holds unused) covers the request's buffers and temporaries, and so does
//     the server's budget; a request that cannot fit while nothing else runs
//     fails with BCX_MEM_ALLOCATION_FAILURE;
//   * small requests that wait together with the same (kind, dtype, value
//     size) are packed into one batch and run as ONE segmented launch
//     (bcx_segmented_sort_pairs / bcx_segmented_scan / bcx_segmented_reduce);
//     large requests run alone with the plain kernels;
//   * each batch copies its inputs in, computes and copies results out on its
//     slot stream, so copies and kernels of different batches overlap;
//   * a host callback on the slot stream stamps the completion time of every
//     request in the batch and returns its memory to the budget.
// Buffers may be host memory (copied in and out on the slot stream) or
// device-resident (copied device to device into the batch and back; a lone
// request still computes in its own batch buffer so inputs stay untouched).
// Integer results are identical alone and batched; float scan/reduce use the
// compensated kernels in both cases (same tolerance, possibly different
// association).
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

#include "bcx.h"
#include "bcx_internal.h"

namespace bcx {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket;
  bcx_request r;
  Clock::time_point submitted;
  Clock::time_point finished;
  std::atomic<int> done{0};
  bcx_status status = BCX_SUCCESS;
};

struct Batch;

struct Slot {
  cudaStream_t stream = nullptr;
  bool busy = false;
  // Page-locked staging for a batch's segment offsets and copy pieces; reused
  // only after the slot's previous batch has completed.
  char *stage = nullptr;
  size_t stage_bytes = 0;
};

struct Batch {
  struct bcx_server *server = nullptr;
  int slot = -1;
  std::vector<std::shared_ptr<Request>> reqs;
  size_t bytes = 0;  // budget charged
  void *dev = nullptr;  // one device allocation for the whole batch
};

size_t elem_size(bcx_dtype t) { return dtype_size(t); }

}  // namespace
}  // namespace bcx

struct bcx_server {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<bcx::Request>> pending;
  std::map<uint64_t, std::shared_ptr<bcx::Request>> all;
  std::vector<bcx::Slot> slots;
  size_t budget = 0, used = 0;
  size_t small_limit = 1 << 18;     // requests up to this many elements may be batched
  size_t batch_elems = 1 << 24;     // elements per batch
  size_t batch_count = 4096;        // requests per batch
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread scheduler;
  int device = 0;
  // Fault injection for tests (bcx_server_inject_faults): a fixed figure for
  // the device's free memory instead of the measured one (0 = measure), and a
  // number of batch allocations to fail.
  size_t fake_free = 0;
  int fail_allocs = 0;
  // statistics
  uint64_t completed = 0, batches = 0, batched_requests = 0;
  std::vector<double> latencies_ms;
};

namespace bcx {
namespace {

// Device bytes a request needs (inputs/outputs plus its temporaries, for a
// batch of one).
size_t request_bytes(const bcx_request &r) {
  const size_t es = elem_size(r.dtype);
  switch (r.kind) {
    case BCX_REQ_SORT_PAIRS: return align256(r.n * es) + align256(r.n * r.value_bytes);
    case BCX_REQ_EXCLUSIVE_SCAN: return 2 * align256(r.n * es);
    case BCX_REQ_REDUCE: return align256(r.n * es) + 256;
  }
  return 0;
}

void CUDART_CB on_batch_done(void *p) {
  Batch *b = static_cast<Batch *>(p);
  const auto now = Clock::now();
  bcx_server *srv = b->server;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (auto &r : b->reqs) {
      r->finished = now;
      r->done.store(1);
      srv->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->submitted).count());
    }
    srv->completed += b->reqs.size();
    srv->used -= b->bytes;
    srv->slots[b->slot].busy = false;
  }
  srv->cv.notify_all();
  delete b;
}

// Runs a batch's operation on device buffers that are already in place:
// sort sorts (keys, values) in place, scan writes `second`, reduce writes one
// result per segment to `second`.  k == 1 uses the plain kernels.
bcx_status run_op(const bcx_request &r0, cudaStream_t s, size_t k, size_t n, void *keys, void *second,
                  const uint64_t *d_offs, void *tmp, size_t temp_bytes) {
  // A NULL temp with a size pointer would be a size query: pass no pointer
  // when the call needs no temporary storage.
  size_t tb_val = temp_bytes;
  size_t *tbp = temp_bytes ? &tb_val : nullptr;
  if (!temp_bytes) tmp = nullptr;
  const int comp = (r0.dtype == BCX_FLOAT || r0.dtype == BCX_DOUBLE) ? 1 : 0;
  unsigned char zero[8] = {0};
  if (r0.kind == BCX_REQ_SORT_PAIRS) {
    if (k == 1)
      return r0.value_bytes ? bcx_sort_pairs(s, r0.dtype, r0.value_bytes, keys, second, n, 0, tmp, tbp)
                            : bcx_sort_keys(s, r0.dtype, keys, n, 0, tmp, tbp);
    return bcx_segmented_sort_pairs(s, r0.dtype, r0.value_bytes, keys, second, n, d_offs, k, 0, tmp, tbp);
  }
  if (r0.kind == BCX_REQ_EXCLUSIVE_SCAN) {
    if (k == 1) return bcx_scan(s, r0.dtype, BCX_PLUS, 1, zero, keys, second, n, comp, tmp, tbp);
    return bcx_segmented_scan(s, r0.dtype, BCX_PLUS, 1, zero, keys, second, n, d_offs, k, comp, tmp, tbp);
  }
  if (k == 1) return bcx_reduce(s, r0.dtype, BCX_PLUS, keys, n, second, comp, tmp, tbp);
  return bcx_segmented_reduce(s, r0.dtype, BCX_PLUS, keys, d_offs, k, zero, second, comp, tmp, tbp);
}

bool device_resident(const bcx_request &r) { return (r.flags & BCX_REQ_DEVICE_RESIDENT) != 0; }

// A lone device-resident request computes straight on the caller's buffers
// (a sort first copies its inputs to the outputs unless they alias), so its
// only allocation is the temporary storage.
bcx_status launch_direct(bcx_server *srv, Batch *b, size_t temp_bytes) {
  cudaStream_t s = srv->slots[b->slot].stream;
  const bcx_request &r = b->reqs[0]->r;
  const size_t es = elem_size(r.dtype);
  if (temp_bytes) BCX_CUDA(cudaMallocAsync(&b->dev, temp_bytes, s));
  bcx_status rc = BCX_SUCCESS;
  if (r.n) {
    if (r.kind == BCX_REQ_SORT_PAIRS) {
      if (r.out != r.keys) BCX_CUDA(cudaMemcpyAsync(r.out, r.keys, r.n * es, cudaMemcpyDeviceToDevice, s));
      if (r.value_bytes && r.out_values != r.values)
        BCX_CUDA(cudaMemcpyAsync(r.out_values, r.values, r.n * r.value_bytes, cudaMemcpyDeviceToDevice, s));
      rc = run_op(r, s, 1, r.n, r.out, r.out_values, nullptr, b->dev, temp_bytes);
    } else {
      rc = run_op(r, s, 1, r.n, const_cast<void *>(r.keys), r.out, nullptr, b->dev, temp_bytes);
    }
  } else if (r.kind == BCX_REQ_REDUCE) {
    BCX_CUDA(cudaMemsetAsync(r.out, 0, es, s));
  }
  if (rc)
    for (auto &q : b->reqs) q->status = rc;
  if (b->dev) BCX_CUDA(cudaFreeAsync(b->dev, s));
  BCX_CUDA(cudaLaunchHostFunc(s, on_batch_done, b));
  return BCX_SUCCESS;
}

// Appends the pieces that move `bytes` bytes from src to dst.
void add_pieces(std::vector<CopyChunk> &v, const void *src, void *dst, size_t bytes) {
  for (size_t o = 0; o < bytes; o += kCopyChunkBytes)
    v.push_back(CopyChunk{static_cast<const char *>(src) + o, static_cast<char *>(dst) + o,
                          uint64_t(std::min(kCopyChunkBytes, bytes - o)), 0});
}

// Enqueue one batch on its slot stream.  Called without the server lock.
// Layout of the batch allocation:
// keys/input | values or output | offsets + copy pieces | temp.  Host
// buffers move with one copy per buffer; device-resident buffers move with
// one gather launch in and one scatter launch out for the whole batch.
bcx_status launch_batch(bcx_server *srv, Batch *b, size_t temp_bytes) {
  Slot &slot = srv->slots[b->slot];
  cudaStream_t s = slot.stream;
  const bcx_request &r0 = b->reqs[0]->r;
  const bool dev_res = device_resident(r0);
  const size_t k = b->reqs.size();
  if (dev_res && k == 1) return launch_direct(srv, b, temp_bytes);
  const size_t es = elem_size(r0.dtype);
  size_t n = 0;
  for (auto &r : b->reqs) n += r->r.n;
  const size_t a_keys = 0;
  const size_t a_second = align256(n * es);
  const size_t second_bytes = r0.kind == BCX_REQ_SORT_PAIRS ? n * r0.value_bytes
                              : r0.kind == BCX_REQ_EXCLUSIVE_SCAN ? n * es
                                                                   : k * es;
  const size_t a_meta = a_second + align256(second_bytes);
  char *base = nullptr;  // known after the allocation; pieces are built relative to 0 first
  // Offsets and (device-resident) pieces, relative to the batch allocation.
  std::vector<uint64_t> offsets(k + 1, 0);
  std::vector<CopyChunk> gather, scatter;
  size_t off = 0;
  for (size_t i = 0; i < k; ++i) {
    const bcx_request &r = b->reqs[i]->r;
    offsets[i] = off;
    if (dev_res) {
      add_pieces(gather, r.keys, reinterpret_cast<void *>(a_keys + off * es), r.n * es);
      if (r.kind == BCX_REQ_SORT_PAIRS) {
        add_pieces(gather, r.values, reinterpret_cast<void *>(a_second + off * r.value_bytes), r.n * r.value_bytes);
        add_pieces(scatter, reinterpret_cast<void *>(a_keys + off * es), r.out, r.n * es);
        add_pieces(scatter, reinterpret_cast<void *>(a_second + off * r.value_bytes), r.out_values,
                   r.n * r.value_bytes);
      } else if (r.kind == BCX_REQ_EXCLUSIVE_SCAN) {
        add_pieces(scatter, reinterpret_cast<void *>(a_second + off * es), r.out, r.n * es);
      } else {
        add_pieces(scatter, reinterpret_cast<void *>(a_second + i * es), r.out, es);
      }
    }
    off += r.n;
  }
  offsets[k] = off;
  const size_t offs_bytes = align256((k + 1) * sizeof(uint64_t));
  const size_t meta_bytes = offs_bytes + (gather.size() + scatter.size()) * sizeof(CopyChunk);
  const size_t a_temp = a_meta + align256(meta_bytes);
  const size_t total = a_temp + temp_bytes;
  if (slot.stage_bytes < meta_bytes) {
    if (slot.stage) BCX_CUDA(cudaFreeHost(slot.stage));
    slot.stage = nullptr;
    slot.stage_bytes = 0;
    const size_t want = std::max(meta_bytes, size_t(1) << 20);
    BCX_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&slot.stage), want, cudaHostAllocDefault));
    slot.stage_bytes = want;
  }
  BCX_CUDA(cudaMallocAsync(&b->dev, total, s));
  base = static_cast<char *>(b->dev);
  // Rebase the batch-relative addresses of the pieces.
  for (auto &c : gather) c.dst = base + reinterpret_cast<uintptr_t>(c.dst);
  for (auto &c : scatter) c.src = base + reinterpret_cast<uintptr_t>(c.src);
  std::memcpy(slot.stage, offsets.data(), (k + 1) * sizeof(uint64_t));
  CopyChunk *stage_pieces = reinterpret_cast<CopyChunk *>(slot.stage + offs_bytes);
  if (!gather.empty()) std::memcpy(stage_pieces, gather.data(), gather.size() * sizeof(CopyChunk));
  if (!scatter.empty())
    std::memcpy(stage_pieces + gather.size(), scatter.data(), scatter.size() * sizeof(CopyChunk));
  BCX_CUDA(cudaMemcpyAsync(base + a_meta, slot.stage, meta_bytes, cudaMemcpyHostToDevice, s));
  const uint64_t *d_offs = reinterpret_cast<const uint64_t *>(base + a_meta);
  const CopyChunk *d_pieces = reinterpret_cast<const CopyChunk *>(base + a_meta + offs_bytes);
  // inputs
  if (dev_res) {
    bcx_status rc = copy_chunks(d_pieces, gather.size(), s);
    if (rc) return rc;
  } else {
    off = 0;
    for (size_t i = 0; i < k; ++i) {
      const bcx_request &r = b->reqs[i]->r;
      if (r.n) {
        BCX_CUDA(cudaMemcpyAsync(base + a_keys + off * es, r.keys, r.n * es, cudaMemcpyDefault, s));
        if (r.kind == BCX_REQ_SORT_PAIRS && r.value_bytes)
          BCX_CUDA(cudaMemcpyAsync(base + a_second + off * r.value_bytes, r.values, r.n * r.value_bytes,
                                   cudaMemcpyDefault, s));
      }
      off += r.n;
    }
  }
  bcx_status rc = run_op(r0, s, k, n, base + a_keys, base + a_second, d_offs, base + a_temp, temp_bytes);
  if (rc)
    for (auto &r : b->reqs) r->status = rc;
  // outputs
  if (dev_res) {
    bcx_status rc2 = copy_chunks(d_pieces + gather.size(), scatter.size(), s);
    if (rc2) return rc2;
  } else {
    off = 0;
    for (size_t i = 0; i < k; ++i) {
      const bcx_request &r = b->reqs[i]->r;
      if (r.kind == BCX_REQ_SORT_PAIRS) {
        if (r.n) {
          BCX_CUDA(cudaMemcpyAsync(r.out, base + a_keys + off * es, r.n * es, cudaMemcpyDefault, s));
          if (r.value_bytes)
            BCX_CUDA(cudaMemcpyAsync(r.out_values, base + a_second + off * r.value_bytes, r.n * r.value_bytes,
                                     cudaMemcpyDefault, s));
        }
      } else if (r.kind == BCX_REQ_EXCLUSIVE_SCAN) {
        if (r.n) BCX_CUDA(cudaMemcpyAsync(r.out, base + a_second + off * es, r.n * es, cudaMemcpyDefault, s));
      } else {
        BCX_CUDA(cudaMemcpyAsync(r.out, base + a_second + i * es, es, cudaMemcpyDefault, s));
      }
      off += r.n;
    }
  }
  BCX_CUDA(cudaFreeAsync(b->dev, s));
  BCX_CUDA(cudaLaunchHostFunc(s, on_batch_done, b));
  return BCX_SUCCESS;
}

// Temporary bytes of a batch (query protocol of the underlying call).  The
// query sees 256-byte aligned stand-in pointers, like the batch allocation's.
size_t batch_temp(const std::vector<std::shared_ptr<Request>> &reqs, size_t n) {
  const bcx_request &r0 = reqs[0]->r;
  const size_t k = reqs.size();
  size_t tb = 0;
  unsigned char zero[8] = {0};
  void *p = reinterpret_cast<void *>(uintptr_t(256));
  const uint64_t *po = reinterpret_cast<const uint64_t *>(p);
  bcx_status rc = BCX_SUCCESS;
  if (r0.kind == BCX_REQ_SORT_PAIRS) {
    if (k == 1)
      rc = r0.value_bytes ? bcx_sort_pairs(nullptr, r0.dtype, r0.value_bytes, p, p, n, 0, nullptr, &tb)
                          : bcx_sort_keys(nullptr, r0.dtype, p, n, 0, nullptr, &tb);
    else
      rc = bcx_segmented_sort_pairs(nullptr, r0.dtype, r0.value_bytes, p, p, n, po, k, 0, nullptr, &tb);
  } else if (r0.kind == BCX_REQ_EXCLUSIVE_SCAN) {
    const int comp = (r0.dtype == BCX_FLOAT || r0.dtype == BCX_DOUBLE) ? 1 : 0;
    if (k == 1) rc = bcx_scan(nullptr, r0.dtype, BCX_PLUS, 1, zero, p, p, n, comp, nullptr, &tb);
    else rc = bcx_segmented_scan(nullptr, r0.dtype, BCX_PLUS, 1, zero, p, p, n, po, k, comp, nullptr, &tb);
  } else {
    const int comp = (r0.dtype == BCX_FLOAT || r0.dtype == BCX_DOUBLE) ? 1 : 0;
    if (k == 1) rc = bcx_reduce(nullptr, r0.dtype, BCX_PLUS, p, n, p, comp, nullptr, &tb);
    else rc = bcx_segmented_reduce(nullptr, r0.dtype, BCX_PLUS, p, po, k, zero, p, comp, nullptr, &tb);
  }
  return rc ? 0 : tb;
}

// Device memory a new batch can still get: the driver's free memory plus what
// the stream-ordered pool holds unused (freed batches stay cached there).
size_t available_memory(const bcx_server *srv) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, srv->device) == cudaSuccess) {
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      free_b += size_t(reserved - used);
  }
  return free_b;
}

// Takes one injected allocation failure, if any are left (server lock held).
bool take_injected_failure(bcx_server *srv) {
  if (srv->fail_allocs <= 0) return false;
  --srv->fail_allocs;
  return true;
}

// No request waiting or running (server lock held).
bool idle_locked(const bcx_server *srv) {
  if (!srv->pending.empty()) return false;
  for (auto &sl : srv->slots)
    if (sl.busy) return false;
  return true;
}

bool same_group(const bcx_request &a, const bcx_request &b) {
  return a.kind == b.kind && a.dtype == b.dtype && a.value_bytes == b.value_bytes &&
         device_resident(a) == device_resident(b);
}

// The scheduler never holds the server lock across a CUDA call: batch
// completions run as host functions on CUDA's callback thread and take the
// lock, and a CUDA call that waits for stream progress (a copy from pageable
// memory, first-use device setup) would otherwise wait for a callback that
// waits for the lock.
void scheduler_loop(bcx_server *srv) {
  cudaSetDevice(srv->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  while (true) {
    srv->cv.wait(lk, [&] {
      if (srv->stop) return true;
      if (srv->pending.empty()) return false;
      for (auto &sl : srv->slots)
        if (!sl.busy) return true;
      return false;
    });
    if (srv->stop && srv->pending.empty()) break;
    int slot = -1;
    for (size_t i = 0; i < srv->slots.size(); ++i)
      if (!srv->slots[i].busy) {
        slot = int(i);
        break;
      }
    if (slot < 0 || srv->pending.empty()) continue;
    // Build a batch around the oldest request (only this thread removes
    // requests from `pending`, so the batch stays valid while unlocked).
    auto first = srv->pending.front();
    std::vector<std::shared_ptr<Request>> reqs{first};
    size_t n = first->r.n;
    if (first->r.n <= srv->small_limit) {
      for (auto it = srv->pending.begin() + 1; it != srv->pending.end(); ++it) {
        const auto &q = *it;
        if (reqs.size() >= srv->batch_count) break;
        if (!same_group(q->r, first->r) || q->r.n > srv->small_limit) continue;
        if (n + q->r.n > srv->batch_elems) break;
        reqs.push_back(q);
        n += q->r.n;
      }
    }
    const size_t fake = srv->fake_free;
    lk.unlock();
    const size_t temp = batch_temp(reqs, n);
    size_t bytes = 0;
    if (reqs.size() == 1 && device_resident(first->r)) {
      bytes = temp;  // computes on the caller's buffers
    } else {
      for (auto &r : reqs) bytes += request_bytes(r->r);
      // offsets and copy pieces: at most 4 buffers per request, one piece per
      // started kCopyChunkBytes of each
      const size_t pieces = 4 * reqs.size() + 2 * bytes / kCopyChunkBytes;
      bytes += temp + 3 * 256 + align256((reqs.size() + 1) * 8) + pieces * sizeof(CopyChunk);
    }
    // Admission by free device memory, measured now (outside the lock), and by
    // the server's budget.
    const size_t avail = fake ? fake : available_memory(srv);
    lk.lock();
    const bool fits = srv->used + bytes <= srv->budget && bytes <= avail;
    if (!fits && srv->used > 0) {
      // Not enough memory right now: wait for a completion to free some.
      srv->cv.wait(lk);
      continue;
    }
    if (!fits && bytes > avail) {
      // Nothing of ours is running and the device still lacks the memory:
      // fail the batch's requests instead of waiting for memory that only
      // another process could free.
      for (auto &r : reqs) {
        auto it = std::find(srv->pending.begin(), srv->pending.end(), r);
        if (it != srv->pending.end()) srv->pending.erase(it);
        r->status = BCX_MEM_ALLOCATION_FAILURE;
        r->finished = Clock::now();
        r->done.store(1);
      }
      srv->cv.notify_all();
      continue;
    }
    // Admit: remove from pending (preserving the order of the rest).
    for (auto &r : reqs) {
      auto it = std::find(srv->pending.begin(), srv->pending.end(), r);
      if (it != srv->pending.end()) srv->pending.erase(it);
    }
    Batch *b = new Batch();
    b->server = srv;
    b->slot = slot;
    b->reqs = reqs;
    b->bytes = bytes;
    srv->slots[slot].busy = true;
    srv->used += bytes;
    srv->batches += 1;
    if (reqs.size() > 1) srv->batched_requests += reqs.size();
    const bool inject = take_injected_failure(srv);
    lk.unlock();
    // On success the batch belongs to its completion callback from here on.
    bcx_status rc = BCX_SUCCESS;
    if (inject) {
      set_error("server: injected allocation failure");
      rc = BCX_MEM_ALLOCATION_FAILURE;
    } else {
      rc = launch_batch(srv, b, temp);
    }
    if (rc && b->dev) cudaFreeAsync(b->dev, srv->slots[slot].stream);
    lk.lock();
    if (rc) {
      for (auto &r : reqs) {
        r->status = rc;
        r->finished = Clock::now();
        r->done.store(1);
      }
      srv->used -= bytes;
      srv->slots[slot].busy = false;
      delete b;
      srv->cv.notify_all();
    }
  }
}

}  // namespace
}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_server_create(bcx_server **out, int slots, size_t memory_budget_bytes) {
  clear_error();
  BCX_CHECK(out && slots > 0 && slots <= 64, BCX_INVALID_VALUE, "bad server arguments");
  auto *srv = new bcx_server();
  BCX_CUDA(cudaGetDevice(&srv->device));
  if (memory_budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    BCX_CUDA(cudaMemGetInfo(&free_b, &total_b));
    memory_budget_bytes = free_b / 2;
  }
  srv->budget = memory_budget_bytes;
  srv->slots.resize(size_t(slots));
  for (auto &sl : srv->slots) BCX_CUDA(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
  srv->scheduler = std::thread(scheduler_loop, srv);
  *out = srv;
  return BCX_SUCCESS;
}

bcx_status bcx_server_configure(bcx_server *srv, size_t small_limit, size_t batch_elems, size_t batch_count) {
  BCX_CHECK(srv, BCX_INVALID_VALUE, "NULL server");
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->small_limit = small_limit;
  if (batch_elems) srv->batch_elems = batch_elems;
  if (batch_count) srv->batch_count = batch_count;
  return BCX_SUCCESS;
}

bcx_status bcx_server_inject_faults(bcx_server *srv, size_t fake_free_bytes, int fail_allocations) {
  BCX_CHECK(srv, BCX_INVALID_VALUE, "NULL server");
  BCX_CHECK(fail_allocations >= 0, BCX_INVALID_VALUE, "fail_allocations must be >= 0");
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->fake_free = fake_free_bytes;
    srv->fail_allocs = fail_allocations;
  }
  srv->cv.notify_all();
  return BCX_SUCCESS;
}

bcx_status bcx_server_submit(bcx_server *srv, const bcx_request *req, uint64_t *ticket) {
  clear_error();
  BCX_CHECK(srv && req && ticket, BCX_INVALID_VALUE, "NULL argument");
  BCX_CHECK(req->kind >= BCX_REQ_SORT_PAIRS && req->kind <= BCX_REQ_REDUCE, BCX_INVALID_VALUE, "bad request kind");
  BCX_CHECK(dtype_valid(req->dtype), BCX_INVALID_VALUE, "bad dtype");
  BCX_CHECK(req->n == 0 || req->keys, BCX_INVALID_VALUE, "request without input");
  BCX_CHECK(req->n == 0 || req->out, BCX_INVALID_VALUE, "request without output");
  BCX_CHECK(req->kind != BCX_REQ_SORT_PAIRS || req->value_bytes == 0 || (req->values && req->out_values),
            BCX_INVALID_VALUE, "sort request without values");
  auto r = std::make_shared<Request>();
  r->r = *req;
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    BCX_CHECK(request_bytes(*req) <= srv->budget, BCX_MEM_ALLOCATION_FAILURE,
              "request needs more device memory than the server budget");
    r->ticket = srv->next_ticket++;
    srv->pending.push_back(r);
    srv->all[r->ticket] = r;
    *ticket = r->ticket;
  }
  srv->cv.notify_all();
  return BCX_SUCCESS;
}

bcx_status bcx_server_wait_for(bcx_server *srv, uint64_t ticket, double timeout_ms, double *latency_ms) {
  BCX_CHECK(srv, BCX_INVALID_VALUE, "NULL server");
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->all.find(ticket);
  BCX_CHECK(it != srv->all.end(), BCX_INVALID_VALUE, "unknown ticket %llu", (unsigned long long)ticket);
  std::shared_ptr<Request> r = it->second;
  auto ready = [&] { return r->done.load() != 0; };
  if (timeout_ms < 0) {
    srv->cv.wait(lk, ready);
  } else if (!srv->cv.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
    set_error("request %llu not finished after %.0f ms", (unsigned long long)ticket, timeout_ms);
    return BCX_DEVICE_TIMEOUT;  // the ticket stays valid
  }
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
  srv->all.erase(ticket);
  if (r->status) set_error("request %llu failed", (unsigned long long)ticket);
  return r->status;
}

bcx_status bcx_server_wait(bcx_server *srv, uint64_t ticket, double *latency_ms) {
  return bcx_server_wait_for(srv, ticket, -1.0, latency_ms);
}

bcx_status bcx_server_drain(bcx_server *srv) {
  BCX_CHECK(srv, BCX_INVALID_VALUE, "NULL server");
  std::unique_lock<std::mutex> lk(srv->mu);
  srv->cv.wait(lk, [&] { return idle_locked(srv); });
  return BCX_SUCCESS;
}

bcx_status bcx_server_stats(bcx_server *srv, bcx_server_stats_t *st) {
  BCX_CHECK(srv && st, BCX_INVALID_VALUE, "NULL argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  std::memset(st, 0, sizeof(*st));
  st->completed = srv->completed;
  st->batches = srv->batches;
  st->batched_requests = srv->batched_requests;
  st->pending = srv->pending.size();
  st->used_bytes = srv->used;
  std::vector<double> v = srv->latencies_ms;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) { return v[std::min(v.size() - 1, size_t(p * (v.size() - 1) + 0.5))]; };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = v.back();
  }
  return BCX_SUCCESS;
}

bcx_status bcx_server_reset_stats(bcx_server *srv) {
  BCX_CHECK(srv, BCX_INVALID_VALUE, "NULL server");
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->completed = srv->batches = srv->batched_requests = 0;
  srv->latencies_ms.clear();
  return BCX_SUCCESS;
}

bcx_status bcx_server_destroy(bcx_server *srv) {
  if (!srv) return BCX_SUCCESS;
  {
    // Requests still running after a minute mean the GPU or a caller's
    // buffers are stuck: report it and leave the server (and its streams)
    // alive rather than block the caller forever.
    std::unique_lock<std::mutex> lk(srv->mu);
    if (!srv->cv.wait_for(lk, std::chrono::seconds(60), [&] { return idle_locked(srv); })) {
      set_error("server destroy: requests still running after 60 s; server left alive");
      return BCX_DEVICE_TIMEOUT;
    }
  }
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv.notify_all();
  if (srv->scheduler.joinable()) srv->scheduler.join();
  for (auto &sl : srv->slots) {
    cudaStreamDestroy(sl.stream);
    if (sl.stage) cudaFreeHost(sl.stage);
  }
  delete srv;
  return BCX_SUCCESS;
}

}  // extern "C"
