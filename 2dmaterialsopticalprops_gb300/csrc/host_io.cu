// host_io.cu -- host <-> device transfers of the large arrays (basis in,
// spectra out) for callers whose buffers are ordinary pageable memory.
//
// A pageable cudaMemcpy goes through the driver's own small bounce buffer at a
// fraction of the link rate.  Here each context owns a ring of two page-locked
// staging buffers and a few host copy threads: the DMA of one chunk overlaps
// the host copy of the previous one, so a Fortran array (or a NumPy array)
// moves at close to the page-locked rate.  Page-locked caller buffers are
// detected and copied directly.  The basis upload also overlaps its copies
// with the on-device transposes (two device staging buffers, a copy stream).

#include <algorithm>
#include <condition_variable>
#include <exception>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "rpa_internal.cuh"

namespace rpa {

// Splits one memcpy over a fixed set of threads; one copy at a time.
struct CopyPool {
  std::vector<std::thread> th;
  std::mutex m;
  std::condition_variable cv, cv_done;
  char* dst = nullptr;
  const char* src = nullptr;
  size_t n = 0, piece = 0;
  unsigned gen = 0;
  int pending = 0;
  bool stop = false;

  explicit CopyPool(int nt) {
    try {
      for (int t = 0; t < nt; ++t) th.emplace_back([this, t] { loop(t); });
    } catch (...) {
      shutdown();  // join the threads already started before the exception leaves
      throw;
    }
  }
  ~CopyPool() { shutdown(); }
  void shutdown() {
    {
      std::lock_guard<std::mutex> l(m);
      stop = true;
      ++gen;
    }
    cv.notify_all();
    for (auto& x : th)
      if (x.joinable()) x.join();
  }
  void loop(int t) {
    unsigned seen = 0;
    for (;;) {
      char* d;
      const char* s;
      size_t nn, pc;
      {
        std::unique_lock<std::mutex> l(m);
        cv.wait(l, [&] { return gen != seen; });
        seen = gen;
        if (stop) return;
        d = dst;
        s = src;
        nn = n;
        pc = piece;
      }
      const size_t off = (size_t)t * pc;
      if (off < nn) std::memcpy(d + off, s + off, std::min(pc, nn - off));
      {
        std::lock_guard<std::mutex> l(m);
        if (--pending == 0) cv_done.notify_one();
      }
    }
  }
  void copy(void* d, const void* s, size_t bytes) {
    const size_t nt = th.size();
    std::unique_lock<std::mutex> l(m);
    dst = static_cast<char*>(d);
    src = static_cast<const char*>(s);
    n = bytes;
    piece = ((bytes + nt - 1) / nt + 4095) & ~(size_t)4095;
    pending = (int)nt;
    ++gen;
    cv.notify_all();
    cv_done.wait(l, [&] { return pending == 0; });
  }
};

static constexpr size_t RING_BYTES = (size_t)64 << 20;  // per staging buffer
static constexpr size_t DIRECT_BELOW = (size_t)4 << 20;

// Page-locked host memory and memory the device can address (device or
// managed allocations) are copied directly by the DMA engines; only ordinary
// pageable memory goes through the staging ring.
static bool direct_copy(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void host_io_release(rpa_ctx* c);

static int ensure_ring(rpa_ctx* c) {
  if (c->io.pool) return RPA_OK;  // the pool is made last: the ring is complete
  host_io_release(c);             // whatever an earlier, failed attempt left
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaHostAlloc(&c->io.ring[b], RING_BYTES, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->io.ev[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->io.ev[2 + b], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->io.copy_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    host_io_release(c);
    return cuda_fail(c, e, "page-locked staging ring");
  }
  const unsigned hw = std::thread::hardware_concurrency();
  try {
    c->io.pool = new CopyPool((int)std::max(1u, std::min(8u, hw ? hw : 4u)));
  } catch (const std::exception& ex) {
    // no exception crosses the C ABI: thread or memory exhaustion is an error code
    host_io_release(c);
    return fail(c, RPA_ENOMEM, "host copy threads: %s", ex.what());
  }
  return RPA_OK;
}

int host_io_prepare(rpa_ctx* c) { return ensure_ring(c); }

void host_io_release(rpa_ctx* c) {
  delete c->io.pool;
  c->io.pool = nullptr;
  for (int b = 0; b < 2; ++b)
    if (c->io.ring[b]) cudaFreeHost(c->io.ring[b]), c->io.ring[b] = nullptr;
  for (auto& e : c->io.ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  if (c->io.copy_stream) cudaStreamDestroy(c->io.copy_stream), c->io.copy_stream = nullptr;
}

int copy_d2h(rpa_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return RPA_OK;
  if (bytes < DIRECT_BELOW || direct_copy(dst)) {
    RPA_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
    return RPA_OK;
  }
  RPA_TRY(ensure_ring(c));
  char* d = static_cast<char*>(dst);
  const char* s = static_cast<const char*>(src);
  // chunk j: DMA into ring[j % 2] on the context stream; the host threads copy
  // chunk j - 1 out of the other buffer meanwhile
  size_t prev_off = 0, prev_len = 0;
  int j = 0;
  for (size_t off = 0; off < bytes; off += RING_BYTES, ++j) {
    const size_t len = std::min(RING_BYTES, bytes - off);
    const int b = j & 1;
    RPA_CUDA(c, cudaMemcpyAsync(c->io.ring[b], s + off, len, cudaMemcpyDeviceToHost, c->stream));
    RPA_CUDA(c, cudaEventRecord(c->io.ev[b], c->stream));
    if (j > 0) {
      RPA_CUDA(c, cudaEventSynchronize(c->io.ev[b ^ 1]));
      c->io.pool->copy(d + prev_off, c->io.ring[b ^ 1], prev_len);
    }
    prev_off = off;
    prev_len = len;
  }
  const int b = (j - 1) & 1;
  RPA_CUDA(c, cudaEventSynchronize(c->io.ev[b]));
  c->io.pool->copy(d + prev_off, c->io.ring[b], prev_len);
  return RPA_OK;
}

// Coefficients of nks k-points, Fortran blocks C(npwx, nbnd) of complex
// doubles, into dst[k][i][b]: chunks of whole k-points go through two device
// staging buffers, the copy of chunk j on the copy stream overlapping the
// transpose of chunk j - 1 on the context stream.  Pageable sources pass
// through the page-locked ring first (host threads), which overlaps the DMA of
// the previous chunk.
int upload_basis(rpa_ctx* c, const double* coeff, int nks, int nbnd, int npwx, double2* dst) {
  const size_t per_k = (size_t)nbnd * npwx * sizeof(double2);
  RPA_TRY(ensure_ring(c));
  const bool pinned = direct_copy(coeff);
  // device chunk: up to 256 MB of whole k-points (at least one); a pageable
  // source also fits the chunk in one ring buffer
  size_t cap = pinned ? ((size_t)256 << 20) : RING_BYTES;
  const int kc = (int)std::max<size_t>(1, std::min<size_t>(nks, cap / per_k));
  const size_t chunk = per_k * kc;
  RPA_TRY(ensure(c, c->d_tmp, 2 * chunk));
  if (!pinned && chunk > RING_BYTES) {
    // one k-point larger than a ring buffer: plain (driver-staged) copies
    for (int k0 = 0; k0 < nks; k0 += kc) {
      const int nk = std::min(kc, nks - k0);
      RPA_CUDA(c, cudaMemcpyAsync(c->d_tmp.p, reinterpret_cast<const char*>(coeff) + per_k * k0, per_k * nk,
                                  cudaMemcpyHostToDevice, c->stream));
      launch_basis_transpose(c->d_tmp.as<double2>(), dst + (per_k / sizeof(double2)) * k0, nk, nbnd, npwx, c->stream);
      RPA_CUDA(c, cudaGetLastError());
      ++c->launches;
    }
    return RPA_OK;
  }
  cudaEvent_t* cdone = c->io.ev;       // copy j into device buffer j % 2 done (ring j % 2 free again)
  cudaEvent_t* tdone = c->io.ev + 2;   // transpose j done (device buffer j % 2 free again)
  int j = 0;
  for (int k0 = 0; k0 < nks; k0 += kc, ++j) {
    const int nk = std::min(kc, nks - k0);
    const int b = j & 1;
    const size_t len = per_k * nk;
    const char* src = reinterpret_cast<const char*>(coeff) + per_k * k0;
    char* dbuf = c->d_tmp.as<char>() + (size_t)b * chunk;
    if (j >= 2) RPA_CUDA(c, cudaStreamWaitEvent(c->io.copy_stream, tdone[b], 0));
    if (pinned) {
      RPA_CUDA(c, cudaMemcpyAsync(dbuf, src, len, cudaMemcpyDefault, c->io.copy_stream));
    } else {
      if (j >= 2) RPA_CUDA(c, cudaEventSynchronize(cdone[b]));  // ring b still feeding copy j - 2
      c->io.pool->copy(c->io.ring[b], src, len);
      RPA_CUDA(c, cudaMemcpyAsync(dbuf, c->io.ring[b], len, cudaMemcpyHostToDevice, c->io.copy_stream));
    }
    RPA_CUDA(c, cudaEventRecord(cdone[b], c->io.copy_stream));
    RPA_CUDA(c, cudaStreamWaitEvent(c->stream, cdone[b], 0));
    launch_basis_transpose(reinterpret_cast<const double2*>(dbuf), dst + (per_k / sizeof(double2)) * k0, nk, nbnd,
                           npwx, c->stream);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
    RPA_CUDA(c, cudaEventRecord(tdone[b], c->stream));
  }
  return RPA_OK;
}

}  // namespace rpa
