// batch.cu -- batched loss-function chains: one grouped-tile S0 launch per
// tile shape and the conversion, KK and Dyson of every q-point, captured in
// one CUDA graph per batch.
//
// No counterpart in the reference, whose drivers run one q-point per process
// (the q loop of Sloss.f90:292).  A batch owns one shared context per q-point
// slot (the parent's resident basis, own buffers and stream).  rpa_batch_run
// takes up to max_q W requests and
//   1. per q-point, on its context: the k map and q, then rpa_chi0 with the
//      accumulation deferred -- pairs, windows, sort, tensor-core vertices and
//      the pre-split B tiles run, and the accumulation's launch is described
//      (AccGroupItem) instead of made -- the KK kernel matrix and V on the
//      device and every buffer of the later stages sized;
//   2. captures one graph: for each tile shape present, one grouped launch of
//      k_accum_ws_group over all q-points of that shape (each CTA finds its
//      q-point, frequency rows and tile pair from the item table), then per
//      q-point, as parallel branches on the q-points' streams, the conversion
//      of S0 to FP64, the KK transform and the FP64 Dyson solve (W, eps^-1);
//   3. launches the graph once (no host synchronisation inside it);
//      rpa_batch_wait then reads every q-point's status flags, eps^-1_11 and
//      W.  Between rpa_batch_launch and rpa_batch_wait the host is free: with
//      two batches, the per-request part of one runs while the other's graph
//      executes.
// Step 1 keeps the host decisions the chain needs (transition counts, the
// window bound, operand scales), which is why it stays outside the graph.

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "k_accum_ws.cuh"

namespace rpa {
int kk_prepare(rpa_ctx* c, int variant, int no, double domega);
int kk_run(rpa_ctx* c, int variant, int no, double domega);
int dyson_prepare(rpa_ctx* c, const double* V_host, bool want_epsinv);
int dyson_enqueue(rpa_ctx* c, bool want_epsinv, const double2** head_dev);
int df_to_f64(rpa_ctx* c, size_t n, int nw, bool cplx);
}  // namespace rpa

using namespace rpa;

struct rpa_batch {
  rpa_ctx* parent = nullptr;
  int device = 0;
  std::vector<rpa_ctx*> ctx;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  DevBuf d_items;
  void* h_items = nullptr;
  size_t h_items_bytes = 0;
  double times[4] = {0, 0, 0, 0};
  int groups = 0;
  long long nodes = 0;
  std::string err;
  // a launched batch awaiting rpa_batch_wait
  bool pending = false;
  cudaGraphExec_t exec = nullptr;
  std::vector<rpa_request> reqs;
  std::vector<const double2*> heads;
  int* status = nullptr;
  std::chrono::steady_clock::time_point t_launch;
};

namespace {

int bfail(rpa_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

double secs(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

}  // namespace

extern "C" {

int rpa_batch_create(rpa_batch** out, rpa_ctx* parent, int max_q) {
  if (!out || !parent || max_q < 1) return RPA_EINVAL;
  if (parent->precision != RPA_PREC_MIXED) return RPA_ESTATE;
  rpa_batch* b = new rpa_batch();
  b->parent = parent;
  b->device = parent->device;
  cudaSetDevice(b->device);
  int rc = RPA_OK;
  for (int i = 0; i < max_q && rc == RPA_OK; ++i) {
    rpa_ctx* c = nullptr;
    rc = rpa_create_shared(&c, parent, RPA_PREC_MIXED);
    if (rc == RPA_OK) b->ctx.push_back(c);
  }
  cudaError_t e = cudaSuccess;
  if (rc == RPA_OK) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (rc == RPA_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->join.assign(max_q, nullptr);
  for (int i = 0; i < max_q && rc == RPA_OK && e == cudaSuccess; ++i)
    e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
  // the grouped kernels' shared-memory limits, set once outside any capture
  int gbs[16], nios[16];
  const int nv = std::min(acc_variant_list(false, gbs, nios, 16), 16);
  for (int i = 0; i < nv && rc == RPA_OK && e == cudaSuccess; ++i)
    for (int sepa = 0; sepa < 2 && e == cudaSuccess; ++sepa)
      e = launch_ws_group_real(nullptr, b->device, sepa != 0, gbs[i], nios[i], nullptr, 0, 0);
  if (rc != RPA_OK || e != cudaSuccess) {
    rpa_batch_destroy(b);
    return rc != RPA_OK ? rc : RPA_ECUDA;
  }
  *out = b;
  return RPA_OK;
}

int rpa_batch_launch(rpa_batch* b, int nq, const rpa_request* reqs, int* status) {
  if (!b || !reqs || !status || nq < 1) return bfail(b, RPA_EINVAL, "rpa_batch_run: bad arguments");
  if (b->pending) return bfail(b, RPA_ESTATE, "rpa_batch_launch: the previous batch was not waited for");
  if (nq > (int)b->ctx.size()) return bfail(b, RPA_EINVAL, "rpa_batch_run: more requests than slots");
  for (int i = 0; i < nq; ++i) {
    const rpa_request& r = reqs[i];
    if (r.kind != RPA_REQ_W || r.args.mode != RPA_MODE_CHARGE || r.kk_variant != RPA_KK_SLOSS_REAL)
      return bfail(b, RPA_EINVAL, "rpa_batch_run: a batch takes W requests (charge mode, Sloss KK) only");
  }
  cudaSetDevice(b->device);
  const auto t0 = std::chrono::steady_clock::now();
  // ---- 1. per q-point: everything up to the pre-split B tiles, deferred accumulation
  for (int i = 0; i < nq; ++i) {
    const rpa_request& r = reqs[i];
    rpa_ctx* c = b->ctx[i];
    int rc = rpa_kmap(c, r.ntot, r.ktot, r.K1, r.R1, r.K2, r.R2, r.iG0);
    if (rc == RPA_OK) rc = rpa_set_q(c, r.q, r.nlf, r.ilf, r.parG);
    if (rc == RPA_OK) {
      c->defer_acc = true;
      rc = rpa_chi0(c, &r.args, nullptr, nullptr);
      c->defer_acc = false;
    }
    if (rc == RPA_OK) rc = kk_prepare(c, RPA_KK_SLOSS_REAL, r.args.no, r.args.domega);
    if (rc == RPA_OK) {
      std::vector<double> V;
      genV_of(c, r.c0, r.eps, V);
      rc = dyson_prepare(c, V.data(), false);
    }
    if (rc == RPA_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = RPA_ECUDA;
    status[i] = rc;
  }
  // ---- item tables, one group per tile shape
  struct Key {
    int gb, nio, sepa;
    bool operator<(const Key& o) const {
      return gb != o.gb ? gb < o.gb : (nio != o.nio ? nio < o.nio : sepa < o.sepa);
    }
  };
  std::map<Key, std::vector<AccGroupItem>> groups;
  for (int i = 0; i < nq; ++i) {
    rpa_ctx* c = b->ctx[i];
    if (status[i] != RPA_OK || !c->deferred) continue;
    AccGroupItem it;
    std::memcpy(&it, c->deferred_item, sizeof it);
    if (it.nrb * (long long)it.npy * it.npz == 0) continue;
    groups[{c->deferred_gb, c->deferred_nio, c->deferred_sepa ? 1 : 0}].push_back(it);
  }
  size_t nitems = 0;
  for (auto& g : groups) {
    long long cta = 0;
    for (AccGroupItem& it : g.second) {
      it.cta0 = cta;
      cta += (long long)it.nrb * it.npy * it.npz;
    }
    if (cta > 0x7fffffffLL) return bfail(b, RPA_EINVAL, "rpa_batch_run: more than 2^31 CTAs in one grouped launch");
    nitems += g.second.size();
  }
  const size_t ibytes = std::max<size_t>(1, nitems) * sizeof(AccGroupItem);
  if (b->h_items_bytes < ibytes) {
    if (b->h_items) cudaFreeHost(b->h_items);
    b->h_items = nullptr;
    b->h_items_bytes = 0;
    if (cudaHostAlloc(&b->h_items, ibytes, cudaHostAllocDefault) != cudaSuccess)
      return bfail(b, RPA_ENOMEM, "rpa_batch_run: page-locked item table");
    b->h_items_bytes = ibytes;
  }
  {
    // device item table (allocated through the first slot's context, which
    // reports an allocation failure)
    rpa_ctx* c0 = b->ctx[0];
    if (ensure(c0, b->d_items, ibytes) != RPA_OK) return bfail(b, RPA_ENOMEM, "rpa_batch_run: device item table");
  }
  {
    size_t off = 0;
    for (auto& g : groups) {
      std::memcpy(static_cast<char*>(b->h_items) + off * sizeof(AccGroupItem), g.second.data(),
                  g.second.size() * sizeof(AccGroupItem));
      off += g.second.size();
    }
  }
  if (nitems && cudaMemcpyAsync(b->d_items.p, b->h_items, nitems * sizeof(AccGroupItem), cudaMemcpyHostToDevice,
                                b->stream) != cudaSuccess)
    return bfail(b, RPA_ECUDA, "rpa_batch_run: item table upload");
  const auto t1 = std::chrono::steady_clock::now();
  // ---- 2. one graph: grouped accumulations, then per q-point conversion, KK, Dyson
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<const double2*>& heads = b->heads;
  heads.assign(nq, nullptr);
  std::string cerr;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess)
    return bfail(b, RPA_ECUDA, "rpa_batch_run: cudaStreamBeginCapture");
  {
    size_t off = 0;
    for (auto& g : groups) {
      const AccGroupItem& last = g.second.back();
      const long long nctas = last.cta0 + (long long)last.nrb * last.npy * last.npz;
      const AccGroupItem* dev = b->d_items.as<AccGroupItem>() + off;
      if (launch_ws_group_real(b->stream, b->device, g.first.sepa != 0, g.first.gb, g.first.nio, dev,
                               (int)g.second.size(), nctas) != cudaSuccess && cerr.empty())
        cerr = "grouped accumulation launch";
      off += g.second.size();
    }
    b->groups = (int)groups.size();
    if (cudaEventRecord(b->fork, b->stream) != cudaSuccess && cerr.empty()) cerr = "fork event";
    for (int i = 0; i < nq; ++i) {
      rpa_ctx* c = b->ctx[i];
      if (status[i] != RPA_OK) continue;
      const rpa_request& r = reqs[i];
      if (cudaStreamWaitEvent(c->stream, b->fork, 0) != cudaSuccess && cerr.empty()) cerr = "fork wait";
      int rc = RPA_OK;
      if (c->deferred) rc = df_to_f64(c, (size_t)c->deferred_nw * c->nlf * c->nlf, c->deferred_nw, false);
      if (rc == RPA_OK) rc = kk_run(c, RPA_KK_SLOSS_REAL, r.args.no, r.args.domega);
      if (rc == RPA_OK) rc = dyson_enqueue(c, false, &heads[i]);
      if (rc != RPA_OK && cerr.empty()) cerr = "q-point " + std::to_string(i) + ": " + c->err;
      if (cudaEventRecord(b->join[i], c->stream) != cudaSuccess && cerr.empty()) cerr = "join event";
      if (cudaStreamWaitEvent(b->stream, b->join[i], 0) != cudaSuccess && cerr.empty()) cerr = "join wait";
    }
  }
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
  if (ec != cudaSuccess || !cerr.empty()) {
    if (graph) cudaGraphDestroy(graph);
    return bfail(b, RPA_ECUDA, "rpa_batch_run: graph capture failed (" + (cerr.empty() ? std::string(cudaGetErrorString(ec)) : cerr) + ")");
  }
  size_t nnodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nnodes);
  b->nodes = (long long)nnodes;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return bfail(b, RPA_ECUDA, std::string("rpa_batch_run: cudaGraphInstantiate: ") + cudaGetErrorString(ei));
  const auto t2 = std::chrono::steady_clock::now();
  const cudaError_t el = cudaGraphLaunch(exec, b->stream);
  if (el != cudaSuccess) {
    cudaGraphExecDestroy(exec);
    return bfail(b, RPA_ECUDA, std::string("rpa_batch_run: graph launch: ") + cudaGetErrorString(el));
  }
  b->exec = exec;
  b->reqs.assign(reqs, reqs + nq);
  b->status = status;
  b->pending = true;
  b->t_launch = t2;
  b->times[0] = secs(t0, t1);
  b->times[1] = secs(t1, t2);
  return RPA_OK;
}

int rpa_batch_wait(rpa_batch* b) {
  if (!b || !b->pending) return bfail(b, RPA_ESTATE, "rpa_batch_wait: no launched batch");
  cudaSetDevice(b->device);
  b->pending = false;
  const cudaError_t el = cudaStreamSynchronize(b->stream);
  cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  if (el != cudaSuccess) return bfail(b, RPA_ECUDA, std::string("rpa_batch_wait: graph execution: ") + cudaGetErrorString(el));
  const auto t3 = std::chrono::steady_clock::now();
  const int nq = (int)b->reqs.size();
  const rpa_request* reqs = b->reqs.data();
  int* status = b->status;
  std::vector<const double2*>& heads = b->heads;
  // ---- 3. status and outputs per q-point
  int first_bad = RPA_OK;
  for (int i = 0; i < nq; ++i) {
    rpa_ctx* c = b->ctx[i];
    const rpa_request& r = reqs[i];
    if (status[i] != RPA_OK) {
      if (first_bad == RPA_OK) {
        first_bad = status[i];
        b->err = "q-point " + std::to_string(i) + ": " + c->err;
      }
      continue;
    }
    int fl[4] = {0, 0, 0, 0};
    int rc = cudaMemcpy(fl, c->d_flags.p, sizeof fl, cudaMemcpyDeviceToHost) == cudaSuccess ? RPA_OK : RPA_ECUDA;
    if (rc == RPA_OK && fl[2]) rc = fail(c, RPA_ETIMEOUT, "batch: a tensor-core completion wait timed out");
    if (rc == RPA_OK && fl[0]) rc = fail(c, RPA_ESINGULAR, "singular matrix in gjel at %d frequencies", fl[0]);
    const int nwo = r.args.no - 1, np = c->nlf * c->nlf;
    if (rc == RPA_OK && r.head_out &&
        cudaMemcpy(r.head_out, heads[i], sizeof(double2) * nwo, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = RPA_ECUDA;
    if (rc == RPA_OK && r.WT_out) {
      rc = ensure(c, c->d_tmp, sizeof(double2) * (size_t)nwo * np);
      if (rc == RPA_OK) {
        launch_transpose_wp_to_fortran(c->d_WT.as<double>(), c->d_tmp.as<double>(), nwo, np, 2, c->stream);
        rc = copy_d2h(c, r.WT_out, c->d_tmp.p, sizeof(double2) * (size_t)nwo * np);
      }
      if (rc == RPA_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = RPA_ECUDA;
    }
    if (rc == RPA_OK) {
      c->have_chi0 = true;
      c->have_W = true;
    }
    status[i] = rc;
    if (rc != RPA_OK && first_bad == RPA_OK) {
      first_bad = rc;
      b->err = "q-point " + std::to_string(i) + ": " + c->err;
    }
  }
  const auto t4 = std::chrono::steady_clock::now();
  b->times[2] = secs(b->t_launch, t3);
  b->times[3] = secs(t3, t4);
  return first_bad;
}

int rpa_batch_run(rpa_batch* b, int nq, const rpa_request* reqs, int* status) {
  const int rc = rpa_batch_launch(b, nq, reqs, status);
  if (rc != RPA_OK) return rc;
  return rpa_batch_wait(b);
}

int rpa_batch_info(const rpa_batch* b, double* times4, int* groups, long long* nodes) {
  if (!b) return RPA_EINVAL;
  if (times4)
    for (int i = 0; i < 4; ++i) times4[i] = b->times[i];
  if (groups) *groups = b->groups;
  if (nodes) *nodes = b->nodes;
  return RPA_OK;
}

const char* rpa_batch_last_error(const rpa_batch* b) { return b ? b->err.c_str() : "no batch"; }

int rpa_batch_destroy(rpa_batch* b) {
  if (!b) return RPA_EINVAL;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (!b->ctx.empty()) release(b->d_items);
  for (rpa_ctx* c : b->ctx) rpa_destroy(c);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->h_items) cudaFreeHost(b->h_items);
  delete b;
  return RPA_OK;
}

}  // extern "C"
