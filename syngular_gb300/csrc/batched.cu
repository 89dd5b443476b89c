// Batched MPO x MPS + TT-SVD rounding + overlap over many independent
// instances of uneven size (the batched workload's C entry points).
//
// A plan holds, per instance, the workspace the fused round and the overlap
// need; instances are dealt longest-first onto `lanes` stream lanes (the
// least-loaded lane by workspace bytes), and each lane runs its instances one
// after another inside one workspace region, so device memory is the sum over
// lanes of the largest instance of the lane.  A launch forks the lanes off
// the caller's stream with events and joins them back, enqueueing everything
// without a host synchronisation or allocation, so it can be captured into a
// CUDA graph and replayed.  The plan is host data; the lanes' streams and
// events are created on the first launch (on the current device) and
// released by sgt_batched_plan_destroy.
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

extern "C" {
SGT_API size_t sgt_mpo_mps_round_workspace_size(int n, const int64_t* wshape, const int64_t* xshape, int64_t chi,
                                                int precision);
SGT_API int sgt_mpo_mps_round(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                              const int64_t* xshape, int64_t chi, int precision, double* const* out,
                              double* spectra, double* discarded, int* status, void* ws, size_t ws_bytes,
                              void* stream);
SGT_API size_t sgt_overlap_workspace_size(int n, const int64_t* xshape, const int64_t* yshape);
SGT_API int sgt_overlap_sweep(int n, const double* const* X, const int64_t* xshape, const double* const* Y,
                              const int64_t* yshape, double* result, void* ws, size_t ws_bytes, void* stream);
SGT_API int sgt_svd_round_shapes(int n, const int64_t* shape, int64_t chi, int64_t* out_shape,
                                 int64_t* spec_count);
}

struct sgt_batched_plan_s {
  struct Inst {
    int n = 0;
    int64_t chi = 0;
    std::vector<int64_t> wshape, xshape, oshape;
    size_t ws = 0;
    int lane = 0;
  };
  int precision = 0;
  std::vector<Inst> inst;
  std::vector<std::vector<int>> lanes;  // instance indices per lane, in launch order
  std::vector<size_t> lane_off, lane_bytes;
  size_t total = 0;
  std::mutex mu;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done;
  cudaEvent_t fork = nullptr;
};

namespace {

int create_streams(sgt_batched_plan_s* p) {
  std::lock_guard<std::mutex> g(p->mu);
  if (!p->streams.empty()) return SGT_OK;
  SGT_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
  for (size_t l = 0; l < p->lanes.size(); ++l) {
    cudaStream_t s;
    cudaEvent_t e;
    SGT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    SGT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    p->streams.push_back(s);
    p->done.push_back(e);
  }
  return SGT_OK;
}

}  // namespace

extern "C" {

// count instances; n[i] sites each, wshape[i] (4 n[i]) / xshape[i] (3 n[i])
// shapes, chi[i] the rounding bond; lanes >= 1.  *plan receives the plan,
// *ws_bytes the workspace one launch needs (256-byte aligned regions).
SGT_API int sgt_batched_plan_create(int count, const int* n, const int64_t* const* wshape,
                                    const int64_t* const* xshape, const int64_t* chi, int precision, int lanes,
                                    sgt_batched_plan_s** plan, size_t* ws_bytes) {
  SGT_REQUIRE(count >= 1 && n && wshape && xshape && chi && plan && ws_bytes && lanes >= 1, SGT_ERR_INVALID,
              "batched_plan: bad argument");
  auto* p = new sgt_batched_plan_s();
  p->precision = precision;
  p->inst.resize(count);
  for (int i = 0; i < count; ++i) {
    auto& in = p->inst[i];
    in.n = n[i];
    in.chi = chi[i];
    if (in.n < 1 || !wshape[i] || !xshape[i]) {
      delete p;
      SGT_REQUIRE(false, SGT_ERR_INVALID, "batched_plan: instance %d has no sites", i);
    }
    in.wshape.assign(wshape[i], wshape[i] + 4 * (size_t)in.n);
    in.xshape.assign(xshape[i], xshape[i] + 3 * (size_t)in.n);
    const size_t wr = sgt_mpo_mps_round_workspace_size(in.n, in.wshape.data(), in.xshape.data(), in.chi, precision);
    // rounded shapes (product bond l * b, physical out leg, right l' * b')
    std::vector<int64_t> pshape(3 * (size_t)in.n), cnt((size_t)std::max(1, in.n - 1));
    for (int k = 0; k < in.n; ++k) {
      pshape[3 * k] = in.xshape[3 * k] * in.wshape[4 * k];
      pshape[3 * k + 1] = in.wshape[4 * k + 2];
      pshape[3 * k + 2] = in.xshape[3 * k + 2] * in.wshape[4 * k + 3];
    }
    in.oshape.resize(3 * (size_t)in.n);
    const int rc = sgt_svd_round_shapes(in.n, pshape.data(), in.chi, in.oshape.data(), cnt.data());
    const size_t wo = rc == SGT_OK ? sgt_overlap_workspace_size(in.n, in.xshape.data(), in.oshape.data()) : 0;
    if (wr == 0 || wo == 0 || rc != SGT_OK) {
      delete p;
      SGT_REQUIRE(false, SGT_ERR_INVALID, "batched_plan: instance %d has inconsistent shapes", i);
    }
    in.ws = (std::max(wr, wo) + 255) & ~size_t(255);
  }
  // most work first onto the least-loaded lane (longest-processing-time
  // order); an instance's work is the rounding's leading term, per bond the
  // squared product bond times the bond matrix side (d chi)
  std::vector<double> work(count, 0.0);
  for (int i = 0; i < count; ++i) {
    const auto& in = p->inst[i];
    for (int k = 0; k < in.n; ++k) {
      const double r = (double)(in.xshape[3 * k] * in.wshape[4 * k]);
      const double r2 = (double)(in.xshape[3 * k + 2] * in.wshape[4 * k + 3]);
      work[i] += r * r * (double)in.wshape[4 * k + 2] * std::min(r2, (double)in.chi);
    }
  }
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  const int L = std::min(lanes, count);
  std::vector<double> load(L, 0.0);
  p->lanes.assign(L, {});
  for (int i : order) {
    const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    p->lanes[l].push_back(i);
    p->inst[i].lane = l;
    load[l] += work[i];
  }
  p->lane_off.assign(L, 0);
  p->lane_bytes.assign(L, 0);
  size_t off = 0;
  for (int l = 0; l < L; ++l) {
    size_t mx = 0;
    for (int i : p->lanes[l]) mx = std::max(mx, p->inst[i].ws);
    p->lane_off[l] = off;
    p->lane_bytes[l] = mx;
    off += mx;
  }
  p->total = off;
  *plan = p;
  *ws_bytes = off;
  return SGT_OK;
}

// Lane of instance i (-1 if out of range): the deal the plan made.
SGT_API int sgt_batched_plan_lane(const sgt_batched_plan_s* plan, int i) {
  if (!plan || i < 0 || i >= (int)plan->inst.size()) return -1;
  return plan->inst[i].lane;
}

// Rounded core shapes of instance i (3 n[i] values) into out_shape.
SGT_API int sgt_batched_plan_out_shape(const sgt_batched_plan_s* plan, int i, int64_t* out_shape) {
  SGT_REQUIRE(plan && out_shape && i >= 0 && i < (int)plan->inst.size(), SGT_ERR_INVALID,
              "batched_plan_out_shape: bad argument");
  std::copy(plan->inst[i].oshape.begin(), plan->inst[i].oshape.end(), out_shape);
  return SGT_OK;
}

// Enqueue every instance: W[i], X[i], out[i] are arrays of n[i] device
// pointers; spectra[i], discarded[i], status[i], overlap[i] (2 doubles:
// mantissa, exponent of <X|round(W X)>) are device buffers sized as for
// sgt_mpo_mps_round / sgt_overlap_sweep.  ws: at least the plan's bytes.
SGT_API int sgt_batched_launch(sgt_batched_plan_s* plan, const double* const* const* W,
                               const double* const* const* X, double* const* const* out,
                               double* const* spectra, double* const* discarded, int* const* status,
                               double* const* overlap, void* ws, size_t ws_bytes, void* stream) {
  using namespace sgt;
  SGT_REQUIRE(plan && W && X && out && overlap && ws, SGT_ERR_INVALID, "batched_launch: null argument");
  SGT_REQUIRE(ws_bytes >= plan->total, SGT_ERR_WORKSPACE, "batched_launch: workspace %zu < %zu bytes", ws_bytes,
              plan->total);
  SGT_TRY(create_streams(plan));
  cudaStream_t caller = as_stream(stream);
  SGT_CUDA(cudaEventRecord(plan->fork, caller));
  // A failure part-way still joins every lane forked so far back into the
  // caller's stream (an unjoined lane would invalidate a stream capture and
  // hide the real error); the first error code is returned, with its message.
  int first = SGT_OK;
  std::string msg;
  for (size_t l = 0; l < plan->lanes.size(); ++l) {
    cudaStream_t s = plan->streams[l];
    if (cudaStreamWaitEvent(s, plan->fork, 0) != cudaSuccess) {
      if (first == SGT_OK) first = SGT_ERR_CUDA, msg = "batched_launch: cudaStreamWaitEvent failed";
      break;
    }
    char* base = static_cast<char*>(ws) + plan->lane_off[l];
    for (int i : plan->lanes[l]) {
      if (first != SGT_OK) break;
      const auto& in = plan->inst[i];
      int rc = sgt_mpo_mps_round(in.n, W[i], in.wshape.data(), X[i], in.xshape.data(), in.chi, plan->precision,
                                 out[i], spectra ? spectra[i] : nullptr, discarded ? discarded[i] : nullptr,
                                 status ? status[i] : nullptr, base, plan->lane_bytes[l], s);
      if (rc == SGT_OK)
        rc = sgt_overlap_sweep(in.n, X[i], in.xshape.data(), out[i], in.oshape.data(), overlap[i], base,
                               plan->lane_bytes[l], s);
      if (rc != SGT_OK) first = rc, msg = get_error();
    }
    const bool joined = cudaEventRecord(plan->done[l], s) == cudaSuccess &&
                        cudaStreamWaitEvent(caller, plan->done[l], 0) == cudaSuccess;
    if (!joined && first == SGT_OK) first = SGT_ERR_CUDA, msg = "batched_launch: joining a lane failed";
    if (first != SGT_OK) break;
  }
  if (first != SGT_OK) set_error("%s", msg.c_str());
  return first;
}

SGT_API void sgt_batched_plan_destroy(sgt_batched_plan_s* plan) {
  if (!plan) return;
  for (auto s : plan->streams) cudaStreamDestroy(s);
  for (auto e : plan->done) cudaEventDestroy(e);
  if (plan->fork) cudaEventDestroy(plan->fork);
  delete plan;
}

}  // extern "C"
