// host_pipeline.cu -- segmented sum, max and argmax of a float64
// ListOffsetArray held in (pinned) HOST memory, with the transfers overlapped.
//
// The lists are cut into chunks at list boundaries (the host offsets say
// where, so nothing waits on the device).  For chunk c, a copy-in stream
// moves its offsets and content into the device workspace at their global
// positions, the caller's stream reduces it (offsets may start anywhere and
// content is indexed globally, so the chunk needs no rebasing), and a
// copy-out stream returns its three results.  Copies of chunk c+1, the
// reduction of chunk c and the copies back of chunk c-1 run at the same time.
// The call returns after enqueueing; the caller's stream is made to wait for
// the last copy back, so synchronising that stream waits for everything.
#include <mutex>
#include <vector>

#include "reduce_ops.cuh"

using namespace gb;

namespace {

constexpr int kMaxChunks = 64;
constexpr int kMaxDev = 64;

struct PipeStreams {
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t ready[kMaxChunks], done[kMaxChunks], start, finish;
  bool init = false;
};
std::mutex g_pipe_mutex;
PipeStreams g_pipe[kMaxDev];

cudaError_t pipe_streams(PipeStreams** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pipe_mutex);
  PipeStreams& p = g_pipe[dev];
  if (!p.init) {
    e = cudaStreamCreateWithFlags(&p.in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.out, cudaStreamNonBlocking);
    for (int i = 0; i < kMaxChunks && e == cudaSuccess; i++) {
      e = cudaEventCreateWithFlags(&p.ready[i], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.done[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.finish, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    p.init = true;
  }
  *out = &p;
  return cudaSuccess;
}

}  // namespace

// Host buffers: h_x (content, indexed globally), h_offsets [nlists + 1] and the
// three outputs [nlists]; pinned memory lets the copies overlap.  Device
// workspace: d_x (at least h_offsets[nlists] elements; element j is stored at
// d_x[j]), d_offsets [nlists + 1] and the three device outputs [nlists].
// chunks: 1..64 (clamped).  Same results as awkward_reduce_sum_float64_float64_64,
// awkward_reduce_max_float64_float64_64 (identity -inf) and
// awkward_reduce_argmax_float64_64 on the whole array.
GB_EXPORT int awkward_gb300_reduce_sum_max_argmax_host_float64(
    double* h_sum, double* h_max, int64_t* h_argmax, const double* h_x, const int64_t* h_offsets,
    int64_t nlists, double* d_x, int64_t* d_offsets, double* d_sum, double* d_max,
    int64_t* d_argmax, int64_t chunks, void* stream) {
  if (nlists <= 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  PipeStreams* p = nullptr;
  cudaError_t e = pipe_streams(&p);
  if (e != cudaSuccess) return (int)e;
  // the per-device copy streams and events are shared: one caller enqueues at a time
  static std::mutex enqueue_mutex;
  std::lock_guard<std::mutex> lock(enqueue_mutex);
  int C = (int)(chunks < 1 ? 1 : (chunks > kMaxChunks ? kMaxChunks : chunks));
  if (C > nlists) C = (int)nlists;
  // the copy streams start after work already queued on the caller's stream
  e = cudaEventRecord(p->start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(p->in, p->start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(p->out, p->start, 0);
  FixedSumOp<double> sum_op{};
  ExtremumOp<double, true> max_op{};
  max_op.ident = -INFINITY;
  ArgExtremumOp<double, true> arg_op{};
  // chunk boundaries balanced by elements + lists
  const long long e0 = h_offsets[0], eN = h_offsets[nlists];
  const long long D = nlists + (eN - e0);
  std::vector<long long> cut(C + 1, 0);
  cut[C] = nlists;
  for (int c = 1; c < C; c++) {
    const long long target = D * c / C;
    long long lo = cut[c - 1], hi = nlists;  // first l with l + (offsets[l] - e0) >= target
    while (lo < hi) {
      const long long mid = (lo + hi) / 2;
      if (mid + (h_offsets[mid] - e0) < target) lo = mid + 1;
      else hi = mid;
    }
    cut[c] = lo;
  }
  for (int c = 0; c < C && e == cudaSuccess; c++) {
    const long long l0 = cut[c], l1 = cut[c + 1];
    if (l1 <= l0) continue;
    const long long a = h_offsets[l0], b = h_offsets[l1];
    e = cudaMemcpyAsync(d_offsets + l0, h_offsets + l0, sizeof(int64_t) * (size_t)(l1 - l0 + 1),
                        cudaMemcpyHostToDevice, p->in);
    if (e == cudaSuccess && b > a)
      e = cudaMemcpyAsync(d_x + a, h_x + a, sizeof(double) * (size_t)(b - a),
                          cudaMemcpyHostToDevice, p->in);
    if (e == cudaSuccess) e = cudaEventRecord(p->ready[c], p->in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, p->ready[c], 0);
    const long long n = l1 - l0;
    if (e == cudaSuccess)
      e = launch_seg_reduce(sum_op, d_x, d_offsets + l0, n, d_sum + l0, 0, nullptr, s);
    if (e == cudaSuccess)
      e = launch_seg_reduce(max_op, d_x, d_offsets + l0, n, d_max + l0, 0, nullptr, s);
    if (e == cudaSuccess)
      e = launch_seg_reduce(arg_op, d_x, d_offsets + l0, n, d_argmax + l0, 0, nullptr, s);
    if (e == cudaSuccess) e = cudaEventRecord(p->done[c], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->out, p->done[c], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_sum + l0, d_sum + l0, sizeof(double) * (size_t)n,
                          cudaMemcpyDeviceToHost, p->out);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_max + l0, d_max + l0, sizeof(double) * (size_t)n,
                          cudaMemcpyDeviceToHost, p->out);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_argmax + l0, d_argmax + l0, sizeof(int64_t) * (size_t)n,
                          cudaMemcpyDeviceToHost, p->out);
  }
  if (e == cudaSuccess) e = cudaEventRecord(p->finish, p->out);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, p->finish, 0);
  return (int)e;
}
