// Multi-dot filter in one CUDA graph (no counterpart in the reference, whose
// parallel dimension is independent random starts run by MPI ranks,
// filter_mpi/filter.c:100-104, mod_filter.c:155-159; here independent dots
// of uneven size share one GPU).
//
// Each dot has its own context (grid, potential, projector table, stream,
// ring, autotuner decisions).  fbse_batch_create validates every dot, uploads
// its Newton coefficients, runs each dot's filter once the ordinary way
// (buffers sized, launch shapes autotuned) and then captures the filters of
// all dots into one graph: a root stream forks to every dot's stream (an
// event each), every dot enqueues its whole kernel sequence -- pack, the
// nCheby - 1 H psi of p_hnorm, the K-blocked accumulations -- and joins back.
// The dots are independent branches of the graph, so small dots run beside
// large ones, and one cudaGraphLaunch replaces every per-kernel launch of
// every dot.  Replays are bit-identical to the sequential path (the same
// kernels with the same arguments).
#include <vector>

#include "fbse_internal.cuh"

namespace fbse {
int newton_filter(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin, double de,
                  const double *psi0, long nstart, double *filtered);
int newton_filter_prepare(fbse_ctx *c, const double *an, long ncheby, long m, long nstart, double de,
                          double *a_dev, long *K);
int newton_filter_enqueue(fbse_ctx *c, const double *zn, long ncheby, long m, double vmin, double de,
                          const double *psi0, long nstart, double *filtered, const double *a_dev, long K);
}  // namespace fbse

struct fbse_batch {
  std::vector<fbse_batch_dot> dots;
  std::vector<std::vector<double>> zn, an;  // host copies (the graph's kernels take zn values as arguments)
  std::vector<double *> a_dev;
  std::vector<long> K;
  cudaStream_t root = nullptr;
  std::vector<cudaEvent_t> ev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long nodes = 0;
  std::string err;
};

using namespace fbse;

static int berr(fbse_batch *b, int code, const std::string &m)
{
  b->err = m;
  return code;
}

static void batch_free(fbse_batch *b)
{
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
  for (double *p : b->a_dev)
    if (p) cudaFree(p);
  if (b->root) cudaStreamDestroy(b->root);
  delete b;
}

extern "C" {

int fbse_batch_create(fbse_batch **out, const fbse_batch_dot *dots, int ndots)
{
  if (!out || !dots || ndots < 1) return FBSE_ERR_ARG;
  *out = nullptr;
  fbse_batch *b = new fbse_batch();
  b->dots.assign(dots, dots + ndots);
  int rc = FBSE_OK;
  for (int i = 0; i < ndots && !rc; i++) {
    const fbse_batch_dot &d = dots[i];
    if (!d.ctx || !d.zn || !d.an || !d.psi0 || !d.filtered) {
      rc = berr(b, FBSE_ERR_ARG, "dot " + std::to_string(i) + ": null pointer");
      break;
    }
    for (int j = 0; j < i; j++)
      if (dots[j].ctx == d.ctx) rc = berr(b, FBSE_ERR_ARG, "each dot needs its own context");
    if (rc) break;
    b->zn.emplace_back(d.zn, d.zn + d.ncheby);
    b->an.emplace_back(d.an, d.an + 2 * d.m * d.ncheby);
    double *a = nullptr;
    if (cudaMalloc(&a, (size_t)d.m * d.ncheby * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      rc = berr(b, FBSE_ERR_OOM, "dot " + std::to_string(i) + ": coefficients");
      break;
    }
    b->a_dev.push_back(a);
    long K = 0;
    if ((rc = newton_filter_prepare(d.ctx, d.an, d.ncheby, d.m, d.nstart, d.de, a, &K))) {
      b->err = "dot " + std::to_string(i) + ": " + d.ctx->err;
      break;
    }
    b->K.push_back(K);
    // one ordinary run: every buffer sized, every launch shape decided
    if ((rc = newton_filter(d.ctx, d.zn, d.an, d.ncheby, d.m, d.vmin, d.de, d.psi0, d.nstart, d.filtered))) {
      b->err = "dot " + std::to_string(i) + ": " + d.ctx->err;
      break;
    }
    long K2 = 0;  // the ring must not have changed size
    if ((rc = newton_filter_prepare(d.ctx, d.an, d.ncheby, d.m, d.nstart, d.de, a, &K2)) || K2 != K) {
      if (!rc) rc = berr(b, FBSE_ERR_STATE, "dot " + std::to_string(i) + ": ring size changed");
      break;
    }
  }
  if (!rc && cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking) != cudaSuccess)
    rc = berr(b, FBSE_ERR_CUDA, "root stream");
  if (!rc) {
    b->ev.resize(ndots + 1, nullptr);
    for (auto &e : b->ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = berr(b, FBSE_ERR_CUDA, "events");
  }
  if (!rc) {
    cudaDeviceSynchronize();
    // capture: fork from the root stream, every dot's kernels on its own
    // stream, join back
    if (cudaStreamBeginCapture(b->root, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      rc = berr(b, FBSE_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(cudaGetLastError()));
    } else {
      int crc = FBSE_OK;
      if (cudaEventRecord(b->ev[ndots], b->root) != cudaSuccess) crc = FBSE_ERR_CUDA;
      for (int i = 0; i < ndots && !crc; i++) {
        const fbse_batch_dot &d = b->dots[i];
        if (cudaStreamWaitEvent(d.ctx->stream, b->ev[ndots], 0) != cudaSuccess) { crc = FBSE_ERR_CUDA; break; }
        if ((crc = newton_filter_enqueue(d.ctx, b->zn[i].data(), d.ncheby, d.m, d.vmin, d.de, d.psi0, d.nstart,
                                         d.filtered, b->a_dev[i], b->K[i]))) {
          b->err = "dot " + std::to_string(i) + " capture: " + d.ctx->err;
          break;
        }
        if (cudaEventRecord(b->ev[i], d.ctx->stream) != cudaSuccess ||
            cudaStreamWaitEvent(b->root, b->ev[i], 0) != cudaSuccess)
          crc = FBSE_ERR_CUDA;
      }
      const cudaError_t e = cudaStreamEndCapture(b->root, &b->graph);
      if (crc || e != cudaSuccess) {
        cudaGetLastError();
        rc = crc ? crc : berr(b, FBSE_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
        if (b->err.empty()) b->err = "capture failed";
      }
    }
  }
  if (!rc) {
    size_t nn = 0;
    cudaGraphGetNodes(b->graph, nullptr, &nn);
    b->nodes = (long)nn;
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
      rc = berr(b, FBSE_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(cudaGetLastError()));
  }
  *out = b;  // returned even on failure so that fbse_batch_last_error can explain
  return rc;
}

int fbse_batch_run(fbse_batch *b)
{
  if (!b || !b->exec) return b ? berr(b, FBSE_ERR_STATE, "no graph") : FBSE_ERR_ARG;
  if (cudaGraphLaunch(b->exec, b->root) != cudaSuccess || cudaStreamSynchronize(b->root) != cudaSuccess)
    return berr(b, FBSE_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(cudaGetLastError()));
  g_launches += b->nodes;
  for (const fbse_batch_dot &d : b->dots) {
    const int rc = check_dev_status(d.ctx);
    if (rc) return berr(b, rc, d.ctx->err);
  }
  return FBSE_OK;
}

int fbse_batch_run_sequential(fbse_batch *b)
{
  if (!b) return FBSE_ERR_ARG;
  for (size_t i = 0; i < b->dots.size(); i++) {
    const fbse_batch_dot &d = b->dots[i];
    const int rc = newton_filter(d.ctx, b->zn[i].data(), b->an[i].data(), d.ncheby, d.m, d.vmin, d.de, d.psi0,
                                 d.nstart, d.filtered);
    if (rc) return berr(b, rc, "dot " + std::to_string(i) + ": " + d.ctx->err);
  }
  return FBSE_OK;
}

long fbse_batch_graph_nodes(const fbse_batch *b) { return b ? b->nodes : -1; }

const char *fbse_batch_last_error(const fbse_batch *b) { return b ? b->err.c_str() : "null batch"; }

void fbse_batch_destroy(fbse_batch *b)
{
  if (!b) return;
  if (b->root) cudaStreamSynchronize(b->root);
  batch_free(b);
}

}  // extern "C"
