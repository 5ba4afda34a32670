// Lanczos ground states of many sectors at once, each sector's steps
// replayed from a captured CUDA graph.
//
// The recurrence is LanczosEigenvalue's (pyqcm src_ed/Hamiltonian/
// Lanczos.hpp:41-95), with alpha/beta and the step index kept on the device
// (lanczos_step_nodes), so a chunk of K steps needs no host round trip: each
// sector's K steps are built once as a CUDA graph (a chain of kernel nodes)
// and relaunched chunk after chunk on a stream of the sector's own.  The host launches the graphs of the
// sectors still running (they run concurrently, one stream each), waits once
// per chunk, reads the new coefficients and applies the reference's test
// (Ritz residual |z_last beta_j| below tol) step by step, so each sector
// stops at the same step and with the same energy as the host-driven
// recurrence (the same kernels, grids and summation order: bitwise equal on
// the FP64 product).  Sectors of different sizes run side by side; a finished
// sector's graph is simply no longer launched.  The ground-state vectors are
// then replayed (LanczosEigenvector, Lanczos.hpp:109-143) on the same
// streams, all sectors at once.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "qcmg.h"
#include "qcmg_blas.h"
#include "qcmg_internal.h"
#include "qcmg_krylov.h"
#include "qcmg_tridiag.h"

namespace qcmg {

namespace {

struct BatchSector {
  qcmg_hamiltonian* H = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t saved_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DevBuf<double> r, q, coef, part;  // coef: alpha (cap) then beta (cap)
  DevBuf<int> flags;                // j, done
  std::vector<double> alpha, beta, z;
  int checked = 0;                  // coefficients examined so far
  int niter = 0;
  double e0 = 0.0;
  int status = QCMG_OK;
  bool running = true;
  ~BatchSector() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }
};

}  // namespace

// The seeded start vector of H on the device (generated once per handle
// and seed, as lanczos_ground_state keeps it).
static const double* seeded_start_dev(qcmg_hamiltonian* H, unsigned seed) {
  const size_t n = H->dim;
  if (!(H->seed_ok && H->seed_key == seed && H->seed_vec.n == n)) {
    H->seed_ok = false;
    std::vector<double> hx0(n);
    seeded_vector(n, seed, hx0.data());
    H->seed_vec.upload(hx0.data(), n, H->stream);
    QCMG_CUDA(cudaStreamSynchronize(H->stream));  // hx0 goes out of scope
    H->seed_key = seed;
    H->seed_ok = true;
  }
  return H->seed_vec.p;
}

void lanczos_batch(int nsec, qcmg_hamiltonian* const* Hs, unsigned seed, double tol, int max_iter,
                   int chunk, double* E0, int* niter, double* const* psi, int* status) {
  chunk = std::max(2, chunk + (chunk & 1));  // even: every chunk starts on the same buffers
  const int cap = max_iter + chunk + 1;
  std::vector<std::unique_ptr<BatchSector>> S(nsec);
  for (int i = 0; i < nsec; ++i) {
    S[i].reset(new BatchSector);
    BatchSector& b = *S[i];
    b.H = Hs[i];
    QCMG_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    b.saved_stream = b.H->stream;
  }
  // the handles launch on the batch's streams while it runs
  struct Restore {
    std::vector<std::unique_ptr<BatchSector>>& S;
    ~Restore() {
      for (auto& b : S)
        if (b && b->H) b->H->stream = b->saved_stream;
    }
  } restore{S};
  for (auto& bp : S) {
    BatchSector& b = *bp;
    const size_t n = b.H->dim;
    b.r.alloc(n);
    b.q.alloc(n);
    b.coef.alloc(2 * (size_t)cap);
    b.part.alloc(kRedBlocks);
    b.flags.alloc(2);
    const double* x0 = seeded_start_dev(b.H, seed);
    b.H->stream = b.stream;
    QCMG_CUDA(cudaMemcpyAsync(b.r.p, x0, n * 8, cudaMemcpyDeviceToDevice, b.stream));
    QCMG_CUDA(cudaMemsetAsync(b.q.p, 0, n * 8, b.stream));
    QCMG_CUDA(cudaMemsetAsync(b.coef.p, 0, 2 * (size_t)cap * 8, b.stream));
    QCMG_CUDA(cudaMemsetAsync(b.flags.p, 0, 2 * sizeof(int), b.stream));
    // K steps of this sector as a chain of kernel nodes (built explicitly,
    // not captured: another host thread's device-wide synchronization cannot
    // invalidate it)
    LanczosDevState st{b.coef.p, b.coef.p + cap, b.part.p, b.flags.p, b.flags.p + 1, cap};
    qcmg_hamiltonian* H = b.H;
    GraphChain gc;
    QCMG_CUDA(cudaGraphCreate(&b.graph, 0));
    gc.graph = b.graph;
    auto product = [H, &gc](const double* x, double* y) { matvec_node(H, x, y, true, gc); };
    for (int t = 0; t < chunk; ++t) {
      if (t % 2 == 0)
        lanczos_step_nodes(st, b.r.p, b.q.p, n, gc, product);
      else
        lanczos_step_nodes(st, b.q.p, b.r.p, n, gc, product);
    }
    QCMG_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
  }
  for (auto& bp : S) QCMG_CUDA(cudaStreamSynchronize(bp->stream));
  // pinned landing area per sector: j, done, then the chunk's new alpha and
  // beta (the coefficients from the last examined step on)
  const size_t slot = 1 + 2 * (size_t)chunk;  // doubles: the two ints fit in the first
  double* pinned = nullptr;
  QCMG_CUDA(cudaMallocHost(&pinned, (size_t)nsec * slot * sizeof(double)));
  struct FreePinned {
    double* p;
    ~FreePinned() {
      if (p) cudaFreeHost(p);
    }
  } free_pinned{pinned};
  for (;;) {
    bool any = false;
    for (int i = 0; i < nsec; ++i) {
      BatchSector& b = *S[i];
      if (!b.running) continue;
      any = true;
      QCMG_CUDA(cudaGraphLaunch(b.exec, b.stream));
      double* land = pinned + (size_t)i * slot;
      const int from = b.checked, cnt = std::min(chunk, cap - from);
      QCMG_CUDA(cudaMemcpyAsync(land, b.flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, b.stream));
      QCMG_CUDA(cudaMemcpyAsync(land + 1, b.coef.p + from, cnt * 8, cudaMemcpyDeviceToHost, b.stream));
      QCMG_CUDA(cudaMemcpyAsync(land + 1 + chunk, b.coef.p + cap + from, cnt * 8,
                                cudaMemcpyDeviceToHost, b.stream));
    }
    if (!any) break;
    for (int i = 0; i < nsec; ++i) {
      BatchSector& b = *S[i];
      if (!b.running) continue;
      QCMG_CUDA(cudaStreamSynchronize(b.stream));
      const double* land = pinned + (size_t)i * slot;
      int hj[2];
      std::memcpy(hj, land, 2 * sizeof(int));
      const int j = hj[0], from = b.checked;
      // the reference's stopping test, step by step over the new coefficients
      bool stop = false;
      for (int k = from; k < j && !stop; ++k) {
        b.alpha.push_back(land[1 + (k - from)]);
        b.beta.push_back(land[1 + chunk + (k - from)]);
        b.e0 = tridiag_lowest(b.alpha, b.beta, b.z);
        const double ritz = std::fabs(b.z.back() * b.beta.back());
        if (!std::isfinite(b.e0) || !std::isfinite(ritz)) {
          b.status = QCMG_ERR_NUMERIC;
          stop = true;
        } else if (ritz <= tol) {
          stop = true;
        } else if ((int)b.alpha.size() > max_iter) {
          b.status = QCMG_ERR_NOCONV;
          stop = true;
        }
      }
      b.checked = (int)b.alpha.size();
      if (!stop && hj[1] != 0) {  // capacity reached on the device
        b.status = QCMG_ERR_NOCONV;
        stop = true;
      }
      if (stop) {
        b.running = false;
        b.niter = (int)b.alpha.size();
      }
    }
  }
  // eigenvector replay (LanczosEigenvector), all sectors at once
  std::vector<DevBuf<double>> gs(nsec);
  for (int i = 0; i < nsec; ++i) {
    BatchSector& b = *S[i];
    if (!psi || !psi[i] || b.status != QCMG_OK) continue;
    const size_t n = b.H->dim;
    const double* x0 = b.H->seed_vec.p;
    gs[i].alloc(n);
    QCMG_CUDA(cudaMemcpyAsync(gs[i].p, x0, n * 8, cudaMemcpyDeviceToDevice, b.stream));
    scale(gs[i].p, b.z[0], n, b.stream);
    QCMG_CUDA(cudaMemcpyAsync(b.r.p, x0, n * 8, cudaMemcpyDeviceToDevice, b.stream));
    QCMG_CUDA(cudaMemsetAsync(b.q.p, 0, n * 8, b.stream));
    for (size_t k = 1; k < b.z.size(); ++k) {
      matvec(b.H, b.r.p, b.q.p, true);
      replay_step(b.r.p, b.q.p, gs[i].p, b.alpha[k - 1], b.beta[k - 1], b.z[k], n, b.stream);
    }
    QCMG_CUDA(cudaMemcpyAsync(psi[i], gs[i].p, n * 8, cudaMemcpyDeviceToHost, b.stream));
  }
  for (int i = 0; i < nsec; ++i) {
    BatchSector& b = *S[i];
    QCMG_CUDA(cudaStreamSynchronize(b.stream));
    E0[i] = b.e0;
    if (niter) niter[i] = b.niter;
    if (status) status[i] = b.status;
  }
}

}  // namespace qcmg

using namespace qcmg;

extern "C" int qcmg_lanczos_batch(int n, qcmg_hamiltonian* const* H, unsigned seed, double tol,
                                  int max_iter, int chunk, double* E0, int* niter,
                                  double* const* psi, int* status) {
  try {
    clear_error();
    QCMG_CHECK_ARG(n >= 0, "n must not be negative");
    if (n == 0) return QCMG_OK;
    QCMG_CHECK_ARG(H != nullptr && E0 != nullptr, "NULL argument");
    QCMG_CHECK_ARG(tol > 0.0 && max_iter > 0 && chunk > 0, "tol, max_iter and chunk must be positive");
    std::vector<qcmg_hamiltonian*> hs(H, H + n);
    for (auto* h : hs) {
      QCMG_CHECK_ARG(h != nullptr, "NULL handle");
      QCMG_CHECK_ARG(h->dim > 0, "empty sector");
      QCMG_CHECK_ARG(h->device == hs[0]->device, "all handles must be on one device");
    }
    std::vector<qcmg_hamiltonian*> order(hs);
    std::sort(order.begin(), order.end());
    QCMG_CHECK_ARG(std::adjacent_find(order.begin(), order.end()) == order.end(),
                   "a handle appears twice in the batch");
    // lock every handle, in address order
    std::vector<std::unique_lock<std::mutex>> locks;
    for (auto* h : order) locks.emplace_back(h->mu);
    QCMG_CUDA(cudaSetDevice(hs[0]->device));
    lanczos_batch(n, hs.data(), seed, tol, max_iter, chunk, E0, niter, psi, status);
    return QCMG_OK;
  } catch (const Error& e) {
    set_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return QCMG_ERR_CUDA;
  }
}
