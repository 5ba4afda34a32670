// Krylov solver drivers (host control flow, device vectors).
#pragma once

#include <vector>

#include "qcmg_internal.h"

namespace qcmg {

struct LanczosResult {
  std::vector<double> alpha, beta;
  double energy = 0.0;
  int niter = 0;
  // reorthogonalized solves: device time of the products and of the
  // Gram-Schmidt sweeps, their algorithmic bytes (16 per stored element per
  // pass), restarts and the vectors held
  double product_ms = 0.0, reorth_ms = 0.0, reorth_bytes = 0.0;
  int restarts = 0, vectors = 0;
};

struct BandResult {
  int M = 0;
  std::vector<double> evals;  // M
  std::vector<double> Q;      // p x M, row-major
};

int multidot_blocks(size_t n);
void multidot_launch(int m, const double* const* V, const double* w, size_t n, double* part,
                     double* out, cudaStream_t s);

void seeded_vector(size_t dim, unsigned seed, double* out);

LanczosResult lanczos_ground_state(qcmg_hamiltonian* H, const double* x0_host, unsigned seed,
                                   double tol, int max_iter, int reorth, double* psi_host);

struct GreenResult {
  std::vector<double> a;  // n
  std::vector<double> b;  // n + 1, b[0] = 1
};

// The continued-fraction Lanczos of one normalized start vector (host or
// device memory).
GreenResult lanczos_green(qcmg_hamiltonian* H, const double* psi0, bool on_device, double accur,
                          int max_iter);

struct BlockResult {
  int M = 0;              // block steps
  int pa = 0;             // block size after the start block's deflation
  std::vector<double> A;  // M blocks pa x pa, row-major
  std::vector<double> B;  // M blocks pa x pa (the last one is the truncation residual)
  std::vector<double> W;  // pa x p, row-major: phi = q W
};

BlockResult block_lanczos(qcmg_hamiltonian* H, int p, const double* phi_in, bool on_device,
                          int M0, int max_iter, double acc_defl, double acc_band);

// phi_in: p start vectors of length dim, vector k at phi_in + k*dim, in
// host memory or (phi_on_device) in the handle's device memory.
BandResult band_lanczos(qcmg_hamiltonian* H, int p, const double* phi_in, bool phi_on_device,
                        int M0, int max_iter, double acc_defl, double acc_band);

void launch_apply_c(int L, int orb, int spin, int pm, int nup, int ndn, const double* x, double* y,
                    double z, bool accumulate, cudaStream_t s);

void green_function_batch(int L, int M, const double* e, const double* v, int nz, const double* z,
                          double* G, cudaStream_t s);

}  // namespace qcmg
