// Lattice integrals over the cluster Green function (host declarations).
#pragma once

#include "qcmg_internal.h"

namespace qcmg {

// One spin block of a lattice model instance: inter-cluster hopping in
// Fourier form, the k-independent difference Hdiff = H - Hc, the positions of
// the Green-function orbitals, and the cluster Green function (Q-matrix and
// bath hybridization) set separately.
struct Lattice {
  int device = 0;
  int L = 0, nR = 0, nel = 0;
  DevBuf<double> R;      // nR x 3, reduced superlattice coordinates
  DevBuf<double> gpos;   // L x 3, reduced coordinates
  DevBuf<double> hdiff;  // L x L complex, row-major
  DevBuf<int> el_r, el_c, el_n;  // grouped by translation n (stable order within a group)
  DevBuf<double> el_v;   // nel complex
  DevBuf<int> el_start;  // nR + 1: the elements of translation n are [el_start[n], el_start[n+1])
  std::vector<double> R_host;
  // phase tables of a K grid, e^{2 pi i K_x R_n,x} per grid index and n (and
  // likewise for y, z), cached for the last grid asked for
  DevBuf<double> tab;
  int tab_gx = 0, tab_gy = 0, tab_gz = 0;
  double tab_off = -1.0;
  const double* phase_tables(int gx, int gy, int gz, double off, cudaStream_t s);
  int M = -1;
  DevBuf<double> e;      // M poles
  DevBuf<double> v;      // L x M complex, column-major
  int nb = 0;
  DevBuf<double> tcb;    // L x nb complex, column-major
  DevBuf<double> eb;     // nb
  DevBuf<double> base, logdetG;
  int prepared_nw = 0;
  cudaStream_t stream = nullptr;

  void prepare(int nw, const double* z, cudaStream_t s);
  double sef_grid(int nw, const double* w, const double* wt, int nkx, int nky, int nkz,
                  cudaStream_t s);
  void cpt(int nz, const double* z, int nk, const double* K, double* g, cudaStream_t s);
  void projected(int nw, const double* w, int kside, int dimk, double* pgf, cudaStream_t s);
  // mean over the K grid ((i + off)/gx, ...) of the CPT Green function
  // (G(z)^-1 - V(K))^-1, for nz complex frequencies z (re, im pairs);
  // out: nz x L x L complex, row-major
  void kmean(int nz, const double* z, int gx, int gy, int gz, double off, double* out,
             cudaStream_t s);
  // the same mean with the phases of nmom (<= 16) translations R (nmom x 3,
  // the basis of the lattice's own R):
  //   out[w][m] = mean_K exp(2 pi i K.R_m) (G(z_w)^-1 - V(K))^-1
  // nmom = 0: the plain mean (one L x L block per frequency)
  void kmoments(int nz, const double* z, int gx, int gy, int gz, double off, int nmom,
                const double* R, double* out, cudaStream_t s);
};

// Cluster self-energy Sigma(z) = z - t_c - Gamma(z) - G(z)^-1 for nz complex
// frequencies, with G(z) from the Q-matrix (L x M, column-major a + L i) and
// Gamma(z) from the cluster-bath block tcb (column-major r + L i) and the
// bath energies eb; t_c row-major; all arrays on the device; sigma (and
// gamma when not null) nz x L x L row-major.
void self_energy_batch(int L, int M, const double* e, const double* v, int nb, const double* tcb,
                       const double* eb, const double* tc, int nz, const double* z, double* sigma,
                       double* gamma, cudaStream_t s);

}  // namespace qcmg

struct qcmg_lattice {
  qcmg::Lattice lat;
  std::mutex mu;
};
