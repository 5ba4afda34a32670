// The lattice integrals of pyqcm's QCM layer on the GB300 engine: the 'G'
// branches a maintainer adds to src_qcm (the ED side is
// qcmg_pyqcm_adapter.hpp).  Header-only; include it after the reference's
// own headers, in a translation unit linked against libqcmg:
//
//   #include "lattice_model_instance.hpp"
//   #include "qcm_ED.hpp"
//   #include "qcmg_pyqcm_lattice_adapter.hpp"
//
// Each function returns false when the instance is outside what the engine
// covers (several clusters per unit cell, Nambu or spin-flip mixing, more
// than one band, an external lattice hybridization); the caller then runs
// its own code.  Engine errors reach the caller as the reference's
// qcm_error (qcm_throw).
//
// Per spin block the engine takes, once per instance, what
// lattice_model_instance::set_V (src_qcm/CPT.cpp:22-64) assembles per
// (k, w): the translations `neighbor` (superlattice basis), the
// inter-cluster elements IGF_elem of every term times its parameter value,
// the k-independent part H - Hc, and the orbital positions
// Green_to_position; then the cluster's Lehmann form (ED::qmatrix) and its
// bath (ED::hybridization).
#ifndef QCMG_PYQCM_LATTICE_ADAPTER_HPP
#define QCMG_PYQCM_LATTICE_ADAPTER_HPP

#include <complex>
#include <string>
#include <vector>

#include "qcmg.h"

// the discrete frequency grid of the QCM layer (src_qcm/QCM.cpp:40-41)
extern vector<double> grid_freqs;
extern vector<double> grid_weights;

namespace qcmg_lattice_adapter {

inline void check(int code) {
  if (code != 0) {
    char buf[512];
    qcmg_last_error(buf, sizeof buf);
    qcm_throw(std::string("GB300 lattice engine: ") + buf);
  }
}

// One spin block's engine handle, released on scope exit.
struct Block {
  qcmg_lattice* lat = nullptr;
  Block() = default;
  Block(const Block&) = delete;
  Block& operator=(const Block&) = delete;
  ~Block() {
    if (lat) qcmg_lattice_destroy(lat);
  }
};

// The instances the engine covers: one cluster per unit cell, one band,
// spin-diagonal mixing (normal or up_down), no external hybridization.
inline bool supported(const lattice_model_instance& I) {
  const lattice_model& M = *I.model;
  return M.clusters.size() == 1 && M.n_mixed == 1 && M.n_band == 1 && M.hybrid == nullptr &&
         (M.mixing == HS_mixing::normal || M.mixing == HS_mixing::up_down);
}

// ED label of the instance's (single) cluster, as
// lattice_model_instance::Potthoff_functional forms it
// (src_qcm/lattice_model_instance.cpp:509-516).
inline size_t cluster_label(const lattice_model_instance& I) {
  const lattice_model& M = *I.model;
  return (size_t)(M.nsys * I.label + M.clusters[0].sys_start);
}

// Builds the engine handle of one spin block of a solved instance.
inline void make_block(lattice_model_instance& I, bool spin_down, Block& b) {
  const lattice_model& M = *I.model;
  const int L = (int)M.dim_GF;
  std::vector<double> R(3 * M.neighbor.size());
  for (size_t n = 0; n < M.neighbor.size(); ++n) {
    R[3 * n] = (double)M.neighbor[n].x;
    R[3 * n + 1] = (double)M.neighbor[n].y;
    R[3 * n + 2] = (double)M.neighbor[n].z;
  }
  // the k-dependent elements, with their parameter values (set_V)
  std::vector<int32_t> er, ec, en;
  std::vector<double> ev;
  for (auto& op : M.term) {
    auto it = I.params.find(op.second->name);
    if (it == I.params.end()) continue;
    const double pv = it->second;
    for (auto& e : spin_down ? op.second->IGF_elem_down : op.second->IGF_elem) {
      er.push_back((int32_t)e.r);
      ec.push_back((int32_t)e.c);
      en.push_back((int32_t)e.n);
      const Complex v = e.v * pv;
      ev.push_back(v.real());
      ev.push_back(v.imag());
    }
  }
  // H - Hc (k-independent), row-major interleaved
  matrix<Complex> D(spin_down ? I.H_down : I.H);
  if (spin_down)
    I.Hc_down.add(D, -1.0);
  else
    I.Hc.add(D, -1.0);
  std::vector<double> hd(2 * (size_t)L * L);
  for (int r = 0; r < L; ++r)
    for (int c = 0; c < L; ++c) {
      hd[2 * ((size_t)r * L + c)] = D(r, c).real();
      hd[2 * ((size_t)r * L + c) + 1] = D(r, c).imag();
    }
  std::vector<double> gpos(3 * (size_t)L);
  for (int i = 0; i < L; ++i) {
    gpos[3 * i] = M.Green_to_position[i].x;
    gpos[3 * i + 1] = M.Green_to_position[i].y;
    gpos[3 * i + 2] = M.Green_to_position[i].z;
  }
  check(qcmg_lattice_create(L, (int)M.neighbor.size(), R.data(), (int)er.size(), er.data(),
                            ec.data(), en.data(), ev.data(), hd.data(), gpos.data(), &b.lat));
  // the cluster's Lehmann form (poles x orbitals) and its diagonal bath
  const size_t label = cluster_label(I);
  auto q = ED::qmatrix(spin_down, label);
  std::vector<double> eb;
  std::vector<Complex> tcb;
  if (M.bath_exists) {
    auto h = ED::hybridization(spin_down, label);
    eb = h.first;
    tcb = h.second;
  }
  check(qcmg_lattice_set_green(
      b.lat, (int)q.first.size(), q.first.data(), reinterpret_cast<const double*>(q.second.data()),
      (int)eb.size(), eb.empty() ? nullptr : reinterpret_cast<const double*>(tcb.data()),
      eb.empty() ? nullptr : eb.data()));
}

inline std::vector<bool> spin_blocks(const lattice_model_instance& I) {
  if (I.model->mixing == HS_mixing::up_down) return {false, true};
  return {false};
}

// The frequency loop of the grid path of
// lattice_model_instance::Potthoff_functional
// (src_qcm/lattice_model_instance.cpp:520-546): Iv = sum over the grid
// frequencies and wavevectors of log|det(VG - 1)|, both spins.
inline bool potthoff_grid(lattice_model_instance& I, double& Iv) {
  if (!supported(I) || grid_freqs.empty()) return false;
  if (!I.gf_solved) I.Green_function_solve();
  int nkx, nky, nkz;
  QCM::get_wavevector_grid(nkx, nky, nkz);
  const int d = I.model->spatial_dimension;
  double total = 0.0;
  for (bool sd : spin_blocks(I)) {
    Block b;
    make_block(I, sd, b);
    double v = 0.0;
    check(qcmg_sef_grid(b.lat, (int)grid_freqs.size(), grid_freqs.data(), grid_weights.data(), nkx,
                        d >= 2 ? nky : 1, d >= 3 ? nkz : 1, &v));
    total += v;
  }
  if (I.model->mixing == HS_mixing::normal) total *= 2.0;
  Iv = total;
  return true;
}

// QCM::periodized_Green_function (src_qcm/QCM.cpp:526-542): g(k, w) for
// every wavevector k (physical basis), one call for all of them.
inline bool periodized_Green_function(lattice_model_instance& I, Complex w,
                                      const vector<vector3D<double>>& k, bool spin_down,
                                      vector<Complex>& g) {
  if (!supported(I)) return false;
  if (!I.gf_solved) I.Green_function_solve();
  lattice_model& M = *I.model;  // basis3D::to is not const
  std::vector<double> K(3 * k.size());
  for (size_t i = 0; i < k.size(); ++i) {
    vector3D<double> r = M.superdual.to(M.physdual.from(k[i]));
    K[3 * i] = r.x;
    K[3 * i + 1] = r.y;
    K[3 * i + 2] = r.z;
  }
  Block b;
  make_block(I, spin_down && M.mixing == HS_mixing::up_down, b);
  const double z[2] = {w.real(), w.imag()};
  g.assign(k.size(), Complex(0.0));
  check(qcmg_cpt_periodized(b.lat, 1, z, (int)k.size(), K.data(),
                            reinterpret_cast<double*>(g.data())));
  return true;
}

// lattice_model_instance::projected_Green_function at the CDMFT frequencies
// i w (src_qcm/CPT.cpp:283-345): one call for all of them, on the
// kside^dim midpoint grid the CDMFT host function uses.
inline bool projected_Green_function(lattice_model_instance& I, const vector<double>& w,
                                     int kside, bool spin_down, vector<matrix<Complex>>& P) {
  if (!supported(I)) return false;
  if (!I.gf_solved) I.Green_function_solve();
  const lattice_model& M = *I.model;
  const int L = (int)M.dim_GF;
  Block b;
  make_block(I, spin_down && M.mixing == HS_mixing::up_down, b);
  std::vector<double> out(2 * w.size() * (size_t)L * L);
  check(qcmg_cdmft_projected(b.lat, (int)w.size(), w.data(), kside, M.spatial_dimension,
                             out.data()));
  P.assign(w.size(), matrix<Complex>(L));
  for (size_t i = 0; i < w.size(); ++i)
    for (int r = 0; r < L; ++r)
      for (int c = 0; c < L; ++c) {
        const size_t o = 2 * ((i * L + r) * (size_t)L + c);
        P[i](r, c) = Complex(out[o], out[o + 1]);
      }
  return true;
}

// lattice_model_instance::dos with use_grid (src_qcm/average.cpp:294-347):
// -(1/pi) Im Tr of the wavevector-grid mean of Gcpt(k, w) / L, per spin
// block (the up value repeated for normal mixing).
inline bool dos_grid(lattice_model_instance& I, Complex w, vector<double>& d) {
  if (!supported(I)) return false;
  if (!I.gf_solved) I.Green_function_solve();
  const lattice_model& M = *I.model;
  const int L = (int)M.dim_GF;
  int nkx, nky, nkz;
  QCM::get_wavevector_grid(nkx, nky, nkz);
  const int dim = M.spatial_dimension;
  const double z[2] = {w.real(), w.imag()};
  d.clear();
  for (bool sd : spin_blocks(I)) {
    Block b;
    make_block(I, sd, b);
    std::vector<double> out(2 * (size_t)L * L);
    check(qcmg_lattice_kmean(b.lat, 1, z, nkx, dim >= 2 ? nky : 1, dim >= 3 ? nkz : 1, 0.0,
                             out.data()));
    double tr = 0.0;
    for (int a = 0; a < L; ++a) tr += out[2 * ((size_t)a * L + a) + 1];
    d.push_back(-tr / M_PI / L);  // per orbital of the one band
  }
  if (d.size() == 1) d.push_back(d[0]);
  return true;
}

}  // namespace qcmg_lattice_adapter

#endif
