// Reference-side adapter: a pyqcm Hamiltonian format backed by libqcmg.
//
// This header is compiled INSIDE pyqcm (it uses pyqcm's own types:
// Hamiltonian<HF>, model, sector, Q_matrix, state) and is the code a pyqcm
// maintainer adds to select the GPU engine with Hamiltonian_format = 'G'.
// It replaces, for factorizable instances (trivial point group, normal or
// up_down mixing), Hamiltonian_Factorized
// (src_ed/Hamiltonian/Hamiltonian_Factorized.hpp) and the Lanczos /
// band-Lanczos drivers it inherits from Hamiltonian<HF>
// (src_ed/Hamiltonian/Hamiltonian_base.hpp:96-254).
//
// Only real Hilbert spaces are served (every factorized configuration of
// the reference is real); complex instances keep the CPU format.
#pragma once

#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "qcmg.h"

template <typename HilbertField>
class Hamiltonian_GPU : public Hamiltonian<HilbertField> {
 public:
  Hamiltonian_GPU(shared_ptr<model> the_model, const map<string, double>& value, sector sec) {
    this->the_model = the_model;
    this->sec = sec;
    const int L = (int)the_model->n_orb;
    // Sum the terms of the value map into one list of hops per spin and one
    // list of density-density pairs (Hamiltonian_Factorized::HS_ops_map).
    map<pair<int, int>, double> hop, pairs;
    for (auto& v : value) {
      if (v.second == 0.0) continue;
      Hermitian_operator& op = *the_model->term.at(v.first);
      for (auto& e : op.matrix_elements()) {
        const int r = (int)e.r, c = (int)e.c;
        const double x = v.second * e.v.real();
        if (op.is_interaction)
          pairs[{std::min(r, c), std::max(r, c)}] += x;
        else
          hop[{r, c}] += x;
      }
    }
    std::vector<int32_t> ur, uc, dr, dc, pr, pc;
    std::vector<double> uv, dv, pv;
    for (auto& h : hop) {
      const int r = h.first.first, c = h.first.second;
      if (r < L && c < L) {
        ur.push_back(r); uc.push_back(c); uv.push_back(h.second);
      } else if (r >= L && c >= L) {
        dr.push_back(r - L); dc.push_back(c - L); dv.push_back(h.second);
      } else {
        qcm_ED_throw("Hamiltonian_format 'G': spin-flip terms do not factorize");
      }
    }
    for (auto& p : pairs) {
      pr.push_back(p.first.first); pc.push_back(p.first.second); pv.push_back(p.second);
    }
    check(qcmg_hamiltonian_create(L, sec.Nup(), sec.Ndw(), (int)ur.size(), ur.data(), uc.data(),
                                  uv.data(), (int)dr.size(), dr.data(), dc.data(), dv.data(),
                                  (int)pr.size(), pr.data(), pc.data(), pv.data(), &H_));
    size_t dim = 0;
    check(qcmg_hamiltonian_dims(H_, nullptr, nullptr, &dim));
    this->dim = dim;
  }

  ~Hamiltonian_GPU() override { qcmg_hamiltonian_destroy(H_); }

  // y += H x  (Hamiltonian::mult_add)
  void mult_add(vector<HilbertField>& x, vector<HilbertField>& y) override {
    check(qcmg_matvec(H_, (const double*)x.data(), (double*)y.data(), QCMG_ACCUMULATE));
  }

  // Lanczos ground state on the device (Hamiltonian::states, method 'L').
  vector<shared_ptr<state<HilbertField>>> states(double& GS_energy) override {
    auto gs = make_shared<state<HilbertField>>(this->sec, this->dim);
    double e0 = 0.0;
    int niter = 0;
    check(qcmg_lanczos_ground_state(H_, nullptr, (unsigned)global_int("seed"),
                                    global_double("accur_lanczos"),
                                    (int)global_int("max_iter_lanczos"), 0, &e0,
                                    (double*)gs->psi.data(), &niter, nullptr, nullptr, 0));
    gs->energy = e0;
    if (e0 < GS_energy) GS_energy = e0;
    vector<shared_ptr<state<HilbertField>>> out;
    out.push_back(gs);
    return out;
  }

  double GS_energy() override {
    double e0 = 0.0;
    check(qcmg_lanczos_ground_state(H_, nullptr, (unsigned)global_int("seed"),
                                    global_double("accur_lanczos"),
                                    (int)global_int("max_iter_lanczos"), 0, &e0, nullptr,
                                    nullptr, nullptr, nullptr, 0));
    return e0;
  }

  // Band Lanczos on the device (Hamiltonian::build_Q_matrix).
  Q_matrix<HilbertField> build_Q_matrix(vector<vector<HilbertField>>& phi) override {
    const int p = (int)phi.size();
    if (this->dim == 0 || p == 0) return Q_matrix<HilbertField>(0, 0);
    std::vector<const double*> ptrs(p);
    for (int k = 0; k < p; ++k) ptrs[k] = (const double*)phi[k].data();
    const int M = (int)(14 * p * std::log(1.0 * this->dim));
    const int maxit = (int)global_int("max_iter_BL");
    const int cap = maxit + 2 * p + 2;
    std::vector<double> ev(cap), Q((size_t)p * cap);
    int Mo = 0;
    check(qcmg_band_lanczos_ptrs(H_, p, ptrs.data(), M, maxit, global_double("accur_deflation"),
                                 global_double("accur_band_lanczos"), &Mo, ev.data(), Q.data(),
                                 cap));
    Q_matrix<HilbertField> out(p, Mo);
    for (int i = 0; i < Mo; ++i) out.e[i] = ev[i];
    for (int a = 0; a < p; ++a)
      for (int i = 0; i < Mo; ++i) out.v(a, i) = Q[(size_t)a * Mo + i];
    return out;
  }

 private:
  qcmg_hamiltonian* H_ = nullptr;

  static void check(int code) {
    if (code != QCMG_OK) {
      char buf[512];
      qcmg_last_error(buf, sizeof(buf));
      qcm_ED_throw(std::string("GPU Hamiltonian: ") + buf);
    }
  }
};
