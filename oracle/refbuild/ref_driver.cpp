// Oracle driver: runs the reference's own exact-diagonalization and lattice
// code (compiled from its sources, see Makefile) on a small text spec and
// writes every intermediate that the GPU path must reproduce as raw
// little-endian arrays plus a manifest.  Test infrastructure only.
//
// Spec lines (whitespace separated, '#' starts a comment):
//   gchar NAME C | gdouble NAME X | gint NAME N | gbool NAME 0/1
//   model NAME N_SITES N_BATH                 -> ED::new_model (trivial group)
//   el MODEL OP TYPE R C V                    -> element of operator OP (type one-body/interaction)
//   param NAME VALUE                          -> coefficient in the instance value map
//   instance MODEL SECTORS LABEL              -> ED::new_model_instance
//   halfbasis L N                             -> ED_halfbasis bin list
//   hamiltonian MODEL SECTOR TAG              -> Hamiltonian_Factorized: half-operators, x0, H.x0
//   lanczos MODEL SECTOR TAG                  -> LanczosEigenvalue/Eigenvector from x0
//   hcheck MODEL SECTOR TAG                   -> one timed mult_add on x0: sum, norm^2, <x0,Hx0>,
//                                                4096 sampled elements (large sectors)
//   lanczos_e0 MODEL SECTOR TAG               -> LanczosEigenvalue from x0: E0, alpha, beta, time
//   destroy MODEL SECTOR ORB SPIN PM TAG      -> c / c^dagger applied to x0 (factorized branch)
//   gs LABEL TAG                              -> ED::ground_state_solve
//   qmatrix LABEL SPIN TAG                    -> ED::Green_function_solve + ED::qmatrix
//   gz LABEL SPIN RE IM TAG                   -> ED::Green_function(z)
//   hyb LABEL SPIN RE IM TAG                  -> ED::hybridization_function(z)
//   sigma LABEL SPIN RE IM TAG                -> ED::self_energy(z)
//   omega LABEL TAG                           -> ED::Potthoff_functional (cluster part)
// Lattice (QCM) commands, mirroring the pyqcm Python calls:
//   ops MODEL                                 -> creates the cluster-only operators given by el
//   lat_cluster MODEL x y z [x y z ...]       -> QCM::add_cluster + QCM::add_system
//   lat_model NAME a1x a1y a1z [a2x a2y a2z]  -> QCM::new_lattice_model (unit cell = identity)
//   lat_hop NAME lx ly lz AMP TAU SIGMA       -> QCM::hopping_operator
//   lat_inter NAME AMP TYPE                   -> QCM::interaction_operator (on-site)
//   lat_dw NAME TYPE Qx Qy Qz AMP PHASE       -> QCM::density_wave
//   lat_param NAME VALUE | lat_equiv NAME MULT REF
//   lat_sector S                              -> target sector of the system
//   lat_instance LABEL                        -> QCM::set_parameters + new_model_instance
//   lat_kgrid NX NY NZ                        -> QCM::set_wavevector_grid
//   lat_wgrid N w_1..w_N p_1..p_N             -> discrete frequency grid
//   lat_sef LABEL TAG                         -> QCM::Potthoff_functional
//   lat_dos LABEL TAG NZ (re im)x NZ          -> QCM::dos on the wavevector grid
//   lat_ave LABEL TAG OP...                   -> QCM::averages of the named operators
//   lat_gper LABEL TAG NZ (re im)x NZ NK (kx ky kz)x NK -> periodized_Green_function
//   lat_tk LABEL TAG NK (kx ky kz)x NK        -> QCM::tk
//   lat_dump LABEL TAG                        -> neighbours, inter-cluster elements, H, Hc
//   lat_varia NAME...                         -> QCM::CDMFT_variational_set (cluster 0)
//   lat_host LABEL TAG NW w.. wt..            -> QCM::CDMFT_host (+ get_CDMFT_host)
//   lat_dist LABEL TAG NP p..                 -> QCM::CDMFT_distance (cluster 0)
//   lat_resid LABEL NP p.. | lat_grad LABEL NP p.. -> QCM::CDMFT_residuals / CDMFT_gradient
//                                                (cluster 0), printed on standard output
// SPEC "-" reads the commands from standard input and answers each with "@@".
#include <chrono>
#include <complex>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "QCM.hpp"
#include "lattice_model.hpp"
#include "lattice_model_instance.hpp"
#include "global_parameter.hpp"
#include "model_instance.hpp"
#include "qcm_ED.hpp"
#include "Hamiltonian/Hamiltonian_Factorized.hpp"
#include "Operators/one_body_operator.hpp"

using namespace std;
typedef complex<double> cplx;

extern map<string, shared_ptr<model>> models;
extern map<size_t, shared_ptr<model_instance_base>> model_instances;
extern std::normal_distribution<double> normal_dis;
extern shared_ptr<lattice_model> qcm_model;
extern map<int, unique_ptr<lattice_model_instance>> lattice_model_instances;
extern vector<double> grid_freqs;
extern vector<double> grid_weights;

static string outdir = ".";
static ofstream manifest;

template <class T>
static void put(const string& name, const char* dtype, const vector<size_t>& shape,
                const T* data, size_t n) {
  string fn = outdir + "/" + name + ".bin";
  FILE* f = fopen(fn.c_str(), "wb");
  if (!f) throw runtime_error("cannot write " + fn);
  if (n) fwrite(data, sizeof(T), n, f);
  fclose(f);
  manifest << name << ' ' << dtype;
  for (auto s : shape) manifest << ' ' << s;
  manifest << '\n';
  manifest.flush();
}
static void put_d(const string& name, const vector<double>& v) {
  put(name, "f8", {v.size()}, v.data(), v.size());
}
static void put_scalar(const string& name, double x) { put(name, "f8", {}, &x, 1); }
static void put_cmat(const string& name, const matrix<cplx>& m) {
  // row-major (r, c) complex128 for numpy
  vector<cplx> rm(m.r * m.c);
  for (size_t i = 0; i < m.r; i++)
    for (size_t j = 0; j < m.c; j++) rm[i * m.c + j] = m(i, j);
  put(name, "c16", {m.r, m.c}, rm.data(), rm.size());
}

struct Spec {
  map<string, map<string, vector<matrix_element<double>>>> elements;  // model -> op -> elems
  map<string, map<string, string>> optype;
  map<string, double> params;
  set<string> ops_created;
  vector<pair<string, double>> lat_values;
  vector<tuple<string, double, string>> lat_equiv;
  bool lat_params_set = false;
};

static void create_ops(Spec& S, const string& model) {
  for (auto& op : S.elements[model]) {
    string key = model + "/" + op.first;
    if (S.ops_created.count(key)) continue;
    ED::new_operator(model, op.first, S.optype[model][op.first], op.second);
    S.ops_created.insert(key);
  }
}

static map<string, double> values_for(Spec& S, const string& model) {
  map<string, double> v;
  for (auto& p : S.params)
    if (S.elements[model].count(p.first)) v[p.first] = p.second;
  return v;
}

static void dump_halfop(const string& tag, shared_ptr<HS_half_operator<double>> h) {
  vector<uint32_t> IJ;
  vector<double> val;
  for (auto& g : h->v)
    for (auto& e : g.second) {
      IJ.push_back(e.first);
      IJ.push_back(e.second);
      val.push_back(g.first);
    }
  put(tag + "_IJ", "u4", {val.size(), 2}, IJ.data(), IJ.size());
  put_d(tag + "_val", val);
  vector<uint32_t> dr;
  vector<double> dv;
  for (auto& d : h->diag_elem) {
    dr.push_back((uint32_t)d.r);
    dv.push_back(d.v);
  }
  put(tag + "_diag_r", "u4", {dr.size()}, dr.data(), dr.size());
  put_d(tag + "_diag_v", dv);
  uint32_t dim = h->dim;
  put(tag + "_dim", "u4", {}, &dim, 1);
}

static vector<double> seeded_start(size_t dim) {
  vector<double> x(dim);
  random(x, normal_dis);
  return x;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    cerr << "usage: qcm_ref_driver SPEC OUTDIR\n";
    return 2;
  }
  outdir = argv[2];
  manifest.open(outdir + "/manifest.txt");
  qcm_model = make_shared<lattice_model>();
  QCM::global_parameter_init();
  Spec S;
  // SPEC "-": commands from standard input, each answered by a line "@@"
  // once done (results of lat_resid / lat_grad on the line before)
  const bool interactive = string(argv[1]) == "-";
  ifstream fin;
  if (!interactive) fin.open(argv[1]);
  istream& in = interactive ? cin : fin;
  string line;
  try {
    while (getline(in, line)) {
      struct Done {
        bool on;
        ~Done() {
          if (on) cout << "@@" << endl;
        }
      } done{interactive};
      auto hash = line.find('#');
      if (hash != string::npos) line = line.substr(0, hash);
      istringstream ss(line);
      string cmd;
      if (!(ss >> cmd)) continue;
      if (cmd == "gchar") {
        string n; char c; ss >> n >> c; set_global_char(n, c);
      } else if (cmd == "gdouble") {
        string n; double x; ss >> n >> x; set_global_double(n, x);
      } else if (cmd == "gint") {
        string n; size_t x; ss >> n >> x; set_global_int(n, x);
      } else if (cmd == "gbool") {
        string n; int x; ss >> n >> x; set_global_bool(n, x != 0);
      } else if (cmd == "model") {
        string n; size_t ns, nb; ss >> n >> ns >> nb;
        ED::new_model(n, ns, nb, {}, false);
      } else if (cmd == "el") {
        string m, op, type; size_t r, c; double v;
        ss >> m >> op >> type >> r >> c >> v;
        S.elements[m][op].push_back(matrix_element<double>(r, c, v));
        S.optype[m][op] = type;
      } else if (cmd == "param") {
        string n; double v; ss >> n >> v; S.params[n] = v;
      } else if (cmd == "instance") {
        string m, sec; size_t label; ss >> m >> sec >> label;
        create_ops(S, m);
        auto v = values_for(S, m);
        ED::new_model_instance(m, v, sec, label);
      } else if (cmd == "halfbasis") {
        int L, N; ss >> L >> N;
        ED_halfbasis B(L, N);
        put("halfbasis_L" + to_string(L) + "_N" + to_string(N), "u4", {B.bin.size()},
            B.bin.data(), B.bin.size());
      } else if (cmd == "hamiltonian" || cmd == "lanczos") {
        string m, secs, tag; ss >> m >> secs >> tag;
        create_ops(S, m);
        auto mod = models.at(m);
        if (!mod->is_factorized)
          throw runtime_error("model " + m + " is not factorized: create an instance with format F first");
        sector sec(secs);
        auto v = values_for(S, m);
        Hamiltonian_Factorized<double> H(mod, v, sec);
        vector<double> x0 = seeded_start(H.dim);
        if (cmd == "hamiltonian") {
          put_d(tag + "_x0", x0);
          vector<double> y(H.dim, 0.0);
          H.mult_add(x0, y);
          put_d(tag + "_Hx0", y);
          for (auto& t : v) {
            auto* ob = dynamic_cast<one_body_operator<double>*>(mod->term.at(t.first).get());
            if (!ob) continue;
            if (ob->half_operators.count(sec.Nup()))
              dump_halfop(tag + "_" + t.first + "_up", ob->half_operators.at(sec.Nup()));
            if (ob->half_operators_dw.count(sec.Ndw()))
              dump_halfop(tag + "_" + t.first + "_dn", ob->half_operators_dw.at(sec.Ndw()));
          }
        } else {
          vector<double> alpha, beta, energy;
          size_t niter = 0;
          vector<double> gs(x0);
          LanczosEigenvalue(H, gs, alpha, beta, energy, niter, false);
          put_d(tag + "_alpha", alpha);
          put_d(tag + "_beta", beta);
          put_scalar(tag + "_E0", energy[0]);
          LanczosEigenvector(H, gs, alpha, beta, false);
          put_d(tag + "_psi", gs);
        }
      } else if (cmd == "hcheck" || cmd == "lanczos_e0") {
        // Large sectors: no vector is written.  hcheck: one timed mult_add on
        // the seeded start x0, reduced to scalars and a fixed sample of y;
        // lanczos_e0: LanczosEigenvalue only (energy, alpha, beta, time).
        string m, secs, tag; ss >> m >> secs >> tag;
        create_ops(S, m);
        auto mod = models.at(m);
        if (!mod->is_factorized)
          throw runtime_error("model " + m + " is not factorized: create an instance with format F first");
        sector sec(secs);
        auto v = values_for(S, m);
        Hamiltonian_Factorized<double> H(mod, v, sec);
        vector<double> x0 = seeded_start(H.dim);
        if (cmd == "hcheck") {
          vector<double> y(H.dim, 0.0);
          auto t0 = chrono::steady_clock::now();
          H.mult_add(x0, y);
          double sec_s = chrono::duration<double>(chrono::steady_clock::now() - t0).count();
          double s1 = 0, s2 = 0, sxy = 0;
          for (size_t i = 0; i < H.dim; i++) { s1 += y[i]; s2 += y[i] * y[i]; sxy += x0[i] * y[i]; }
          put_scalar(tag + "_sum", s1);
          put_scalar(tag + "_norm2", s2);
          put_scalar(tag + "_xy", sxy);
          put_scalar(tag + "_mult_add_s", sec_s);
          // sample index k: (k * 2654435761 + 12345) mod dim
          const size_t ns = 4096;
          vector<double> samp(ns);
          vector<uint64_t> at(ns);
          for (size_t k = 0; k < ns; k++) {
            at[k] = (k * 2654435761ull + 12345ull) % H.dim;
            samp[k] = y[at[k]];
          }
          put(tag + "_at", "u8", {ns}, at.data(), ns);
          put_d(tag + "_y", samp);
          uint64_t dim = H.dim;
          put(tag + "_dim", "u8", {}, &dim, 1);
        } else {
          vector<double> alpha, beta, energy;
          size_t niter = 0;
          auto t0 = chrono::steady_clock::now();
          LanczosEigenvalue(H, x0, alpha, beta, energy, niter, true);
          double sec_s = chrono::duration<double>(chrono::steady_clock::now() - t0).count();
          put_d(tag + "_alpha", alpha);
          put_d(tag + "_beta", beta);
          put_scalar(tag + "_E0", energy[0]);
          put_scalar(tag + "_seconds", sec_s);
        }
      } else if (cmd == "destroy") {
        string m, secs, tag; int orb, spin, pm; ss >> m >> secs >> orb >> spin >> pm >> tag;
        auto mod = models.at(m);
        sector sec(secs);
        auto B = mod->provide_factorized_basis(sec);
        state<double> st(sec, B->dim);
        st.psi = seeded_start(B->dim);
        symmetric_orbital a;
        a.orb = orb; a.spin = spin; a.irrep = 0; a.nambu = 0;
        vector<double> y;
        mod->create_or_destroy(pm, a, st, y, 1.0);
        put_d(tag + "_x", st.psi);
        put_d(tag + "_y", y);
      } else if (cmd == "gs") {
        size_t label; string tag; ss >> label >> tag;
        auto r = ED::ground_state_solve(label);
        put_scalar(tag + "_E0", r.first);
      } else if (cmd == "qmatrix") {
        size_t label; int spin; string tag; ss >> label >> spin >> tag;
        ED::Green_function_solve(label);
        auto q = ED::qmatrix(spin != 0, label);
        put_d(tag + "_e", q.first);
        size_t M = q.first.size();
        size_t L = M ? q.second.size() / M : 0;
        put(tag + "_v", "c16", {M, L}, q.second.data(), q.second.size());
      } else if (cmd == "gz" || cmd == "hyb" || cmd == "sigma") {
        size_t label; int spin; double re, im; string tag;
        ss >> label >> spin >> re >> im >> tag;
        cplx z(re, im);
        ED::Green_function_solve(label);
        matrix<cplx> G;
        if (cmd == "gz") G = ED::Green_function(z, spin != 0, label, false);
        else if (cmd == "hyb") G = ED::hybridization_function(z, spin != 0, label);
        else G = ED::self_energy(z, spin != 0, label);
        put_cmat(tag, G);
      } else if (cmd == "omega") {
        size_t label; string tag; ss >> label >> tag;
        ED::Green_function_solve(label);
        put_scalar(tag, ED::Potthoff_functional(label));
      } else if (cmd == "ops") {
        string m; ss >> m;
        create_ops(S, m);
      } else if (cmd == "lat_cluster") {
        string m; ss >> m;
        vector<vector3D<int64_t>> pos;
        int64_t x, y, z;
        while (ss >> x >> y >> z) pos.push_back(vector3D<int64_t>(x, y, z));
        QCM::add_cluster(vector3D<int64_t>(0, 0, 0), pos, -1, false);
        QCM::add_system(m, 0);
      } else if (cmd == "lat_model") {
        string name; ss >> name;
        vector<int64_t> sl;
        int64_t v;
        while (ss >> v) sl.push_back(v);
        vector<int64_t> uc(sl.size(), 0);
        for (size_t i = 0; i < sl.size() / 3; i++) uc[i * 4] = 1;
        QCM::new_lattice_model(name, sl, uc);
      } else if (cmd == "lat_hop") {
        string name; int64_t x, y, z; double amp; int tau, sigma;
        ss >> name >> x >> y >> z >> amp >> tau >> sigma;
        vector3D<int64_t> lk(x, y, z);
        QCM::hopping_operator(name, lk, amp, 1, 1, tau, sigma);
      } else if (cmd == "lat_inter") {
        string name, type; double amp; ss >> name >> amp >> type;
        vector3D<int64_t> lk(0, 0, 0);
        QCM::interaction_operator(name, lk, amp, 1, 1, type);
      } else if (cmd == "lat_dw") {
        string name, type; double qx, qy, qz, amp, phase;
        ss >> name >> type >> qx >> qy >> qz >> amp >> phase;
        vector3D<int64_t> lk(0, 0, 0);
        QCM::density_wave(name, lk, complex<double>(amp), 0, vector3D<double>(qx, qy, qz), phase, type);
      } else if (cmd == "lat_param") {
        string n; double v; ss >> n >> v; S.lat_values.push_back({n, v});
      } else if (cmd == "lat_equiv") {
        string n, r; double m; ss >> n >> m >> r; S.lat_equiv.push_back(make_tuple(n, m, r));
      } else if (cmd == "lat_sector") {
        string sec; ss >> sec; qcm_model->sector_strings.assign(1, sec);
      } else if (cmd == "lat_instance") {
        int label; ss >> label;
        if (!S.lat_params_set) {
          QCM::set_parameters(S.lat_values, S.lat_equiv);
          S.lat_params_set = true;
        } else {
          for (auto& p : S.lat_values) QCM::set_parameter(p.first, p.second);
        }
        QCM::new_model_instance(label);
      } else if (cmd == "lat_set") {
        string n; double v; ss >> n >> v;
        for (auto& p : S.lat_values) if (p.first == n) p.second = v;
        QCM::set_parameter(n, v);
      } else if (cmd == "lat_kgrid") {
        int a, b, c; ss >> a >> b >> c; QCM::set_wavevector_grid(a, b, c);
      } else if (cmd == "lat_wgrid") {
        int n; ss >> n;
        grid_freqs.resize(n); grid_weights.resize(n);
        for (int i = 0; i < n; i++) ss >> grid_freqs[i];
        for (int i = 0; i < n; i++) ss >> grid_weights[i];
      } else if (cmd == "lat_sef") {
        int label; string tag; ss >> label >> tag;
        put_scalar(tag, QCM::Potthoff_functional(label));
      } else if (cmd == "lat_ave") {
        // lat_ave LABEL TAG OP... : QCM::averages of the named one-body
        // operators on the wavevector and frequency grids, in that order
        int label; string tag, op; ss >> label >> tag;
        vector<string> ops;
        while (ss >> op) ops.push_back(op);
        auto ave = QCM::averages(ops, label);
        vector<double> v;
        for (auto& a : ave) v.push_back(a.second);
        put_d(tag, v);
      } else if (cmd == "lat_pe") {
        // lat_pe LABEL TAG : QCM::potential_energy on the wavevector and
        // frequency grids
        int label; string tag; ss >> label >> tag;
        put_scalar(tag, QCM::potential_energy(label));
      } else if (cmd == "lat_dos") {
        // lat_dos LABEL TAG NZ (re im)x NZ: QCM::dos on the wavevector grid,
        // one row of 2 n_band values per frequency
        int label, nz; string tag; ss >> label >> tag >> nz;
        vector<double> all;
        size_t width = 0;
        for (int i = 0; i < nz; i++) {
          double re, im; ss >> re >> im;
          vector<double> d = QCM::dos(cplx(re, im), label, true);
          width = d.size();
          all.insert(all.end(), d.begin(), d.end());
        }
        put(tag, "f8", {(size_t)nz, width}, all.data(), all.size());
      } else if (cmd == "lat_gper" || cmd == "lat_tk") {
        int label; string tag; ss >> label >> tag;
        vector<cplx> zs;
        if (cmd == "lat_gper") {
          int nz; ss >> nz;
          for (int i = 0; i < nz; i++) { double re, im; ss >> re >> im; zs.push_back(cplx(re, im)); }
        }
        int nk; ss >> nk;
        vector<vector3D<double>> ks;
        for (int i = 0; i < nk; i++) { double a, b, c; ss >> a >> b >> c; ks.push_back(vector3D<double>(a, b, c)); }
        vector<cplx> out;
        size_t d = 0;
        if (cmd == "lat_gper") {
          for (auto z : zs) {
            auto G = QCM::periodized_Green_function(z, ks, false, label);
            for (auto& g : G) { d = g.r; for (size_t i = 0; i < g.r; i++) for (size_t j = 0; j < g.c; j++) out.push_back(g(i, j)); }
          }
          put(tag, "c16", {zs.size(), ks.size(), d, d}, out.data(), out.size());
        } else {
          auto T = QCM::tk(ks, false, label);
          for (auto& g : T) { d = g.r; for (size_t i = 0; i < g.r; i++) for (size_t j = 0; j < g.c; j++) out.push_back(g(i, j)); }
          put(tag, "c16", {ks.size(), d, d}, out.data(), out.size());
        }
      } else if (cmd == "lat_gc" || cmd == "lat_V" || cmd == "lat_gcpt") {
        int label; string tag; double re, im; ss >> label >> tag >> re >> im;
        cplx z(re, im);
        matrix<cplx> M;
        if (cmd == "lat_gc") {
          M = QCM::cluster_Green_function(0, z, false, label, false);
        } else {
          double a, b, c; ss >> a >> b >> c;
          vector3D<double> k(a, b, c);
          if (cmd == "lat_V") M = QCM::V_matrix(z, k, false, label);
          else M = QCM::CPT_Green_function(z, k, false, label);
        }
        put_cmat(tag, M);
      } else if (cmd == "lat_dump") {
        int label; string tag; ss >> label >> tag;
        auto& I = *lattice_model_instances.at(label);
        auto& M = *qcm_model;
        vector<double> nb;
        for (auto& n : M.neighbor) { nb.push_back(n.x); nb.push_back(n.y); nb.push_back(n.z); }
        put(tag + "_neighbors", "f8", {M.neighbor.size(), 3}, nb.data(), nb.size());
        vector<double> gp;
        for (auto& p : M.Green_to_position) { gp.push_back(p.x); gp.push_back(p.y); gp.push_back(p.z); }
        put(tag + "_gpos", "f8", {M.Green_to_position.size(), 3}, gp.data(), gp.size());
        vector<double> el;  // r, c, n, re, im (parameter value applied)
        for (auto& op : M.term) {
          auto it = I.params.find(op.second->name);
          if (it == I.params.end()) continue;
          for (auto& e : op.second->IGF_elem) {
            cplx v = e.v * it->second;
            el.insert(el.end(), {(double)e.r, (double)e.c, (double)e.n, v.real(), v.imag()});
          }
        }
        put(tag + "_igf", "f8", {el.size() / 5, 5}, el.data(), el.size());
        put_cmat(tag + "_H", I.H);
        matrix<cplx> Hc = I.Hc.build_matrix();
        put_cmat(tag + "_Hc", Hc);
        vector<double> sd;
        for (int i = 0; i < 3; i++) { vector3D<double> e(i == 0, i == 1, i == 2); auto v = M.superdual.to(M.physdual.from(e)); sd.push_back(v.x); sd.push_back(v.y); sd.push_back(v.z); }
        put(tag + "_kmap", "f8", {3, 3}, sd.data(), sd.size());
      } else if (cmd == "lat_varia") {
        vector<string> names; string n;
        while (ss >> n) names.push_back(n);
        vector<vector<string>> v(1, names);
        QCM::CDMFT_variational_set(v);
      } else if (cmd == "lat_host") {
        int label; string tag; int nw; ss >> label >> tag >> nw;
        vector<double> w(nw), wt(nw);
        for (int i = 0; i < nw; i++) ss >> w[i];
        for (int i = 0; i < nw; i++) ss >> wt[i];
        QCM::CDMFT_host(w, wt, label);
        auto Hh = QCM::get_CDMFT_host(false, label);
        vector<cplx> out;
        size_t d = 0;
        for (auto& row : Hh) for (auto& g : row) { d = g.r; for (size_t i = 0; i < g.r; i++) for (size_t j = 0; j < g.c; j++) out.push_back(g(i, j)); }
        put(tag, "c16", {(size_t)nw, d, d}, out.data(), out.size());
      } else if (cmd == "lat_resid" || cmd == "lat_grad") {
        // lat_resid / lat_grad LABEL NP p.. : QCM::CDMFT_residuals /
        // CDMFT_gradient (cluster 0), printed on one stdout line
        int label, np_; ss >> label >> np_;
        vector<double> p(np_);
        for (int i = 0; i < np_; i++) ss >> p[i];
        vector<double> r = cmd == "lat_resid" ? QCM::CDMFT_residuals(p, 0, label)
                                              : QCM::CDMFT_gradient(p, 0, label);
        cout << "R " << r.size();
        cout.precision(17);
        for (double v : r) cout << ' ' << v;
        cout << '\n';
      } else if (cmd == "lat_dist") {
        int label; string tag; int np; ss >> label >> tag >> np;
        vector<double> p(np);
        for (int i = 0; i < np; i++) ss >> p[i];
        put_scalar(tag, QCM::CDMFT_distance(p, 0, label));
      } else {
        throw runtime_error("unknown spec command: " + cmd);
      }
      // A token the stream could not read leaves zeros behind: refuse it
      // (reading to the end of the line, as the list commands do, is fine).
      if (ss.fail() && !ss.eof()) throw runtime_error("malformed arguments in spec line: " + line.substr(0, 80));
    }
  } catch (std::exception& e) {
    cerr << "oracle driver error: " << e.what() << endl;
    return 1;
  }
  return 0;
}
