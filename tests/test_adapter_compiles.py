"""The reference-side adapter (include/qcmg_pyqcm_adapter.hpp) against the
reference itself: it compiles against the reference's own headers as a
Hamiltonian<double> subclass, and a program built from the reference's
compiled objects (oracle/_ref), the adapter and libqcmg runs the adapter
inside the reference's own ED layer.  Runs only where the reference tree is
present (QCMG_REFERENCE_DIR, default /root/reference); no GPU is needed: on a
machine without one, the engine's error must reach the reference's caller as
a qcm_error thrown by its own qcm_ED_throw."""
import glob
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

REF = os.environ.get("QCMG_REFERENCE_DIR", "/root/reference")
REF_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
LIBDIR = os.path.join(ROOT, "pyqcm_gb300", "_build")

pytestmark = pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")


def _includes():
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "refbuild", "shim")]
    for d in ("src_ed", "src_ed/Hamiltonian", "src_ed/Operators", "src_qcm", "src_util",
              "external/cubature"):
        inc.append("-I" + os.path.join(REF, d))
    return inc


def test_adapter_compiles_against_reference_headers():
    src = r'''
#include "model_instance.hpp"
#include "qcmg_pyqcm_adapter.hpp"
template class Hamiltonian_GPU<double>;
Hamiltonian<double>* make(shared_ptr<model> m, const map<string, double>& v, sector s) {
  return new Hamiltonian_GPU<double>(m, v, s);
}
'''
    with tempfile.TemporaryDirectory() as t:
        f = os.path.join(t, "adapter.cpp")
        with open(f, "w") as fh:
            fh.write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w"] + _includes() + [f],
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


# A 4-site chain built through the reference's ED:: API, then the adapter's
# constructor, mult_add and states() as the reference's model_instance would
# call them.  Exit 3: a qcm_error reached the caller (its text is printed).
LINK_SRC = r'''
#include <iostream>
#include "QCM.hpp"
#include "qcm_ED.hpp"
#include "model_instance.hpp"
#include "qcmg_pyqcm_adapter.hpp"
extern map<string, shared_ptr<model>> models;
int main() {
  QCM::global_parameter_init();
  ED::new_model("chain", 4, 0, {}, false);
  vector<matrix_element<double>> t;
  for (int i = 0; i < 3; ++i) {
    t.push_back(matrix_element<double>(i, i + 1, -1.0));
    t.push_back(matrix_element<double>(i + 4, i + 5, -1.0));
  }
  ED::new_operator("chain", "t", "one-body", t);
  vector<matrix_element<double>> u;
  for (int i = 0; i < 4; ++i) u.push_back(matrix_element<double>(i, i + 4, 1.0));
  ED::new_operator("chain", "U", "interaction", u);
  map<string, double> v{{"t", 1.0}, {"U", 4.0}};
  try {
    Hamiltonian_GPU<double> H(models.at("chain"), v, sector("R0:N4:S0"));
    vector<double> x(H.dim, 0.0), y(H.dim, 0.0);
    x[0] = 1.0;
    H.mult_add(x, y);
    double e0 = 1e12;
    auto st = H.states(e0);
    std::cout << "dim " << H.dim << " E0 " << e0 << std::endl;
    return 0;
  } catch (const qcm_error& e) {
    std::cout << "qcm_error: " << e.what() << std::endl;
    return 3;
  }
}
'''


def _openblas():
    import scipy
    d = os.path.abspath(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs"))
    libs = glob.glob(os.path.join(d, "libscipy_openblas*.so"))
    return d, os.path.basename(libs[0]) if libs else None


def test_adapter_runs_inside_the_reference():
    """Links the adapter with the reference's own objects and libqcmg, then
    runs it through the reference's ED layer: with a GPU it constructs,
    multiplies and solves; without one, the engine's 'no usable CUDA device'
    reaches the caller as the reference's qcm_error."""
    objs = [o for o in glob.glob(os.path.join(REF_OBJ, "**", "*.o"), recursive=True)
            if not o.endswith("ref_driver.o")]
    if not objs or not os.path.exists(os.path.join(LIBDIR, "libqcmg.so")):
        pytest.skip("the reference oracle or libqcmg is not built")
    bdir, blas = _openblas()
    if not blas:
        pytest.skip("SciPy's OpenBLAS not found")
    with tempfile.TemporaryDirectory() as t:
        src = os.path.join(t, "main.cpp")
        exe = os.path.join(t, "adapter_run")
        with open(src, "w") as fh:
            fh.write(LINK_SRC)
        cmd = (["g++", "-std=c++17", "-O1", "-w", "-fopenmp"] + _includes() + [src, "-o", exe]
               + objs + ["-L" + LIBDIR, "-lqcmg", "-Wl,-rpath," + LIBDIR,
                         "-L" + bdir, "-l:" + blas, "-Wl,-rpath," + bdir])
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    out = run.stdout
    import torch
    if torch.cuda.is_available():
        assert run.returncode == 0, out + run.stderr
        assert "dim 36" in out
    else:
        assert run.returncode == 3, out + run.stderr
        assert "qcm_error: GPU Hamiltonian: no usable CUDA device" in out, out


def test_lattice_adapter_compiles_against_reference_headers():
    src = r'''
#include "lattice_model_instance.hpp"
#include "qcm_ED.hpp"
#include "QCM.hpp"
#include "qcmg_pyqcm_lattice_adapter.hpp"
bool sef(lattice_model_instance& I, double& v) { return qcmg_lattice_adapter::potthoff_grid(I, v); }
bool gper(lattice_model_instance& I, const vector<vector3D<double>>& k, vector<Complex>& g) {
  return qcmg_lattice_adapter::periodized_Green_function(I, Complex(0.0, 0.5), k, false, g);
}
bool pgf(lattice_model_instance& I, const vector<double>& w, vector<matrix<Complex>>& P) {
  return qcmg_lattice_adapter::projected_Green_function(I, w, 8, false, P);
}
bool dos(lattice_model_instance& I, vector<double>& d) {
  return qcmg_lattice_adapter::dos_grid(I, Complex(0.1, 0.1), d);
}
'''
    with tempfile.TemporaryDirectory() as t:
        f = os.path.join(t, "lattice_adapter.cpp")
        with open(f, "w") as fh:
            fh.write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w"] + _includes() + [f],
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


# The AF-free 2x2 plaquette lattice (t = 1, U = 4, mu = 2) built through the
# reference's QCM:: API; the Potthoff functional's grid frequency loop through
# the lattice adapter.  Exit 3: a qcm_error reached the caller.
LATTICE_LINK_SRC = r'''
#include <iostream>
#include "QCM.hpp"
#include "qcm_ED.hpp"
#include "lattice_model_instance.hpp"
#include "qcmg_pyqcm_lattice_adapter.hpp"
extern shared_ptr<lattice_model> qcm_model;
extern map<int, unique_ptr<lattice_model_instance>> lattice_model_instances;
int main() {
  qcm_model = make_shared<lattice_model>();  // as the reference's module initialization does
  QCM::global_parameter_init();
  ED::new_model("clus", 4, 0, {}, false);
  vector<vector3D<int64_t>> pos{{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}};
  QCM::add_cluster(vector3D<int64_t>(0, 0, 0), pos, -1, false);
  QCM::add_system("clus", 0);
  vector<int64_t> superlattice{2, 0, 0, 0, 2, 0}, unit_cell{1, 0, 0, 0, 1, 0};
  QCM::new_lattice_model("L", superlattice, unit_cell);
  vector3D<int64_t> on_site(0, 0, 0), ex(1, 0, 0), ey(0, 1, 0);
  QCM::interaction_operator("U", on_site, 1.0, 1, 1, "Hubbard");
  QCM::hopping_operator("t", ex, -1.0, 1, 1, 1, 0);
  QCM::hopping_operator("t", ey, -1.0, 1, 1, 1, 0);
  vector<pair<string, double>> values{{"t", 1.0}, {"U", 4.0}, {"mu", 2.0}};
  vector<tuple<string, double, string>> equiv;
  QCM::set_parameters(values, equiv);
  qcm_model->sector_strings.assign(1, "R0:N4:S0");
  QCM::new_model_instance(0);
  QCM::set_wavevector_grid(8, 8, 1);
  grid_freqs = {0.1, 0.5, 2.0, 8.0};
  grid_weights = {0.25, 0.25, 0.25, 0.25};
  try {
    double Iv = 0.0;
    bool done = qcmg_lattice_adapter::potthoff_grid(*lattice_model_instances.at(0), Iv);
    std::cout << "covered " << done << " Iv " << Iv << std::endl;
    return 0;
  } catch (const qcm_error& e) {
    std::cout << "qcm_error: " << e.what() << std::endl;
    return 3;
  }
}
'''


def test_lattice_adapter_runs_inside_the_reference():
    """Links the lattice adapter with the reference's own objects and
    libqcmg and runs the Potthoff functional's frequency loop through it on a
    lattice model built by the reference's QCM layer (whose cluster solve
    runs on the CPU): without a GPU, the engine's error reaches the caller as
    the reference's qcm_error."""
    objs = [o for o in glob.glob(os.path.join(REF_OBJ, "**", "*.o"), recursive=True)
            if not o.endswith("ref_driver.o")]
    if not objs or not os.path.exists(os.path.join(LIBDIR, "libqcmg.so")):
        pytest.skip("the reference oracle or libqcmg is not built")
    bdir, blas = _openblas()
    if not blas:
        pytest.skip("SciPy's OpenBLAS not found")
    with tempfile.TemporaryDirectory() as t:
        src = os.path.join(t, "main.cpp")
        exe = os.path.join(t, "lattice_adapter_run")
        with open(src, "w") as fh:
            fh.write(LATTICE_LINK_SRC)
        cmd = (["g++", "-std=c++17", "-O1", "-w", "-fopenmp"] + _includes() + [src, "-o", exe]
               + objs + ["-L" + LIBDIR, "-lqcmg", "-Wl,-rpath," + LIBDIR,
                         "-L" + bdir, "-l:" + blas, "-Wl,-rpath," + bdir])
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    out = run.stdout
    import torch
    if torch.cuda.is_available():
        assert run.returncode == 0, out + run.stderr
        assert "covered 1" in out
    else:
        assert run.returncode == 3, out + run.stderr
        assert "qcm_error: GB300 lattice engine:" in out, out
