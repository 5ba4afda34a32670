"""The reference-side adapter (include/qcmg_pyqcm_adapter.hpp) compiles
against the reference's own headers as a Hamiltonian<double> subclass.
Runs only where the reference tree is present (syntax check, no GPU)."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

REF = "/root/reference"


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
def test_adapter_compiles_against_reference_headers():
    src = r'''
#include "model_instance.hpp"
#include "qcmg_pyqcm_adapter.hpp"
template class Hamiltonian_GPU<double>;
Hamiltonian<double>* make(shared_ptr<model> m, const map<string, double>& v, sector s) {
  return new Hamiltonian_GPU<double>(m, v, s);
}
'''
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "refbuild", "shim")]
    for d in ("src_ed", "src_ed/Hamiltonian", "src_ed/Operators", "src_qcm", "src_util",
              "external/cubature"):
        inc.append("-I" + os.path.join(REF, d))
    with tempfile.TemporaryDirectory() as t:
        f = os.path.join(t, "adapter.cpp")
        with open(f, "w") as fh:
            fh.write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w"] + inc + [f],
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
