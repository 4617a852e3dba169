"""The C++ drop-in header compiles on a machine without a GPU (syntax and templates only)."""
import subprocess

from conftest import REPO


def test_cpp_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "iqs_gb300/qureg.hpp"\n'
                   "template class iqs::QubitRegister<ComplexDP>;\n"
                   "template class iqs::QubitRegister<ComplexSP>;\n"
                   "template class iqs::NoisyQureg<ComplexDP>;\n"
                   "template class iqs::QubitRegisterMetric<ComplexDP>;\n"
                   "template class iqs::QubitRegisterMetric<ComplexSP>;\n"
                   "template class iqs::NoisyQureg<ComplexSP>;\n"
                   "template class iqs::ChiMatrix<ComplexSP, 16, 32>;\n"
                   "int main() { return 0; }\n")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(REPO / "include"), str(src)], check=True)
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "shim_driver.cpp")], check=True)
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "qaoa_driver.cpp")], check=True)
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "noise_driver.cpp")], check=True)


def test_tinymatrix_and_chimatrix_reference_unit_tests(tmp_path):
    """The reference's TinyMatrix / ChiMatrix unit tests against the drop-in header
    (tests/cpp/tinymatrix_driver.cpp); host code only."""
    exe = tmp_path / "tm"
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "tinymatrix_driver.cpp"), "-L", str(libdir), "-liqsg",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_permutation_and_gate_counter_reference_unit_tests(tmp_path):
    """The reference's Permutation and GateCounter unit tests against the drop-in header
    (tests/cpp/permutation_driver.cpp); host code only."""
    exe = tmp_path / "pd"
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "permutation_driver.cpp"), "-L", str(libdir), "-liqsg",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
