"""The C++ IAlgorithm adapter (openbcsim_gb300/adapter/GB300Algorithm.hpp)
compiles against the reference's own headers and links against the engine
(where the reference sources are present; nothing here needs a GPU)."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle.oracle import reference_sources

REF = reference_sources()
ADAPTER = os.path.join(ROOT, "openbcsim_gb300", "adapter", "GB300Algorithm.hpp")


def adapter_source():
    with open(ADAPTER) as f:
        return f.read()


MAIN = r'''
#include <iostream>
#include "GB300Algorithm.hpp"
int main() {
    bcsim::IAlgorithm::s_ptr sim(new bcsim::GB300Algorithm);
    sim->set_parameter("sound_speed", "1540");
    try { sim->set_parameter("nope", "1"); } catch (const std::runtime_error& e) { std::cout << e.what() << std::endl; }
    try { std::vector<std::vector<std::complex<float>>> out; sim->simulate_lines(out); }
    catch (const std::runtime_error& e) { std::cout << e.what() << std::endl; }
    std::cout << sim->get_parameter("sound_speed") << std::endl;
    return 0;
}
'''


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="reference sources not present")
def test_adapter_compiles_links_and_reports_errors(tmp_path):
    from openbcsim_gb300 import build

    lib = build.build()
    d = tmp_path / "algorithm"
    d.mkdir()
    (d / "GB300Algorithm.hpp").write_text(adapter_source())
    (d / "main.cpp").write_text(MAIN)
    srcs = [f"{REF}/core/ScanSequence.cpp", f"{REF}/core/BeamProfile.cpp"]
    exe = tmp_path / "adapter"
    cmd = ["g++", "-std=c++14", "-O1", "-w", f"-I{REF}/core/algorithm", f"-I{REF}/core", f"-I{ROOT}/include", str(d / "main.cpp"), *srcs,
           "-o", str(exe), f"-L{os.path.dirname(lib)}", "-lbcsim_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stderr
    lines = run.stdout.splitlines()
    assert lines[0] == "illegal parameter name: 'nope'"
    assert lines[1] == "Scan sequence not configured."
    assert float(lines[2]) == 1540.0
