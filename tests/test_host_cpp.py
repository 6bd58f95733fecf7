"""The C++ drop-in driver (supermc_gb300/host): its ParameterReader follows the
reference's parsing rules (src/ParameterReader.cpp), and the superMC program
fails cleanly without a GPU.  Host code only."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HOST = os.path.join(os.path.dirname(HERE), "supermc_gb300", "host")

PROGRAM = r'''
#include <cstdio>
#include "ParameterReader.h"
int main(int argc, char *argv[]) {
  smc::ParameterReader r;
  r.readFromFile(argv[1]);
  r.readFromArguments(argc, argv, "#", 2);
  std::printf("%g %g %g %d\n", r.getVal("nev"), r.getVal("Alpha"), r.getVal("ecm"), (int)r.exist("maxX"));
  int errors = 0;
  try { r.getVal("no_such_key"); } catch (const smc::ParameterError &) { errors++; }
  try { r.phraseOneLine("novalue"); } catch (const smc::ParameterError &) { errors++; }
  try { r.readFromFile("/nonexistent/parameters.dat"); } catch (const smc::ParameterError &) { errors++; }
  std::printf("%d %g\n", errors, r.getVal("missing", 7.5));
  return 0;
}
'''


@pytest.fixture(scope="module")
def reader_exe(tmp_path_factory):
    d = tmp_path_factory.mktemp("pr")
    src = d / "t.cpp"
    src.write_text(PROGRAM)
    exe = d / "t"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", HOST, str(src), os.path.join(HOST, "ParameterReader.cpp"),
                           "-o", str(exe)])
    return exe


def test_parameter_reader_rules(reader_exe, tmp_path):
    pfile = tmp_path / "parameters.dat"
    pfile.write_text("nev = 100   # events\n  ALPHA=0.118\n\n# comment only\nmaxx = 13\necm = 200\n")
    out = subprocess.run([str(reader_exe), str(pfile), "nev=7", "Ecm = 2760 # override"], capture_output=True,
                         text=True, check=True).stdout.split("\n")
    assert out[0] == "7 0.118 2760 1"
    assert out[1] == "3 7.5"


def test_driver_without_gpu_reports_and_exits(tmp_path):
    from supermc_gb300 import build
    exe = build.EXE
    if not os.path.exists(exe):
        pytest.skip("library not built")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    (tmp_path / "parameters.dat").write_text("operation = 9\nnev = 10\n")
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1
    assert "smc_create" in r.stderr
