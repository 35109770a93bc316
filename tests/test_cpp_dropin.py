"""The C++ drop-in classes (include/splash_muscl.hpp): a driver with the
reference driver's call sequence, compiled against the header and the
library, must write the same output files as the reference (golden texts
produced by the reference itself, tests/golden/gen_golden.py)."""
import json
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import load

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300"
DRIVER = Path(__file__).resolve().parent / "cpp" / "drop_in_driver.cpp"


def compile_driver(out: Path, syntax_only=False):
    cmd = ["g++", "-std=c++17", "-O2", f"-I{REPO / 'include'}", str(DRIVER)]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        cmd += ["-o", str(out), f"-L{PKG / 'lib'}", "-lsplash_gb300", f"-Wl,-rpath,{PKG / 'lib'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_header_compiles_with_reference_names():
    compile_driver(None, syntax_only=True)


def test_json_reader_and_mesh_sizes(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(r'''
#define SPLASH_REFERENCE_NAMES
#include "splash_muscl.hpp"
#include <cassert>
#include <sstream>
int main() {
  std::istringstream is("{ \"dim\": 5, \"dt\": 0.25, \"gam3d\":1.333333333, \"accretion_on\":true,"
                        " \"friction_on\": false, \"name\": \"x\" }");
  json j = json::parse(is);
  double dt = j["dt"]; size_t dim = j["dim"]; bool a = j["accretion_on"]; bool f = j["friction_on"];
  assert(dt == 0.25 && dim == 5 && a && !f);
  std::string n = j["name"]; assert(n == "x");
  pmp::SurfaceMesh m = pmp::icosphere_hex(4); assert(m.n_faces() == 2562);
  assert(pmp::quad_sphere(3).n_faces() == 384);
  return 0;
}''')
    exe = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", f"-I{REPO / 'include'}", str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe)], check=True)


def _numbers(text):
    return np.array([float(x) for x in text.split()])


@pytest.mark.gpu
def test_drop_in_driver_writes_reference_files(tmp_path):
    import splash_gb300 as sg

    w = load("writers_hex3_hllcp.npz")
    files = dict(zip(w["files"].tolist(), w["texts"].tolist()))
    exe = tmp_path / "driver"
    compile_driver(exe)
    (tmp_path / "input").mkdir()
    (tmp_path / "results").mkdir()
    p = {"dim": 5, "dt": float(w["dt0"]), "t_max": 1e9, "maxstep": 10**9, "skipstep": 100,
         "gam3d": 4 / 3, "omega_ns": 0.0, "threads": 8, "accretion_on": True,
         "accretion_rate": 1e-2, "e_acc": 0.5, "omega_acc_abs": 0.5, "tilt_angle": 0.2,
         "acc_width": 0.1, "alpha": 1e-6, "friction_on": True}
    (tmp_path / "input" / "parameters.json").write_text(json.dumps(p))
    sg.initial_conditions.write_input_dat(tmp_path / "input" / "input.dat", w["U0"])
    env = dict(os.environ)
    res = subprocess.run([str(exe), "hex", "3", "3", str(int(w["steps"])), repr(float(w["dt0"])), "1"],
                         cwd=tmp_path, capture_output=True, text=True, env=env)
    assert res.returncode == 0, res.stderr
    out = tmp_path / "results"
    # geometry writers: identical text (15 significant digits of bit-identical values)
    for name in ("face_centers.dat", "faces.dat", "vertices.dat"):
        assert (out / name).read_text() == files[name], name
    # state writers (6 significant digits): same numbers
    for name in ("rho.dat", "p.dat", "omega.dat", "curl.dat", "final_state.dat"):
        a, b = _numbers((out / name).read_text()), _numbers(files[name])
        assert a.shape == b.shape, name
        assert np.allclose(a, b, rtol=2e-6, atol=1e-300), name
    # the per-step line (6 significant digits): same times, mass gains and L
    log_a = [l for l in (out / "steplog.txt").read_text().splitlines() if l]
    log_b = [l for l in files["steplog.txt"].splitlines() if l]
    assert len(log_a) == len(log_b) == int(w["steps"])
    num = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?")
    for la, lb in zip(log_a, log_b):
        na, nb = np.array(num.findall(la), dtype=float), np.array(num.findall(lb), dtype=float)
        assert na.shape == nb.shape == (6,), (la, lb)
        assert np.allclose(na, nb, rtol=2e-5, atol=1e-9), (la, lb)
    lc_a = _numbers((out / "lightcurves.txt").read_text()).reshape(-1, 5)
    lc_b = _numbers(files["lightcurves.txt"]).reshape(-1, 5)
    assert np.allclose(lc_a, lc_b, rtol=1e-12, atol=0)
    # write_t_L: the built reference writes no Lx/Ly/Lz (its loop counter is
    # uninitialised, physics/adiabatic.hpp:181); here they hold l_x, l_y, l_z
    fin = _numbers((out / "final_state.dat").read_text()).reshape(-1, 5)
    for k, name in enumerate(("Lx.dat", "Ly.dat", "Lz.dat")):
        lines = (out / name).read_text().splitlines()
        assert len(lines) == 2
        vals = _numbers(lines[1])[1:]
        assert np.allclose(vals, fin[:, k + 1], rtol=2e-6, atol=1e-300)
