"""Generates tests/golden/ic_recipes_<mesh><n>.npz from the reference's own
initial-condition recipes (make_input.py in the reference checkout).

pandas is not installed, so a minimal stand-in module is placed in
sys.modules before the reference's make_input.py is loaded: read_table
parses the whitespace table into an array (column access and np.array()
work as the recipes use them) and DataFrame(...).to_csv records the array
and the float_format it was asked to write.  The recipes run in a scratch
directory whose results/face_centers.dat holds the unit face centres in the
C++ writer's format (15 significant digits), from this repository's
geometry (bit-identical to the reference's, tests/test_geometry.py).

Usage:  python tests/golden/gen_ic_golden.py --ref-root <reference checkout>
It is never run by the test-suite (the fixtures are committed).
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "muscl-scheme-on-spherical-mesh-wip_gb300"))

RECIPES = ["make_input_4", "make_input_4_cos_bell", "make_input_5", "make_input_5_sp_layer",
           "make_input_5_cos_bell", "make_input_5_const_entr"]
RECORDED: list = []


class _Table:
    """What the recipes use of a pandas DataFrame."""

    def __init__(self, data=None):
        self.data = np.asarray(data, dtype=np.float64)

    def __getitem__(self, col):
        return self.data[:, col]

    def __array__(self, dtype=None, copy=None):
        return self.data if dtype is None else self.data.astype(dtype)

    def to_csv(self, path, index=False, sep=" ", header=False, float_format=None):
        RECORDED.append({"path": str(path), "data": self.data.copy(), "float_format": float_format,
                         "index": index, "sep": sep, "header": header})


def _read_table(path, header=None, delimiter=None):
    rows = [line.split() for line in Path(path).read_text().splitlines() if line.strip()]
    return _Table(np.array(rows, dtype=np.float64))


def pandas_stub() -> types.ModuleType:
    m = types.ModuleType("pandas")
    m.read_table = _read_table
    m.DataFrame = lambda data=None, **kw: _Table(data)
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", required=True, help="reference checkout (holds make_input.py)")
    a = ap.parse_args()
    import splash_gb300 as sg
    from splash_gb300.input_recipes import format_face_centers

    src = Path(a.ref_root) / "make_input.py"
    sys.modules["pandas"] = pandas_stub()
    cwd = os.getcwd()
    for kind, level in (("hex", 3), ("quad", 3)):
        mesh = sg.Mesh({"hex": 0, "quad": 1}[kind], level)
        fc_text = format_face_centers(sg.Geometry(mesh).unit_face_centers())
        out = {"face_centers_text": np.array(fc_text)}
        with tempfile.TemporaryDirectory() as td:
            (Path(td) / "results").mkdir()
            (Path(td) / "input").mkdir()
            (Path(td) / "results" / "face_centers.dat").write_text(fc_text)
            os.chdir(td)
            try:
                spec = importlib.util.spec_from_file_location("ref_make_input", src)
                mod = importlib.util.module_from_spec(spec)
                RECORDED.clear()
                spec.loader.exec_module(mod)  # the module runs its active recipe on load
                for name in RECIPES:
                    RECORDED.clear()
                    getattr(mod, name)()
                    rec = RECORDED[-1]
                    assert rec["path"] == "input/input.dat" and rec["sep"] == " " and not rec["header"]
                    out[name] = rec["data"]
                    out[name + "__float_format"] = np.array(rec["float_format"] or "")
            finally:
                os.chdir(cwd)
        np.savez_compressed(HERE / f"ic_recipes_{kind}{level}.npz", **out)
        print(f"ic_recipes_{kind}{level}: {', '.join(f'{n} {out[n].shape}' for n in RECIPES)}")


if __name__ == "__main__":
    main()
