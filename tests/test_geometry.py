"""Host geometry vs the reference's own members (golden fixtures made by
running the reference, tests/golden/gen_golden.py): bit-exact."""
import hashlib
import json

import numpy as np
import pytest

from helpers import GOLDEN, load, mesh_of

ARRAYS = ["vertices", "face_off", "face_vtx", "nbr_off", "nbr", "nbr_edge", "face_centers",
          "normals", "area", "edge_normals", "bm_dist", "h_plus", "h_minus", "ff_plus",
          "ff_minus", "beta_plus", "beta_minus"]


@pytest.mark.parametrize("kind,level", [("hex", 2), ("hex", 3), ("quad", 3)])
def test_geometry_bit_exact(kind, level):
    import splash_gb300 as sg

    ref = load(f"geom_{kind}{level}.npz")
    g = sg.Geometry(mesh_of(kind, level))
    for name in ARRAYS:
        a, b = g[name], ref[name]
        assert a.shape == b.shape, name
        if a.dtype.kind == "f":
            assert np.array_equal(a.view(np.uint64), b.astype(np.float64).view(np.uint64)), name
        else:
            assert np.array_equal(a, b), name
    assert g.h0 == float(ref["h0"])


@pytest.mark.parametrize("key", ["hex4", "hex6", "hex7", "quad4", "quad6", "hex9", "quad9"])
def test_geometry_hashes(key):
    """Every geometry array, up to the large-mesh workloads' hex(9) (2,621,442
    faces) and quad(9) (1,572,864), hashed against the reference's members."""
    import splash_gb300 as sg

    data = json.loads((GOLDEN / "geom_hashes.json").read_text())["hashes"][key]
    kind, level = key[:-1], int(key[-1])
    g = sg.Geometry(mesh_of(kind, level))
    for name in ARRAYS:
        a = np.ascontiguousarray(g[name])
        a = a.astype("<i4") if a.dtype.kind == "i" else a.astype("<f8")
        assert hashlib.sha256(a.tobytes()).hexdigest() == data[name], f"{key}:{name}"
    assert float(g.h0).hex() == data["h0"]


@pytest.mark.parametrize("kind,level,nf", [("hex", 3, 642), ("hex", 4, 2562), ("quad", 3, 384),
                                           ("ico", 2, 320)])
def test_mesh_sizes_and_invariants(kind, level, nf):
    """F, S = sum of valences, closed-manifold edge pairing, betas sum to 1
    (the reference's own sanity checks, MUSCL_geometry.hpp:513-525)."""
    import splash_gb300 as sg

    g = sg.Geometry(mesh_of(kind, level))
    assert g.n_faces == nf == sg.n_faces_of(mesh_of(kind, level))
    off, nbe = g["face_off"], g["nbr_edge"]
    # every edge neighbour relation is symmetric
    for f in range(g.n_faces):
        for s in range(off[f], off[f + 1]):
            nb = nbe[s]
            assert f in nbe[off[nb]:off[nb + 1]]
    assert np.all(np.abs(g["beta_plus"].sum(axis=1) - 1) < 1e-8)
    assert np.all(np.abs(g["beta_minus"].sum(axis=1) - 1) < 1e-8)
    assert np.all(g["area"] > 0)
    assert abs(g["area"].sum() - 4 * np.pi) < 1e-9


def test_user_mesh_arrays_match_generated():
    """A mesh passed as arrays gives the same geometry as the generator."""
    import splash_gb300 as sg

    g = sg.Geometry(sg.icosphere_hex(2))
    m = sg.Mesh(vertices=g["vertices"], face_offsets=g["face_off"], face_vertices=g["face_vtx"])
    g2 = sg.Geometry(m)
    for name in ARRAYS:
        assert np.array_equal(g[name], g2[name]), name


def test_bad_mesh_rejected():
    import splash_gb300 as sg

    v = np.eye(3)
    m = sg.Mesh(vertices=v, face_offsets=np.array([0, 3]), face_vertices=np.array([0, 1, 5]))
    with pytest.raises(sg.SplashError):
        sg.Geometry(m)
